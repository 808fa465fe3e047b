/*
 * rbc3d_gpu.h -- C ABI of the GB300 implementation of RBC3D's Ewald-split
 * boundary-integral matvec (real-space Stokeslet/stresslet pair sums over cell
 * lists, PME spread / k-space influence / gather, singular and near-singular
 * polar-patch corrections, wall triangle quadrature, wall no-slip GMRES).
 *
 * Every entry point replaces one Fortran module procedure of RBC3D (cited per
 * function, paths relative to the RBC3D source tree).  Conventions:
 *
 *  - Plain pointers and sizes only.  All arrays are caller-owned HOST buffers;
 *    device buffers are owned by the context.  Calls are synchronous at the ABI
 *    edge.  One context per host thread.
 *  - Layouts follow the Fortran column-major arrays of the reference:
 *      point arrays   x(N,3)   -> x[c*N + p], c = 0..2 (SoA)
 *      cell point p  = icell*nlat*nlon + ilon*nlat + ilat   (ilat fastest),
 *                      i.e. the order of SourceList_UpdateCoord / TargetList_Update
 *      spline tables  per cell: u, u1, u2, u12 (in this order), each
 *                      (m=2*nlat, n=nlon, nvar) column-major -> 4*m*n*nvar doubles
 *                      per cell (t_spline of ModDataStruct), cells consecutive
 *      wall e2v(nele,3) 1-based vertex ids (ModWall), column-major
 *  - Velocity outputs ACCUMULATE into v (v += ...), like the reference L2
 *    routines, except the L3 drivers that overwrite (documented per call).
 *  - Every call returns an rbc3d_status; rbc3d_last_error() gives text.
 */
#ifndef RBC3D_GPU_H
#define RBC3D_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

#define RBC3D_ABI_VERSION 1
#define RBC3D_MAX_CELLTYPES 8
#define RBC3D_NBR_MAX 32 /* NMax of NbrRbcList_Create, ModRbcSingInt.F90:319 */

typedef int rbc3d_status;
enum {
  RBC3D_OK = 0,
  RBC3D_ERR_ARG = 1,      /* bad argument / size */
  RBC3D_ERR_CUDA = 2,     /* CUDA runtime or cuFFT failure */
  RBC3D_ERR_TIMEOUT = 3,  /* a bounded device wait ran out */
  RBC3D_ERR_NOCONV = 4,   /* GMRES reached max_it without meeting rtol */
  RBC3D_ERR_OVERFLOW = 5, /* neighbour-cell list above RBC3D_NBR_MAX, or a
                             work list above its capacity */
  RBC3D_ERR_STATE = 6,    /* call order (e.g. no cells set) */
  RBC3D_ERR_NOMEM = 7
};

/* Arithmetic of one matvec. */
enum {
  RBC3D_FP64 = 0,  /* plain form: everything FP64 */
  RBC3D_FP32C = 1, /* pair sums, spread, FFT, gather in FP32 with per-target
                      compensated accumulation; self / near-singular
                      corrections FP64 */
  RBC3D_FP32M = 2, /* as FP32C, but the own-cell polar patch (RBC_SingInt) in
                      FP32 with FP64-accurate (hi/lo) positions; needs the
                      uniform longitude grid phi(j) = j*2*pi/nlon */
  RBC3D_FP32D = 3  /* as FP32C, but the own-cell polar patch in float-float
                      arithmetic (hi + lo FP32 pairs, 48 significant bits) on
                      the FP32 pipe: agrees with the FP64 patch to 2e-12;
                      needs the uniform longitude grid */
};

/* Target lists (t_TargetList instances of ModData.F90:19-20). */
enum {
  RBC3D_TLIST_RBC = 0,  /* tlist_rbc: all cell surface points */
  RBC3D_TLIST_WALL = 1, /* tlist_wall: all wall vertices (Acoef = 2) */
  RBC3D_TLIST_RAW = 2   /* TargetList_CreateFromRaw (Acoef = 2, indx = -1) */
};

/* Term selection for rbc3d_matvec. */
enum {
  RBC3D_TERM_REAL = 1u,   /* AddIntOnRbcs pair sums (incl. mask) */
  RBC3D_TERM_CORR = 2u,   /* RBC_SingInt + RBC_NearSingInt */
  RBC3D_TERM_LINEAR = 4u, /* AddLinearInt */
  RBC3D_TERM_PME = 8u,    /* PME_Distrib_Source/Transform/Add_Interp_Vel */
  RBC3D_TERM_WALLS = 16u, /* AddIntOnWalls */
  RBC3D_TERM_ALL = 31u
};

typedef struct rbc3d_params {
  double Lb[3];  /* periodic box (ModConf Lb) */
  double alpha;  /* Ewald splitting parameter alpha_Ewd */
  double rc;     /* real-space cut-off rc_Ewd */
  double eps;    /* Ewald tolerance eps_Ewd (informational / default rtol) */
  int Nb[3];     /* PME mesh Nb_Ewd */
  int P;         /* B-spline points PBspln_Ewd */
  int nlat, nlon;/* cell surface grid (Gauss x uniform), shared by all cells */
  int ncelltypes;
  double viscRat[RBC3D_MAX_CELLTYPES]; /* -> Acoef/Bcoef by initCOEFs */
  double vBkg[3];                      /* background velocity */
} rbc3d_params;

typedef struct rbc3d_counts {
  long long pairs_within_rc;  /* (target, source) pairs with r < rc, last real-space pass */
  long long nbr_items;        /* (target, other cell) near-singular candidates */
  long long nearsing_items;   /* candidates that passed the distance check */
  long long self_items;       /* targets given RBC_SingInt */
  long long wall_pairs;       /* (target, triangle) pairs within rc */
  long long wall_duffy;       /* of which integrated with Duffy's rule */
  int nbr_overflow;           /* targets whose neighbour list exceeded RBC3D_NBR_MAX */
  long long kernel_launches;  /* kernels of this library launched so far on the context */
  long long screen_misses;    /* FP32C near-singular screen: screened items the FP64
                                 test would correct (counted with RBC3D_VERIFY_SCREEN=1) */
  long long near_replays;     /* FP32 modes: candidates given the FP32 projection replay */
  long long near_projections; /* candidates given the FP64 projection */
} rbc3d_counts;

typedef struct rbc3d_solve_opts {
  double rtol;   /* converged when ||r|| < rtol*||b||, b the right-hand side
                    (KSPSetTolerances rtol, KSPConvergedDefault) */
  int max_it;    /* KSPSetTolerances max_it */
  int restart;   /* GMRES restart (PETSc default 30) */
  int prec;      /* matvec arithmetic: RBC3D_FP64, or an FP32 mode
                    (RBC3D_FP32C, RBC3D_FP32M) for a mixed-precision solve:
                    inner GMRES cycles with the FP32 operator correct x
                    against the FP64 residual b - A x (iterative refinement),
                    and convergence is judged on that FP64 residual */
  int guess;     /* 0: zero increment (reference); 1: caller-supplied guess;
                    2: caller-supplied guess scaled by a = <b,Ax0>/||Ax0||^2
                    (never a larger initial residual than 0);
                    3: two guess vectors x1, x2 (2 x dof doubles), combined
                    as p x1 + q x2 with the least-squares p, q (one extra
                    matvec);
                    4: wall solve only: the prediction of the learned
                    spectral operator (rbc3d_wall_spectral_init);
                    5: wall solve only: that prediction as x0, and the
                    operator as a right preconditioner (GMRES on A M; the
                    residual and the convergence test stay those of
                    b - A x): the inverse of each axial mode whose learned
                    basis is complete, the identity on the others */
} rbc3d_solve_opts;

typedef struct rbc3d_solve_stats {
  int iterations;
  int converged;       /* 1 if ||r||/||b|| <= rtol */
  double rnorm0;       /* ||b - A x0|| */
  double rnorm;        /* final residual norm (true residual, recomputed) */
  double bnorm;
  double ms;           /* wall time of the solve */
  int matvecs;         /* operator applications, FP64 and FP32 */
  int refinements;     /* mixed-precision solves: FP32 corrections applied (0 for FP64) */
} rbc3d_solve_stats;

typedef struct rbc3d_ctx rbc3d_ctx;

/* ---- context --------------------------------------------------------- */
/* Replaces PME_Init (ModPME.F90:252) + the Ewald tables of ModEwaldFunc.F90
 * + initCOEFs (ModConf.F90:327) + RbcPolarPatch_Create (ModPolarPatch.F90:27). */
rbc3d_status rbc3d_create(const rbc3d_params* prm, rbc3d_ctx** out);
/* Replaces PME_Finalize (ModPME.F90:342). */
rbc3d_status rbc3d_destroy(rbc3d_ctx* ctx);
const char* rbc3d_last_error(const rbc3d_ctx* ctx);
int rbc3d_abi_version(void);

/* Derived Ewald parameters: SetEwaldPrms (ModConf.F90:348-408), single rank.
 * Returns rc (capped at min(Lb)/3.001) and Nb for the given alpha/eps. */
rbc3d_status rbc3d_ewald_prms(double alpha, double eps, const double Lb[3],
                              int P, double* rc, int Nb[3]);

/* ---- surfaces -------------------------------------------------------- */
/* Cell grid: th(nlat) Gauss colatitudes, phi(nlon), w(nlat) = Gauss weight *
 * 2*pi/nlon (RBC_Create, ModRbc.F90:92-94). */
rbc3d_status rbc3d_set_cell_grid(rbc3d_ctx* ctx, const double* th,
                                 const double* phi, const double* w);
/* Cell geometry: SourceList_UpdateCoord + TargetList_Update for rbcs
 * (ModSourceList.F90:92, ModTargetList.F90:95) plus the geometry consumed by
 * the corrections (RBC_ComputeGeometry / Rbc_BuildSurfaceSource xFlag,
 * ModRbc.F90:404,716): x, a3 (N x 3), detJ (N), area, meshSize (ncell),
 * celltype (ncell, 0-based), spline tables of x (nvar 3), a3 (3), detJ (1). */
rbc3d_status rbc3d_set_cells(rbc3d_ctx* ctx, int ncell, const int* celltype,
                             const double* x, const double* a3,
                             const double* detJ, const double* area,
                             const double* meshSize, const double* spl_x,
                             const double* spl_a3, const double* spl_detJ);
/* Cell densities: SourceList_UpdateDensity (ModSourceList.F90:160) + the
 * FdetJ / GdetJ splines (Rbc_BuildSurfaceSource fFlag/gFlag).  f, g are the
 * raw surface densities (N x 3); either pair may be NULL (left unchanged). */
rbc3d_status rbc3d_set_cell_density(rbc3d_ctx* ctx, const double* f,
                                    const double* g, const double* spl_FdetJ,
                                    const double* spl_GdetJ);
/* Walls (one wall): Wall_ComputeGeometry + SourceList_UpdateCoord(walls) +
 * TargetList_Update(walls) (ModWall.F90:118, ModTimeInt.F90:80-82).
 * x (nvert x 3), e2v (nele x 3, 1-based), indxVertGlb (nvert, 1-based unique
 * vertex id, GlobData_Init ModData.F90:47-58). */
/* The same two steps from the raw surface fields alone, with the derived
 * geometry and tables computed on the device as the reference derives them:
 * set_cells_x = RBC_ComputeGeometry (a3, detJ, area, meshSize; ModRbc.F90:404)
 * + Rbc_BuildSurfaceSource(xFlag) (the x, a3, detJ spline tables through
 * ShAnalGau, ShFilter to degree < nlat0, ShSynthEqu, Spline_Build_On_Sphere;
 * ModRbc.F90:716) + SourceList_UpdateCoord + TargetList_Update;
 * set_cell_density_x = Rbc_BuildSurfaceSource(fFlag/gFlag) +
 * SourceList_UpdateDensity.  x, f, g: N x 3; f or g may be NULL.
 * Both return once the caller's arrays have been copied; the derivation
 * continues on the device, ordered before every later call on the context
 * (an error in it is reported by the next call that waits for it). */
rbc3d_status rbc3d_set_cells_x(rbc3d_ctx* ctx, int ncell, const int* celltype, int nlat0, const double* x);
rbc3d_status rbc3d_set_cell_density_x(rbc3d_ctx* ctx, int nlat0, const double* f, const double* g);
rbc3d_status rbc3d_set_walls(rbc3d_ctx* ctx, int nvert, int nele,
                             const double* x, const int* e2v,
                             const int* indxVertGlb);
rbc3d_status rbc3d_set_wall_density(rbc3d_ctx* ctx, const double* f);
rbc3d_status rbc3d_get_wall_density(rbc3d_ctx* ctx, double* f);
/* TargetList_CreateFromRaw (ModTargetList.F90:137). */
rbc3d_status rbc3d_set_raw_targets(rbc3d_ctx* ctx, int n, const double* x);
int rbc3d_num_targets(const rbc3d_ctx* ctx, int tlist);

/* ---- L2 operators (accumulate into v) -------------------------------- */
/* AddIntOnRbcs(c1,c2,tlist,v), ModIntOnRbcs.F90:25: real-space pair sums with
 * the same-cell mask, RBC_SingInt, RBC_NearSingInt per neighbour cell and
 * AddLinearInt. */
rbc3d_status rbc3d_add_int_on_rbcs(rbc3d_ctx* ctx, int tlist, double c1,
                                   double c2, int prec, double* v);
/* AddIntOnWalls(c1,tlist,v), ModIntOnWalls.F90:37 (self wall via the sparse
 * operator of rbc3d_prepare_sing_int_on_wall for wall targets). */
rbc3d_status rbc3d_add_int_on_walls(rbc3d_ctx* ctx, int tlist, double c1,
                                    int prec, double* v);
/* PrepareSingIntOnWall(wall), ModIntOnWalls.F90:181: assembles the self-wall
 * 3nvert x 3nvert operator once (CSR, FP64). */
rbc3d_status rbc3d_prepare_sing_int_on_wall(rbc3d_ctx* ctx);
/* PME_Distrib_Source(c1,c2,cells,walls), ModPME.F90:58 */
rbc3d_status rbc3d_pme_distrib_source(rbc3d_ctx* ctx, double c1, double c2,
                                      int cells, int walls, int prec);
/* PME_Transform, ModPME.F90:137 */
rbc3d_status rbc3d_pme_transform(rbc3d_ctx* ctx);
/* PME_Add_Interp_Vel(tlist,v), ModPME.F90:228 */
rbc3d_status rbc3d_pme_add_interp_vel(rbc3d_ctx* ctx, int tlist, double* v);

/* Composite matvec, all terms on the device with one download: the sum that
 * Compute_Rhs / CalcVelocityField / Compute_Wall_Residual_Vel assemble from
 * the L2 calls above (ModVelSolver.F90:476-490, ModPostProcess.F90:39-51,
 * ModNoSlip.F90:175-184), without background velocity.  v += result; with
 * v == NULL the result stays in device memory (no transfer). */
rbc3d_status rbc3d_matvec(rbc3d_ctx* ctx, int tlist, double c1, double c2,
                          unsigned terms, int prec, double* v);

/* ---- L3 drivers ------------------------------------------------------- */
/* Compute_Wall_Residual_Vel(v), ModNoSlip.F90:153.  Overwrites v (nvert x 3). */
rbc3d_status rbc3d_compute_wall_residual_vel(rbc3d_ctx* ctx, int prec,
                                             double* v);
/* NoSlipWall, ModNoSlip.F90:45: GMRES on the wall-density increment (PCNONE),
 * wall f <- f0 + finc.  guess: NULL or a dof-length (3*unique vertices,
 * xyz-interleaved per unique vertex as AssembleArray) initial increment
 * (two of them back to back for guess mode 3). */
rbc3d_status rbc3d_no_slip_wall(rbc3d_ctx* ctx, const rbc3d_solve_opts* opt,
                                const double* guess, rbc3d_solve_stats* st);
/* Solve_RBC_Vel, ModVelSolver.F90:44-132 (Deflate off): GMRES (FP64 matvec
 * and Arnoldi, opt->prec ignored) on the spherical-harmonic coefficients of
 * the cell surface velocities, degree < nlat0 (the layout of Glob_Sph_Trans,
 * ModVelSolver.F90:641-719: per cell a(m,n) for m < nlat0, n >= m, then
 * b(m,n) for 1 <= m < nlat0, three components each; rbc3d_cell_dof values).
 * The right-hand side is Compute_Rhs (single layer of cells and walls, PME,
 * 2 vBkg/Acoef), the operator MyMatMult (g from the coefficients, its spline
 * rebuilt as Rbc_BuildSurfaceSource, double layer with c2 = -1/(4 pi), plus
 * g).  sol: NULL, or the solution vector, used as the initial guess when
 * opt->guess != 0 (KSPSetInitialGuessNonzero) and overwritten with the
 * solution.  v: surface velocities (npt x 3) out.  With every viscRat = 1
 * the solution is the right-hand side (no GMRES).  Needs even nlon and
 * 2 (nlat0 - 1) < nlon.  The cells' g (and its spline) are left at the
 * solution. */
rbc3d_status rbc3d_solve_rbc_vel(rbc3d_ctx* ctx, const rbc3d_solve_opts* opt,
                                 int nlat0, double* sol, double* v,
                                 rbc3d_solve_stats* st);
/* Length of the coefficient vector of rbc3d_solve_rbc_vel: 3 nlat0^2 ncell. */
int rbc3d_cell_dof(const rbc3d_ctx* ctx, int nlat0);

/* ---- membrane mechanics (FP64) ------------------------------------------
 * Positions are on the cell grid of rbc3d_set_cell_grid, SoA 3 x (ncell nlat
 * nlon), point index cell*nlat*nlon + ilon*nlat + ilat.  Surface derivatives
 * are those of the degree < nlat spherical-harmonic expansion on the Gauss
 * grid (ShAnalGau + ShGradGau, ModSphpk.F90:74-105, 377-417). */

/* Reference cells (rbcRefs), one per cell type: their positions xref
 * (3 x ntypes nlat nlon) and the moduli of Shell_ElasStrs / Shell_Bend
 * (ES shear, ED area dilation, EB bending; t_rbc%ES/ED/EB).  Replaces the
 * reference-cell set-up of the drivers (RBC_Create + RBC_ComputeGeometry on
 * rbcRefs, e.g. examples/case/tube.F90). */
rbc3d_status rbc3d_set_ref_cells(rbc3d_ctx* ctx, int ntypes, const double* xref,
                                 const double* ES, const double* ED, const double* EB);

/* RBC_ComputeGeometry (ModRbc.F90:404-509) of ncell cells at positions x:
 * unit normals a3 (3 x N), detJ = |x_th x x_phi| / sin(th) (N), area and
 * volume per cell; any output may be NULL. */
rbc3d_status rbc3d_cell_geometry(rbc3d_ctx* ctx, int ncell, const double* x, double* a3,
                                 double* detJ, double* area, double* vol);

/* Shell_ResForce (ModRbc.F90:815-899) of every cell at positions x against
 * the reference cell of its type: f (3 x N, Cartesian), the residual force
 * whose negative Compute_Rbc_Vel (ModTimeInt.F90:747-752) takes as traction. */
rbc3d_status rbc3d_shell_res_force(rbc3d_ctx* ctx, int ncell, const int* celltype,
                                   const double* x, double* f);

/* AddIntraCellRepulsionForce (ModRepulsion.F90:126-266): for every point of a
 * cell, the nearest point of the same cell that is farther than the polar
 * patch radius on the reference sphere, closer than epsDist = 2 sqrt(area) /
 * nlat, and seen against its outward normal (cosine >= 0.707); if one exists
 * at distance d, f += force_coef exp(1 - d / epsDist) a3 at that point.
 * x, a3, f: 3 x N; area per cell; count (may be NULL): points pushed. */
rbc3d_status rbc3d_intra_cell_repulsion(rbc3d_ctx* ctx, int ncell, const double* x,
                                        const double* a3, const double* area,
                                        double force_coef, double* f, int* count);
/* InterCellRepulsion (ModRepulsion.F90:270-402) with Closest_Neighbor_Cell and
 * Closest_Neighbor_Wall (:480-613), one rank: every point of the context's
 * cells finds the nearest point of another cell (over the 27 hash cells
 * around it; projected onto that cell's spline surface, Spline_FindProjection,
 * when within 2 epsDist) and the nearest point of the wall's triangles
 * (MinDistToTri); closer than epsDist it moves by 0.5 xx (epsDist - rr) / rr,
 * xx its separation.  Cells whose type has |viscRat| < viscRatThresh move
 * point by point; with rigidsep the others move rigidly by the mean move of
 * their moved points.  x (3 x N, out): the moved positions (the context keeps
 * the old ones until the next rbc3d_set_cells); distMin: the minimum surface
 * separation found; nmoved: points moved (both may be NULL). */
rbc3d_status rbc3d_inter_cell_repulsion(rbc3d_ctx* ctx, double epsDist, double viscRatThresh, int rigidsep,
                                        double* x, double* distMin, int* nmoved);
/* MyMatMult of ModNoSlip.F90:255 on a dof-length vector: y = A u. */
rbc3d_status rbc3d_wall_matmult(rbc3d_ctx* ctx, int prec, const double* u,
                                double* y);
/* CalcVelocityField(tlist,v), ModPostProcess.F90:29.  Overwrites v. */
rbc3d_status rbc3d_calc_velocity_field(rbc3d_ctx* ctx, int tlist, int prec,
                                       double* v);

rbc3d_status rbc3d_get_counts(const rbc3d_ctx* ctx, rbc3d_counts* out);

/* ---- learned wall-density initial guess (no counterpart in the reference) --
 * A per-vertex MLP: nin -> width (SiLU) x depth -> nout.  GEMMs run on the
 * tensor cores with BF16 operands and FP32 accumulation (tcgen05.mma with
 * TMEM accumulators);
 * master weights, Adam moments and the loss are FP32.  Row-major FP32 host
 * arrays.  Parameters are packed [W_0 (dout x din), b_0, W_1, b_1, ...]. */
typedef struct rbc3d_mlp rbc3d_mlp;
rbc3d_status rbc3d_mlp_create(int nin, int width, int depth, int nout, unsigned long long seed, rbc3d_mlp** out);
rbc3d_status rbc3d_mlp_destroy(rbc3d_mlp* m);
long long rbc3d_mlp_num_params(const rbc3d_mlp* m);
rbc3d_status rbc3d_mlp_params(rbc3d_mlp* m, float* host, int get);
rbc3d_status rbc3d_mlp_forward(rbc3d_mlp* m, int n, const float* x, float* y);
/* Mean-squared-error loss and packed FP32 gradients of the batch (x, t). */
rbc3d_status rbc3d_mlp_gradients(rbc3d_mlp* m, int n, const float* x, const float* t, float* grads, float* loss);
/* One Adam step (beta1 0.9, beta2 0.999, eps 1e-8) on the batch; loss before the step. */
rbc3d_status rbc3d_mlp_train_step(rbc3d_mlp* m, int n, const float* x, const float* t, float lr, float* loss);
/* Right-hand side of the wall solve, b = -AssembleArray(Compute_Wall_Residual_Vel)
 * (ModNoSlip.F90:110-113) for the current wall density: ndof values. */
rbc3d_status rbc3d_wall_rhs(rbc3d_ctx* ctx, int prec, double* b);

/* Learned spectral operator of the wall solve (no counterpart in the
 * reference, whose NoSlipWall starts from a zero increment).  For a wall that
 * is a uniform stack of nring rings along the periodic z axis (unique vertex
 * g = ring * nper + i, every element shifted by one ring again an element),
 * the wall operator is block diagonal in the axial Fourier modes; the model
 * learns each mode's block from the solved pairs of the run: per mode an
 * orthonormal basis of the transformed right-hand sides and the matching
 * solutions, grown by Gram-Schmidt while a pair's new direction exceeds tau
 * times the mode's norm (tau 1e-7 works).  The prediction for b is the
 * least-squares fit of its solution on the pairs seen, mode by mode.
 * init: checks the mesh (RBC3D_ERR_ARG if it is not such a stack), resets
 * the model; record != 0 makes every converged rbc3d_no_slip_wall teach the
 * model the pair (b - r, x), r the true residual it stopped at (= A x).
 * The wall's next rbc3d_set_walls discards the model.
 * add: the pair (A x, x) for a solved increment x (ndof values, the layout of
 * rbc3d_wall_rhs; A x is formed with the FP64 wall operator, so the pair is
 * exact whatever the tolerance x was solved to); *added (may be NULL) = the
 * number of modes whose basis grew.
 * predict: x0 (ndof) for the right-hand side b, and rem (ndof, may be NULL)
 * the part of b outside the learned span.
 * size: modes, basis size per mode (nmodes ints, may be NULL), pairs seen. */
rbc3d_status rbc3d_wall_spectral_init(rbc3d_ctx* ctx, int nring, double tau, int record);
rbc3d_status rbc3d_wall_spectral_add(rbc3d_ctx* ctx, const double* x, int* added);
rbc3d_status rbc3d_wall_spectral_predict(rbc3d_ctx* ctx, const double* b, double* x0, double* rem);
rbc3d_status rbc3d_wall_spectral_size(rbc3d_ctx* ctx, int* nmodes, int* nbasis, long long* pairs);

/* MinDistToTri(xTar, x, s0, t0, x0), ModIntOnWalls.F90:480 (host code, no
 * context): distance from xtar to the triangle x(3,3) (column-major, x(l,:)
 * vertex l), the barycentric (s0, t0) of the closest point and the point x0.
 * For host callers of the reference's repulsion routines
 * (ModRepulsion.F90:600) once ModIntOnWalls is replaced; outputs may be NULL. */
rbc3d_status rbc3d_min_dist_to_tri(const double xtar[3], const double x[9], double* s0, double* t0,
                                   double x0[3], double* dist);

/* Allocation-free linear double-layer term.  No counterpart in the reference:
 * it serves callers that cannot allocate device memory -- programs whose
 * device arrays belong to another owner (OpenACC / CUDA Fortran data regions,
 * an application memory pool) or loops in which a cudaMalloc would
 * synchronise the device.  It computes the AddLinearInt term
 * (v += c2 * xvint / Acoef for nt targets) from caller-owned DEVICE arrays
 * laid out as the rest of this ABI (x, g, a3: 3N; detJ: N; w: nlat;
 * celltype: ncell; Acoef: nt; v: 3 nt), enqueued on `stream` (a
 * cudaStream_t, NULL for the default stream).  It allocates nothing: its
 * per-cell scratch is a fixed array inside the library, so ncell is limited
 * to 8192 (larger values, or nlat*nlon*ncell above INT_MAX, return
 * RBC3D_ERR_ARG).  Every call looks up that array's device address on the
 * current device (the first lookup on a device loads the library's device
 * code); make the first call before any stream capture.  The array is shared
 * by every call: calls that overlap on the GPU race.  Cell types are read on
 * the device: a cell whose type lies outside [0, ncelltypes) contributes
 * nothing.  ncell == 0, nt == 0 or c2 == 0 return RBC3D_OK without touching
 * v. */
rbc3d_status rbc3d_add_linear_int_noalloc(int ncell, int nlat, int nlon, const double* x, const double* g,
                                          const double* a3, const double* detJ, const double* w,
                                          const int* celltype, int ncelltypes, const double* viscRat,
                                          const double Lb[3], double c2, int nt, const double* Acoef, double* v,
                                          void* stream);

/* ---- device timing (replaces the per-step MPI_WTime print of TimeInt_*,
 * ModTimeInt.F90:119,166-174, with CUDA events on the context stream) ---- */
#define RBC3D_NSTAGE 8
/* Stages: 0 pair sums, 1 self patch, 2 near-singular, 3 linear term,
 * 4 wall quadrature / self-wall SpMV, 5 PME spread, 6 PME FFT + influence,
 * 7 PME gather. */
rbc3d_status rbc3d_set_profiling(rbc3d_ctx* ctx, int on);
/* Sum of the device time per stage (ms) since the last call, and the number of
 * recorded executions per stage; resets the record. */
rbc3d_status rbc3d_stage_times(rbc3d_ctx* ctx, double ms[RBC3D_NSTAGE], int count[RBC3D_NSTAGE]);
/* Event pair on the context stream around any sequence of calls. */
rbc3d_status rbc3d_timer_start(rbc3d_ctx* ctx);
rbc3d_status rbc3d_timer_stop(rbc3d_ctx* ctx, double* ms);

/* Page-locked host buffers for the caller's staging arrays (faster uploads). */
rbc3d_status rbc3d_host_alloc(unsigned long long bytes, void** out);
rbc3d_status rbc3d_host_free(void* p);
/* Measured FMA throughput of this GPU (TFLOP/s, 2 flops per FMA) for FP32
 * (prec = RBC3D_FP32C) or FP64 (RBC3D_FP64): a register-resident FMA chain
 * over all SMs, used as the roofline of the CUDA-core-bound kernels. */
rbc3d_status rbc3d_fma_peak(int prec, double* tflops);
/* Measured host-to-device copy bandwidth (GB/s) of this GPU from page-locked
 * memory: one copy of `bytes` timed with CUDA events (best of 3 after a
 * warm-up); the floor of the uploads an end-to-end step makes. */
rbc3d_status rbc3d_h2d_bandwidth(unsigned long long bytes, double* gbs);

#ifdef __cplusplus
}
#endif
#endif /* RBC3D_GPU_H */
