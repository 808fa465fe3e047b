"""Generate the committed golden fixture of a small seeded workload.

Inputs: 3 biconcave cells (25x50 grid) in a periodic cube L = 12, SL + DL
densities (viscRat 5), alpha for rc = 3, PME 32^3, P = 6.  Output: the FP64
oracle velocity of AddIntOnRbcs + PME (c1 = c2 = 1/(4 pi)) at every cell
point, plus the counts.  Run from the repository root:

    python tests/golden/make_golden.py
"""
import math
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from rbc3d_gb300 import geometry as G  # noqa: E402
from rbc3d_gb300.abi import Context, Library, TLIST_RBC, TERM_ALL  # noqa: E402

SEED = 7


def workload():
    rng = np.random.default_rng(SEED)
    L = 12.0
    cells = G.make_cells(rng, 3, [L] * 3, 2.7, with_g=True)
    prm = dict(Lb=[L] * 3, alpha=G.alpha_for_cutoff(3.0, 1e-6), rc=3.0, eps=1e-6, Nb=[32] * 3, P=6, nlat=25, nlon=50,
               ncelltypes=1, viscRat=[5.0], vBkg=[0, 0, 0])
    return prm, cells


def workload_near():
    """Two cells side by side with a 0.13 gap at the rims, viscRat 5, and raw
    targets 0.003 and 0.05 off one surface on both sides."""
    rng = np.random.default_rng(SEED + 1)
    L = 12.0
    centres = np.array([[4.5, 6.0, 6.0], [4.5 + 2.9, 6.0, 6.0]])
    cells = G.make_cells(rng, 2, [L] * 3, 2.0, with_g=True, centres=centres, rotations=[np.eye(3), np.eye(3)])
    prm = dict(Lb=[L] * 3, alpha=G.alpha_for_cutoff(3.0, 1e-6), rc=3.0, eps=1e-6, Nb=[32] * 3, P=6, nlat=25, nlon=50,
               ncelltypes=1, viscRat=[5.0], vBkg=[0, 0, 0])
    pick = np.array([0, 137, 612, 640, 1001])  # points of cell 0
    raw = []
    for d in (0.003, -0.003, 0.05, -0.05):
        raw.append(cells.x[:, pick] + d * cells.a3[:, pick])
    raw = np.ascontiguousarray(np.concatenate(raw, axis=1))
    return prm, cells, raw


def main():
    import subprocess
    subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "-s"], check=True)
    lib = Library(os.path.join(ROOT, "oracle", "liboracle_rbc3d.so"), "rbc3d_oracle_")
    prm, cells = workload()
    ctx = Context(lib, prm)
    ctx.set_cells(cells)
    ctx.set_cell_density(f=cells.f, g=cells.g, spl_F=cells.spl_F, spl_G=cells.spl_G)
    c = 1 / (4 * math.pi)
    v = ctx.matvec(TLIST_RBC, c, c, TERM_ALL)
    cnt = ctx.counts()
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden_3cells_sldl.npz")
    np.savez_compressed(out, v=v, x=cells.x, f=cells.f, g=cells.g, pairs=cnt["pairs_within_rc"],
                        nbr=cnt["nbr_items"], near=cnt["nearsing_items"])
    print(out, v.shape, cnt)
    prm, cells, raw = workload_near()
    ctx = Context(lib, prm)
    ctx.set_cells(cells)
    ctx.set_cell_density(f=cells.f, g=cells.g, spl_F=cells.spl_F, spl_G=cells.spl_G)
    ctx.set_raw_targets(raw)
    v = ctx.matvec(TLIST_RBC, c, c, TERM_ALL)
    cnt = ctx.counts()
    from rbc3d_gb300.abi import TLIST_RAW
    vr = ctx.matvec(TLIST_RAW, c, c, TERM_ALL)
    cntr = ctx.counts()
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden_near_2cells.npz")
    np.savez_compressed(out, v=v, vraw=vr, raw=raw, near=cnt["nearsing_items"], near_raw=cntr["nearsing_items"],
                        nbr=cnt["nbr_items"], pairs=cnt["pairs_within_rc"])
    print(out, cnt["nearsing_items"], cntr["nearsing_items"])


if __name__ == "__main__":
    main()
