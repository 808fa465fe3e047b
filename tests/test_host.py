"""Host-side producers and the multi-process plumbing (CPU)."""
import math
import os
import subprocess
import sys

import numpy as np

from conftest import ROOT
from rbc3d_gb300 import geometry as G


def test_gauss_grid_weights():
    th, phi, w = G.gauss_grid(25, 50)
    assert np.all(np.diff(th) > 0) and abs(w.sum() * 50 / (2 * np.pi) - 2.0) < 1e-13


def test_biconcave_geometry():
    rng = np.random.default_rng(0)
    cells = G.make_cells(rng, 2, [12.0] * 3, 3.0)
    # unit normals, outward (x - centre) . n > 0 on average
    n = cells.a3.reshape(3, 2, -1)
    assert np.allclose((n ** 2).sum(0), 1.0)
    # area of the Evans-Fung cell with equivalent radius 1 (about 1.34 x 4 pi)
    assert np.allclose(cells.area, cells.area[0]) and 16.0 < cells.area[0] < 17.5
    # volume by the divergence theorem ~ 4/3 pi (equivalent radius 1)
    nv = 25 * 50
    x = cells.x[:, :nv]
    ds = cells.detJ[:nv] * np.tile(cells.w, 50)
    vol = (x * cells.a3[:, :nv]).sum(0) @ ds / 3
    assert abs(vol - 4 / 3 * math.pi) / (4 / 3 * math.pi) < 0.02


def test_sphere_geometry():
    cells = G.make_sphere_cells(np.zeros((1, 3)), radius=1.0)
    assert abs(cells.area[0] - 4 * np.pi) < 1e-12


def test_tube_mesh():
    w = G.make_tube(8.0, 48.0, 48, 192, (8.25, 8.25))
    assert w.nvert == 48 * 193 and w.nele == 2 * 48 * 192 and w.ndof == 3 * 48 * 192
    assert w.glb.min() == 1 and w.glb.max() == 48 * 192
    # the z = Lz ring maps onto the z = 0 ring
    assert np.all(w.glb[-48:] == w.glb[:48])


def test_ewald_parameters():
    # SetEwaldPrms (ModConf.F90:348-408) at eps = 1e-6 gives s = 4.2361
    assert abs(G.ewald_s(1e-6) - 4.2361) < 1e-3
    assert abs(G.alpha_for_cutoff(3.0, 1e-6) - 1.5757) < 1e-3


def test_replica_max_over_ranks_gloo():
    """bench.py's max-over-ranks reduction with world_size 2 on gloo."""
    code = r'''
import os, sys
sys.path.insert(0, %r)
import torch.distributed as dist
import bench
dist.init_process_group("gloo")
r = dist.get_rank()
m = bench.dist_max(dist, 1.5 + r)
assert m == 2.5, m
bench.barrier(dist)
print("ok", r)
''' % ROOT
    env = dict(os.environ, MASTER_ADDR="127.0.0.1", MASTER_PORT="29577", WORLD_SIZE="2")
    procs = []
    for r in range(2):
        e = dict(env, RANK=str(r), LOCAL_RANK=str(r))
        procs.append(subprocess.Popen([sys.executable, "-c", code], env=e, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = [p.communicate(timeout=120) for p in procs]
    assert all(p.returncode == 0 for p in procs), outs
