"""Golden fixtures (tests/golden/make_golden.py): the oracle reproduces them
on the CPU; the GPU path matches them (FP64 plain form to 1e-10, FP32C to the
1e-6 relative-L2 bar)."""
import math
import os

import numpy as np
import pytest

from conftest import ROOT
from rbc3d_gb300.abi import Context, FP32C, FP32D, FP32M, FP64, TERM_ALL, TLIST_RAW, TLIST_RBC

import importlib.util

_spec = importlib.util.spec_from_file_location("make_golden", os.path.join(ROOT, "tests", "golden", "make_golden.py"))
mg = importlib.util.module_from_spec(_spec)
_spec.loader.exec_module(mg)
C = 1 / (4 * math.pi)


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def _run(lib, prec, near=False):
    if near:
        prm, cells, raw = mg.workload_near()
    else:
        prm, cells = mg.workload()
        raw = None
    ctx = Context(lib, prm)
    ctx.set_cells(cells)
    ctx.set_cell_density(f=cells.f, g=cells.g, spl_F=cells.spl_F, spl_G=cells.spl_G)
    v = ctx.matvec(TLIST_RBC, C, C, TERM_ALL, prec)
    cnt = ctx.counts()
    vr = None
    if raw is not None:
        ctx.set_raw_targets(raw)
        vr = ctx.matvec(TLIST_RAW, C, C, TERM_ALL, prec)
    ctx.close()
    return v, vr, cnt


def test_inputs_reproducible():
    g = np.load(os.path.join(ROOT, "tests", "golden", "golden_3cells_sldl.npz"))
    prm, cells = mg.workload()
    # the same draws; the fields may differ from the fixture by summation-order rounding
    assert np.array_equal(cells.x, g["x"])
    assert np.allclose(cells.f, g["f"], rtol=0, atol=1e-13) and np.allclose(cells.g, g["g"], rtol=0, atol=1e-13)


def test_oracle_reproduces_golden(oracle):
    g = np.load(os.path.join(ROOT, "tests", "golden", "golden_3cells_sldl.npz"))
    v, _, cnt = _run(oracle, FP64)
    assert rel(v, g["v"]) < 1e-12 and cnt["pairs_within_rc"] == int(g["pairs"])
    g2 = np.load(os.path.join(ROOT, "tests", "golden", "golden_near_2cells.npz"))
    v, vr, cnt = _run(oracle, FP64, near=True)
    assert rel(v, g2["v"]) < 1e-12 and rel(vr, g2["vraw"]) < 1e-12
    assert cnt["nearsing_items"] == int(g2["near"]) > 0


@pytest.mark.gpu
@pytest.mark.parametrize("prec,tol", [(FP64, 1e-10), (FP32C, 1e-6), (FP32M, 1e-6), (FP32D, 1e-6)])
def test_gpu_matches_golden(gpu, prec, tol):
    g = np.load(os.path.join(ROOT, "tests", "golden", "golden_3cells_sldl.npz"))
    v, _, cnt = _run(gpu, prec)
    assert rel(v, g["v"]) < tol
    g2 = np.load(os.path.join(ROOT, "tests", "golden", "golden_near_2cells.npz"))
    v, vr, cnt = _run(gpu, prec, near=True)
    assert rel(v, g2["v"]) < tol
    assert rel(vr, g2["vraw"]) < tol
    assert cnt["nearsing_items"] == int(g2["near"])
