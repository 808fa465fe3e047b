"""The C ABI: every function include/rbc3d_gpu.h declares is exported by the
GPU library (no compute calls: this runs on CPU-only hosts too), and the
oracle exports the same surface under its own prefix."""
import ctypes
import os
import re

from conftest import ROOT


def declared():
    h = open(os.path.join(ROOT, "include", "rbc3d_gpu.h")).read()
    h = re.sub(r"/\*.*?\*/", "", h, flags=re.S)
    return sorted(set(re.findall(r"\b(rbc3d_\w+)\s*\(", h)))


def test_header_declares_entry_points():
    names = declared()
    for n in ("rbc3d_create", "rbc3d_add_int_on_rbcs", "rbc3d_add_int_on_walls", "rbc3d_pme_distrib_source",
              "rbc3d_pme_transform", "rbc3d_pme_add_interp_vel", "rbc3d_no_slip_wall", "rbc3d_matvec"):
        assert n in names


def test_gpu_library_exports_every_symbol():
    from rbc3d_gb300 import build
    path = build.build()
    lib = ctypes.CDLL(path)
    missing = [n for n in declared() if not hasattr(lib, n)]
    assert not missing, missing
    assert lib.rbc3d_abi_version() == 1


def test_oracle_exports_the_shared_surface(oracle):
    from rbc3d_gb300.abi import SIGNATURES
    for name, _, _ in SIGNATURES:
        assert hasattr(oracle.lib, "rbc3d_oracle_" + name), name


def test_product_package_has_no_oracle_path():
    """The product code never loads or references the oracle."""
    pkg = os.path.join(ROOT, "rbc3d_gb300")
    for dirpath, _, files in os.walk(pkg):
        if "_build" in dirpath:
            continue
        for f in files:
            if f.endswith((".py", ".cu", ".cuh", ".hpp")):
                src = open(os.path.join(dirpath, f)).read()
                assert "liboracle" not in src and "oracle/" not in src, f


def test_create_rejects_bad_params():
    """Argument checks happen before any CUDA call."""
    from rbc3d_gb300 import library
    from rbc3d_gb300.abi import Params
    lib = library(build_if_missing=True)
    p = Params()  # all zeros: invalid
    h = ctypes.c_void_p()
    assert lib.fn["create"](ctypes.byref(p), ctypes.byref(h)) == 1


def test_cell_grid_uploaded_once_per_grid(oracle):
    """Context.set_cells calls rbc3d_set_cell_grid (RbcPolarPatch_Create and
    the grid tables) when the grid changes, not on every position update."""
    import numpy as np

    from rbc3d_gb300 import geometry as G
    from rbc3d_gb300.abi import Context
    prm, cells, _ = G.config("C1", ncell=2)
    calls = []
    real = oracle.fn["set_cell_grid"]

    def counting(*args):
        calls.append(1)
        return real(*args)

    oracle.fn["set_cell_grid"] = counting
    try:
        ctx = Context(oracle, prm)
        ctx.set_cells(cells)
        ctx.set_cells(cells)
        assert len(calls) == 1
        # another grid (latitudes moved) goes up again, and the first one after it
        other = type("Cells", (), {k: getattr(cells, k) for k in dir(cells) if not k.startswith("_")})()
        other.th = np.array(cells.th) * (1 - 1e-9)
        ctx.set_cells(other)
        ctx.set_cells(cells)
        assert len(calls) == 3
        # an explicit grid call is remembered
        ctx.set_cell_grid(other.th, cells.phi, cells.w)
        ctx.set_cells(cells)
        assert len(calls) == 5
        ctx.close()
    finally:
        oracle.fn["set_cell_grid"] = real


def test_precision_modes_match_the_header():
    from rbc3d_gb300 import abi
    h = open(os.path.join(ROOT, "include", "rbc3d_gpu.h")).read()
    vals = {k: int(v) for k, v in re.findall(r"\bRBC3D_(FP64|FP32C|FP32M|FP32D)\s*=\s*(\d+)", h)}
    assert vals == {"FP64": abi.FP64, "FP32C": abi.FP32C, "FP32M": abi.FP32M, "FP32D": abi.FP32D}
