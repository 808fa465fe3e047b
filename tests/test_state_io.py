"""Restart files (WriteRestart / ReadRestart, ModIO.F90:742-921) and Exodus
Tri3 wall meshes (ReadWallMesh, ModIO.F90:547-605; Wall_Build_V2V,
ModWall.F90:65-114)."""
import os
import struct

import numpy as np
import pytest

from rbc3d_gb300 import geometry as G
from rbc3d_gb300 import state_io as S


def test_restart_round_trip_and_record_layout(tmp_path):
    prm, cells, wall = G.config("C3", ncell=3)
    r = S.Restart(Lb=np.array(prm["Lb"]), lt=120, time=0.12, vBkg=np.array(prm["vBkg"]),
                  cells=S.cells_to_restart(cells, 12),
                  walls=[S.RestartWall(wall.x.T.copy(), np.sin(wall.x.T), wall.e2v.T.copy())])
    p = tmp_path / "restart.dat"
    S.write_restart(p, r)
    raw = p.read_bytes()
    # first record: Lb(3) as 24 bytes framed by 4-byte length markers
    assert struct.unpack("<i", raw[:4])[0] == 24 and struct.unpack("<i", raw[28:32])[0] == 24
    assert np.array_equal(np.frombuffer(raw[4:28], "<f8"), r.Lb)
    # the first cell's positions: Fortran order x(nlat, nlon, 3)
    q = S.read_restart(p)
    assert q.lt == 120 and q.time == 0.12 and np.array_equal(q.Lb, r.Lb) and np.array_equal(q.vBkg, r.vBkg)
    assert len(q.cells) == 3 and len(q.walls) == 1
    for a, b in zip(q.cells, r.cells):
        assert (a.nlat0, a.nlon0, a.nlat, a.nlon, a.celltype) == (12, 24, 25, 50, 1)
        assert np.array_equal(a.x, b.x) and a.starting_area == b.starting_area
    X, ct = S.restart_positions(q)
    assert np.array_equal(X, cells.x) and np.array_equal(ct, cells.celltype)
    w = q.walls[0]
    assert np.array_equal(w.x, wall.x.T) and np.array_equal(w.e2v, wall.e2v.T) and np.array_equal(w.f, np.sin(wall.x.T))
    # a truncated file is an error, not a short read
    (tmp_path / "cut.dat").write_bytes(raw[:-10])
    with pytest.raises(EOFError):
        S.read_restart(tmp_path / "cut.dat")


def test_wall_mesh_round_trip_and_periodic_vertices(tmp_path):
    wall = G.make_tube(8.0, 48.0, 48, 192, (8.25, 8.25))
    p = tmp_path / "tube.e"
    S.write_wall_mesh(p, wall.x.T, wall.e2v.T)
    x, e2v = S.read_wall_mesh(p)
    assert np.array_equal(x, wall.x.T) and np.array_equal(e2v, wall.e2v.T)
    w2 = S.wall_from_mesh(p, [16.5, 16.5, 48.0])
    # Wall_Build_V2V + GlobData_Init reproduce the tube's own unique-vertex ids
    assert np.array_equal(w2.glb, wall.glb) and w2.ndof == wall.ndof


def reference_file(rel):
    """A file of the RBC3D source tree, found under the directory named by the
    environment variable RBC3D_REFERENCE_DIR; the test is skipped without it."""
    root = os.environ.get("RBC3D_REFERENCE_DIR")
    if not root or not os.path.exists(os.path.join(root, rel)):
        pytest.skip(f"RBC3D_REFERENCE_DIR does not hold {rel}")
    return os.path.join(root, rel)


def test_reads_reference_example_mesh():
    x, e2v = S.read_wall_mesh(reference_file("examples/case/Input/new_cyl_D6_L13_33.e"))
    assert x.shape == (1328, 3) and e2v.shape == (2404, 3)
    assert e2v.min() == 1 and e2v.max() == 1328
    # every vertex is used and every triangle has positive area
    assert len(np.unique(e2v)) == 1328
    a = np.cross(x[e2v[:, 1] - 1] - x[e2v[:, 0] - 1], x[e2v[:, 2] - 1] - x[e2v[:, 0] - 1])
    assert np.linalg.norm(a, axis=1).min() > 0


def test_cell_shape_export_import_round_trip(tmp_path):
    from conftest import ROOT
    z = np.load(os.path.join(ROOT, "tests", "golden", "sickle_cell.npz"))
    c = S.CellShape(int(z["nlat0"]), int(z["nlon0"]), int(z["nlat"]), int(z["nlon"]), int(z["celltype"]),
                    np.asarray(z["x"]))
    p = tmp_path / "cell.dat"
    S.export_write_rbc(p, c)
    d = S.import_read_rbc(p, recentre=False)
    assert (d.nlat0, d.nlon0, d.nlat, d.nlon, d.celltype) == (12, 24, 36, 72, 1)
    assert np.array_equal(d.x, c.x)
    e = S.import_read_rbc(p, xc=[1.0, 2.0, 3.0])
    assert np.allclose(e.x, c.x + np.array(S.IMPORT_SHIFT) + [1.0, 2.0, 3.0], rtol=0, atol=1e-14)


def test_sickle_fixture_matches_reference_file():
    from conftest import ROOT
    z = np.load(os.path.join(ROOT, "tests", "golden", "sickle_cell.npz"))
    c = S.import_read_rbc(reference_file("sample_files/sample_cells/SickleCell.dat"))
    assert np.array_equal(c.x, z["x"]) and c.nlat == 36 and c.nlon == 72
