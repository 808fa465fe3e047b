"""State formats on either side of the path: RBC3D restart files, exported
cell shapes and Exodus Tri3 wall meshes.

* Restart files (WriteRestart / ReadRestart, ModIO.F90:742-921): Fortran
  sequential unformatted records as gfortran writes them (each record framed
  by a little-endian 4-byte length before and after; on reading, a negative
  leading marker means that sub-records of the same record follow, as
  gfortran splits records longer than 2^31 - 1 bytes).  Record order: Lb(3); lt; time; vBkg(3); nrbc; per cell
  (nlat0, nlon0), (nlat, nlon), celltype, starting_area, x(nlat, nlon, 3);
  nwall; per wall (nvert, nele), x(nvert, 3), f(nvert, 3), e2v(nele, 3).
  Integers are 4-byte, reals 8-byte, arrays in Fortran (column-major) order.
* Wall meshes (ReadWallMesh, ModIO.F90:547-605): Exodus II files (netCDF
  classic) with num_nodes, num_elem, num_nod_per_el1 = 3, coordx/y/z and
  connect1 (1-based), read with scipy's netCDF reader.
* Periodic vertex identification (Wall_Build_V2V, ModWall.F90:65-114) and
  the global vertex numbering of GlobData_Init (ModData.F90:51-62).
"""
from __future__ import annotations

import struct
from dataclasses import dataclass, field

import numpy as np

from . import geometry as G

_MAXREC = 2 ** 31 - 1


def _write_record(fh, payload: bytes):
    n = len(payload)
    if n > _MAXREC:
        raise ValueError("record longer than 2^31 - 1 bytes")
    fh.write(struct.pack("<i", n)); fh.write(payload); fh.write(struct.pack("<i", n))


def _read_record(fh) -> bytes:
    out = bytearray()
    while True:
        hdr = fh.read(4)
        if len(hdr) < 4:
            raise EOFError("restart file ends inside a record")
        n = struct.unpack("<i", hdr)[0]
        data = fh.read(abs(n))
        tail = fh.read(4)
        if len(data) < abs(n) or len(tail) < 4:
            raise EOFError("restart file ends inside a record")
        out += data
        if n >= 0:
            return bytes(out)


def _f(a, dtype):
    return np.asfortranarray(np.asarray(a, dtype=dtype)).tobytes(order="F")


@dataclass
class RestartCell:
    nlat0: int
    nlon0: int
    nlat: int
    nlon: int
    celltype: int          # 1-based, as the reference
    starting_area: float
    x: np.ndarray          # (nlat, nlon, 3)


@dataclass
class RestartWall:
    x: np.ndarray          # (nvert, 3)
    f: np.ndarray          # (nvert, 3)
    e2v: np.ndarray        # (nele, 3), 1-based


@dataclass
class Restart:
    Lb: np.ndarray
    lt: int
    time: float
    vBkg: np.ndarray
    cells: list = field(default_factory=list)
    walls: list = field(default_factory=list)


def write_restart(path, r: Restart):
    """WriteRestart (ModIO.F90:742-784)."""
    with open(path, "wb") as fh:
        _write_record(fh, _f(r.Lb, "<f8"))
        _write_record(fh, struct.pack("<i", int(r.lt)))
        _write_record(fh, struct.pack("<d", float(r.time)))
        _write_record(fh, _f(r.vBkg, "<f8"))
        _write_record(fh, struct.pack("<i", len(r.cells)))
        for c in r.cells:
            _write_record(fh, struct.pack("<ii", c.nlat0, c.nlon0))
            _write_record(fh, struct.pack("<ii", c.nlat, c.nlon))
            _write_record(fh, struct.pack("<i", c.celltype))
            _write_record(fh, struct.pack("<d", float(c.starting_area)))
            _write_record(fh, _f(c.x, "<f8"))
        _write_record(fh, struct.pack("<i", len(r.walls)))
        for w in r.walls:
            _write_record(fh, struct.pack("<ii", w.x.shape[0], w.e2v.shape[0]))
            _write_record(fh, _f(w.x, "<f8"))
            _write_record(fh, _f(w.f, "<f8"))
            _write_record(fh, _f(w.e2v, "<i4"))


def read_restart(path) -> Restart:
    """ReadRestart (ModIO.F90:792-921); sizes are checked against the records."""
    def arr(rec, dtype, shape):
        a = np.frombuffer(rec, dtype=dtype)
        if a.size != int(np.prod(shape)):
            raise ValueError(f"restart record of {a.size} values, expected {shape}")
        return np.array(a.reshape(shape, order="F"))

    with open(path, "rb") as fh:
        Lb = arr(_read_record(fh), "<f8", (3,))
        lt = struct.unpack("<i", _read_record(fh))[0]
        time = struct.unpack("<d", _read_record(fh))[0]
        vBkg = arr(_read_record(fh), "<f8", (3,))
        r = Restart(Lb=Lb, lt=lt, time=time, vBkg=vBkg)
        for _ in range(struct.unpack("<i", _read_record(fh))[0]):
            nlat0, nlon0 = struct.unpack("<ii", _read_record(fh))
            nlat, nlon = struct.unpack("<ii", _read_record(fh))
            celltype = struct.unpack("<i", _read_record(fh))[0]
            sa = struct.unpack("<d", _read_record(fh))[0]
            x = arr(_read_record(fh), "<f8", (nlat, nlon, 3))
            r.cells.append(RestartCell(nlat0, nlon0, nlat, nlon, celltype, sa, x))
        for _ in range(struct.unpack("<i", _read_record(fh))[0]):
            nvert, nele = struct.unpack("<ii", _read_record(fh))
            x = arr(_read_record(fh), "<f8", (nvert, 3))
            f = arr(_read_record(fh), "<f8", (nvert, 3))
            e2v = arr(_read_record(fh), "<i4", (nele, 3))
            r.walls.append(RestartWall(x, f, e2v))
    return r


def cells_to_restart(cells, nlat0, celltype_base=1):
    """RestartCell records of the cells' current positions (SoA point layout)."""
    nv = cells.nlat * cells.nlon
    out = []
    for c in range(cells.ncell):
        xc = cells.x[:, c * nv:(c + 1) * nv].reshape(3, cells.nlon, cells.nlat).transpose(2, 1, 0)
        out.append(RestartCell(nlat0, 2 * nlat0, cells.nlat, cells.nlon, int(cells.celltype[c]) + celltype_base,
                               float(cells.area[c]), np.ascontiguousarray(xc)))
    return out


def restart_positions(r: Restart):
    """Cell positions of a restart in the SoA point layout (3, N) and the
    0-based cell types."""
    if not r.cells:
        return np.zeros((3, 0)), np.zeros(0, dtype=np.int32)
    X = np.stack([c.x for c in r.cells])  # (ncell, nlat, nlon, 3)
    return G._to_points(X), np.array([c.celltype - 1 for c in r.cells], dtype=np.int32)


# ---------------------------------------------------------------------------
# Cell shapes (ExportWriteRBC / ImportReadRBC, ModIO.F90:613-683): list-directed
# text, "nlat0 nlon0", "nlat nlon", "celltype", then x(nlat, nlon, 3) in
# Fortran order.  ImportReadRBC recentres the shape by (-5.25, -5.25, -5/7)
# (the exported cell was offset to fit its box) and optionally adds xc.
IMPORT_SHIFT = (-5.25, -5.25, -5.0 / 7.0)


@dataclass
class CellShape:
    nlat0: int
    nlon0: int
    nlat: int
    nlon: int
    celltype: int          # 1-based
    x: np.ndarray          # (nlat, nlon, 3)


def export_write_rbc(path, c: CellShape):
    """ExportWriteRBC: the header lines and the positions, four values per line."""
    flat = np.asarray(c.x, dtype=np.float64).reshape(-1, order="F")
    with open(path, "w") as fh:
        fh.write(f" {c.nlat0:11d} {c.nlon0:11d}\n {c.nlat:11d} {c.nlon:11d}\n {c.celltype:11d}\n")
        for i in range(0, flat.size, 4):
            fh.write("".join(f" {v:25.17E}" for v in flat[i:i + 4]) + "\n")


def import_read_rbc(path, xc=None, recentre=True) -> CellShape:
    """ImportReadRBC: read a cell shape, recentre it as the reference does,
    shift it by xc."""
    with open(path) as fh:
        tok = fh.read().split()
    nlat0, nlon0, nlat, nlon, celltype = (int(t) for t in tok[:5])
    vals = np.array([float(t.replace("D", "E").replace("d", "e")) for t in tok[5:5 + 3 * nlat * nlon]])
    if vals.size != 3 * nlat * nlon:
        raise ValueError(f"{path}: {vals.size} position values, expected {3 * nlat * nlon}")
    x = vals.reshape((nlat, nlon, 3), order="F").copy()
    if recentre:
        x += np.asarray(IMPORT_SHIFT)
    if xc is not None:
        x += np.asarray(xc, dtype=np.float64)
    return CellShape(nlat0, nlon0, nlat, nlon, celltype, x)


def read_wall_mesh(path):
    """ReadWallMesh: (x (nvert, 3), e2v (nele, 3) 1-based) of a Tri3 Exodus file."""
    from scipy.io import netcdf_file
    with netcdf_file(path, "r", mmap=False) as f:
        if int(f.dimensions.get("num_nod_per_el1", 0)) != 3:
            raise ValueError(f"{path}: the mesh is not of Tri3 type")
        x = np.stack([np.array(f.variables[k][:], dtype=np.float64) for k in ("coordx", "coordy", "coordz")], axis=1)
        e2v = np.array(f.variables["connect1"][:], dtype=np.int32)
    return x, e2v


def write_wall_mesh(path, x, e2v):
    """A minimal Tri3 Exodus II file (netCDF classic) that read_wall_mesh and
    ReadWallMesh accept."""
    from scipy.io import netcdf_file
    x = np.asarray(x, dtype=np.float64)
    e2v = np.asarray(e2v, dtype=np.int32)
    with netcdf_file(path, "w") as f:
        f.createDimension("num_dim", 3)
        f.createDimension("num_nodes", x.shape[0])
        f.createDimension("num_elem", e2v.shape[0])
        f.createDimension("num_el_blk", 1)
        f.createDimension("num_el_in_blk1", e2v.shape[0])
        f.createDimension("num_nod_per_el1", 3)
        for k, name in enumerate(("coordx", "coordy", "coordz")):
            v = f.createVariable(name, "d", ("num_nodes",))
            v[:] = x[:, k]
        c = f.createVariable("connect1", "i", ("num_el_in_blk1", "num_nod_per_el1"))
        c.elem_type = b"TRI3"
        c[:] = e2v


def build_v2v(x, Lb):
    """Wall_Build_V2V: v2v[i] = the 1-based earlier vertex that vertex i
    duplicates across the periodic box, else 0."""
    x = np.asarray(x, dtype=np.float64)
    Lb = np.asarray(Lb, dtype=np.float64)
    eps = Lb.min() * 1e-5
    xmin, xmax = x.min(axis=0), x.max(axis=0)
    bd = [i for i in range(x.shape[0])
          if np.abs(x[i] - xmin).min() < eps or np.abs(x[i] - xmax).min() < eps]
    v2v = np.zeros(x.shape[0], dtype=np.int32)
    for p1 in range(len(bd) - 1):
        i1 = bd[p1]
        if v2v[i1] > 0:
            continue
        d = x[bd[p1 + 1:]] - x[i1]
        q = d / Lb
        d = d - np.sign(q) * np.floor(np.abs(q) + 0.5) * Lb  # Fortran nint: halves away from zero
        hit = np.abs(d).max(axis=1) < eps
        for p2 in np.nonzero(hit)[0]:
            v2v[bd[p1 + 1 + p2]] = i1 + 1
    return v2v


def global_vertex_index(v2v, start=0):
    """indxVertGlb of one wall (GlobData_Init, ModData.F90:51-62): 1-based
    unique ids, duplicates taking their partner's id."""
    glb = np.zeros(len(v2v), dtype=np.int32)
    p = start
    for i, j in enumerate(v2v):
        if j == 0:
            p += 1
            glb[i] = p
        else:
            glb[i] = glb[j - 1]
    return glb


def wall_from_mesh(path, Lb):
    """A geometry.Wall from an Exodus Tri3 mesh in the periodic box Lb."""
    x, e2v = read_wall_mesh(path)
    glb = global_vertex_index(build_v2v(x, Lb))
    return G.Wall(nvert=x.shape[0], nele=e2v.shape[0], x=np.ascontiguousarray(x.T),
                  e2v=np.ascontiguousarray(e2v.T), glb=glb, ndof=3 * int(glb.max()))
