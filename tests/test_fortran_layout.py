"""The Fortran binding (fortran/ModRbc3dGpu.F90) against the C header.

No Fortran compiler is needed: the bind(C) derived types are laid out here
with the C interoperability rules (each component at the next multiple of
its alignment, the size rounded up to the largest alignment) and compared
with sizeof / offsetof of the C structs, printed by a small C program that
gcc compiles against include/rbc3d_gpu.h.  Every interface body is checked
against the header's prototype: the bound name exists, the argument count
matches, and each argument is passed by value exactly where C takes a
scalar (an address where C takes a pointer or an array)."""
import os
import re
import shutil
import subprocess

import pytest

from conftest import ROOT

F90 = os.path.join(ROOT, "fortran", "ModRbc3dGpu.F90")
HDR = os.path.join(ROOT, "include", "rbc3d_gpu.h")
KINDS = {"real(c_double)": (8, 8), "integer(c_int)": (4, 4), "integer(c_long_long)": (8, 8)}
STRUCTS = ["rbc3d_params", "rbc3d_counts", "rbc3d_solve_opts", "rbc3d_solve_stats"]


def fortran_source():
    src = open(F90).read()
    src = re.sub(r"!.*", "", src)                 # comments
    return re.sub(r"&\s*\n\s*", " ", src)         # continuation lines


def parameters(src):
    return {m.group(1).lower(): int(m.group(2))
            for m in re.finditer(r"\b(\w+)\s*=\s*(\d+)\b", src)}


def fortran_types(src):
    params = parameters(src)
    out = {}
    for m in re.finditer(r"type\s*,\s*bind\s*\(\s*C\s*\)\s*::\s*(\w+)(.*?)end\s+type", src, re.S | re.I):
        name, body = m.group(1).lower(), m.group(2)
        fields = []
        for line in body.splitlines():
            d = re.match(r"\s*(real\(c_double\)|integer\(c_int\)|integer\(c_long_long\))\s*::\s*(.+)", line, re.I)
            if not d:
                continue
            size, align = KINDS[d.group(1).lower()]
            for ent in re.findall(r"(\w+)\s*(?:\(([^)]*)\))?", d.group(2)):
                n = 1
                if ent[1]:
                    dim = ent[1].strip().lower()
                    n = int(dim) if dim.isdigit() else params[dim]
                fields.append((ent[0].lower(), size, align, n))
        off, amax, lay = 0, 1, {}
        for fname, size, align, n in fields:
            off = (off + align - 1) // align * align
            lay[fname] = (off, size * n)
            off += size * n
            amax = max(amax, align)
        out[name] = (lay, (off + amax - 1) // amax * amax)
    return out


def c_layouts(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    hdr = open(HDR).read()
    lines = ['#include <stdio.h>', '#include <stddef.h>', f'#include "{HDR}"', "int main(void) {"]
    for s in STRUCTS:
        body = re.search(r"typedef struct " + s + r"\s*\{(.*?)\}\s*" + s + ";", hdr, re.S).group(1)
        body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
        lines.append(f'  printf("{s} size %zu\\n", sizeof({s}));')
        for decl in body.split(";"):
            for name in re.findall(r"(\w+)\s*(?:\[[^\]]*\])?\s*(?:,|$)", decl.strip()):
                if name in ("double", "int", "long", "unsigned"):
                    continue
                lines.append(f'  printf("{s} {name} %zu %zu\\n", offsetof({s}, {name}), '
                             f'sizeof((({s}*)0)->{name}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    exe = tmp_path / "layout"
    src.write_text("\n".join(lines))
    subprocess.run([cc, "-std=c99", "-o", str(exe), str(src)], check=True)
    out = {}
    for row in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.splitlines():
        p = row.split()
        if p[1] == "size":
            out.setdefault(p[0], [{}, 0])[1] = int(p[2])
        else:
            out.setdefault(p[0], [{}, 0])[0][p[1].lower()] = (int(p[2]), int(p[3]))
    return out


def test_bind_c_types_match_the_c_structs(tmp_path):
    f = fortran_types(fortran_source())
    c = c_layouts(tmp_path)
    for s in STRUCTS:
        assert s in f, s
        flay, fsize = f[s]
        clay, csize = c[s]
        assert fsize == csize, (s, fsize, csize)
        assert flay == clay, (s, flay, clay)


def c_prototypes():
    h = re.sub(r"/\*.*?\*/", "", open(HDR).read(), flags=re.S)
    out = {}
    for m in re.finditer(r"\b(?:rbc3d_status|int|const char\*)\s+(rbc3d_\w+)\s*\(([^)]*)\)\s*;", h):
        args = [a.strip() for a in m.group(2).split(",") if a.strip() and a.strip() != "void"]
        out[m.group(1)] = ["addr" if ("*" in a or "[" in a) else "value" for a in args]
    return out


def fortran_interfaces(src):
    out = {}
    block = re.search(r"\binterface\b(.*?)\bend\s+interface\b", src, re.S | re.I).group(1)
    for m in re.finditer(r"function\s+(\w+)\s*\(([^)]*)\)\s*bind\s*\(\s*C\s*,\s*name\s*=\s*\"(\w+)\"\s*\)(.*?)end\s+function",
                         block, re.S | re.I):
        dummies = [a.strip().lower() for a in m.group(2).split(",") if a.strip()]
        attrs = {}
        for line in m.group(4).splitlines():
            d = re.match(r"\s*([^:]+)::\s*(.+)", line)
            if not d:
                continue
            spec = d.group(1).lower().replace(" ", "")
            names = [n.lower() for n in re.findall(r"(\w+)\s*(?:\([^)]*\))?", d.group(2))]
            for n in names:
                by_value = "value" in spec.split(",") and not spec.startswith("type(c_ptr)")
                attrs[n] = "value" if by_value else "addr"
        out[m.group(3)] = [attrs.get(dm) for dm in dummies]
    return out


def test_interface_bodies_match_the_prototypes():
    c = c_prototypes()
    f = fortran_interfaces(fortran_source())
    assert len(f) >= 30
    for name, kinds in f.items():
        assert name in c, name
        assert kinds == c[name], (name, kinds, c[name])
    # the module binds every entry point of the drop-in surface
    for name in ("rbc3d_create", "rbc3d_add_int_on_rbcs", "rbc3d_add_int_on_walls", "rbc3d_pme_distrib_source",
                 "rbc3d_pme_transform", "rbc3d_pme_add_interp_vel", "rbc3d_no_slip_wall", "rbc3d_solve_rbc_vel",
                 "rbc3d_compute_wall_residual_vel", "rbc3d_prepare_sing_int_on_wall"):
        assert name in f, name
