"""The Fortran binding (fortran/swfd_mod.f90) against the C ABI.

No Fortran compiler exists here, so the module is checked as text: every
bind(C) interface must name an entry point of include/swfd.h, every entry
point must have one, and each dummy argument must pass what the C prototype
takes (a scalar by value, a pointer as an array or scalar by reference or as
type(c_ptr) by value, a pointer to a pointer as type(c_ptr) by reference).
The bind(C) derived types must list the fields of the ctypes structures of
the package in order and kind, and the named constants must equal the
package's.
"""
import ctypes as C
import re
from pathlib import Path

import pytest

from sweeping_fd_weno_gb300 import abi

ROOT = Path(__file__).resolve().parents[1]
MOD = ROOT / "fortran" / "swfd_mod.f90"
HEADER = ROOT / "include" / "swfd.h"

C_BASE = {"int32_t": "int32", "swfd_status": "int32", "int64_t": "int64", "double": "double",
          "float": "float", "char": "char", "size_t": "size_t"}
F_KIND = {"integer(c_int32_t)": "int32", "integer(c_int64_t)": "int64",
          "real(c_double)": "double", "real(c_float)": "float", "integer(c_size_t)": "size_t",
          "character(kind=c_char)": "char"}


def strip_comments(text):
    return "\n".join(line.split("!", 1)[0] for line in text.splitlines())


def join_continuations(text):
    return re.sub(r"&\s*\n\s*", " ", text)


def c_prototypes():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    out = {}
    for m in re.finditer(r"^(swfd_status|const char\*)\s+(swfd_\w+)\s*\(([^;]*)\);", text, re.M):
        params = []
        for a in " ".join(m.group(3).split()).split(","):
            a = a.strip().replace("const ", "")
            stars = a.count("*")
            base = a.replace("*", " ").split()[0]
            params.append((C_BASE.get(base, base), stars))
        out[m.group(2)] = (m.group(1), params)
    return out


def f_interfaces():
    text = join_continuations(strip_comments(MOD.read_text()))
    out = {}
    pat = re.compile(r"^\s*(integer\(c_int32_t\)|type\(c_ptr\))\s+function\s+(\w+)\s*\(([^)]*)\)\s*"
                     r"bind\(C,\s*name=\"(\w+)\"\)(.*?)end function", re.S | re.M)
    for m in pat.finditer(text):
        ret, fname, args, cname, body = m.groups()
        assert fname == cname, (fname, cname)
        names = [a.strip() for a in args.split(",") if a.strip()]
        decl = {}
        for line in body.splitlines():
            line = line.strip()
            if "::" not in line or line.startswith("import"):
                continue
            lhs, rhs = (s.strip() for s in line.split("::"))
            attrs = [s.strip() for s in lhs.split(",")]
            for v in (s.strip() for s in rhs.split(",")):
                arr = v.endswith("(*)")
                decl[v.replace("(*)", "")] = (attrs[0], "value" in attrs[1:], arr)
        out[cname] = (ret, [decl[n] for n in names])
    return out


def compatible(f_arg, c_param):
    ftype, by_value, _ = f_arg
    base, stars = c_param
    if ftype == "type(c_ptr)":
        return stars == (1 if by_value else 2)
    if by_value:
        return stars == 0 and F_KIND.get(ftype) == base
    if ftype.startswith("type("):  # a bind(C) derived type by reference
        return stars == 1 and ftype[5:-1] == base
    return stars == 1 and F_KIND.get(ftype) == base


def test_every_entry_point_has_one_interface():
    assert sorted(f_interfaces()) == sorted(c_prototypes())


@pytest.mark.parametrize("name", sorted(c_prototypes()))
def test_interface_arguments_match_the_prototype(name):
    cret, cparams = c_prototypes()[name]
    fret, fargs = f_interfaces()[name]
    assert fret == ("type(c_ptr)" if cret == "const char*" else "integer(c_int32_t)")
    assert len(fargs) == len(cparams), (name, fargs, cparams)
    for k, (fa, cp) in enumerate(zip(fargs, cparams)):
        assert compatible(fa, cp), (name, k, fa, cp)
    # the ctypes prototype of the package takes as many arguments
    assert len(abi._SIGS[name][1]) == len(cparams)


def f_types():
    text = join_continuations(strip_comments(MOD.read_text()))
    out = {}
    for m in re.finditer(r"type,\s*bind\(C\)\s*::\s*(\w+)(.*?)end type", text, re.S):
        fields = []
        for line in m.group(2).splitlines():
            if "::" not in line:
                continue
            kind, var = (s.strip() for s in line.split("::"))
            n = 1
            mm = re.match(r"(\w+)\((\d+)\)", var)
            if mm:
                var, n = mm.group(1), int(mm.group(2))
            fields.append((var, F_KIND[kind], n))
        out[m.group(1)] = fields
    return out


CT = {C.c_int32: "int32", C.c_int64: "int64", C.c_double: "double"}


def ctypes_fields(struct):
    out = []
    for name, t in struct._fields_:
        if issubclass(t, C.Array):
            out.append((name, CT[t._type_], t._length_))
        else:
            out.append((name, CT[t], 1))
    return out


@pytest.mark.parametrize("ftype,struct", [("swfd_config", abi.SwfdConfig),
                                          ("swfd_sweep_stats", abi.SwfdSweepStats),
                                          ("swfd_profile", abi.SwfdProfile),
                                          ("swfd_batch_config", abi.SwfdBatchConfig)])
def test_derived_types_match_the_structs(ftype, struct):
    assert f_types()[ftype] == ctypes_fields(struct)


def test_named_constants_match_the_package():
    text = strip_comments(MOD.read_text())
    consts = {m.group(1): int(m.group(2)) for m in
              re.finditer(r"parameter\s*::\s*(SWFD_\w+)\s*=\s*(-?\d+)", text)}
    expect = {"SWFD_ABI_VERSION": abi.ABI_VERSION, "SWFD_OK": abi.OK}
    for n in dir(abi):
        if n.startswith("ERR_"):
            expect["SWFD_" + n] = getattr(abi, n)
    for n, v in {"MATLAB_1D": abi.MATLAB_1D, "SEDOV_1D": abi.SEDOV_1D, "VORTEX_2D": abi.VORTEX_2D,
                 "SEDOV_2D": abi.SEDOV_2D, "JET_2D": abi.JET_2D,
                 "SHOCK_DIFFRACTION": abi.SHOCK_DIFFRACTION,
                 "DETONATION": abi.DETONATION}.items():
        expect["SWFD_PROBLEM_" + n] = v
    for n in ("LITERALS_DOUBLE", "LITERALS_QUAD", "PRECISION_FP64", "PRECISION_FP32_BULK",
              "UBAR_SEQUENTIAL", "UBAR_TREE", "SWEEP_PARALLEL", "SWEEP_SEQUENTIAL"):
        expect["SWFD_" + n] = getattr(abi, n)
    assert consts == expect
