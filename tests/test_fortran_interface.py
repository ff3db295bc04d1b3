"""The Fortran host side (mom5_gb300/fortran/mom5gpu_mod.F90) cannot be compiled
here (no Fortran compiler on either machine), so its ISO_C_BINDING interfaces
are checked against the C ABI by reading both: every bind(C) name is declared
in include/mom5gpu.h and exported by the library, with the same number of
arguments, and each argument passed by value in Fortran is a scalar in C and
each one passed by reference is a pointer."""
import os
import re

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
F90 = os.path.join(HERE, "..", "mom5_gb300", "fortran", "mom5gpu_mod.F90")
HDR = os.path.join(HERE, "..", "include", "mom5gpu.h")


def fortran_interfaces():
    src = open(F90).read()
    body = src[src.index("interface"):src.index("end interface")]
    out = {}
    pat = re.compile(r"(?:integer\(c_int\)\s+function|type\(c_ptr\)\s+function|subroutine)\s+(\w+)\s*\(([^)]*)\)"
                     r"\s*&?\s*bind\(C,\s*name=\"(\w+)\"\)(.*?)end (?:function|subroutine)", re.S)
    for m in pat.finditer(body):
        args = [a.strip() for a in m.group(2).replace("&", " ").split(",") if a.strip()]
        decls = m.group(4)
        by_value = {}
        for a in args:
            d = re.search(r"^[^!\n]*::[^!\n]*\b%s\b[^!\n]*$" % re.escape(a), decls, re.M)
            assert d, f"{m.group(3)}: no declaration of {a}"
            by_value[a] = "value" in d.group(0).split("::")[0]
        out[m.group(3)] = [by_value[a] for a in args]
    return out


def c_prototypes():
    src = re.sub(r"/\*.*?\*/", "", open(HDR).read(), flags=re.S)
    out = {}
    for m in re.finditer(r"^\s*[\w\s\*]*?\b(mom5gpu_\w+)\s*\(([^;{]*?)\)\s*;", src, re.M | re.S):
        params = [p.strip() for p in m.group(2).split(",") if p.strip() and p.strip() != "void"]
        out[m.group(1)] = [("*" in p) or ("[" in p) for p in params]
    return out


def test_every_fortran_binding_matches_the_header():
    fi, cp = fortran_interfaces(), c_prototypes()
    assert len(fi) >= 30
    for name, by_value in fi.items():
        assert name in cp, f"{name} is bound in Fortran but not declared in the header"
        ptrs = cp[name]
        assert len(ptrs) == len(by_value), f"{name}: {len(by_value)} Fortran arguments, {len(ptrs)} in C"
        for i, (v, p) in enumerate(zip(by_value, ptrs)):
            # a c_ptr passed by value is a pointer in C (the domain handle, a host buffer)
            if v and p:
                continue
            assert (not v) == p, f"{name} argument {i + 1}: Fortran {'value' if v else 'reference'}, C {'pointer' if p else 'scalar'}"


def test_every_fortran_binding_is_exported():
    from mom5_gb300 import build, capi
    build.build()
    lib = capi.lib()
    for name in fortran_interfaces():
        assert hasattr(lib, name), name
