"""The C-ABI library loads without a GPU and exports every function that
include/openmhd_gb300.h declares (no compute calls)."""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "openmhd_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:int|void|double|size_t)\s+\**\s*(\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    from openmhd_gb300 import _lib
    from openmhd_gb300.build import build

    build()
    return _lib.load()


def test_header_declares_reference_routines():
    names = declared_functions()
    for ref in ["u2v_", "limiter_", "flux_solver_", "rk_tvd21_", "rk_tvd22_", "rk_std21_", "rk_std22_",
                "glm_ss2_", "set_dt_", "bc_", "flux_resistive_", "set_dt_resistive_"]:
        assert ref in names
    assert len(names) >= 55


def test_every_declared_symbol_is_exported(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_bindings_cover_header():
    from openmhd_gb300 import _lib

    bound = {n for n, _, _ in _lib.SIGNATURES}
    assert set(declared_functions()) <= bound


def test_abi_version_without_gpu(lib):
    assert lib.omhd_abi_version() == 1


def test_product_does_not_reference_oracle():
    """The shipped package never imports or links the CPU oracle."""
    pkg = os.path.join(ROOT, "openmhd_gb300")
    for dirpath, _, files in os.walk(pkg):
        for f in files:
            if f.endswith((".py", ".cu", ".cuh", ".h")):
                src = open(os.path.join(dirpath, f)).read()
                assert "import oracle" not in src and "from oracle" not in src, f
                assert "omhd_oracle" not in src, f


def test_plain_c_program_links_every_symbol(lib, tmp_path):
    """A C99 program that includes the header, takes the address of every
    declared function and calls omhd_abi_version() compiles with -pedantic
    -Werror, links against libopenmhd_gb300.so and runs without a GPU: the
    header is the ABI a Fortran or C driver links to."""
    import subprocess

    names = declared_functions()
    src = tmp_path / "abi.c"
    src.write_text(
        '#include <stdio.h>\n#include "openmhd_gb300.h"\n'
        "typedef void (*fn)(void);\n"
        "static const fn table[] = {\n" + ",\n".join(f"  (fn){n}" for n in names) + "\n};\n"
        "int main(void) {\n"
        '  printf("%d %d\\n", omhd_abi_version(), (int)(sizeof table / sizeof table[0]));\n'
        "  return 0;\n}\n")
    libdir = os.path.join(ROOT, "openmhd_gb300")
    exe = tmp_path / "abi"
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-I", os.path.join(ROOT, "include"),
                    str(src), "-L", libdir, "-lopenmhd_gb300", f"-Wl,-rpath,{libdir}", "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()
    assert out == ["1", str(len(names))]


def _c_prototypes():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    protos = {}
    for ret, name, params in re.findall(r"^\s*(int|void|double|size_t)\s+\**\s*(\w+)\s*\(([^)]*)\)\s*;", text,
                                        flags=re.M | re.S):
        plist = [] if params.strip() in ("", "void") else [p.strip() for p in params.split(",")]
        parsed = []
        for p in plist:
            base = "double" if "double" in p else "int" if re.search(r"\bint\b", p) else "other"
            parsed.append((base, "*" in p or "[" in p))
        protos[name] = (ret, parsed)
    return protos


def test_fortran_module_matches_c_prototypes():
    """include/openmhd_gb300.f90 cannot be compiled here (no Fortran compiler),
    so its bind(C) interfaces are checked against the C header as text: every
    bound name is declared, functions return int and subroutines void, and each
    dummy argument has the C parameter's base type and passing mode (VALUE <->
    by value, arrays and non-VALUE scalars <-> pointers)."""
    src = open(os.path.join(ROOT, "include", "openmhd_gb300.f90")).read()
    protos = _c_prototypes()
    blocks = re.findall(r"^\s*(integer\(c_int\) function|subroutine)\s+\w+\(([^)]*)\)\s*bind\(C,\s*name=\"(\w+)\"\)"
                        r"(.*?)^\s*end (?:function|subroutine)", src, flags=re.M | re.S | re.I)
    assert len(blocks) >= 24
    for kind, args, cname, body in blocks:
        assert cname in protos, cname
        ret, params = protos[cname]
        assert ret == ("int" if kind.startswith("integer") else "void"), cname
        names = [a.strip() for a in args.split(",") if a.strip()]
        assert len(names) == len(params), cname
        decl = {}
        for line in body.splitlines():
            m = re.match(r"\s*(integer\(c_int\)|real\(c_double\))([^:]*)::(.*)", line, flags=re.I)
            if not m:
                continue
            base = "int" if m.group(1).lower().startswith("integer") else "double"
            by_value = "value" in m.group(2).lower()
            for item in re.findall(r"(\w+)(\([^)]*\))?", m.group(3)):
                decl[item[0].lower()] = (base, by_value, bool(item[1]))
        for a, (cbase, cptr) in zip(names, params):
            base, by_value, is_array = decl[a.lower()]
            assert base == cbase, (cname, a)
            assert by_value == (not cptr), (cname, a)
            if is_array:
                assert cptr, (cname, a)


# The reference's subroutine argument lists (2D_basic/u2v.f90, limiter.f90,
# flux_solver.f90, rk.f90, glm_ss2.f90, set_dt.f90, bc.f90;
# 2D_reconnection/flux_resistive.f90), one letter per argument: d = real(8),
# i = integer.
REFERENCE_ARGS = {
    "u2v_": "ddii",              # u2v(U,V,ix,jx)
    "limiter_": "dddiiii",       # limiter(wk,wL,wR,ix,jx,dir,type)
    "flux_solver_": "ddddiiii",  # flux_solver(F,VL,VR,ch,ix,jx,dir,type)
    "rk_tvd21_": "ddddddii",     # rk_tvd21(wk,wk1,wF,wG,dt,dx,ix,jx)
    "rk_tvd22_": "ddddddii",
    "rk_std21_": "ddddddii",
    "rk_std22_": "dddddii",      # rk_std22(wk,wF,wG,dt,dx,ix,jx)
    "glm_ss2_": "dddii",         # glm_ss2(U,ch,dt,ix,jx)
    "set_dt_": "ddddddii",       # set_dt(U,V,vmax,dt,dx,cfl,ix,jx)
    "bc_": "dii",                # bc(U,ix,jx)
    "flux_resistive_": "dddddiii",  # flux_resistive(F,U,x,y,dx,ix,jx,dir)
    "set_dt_resistive_": "ddd",  # set_dt_resistive(dt,dx,cfl)
}


def test_link_level_dropins_take_the_reference_argument_lists():
    """gfortran passes every argument by reference and calls lowercase names
    with a trailing underscore: each drop-in returns void and takes, in order,
    a pointer of the reference argument's type for every argument."""
    protos = _c_prototypes()
    for name, kinds in REFERENCE_ARGS.items():
        ret, params = protos[name]
        assert ret == "void", name
        got = "".join("d" if base == "double" else "i" for base, _ in params)
        assert got == kinds, (name, got)
        assert all(ptr for _, ptr in params), name
