"""Build and drive the reference's own Fortran, translated to C (oracle/_ref/).

TEST INFRASTRUCTURE ONLY.  Nothing in the product (openmhd_gb300/) imports or
runs this module.

No Fortran compiler exists where this project is built or tested, so the
reference's serial CPU path cannot be compiled as it stands.  This recipe runs
oracle/f90sub.py over the reference's own source files of four problem
directories, exactly as they lie in the OpenMHD checkout, and compiles the C it
produces (with oracle/ref_harness.c, which records the driver's snapshots)
into oracle/_ref/lib<problem>.so (OpenMP on the loops the reference marks
!$omp, so the drivers run on all host cores):

  2D_basic         main.f90, model.f90 (Orszag-Tang), u2v, limiter, flux_solver,
                   rk, glm_ss2, set_dt, bc
  2D_KH            the same routines, 2D_KH/model.f90, main.f90 and bc.f90
                   (bc_for_U / bc_for_F / bc_for_G: reflecting y walls)
  2D_reconnection  the same plus flux_resistive.f90 (eta, set_dt_resistive) and
                   its symmetry-wall bc.f90
  3D_basic         the 3D routines, model.f90 (field loop), main.f90, bc.f90

The main program's size and run parameters (ix, jx, kx, loop_max, tend,
dtout, cfl, lm_type, flux_type, time_type), which a user of the reference sets
by editing main.f90, are read at run time from slots this module fills, so one
library serves every grid the tests use.  The snapshot writer
(fileio_output) becomes a call into the harness, and a 2D driver's model call
can take an injected initial state (set_initial_2d: the benchmark runs the
reference's KH driver from the configuration's own state).  Everything else is
the reference's code.  Without the checkout (the GPU host), the translation
already in oracle/_ref/ is compiled as it is.

    python -m oracle.ref <path of the OpenMHD checkout>      # build all four
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
# where the reference checkout lies in the container that builds the oracle;
# OPENMHD_REFERENCE overrides it
REFERENCE = os.environ.get("OPENMHD_REFERENCE", "/root/reference")

ROUTINES = ["u2v.f90", "limiter.f90", "flux_solver.f90", "rk.f90", "glm_ss2.f90", "set_dt.f90", "bc.f90"]
PROBLEMS = {
    "2D_basic": (2, ROUTINES + ["model.f90", "main.f90"]),
    "2D_KH": (2, ROUTINES + ["model.f90", "main.f90"]),
    "2D_reconnection": (2, ROUTINES + ["flux_resistive.f90", "model.f90", "main.f90"]),
    "3D_basic": (3, ROUTINES + ["model.f90", "main.f90"]),
}
IPAR = {"ix": 0, "jx": 1, "kx": 2, "loop_max": 3, "lm_type": 4, "flux_type": 5, "time_type": 6}
DPAR = {"tend": 0, "dtout": 1, "cfl": 2}
CFLAGS = ["-O2", "-ffp-contract=off", "-fno-fast-math", "-std=gnu11", "-fPIC", "-fopenmp", "-w"]


def available(reference: str | None = None) -> bool:
    reference = reference or REFERENCE
    return all(os.path.isfile(os.path.join(reference, p, "main.f90")) for p in PROBLEMS)


def lib_path(problem: str) -> str:
    return os.path.join(OUT, f"lib{problem}.so")


def translate(problem: str, reference: str | None = None) -> str:
    from oracle import f90sub

    reference = reference or REFERENCE
    nd, files = PROBLEMS[problem]
    d = os.path.join(reference, problem)
    units = f90sub.parse_files([os.path.join(d, f) for f in files], d)
    overrides = {"program": {}}
    for name, k in IPAR.items():
        overrides["program"][name] = f"(f90_ipar_set[{k}] ? f90_ipar[{k}] : ({{orig}}))"
    for name, k in DPAR.items():
        overrides["program"][name] = f"(f90_dpar_set[{k}] ? f90_dpar[{k}] : ({{orig}}))"
    if nd == 2:
        hooks = {"fileio_output": ("ref_snapshot_2d", [1, 2, 3, 4, 5, 6, 7], ["dx", "dt", "ch"]),
                 # the driver's model call may take an injected initial state instead
                 "model": ("ref_model_2d", [0, 1, 2, 3, 4, 5, 6], [])}
    else:
        hooks = {"fileio_output": ("ref_snapshot_3d", [1, 2, 3, 4, 5, 6, 7, 8, 9], ["dx", "dt", "ch"])}
    header = (f"/* generated by oracle/f90sub.py from the reference's {problem}/"
              f"{{{','.join(files)}}}; test infrastructure, not committed */")
    return f90sub.emit_c(units, "f90_", overrides, hooks, header)


def translated(problem: str) -> bool:
    """True when the C translation of `problem` is present in oracle/_ref/
    (made where the checkout exists; it travels with the working tree)."""
    return os.path.isfile(os.path.join(OUT, f"{problem}.c"))


def build(problem: str, reference: str | None = None, force: bool = False) -> str:
    """Translate (when the checkout is present) and compile one problem
    directory; without the checkout, compile the translation already in
    oracle/_ref/."""
    reference = reference or REFERENCE
    so = lib_path(problem)
    c_path = os.path.join(OUT, f"{problem}.c")
    have_src = os.path.isfile(os.path.join(reference, problem, "main.f90"))
    if have_src:
        srcs = [os.path.join(reference, problem, f) for f in PROBLEMS[problem][1]]
        deps = srcs + [os.path.join(HERE, "f90sub.py"), os.path.join(HERE, "ref_harness.c"), __file__]
    elif os.path.isfile(c_path):
        deps = [c_path, os.path.join(HERE, "ref_harness.c")]
    else:
        raise FileNotFoundError(f"neither the OpenMHD checkout nor {c_path} is present")
    if not force and os.path.exists(so) and all(os.path.getmtime(p) <= os.path.getmtime(so) for p in deps):
        return so
    os.makedirs(OUT, exist_ok=True)
    if have_src:
        with open(c_path, "w") as f:
            f.write(translate(problem, reference))
    tmp = so + ".tmp"
    nd = PROBLEMS[problem][0]
    cmd = [os.environ.get("CC", "gcc")] + CFLAGS + (["-DREF_MODEL_HOOK_2D"] if nd == 2 else []) + [
        "-shared", "-o", tmp, c_path, os.path.join(HERE, "ref_harness.c"), "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compiling the translated {problem} failed:\n{r.stderr[-4000:]}")
    os.replace(tmp, so)
    return so


def build_all(reference: str | None = None, force: bool = False) -> list[str]:
    return [build(p, reference, force) for p in PROBLEMS]


def buildable(reference: str | None = None) -> bool:
    return available(reference) or all(translated(p) for p in PROBLEMS)


def set_initial_2d(problem: str, U=None, x=None, y=None, dx: float = 0.0) -> None:
    """Make the 2D driver of `problem` start from U (reference layout, ghosts
    included) with coordinates x, y and spacing dx instead of running its
    model.f90; U=None restores the driver's own model."""
    lib = load(problem)
    if U is None:
        lib.ref_set_initial_2d(None, None, None, C.c_double(0.0), 0, 0)
        return
    U = np.ascontiguousarray(U, dtype=np.float64)
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.ascontiguousarray(y, dtype=np.float64)
    if lib.ref_set_initial_2d(C.c_void_p(U.ctypes.data), C.c_void_p(x.ctypes.data), C.c_void_p(y.ctypes.data),
                              C.c_double(dx), int(U.shape[-1]), int(U.shape[-2])):
        raise MemoryError("could not keep the initial state")


_libs: dict = {}


def load(problem: str) -> C.CDLL:
    if problem not in _libs:
        so = lib_path(problem)
        if not os.path.exists(so):
            raise FileNotFoundError(f"{so} is not built (python -m oracle.ref <OpenMHD checkout>)")
        _libs[problem] = C.CDLL(so)
    return _libs[problem]


def routine(problem: str, name: str):
    """The translated reference subroutine `name` (all arguments by reference)."""
    fn = getattr(load(problem), "f90_" + name)
    fn.restype = None
    return fn


def byref_args(*vals):
    """ctypes arguments for a by-reference call: numpy float64 arrays as
    pointers, Python ints as int*, floats as double*."""
    out, keep = [], []
    for v in vals:
        if isinstance(v, np.ndarray):
            assert v.dtype == np.float64 and v.flags.c_contiguous
            out.append(C.c_void_p(v.ctypes.data))
        elif isinstance(v, (bool, int, np.integer)):
            c = C.c_int(int(v))
            keep.append(c)
            out.append(C.byref(c))
        elif isinstance(v, C._SimpleCData):
            out.append(C.byref(v))
        else:
            c = C.c_double(float(v))
            keep.append(c)
            out.append(C.byref(c))
    return out, keep


def call(problem: str, name: str, *vals):
    args, keep = byref_args(*vals)
    lib = load(problem)
    C.c_int.in_dll(lib, "f90_stopped").value = 0
    routine(problem, name)(*args)
    return C.c_int.in_dll(lib, "f90_stopped").value


def run_main(problem: str, **params) -> tuple[int, list[dict]]:
    """Run the reference's main program with the given parameters (names of
    main.f90's parameters); returns (line of a STOP or 0, snapshots), each
    snapshot {t, dx, dt, ch, U (numpy, reference layout), x, y, z}."""
    lib = load(problem)
    iset = (C.c_int * 16).in_dll(lib, "f90_ipar_set")
    ival = (C.c_int * 16).in_dll(lib, "f90_ipar")
    dset = (C.c_int * 16).in_dll(lib, "f90_dpar_set")
    dval = (C.c_double * 16).in_dll(lib, "f90_dpar")
    for k in range(16):
        iset[k] = 0
        dset[k] = 0
    for name, v in params.items():
        if name in IPAR:
            iset[IPAR[name]], ival[IPAR[name]] = 1, int(v)
        elif name in DPAR:
            dset[DPAR[name]], dval[DPAR[name]] = 1, float(v)
        else:
            raise KeyError(f"main.f90 has no run parameter {name}")
    lib.ref_snap_clear()
    C.c_int.in_dll(lib, "f90_stopped").value = 0
    lib.f90_main.restype = C.c_int
    stopped = lib.f90_main()
    snaps = []
    dims = (C.c_int * 3)()
    vals = (C.c_double * 4)()
    for k in range(lib.ref_snap_count()):
        lib.ref_snap_info(k, dims, vals)
        ix, jx, kx = dims[0], dims[1], dims[2]
        shape = (9, jx, ix) if PROBLEMS[problem][0] == 2 else (9, kx, jx, ix)
        U = np.empty(shape)
        x, y, z = np.empty(ix), np.empty(jx), np.empty(kx)
        lib.ref_snap_copy(k, C.c_void_p(U.ctypes.data), C.c_void_p(x.ctypes.data), C.c_void_p(y.ctypes.data),
                          C.c_void_p(z.ctypes.data))
        snaps.append({"t": vals[0], "dx": vals[1], "dt": vals[2], "ch": vals[3], "U": U, "x": x, "y": y, "z": z})
    lib.ref_snap_clear()
    return stopped, snaps


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python -m oracle.ref <path of the OpenMHD checkout>")
    for p in build_all(sys.argv[1], force=True):
        print(p)
