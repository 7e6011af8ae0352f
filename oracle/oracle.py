"""ctypes front end of the CPU oracle (oracle/omhd_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline legs of bench.py, to check results against.  The product (openmhd_gb300/)
never imports it.  Parity status: pinned to the reference's own source, which
oracle/ref.py executes through a mechanical C translation (no Fortran compiler
is available): tests/test_ref_translation.py and tests/test_ref_golden.py.

State arrays are numpy float64 arrays shaped (9, jx, ix) or (9, kx, jx, ix):
the same memory as the reference's column-major U(ix,jx[,kx],var).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")

OK, NEG_PRESSURE, NEG_DENSITY, DT_TOO_SMALL, BAD_ARG = range(5)


class BCSpec(C.Structure):
    _fields_ = [("kind", C.c_int * 6), ("flip", C.c_int * 6)]


class Err(C.Structure):
    _fields_ = [("code", C.c_int), ("i", C.c_int), ("j", C.c_int), ("k", C.c_int), ("value", C.c_double)]


class Cfg(C.Structure):
    _fields_ = [("ix", C.c_int), ("jx", C.c_int), ("kx", C.c_int), ("nd", C.c_int),
                ("dx", C.c_double), ("dy", C.c_double), ("dz", C.c_double),
                ("cfl", C.c_double), ("gamma", C.c_double),
                ("lm_type", C.c_int), ("flux_type", C.c_int), ("time_type", C.c_int),
                ("eta_kind", C.c_int), ("bc", BCSpec)]


class Model(C.Structure):
    _fields_ = [("kind", C.c_int), ("amp", C.c_double), ("bx0", C.c_double),
                ("phase_x", C.c_double), ("phase_y", C.c_double), ("beta", C.c_double),
                ("pert", C.c_double), ("seed", C.c_uint64),
                ("x0", C.c_double), ("y0", C.c_double), ("z0", C.c_double)]


def build(force: bool = False) -> None:
    """Compile the oracle shared libraries with the committed Makefile."""
    libs = [os.path.join(BUILD, n) for n in ("libomhd_oracle.so", "libomhd_oracle_omp.so")]
    src = os.path.join(HERE, "omhd_oracle.c")
    if not force and all(os.path.exists(p) and os.path.getmtime(p) >= os.path.getmtime(src) for p in libs):
        return
    subprocess.run(["make", "-s", "-C", HERE], check=True)


_LIBS: dict[bool, C.CDLL] = {}


def lib(omp: bool = False) -> C.CDLL:
    if omp not in _LIBS:
        build()
        path = os.path.join(BUILD, "libomhd_oracle_omp.so" if omp else "libomhd_oracle.so")
        L = C.CDLL(path)
        P, I, D = C.c_void_p, C.c_int, C.c_double
        sig = {
            "omo_set_gamma": (None, [D]),
            "omo_u2v": (I, [P, P, I, I, I, C.POINTER(Err)]),
            "omo_limiter": (None, [P, P, P, I, I, I, I, I]),
            "omo_flux_solver": (None, [P, P, P, D, I, I, I, I, I]),
            "omo_rk_tvd21": (None, [P, P, P, P, P, D, D, D, D, I, I, I, I]),
            "omo_rk_tvd22": (None, [P, P, P, P, P, D, D, D, D, I, I, I, I]),
            "omo_rk_std21": (None, [P, P, P, P, P, D, D, D, D, I, I, I, I]),
            "omo_rk_std22": (None, [P, P, P, P, D, D, D, D, I, I, I, I]),
            "omo_glm_ss2": (None, [P, D, D, I, I, I]),
            "omo_set_dt": (I, [P, P, C.POINTER(C.c_double), C.POINTER(C.c_double), D, D, D, D, I, I, I, I,
                               C.POINTER(Err)]),
            "omo_set_dt_resistive": (None, [C.POINTER(C.c_double), D, D, I]),
            "omo_bc": (None, [P, I, I, I, I, C.POINTER(BCSpec)]),
            "omo_facefix": (None, [P, P, I, I, I, I, C.POINTER(BCSpec)]),
            "omo_eta": (D, [I, D, D, D]),
            "omo_branch_counts": (None, [C.POINTER(C.c_longlong * 8), I]),
            "omo_flux_resistive": (None, [P, P, P, P, P, D, I, I, I, I, I, I]),
            "omo_step": (I, [C.POINTER(Cfg), P, P, P, P, P, C.POINTER(C.c_double), C.POINTER(C.c_double),
                             C.POINTER(C.c_double), C.POINTER(Err)]),
            "omo_workspace_doubles": (C.c_size_t, [C.POINTER(Cfg)]),
            "omo_uniform_pm1": (D, [C.c_uint64, C.c_uint64]),
            "omo_grid": (None, [P, I, D, D]),
            "omo_model_fill": (None, [C.POINTER(Model), P, P, P, P, I, I, I, D, D, D]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _LIBS[omp] = L
    return _LIBS[omp]


def _p(a: np.ndarray) -> int:
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data


def bcspec(kind, flip) -> BCSpec:
    b = BCSpec()
    for q in range(6):
        b.kind[q] = int(kind[q])
        b.flip[q] = int(flip[q])
    return b


class OracleError(RuntimeError):
    def __init__(self, err: Err):
        super().__init__(f"oracle status {err.code} at ({err.i},{err.j},{err.k}) value {err.value}")
        self.code = err.code
        self.err = err


class Grid:
    """One problem instance advanced by the CPU oracle, mirroring the
    reference driver (2D_basic/main.f90:56-188)."""

    def __init__(self, nd, ix, jx, kx=1, dx=1.0, dy=1.0, dz=1.0, x0=0.0, y0=0.0, z0=0.0, cfl=0.4,
                 gamma=5.0 / 3.0, lm_type=1, flux_type=3, time_type=0, eta_kind=0,
                 bc_kind=(0,) * 6, bc_flip=(0,) * 6, omp=False):
        self.L = lib(omp)
        self.cfg = Cfg()
        c = self.cfg
        c.ix, c.jx, c.kx, c.nd = ix, jx, (kx if nd == 3 else 1), nd
        c.dx, c.dy, c.dz = dx, dy, (dz if nd == 3 else dx)
        c.cfl, c.gamma = cfl, gamma
        c.lm_type, c.flux_type, c.time_type, c.eta_kind = lm_type, flux_type, time_type, eta_kind
        c.bc = bcspec(bc_kind, bc_flip)
        self.shape = (9, jx, ix) if nd == 2 else (9, kx, jx, ix)
        self.n = ix * jx * c.kx
        self.ws = np.zeros(int(self.L.omo_workspace_doubles(C.byref(c))), dtype=np.float64)
        self.x = np.zeros(ix)
        self.y = np.zeros(jx)
        self.z = np.zeros(c.kx)
        self.L.omo_grid(_p(self.x), ix, x0, dx)
        self.L.omo_grid(_p(self.y), jx, y0, dy)
        self.L.omo_grid(_p(self.z), c.kx, z0, c.dz)
        self.x0, self.y0, self.z0 = x0, y0, z0
        self.U = np.zeros(self.shape)
        self.t = 0.0
        self.last_dt = 0.0
        self.last_ch = 0.0
        self.steps = 0

    @classmethod
    def from_solver_config(cls, sc, omp: bool = False) -> "Grid":
        """Build from an openmhd_gb300.solver.SolverConfig-like object (duck typed)."""
        from_names = {"flat": 0, "minmod": 1, "mc": 2, "vanleer": 3, "koren": 4}
        fl = {"llf": 0, "hll": 1, "hllc": 2, "hlld": 3, "lhlld": 4}
        eta = {"none": 0, "recon2d": 1, "harris_xz": 2}
        return cls(sc.nd, sc.ix, sc.jx, sc.kx, sc.dx, sc.dy, sc.dz, sc.x0, sc.y0, sc.z0, sc.cfl, sc.gamma,
                   from_names[sc.limiter], fl[sc.flux], 0 if sc.time == "tvdrk2" else 1, eta[sc.eta],
                   sc.bc_kind, sc.bc_flip, omp=omp)

    def model(self, kind, amp=1.0, bx0=0.0, phase_x=0.0, phase_y=0.0, beta=0.2, pert=0.0, seed=0):
        m = Model()
        m.kind, m.amp, m.bx0, m.phase_x, m.phase_y = kind, amp, bx0, phase_x, phase_y
        m.beta, m.pert, m.seed = beta, pert, seed
        m.x0, m.y0, m.z0 = self.x0, self.y0, self.z0
        c = self.cfg
        self.L.omo_set_gamma(c.gamma)
        self.L.omo_model_fill(C.byref(m), _p(self.U), _p(self.x), _p(self.y), _p(self.z), c.ix, c.jx, c.kx,
                              c.dx, c.dy, c.dz)
        self.bc()
        return self

    def bc(self):
        c = self.cfg
        self.L.omo_bc(_p(self.U), c.ix, c.jx, c.kx, c.nd, C.byref(c.bc))

    def step(self, n: int = 1):
        dt = C.c_double()
        ch = C.c_double()
        t = C.c_double(self.t)
        e = Err()
        for _ in range(n):
            st = self.L.omo_step(C.byref(self.cfg), _p(self.U), _p(self.ws), _p(self.x), _p(self.y),
                                 _p(self.z), C.byref(t), C.byref(dt), C.byref(ch), C.byref(e))
            if st:
                raise OracleError(e)
            self.steps += 1
        self.t = t.value
        self.last_dt = dt.value
        self.last_ch = ch.value
        return self

    def run_until(self, tend: float, max_steps: int = 100000):
        while self.t < tend and self.steps < max_steps:  # main.f90:73
            self.step(1)
        return self


# ---- routine-level helpers (numpy arrays in reference layout) ----
def u2v(U: np.ndarray, nd: int):
    L = lib()
    shp = U.shape
    ix, jx = shp[-1], shp[-2]
    kx = shp[-3] if nd == 3 else 1
    V = np.zeros((4,) + shp[1:])
    e = Err()
    st = L.omo_u2v(_p(U), _p(V), ix, jx, kx, C.byref(e))
    return V, st, e


def uniform_pm1(seed: int, n: int) -> float:
    return float(lib().omo_uniform_pm1(seed, n))


BRANCHES = ["FL", "FR", "HLLCG_L", "HLLCG_R", "Lstar", "Rstar", "Lstar2", "Rstar2"]


def branch_counts(reset: bool = True) -> dict:
    """HLLD branch histogram of the serial oracle since the last reset."""
    out = (C.c_longlong * 8)()
    lib().omo_branch_counts(C.byref(out), 1 if reset else 0)
    return dict(zip(BRANCHES, list(out)))


def flux_faces(VL: np.ndarray, VR: np.ndarray, ch: float, dir: int, type_: int = 3) -> np.ndarray:
    """Fluxes for a batch of face-state pairs given as (9, m) arrays (w slots:
    vx, vy, vz, p, rho, Bx, By, Bz, psi).  The pairs are laid on dir-faces of a
    tiny grid so that the reference routine's own loop bounds apply."""
    m = VL.shape[1]
    if dir == 1:
        ix, jx = 2, m + 2
        shape = (9, jx, ix)
        def put(a, src):
            a[:, 1:-1, 0] = src
        def get(a):
            return a[:, 1:-1, 0]
    else:
        ix, jx = m + 2, 2
        shape = (9, jx, ix)
        def put(a, src):
            a[:, 0, 1:-1] = src
        def get(a):
            return a[:, 0, 1:-1]
    L = np.zeros(shape); R = np.zeros(shape); F = np.zeros(shape)
    L[4] = 1.0; R[4] = 1.0; L[3] = 1.0; R[3] = 1.0
    put(L, VL); put(R, VR)
    lib().omo_flux_solver(_p(F), _p(L), _p(R), ch, ix, jx, 1, dir, type_)
    return get(F).copy()
