"""Generate the golden fixtures in tests/golden/ with the CPU oracle.

The reference (Fortran 90) ships no golden data and cannot be compiled here,
so these fixtures pin the oracle's restatement of it: any later change to the
oracle or to the GPU path that moves a digit shows up in the tests.  Inputs
are seeded and small so the files stay a few hundred KB.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402


def w(vx, vy, vz, p, ro, bx, by, bz, ps=0.0):
    return np.array([vx, vy, vz, p, ro, bx, by, bz, ps], float)


# face-state pairs that hit each HLLD branch (flux_solver.f90:412-572)
HLLD_CASES = {
    "FL": (w(10, 0.1, 0, 1, 1, 0.5, 0.3, 0.1), w(10.2, 0, 0.1, 0.9, 1.1, 0.5, 0.2, 0)),
    "FR": (w(-10, 0.1, 0, 1, 1, 0.5, 0.3, 0.1), w(-10.2, 0, 0.1, 0.9, 1.1, 0.5, 0.2, 0)),
    "HLLCG_L": (w(0.3, 0.1, 0, 0.01, 1, 2.0, 0, 0), w(0.3, 0.1, 0, 0.01, 1, 2.0, 0, 0, 0.1)),
    "HLLCG_R": (w(-0.3, 0, 0.2, 0.01, 1, 2.0, 0, 0), w(-0.3, 0, 0.2, 0.01, 1, 2.0, 0, 0, -0.1)),
    "Lstar": (w(1.5, 0.2, 0.1, 1, 1, 0.3, 0.5, 0.2), w(1.4, 0.1, 0, 0.9, 1.1, 0.3, 0.4, 0.3)),
    "Rstar": (w(-1.5, 0.2, 0.1, 1, 1, 0.3, 0.5, 0.2), w(-1.4, 0.1, 0, 0.9, 1.1, 0.3, 0.4, 0.3)),
    "Lstar2": (w(0.1, 0.2, 0.1, 1, 1, 1.0, 0.5, 0.2), w(0.05, 0.1, 0, 0.9, 1.1, 1.0, 0.4, 0.3)),
    "Rstar2": (w(-0.1, 0.2, 0.1, 1, 1, 1.0, 0.5, 0.2), w(-0.05, 0.1, 0, 0.9, 1.1, 1.0, 0.4, 0.3)),
}
DIR2_PERM = [1, 2, 0, 3, 4, 6, 7, 5, 8]  # w slots seen from a y face: (vn,vt1,vt2)=(vy,vz,vx)


def rotate_for_dir(a: np.ndarray, d: int) -> np.ndarray:
    if d == 1:
        return a
    return a[np.argsort(DIR2_PERM)]


def ot_grid(n: int, lm: int = 2, flux: int = 3):
    dx = 2 * (4 * math.atan(1.0)) / n
    return O.Grid(2, n + 2, n + 2, 1, dx, dx, dx, 0.0, 0.0, 0.0, 0.4, 5.0 / 3.0, lm, flux, 0, 0)


def kh_grid(nx: int, ny: int):
    return O.Grid(2, nx + 2, ny + 2, 1, 40.0 / nx, 40.0 / ny, 40.0 / nx, 0.0, -20.0, 0.0, 0.4, 5.0 / 3.0, 1, 3, 0, 0,
                  (0, 0, 1, 1, 0, 0), (0,) * 6)


def recon_grid():
    f = lambda *s: sum(1 << (q - 1) for q in s)  # noqa: E731
    return O.Grid(2, 34, 26, 1, 0.25, 0.25, 0.25, -4.0, -3.0, 0.0, 0.4, 5.0 / 3.0, 2, 3, 1, 1,
                  (1, 1, 1, 1, 0, 0), (f(1, 3, 7, 9), f(1, 3, 7, 9), f(2, 3, 6, 9), f(2, 7), 0, 0))


def harris_grid(nx=12, ny=8, nz=12):
    f = lambda *s: sum(1 << (q - 1) for q in s)  # noqa: E731
    dx = 200.0 / nx
    return O.Grid(3, nx + 2, ny + 2, nz + 2, dx, dx, dx, -100.0, -ny * dx / 2, -100.0, 0.4, 5.0 / 3.0, 2,
                  3, 0, 2, (0, 0, 0, 0, 1, 1), (0, 0, 0, 0, f(3, 8), f(3, 8)))


def runs():
    out = {}
    g = ot_grid(32).model(0)
    out["ot32_U0"] = g.U.copy()
    g.step(1)
    out["ot32_U1"] = g.U.copy()
    out["ot32_dt1"] = np.array([g.last_dt, g.last_ch])
    g.step(4)
    out["ot32_U5"] = g.U.copy()
    g = kh_grid(32, 16).model(1, amp=0.5, bx0=0.2, pert=0.01, seed=0)
    out["kh32x16_U0"] = g.U.copy()
    g.step(3)
    out["kh32x16_U3"] = g.U.copy()
    g = recon_grid().model(1, amp=0.3, bx0=0.5, pert=0.05, seed=3)
    out["recon_U0"] = g.U.copy()
    g.step(2)
    out["recon_U2"] = g.U.copy()
    g = harris_grid().model(2, beta=0.2, amp=2e-3, seed=0)
    out["harris_U0"] = g.U.copy()
    g.step(2)
    out["harris_U2"] = g.U.copy()
    return out


def hlld_kats():
    out = {}
    for name, (l, r) in HLLD_CASES.items():
        for d in (1, 2):
            ll, rr = rotate_for_dir(l, d), rotate_for_dir(r, d)
            out[f"hlld_{name}_d{d}_L"] = ll
            out[f"hlld_{name}_d{d}_R"] = rr
            out[f"hlld_{name}_d{d}_F"] = O.flux_faces(ll[:, None], rr[:, None], 0.7, d)[:, 0]
    return out


def limiter_kats():
    out = {}
    wk = np.array([0.0, 1.0, 1.0, 3.0, 2.0, -1.0, -1.0, -0.0, 0.5, 0.25, 0.125, 4.0, -2.0, 7.0])
    plane = np.ascontiguousarray(np.tile(wk, (3, 1)))  # (jx=3, ix=14): one interior row
    L = O.lib()
    for t in range(5):
        wL = np.full_like(plane, 9.0)
        wR = np.full_like(plane, -9.0)
        L.omo_limiter(plane.ctypes.data, wL.ctypes.data, wR.ctypes.data, 14, 3, 1, 1, t)
        out[f"lim_t{t}_wk"] = wk
        out[f"lim_t{t}_wL"] = wL[1].copy()
        out[f"lim_t{t}_wR"] = wR[1].copy()
    return out


def main():
    O.build()
    data = {}
    data.update(runs())
    data.update(hlld_kats())
    data.update(limiter_kats())
    path = os.path.join(HERE, "oracle_golden.npz")
    np.savez_compressed(path, **data)
    print(f"wrote {path} ({os.path.getsize(path)} bytes, {len(data)} arrays)")


if __name__ == "__main__":
    main()
