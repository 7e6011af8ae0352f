"""Record outputs of the reference's own Fortran, executed through its C
translation (oracle/ref.py), as fixtures for machines without the OpenMHD
checkout.

For each of the four reference drivers (2D_basic, 2D_KH, 2D_reconnection,
3D_basic main.f90 with their model.f90) on a small grid it stores the first
and the last snapshot the driver writes (state with ghosts, t, dx, dt, ch and
coordinates), and for the HLLD solver of flux_solver.f90 the flux of each
branch-forcing face pair in tests/golden/oracle_golden.npz.
tests/test_ref_golden.py replays the drivers with the oracle and requires the
same bits.

    python tests/golden/make_ref_golden.py <path of the OpenMHD checkout>
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

RUNS = {
    "2D_basic": dict(ix=18, jx=18, tend=0.4, dtout=0.2, lm_type=2, flux_type=3),
    "2D_KH": dict(ix=18, jx=26, tend=4.0, dtout=2.0, lm_type=1, flux_type=3),
    "2D_reconnection": dict(ix=34, jx=18, tend=16.0, dtout=8.0, lm_type=1, flux_type=3),
    "3D_basic": dict(ix=10, jx=8, kx=12, tend=0.06, dtout=0.03, lm_type=1, flux_type=3),
}


def main(reference: str) -> None:
    from oracle import ref
    from test_ref_translation import ref_flux_faces

    ref.build_all(reference)
    out = {}
    for problem, params in RUNS.items():
        stopped, snaps = ref.run_main(problem, **params)
        assert stopped == 0 and len(snaps) >= 2, (problem, stopped, len(snaps))
        for tag, s in (("first", snaps[0]), ("last", snaps[-1])):
            for k in ("U", "x", "y", "z"):
                out[f"{problem}_{tag}_{k}"] = s[k]
            out[f"{problem}_{tag}_tdxdtch"] = np.array([s["t"], s["dx"], s["dt"], s["ch"]])
        out[f"{problem}_params"] = np.array([f"{k}={v}" for k, v in params.items()])
    gold = np.load(os.path.join(HERE, "oracle_golden.npz"))
    for name in ("FL", "FR", "HLLCG_L", "HLLCG_R", "Lstar", "Rstar", "Lstar2", "Rstar2"):
        for d in (1, 2):
            L, R = gold[f"hlld_{name}_d{d}_L"], gold[f"hlld_{name}_d{d}_R"]
            out[f"hlld_{name}_d{d}_F"] = ref_flux_faces(ref, L[:, None], R[:, None], 0.7, d)[:, 0]
    path = os.path.join(HERE, "ref_translated_golden.npz")
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_ref_golden.py <path of the OpenMHD checkout>")
    main(sys.argv[1])
