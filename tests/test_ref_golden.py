"""The oracle against fixtures recorded from the reference's own Fortran,
executed through its C translation (tests/golden/make_ref_golden.py ran the
reference drivers of 2D_basic, 2D_KH, 2D_reconnection and 3D_basic and its HLLD
solver and stored what they produced).  Runs without the OpenMHD checkout:
the oracle, started from each driver's first snapshot, must reach its last
snapshot with the same time, dt, ch and bits, and reproduce the reference's
HLLD flux of every branch.  tests/test_ref_translation.py makes the same
comparisons against the executed reference itself, over more cases."""
import os

import numpy as np
import pytest

from test_ref_translation import DEFAULTS, GRID

GOLD = os.path.join(os.path.dirname(__file__), "golden", "ref_translated_golden.npz")


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


@pytest.mark.parametrize("problem", ["2D_basic", "2D_KH", "2D_reconnection", "3D_basic"])
def test_oracle_reproduces_reference_driver(oracle_mod, gold, problem):
    from oracle.oracle import Grid

    params = dict(DEFAULTS[problem])
    for kv in gold[f"{problem}_params"]:
        k, v = str(kv).split("=")
        params[k] = float(v) if "." in v else int(v)
    U0 = gold[f"{problem}_first_U"]
    t0, dx, _, _ = gold[f"{problem}_first_tdxdtch"]
    nd = 2 if U0.ndim == 3 else 3
    ix, jx = U0.shape[-1], U0.shape[-2]
    kx = U0.shape[1] if nd == 3 else 1
    g = Grid(nd, ix, jx, kx, dx, dx, dx, cfl=params["cfl"], lm_type=params["lm_type"],
             flux_type=params["flux_type"], time_type=params["time_type"], **GRID[problem])
    g.U[...] = U0
    g.t = t0
    g.x[:], g.y[:] = gold[f"{problem}_first_x"], gold[f"{problem}_first_y"]
    if nd == 3:
        g.z[:] = gold[f"{problem}_first_z"]
    t1, _, dt1, ch1 = gold[f"{problem}_last_tdxdtch"]
    while g.t < t1:
        g.step(1)
    assert g.t == t1 and g.last_dt == dt1 and g.last_ch == ch1
    assert np.array_equal(g.U, gold[f"{problem}_last_U"]), np.abs(g.U - gold[f"{problem}_last_U"]).max()


@pytest.mark.parametrize("d", [1, 2])
@pytest.mark.parametrize("name", ["FL", "FR", "HLLCG_L", "HLLCG_R", "Lstar", "Rstar", "Lstar2", "Rstar2"])
def test_oracle_reproduces_reference_hlld(oracle_mod, gold, name, d):
    og = np.load(os.path.join(os.path.dirname(__file__), "golden", "oracle_golden.npz"))
    L, R = og[f"hlld_{name}_d{d}_L"], og[f"hlld_{name}_d{d}_R"]
    F = oracle_mod.flux_faces(L[:, None], R[:, None], 0.7, d)[:, 0]
    assert np.array_equal(F, gold[f"hlld_{name}_d{d}_F"])
