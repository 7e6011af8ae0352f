"""The oracle against the reference's own Fortran, executed.

No Fortran compiler exists here, so oracle/ref.py translates the reference's
source files mechanically into C (oracle/f90sub.py) and builds one library per
problem directory into oracle/_ref/.  These tests compare the hand-written
oracle (oracle/omhd_oracle.c), which every GPU parity test uses as its
reference, with that executed reference text, bit for bit:

* the reference drivers themselves (2D_basic, 2D_KH, 2D_reconnection and
  3D_basic main.f90 with their model.f90): the oracle, started from the
  driver's first snapshot, must reach every later snapshot with the same time
  and the same bits in every cell, ghosts included, over every limiter
  (flat, minmod, MC, van Leer, Koren), every flux (LLF, HLL, HLLC, HLLD,
  LHLLD) and both time integrators;
* each routine on seeded random states (u2v, limiter, flux_solver, rk_*,
  glm_ss2, set_dt, bc, bc_for_U/F/G, flux_resistive, set_dt_resistive),
  2D and 3D, and the HLLD solver on the constructed states that force each of
  its eight branches;
* the reference's failure exits (negative pressure in u2v, dt below 1e-7 in
  set_dt) stop where the oracle reports the same failure.

The routine-level GPU kernels are tested bitwise against the oracle
(tests/test_gpu_routines.py), so this closes the chain: reference source ->
oracle -> CUDA.  Needs the reference checkout to build oracle/_ref; without
it, tests/test_ref_golden.py checks the oracle against fixtures recorded from
the executed reference instead."""
import ctypes as C

import numpy as np
import pytest

from helpers import random_state

MX, MY, MZ, EN, RO, BX, BY, BZ, PS = range(9)


def f(*v):
    return sum(1 << x for x in v)


@pytest.fixture(scope="module")
def ref():
    from oracle import ref as R

    if not R.available():
        if all(__import__("os").path.exists(R.lib_path(p)) for p in R.PROBLEMS):
            return R
        pytest.skip("the OpenMHD checkout is not present: tests/test_ref_golden.py covers the oracle")
    R.build_all()
    return R


# problem -> oracle Grid keywords (boundaries and resistivity as the problem's bc.f90 / main.f90 set them)
GRID = {
    "2D_basic": dict(),
    "2D_KH": dict(bc_kind=(0, 0, 1, 1, 0, 0), bc_flip=(0, 0, f(MY, BY), f(MY, BY), 0, 0)),
    "2D_reconnection": dict(eta_kind=1, bc_kind=(1, 1, 1, 1, 0, 0),
                            bc_flip=(f(MX, MZ, BY, PS), f(MX, MZ, BY, PS), f(MY, MZ, BX, PS), f(MY, BY), 0, 0)),
    "3D_basic": dict(),
}
# the reference's defaults (main.f90) for what a run leaves unset
DEFAULTS = {"2D_basic": dict(cfl=0.4, lm_type=1, flux_type=3, time_type=0),
            "2D_KH": dict(cfl=0.4, lm_type=1, flux_type=3, time_type=0),
            "2D_reconnection": dict(cfl=0.35, lm_type=1, flux_type=3, time_type=0),
            "3D_basic": dict(cfl=0.3, lm_type=1, flux_type=3, time_type=0)}


def drive_and_compare(R, problem, **params):
    """Run the reference driver, replay it with the oracle from its first
    snapshot, and require identical times and bits at every later snapshot."""
    from oracle.oracle import Grid

    stopped, snaps = R.run_main(problem, **params)
    assert stopped == 0 and len(snaps) >= 3, (stopped, len(snaps))
    p = dict(DEFAULTS[problem], **params)
    s0 = snaps[0]
    U0 = s0["U"]
    nd = 2 if U0.ndim == 3 else 3
    ix, jx = U0.shape[-1], U0.shape[-2]
    kx = U0.shape[1] if nd == 3 else 1
    dx = s0["dx"]
    g = Grid(nd, ix, jx, kx, dx, dx, dx, cfl=p["cfl"], lm_type=p["lm_type"], flux_type=p["flux_type"],
             time_type=p["time_type"], **GRID[problem])
    g.U[...] = U0
    g.x[:], g.y[:] = s0["x"], s0["y"]
    if nd == 3:
        g.z[:] = s0["z"]
    for s in snaps[1:]:
        while g.t < s["t"]:
            g.step(1)
        assert g.t == s["t"], (problem, params, g.t, s["t"])
        assert g.last_dt == s["dt"] and g.last_ch == s["ch"]
        assert np.array_equal(g.U, s["U"]), (problem, params, s["t"], np.abs(g.U - s["U"]).max())
    return g.steps


@pytest.mark.parametrize("time_type", [0, 1])
@pytest.mark.parametrize("flux_type", [0, 1, 2, 3, 4])
@pytest.mark.parametrize("lm_type", [0, 1, 2, 3, 4])
def test_2d_basic_driver_bitwise(ref, oracle_mod, lm_type, flux_type, time_type):
    """2D_basic/main.f90 with 2D_basic/model.f90 (Orszag-Tang), 24x20 cells."""
    drive_and_compare(ref, "2D_basic", ix=26, jx=22, tend=0.3, dtout=0.1, lm_type=lm_type, flux_type=flux_type,
                      time_type=time_type)


@pytest.mark.parametrize("lm_type,flux_type", [(1, 3), (2, 3), (2, 1)])
def test_kh_driver_bitwise(ref, oracle_mod, lm_type, flux_type):
    """2D_KH/main.f90 with its model and reflecting y walls (bc_for_U/F/G)."""
    drive_and_compare(ref, "2D_KH", ix=34, jx=42, tend=3.0, dtout=1.0, lm_type=lm_type, flux_type=flux_type)


@pytest.mark.parametrize("lm_type,time_type", [(1, 0), (2, 1)])
def test_reconnection_driver_bitwise(ref, oracle_mod, lm_type, time_type):
    """2D_reconnection/main.f90: Harris sheet + X-point perturbation, resistive
    fluxes with eta(x, y), set_dt_resistive and the symmetry walls of its bc.f90."""
    drive_and_compare(ref, "2D_reconnection", ix=130, jx=66, tend=4.0, dtout=1.0, lm_type=lm_type,
                      time_type=time_type)


@pytest.mark.parametrize("lm_type,flux_type", [(1, 3), (2, 2), (4, 4)])
def test_3d_basic_driver_bitwise(ref, oracle_mod, lm_type, flux_type):
    """3D_basic/main.f90 with its field-loop model, periodic in x, y and z."""
    drive_and_compare(ref, "3D_basic", ix=14, jx=12, kx=18, tend=0.1, dtout=0.04, lm_type=lm_type,
                      flux_type=flux_type)


# ---------------------------------------------------------------------------
# routine level
# ---------------------------------------------------------------------------
SHAPES = {"2D_basic": (21, 17), "3D_basic": (9, 8, 11)}


def _dims(shape):
    return (shape[1], shape[0], 1) if len(shape) == 2 else (shape[2], shape[1], shape[0])


def _sizes(problem, shape):
    ix, jx, kx = _dims(shape)
    return (ix, jx) if problem.startswith("2D") else (ix, jx, kx)


@pytest.mark.parametrize("problem", ["2D_basic", "3D_basic"])
def test_routines_bitwise(ref, oracle_mod, problem):
    L = oracle_mod.lib()
    shape = SHAPES[problem]
    ix, jx, kx = _dims(shape)
    nd = len(shape)
    sz = _sizes(problem, shape)
    p = oracle_mod._p
    U = random_state(shape, 1)
    # u2v
    V = np.zeros((4,) + shape)
    assert ref.call(problem, "u2v", U, V, *sz) == 0
    Vo, st, _ = oracle_mod.u2v(U, nd)
    assert st == 0 and np.array_equal(V, Vo)
    # limiter, every type and direction
    wk = random_state(shape, 2)[3]
    for typ in range(5):
        for d in range(1, nd + 1):
            wL, wR = np.zeros(shape), np.zeros(shape)
            oL, oR = np.zeros(shape), np.zeros(shape)
            ref.call(problem, "limiter", wk, wL, wR, *sz, d, typ)
            L.omo_limiter(p(wk), p(oL), p(oR), ix, jx, kx, d, typ)
            assert np.array_equal(wL, oL) and np.array_equal(wR, oR), (typ, d)
    # flux_solver, every type and direction, on random face states
    VL, VR = random_state(shape, 3), random_state(shape, 4)
    for typ in range(5):
        for d in range(1, nd + 1):
            F, Fo = np.zeros((9,) + shape), np.zeros((9,) + shape)
            ref.call(problem, "flux_solver", F, VL, VR, 0.9, *sz, d, typ)
            L.omo_flux_solver(p(Fo), p(VL), p(VR), 0.9, ix, jx, kx, d, typ)
            assert np.array_equal(F, Fo), (typ, d)
    # the four RK stages
    rng = np.random.default_rng(5)
    Fs = [rng.uniform(-1, 1, (9,) + shape) for _ in range(3)]
    dt, dx = 0.0123, 0.05
    fl = Fs[:nd]
    for name in ("rk_tvd21", "rk_tvd22", "rk_std21", "rk_std22"):
        A, B = random_state(shape, 6), random_state(shape, 7)
        Ao, Bo = A.copy(), B.copy()
        if name == "rk_std22":
            ref.call(problem, name, A, *fl, dt, dx, *sz)
            getattr(L, "omo_" + name)(p(Ao), p(Fs[0]), p(Fs[1]), p(Fs[2]), dt, dx, dx, dx, ix, jx, kx, nd)
        else:
            ref.call(problem, name, A, B, *fl, dt, dx, *sz)
            getattr(L, "omo_" + name)(p(Ao), p(Bo), p(Fs[0]), p(Fs[1]), p(Fs[2]), dt, dx, dx, dx, ix, jx, kx, nd)
        assert np.array_equal(A, Ao) and np.array_equal(B, Bo), name
    # glm_ss2, set_dt, bc
    A = random_state(shape, 8)
    Ao = A.copy()
    ref.call(problem, "glm_ss2", A, 1.3, 0.02, *sz)
    L.omo_glm_ss2(p(Ao), 1.3, 0.02, ix, jx, kx)
    assert np.array_equal(A, Ao)
    V, _, _ = oracle_mod.u2v(A, nd)
    vmax, dtr = C.c_double(), C.c_double()
    assert ref.call(problem, "set_dt", A, V, vmax, dtr, 0.05, 0.4, *sz) == 0
    vo, do = C.c_double(), C.c_double()
    e = oracle_mod.Err()
    assert L.omo_set_dt(p(A), p(V), C.byref(vo), C.byref(do), 0.05, 0.05, 0.05, 0.4, ix, jx, kx, nd,
                        C.byref(e)) == 0
    assert vmax.value == vo.value and dtr.value == do.value
    A = random_state(shape, 9)
    Ao = A.copy()
    ref.call(problem, "bc", A, *sz)
    L.omo_bc(p(Ao), ix, jx, kx, nd, C.byref(oracle_mod.bcspec((0,) * 6, (0,) * 6)))
    assert np.array_equal(A, Ao)


def test_failure_exits(ref, oracle_mod):
    """u2v stops on a non-positive pressure and set_dt on dt < 1e-7
    (u2v.f90:34-43, set_dt.f90:55-65), where the oracle reports the same."""
    shape = (12, 10)
    U = random_state(shape, 2)
    U[3, 7, 4] = 0.0
    V = np.zeros((4,) + shape)
    assert ref.call("2D_basic", "u2v", U, V, 10, 12) != 0
    _, st, _ = oracle_mod.u2v(U, 2)
    assert st == 1
    U = random_state(shape, 8)
    V, _, _ = oracle_mod.u2v(U, 2)
    assert ref.call("2D_basic", "set_dt", U, V, C.c_double(), C.c_double(), 1e-9, 0.4, 10, 12) != 0
    e = oracle_mod.Err()
    L = oracle_mod.lib()
    assert L.omo_set_dt(oracle_mod._p(U), oracle_mod._p(V), C.byref(C.c_double()), C.byref(C.c_double()), 1e-9,
                        1e-9, 1e-9, 0.4, 10, 12, 1, 2, C.byref(e)) == 3


def ref_flux_faces(R, VL, VR, ch, d, typ=3):
    """Face pairs through the translated flux_solver, laid out as oracle.flux_faces lays them."""
    m = VL.shape[1]
    if d == 1:
        ix, jx = 2, m + 2
    else:
        ix, jx = m + 2, 2
    L = np.zeros((9, jx, ix))
    Rr = np.zeros((9, jx, ix))
    F = np.zeros((9, jx, ix))
    L[4] = Rr[4] = L[3] = Rr[3] = 1.0
    if d == 1:
        L[:, 1:-1, 0], Rr[:, 1:-1, 0] = VL, VR
    else:
        L[:, 0, 1:-1], Rr[:, 0, 1:-1] = VL, VR
    R.call("2D_basic", "flux_solver", F, L, Rr, ch, ix, jx, d, typ)
    return (F[:, 1:-1, 0] if d == 1 else F[:, 0, 1:-1]).copy()


@pytest.mark.parametrize("d", [1, 2])
@pytest.mark.parametrize("name", ["FL", "FR", "HLLCG_L", "HLLCG_R", "Lstar", "Rstar", "Lstar2", "Rstar2"])
def test_hlld_branches_bitwise(ref, oracle_mod, name, d):
    """The HLLD solver of flux_solver.f90 on the states that force each branch
    (tests/golden/oracle_golden.npz) equals the oracle's flux, which the
    oracle's branch histogram shows took that branch."""
    import os

    gold = np.load(os.path.join(os.path.dirname(__file__), "golden", "oracle_golden.npz"))
    L, R = gold[f"hlld_{name}_d{d}_L"], gold[f"hlld_{name}_d{d}_R"]
    oracle_mod.branch_counts()
    Fo = oracle_mod.flux_faces(L[:, None], R[:, None], 0.7, d)[:, 0]
    assert [k for k, v in oracle_mod.branch_counts().items() if v] == [name]
    F = ref_flux_faces(ref, L[:, None], R[:, None], 0.7, d)[:, 0]
    assert np.array_equal(F, Fo), (F, Fo)


def test_wall_and_resistive_routines_bitwise(ref, oracle_mod):
    """2D_KH/bc.f90 and 2D_reconnection/bc.f90 (bc_for_U, bc_for_F, bc_for_G),
    2D_reconnection/flux_resistive.f90 (both directions, eta(x, y)) and
    set_dt_resistive against the oracle's wall masks and resistive fluxes."""
    L = oracle_mod.lib()
    p = oracle_mod._p
    shape = (14, 19)
    ix, jx, kx = 19, 14, 1
    for problem in ("2D_KH", "2D_reconnection"):
        spec = oracle_mod.bcspec(GRID[problem]["bc_kind"], GRID[problem]["bc_flip"])
        U = random_state(shape, 11)
        Uo = U.copy()
        ref.call(problem, "bc_for_u", U, ix, jx)
        L.omo_bc(p(Uo), ix, jx, kx, 2, C.byref(spec))
        assert np.array_equal(U, Uo), problem
        for d, name in ((1, "bc_for_f"), (2, "bc_for_g")):
            VL, VR = random_state(shape, 12 + d), random_state(shape, 14 + d)
            oL, oR = VL.copy(), VR.copy()
            ref.call(problem, name, VL, VR, ix, jx)
            L.omo_facefix(p(oL), p(oR), ix, jx, kx, d, C.byref(spec))
            assert np.array_equal(VL, oL) and np.array_equal(VR, oR), (problem, name)
    U = random_state(shape, 17)
    dx = 0.37
    x, y, z = np.zeros(ix), np.zeros(jx), np.zeros(1)
    L.omo_grid(p(x), ix, -2.0, dx)
    L.omo_grid(p(y), jx, -3.0, dx)
    for d in (1, 2):
        F = np.random.default_rng(d).uniform(-1, 1, (9,) + shape)
        Fo = F.copy()
        ref.call("2D_reconnection", "flux_resistive", F, U, x, y, dx, ix, jx, d)
        L.omo_flux_resistive(p(Fo), p(U), p(x), p(y), p(z), dx, ix, jx, kx, 2, d, 1)
        assert np.array_equal(F, Fo), d
    for dt0 in (0.5, 50.0):
        dt = C.c_double(dt0)
        ref.call("2D_reconnection", "set_dt_resistive", dt, 0.7, 0.35)
        do = C.c_double(dt0)
        L.omo_set_dt_resistive(C.byref(do), 0.7, 0.35, 1)
        assert dt.value == do.value
