"""CPU checks of the oracle itself: golden fixtures, HLLD branch
coverage, limiter known answers, conservation and symmetry properties."""
import math
import os

import numpy as np
import pytest

from helpers import random_state, rel_l1

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "oracle_golden.npz")


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


@pytest.fixture(scope="module")
def mk():
    import importlib.util

    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(os.path.dirname(GOLD), "make_golden.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


def test_golden_runs_reproduce(oracle_mod, gold, mk):
    cases = [("ot32_U0", "ot32_U1", 1, mk.ot_grid(32)), ("ot32_U0", "ot32_U5", 5, mk.ot_grid(32)),
             ("kh32x16_U0", "kh32x16_U3", 3, mk.kh_grid(32, 16)), ("recon_U0", "recon_U2", 2, mk.recon_grid()),
             ("harris_U0", "harris_U2", 2, mk.harris_grid())]
    for a, b, n, g in cases:
        g.U[...] = gold[a]
        g.step(n)
        assert np.all(rel_l1(g.U, gold[b]) <= 1e-13), (a, b)


def test_models_reproduce_golden_initial_states(oracle_mod, gold, mk):
    g = mk.ot_grid(32).model(0)
    np.testing.assert_allclose(g.U, gold["ot32_U0"], rtol=1e-14, atol=1e-15)
    g = mk.kh_grid(32, 16).model(1, amp=0.5, bx0=0.2, pert=0.01, seed=0)
    np.testing.assert_allclose(g.U, gold["kh32x16_U0"], rtol=1e-14, atol=1e-15)
    g = mk.harris_grid().model(2, beta=0.2, amp=2e-3, seed=0)
    np.testing.assert_allclose(g.U, gold["harris_U0"], rtol=1e-13, atol=1e-15)


@pytest.mark.parametrize("name", ["FL", "FR", "HLLCG_L", "HLLCG_R", "Lstar", "Rstar", "Lstar2", "Rstar2"])
@pytest.mark.parametrize("d", [1, 2])
def test_hlld_branch_coverage(oracle_mod, gold, name, d):
    L, R = gold[f"hlld_{name}_d{d}_L"], gold[f"hlld_{name}_d{d}_R"]
    oracle_mod.branch_counts()
    F = oracle_mod.flux_faces(L[:, None], R[:, None], 0.7, d)[:, 0]
    hit = [k for k, v in oracle_mod.branch_counts().items() if v]
    assert hit == [name]
    assert np.array_equal(F, gold[f"hlld_{name}_d{d}_F"])


def _physical_flux(w, d, gamma=5.0 / 3.0):
    vx, vy, vz, p, ro, bx, by, bz, _ = w
    v = np.array([vx, vy, vz])
    B = np.array([bx, by, bz])
    n = d - 1
    B2, v2, vB = B @ B, v @ v, v @ B
    F = np.zeros(9)
    F[4] = ro * v[n]
    F[0:3] = ro * v[n] * v - B[n] * B
    F[n] += p + 0.5 * B2
    F[3] = (0.5 * ro * v2 + gamma / (gamma - 1) * p + B2) * v[n] - vB * B[n]
    F[5:8] = v[n] * B - B[n] * v
    F[5 + n] = 0.0
    return F


@pytest.mark.parametrize("type_", [1, 2, 3, 4])
def test_identical_states_give_physical_flux(oracle_mod, type_):
    rng = np.random.default_rng(7)
    for _ in range(20):
        w = np.array([*rng.uniform(-1, 1, 3), rng.uniform(0.2, 1), rng.uniform(0.5, 2), *rng.uniform(-1, 1, 3), 0.0])
        for d in (1, 2):
            F = oracle_mod.flux_faces(w[:, None], w[:, None], 0.0, d)[:, 0]
            ref = _physical_flux(w, d)
            ref[4 + d] = 0.0  # GLM flux of Bn with psi = 0, ch = 0
            np.testing.assert_allclose(F, ref, rtol=1e-12, atol=1e-12)


def test_limiter_known_answers(gold):
    wk = gold["lim_t1_wk"]
    # minmod, cell 3 (values 1,3,2): opposite slopes -> flat
    assert gold["lim_t1_wL"][3] == 3.0 and gold["lim_t1_wR"][2] == 3.0
    # minmod, cell 2 (values 1,1,3): one zero slope -> flat
    assert gold["lim_t1_wL"][2] == 1.0
    # MC, cell 9 (0.5,0.25,0.125): gA=-0.25, gB=-0.125, gC=-0.09375 -> grad = -0.09375
    assert gold["lim_t2_wL"][9] == 0.25 - 0.09375 and gold["lim_t2_wR"][8] == 0.25 + 0.09375
    # minmod same cell: grad = 0.5*min = -0.0625
    assert gold["lim_t1_wL"][9] == 0.25 - 0.0625
    # flat: face states are the cell values
    assert np.array_equal(gold["lim_t0_wL"][:-1], wk[:-1]) and np.array_equal(gold["lim_t0_wR"][:-1], wk[1:])
    # edge defaults (limiter.f90:82, :103)
    for t in (1, 2, 3, 4):
        assert gold[f"lim_t{t}_wL"][0] == wk[0] and gold[f"lim_t{t}_wR"][-2] == wk[-1]


def test_conservation_periodic(oracle_mod, mk):
    g = mk.ot_grid(32).model(0)
    t0 = g.U[:, 1:-1, 1:-1].sum(axis=(1, 2))
    mag = np.abs(g.U[:, 1:-1, 1:-1]).sum(axis=(1, 2))
    g.step(5)
    t1 = g.U[:, 1:-1, 1:-1].sum(axis=(1, 2))
    assert np.all(np.abs(t1 - t0)[:5] <= 1e-13 * mag[:5])


def test_transpose_symmetry(oracle_mod, mk):
    """x and y code paths agree: transposing the state (x<->y, vx<->vy,
    Bx<->By) commutes with the step to round-off."""
    g = mk.ot_grid(32).model(0)
    h = mk.ot_grid(32)
    perm = [1, 0, 2, 3, 4, 6, 5, 7, 8]
    h.U[...] = g.U[perm].transpose(0, 2, 1)
    g.step(3)
    h.step(3)
    assert np.abs(g.U - h.U[perm].transpose(0, 2, 1)).max() < 1e-13


def test_uniform_state_and_glm_decay(oracle_mod, mk):
    g = mk.ot_grid(16)
    U = random_state((18, 18), 0)
    U[...] = U[:, :1, :1]
    U[8] = 0.3
    g.U[...] = U
    g.step(1)
    f = math.exp(-0.5 * g.last_dt * g.last_ch / 0.2)
    np.testing.assert_allclose(g.U[:8], U[:8], rtol=1e-14, atol=1e-15)
    np.testing.assert_allclose(g.U[8], f * f * 0.3, rtol=1e-14)


def test_negative_pressure_and_small_dt(oracle_mod, mk):
    g = mk.ot_grid(16).model(0)
    g.U[3, 5, 7] = -1.0
    with pytest.raises(oracle_mod.OracleError) as ei:
        g.step(1)
    assert ei.value.code == oracle_mod.NEG_PRESSURE and (ei.value.err.i, ei.value.err.j) == (7, 5)
    g = mk.ot_grid(16).model(0)
    g.cfg.cfl = 1e-12
    with pytest.raises(oracle_mod.OracleError) as ei:
        g.step(1)
    assert ei.value.code == oracle_mod.DT_TOO_SMALL


def test_3d_axis_rotation_symmetry(oracle_mod):
    """x->y->z rotation of a 3D periodic state commutes with the 3D step."""
    n = 10
    U = random_state((n, n, n), 4, smooth=True)
    g = oracle_mod.Grid(3, n, n, n, 0.1, 0.1, 0.1, lm_type=2)
    h = oracle_mod.Grid(3, n, n, n, 0.1, 0.1, 0.1, lm_type=2)
    g.U[...] = U
    g.bc()
    # rotate (x,y,z) -> (y,z,x): new[z,y,x] = old at x'=y... use axis permutation of the array
    perm = [2, 0, 1, 3, 4, 7, 5, 6, 8]  # (mx,my,mz) <- (mz,mx,my)
    h.U[...] = g.U[perm].transpose(0, 2, 3, 1)
    g.step(2)
    h.step(2)
    back = h.U[[1, 2, 0, 3, 4, 6, 7, 5, 8]].transpose(0, 3, 1, 2)
    assert np.abs(g.U - back).max() < 1e-12


def test_more_problem_setups(oracle_mod):
    """Initial states of the 2D reconnection, Brio-Wu and 3D field-loop setups
    (2D_reconnection/model.f90, 1D_basic/model.f90, 3D_basic/model.f90)."""
    import math

    from openmhd_gb300 import brio_wu, field_loop3d, reconnection2d

    cfg, m = brio_wu(40)
    g = oracle_mod.Grid.from_solver_config(cfg).model(m.kind)
    left, right = g.x < 0, g.x >= 0
    assert np.all(g.U[4][:, left] == 1.0) and np.all(g.U[4][:, right] == 0.125)
    assert np.all(g.U[6][:, left] == 1.0) and np.all(g.U[6][:, right] == -1.0) and np.all(g.U[5] == 0.75)
    assert np.allclose(g.U[3][:, left], 0.5 * (0.75**2 + 1) + 1.0 / (5.0 / 3.0 - 1))

    cfg, m = reconnection2d(64, 24)
    g = oracle_mod.Grid.from_solver_config(cfg).model(m.kind, amp=m.amp, beta=m.beta)
    j = 20
    y = g.y[j]
    assert np.allclose(g.U[4][j, 1:-1], 1 + 1 / math.cosh(y) ** 2 / 0.2)
    far = g.x[1:-1] > 30
    assert np.allclose(g.U[5][j, 1:-1][far], math.tanh(y)) and np.all(g.U[0:3] == 0.0)

    cfg, m = field_loop3d(16, 16, 32)
    g = oracle_mod.Grid.from_solver_config(cfg).model(m.kind, amp=m.amp)
    assert np.all(g.U[0] == 1.0) and np.all(g.U[1] == 1.0) and np.all(g.U[2] == 2.0)
    Bmag = np.sqrt((g.U[5:8] ** 2).sum(axis=0))
    assert 5e-4 < Bmag.max() < 5e-3 and np.mean(Bmag == 0.0) > 0.5  # a loop in a field-free box


def test_flop_counting_build(tmp_path):
    """The flop-counting build of the oracle (oracle/flopcount.cpp) compiles
    and counts a plausible per-cell-update cost on both 2D workloads (about
    1.8-1.9 k flops: four HLLD faces, the limiters, u2v, RK and CFL)."""
    import os
    import re
    import subprocess

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    exe = str(tmp_path / "flopcount")
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-o", exe,
                    os.path.join(root, "oracle", "flopcount.cpp")], check=True)
    for args in (["64", "32", "2"], ["48", "48", "2", "ot"]):
        out = subprocess.run([exe] + args, check=True, capture_output=True, text=True).stdout
        f = float(re.search(r"flops_per_cell_update:\s*([0-9.]+)", out).group(1))
        assert 1500.0 < f < 2300.0, (args, f)


@pytest.mark.parametrize("problem", ["kh", "harris3d"])
def test_openmp_build_equals_serial(oracle_mod, monkeypatch, problem):
    """The OpenMP build of the oracle (the CPU baseline and the 4096^2 parity
    reference) runs the same loops as the serial build with only min/max
    reductions across threads, so it gives the same bits."""
    from openmhd_gb300 import harris3d, kelvin_helmholtz

    monkeypatch.setenv("OMP_NUM_THREADS", "4")
    cfg, m = kelvin_helmholtz(64, 48) if problem == "kh" else harris3d(16, 8, 16)
    out = []
    for omp in (False, True):
        g = oracle_mod.Grid.from_solver_config(cfg, omp=omp)
        g.model(m.kind, amp=m.amp, bx0=m.bx0, pert=m.pert, seed=m.seed, beta=m.beta)
        g.step(3)
        out.append((g.U.copy(), g.t, g.last_dt))
    assert np.array_equal(out[0][0], out[1][0]) and out[0][1:] == out[1][1:]


def test_alfven_wave_second_order_convergence(oracle_mod):
    """Physics check of the oracle with no reference data: a circularly
    polarised Alfven wave (an exact nonlinear solution of ideal MHD: rho = 1,
    p = 0.1, Bx = 1, B_perp = 0.1 (sin, cos)(2 pi (x - t)), v_perp = -B_perp)
    carried for one period on a periodic strip with HLLD + MC + TVD-RK2.  The
    L1 error of By against the translated exact solution shrinks at second
    order (limiters clip the wave's smooth extrema on coarse grids, so the
    rate approaches 2 from below)."""
    gamma, amp = 5.0 / 3.0, 0.1

    def run(n):
        dx = 1.0 / n
        g = oracle_mod.Grid(2, n + 2, 6, dx=dx, dy=dx, x0=-0.5 * dx, y0=0.0, cfl=0.4, gamma=gamma,
                            lm_type=2, flux_type=3)

        def state(t):
            ph = 2 * math.pi * (g.x - t)
            by, bz = amp * np.sin(ph), amp * np.cos(ph)
            U = np.zeros(g.shape)
            U[4] = 1.0
            U[1], U[2] = -by, -bz  # rho v_perp = -B_perp / sqrt(rho)
            U[5], U[6], U[7] = 1.0, by, bz
            U[3] = 0.5 * (by**2 + bz**2) + 0.5 * (1.0 + by**2 + bz**2) + 0.1 / (gamma - 1)
            return U

        g.U[...] = state(0.0)
        g.bc()
        g.run_until(1.0)
        return np.abs(g.U[6, 1:-1, 1:-1] - state(g.t)[6, 1:-1, 1:-1]).mean()

    e32, e64, e128 = run(32), run(64), run(128)
    assert e128 < 2.5e-4
    assert math.log2(e32 / e64) > 1.6 and math.log2(e64 / e128) > 1.8, (e32, e64, e128)


def test_alfven_wave_along_z_in_3d(oracle_mod):
    """The same exact Alfven wave travelling along z through the 3D oracle
    (4 x 4 x n periodic box, B_z = 1, B_perp = 0.1 (sin, cos)(2 pi (z - t))):
    second-order convergence of the z-direction flux, limiter and update."""
    gamma, amp = 5.0 / 3.0, 0.1

    def run(n):
        dz = 1.0 / n
        g = oracle_mod.Grid(3, 6, 6, n + 2, dx=dz, dy=dz, dz=dz, z0=-0.5 * dz, cfl=0.4, gamma=gamma,
                            lm_type=2, flux_type=3)

        def state(t):
            ph = 2 * math.pi * (g.z - t)
            b1, b2 = amp * np.sin(ph), amp * np.cos(ph)
            U = np.zeros(g.shape)
            U[4] = 1.0
            U[0], U[1] = -b1[:, None, None], -b2[:, None, None]
            U[5], U[6], U[7] = b1[:, None, None], b2[:, None, None], 1.0
            U[3] = (b1**2 + b2**2 + 0.5 + 0.1 / (gamma - 1))[:, None, None]
            return U

        g.U[...] = state(0.0)
        g.bc()
        g.run_until(1.0)
        return np.abs(g.U[5, 1:-1, 1:-1, 1:-1] - state(g.t)[5, 1:-1, 1:-1, 1:-1]).mean()

    e32, e64, e128 = run(32), run(64), run(128)
    assert e128 < 2.5e-4
    assert math.log2(e32 / e64) > 1.6 and math.log2(e64 / e128) > 1.8, (e32, e64, e128)
