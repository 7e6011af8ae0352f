"""Fused-step parity: the GB300 solver (two fused stage kernels per TVD-RK2
step) against the CPU oracle's restatement of the reference driver loop
(2D_basic/main.f90:56-188) from the same initial state.

Tolerances: FP64 path within 1e-12 relative L1 per variable after
one step and 1e-9 after N steps; the no-contraction parity build is compared
at 1e-13 (its only departure from the oracle's op sequence is the device exp()
in the GLM factor); the FP32-mixed path within 1e-6 L1 of FP64.  The L1 error
of each variable is normalised by the L1 norm of its physical scale
(helpers.scaled_l1: momentum components by |m|, field components and psi by
|B|), so that components that are ~0 (psi, By, vy early in a run) are not
measured against their own round-off."""
import numpy as np
import pytest

from helpers import interior, rel_l1, scaled_l1

pytestmark = pytest.mark.gpu


def _pair(cfg, model, oracle_mod):
    from openmhd_gb300 import Solver
    from oracle.oracle import Grid

    s = Solver(cfg).init_model(model)
    g = Grid.from_solver_config(cfg)
    g.U[...] = s.get_state_numpy()  # identical initial state on both sides
    return s, g


def _cmp(s, g, tol, label=""):
    U = s.get_state_numpy()
    err = scaled_l1(U, g.U)
    assert np.all(err <= tol), f"{label} scaled L1 per var {err} (own-norm rel L1 {rel_l1(U, g.U)})"
    return err


@pytest.mark.parametrize("precision,tol1,tolN", [("fp64_parity", 1e-13, 1e-12), ("fp64", 1e-12, 1e-9)])
def test_orszag_tang_vs_oracle(cuda_lib, oracle_mod, precision, tol1, tolN):
    from openmhd_gb300 import orszag_tang

    cfg, model = orszag_tang(64, precision=precision)
    s, g = _pair(cfg, model, oracle_mod)
    s.step(1)
    info = s.sync()
    g.step(1)
    assert info.steps == 1 and info.status == 0
    assert abs(info.dt - g.last_dt) <= 1e-15 * g.last_dt
    _cmp(s, g, tol1, "1 step")
    s.step(9)
    s.sync()
    g.step(9)
    _cmp(s, g, tolN, "10 steps")


def test_orszag_tang_4096sq_fp64_vs_oracle(cuda_lib, oracle_mod):
    """The FP64 gate at the 4096^2 size: Orszag-Tang 4096x4096 (HLLD, MC, GLM,
    periodic) on the performance build, 1 step within 1e-12 and 10 steps within
    1e-9 scaled L1 per variable of the oracle (its OpenMP build, which runs the
    same loops as the serial one), from the same initial state."""
    from openmhd_gb300 import Solver, orszag_tang
    from oracle.oracle import Grid

    cfg, model = orszag_tang(4096, precision="fp64")
    assert (cfg.limiter, cfg.flux) == ("mc", "hlld")
    s = Solver(cfg).init_model(model)
    g = Grid.from_solver_config(cfg, omp=True)
    g.U[...] = s.get_state_numpy()
    s.step(1)
    info = s.sync()
    g.step(1)
    assert info.status == 0 and abs(info.dt - g.last_dt) <= 1e-14 * g.last_dt
    _cmp(s, g, 1e-12, "4096^2, 1 step")
    s.step(9)
    info = s.sync()
    g.step(9)
    assert info.status == 0 and info.steps == 10
    _cmp(s, g, 1e-9, "4096^2, 10 steps")


@pytest.mark.parametrize("flux", ["llf", "hll", "hllc", "hlld", "lhlld"])
@pytest.mark.parametrize("limiter", ["flat", "minmod", "mc", "vanleer", "koren"])
def test_scheme_matrix_parity(cuda_lib, oracle_mod, flux, limiter):
    from openmhd_gb300 import orszag_tang

    cfg, model = orszag_tang(32, 24, precision="fp64_parity", flux=flux, limiter=limiter)
    s, g = _pair(cfg, model, oracle_mod)
    s.step(3)
    s.sync()
    g.step(3)
    _cmp(s, g, 1e-13, f"{flux}/{limiter}")


@pytest.mark.parametrize("precision", ["fp64_parity", "fp64"])
def test_kelvin_helmholtz_walls_anisotropic(cuda_lib, oracle_mod, precision):
    from openmhd_gb300 import kelvin_helmholtz

    cfg, model = kelvin_helmholtz(96, 40, precision=precision)
    s, g = _pair(cfg, model, oracle_mod)
    s.step(5)
    s.sync()
    g.step(5)
    _cmp(s, g, 1e-12 if precision == "fp64_parity" else 1e-10, "KH")


@pytest.mark.parametrize("problem,limiter", [("kh", "minmod"), ("ot", "mc")])
def test_many_tiles_per_sm_vs_oracle(cuda_lib, oracle_mod, problem, limiter):
    """Grids with several 16x16 tiles per SM (with ragged edge tiles), so that
    the persistent FP64 kernel walks tile sequences and reuses both of its
    face-state buffers: KH 560x300 (walls in y) with minmod and Orszag-Tang
    416x280 (periodic) with MC, 1 step and 5 steps against the oracle."""
    from openmhd_gb300 import kelvin_helmholtz, orszag_tang

    if problem == "kh":
        cfg, model = kelvin_helmholtz(560, 300, precision="fp64")
    else:
        cfg, model = orszag_tang(416, 280, precision="fp64", limiter=limiter)
    assert cfg.limiter == limiter
    s, g = _pair(cfg, model, oracle_mod)
    s.step(1)
    info = s.sync()
    g.step(1)
    assert info.status == 0 and abs(info.dt - g.last_dt) <= 1e-14 * g.last_dt
    _cmp(s, g, 1e-12, "1 step")
    s.step(4)
    s.sync()
    g.step(4)
    _cmp(s, g, 1e-9, "5 steps")


def test_reconnection_walls_resistive_std_rk2(cuda_lib, oracle_mod):
    """2D_reconnection-style walls (sign flips on every side) + resistive fluxes
    (2D_reconnection/flux_resistive.f90) + standard RK2 (rk_std21/22)."""
    from openmhd_gb300 import ModelSpec, SolverConfig, flip
    from openmhd_gb300.solver import BX, BY, BZ, MX, MY, MZ, PS

    cfg = SolverConfig(nd=2, ix=50, jx=42, dx=0.25, dy=0.25, x0=-6.0, y0=-5.0, limiter="mc", flux="hlld",
                       eta="recon2d", time="rk2", precision="fp64_parity",
                       bc_kind=(1, 1, 1, 1, 0, 0),
                       bc_flip=(flip(MX, MZ, BY, PS), flip(MX, MZ, BY, PS), flip(MY, MZ, BX, PS), flip(MY, BY), 0, 0))
    s, g = _pair(cfg, ModelSpec(kind=1, amp=0.3, bx0=0.5, pert=0.05, seed=3), oracle_mod)
    s.step(4)
    s.sync()
    g.step(4)
    _cmp(s, g, 1e-12, "reconnection")


def test_run_until_matches_reference_step_count(cuda_lib, oracle_mod):
    from openmhd_gb300 import orszag_tang

    cfg, model = orszag_tang(32, precision="fp64")
    s, g = _pair(cfg, model, oracle_mod)
    info = s.run_until(0.3, batch=7)
    g.run_until(0.3)
    assert info.steps == g.steps and info.done == 1
    assert abs(info.t - g.t) <= 1e-13


def test_conservation_periodic_full_size(cuda_lib):
    """Mass, momentum and energy totals are conserved to round-off on a periodic
    grid (size-independent property; 4096^2 Orszag-Tang)."""
    import torch
    from openmhd_gb300 import orszag_tang

    cfg, model = orszag_tang(4096, precision="fp64")
    from openmhd_gb300 import Solver

    s = Solver(cfg).init_model(model)
    s.sync()
    tot0 = s.U[:, 1:-1, 1:-1].sum(dim=(1, 2)).cpu().numpy()
    mag = s.U[:, 1:-1, 1:-1].abs().sum(dim=(1, 2)).cpu().numpy()
    s.step(3)
    info = s.sync()
    assert info.status == 0 and info.steps == 3
    tot1 = s.U[:, 1:-1, 1:-1].sum(dim=(1, 2)).cpu().numpy()
    for v in (0, 1, 2, 3, 4):  # mx, my, mz, E, rho
        assert abs(tot1[v] - tot0[v]) <= 1e-12 * mag[v], (v, tot1[v] - tot0[v])
    torch.cuda.synchronize()


def test_mixed_precision_error_vs_fp64(cuda_lib):
    from openmhd_gb300 import Solver, kelvin_helmholtz

    cfg64, model = kelvin_helmholtz(256, 128, precision="fp64")
    cfgmx, _ = kelvin_helmholtz(256, 128, precision="mixed")
    a = Solver(cfg64).init_model(model)
    b = Solver(cfgmx).init_model(model)
    a.step(20)
    b.step(20)
    a.sync()
    b.sync()
    err = scaled_l1(interior(b.get_state_numpy()), interior(a.get_state_numpy()))
    assert np.all(err <= 1e-6), err


def test_mixed_precision_both_u2v_branches_vs_fp64(cuda_lib):
    """Orszag-Tang 256^2 with a 1.5x field (the batched set's strongest): the
    FP32-mixed path recovers the primitives in binary32 where the internal
    energy is at least the kinetic plus magnetic energy and in FP64 elsewhere;
    this state holds cells of both kinds, and the mixed run stays within 1e-6
    (scaled L1) of FP64 after 20 steps."""
    from openmhd_gb300 import Solver, orszag_tang

    cfg64, model = orszag_tang(256, precision="fp64", amp=1.5)
    cfgmx, _ = orszag_tang(256, precision="mixed", amp=1.5)
    a = Solver(cfg64).init_model(model)
    b = Solver(cfgmx).init_model(model)
    U = interior(a.get_state_numpy())
    rv2 = (U[0] ** 2 + U[1] ** 2 + U[2] ** 2) / U[4]
    B2 = U[5] ** 2 + U[6] ** 2 + U[7] ** 2
    fp64_cells = float(np.mean(U[3] < rv2 + B2))
    assert 0.05 < fp64_cells < 0.95, fp64_cells
    a.step(20)
    b.step(20)
    ia, ib = a.sync(), b.sync()
    assert ia.status == 0 and ib.status == 0 and ia.steps == ib.steps == 20
    err = scaled_l1(interior(b.get_state_numpy()), interior(a.get_state_numpy()))
    print(f"share of FP64-recovered cells {fp64_cells:.2f}; max scaled L1 {err.max():.2e}")
    assert np.all(err <= 1e-6), err


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("var,value,status", [(3, -5.0, 1), (4, -0.5, 2)])
def test_negative_pressure_is_reported_not_trapped(cuda_lib, precision, var, value, status):
    """E < 0 (negative pressure) or rho < 0 (negative density) in one cell is
    reported with the cell's Fortran index (u2v.f90:34-43), in FP64 and in the
    FP32-mixed path (whose binary32 recovery hands every such cell to the FP64
    recovery, or, for rho < 0, reports it from its own binary32 values)."""
    from openmhd_gb300 import Solver, orszag_tang

    cfg, model = orszag_tang(32, precision=precision)
    s = Solver(cfg).init_model(model)
    U = s.get_state_numpy()
    U[var, 10, 12] = value  # at Fortran (13, 11)
    s.put_state(U)
    s.step(2)
    import ctypes as C
    from openmhd_gb300 import _lib

    si = _lib.StepInfo()
    st = s.lib.omhd_solver_sync(s._h, C.byref(si))
    assert st == status and si.status == status
    e = _lib.ErrorInfo()
    s.lib.omhd_solver_last_error(s._h, C.byref(e))
    assert (e.i, e.j) == (13, 11)
    assert si.steps == 0  # the state is not advanced past the failure
    # the context is still usable
    s.put_state(Solver(cfg).init_model(model).get_state_numpy())
    s.step(1)
    assert s.sync().status == 0


def test_graph_replay_matches_stream_launches(cuda_lib):
    from openmhd_gb300 import Solver, orszag_tang

    cfg, model = orszag_tang(128)
    a = Solver(cfg).init_model(model)
    b = Solver(cfg).init_model(model)
    a.step(8)
    b.step_graph(4, replays=2)
    ia, ib = a.sync(), b.sync()
    assert ia.steps == ib.steps == 8
    assert np.array_equal(a.get_state_numpy(), b.get_state_numpy())


@pytest.mark.parametrize("precision,tol", [("fp64_parity", 1e-12), ("fp64", 1e-10)])
def test_harris3d_resistive_vs_oracle(cuda_lib, oracle_mod, precision, tol):
    """3D resistive Harris sheet (conducting z walls, periodic x/y) on a small grid."""
    from openmhd_gb300 import harris3d

    cfg, model = harris3d(24, 12, 24, precision=precision)
    s, g = _pair(cfg, model, oracle_mod)
    s.step(3)
    info = s.sync()
    g.step(3)
    assert info.status == 0 and info.steps == 3
    _cmp(s, g, tol, "harris3d")


@pytest.mark.parametrize("precision,tol", [("fp64_parity", 1e-12), ("fp64", 1e-10)])
def test_harris3d_resistive_multichunk_vs_oracle(cuda_lib, oracle_mod, precision, tol):
    """Resistive Harris sheet on 136x68x136 (dx = dy = dz): five CTA columns
    across x (one ragged) and three z chunks, with the resistivity peak at
    x = z = 0 inside the third column and the second chunk, so the resistivity
    at the face positions of a column and chunk away from the origin
    (tabulated per CTA in the FAST builds) meets the oracle's per-face
    formula."""
    from openmhd_gb300 import harris3d

    cfg, model = harris3d(136, 68, 136, precision=precision)
    s, g = _pair(cfg, model, oracle_mod)
    s.step(3)
    info = s.sync()
    g.step(3)
    assert info.status == 0 and info.steps == 3
    _cmp(s, g, tol, "harris3d multichunk")


def test_harris3d_mixed_error_vs_fp64(cuda_lib):
    """FP32-mixed 3D (resistive Harris sheet 136x68x136, two CTAs per SM)
    within 1e-6 scaled L1 per variable of the FP64 path after 10 steps."""
    from openmhd_gb300 import Solver, harris3d

    cfg64, model = harris3d(136, 68, 136, precision="fp64")
    cfgmx, _ = harris3d(136, 68, 136, precision="mixed")
    a = Solver(cfg64).init_model(model)
    b = Solver(cfgmx).init_model(model)
    a.step(10)
    b.step(10)
    ia, ib = a.sync(), b.sync()
    assert ia.status == 0 and ib.status == 0 and ia.steps == ib.steps == 10
    err = scaled_l1(interior(b.get_state_numpy()), interior(a.get_state_numpy()))
    assert np.all(err <= 1e-6), err


def test_3d_periodic_multichunk_vs_oracle(cuda_lib, oracle_mod):
    """Random smooth periodic 3D state with more z planes than one CTA marches
    (chunk boundaries), MC limiter, no resistivity."""
    from openmhd_gb300 import Solver, SolverConfig
    from oracle.oracle import Grid
    from helpers import random_state

    cfg = SolverConfig(nd=3, ix=12, jx=10, kx=140, dx=0.1, dy=0.1, dz=0.1, limiter="mc", precision="fp64_parity")
    U = random_state((140, 10, 12), 5, smooth=True)
    s = Solver(cfg).put_state(U)
    g = Grid.from_solver_config(cfg)
    g.U[...] = U
    g.bc()
    s.step(2)
    s.sync()
    g.step(2)
    _cmp(s, g, 1e-12, "3d periodic")


@pytest.mark.parametrize("precision,tol", [("fp64_parity", 1e-12), ("fp64", 1e-10)])
def test_reconnection2d_symmetry_walls_vs_oracle(cuda_lib, oracle_mod, precision, tol):
    """2D_reconnection: Harris sheet + X-point perturbation, resistive, all four
    walls with the reference's sign flips (2D_reconnection/bc.f90:6-50)."""
    from openmhd_gb300 import reconnection2d

    cfg, model = reconnection2d(96, 32, precision=precision)
    s, g = _pair(cfg, model, oracle_mod)
    s.step(6)
    s.sync()
    g.step(6)
    _cmp(s, g, tol, "reconnection2d")


def test_brio_wu_to_tend_vs_oracle(cuda_lib, oracle_mod):
    """Brio-Wu shock tube run to t = 0.2 as in 1D_basic/main.f90 (cfl 0.8):
    same step count, states within the N-step tolerance."""
    from openmhd_gb300 import brio_wu

    cfg, model = brio_wu(200, precision="fp64")
    s, g = _pair(cfg, model, oracle_mod)
    info = s.run_until(cfg.tend)
    g.run_until(cfg.tend)
    assert info.steps == g.steps and abs(info.t - g.t) <= 1e-12
    _cmp(s, g, 1e-9, "brio-wu")
    U = s.get_state_numpy()
    assert np.array_equal(U[:, 1, :], U[:, 2, :])  # the strip stays one-dimensional


def test_field_loop3d_vs_oracle(cuda_lib, oracle_mod):
    """3D_basic field-loop advection, all periodic (3D_basic/bc.f90)."""
    from openmhd_gb300 import field_loop3d

    cfg, model = field_loop3d(24, 20, 40, precision="fp64")
    s, g = _pair(cfg, model, oracle_mod)
    s.step(4)
    s.sync()
    g.step(4)
    _cmp(s, g, 1e-10, "field loop")
