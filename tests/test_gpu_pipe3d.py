"""The warp-specialised FP64 3D stage kernel (k_stage3d_pipe: 3 producer warps
build the ring planes and the x / y / z face states of the next plane while 9
consumer warps solve the faces and update the current one; selected by
omhd_set_3d_pipeline(1), the one-role kernel being the default) against the
oracle and against the one-role 3D kernel.

The two kernels do the same arithmetic except that the pipelined one solves y
and z faces in x orientation (the component order of sums such as B^2
changes), so they agree to rounding, not bit for bit."""
import numpy as np
import pytest

from helpers import assert_parity, random_state, scaled_l1

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _pipelined(cuda_lib):
    """Every test here runs the warp-specialised kernel unless it says
    otherwise; the library default (the one-role kernel) is put back after."""
    cuda_lib.omhd_set_3d_pipeline(1)
    yield
    cuda_lib.omhd_set_3d_pipeline(0)


def _oracle_pair(cfg, model=None, U=None):
    from openmhd_gb300 import Solver
    from oracle.oracle import Grid

    s = Solver(cfg)
    if model is not None:
        s.init_model(model)
    else:
        s.put_state(U)
    g = Grid.from_solver_config(cfg, omp=True)
    g.U[...] = s.get_state_numpy()
    return s, g


@pytest.mark.parametrize("limiter", ["mc", "minmod"])
def test_harris_multichunk_ragged_vs_oracle(cuda_lib, oracle_mod, limiter):
    """Resistive Harris sheet 136x68x136: ragged 16x8 columns in x and y, two
    z chunks (128 and 8 planes), conducting z walls; 1 step within 1e-12 and 3
    steps within 1e-10 of the oracle."""
    from openmhd_gb300 import harris3d

    cfg, model = harris3d(136, 68, 136, precision="fp64", limiter=limiter)
    s, g = _oracle_pair(cfg, model)
    s.step(1)
    info = s.sync()
    g.step(1)
    assert info.status == 0 and abs(info.dt - g.last_dt) <= 1e-14 * g.last_dt
    assert_parity(s.get_state_numpy(), g.U, 1e-12, "1 step")
    s.step(2)
    s.sync()
    g.step(2)
    assert_parity(s.get_state_numpy(), g.U, 1e-10, "3 steps")


def test_walls_on_every_side_vs_oracle(cuda_lib, oracle_mod):
    """Smooth random state on 40x20x30 cells with reflecting walls on all six
    sides (different sign masks per side), MC limiter, resistive (eta of the
    2D reconnection setup, dx = dy = dz): exercises the producers' x, y wall
    fixes and both z walls; 2 steps within 1e-10 of the oracle."""
    from openmhd_gb300 import SolverConfig, flip
    from openmhd_gb300.solver import BX, BY, BZ, MX, MY, MZ, PS

    cfg = SolverConfig(nd=3, ix=42, jx=22, kx=32, dx=0.3, dy=0.3, dz=0.3, x0=-6.0, y0=-3.0, z0=-4.5, limiter="mc",
                       precision="fp64", eta="recon2d", bc_kind=(1, 1, 1, 1, 1, 1),
                       bc_flip=(flip(MX, BY, PS), flip(MX, BZ), flip(MY, BX, PS), flip(MY, BZ),
                                flip(MZ, BX, BY), flip(MZ, PS)))
    U = random_state((32, 22, 42), 13, smooth=True)
    s, g = _oracle_pair(cfg, U=U)
    g.bc()
    s.step(2)
    info = s.sync()
    g.step(2)
    assert info.status == 0
    assert_parity(s.get_state_numpy(), g.U, 1e-10, "walls 3D")


@pytest.mark.parametrize("case", ["harris", "field_loop"])
def test_pipelined_and_one_role_kernels_agree(cuda_lib, case):
    from openmhd_gb300 import Solver, field_loop3d, harris3d

    if case == "harris":
        cfg, model = harris3d(160, 80, 160, precision="fp64")
    else:
        cfg, model = field_loop3d(48, 40, 72, precision="fp64")
    out = []
    for on in (1, 0):
        cuda_lib.omhd_set_3d_pipeline(on)
        try:
            s = Solver(cfg).init_model(model)
            s.step(3)
            info = s.sync()
            assert info.status == 0 and info.steps == 3
            out.append((s.get_state_numpy(), info.t))
        finally:
            cuda_lib.omhd_set_3d_pipeline(1)
    (a, ta), (b, tb) = out
    assert abs(ta - tb) <= 1e-14 * tb
    err = scaled_l1(a, b)
    assert np.all(err <= 1e-12), err
