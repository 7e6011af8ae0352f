"""Edge cases of the fused solver: tiny, odd and non-square grids (one ragged
tile, every cell next to a boundary) against the oracle, and NaN canaries in
the stage buffer U1, which stage 1 must overwrite everywhere it is later read
(ghost cells and corners included) before stage 2 reads it."""
import numpy as np
import pytest

from helpers import scaled_l1

pytestmark = pytest.mark.gpu

CASES = ["ot8", "ot9x7", "kh9x7", "kh40x24", "recon12x6", "loop9x7x5"]


def _setup(name, precision):
    from openmhd_gb300 import field_loop3d, kelvin_helmholtz, orszag_tang, reconnection2d

    return {
        "ot8": lambda: orszag_tang(8, precision=precision),
        "ot9x7": lambda: orszag_tang(9, 7, precision=precision),
        "kh9x7": lambda: kelvin_helmholtz(9, 7, precision=precision),
        "kh40x24": lambda: kelvin_helmholtz(40, 24, precision=precision),
        "recon12x6": lambda: reconnection2d(12, 6, precision=precision),
        "loop9x7x5": lambda: field_loop3d(9, 7, 5, precision=precision),
    }[name]()


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("precision,tol", [("fp64_parity", 1e-12), ("fp64", 1e-10)])
def test_tiny_and_odd_grids_vs_oracle(cuda_lib, oracle_mod, name, precision, tol):
    from openmhd_gb300 import Solver
    from oracle.oracle import Grid

    cfg, model = _setup(name, precision)
    s = Solver(cfg).init_model(model)
    g = Grid.from_solver_config(cfg)
    g.U[...] = s.get_state_numpy()
    s.step(3)
    info = s.sync()
    g.step(3)
    assert info.status == 0 and info.steps == 3
    err = scaled_l1(s.get_state_numpy(), g.U)
    assert np.all(err <= tol), (name, err)


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_stage_buffer_nan_canaries(cuda_lib, name, precision):
    import torch

    from openmhd_gb300 import Solver

    cfg, model = _setup(name, precision)
    a = Solver(cfg).init_model(model)
    b = Solver(cfg).init_model(model)
    b.U1.fill_(float("nan"))
    a.step(3)
    b.step(3)
    ia, ib = a.sync(), b.sync()
    assert ia.status == 0 and ib.status == 0 and ia.steps == ib.steps == 3
    assert not torch.isnan(b.U).any()
    assert torch.equal(a.U, b.U)
