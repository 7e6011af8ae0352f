"""omhd_solver_step_host: host state in, n steps, host state out in one call.
Its results equal put_state + step + get_state bit for bit, whether the host
buffers are page-locked (fused upload + first dt, result written straight to
host memory by the last step) or pageable (the copy path), in place or not,
when the run stops early at tend, and when it continues from the device state."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _reference(cfg, U0, n, t=0.0):
    from openmhd_gb300 import Solver

    s = Solver(cfg).put_state(U0, t)
    s.step(n)
    s.sync()
    return s.get_state_numpy()


def _initial(cfg, model, warm=2):
    from openmhd_gb300 import Solver

    s = Solver(cfg).init_model(model)
    s.step(warm)
    s.sync()
    return s.get_state_numpy()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_step_host_matches_copies(cuda_lib, precision):
    from openmhd_gb300 import Solver, kelvin_helmholtz

    cfg, model = kelvin_helmholtz(96, 40, precision=precision)
    U0 = _initial(cfg, model)
    ref = _reference(cfg, U0, 3)
    s = Solver(cfg)
    # page-locked, in place
    pin = torch.from_numpy(U0.copy()).pin_memory()
    assert s.step_host(pin, n=3) == 0
    assert np.array_equal(pin.numpy(), ref)
    # page-locked, separate output
    pin_in = torch.from_numpy(U0.copy()).pin_memory()
    pin_out = torch.zeros_like(pin_in).pin_memory()
    assert s.step_host(pin_in, pin_out, n=3) == 0
    assert np.array_equal(pin_out.numpy(), ref) and np.array_equal(pin_in.numpy(), U0)
    # pageable numpy arrays
    a = U0.copy()
    assert s.step_host(a, n=3) == 0
    assert np.array_equal(a, ref)


def test_step_host_continues_from_device_state(cuda_lib):
    from openmhd_gb300 import Solver, orszag_tang

    cfg, model = orszag_tang(48)
    U0 = _initial(cfg, model, warm=0)
    ref = _reference(cfg, U0, 4)
    s = Solver(cfg)
    out = torch.zeros(cfg.shape, dtype=torch.float64).pin_memory()
    assert s.step_host(torch.from_numpy(U0.copy()).pin_memory(), out, n=2) == 0
    assert s.step_host(None, out, n=2) == 0
    assert np.array_equal(out.numpy(), ref)
    assert s.sync().steps == 4


def test_step_host_stops_at_tend(cuda_lib):
    """The run reaches tend after the first step: the remaining stage kernels
    skip, the result comes from the device state, as with get_state."""
    from openmhd_gb300 import Solver, orszag_tang

    cfg0, model = orszag_tang(48)
    s0 = Solver(cfg0).init_model(model)
    U0 = s0.get_state_numpy()
    s0.step(1)
    info = s0.sync()
    cfg, _ = orszag_tang(48, tend=0.5 * info.t)  # reached after one step
    ref = _reference(cfg, U0, 3)
    s = Solver(cfg)
    pin = torch.from_numpy(U0.copy()).pin_memory()
    assert s.step_host(pin, n=3) == 0
    assert s.sync().steps == 1
    assert np.array_equal(pin.numpy(), ref)


def test_step_host_3d(cuda_lib):
    from openmhd_gb300 import Solver, field_loop3d

    cfg, model = field_loop3d(24, 20, 36)
    U0 = _initial(cfg, model, warm=1)
    ref = _reference(cfg, U0, 2)
    s = Solver(cfg)
    pin = torch.from_numpy(U0.copy()).pin_memory()
    assert s.step_host(pin, n=2) == 0
    assert np.array_equal(pin.numpy(), ref)
