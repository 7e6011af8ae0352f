"""The allocation-free fused 2D step (omhd_step2d_noalloc) against the
ordinary fused solver entry points, through the C ABI.

This entry point exists for callers that cannot call cudaMalloc (a driver
inside an application that owns the whole device memory pool, or a job that
must reserve all device memory at load time): its scratch lives in a fixed
static device array.  Each check runs two calls in a row, because every call
reuses the same array and must clear what has to start at zero.  The file is
named to be collected last, and it passes both alone in a fresh process and
after the other tests."""
import ctypes as C

import numpy as np
import pytest

from helpers import scaled_l1

pytestmark = pytest.mark.gpu

TOL = 1e-12  # FP64 one-step tolerance of the parity tests


def _reference_run(lib, cfg_c, U0, t0, nsteps):
    """The existing entry points: create, put_state, step, sync, get_state."""
    h = C.c_void_p()
    assert lib.omhd_solver_create(C.byref(cfg_c), C.byref(h)) == 0
    try:
        assert lib.omhd_solver_put_state(h, U0.ctypes.data, t0) == 0
        assert lib.omhd_solver_step(h, nsteps) == 0
        from openmhd_gb300 import _lib

        info = _lib.StepInfo()
        assert lib.omhd_solver_sync(h, C.byref(info)) == 0
        out = np.empty_like(U0)
        assert lib.omhd_solver_get_state(h, out.ctypes.data) == 0
        return out, info
    finally:
        lib.omhd_solver_destroy(h)


@pytest.mark.parametrize("problem", ["ot", "kh_mixed", "recon_resistive"])
def test_noalloc_step_matches_solver_twice(cuda_lib, problem):
    import torch

    from openmhd_gb300 import ModelSpec, Solver, SolverConfig, _lib, flip, kelvin_helmholtz, orszag_tang
    from openmhd_gb300.solver import BX, BY, MX, MY, MZ, PS

    lib = cuda_lib
    if problem == "ot":
        cfg, model = orszag_tang(96, 80, precision="fp64")
    elif problem == "kh_mixed":
        cfg, model = kelvin_helmholtz(128, 64, precision="mixed")
    else:
        cfg = SolverConfig(nd=2, ix=66, jx=50, dx=0.25, dy=0.25, x0=-8.0, y0=-6.0, limiter="mc", eta="recon2d",
                           precision="fp64", bc_kind=(1, 1, 1, 1, 0, 0),
                           bc_flip=(flip(MX, MZ, BY, PS), flip(MX, MZ, BY, PS), flip(MY, MZ, BX, PS), flip(MY, BY),
                                    0, 0))
        model = ModelSpec(kind=1, amp=0.3, bx0=0.5, pert=0.05, seed=4)
    U0 = Solver(cfg).init_model(model).get_state_numpy()
    cfg_c = cfg.to_c()
    U_dev = torch.from_numpy(U0.copy()).cuda()
    stream = torch.cuda.current_stream()
    t = 0.0
    ref_in = U0.copy()
    for call in range(2):  # two calls in a row on the same static scratch
        info = _lib.StepInfo()
        st = lib.omhd_step2d_noalloc(U_dev.data_ptr(), C.byref(cfg_c), t, 3, C.c_void_p(stream.cuda_stream),
                                     C.byref(info))
        assert st == 0 and info.status == 0 and info.steps == 3, (call, st, info.status)
        ref_out, ref_info = _reference_run(lib, cfg_c, ref_in, t, 3)
        got = U_dev.cpu().numpy()
        err = scaled_l1(got, ref_out)
        assert np.all(err <= TOL), (call, err)
        assert abs(info.t - ref_info.t) <= 1e-14 * max(1.0, abs(ref_info.t))
        t = info.t
        ref_in = ref_out


def test_noalloc_rejects_grid_beyond_fixed_scratch(cuda_lib):
    import torch

    from openmhd_gb300 import _lib, orszag_tang

    lib = cuda_lib
    cap = int(lib.omhd_step2d_noalloc_max_doubles())
    n = int((cap / 9) ** 0.5) + 16  # square grid whose stage buffer alone exceeds the array
    cfg, _ = orszag_tang(n)
    cfg_c = cfg.to_c()
    U = torch.zeros(cfg.shape, dtype=torch.float64, device="cuda")
    info = _lib.StepInfo()
    lib.omhd_clear_error()
    st = lib.omhd_step2d_noalloc(U.data_ptr(), C.byref(cfg_c), 0.0, 1, None, C.byref(info))
    assert st == 4  # OMHD_BAD_ARG
    e = _lib.ErrorInfo()
    lib.omhd_last_error(C.byref(e))
    assert b"scratch" in e.message
    lib.omhd_clear_error()


def test_noalloc_reports_device_failure_with_cell(cuda_lib):
    """A failure the stage kernels record (here negative pressure) comes back
    from the call as its status and through omhd_last_error() with the
    1-based cell and the value, as the solver's sync reports it."""
    import torch

    from openmhd_gb300 import Solver, _lib, orszag_tang

    lib = cuda_lib
    cfg, model = orszag_tang(32)
    U0 = Solver(cfg).init_model(model).get_state_numpy()
    U0[3, 10, 12] = -5.0  # E < 0 at Fortran (13, 11)
    U = torch.from_numpy(U0).cuda()
    cfg_c = cfg.to_c()
    lib.omhd_clear_error()
    info = _lib.StepInfo()
    st = lib.omhd_step2d_noalloc(U.data_ptr(), C.byref(cfg_c), 0.0, 2, None, C.byref(info))
    e = _lib.ErrorInfo()
    assert st == 1 and info.status == 1 and info.steps == 0
    assert lib.omhd_last_error(C.byref(e)) == 1 and (e.i, e.j) == (13, 11), (e.i, e.j, e.message)
    assert b"negative pressure at 13 11" in e.message
    lib.omhd_clear_error()
    # the next call on the shared scratch starts clean
    U1 = torch.from_numpy(Solver(cfg).init_model(model).get_state_numpy()).cuda()
    st = lib.omhd_step2d_noalloc(U1.data_ptr(), C.byref(cfg_c), 0.0, 2, None, C.byref(info))
    assert st == 0 and info.status == 0 and info.steps == 2
