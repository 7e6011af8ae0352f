"""omhd_solver_create checks its configuration before it touches the GPU, so
the rejections run on any machine: bad arguments give OMHD_BAD_ARG (4) and
resistive runs on unequal spacings OMHD_NOT_SUPPORTED (7), because the
reference's resistive fluxes use one spacing for every direction
(2D_reconnection/flux_resistive.f90, 3D_reconnection_gpu/flux_resistive.cuf)."""
import ctypes as C
import dataclasses

import pytest

from openmhd_gb300.solver import OMHD_BAD_ARG, OMHD_NOT_SUPPORTED


@pytest.fixture(scope="module")
def lib():
    from openmhd_gb300 import _lib
    from openmhd_gb300.build import build

    build()
    return _lib.load()


def _create(lib, cfg):
    h = C.c_void_p()
    st = lib.omhd_solver_create(C.byref(cfg.to_c()), C.byref(h))
    assert not h.value  # nothing is allocated for a rejected configuration
    return st


def test_resistive_needs_equal_spacings(lib):
    from openmhd_gb300 import harris3d, reconnection2d

    cfg, _ = harris3d(9, 6, 10)  # dx, dy, dz = 22.2, 16.7, 20
    assert _create(lib, cfg) == OMHD_NOT_SUPPORTED
    cfg, _ = reconnection2d(12, 6)
    assert _create(lib, dataclasses.replace(cfg, dy=cfg.dx * 1.5)) == OMHD_NOT_SUPPORTED


def test_bad_arguments(lib):
    from openmhd_gb300 import kelvin_helmholtz, orszag_tang

    cfg, _ = orszag_tang(16)
    bad = [
        dataclasses.replace(cfg, ix=3),  # fewer than 2 interior cells
        dataclasses.replace(cfg, nd=4),
        dataclasses.replace(cfg, kx=5),  # 2D with a third extent
        dataclasses.replace(cfg, dx=0.0),
        dataclasses.replace(cfg, dy=float("nan")),
    ]
    kh, _ = kelvin_helmholtz(16, 8)
    bad.append(dataclasses.replace(kh, bc_kind=(0, 0, 0, 1, 0, 0)))  # periodic on one side only
    for c in bad:
        assert _create(lib, c) == OMHD_BAD_ARG, c
    c = cfg.to_c()
    h = C.c_void_p()
    c.lm_type = 5
    assert lib.omhd_solver_create(C.byref(c), C.byref(h)) == OMHD_BAD_ARG
    c = cfg.to_c()
    c.eta_kind = 3
    assert lib.omhd_solver_create(C.byref(c), C.byref(h)) == OMHD_BAD_ARG
    assert lib.omhd_solver_create(C.byref(cfg.to_c()), None) == OMHD_BAD_ARG


def _cfg_array(cfgs):
    from openmhd_gb300 import _lib

    arr = (_lib.Config * len(cfgs))()
    for i, c in enumerate(cfgs):
        arr[i] = c.to_c()
    return arr


def test_ensemble_checks_every_member_first(lib):
    from openmhd_gb300 import harris3d, kelvin_helmholtz, orszag_tang
    from openmhd_gb300.solver import OMHD_BAD_ARG, OMHD_NOT_SUPPORTED

    ot, _ = orszag_tang(32, precision="mixed")
    kh, _ = kelvin_helmholtz(48, 16, precision="mixed")
    h = C.c_void_p()
    cases = [
        ([ot, dataclasses.replace(kh, ix=3)], OMHD_BAD_ARG),  # a bad member anywhere in the list
        ([ot, dataclasses.replace(kh, bc_kind=(1, 0, 1, 1, 0, 0))], OMHD_BAD_ARG),
        ([ot, harris3d(8, 8, 8, precision="mixed")[0]], OMHD_NOT_SUPPORTED),  # 2D members only
        ([dataclasses.replace(ot, precision="fp64_parity")], OMHD_NOT_SUPPORTED),
        ([dataclasses.replace(ot, flux="hll")], OMHD_NOT_SUPPORTED),  # the batched kernel is HLLD
    ]
    for cfgs, code in cases:
        assert lib.omhd_ensemble_create(_cfg_array(cfgs), len(cfgs), C.byref(h)) == code, cfgs
        assert not h.value
    assert lib.omhd_ensemble_create(_cfg_array([ot]), 0, C.byref(h)) == OMHD_BAD_ARG


def test_adjoint_and_noalloc_argument_checks(lib):
    import numpy as np

    from openmhd_gb300 import _lib, field_loop3d, kelvin_helmholtz
    from openmhd_gb300.solver import OMHD_BAD_ARG, OMHD_NOT_SUPPORTED

    kh, _ = kelvin_helmholtz(32, 16)
    h = C.c_void_p()
    assert lib.omhd_adjoint_create(C.byref(kh.to_c()), 0, 1, C.byref(h)) == OMHD_BAD_ARG
    assert lib.omhd_adjoint_create(C.byref(kh.to_c()), 10, 0, C.byref(h)) == OMHD_BAD_ARG
    for c in (dataclasses.replace(kh, limiter="flat"), dataclasses.replace(kh, flux="hllc"),
              dataclasses.replace(kh, time="rk2"), field_loop3d(8, 8, 8)[0]):
        assert lib.omhd_adjoint_create(C.byref(c.to_c()), 10, 5, C.byref(h)) == OMHD_NOT_SUPPORTED, c
    assert not h.value
    U = np.zeros(8)  # never touched: the configuration is refused first
    info = _lib.StepInfo()
    for c in (field_loop3d(8, 8, 8)[0], dataclasses.replace(kh, jx=3),
              dataclasses.replace(kh, bc_kind=(0, 0, 0, 1, 0, 0))):
        st = lib.omhd_step2d_noalloc(U.ctypes.data, C.byref(c.to_c()), 0.0, 1, None, C.byref(info))
        assert st == OMHD_BAD_ARG, c
    # every refusal of the no-alloc step leaves a message for omhd_last_error()
    from openmhd_gb300 import reconnection2d

    rc, _ = reconnection2d(32, 16)
    for c, code, words in ((dataclasses.replace(rc, dy=2 * rc.dx), OMHD_NOT_SUPPORTED, b"equal grid spacings"),
                           (kh, OMHD_BAD_ARG, b"required")):
        lib.omhd_clear_error()
        st = lib.omhd_step2d_noalloc(None if code == OMHD_BAD_ARG else U.ctypes.data, C.byref(c.to_c()), 0.0, 1,
                                     None, C.byref(info))
        e = _lib.ErrorInfo()
        assert st == code and lib.omhd_last_error(C.byref(e)) == code and words in e.message, (st, e.message)
    lib.omhd_clear_error()


def test_routine_wrappers_check_arrays_before_any_gpu_work(lib):
    """The reference-named Python wrappers refuse arrays that are not
    C-contiguous float64, and shapes that are not 2D or 3D planes, before
    anything reaches the device."""
    import numpy as np

    from openmhd_gb300 import routines

    U = np.zeros((9, 6, 7))
    with pytest.raises(TypeError):
        routines.u2v(U.astype(np.float32), np.zeros((4, 6, 7)))
    with pytest.raises(TypeError):
        routines.u2v(np.asfortranarray(U), np.zeros((4, 6, 7)))
    with pytest.raises(ValueError):
        routines.u2v(np.zeros((9, 7)), np.zeros((4, 7)))


def test_routine_wrappers_refuse_undersized_arrays(lib):
    """Every array a wrapper hands to the library must have the shape the
    routine reads or writes, derived from U (or F, wk, VL): an undersized V, F,
    face-state array or coordinate vector is refused before any library call,
    instead of being overrun by a copy or a kernel."""
    import numpy as np

    from openmhd_gb300 import routines

    U = np.zeros((9, 6, 7))
    with pytest.raises(ValueError, match="V has shape"):
        routines.u2v(U, np.zeros((4, 6, 6)))
    with pytest.raises(ValueError, match="V has shape"):
        routines.set_dt(U, np.zeros((3, 6, 7)), 0.1, 0.4)
    with pytest.raises(ValueError, match="wR has shape"):
        routines.limiter(np.zeros((6, 7)), np.zeros((6, 7)), np.zeros((6, 6)), 1, 1)
    with pytest.raises(ValueError, match="VR has shape"):
        routines.flux_solver(np.zeros((9, 6, 7)), np.zeros((9, 6, 7)), np.zeros((9, 5, 7)), 1.0, 1, 3)
    with pytest.raises(ValueError, match="G has shape"):
        routines.rk_tvd21(U, np.zeros_like(U), np.zeros_like(U), np.zeros((9, 6, 6)), dt=0.1, dx=0.1)
    with pytest.raises(ValueError, match="H is required"):
        routines.rk_tvd22(np.zeros((9, 4, 6, 7)), np.zeros((9, 4, 6, 7)), np.zeros((9, 4, 6, 7)),
                          np.zeros((9, 4, 6, 7)), dt=0.1, dx=0.1)
    with pytest.raises(ValueError, match="F has shape"):
        routines.flux_resistive(np.zeros((9, 6, 6)), U, np.zeros(7), np.zeros(6), dx=0.1, dir=1)
    with pytest.raises(ValueError, match="x has shape"):
        routines.flux_resistive(np.zeros_like(U), U, np.zeros(6), np.zeros(6), dx=0.1, dir=1)
    with pytest.raises(ValueError, match="z has shape"):
        U3 = np.zeros((9, 4, 6, 7))
        routines.flux_resistive(np.zeros_like(U3), U3, np.zeros(7), np.zeros(6), np.zeros(3), dx=0.1, dir=1)
    with pytest.raises(ValueError, match="VR has shape"):
        routines.facefix(np.zeros((9, 6, 7)), np.zeros((9, 6, 8)), 1)
    with pytest.raises(ValueError, match="one entry per domain side"):
        routines.bc(U, kind=(0, 0, 0, 0))


def test_step_vjp_arrays_are_checked_on_the_host():
    """The adjoint step's stage inputs are refused in Python unless they are
    contiguous float64 CUDA tensors of the state's shape ({dt, ch, glm} for
    log3): here, without a GPU, every CPU tensor is refused with TypeError."""
    import torch

    from openmhd_gb300.adjoint import _check_device_array

    for a in (torch.zeros(9, 6, 7, dtype=torch.float64), torch.zeros(3), [0.0, 0.0, 0.0]):
        with pytest.raises(TypeError):
            _check_device_array("Un", a, (9, 6, 7))


def test_ensemble_model_count_and_member_index_are_checked_on_the_host():
    """One model per member and member indices in range, refused before the
    library reads a model array or a member handle."""
    from openmhd_gb300.ensemble import Ensemble, batched_problem_set

    cfgs, models = batched_problem_set(4, seed=1)
    ens = Ensemble.__new__(Ensemble)  # the checks run before any GPU work
    ens.cfgs, ens._h = cfgs, None
    with pytest.raises(ValueError):
        ens.init_models(models[:3])
    for i in (-1, 4):
        with pytest.raises(IndexError):
            ens.member_state(i)
