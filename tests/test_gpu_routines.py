"""Routine-level parity: each reference-named C-ABI entry point against the CPU
oracle on the same seeded inputs.  These kernels are built without FMA
contraction, so results are compared for exact equality except where a
transcendental evaluated on the device (cosh/exp in the resistivity) enters."""
import ctypes as C

import numpy as np
import pytest

from helpers import random_state
from oracle import oracle

pytestmark = pytest.mark.gpu

SHAPES = [(29, 37), (7, 9, 11)]  # (jx, ix) and (kx, jx, ix)


def _dims(shape):
    if len(shape) == 2:
        return 2, shape[1], shape[0], 1
    return 3, shape[2], shape[1], shape[0]


def _p(a):
    return a.ctypes.data


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("where", ["host", "device"])
def test_u2v(cuda_lib, oracle_mod, shape, where):
    import torch
    from openmhd_gb300 import routines

    U = random_state(shape, seed=1)
    nd = len(shape)
    Vref, st, _ = oracle_mod.u2v(U, nd)
    assert st == 0
    if where == "host":
        V = np.zeros_like(Vref)
        routines.u2v(U, V)
    else:
        Ut = torch.from_numpy(U).cuda()
        Vt = torch.zeros(Vref.shape, dtype=torch.float64, device="cuda")
        routines.u2v(Ut, Vt)
        V = Vt.cpu().numpy()
    assert np.array_equal(V, Vref)


def test_u2v_negative_pressure_reports_minloc(cuda_lib, oracle_mod):
    from openmhd_gb300 import OmhdError, routines

    U = random_state((12, 10), seed=2)
    U[3, 7, 4] = 0.0  # energy 0 -> p < 0 at Fortran (5, 8)
    U[3, 2, 6] = -100.0  # deeper minimum at Fortran (7, 3)
    V = np.zeros((4, 12, 10))
    with pytest.raises(OmhdError) as ei:
        routines.u2v(U, V)
    assert ei.value.code == 1
    assert "negative pressure at 7 3" in str(ei.value)
    Vref, st, e = oracle_mod.u2v(U, 2)
    assert st == 1 and (e.i + 1, e.j + 1) == (7, 3)


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("type_", [0, 1, 2, 3, 4])
def test_limiter(cuda_lib, oracle_mod, shape, type_):
    from openmhd_gb300 import routines

    L = oracle_mod.lib()
    nd, ix, jx, kx = _dims(shape)
    rng = np.random.default_rng(3 + type_)
    wk = rng.uniform(-1, 1, shape)
    # exact kinks, plateaus and signed zeros
    flat = wk.reshape(-1)
    flat[::7] = 0.25
    flat[1::11] = -0.0
    flat[2::13] = flat[3::13][: len(flat[2::13])]
    for d in range(1, nd + 1):
        wL = np.full(shape, 7.0)
        wR = np.full(shape, -7.0)
        rL, rR = wL.copy(), wR.copy()
        L.omo_limiter(_p(wk), _p(rL), _p(rR), ix, jx, kx, d, type_)
        routines.limiter(wk, wL, wR, d, type_)
        assert np.array_equal(wL, rL), (d, type_)
        assert np.array_equal(wR, rR), (d, type_)


def _face_states(shape, seed):
    """VL/VR pairs mixing near-equal, strongly different and supersonic states."""
    rng = np.random.default_rng(seed)
    U = random_state(shape, seed=seed)
    V, _, _ = oracle.u2v(U, len(shape))
    VL = np.concatenate([V, U[4:9]], axis=0).copy()
    VR = VL * (1.0 + rng.uniform(-0.3, 0.3, VL.shape))
    VR[4] = np.abs(VR[4]) + 0.1
    VR[3] = np.abs(VR[3]) + 0.05
    flat = VL.reshape(9, -1)
    fr = VR.reshape(9, -1)
    fr[:, ::5] = flat[:, ::5]                 # identical states
    fr[0, 1::9] += 6.0
    flat[0, 1::9] += 6.0                      # supersonic to the right -> F = F(L)
    fr[0, 2::9] -= 6.0
    flat[0, 2::9] -= 6.0                      # supersonic to the left  -> F = F(R)
    fr[5:8, 3::9] *= 1e-3                     # weak field -> HLLC-G fallback
    flat[5:8, 3::9] *= 1e-3
    return np.ascontiguousarray(VL), np.ascontiguousarray(VR)


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("type_", [0, 1, 2, 3, 4])
def test_flux_solver(cuda_lib, oracle_mod, shape, type_):
    import torch
    from openmhd_gb300 import routines

    L = oracle_mod.lib()
    nd, ix, jx, kx = _dims(shape)
    VL, VR = _face_states(shape, 10 + type_)
    ch = 1.7
    for d in range(1, nd + 1):
        Fref = np.full((9,) + shape, 3.0)
        L.omo_flux_solver(_p(Fref), _p(VL), _p(VR), ch, ix, jx, kx, d, type_)
        Ft = torch.full((9,) + shape, 5.0, dtype=torch.float64, device="cuda")
        routines.flux_solver(Ft, torch.from_numpy(VL).cuda(), torch.from_numpy(VR).cuda(), ch, d, type_)
        F = Ft.cpu().numpy()
        both_nan = np.isnan(F) & np.isnan(Fref)
        assert np.array_equal(np.where(both_nan, 0, F), np.where(both_nan, 0, Fref)), (d, type_)


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("name", ["rk_tvd21", "rk_tvd22", "rk_std21", "rk_std22"])
def test_rk(cuda_lib, oracle_mod, shape, name):
    from openmhd_gb300 import routines

    L = oracle_mod.lib()
    nd, ix, jx, kx = _dims(shape)
    rng = np.random.default_rng(4)
    U = random_state(shape, 5)
    U1 = random_state(shape, 6)
    F, G, H = (rng.uniform(-1, 1, (9,) + shape) for _ in range(3))
    dt, dx = 0.0123, 0.05
    Ur, U1r = U.copy(), U1.copy()
    fn = getattr(L, "omo_" + name)
    if name == "rk_std22":
        fn(_p(Ur), _p(F), _p(G), _p(H), dt, dx, dx, dx, ix, jx, kx, nd)
        getattr(routines, name)(U, F, G, H if nd == 3 else None, dt=dt, dx=dx)
    else:
        fn(_p(Ur), _p(U1r), _p(F), _p(G), _p(H), dt, dx, dx, dx, ix, jx, kx, nd)
        getattr(routines, name)(U, U1, F, G, H if nd == 3 else None, dt=dt, dx=dx)
    assert np.array_equal(U, Ur)
    assert np.array_equal(U1, U1r)


@pytest.mark.parametrize("shape", SHAPES)
def test_glm_and_set_dt(cuda_lib, oracle_mod, shape):
    from openmhd_gb300 import routines

    L = oracle_mod.lib()
    nd, ix, jx, kx = _dims(shape)
    U = random_state(shape, 7)
    Ur = U.copy()
    L.omo_glm_ss2(_p(Ur), 1.3, 0.02, ix, jx, kx)
    routines.glm_ss2(U, 1.3, 0.02)
    assert np.array_equal(U, Ur)
    V, _, _ = oracle_mod.u2v(U, nd)
    vm, dt = C.c_double(), C.c_double()
    e = oracle_mod.Err()
    L.omo_set_dt(_p(U), _p(V), C.byref(vm), C.byref(dt), 0.05, 0.05, 0.05, 0.4, ix, jx, kx, nd, C.byref(e))
    vmax, dtg = routines.set_dt(U, V, 0.05, 0.4)
    assert vmax == vm.value and dtg == dt.value


def test_set_dt_too_small(cuda_lib):
    from openmhd_gb300 import OmhdError, routines

    U = random_state((10, 12), 8)
    V = np.zeros((4, 10, 12))
    routines.u2v(U, V)
    with pytest.raises(OmhdError) as ei:
        routines.set_dt(U, V, 1e-9, 0.4)
    assert ei.value.code == 3


@pytest.mark.parametrize("shape", SHAPES)
def test_bc_and_facefix(cuda_lib, oracle_mod, shape):
    from openmhd_gb300 import routines

    L = oracle_mod.lib()
    nd, ix, jx, kx = _dims(shape)
    kinds = [(0, 0, 1, 1, 1, 1), (1, 1, 0, 0, 1, 1), (0, 0, 0, 0, 0, 0)]
    flips = [(0, 0, 0b011000110, 0b001000010, 0b010000100, 0b010000100),
             (0b100101010, 0b100101010, 0, 0, 0b001000100, 0b000000001), (0,) * 6]
    for kind, flip in zip(kinds, flips):
        spec = oracle_mod.bcspec(kind, flip)
        U = random_state(shape, 9)
        Ur = U.copy()
        L.omo_bc(_p(Ur), ix, jx, kx, nd, C.byref(spec))
        routines.bc(U, kind, flip)
        assert np.array_equal(U, Ur)
        for d in range(1, nd + 1):
            VL = random_state(shape, 20 + d)
            VR = random_state(shape, 30 + d)
            rL, rR = VL.copy(), VR.copy()
            L.omo_facefix(_p(rL), _p(rR), ix, jx, kx, d, C.byref(spec))
            a = 2 * (d - 1)
            routines.facefix(VL, VR, d, kind[a], flip[a], kind[a + 1], flip[a + 1])
            assert np.array_equal(VL, rL) and np.array_equal(VR, rR)


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("eta_kind", [1, 2])
def test_flux_resistive(cuda_lib, oracle_mod, shape, eta_kind):
    from openmhd_gb300 import routines

    L = oracle_mod.lib()
    nd, ix, jx, kx = _dims(shape)
    U = random_state(shape, 11)
    dx = 0.37
    x = np.zeros(ix); y = np.zeros(jx); z = np.zeros(kx)
    L.omo_grid(_p(x), ix, -2.0, dx)
    L.omo_grid(_p(y), jx, -3.0, dx)
    L.omo_grid(_p(z), kx, -1.5, dx)
    for d in range(1, nd + 1):
        F = np.random.default_rng(d).uniform(-1, 1, (9,) + shape)
        Fr = F.copy()
        L.omo_flux_resistive(_p(Fr), _p(U), _p(x), _p(y), _p(z), dx, ix, jx, kx, nd, d, eta_kind)
        routines.flux_resistive(F, U, x, y, z if nd == 3 else None, dx=dx, dir=d, eta_kind=eta_kind)
        # cosh/exp on the device may differ from the host libm in the last bit
        np.testing.assert_allclose(F, Fr, rtol=1e-14, atol=1e-15)


def test_fortran_dropins_match_c_entry_points(cuda_lib, oracle_mod):
    """The gfortran link-level names (u2v_, set_dt_, ...) call the same kernels."""
    lib = cuda_lib
    U = random_state((10, 12), 12)
    V1 = np.zeros((4, 10, 12))
    V2 = np.zeros((4, 10, 12))
    ix, jx = C.c_int(12), C.c_int(10)
    lib.u2v_(U.ctypes.data, V1.ctypes.data, C.byref(ix), C.byref(jx))
    assert lib.omhd_u2v_2d(U.ctypes.data, V2.ctypes.data, 12, 10) == 0
    assert np.array_equal(V1, V2)
    vmax, dt = C.c_double(), C.c_double()
    dx, cfl = C.c_double(0.05), C.c_double(0.4)
    lib.set_dt_(U.ctypes.data, V1.ctypes.data, C.byref(vmax), C.byref(dt), C.byref(dx), C.byref(cfl),
                C.byref(ix), C.byref(jx))
    L = oracle_mod.lib()
    vm, dtr = C.c_double(), C.c_double()
    e = oracle_mod.Err()
    L.omo_set_dt(U.ctypes.data, V1.ctypes.data, C.byref(vm), C.byref(dtr), 0.05, 0.05, 0.05, 0.4, 12, 10, 1, 2,
                 C.byref(e))
    assert vmax.value == vm.value and dt.value == dtr.value
