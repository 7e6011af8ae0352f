"""Reference-named routine wrappers over the routine-level C ABI.

Each function takes the arrays the reference routine takes (numpy arrays or
torch tensors on any device, float64, reference layout: U shaped (9, jx, ix)
or (9, kx, jx, ix), planes shaped (jx, ix) or (kx, jx, ix)) and forwards
them to libopenmhd_gb300.so.  Host arrays travel through the library's device
mirrors; CUDA tensors are processed in place on torch's current stream.
Failures raise OmhdError with the reference's message (the reference stops).
"""
from __future__ import annotations

import ctypes as C

from . import _lib
from .solver import OmhdError


def _ptr(a) -> int:
    try:
        import numpy as np

        if isinstance(a, np.ndarray):
            if a.dtype != np.float64 or not a.flags.c_contiguous:
                raise TypeError("arrays must be C-contiguous float64")
            return a.ctypes.data
    except ImportError:  # pragma: no cover
        pass
    import torch

    if isinstance(a, torch.Tensor):
        if a.dtype != torch.float64 or not a.is_contiguous():
            raise TypeError("tensors must be contiguous float64")
        return a.data_ptr()
    raise TypeError(f"unsupported array type {type(a)}")


def _dims(U, var_axis: bool = True):
    shp = tuple(U.shape)
    core = shp[1:] if var_axis else shp
    if len(core) == 2:
        return 2, core[1], core[0], 1
    if len(core) == 3:
        return 3, core[2], core[1], core[0]
    raise ValueError(f"bad array shape {shp}")


def _shape_of(a) -> tuple:
    return tuple(int(n) for n in a.shape)


def _expect(name: str, a, shape: tuple):
    """Refuse an array whose shape is not the one the routine reads or writes
    (the library trusts ix/jx/kx and would run past a smaller buffer)."""
    if a is None:
        raise ValueError(f"{name} is required")
    if _shape_of(a) != tuple(shape):
        raise ValueError(f"{name} has shape {_shape_of(a)}, expected {tuple(shape)}")


def _planes(nd: int, ix: int, jx: int, kx: int) -> tuple:
    return (jx, ix) if nd == 2 else (kx, jx, ix)


def _lib_for(*arrays):
    try:
        import torch

        cuda = [a for a in arrays if isinstance(a, torch.Tensor) and a.is_cuda]
        if cuda:
            dev = torch.cuda.current_device()
            bad = [a.device.index for a in cuda if a.device.index != dev]
            if bad:
                raise ValueError(f"CUDA tensors must be on the current device cuda:{dev}, got cuda:{bad[0]}")
    except ImportError:  # pragma: no cover
        pass
    lib = _lib.load()
    lib.omhd_set_abort_on_error(0)
    try:
        import torch

        if any(isinstance(a, torch.Tensor) and a.is_cuda for a in arrays):
            lib.omhd_set_stream(C.c_void_p(torch.cuda.current_stream().cuda_stream))
        else:
            lib.omhd_set_stream(None)
    except ImportError:  # pragma: no cover
        pass
    return lib


def _check(lib, st: int):
    if st:
        info = _lib.ErrorInfo()
        lib.omhd_last_error(C.byref(info))
        lib.omhd_clear_error()
        raise OmhdError(st, info.message.decode(errors="replace"))


def u2v(U, V):
    """u2v(U,V,ix,jx[,kx]) -- 2D_basic/u2v.f90:1-46."""
    nd, ix, jx, kx = _dims(U)
    _expect("U", U, (9,) + _planes(nd, ix, jx, kx))
    _expect("V", V, (4,) + _planes(nd, ix, jx, kx))
    lib = _lib_for(U, V)
    st = lib.omhd_u2v_2d(_ptr(U), _ptr(V), ix, jx) if nd == 2 else lib.omhd_u2v_3d(_ptr(U), _ptr(V), ix, jx, kx)
    _check(lib, st)


def limiter(wk, wL, wR, dir: int, type: int):
    """limiter(wk,wL,wR,ix,jx[,kx],dir,type) -- 2D_basic/limiter.f90:1-318."""
    nd, ix, jx, kx = _dims(wk, var_axis=False)
    _expect("wL", wL, _shape_of(wk))
    _expect("wR", wR, _shape_of(wk))
    lib = _lib_for(wk, wL, wR)
    if nd == 2:
        st = lib.omhd_limiter_2d(_ptr(wk), _ptr(wL), _ptr(wR), ix, jx, dir, type)
    else:
        st = lib.omhd_limiter_3d(_ptr(wk), _ptr(wL), _ptr(wR), ix, jx, kx, dir, type)
    _check(lib, st)


def flux_solver(F, VL, VR, ch: float, dir: int, type: int):
    """flux_solver(F,VL,VR,ch,ix,jx[,kx],dir,type) -- 2D_basic/flux_solver.f90:1-795."""
    nd, ix, jx, kx = _dims(F)
    _expect("F", F, (9,) + _planes(nd, ix, jx, kx))
    _expect("VL", VL, _shape_of(F))
    _expect("VR", VR, _shape_of(F))
    lib = _lib_for(F, VL, VR)
    if nd == 2:
        st = lib.omhd_flux_solver_2d(_ptr(F), _ptr(VL), _ptr(VR), ch, ix, jx, dir, type)
    else:
        st = lib.omhd_flux_solver_3d(_ptr(F), _ptr(VL), _ptr(VR), ch, ix, jx, kx, dir, type)
    _check(lib, st)


def _rk(name: str, U, U1, F, G, H, dt: float, dx: float):
    nd, ix, jx, kx = _dims(U)
    full = (9,) + _planes(nd, ix, jx, kx)
    _expect("U", U, full)
    if U1 is not None:
        _expect("U1", U1, full)
    _expect("F", F, full)
    _expect("G", G, full)
    if nd == 3:
        _expect("H", H, full)
    lib = _lib_for(U, U1, F, G, H)
    if nd == 2:
        fn = getattr(lib, f"omhd_{name}_2d")
        args = ([_ptr(U)] + ([_ptr(U1)] if U1 is not None else []) + [_ptr(F), _ptr(G), dt, dx, ix, jx])
    else:
        fn = getattr(lib, f"omhd_{name}_3d")
        args = ([_ptr(U)] + ([_ptr(U1)] if U1 is not None else []) + [_ptr(F), _ptr(G), _ptr(H), dt, dx, ix, jx, kx])
    _check(lib, fn(*args))


def rk_tvd21(U, U1, F, G, H=None, *, dt: float, dx: float):
    """rk_tvd21 -- 2D_basic/rk.f90:9-35 (U1 = U + dt/dx * flux divergence)."""
    _rk("rk_tvd21", U, U1, F, G, H, dt, dx)


def rk_tvd22(U, U1, F, G, H=None, *, dt: float, dx: float):
    """rk_tvd22 -- 2D_basic/rk.f90:42-66."""
    _rk("rk_tvd22", U, U1, F, G, H, dt, dx)


def rk_std21(U, U1, F, G, H=None, *, dt: float, dx: float):
    """rk_std21 -- 2D_basic/rk.f90:73-99."""
    _rk("rk_std21", U, U1, F, G, H, dt, dx)


def rk_std22(U, F, G, H=None, *, dt: float, dx: float):
    """rk_std22 -- 2D_basic/rk.f90:106-131."""
    _rk("rk_std22", U, None, F, G, H, dt, dx)


def glm_ss2(U, ch: float, dt: float):
    """glm_ss2(U,ch,dt,ix,jx[,kx]) -- 2D_basic/glm_ss2.f90:1-39."""
    nd, ix, jx, kx = _dims(U)
    _expect("U", U, (9,) + _planes(nd, ix, jx, kx))
    lib = _lib_for(U)
    st = lib.omhd_glm_ss2_2d(_ptr(U), ch, dt, ix, jx) if nd == 2 else lib.omhd_glm_ss2_3d(_ptr(U), ch, dt, ix, jx, kx)
    _check(lib, st)


def set_dt(U, V, dx: float, cfl: float):
    """set_dt(U,V,vmax,dt,dx,cfl,ix,jx[,kx]) -- 2D_basic/set_dt.f90:1-68; returns (vmax, dt)."""
    nd, ix, jx, kx = _dims(U)
    _expect("U", U, (9,) + _planes(nd, ix, jx, kx))
    _expect("V", V, (4,) + _planes(nd, ix, jx, kx))
    lib = _lib_for(U, V)
    vmax, dt = C.c_double(), C.c_double()
    if nd == 2:
        st = lib.omhd_set_dt_2d(_ptr(U), _ptr(V), C.byref(vmax), C.byref(dt), dx, cfl, ix, jx)
    else:
        st = lib.omhd_set_dt_3d(_ptr(U), _ptr(V), C.byref(vmax), C.byref(dt), dx, cfl, ix, jx, kx)
    _check(lib, st)
    return vmax.value, dt.value


def bc(U, kind=(0, 0, 0, 0, 0, 0), flip=(0, 0, 0, 0, 0, 0)):
    """Ghost-cell fill -- 2D_basic/bc.f90:1-16 (periodic) and the wall variants."""
    nd, ix, jx, kx = _dims(U)
    _expect("U", U, (9,) + _planes(nd, ix, jx, kx))
    if len(kind) != 6 or len(flip) != 6:
        raise ValueError("kind and flip take one entry per domain side (6)")
    lib = _lib_for(U)
    k = (C.c_int * 6)(*kind)
    f = (C.c_int * 6)(*flip)
    st = lib.omhd_bc_2d(_ptr(U), ix, jx, k, f) if nd == 2 else lib.omhd_bc_3d(_ptr(U), ix, jx, kx, k, f)
    _check(lib, st)


def facefix(VL, VR, dir: int, kind_lo=0, flip_lo=0, kind_hi=0, flip_hi=0):
    """Face-state fix at the domain edges -- main.f90:101-102, 2D_KH/bc.f90:42-83."""
    nd, ix, jx, kx = _dims(VL)
    _expect("VL", VL, (9,) + _planes(nd, ix, jx, kx))
    _expect("VR", VR, _shape_of(VL))
    lib = _lib_for(VL, VR)
    if nd == 2:
        st = lib.omhd_facefix_2d(_ptr(VL), _ptr(VR), ix, jx, dir, kind_lo, flip_lo, kind_hi, flip_hi)
    else:
        st = lib.omhd_facefix_3d(_ptr(VL), _ptr(VR), ix, jx, kx, dir, kind_lo, flip_lo, kind_hi, flip_hi)
    _check(lib, st)


def flux_resistive(F, U, x, y, z=None, *, dx: float, dir: int, eta_kind: int = 1):
    """flux_resistive -- 2D_reconnection/flux_resistive.f90:27-115 (3D: 3D_reconnection_gpu)."""
    nd, ix, jx, kx = _dims(U)
    _expect("U", U, (9,) + _planes(nd, ix, jx, kx))
    _expect("F", F, _shape_of(U))
    _expect("x", x, (ix,))
    _expect("y", y, (jx,))
    if nd == 3:
        _expect("z", z, (kx,))
    lib = _lib_for(F, U, x, y, z)
    if nd == 2:
        st = lib.omhd_flux_resistive_2d(_ptr(F), _ptr(U), _ptr(x), _ptr(y), dx, ix, jx, dir, eta_kind)
    else:
        st = lib.omhd_flux_resistive_3d(_ptr(F), _ptr(U), _ptr(x), _ptr(y), _ptr(z), dx, ix, jx, kx, dir, eta_kind)
    _check(lib, st)
