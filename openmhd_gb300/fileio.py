"""Snapshot files in the reference's format (2D_basic/fileio.f90:16-115,
3D_basic/fileio.f90:16-122) through the C ABI (omhd_fileio_output /
omhd_fileio_input).  Layout: t | ix, jx[, kx] (int32) | x, y[, z] | nine U
planes | four V planes (vx, vy, vz, pr), native byte order, no record markers.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .solver import OmhdError


def _shape(a) -> tuple:
    return tuple(int(n) for n in a.shape)


def write(path: str, t: float, x, y, U, V=None, z=None):
    """Write a field file.  U is (9, jx, ix) or (9, kx, jx, ix) float64 (numpy,
    or a torch tensor on any device); V (4, ...) or None (computed from U on the
    GPU); x, y[, z] hold ix, jx[, kx] coordinates.  Shapes and types are
    checked before the library is called: it trusts ix/jx/kx and would read
    past a smaller buffer."""
    if U.ndim not in (3, 4) or int(U.shape[0]) != 9:
        raise ValueError(f"U has shape {_shape(U)}, expected (9, jx, ix) or (9, kx, jx, ix)")
    nd = U.ndim - 1
    planes = _shape(U)[1:]
    ix, jx = planes[-1], planes[-2]
    kx = planes[0] if nd == 3 else 1
    if nd == 3 and z is None:
        raise ValueError("z is required for a 3D state")
    coords = [np.asarray(x, dtype=np.float64), np.asarray(y, dtype=np.float64)]
    if nd == 3:
        coords.append(np.asarray(z, dtype=np.float64))
    for name, c, n in zip("xyz", coords, (ix, jx, kx)):
        if c.shape != (n,):
            raise ValueError(f"{name} has shape {c.shape}, expected ({n},)")
    if V is not None and _shape(V) != (4,) + planes:
        raise ValueError(f"V has shape {_shape(V)}, expected {(4,) + planes}")
    lib = _lib.load()
    keep = []

    def ptr(a):
        if a is None:
            return None
        if isinstance(a, np.ndarray):
            a = np.ascontiguousarray(a, dtype=np.float64)
            keep.append(a)
            return a.ctypes.data
        if getattr(a, "dtype", None) is None or str(a.dtype) != "torch.float64":
            raise TypeError(f"arrays must be float64, got {getattr(a, 'dtype', type(a))}")
        a = a.contiguous()
        keep.append(a)
        return a.data_ptr()

    st = lib.omhd_fileio_output(str(path).encode(), nd, ix, jx, kx, float(t), ptr(coords[0]), ptr(coords[1]),
                                ptr(coords[2]) if nd == 3 else None, ptr(U), ptr(V))
    if st:
        raise OmhdError(st, f"cannot write {path}")


def read(path: str, nd: int, ix: int, jx: int, kx: int = 1):
    """(t, x, y, z, U) of a field file with the given sizes (incl. ghosts)."""
    if nd not in (2, 3) or ix < 1 or jx < 1 or (nd == 3 and kx < 1):
        raise ValueError(f"bad sizes nd={nd}, ix={ix}, jx={jx}, kx={kx}")
    lib = _lib.load()
    shape = (9, jx, ix) if nd == 2 else (9, kx, jx, ix)
    U = np.empty(shape)
    x, y, z = np.empty(ix), np.empty(jx), np.empty(max(kx, 1))
    t = C.c_double()
    st = lib.omhd_fileio_input(str(path).encode(), nd, ix, jx, kx, C.byref(t), x.ctypes.data, y.ctypes.data,
                               z.ctypes.data, U.ctypes.data)
    if st:
        raise OmhdError(st, f"cannot read {path}")
    return t.value, x, y, (z if nd == 3 else None), U
