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


def write(path: str, t: float, x, y, U, V=None, z=None):
    """Write a field file.  U is (9, jx, ix) or (9, kx, jx, ix) float64 (numpy,
    or a torch tensor on any device); V (4, ...) or None (computed from U on the
    GPU)."""
    lib = _lib.load()
    keep = []

    def ptr(a):
        if a is None:
            return None
        if isinstance(a, np.ndarray):
            a = np.ascontiguousarray(a, dtype=np.float64)
            keep.append(a)
            return a.ctypes.data
        a = a.contiguous()
        keep.append(a)
        return a.data_ptr()

    nd = U.ndim - 1
    shape = tuple(U.shape[1:])
    ix, jx = shape[-1], shape[-2]
    kx = shape[0] if nd == 3 else 1
    st = lib.omhd_fileio_output(str(path).encode(), nd, ix, jx, kx, float(t), ptr(np.asarray(x, dtype=np.float64)),
                                ptr(np.asarray(y, dtype=np.float64)),
                                ptr(np.asarray(z, dtype=np.float64)) if z is not None else None, ptr(U), ptr(V))
    if st:
        raise OmhdError(st, f"cannot write {path}")


def read(path: str, nd: int, ix: int, jx: int, kx: int = 1):
    """(t, x, y, z, U) of a field file with the given sizes (incl. ghosts)."""
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
