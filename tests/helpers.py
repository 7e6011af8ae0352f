"""Shared helpers for the parity tests: seeded valid MHD states and error norms."""
from __future__ import annotations

import numpy as np

GAMMA = 5.0 / 3.0


def random_state(shape_xyz, seed: int = 0, smooth: bool = False) -> np.ndarray:
    """Seeded valid conserved state U, shape (9,) + shape_xyz (reference layout)."""
    rng = np.random.default_rng(seed)
    ro = rng.uniform(0.5, 2.0, shape_xyz)
    v = rng.uniform(-1.0, 1.0, (3,) + tuple(shape_xyz))
    p = rng.uniform(0.2, 1.0, shape_xyz)
    B = rng.uniform(-1.0, 1.0, (3,) + tuple(shape_xyz))
    ps = rng.uniform(-0.1, 0.1, shape_xyz)
    if smooth:
        for a in (ro, p, ps):
            a[...] = 1.0 + 0.1 * (a - a.mean())
    U = np.empty((9,) + tuple(shape_xyz))
    U[0:3] = ro * v
    U[4] = ro
    U[5:8] = B
    U[8] = ps
    v2 = (v * v).sum(axis=0)
    B2 = (B * B).sum(axis=0)
    U[3] = 0.5 * (ro * v2 + B2) + p / (GAMMA - 1)
    return np.ascontiguousarray(U)


from openmhd_gb300.metrics import rel_l1, scaled_l1  # noqa: E402,F401


def interior(U: np.ndarray) -> np.ndarray:
    if U.ndim == 3:
        return U[:, 1:-1, 1:-1]
    return U[:, 1:-1, 1:-1, 1:-1]
