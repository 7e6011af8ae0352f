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


def smooth_state(jx, ix, seed):
    """Seeded smooth state: a few random Fourier modes on a uniform background."""
    rng = np.random.default_rng(seed)
    y, x = np.meshgrid(np.linspace(0, 2 * np.pi, jx), np.linspace(0, 2 * np.pi, ix), indexing="ij")

    def field(mean, amp):
        f = np.full((jx, ix), mean)
        for _ in range(3):
            kx, ky = rng.integers(1, 3, 2)
            f += amp * rng.uniform(-1, 1) * np.sin(kx * x + ky * y + rng.uniform(0, 6.3))
        return f

    ro, p = field(1.0, 0.2), field(0.6, 0.1)
    v = np.stack([field(0.0, 0.5) for _ in range(3)])
    B = np.stack([field(0.0, 0.6) for _ in range(3)])
    U = np.empty((9, jx, ix))
    U[0:3] = ro * v
    U[4] = ro
    U[5:8] = B
    U[8] = field(0.0, 0.05)
    U[3] = 0.5 * (ro * (v * v).sum(0) + (B * B).sum(0)) + p / (5.0 / 3.0 - 1)
    return U


from openmhd_gb300.metrics import rel_l1, scaled_l1  # noqa: E402,F401


def interior(U: np.ndarray) -> np.ndarray:
    if U.ndim == 3:
        return U[:, 1:-1, 1:-1]
    return U[:, 1:-1, 1:-1, 1:-1]
