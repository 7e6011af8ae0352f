"""Error norms used to report mixed-precision and parity errors (host-side
analysis of states copied off the GPU; not part of the stepping path)."""
from __future__ import annotations

import numpy as np

VAR_NAMES = ["mx", "my", "mz", "en", "ro", "bx", "by", "bz", "ps"]


def rel_l1(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """Per-variable relative L1 error of a against b, each variable against its own norm."""
    a = a.reshape(a.shape[0], -1)
    b = b.reshape(b.shape[0], -1)
    num = np.abs(a - b).sum(axis=1)
    den = np.abs(b).sum(axis=1)
    return np.where(den > 0, num / np.where(den > 0, den, 1.0), num)


def scaled_l1(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """Per-variable L1 error of a against b, each variable normalised by the L1
    norm of its physical scale: rho and E by themselves, the momentum
    components by sqrt(2 rho E) (>= |m|, the momentum a cell's total energy
    could carry), the field components and psi by |B|.  Components that are
    ~0 (By, vy, psi early in a run, momentum of a static equilibrium) are
    measured against the scale of the state, not against their own
    round-off."""
    a = a.reshape(a.shape[0], -1)
    b = b.reshape(b.shape[0], -1)
    num = np.abs(a - b).sum(axis=1)
    m = np.sqrt(np.abs(2.0 * b[4] * b[3])).sum()
    B = np.sqrt((b[5:8] ** 2).sum(axis=0)).sum()
    den = np.array([m, m, m, np.abs(b[3]).sum(), np.abs(b[4]).sum(), B, B, B, B])
    floor = max(den.max(), 1e-300) * 1e-12
    return num / np.maximum(den, floor)


def linf(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """Per-variable max-norm error."""
    a = a.reshape(a.shape[0], -1)
    b = b.reshape(b.shape[0], -1)
    return np.abs(a - b).max(axis=1)
