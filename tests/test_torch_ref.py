"""The pure-PyTorch reference step (the autograd reference of the adjoint)
against the oracle, on the CPU: one step with the oracle's own dt and ch,
for periodic, zero-gradient and sign-flipping mirror boundaries."""
import math

import numpy as np
import pytest
import torch

import torch_ref_step as tr
from helpers import random_state, smooth_state

CASES = {
    # name: (limiter, bc_kind, bc_flip)
    "periodic_mc": ("mc", (0, 0, 0, 0, 0, 0), (0,) * 6),
    "kh_walls_minmod": ("minmod", (0, 0, 1, 1, 0, 0), (0,) * 6),
    "flip_walls_minmod": ("minmod", (1, 1, 1, 1, 0, 0), (0b010000001, 0b010000001, 0b001000010, 0b001000010, 0, 0)),
}


class Cfg:
    def __init__(self, ix, jx, dx, dy, limiter, bc_kind, bc_flip):
        self.nd, self.ix, self.jx, self.kx = 2, ix, jx, 1
        self.dx, self.dy, self.dz = dx, dy, dx
        self.x0 = self.y0 = self.z0 = 0.0
        self.cfl, self.gamma = 0.4, 5.0 / 3.0
        self.limiter, self.flux, self.time, self.eta = limiter, "hlld", "tvdrk2", "none"
        self.bc_kind, self.bc_flip = bc_kind, bc_flip


@pytest.mark.parametrize("name", sorted(CASES))
@pytest.mark.parametrize("kind", ["smooth", "random"])
def test_torch_step_matches_oracle(oracle_mod, name, kind):
    lim, bk, bf = CASES[name]
    ix, jx = 22, 18
    cfg = Cfg(ix, jx, 0.3, 0.25, lim, bk, bf)
    g = oracle_mod.Grid.from_solver_config(cfg)
    U0 = smooth_state(jx, ix, 4) if kind == "smooth" else random_state((jx, ix), 9, smooth=True)
    g.U[...] = U0
    g.bc()
    Ubc = g.U.copy()
    g.step(1)
    dt, ch = g.last_dt, g.last_ch
    f = math.exp(-(0.5 * dt * ch / 0.2))
    out = tr.step(torch.from_numpy(Ubc), dt, ch, f, cfg).numpy()
    err = np.abs(out - g.U).max(axis=(1, 2)) / np.maximum(np.abs(g.U).max(axis=(1, 2)), 1e-300)
    assert np.all(err < 1e-13), err


def test_torch_step_bc_and_ghosts(oracle_mod):
    """The torch bc reproduces the oracle's ghost fill, corners included."""
    lim, bk, bf = CASES["flip_walls_minmod"]
    cfg = Cfg(9, 7, 0.3, 0.3, lim, bk, bf)
    g = oracle_mod.Grid.from_solver_config(cfg)
    g.U[...] = random_state((7, 9), 2)
    U = torch.from_numpy(g.U.copy())
    g.bc()
    assert np.array_equal(tr.bc(U, bk, bf).numpy(), g.U)


@pytest.mark.parametrize("d", [1, 2])
def test_torch_hlld_every_branch(oracle_mod, d):
    """The torch HLLD on the golden face states of every branch (and their
    y-rotations) against the oracle's flux."""
    import os

    gold = np.load(os.path.join(os.path.dirname(__file__), "golden", "oracle_golden.npz"))
    names = ["FL", "FR", "HLLCG_L", "HLLCG_R", "Lstar", "Rstar", "Lstar2", "Rstar2"]
    L = np.stack([gold[f"hlld_{k}_d1_L"] for k in names], axis=1)
    R = np.stack([gold[f"hlld_{k}_d1_R"] for k in names], axis=1)
    if d == 2:  # rotate x-face states into y-face states: (vx,vy,vz) -> (vz,vx,vy)
        perm = [2, 0, 1, 3, 4, 7, 5, 6, 8]
        L, R = L[perm], R[perm]
    L, R = np.ascontiguousarray(L), np.ascontiguousarray(R)
    oracle_mod.branch_counts()
    Fo = oracle_mod.flux_faces(L, R, 0.8, d)
    assert all(v == 1 for v in oracle_mod.branch_counts().values())
    Ft = tr.hlld(torch.from_numpy(L), torch.from_numpy(R), 0.8, 5.0 / 3.0, d).numpy()
    assert np.abs(Ft - Fo).max() <= 1e-13 * max(1.0, np.abs(Fo).max())
