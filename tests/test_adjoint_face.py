"""CPU checks of the hand-written face adjoints (omhd_adjoint_face.h) against
central finite differences of the oracle's flux, limiter and u2v, for every
HLLD branch in every direction."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden", "oracle_golden.npz")
BRANCHES = ["FL", "FR", "HLLCG_L", "HLLCG_R", "Lstar", "Rstar", "Lstar2", "Rstar2"]


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("adj") / "adjh.so")
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-shared", "-fPIC", "-o", out,
                    os.path.join(HERE, "adjoint_harness.cpp")], check=True)
    L = C.CDLL(out)
    P, D, I = C.c_void_p, C.c_double, C.c_int
    L.h_hlld_vjp.argtypes = [I, P, P, D, D, P, P, P]
    L.h_recon_vjp.argtypes = [I, D, D, D, D, D, P]
    L.h_u2v_vjp.argtypes = [P, D, P, P]
    return L


def _p(a):
    return a.ctypes.data


def _rot(w, d):
    perm = [1, 2, 0, 3, 4, 6, 7, 5, 8] if d == 2 else [2, 0, 1, 3, 4, 7, 5, 6, 8]
    return w if d == 1 else w[np.argsort(perm)]


def _flux(oracle_mod, L, R, ch, d):
    if d == 3:
        # the oracle's helper lays faces out in 2D; a z face is an x face of the
        # cyclically rotated state (flux_solver.f90:62-70)
        Lr, Rr = L[[2, 0, 1, 3, 4, 7, 5, 6, 8]], R[[2, 0, 1, 3, 4, 7, 5, 6, 8]]
        F = oracle_mod.flux_faces(Lr[:, None], Rr[:, None], ch, 1)[:, 0]
        out = np.zeros(9)
        out[[2, 0, 1, 3, 4, 7, 5, 6, 8]] = F
        return out
    return oracle_mod.flux_faces(L[:, None], R[:, None], ch, d)[:, 0]


def _fd_vjp(oracle_mod, L, R, ch, d, gF):
    gL, gR = np.zeros(9), np.zeros(9)
    for side, X, g in ((0, L, gL), (1, R, gR)):
        for k in range(9):
            h = 1e-6 * max(1.0, abs(X[k]))
            Xp, Xm = X.copy(), X.copy()
            Xp[k] += h
            Xm[k] -= h
            if side == 0:
                fp, fm = _flux(oracle_mod, Xp, R, ch, d), _flux(oracle_mod, Xm, R, ch, d)
            else:
                fp, fm = _flux(oracle_mod, L, Xp, ch, d), _flux(oracle_mod, L, Xm, ch, d)
            g[k] = gF @ (fp - fm) / (2 * h)
    return gL, gR


@pytest.mark.parametrize("name", BRANCHES)
@pytest.mark.parametrize("d", [1, 2, 3])
def test_hlld_vjp_matches_finite_differences(oracle_mod, harness, name, d):
    g = np.load(GOLD)
    L0, R0 = g[f"hlld_{name}_d1_L"], g[f"hlld_{name}_d1_R"]
    if d == 1:
        L, R = L0.copy(), R0.copy()
    else:
        L, R = _rot(L0, d).copy(), _rot(R0, d).copy()
    ch = 0.7
    rng = np.random.default_rng(hash((name, d)) % 2**32)
    oracle_mod.branch_counts()
    _flux(oracle_mod, L, R, ch, d)
    hit = [k for k, v in oracle_mod.branch_counts().items() if v]
    assert hit == [name]
    for _ in range(3):
        gF = rng.standard_normal(9)
        gL, gR = np.zeros(9), np.zeros(9)
        harness.h_hlld_vjp(d, _p(L), _p(R), ch, 5.0 / 3.0, _p(gF), _p(gL), _p(gR))
        fL, fR = _fd_vjp(oracle_mod, L, R, ch, d, gF)
        scale = max(1.0, np.abs(fL).max(), np.abs(fR).max())
        np.testing.assert_allclose(gL, fL, rtol=0, atol=2e-6 * scale)
        np.testing.assert_allclose(gR, fR, rtol=0, atol=2e-6 * scale)


def test_hlld_vjp_random_states(oracle_mod, harness):
    """Random nearby face states (mostly the central HLLD branches)."""
    rng = np.random.default_rng(11)
    seen = set()
    for _ in range(60):
        L = np.array([*rng.uniform(-1, 1, 3), rng.uniform(0.2, 1.0), rng.uniform(0.5, 2.0), *rng.uniform(-1, 1, 3),
                      rng.uniform(-0.1, 0.1)])
        R = L * (1 + rng.uniform(-0.2, 0.2, 9))
        R[3] = abs(R[3])
        R[4] = abs(R[4])
        d = int(rng.integers(1, 4))
        oracle_mod.branch_counts()
        _flux(oracle_mod, L, R, 0.9, d)
        seen |= {k for k, v in oracle_mod.branch_counts().items() if v}
        gF = rng.standard_normal(9)
        gL, gR = np.zeros(9), np.zeros(9)
        harness.h_hlld_vjp(d, _p(L), _p(R), 0.9, 5.0 / 3.0, _p(gF), _p(gL), _p(gR))
        fL, fR = _fd_vjp(oracle_mod, L, R, 0.9, d, gF)
        scale = max(1.0, np.abs(fL).max(), np.abs(fR).max())
        np.testing.assert_allclose(gL, fL, rtol=0, atol=5e-6 * scale)
        np.testing.assert_allclose(gR, fR, rtol=0, atol=5e-6 * scale)
    assert len(seen) >= 3


@pytest.mark.parametrize("type_", [1, 2])
def test_recon_vjp(harness, oracle_mod, type_):
    rng = np.random.default_rng(type_)
    L = oracle_mod.lib()
    for _ in range(200):
        w = rng.uniform(-1, 1, 3)
        gl, gr = rng.standard_normal(2)
        g3 = np.zeros(3)
        harness.h_recon_vjp(type_, w[0], w[1], w[2], gl, gr, _p(g3))

        def f(x):
            wk = np.ascontiguousarray(np.tile(np.r_[x[0], x, x[2]], (3, 1)))  # (jx=3, ix=5)
            wL, wR = np.zeros_like(wk), np.zeros_like(wk)
            L.omo_limiter(_p(wk), _p(wL), _p(wR), 5, 3, 1, 1, type_)
            return wL[1, 2], wR[1, 1]  # cell 2: upper state, lower state

        fd = np.zeros(3)
        for k in range(3):
            h = 1e-7
            xp, xm = w.copy(), w.copy()
            xp[k] += h
            xm[k] -= h
            lp, rp = f(xp)
            lm, rm = f(xm)
            fd[k] = (gl * (lp - lm) + gr * (rp - rm)) / (2 * h)
        np.testing.assert_allclose(g3, fd, atol=1e-6)


def test_u2v_vjp(harness, oracle_mod):
    from helpers import random_state

    rng = np.random.default_rng(5)
    U = random_state((1, 1), 3)[:, 0, 0].copy()
    for _ in range(5):
        gw = rng.standard_normal(9)
        gU = np.zeros(9)
        harness.h_u2v_vjp(_p(U), 5.0 / 3.0, _p(gw), _p(gU))

        def w_of(u):
            V, _, _ = oracle_mod.u2v(u.reshape(9, 1, 1).copy(), 2)
            return np.r_[V[:, 0, 0], u[4:9]]

        fd = np.zeros(9)
        for k in range(9):
            h = 1e-7 * max(1, abs(U[k]))
            up, um = U.copy(), U.copy()
            up[k] += h
            um[k] -= h
            fd[k] = gw @ (w_of(up) - w_of(um)) / (2 * h)
        np.testing.assert_allclose(gU, fd, atol=1e-6)


@pytest.mark.parametrize("d", [1, 2])
def test_hlld_vjp_matches_torch_autograd(harness, d):
    """Exact check (no differencing error): the hand-written HLLD adjoint
    against PyTorch autograd of the pure-torch HLLD, on every branch."""
    import torch

    import torch_ref_step as tr

    g = np.load(GOLD)
    rng = np.random.default_rng(d)
    for name in BRANCHES:
        L0, R0 = g[f"hlld_{name}_d1_L"], g[f"hlld_{name}_d1_R"]
        L, R = (L0, R0) if d == 1 else (_rot(L0, 2), _rot(R0, 2))
        L, R = np.ascontiguousarray(L), np.ascontiguousarray(R)
        gF = rng.standard_normal(9)
        tL = torch.tensor(L[:, None], requires_grad=True)
        tR = torch.tensor(R[:, None], requires_grad=True)
        F = tr.hlld(tL, tR, 0.7, 5.0 / 3.0, d)
        (F[:, 0] * torch.from_numpy(gF)).sum().backward()
        gL, gR = np.zeros(9), np.zeros(9)
        harness.h_hlld_vjp(d, _p(L), _p(R), 0.7, 5.0 / 3.0, _p(gF), _p(gL), _p(gR))
        scale = max(1.0, np.abs(gL).max(), np.abs(gR).max())
        np.testing.assert_allclose(gL, tL.grad[:, 0].numpy(), rtol=0, atol=1e-12 * scale, err_msg=name)
        np.testing.assert_allclose(gR, tR.grad[:, 0].numpy(), rtol=0, atol=1e-12 * scale, err_msg=name)
