"""Pure-PyTorch restatement of one 2D TVD-RK2 step with fixed dt and ch
(test infrastructure: the autograd reference for the hand-written adjoint).

It follows the same reference routines as the oracle -- u2v (u2v.f90:24-27),
minmod / MC reconstruction (limiter.f90:98, :141-158), the face fixes
(main.f90:101-102 periodic, 2D_KH/bc.f90:42-83 mirror), HLLD with the HLLC-G
fallback and the GLM fluxes (flux_solver.f90:352-585), the TVD-RK2 stages
(rk.f90:33-66), bc (bc.f90) and glm_ss2 (glm_ss2.f90) -- as differentiable
tensor code.  Branches are torch.where selections; every quantity that a
branch not taken could make non-finite is computed from a masked ("safe")
operand, so the unselected branches contribute exact zeros to the gradient.
Ties of fmin2 pick the first operand, as in the forward kernels, and the
sign factors of the limiters are constants, so the gradient at a limiter
kink is the same fixed subgradient the CUDA adjoint takes.

Arrays are (9, jx, ix) tensors (reference layout U(ix,jx,var)).
"""
from __future__ import annotations

import torch

MX, MY, MZ, EN, RO, BX, BY, BZ, PS = range(9)
VX, VY, VZ, PR = 0, 1, 2, 3


def u2v(U, gamma):
    ro = U[RO]
    vx, vy, vz = U[MX] / ro, U[MY] / ro, U[MZ] / ro
    rv2 = vx * U[MX] + vy * U[MY] + vz * U[MZ]
    B2 = U[BX] * U[BX] + U[BY] * U[BY] + U[BZ] * U[BZ]
    pr = (gamma - 1) * (U[EN] - 0.5 * (rv2 + B2))
    return torch.stack([vx, vy, vz, pr, ro, U[BX], U[BY], U[BZ], U[PS]])


def _fmin2(a, b):
    return torch.where(b < a, b, a)


def reconstruct(w, axis, lm):
    """Upper and lower face states of the cells 1..n-2 along `axis`.

    Written in the selected-operand form: (sign(c,gA)+sign(c,gB))*min(...) is
    0 when the signs differ and otherwise the selected slope itself (signed),
    so the value is the reference's and the derivative is that of the
    selected branch, also where a slope is exactly zero."""
    n = w.shape[axis]
    wm, w0, wp = w.narrow(axis, 0, n - 2), w.narrow(axis, 1, n - 2), w.narrow(axis, 2, n - 2)
    gA, gB = w0 - wm, wp - w0
    same = (torch.signbit(gA) == torch.signbit(gB)).to(w.dtype).detach()
    aA, aB = gA.abs(), gB.abs()
    sel = torch.where(aB < aA, gB, gA)
    if lm == 1:
        grad = same * 0.5 * sel
    elif lm == 2:
        gC = 0.25 * (wp - wm)
        m1 = _fmin2(aA, aB)
        sAC = (torch.copysign(torch.ones_like(gA), gA) * torch.copysign(torch.ones_like(gC), gC)).detach()
        grad = same * torch.where(gC.abs() < m1, sAC * gC, sel)
    else:
        raise ValueError("limiter")
    return w0 + grad, w0 - grad


def face_states(w, axis, lm, periodic, flip_lo, flip_hi):
    """L and R states of the faces 0..n-2 along `axis` with the face fixes."""
    up, lo = reconstruct(w, axis, lm)
    n = w.shape[axis]
    last = up.narrow(axis, n - 3, 1)
    first = lo.narrow(axis, 0, 1)
    if periodic:
        L0, Rn = last, first
    else:
        L0, Rn = flip_lo * first, flip_hi * last
    return torch.cat([L0, up], axis), torch.cat([lo, Rn], axis)


def hlld(L, R, ch, gamma, d):
    """HLLD flux (flux_solver.f90:352-585) of face states L, R along direction d (1 or 2)."""
    if d == 1:
        vn, vt1, vt2, bn, bt1, bt2 = VX, VY, VZ, BX, BY, BZ
        mn, mt1, mt2 = MX, MY, MZ
    else:
        vn, vt1, vt2, bn, bt1, bt2 = VY, VZ, VX, BY, BZ, BX
        mn, mt1, mt2 = MY, MZ, MX
    r1, r2 = 1.0 / (gamma - 1.0), gamma / (gamma - 1.0)
    hf = 1.001

    def side(S):
        v2 = S[VX] ** 2 + S[VY] ** 2 + S[VZ] ** 2
        B2 = S[BX] ** 2 + S[BY] ** 2 + S[BZ] ** 2
        vB = S[VX] * S[BX] + S[VY] * S[BY] + S[VZ] * S[BZ]
        U = {MX: S[RO] * S[VX], MY: S[RO] * S[VY], MZ: S[RO] * S[VZ], EN: 0.5 * (S[RO] * v2 + B2) + r1 * S[PR]}
        F = {RO: S[RO] * S[vn],
             mn: S[RO] * S[vn] * S[vn] - S[bn] * S[bn] + S[PR] + 0.5 * B2,
             mt1: S[RO] * S[vn] * S[vt1] - S[bn] * S[bt1],
             mt2: S[RO] * S[vn] * S[vt2] - S[bn] * S[bt2],
             EN: (0.5 * S[RO] * v2 + r2 * S[PR] + B2) * S[vn] - vB * S[bn],
             bt1: S[vn] * S[bt1] - S[bn] * S[vt1],
             bt2: S[vn] * S[bt2] - S[bn] * S[vt2]}
        f1 = gamma * S[PR]
        f2 = 4 * S[bn] ** 2
        a = ((f1 + B2) + torch.sqrt(torch.clamp((f1 + B2) ** 2 - f1 * f2, min=0.0))) / (2 * S[RO])
        pt = S[PR] + 0.5 * B2
        return U, F, vB, a, pt

    UL, FL, vBL, aL0, ptL = side(L)
    UR, FR, vBR, aR0, ptR = side(R)
    cf = torch.sqrt(torch.where(aR0 > aL0, aR0, aL0))
    aL = _fmin2(L[vn], R[vn]) - cf
    aR = torch.where(R[vn] > L[vn], R[vn], L[vn]) + cf
    mFL = aL >= 0
    mFR = (~mFL) & (aR <= 0)
    mid = ~(mFL | mFR)
    one = torch.ones_like(aL)
    f1 = 1.0 / (aR - aL)
    Uh = {}
    for k in (MX, MY, MZ):
        Uh[k] = f1 * (aR * UR[k] - aL * UL[k] - FR[k] + FL[k])
    FLf = {**FL, bn: torch.zeros_like(aL)}
    FRf = {**FR, bn: torch.zeros_like(aL)}
    for k in (RO, BX, BY, BZ):
        Uh[k] = f1 * (aR * R[k] - aL * L[k] - FRf[k] + FLf[k])
    roh = torch.where(mid, Uh[RO], one)
    aM = Uh[mn] / roh
    pt = ptL + L[RO] * (aL - L[vn]) * (aM - L[vn])
    dL = torch.where(mid, aL - aM, one)
    dR = torch.where(mid, aR - aM, one)
    roL = torch.where(mid, L[RO] * (aL - L[vn]) / dL, one)
    roR = torch.where(mid, R[RO] * (aR - R[vn]) / dR, one)
    aVL = Uh[bn].abs() / torch.sqrt(roL)
    aVR = Uh[bn].abs() / torch.sqrt(roR)
    mG = mid & ((aL >= aM - hf * aVL) | (aM + hf * aVR >= aR))
    mS = mid & ~mG

    # HLLC-G fallback (flux_solver.f90:447-476)
    f2g = aL * aR
    FG = {}
    FG[bt1] = f1 * (aR * FL[bt1] - aL * FR[bt1] + f2g * (R[bt1] - L[bt1]))
    FG[bt2] = f1 * (aR * FL[bt2] - aL * FR[bt2] + f2g * (R[bt2] - L[bt2]))
    at1 = Uh[mt1] / roh
    at2 = Uh[mt2] / roh
    enL = ((aL - L[vn]) * UL[EN] - ptL * L[vn] + pt * aM
           + Uh[bn] * (vBL - aM * Uh[bn] - at1 * Uh[bt1] - at2 * Uh[bt2])) / dL
    enR = ((aR - R[vn]) * UR[EN] - ptR * R[vn] + pt * aM
           + Uh[bn] * (vBR - aM * Uh[bn] - at1 * Uh[bt1] - at2 * Uh[bt2])) / dR
    sg = (0.5 + torch.copysign(torch.full_like(aM, 0.5), aM)).detach()
    sg2 = 1 - sg
    FG[mn] = sg * (aL * (roL * aM - UL[mn]) + FL[mn]) + sg2 * (aR * (roR * aM - UR[mn]) + FR[mn])
    FG[mt1] = sg * (aL * (roL * at1 - UL[mt1]) + FL[mt1]) + sg2 * (aR * (roR * at1 - UR[mt1]) + FR[mt1])
    FG[mt2] = sg * (aL * (roL * at2 - UL[mt2]) + FL[mt2]) + sg2 * (aR * (roR * at2 - UR[mt2]) + FR[mt2])
    FG[EN] = sg * (aL * (enL - UL[EN]) + FL[EN]) + sg2 * (aR * (enR - UR[EN]) + FR[EN])
    FG[RO] = sg * (aL * (roL - L[RO]) + FL[RO]) + sg2 * (aR * (roR - R[RO]) + FR[RO])

    # L*, R* (:482-507)
    def star(S, US, a, ro, vBS, ptS):
        t = a - S[vn]
        den = torch.where(mS, S[RO] * t * (a - aM) - Uh[bn] ** 2, one)
        f = 1.0 / den
        U1 = {}
        U1[bt1] = S[bt1] * f * (S[RO] * t * t - Uh[bn] ** 2)
        U1[bt2] = S[bt2] * f * (S[RO] * t * t - Uh[bn] ** 2)
        vt1s = S[vt1] - f * Uh[bn] * S[bt1] * (aM - S[vn])
        vt2s = S[vt2] - f * Uh[bn] * S[bt2] * (aM - S[vn])
        U1[RO] = ro
        dd = torch.where(mS, a - aM, one)
        U1[EN] = ((a - S[vn]) * US[EN] - ptS * S[vn] + pt * aM
                  + Uh[bn] * (vBS - aM * Uh[bn] - vt1s * U1[bt1] - vt2s * U1[bt2])) / dd
        U1[mn] = ro * aM
        U1[mt1] = ro * vt1s
        U1[mt2] = ro * vt2s
        return U1, vt1s, vt2s

    UL1, vt1L, vt2L = star(L, UL, aL, roL, vBL, ptL)
    UR1, vt1R, vt2R = star(R, UR, aR, roR, vBR, ptR)
    aL1 = aM - aVL
    aR1 = aM + aVR
    mLs = mS & (aL1 >= 0)
    mRs = mS & ~mLs & (aR1 <= 0)
    mSS = mS & ~(mLs | mRs)
    cons = (MX, MY, MZ, EN)

    FLs, FRs = {}, {}
    for k in cons:
        FLs[k] = aL * (UL1[k] - UL[k]) + FL[k]
        FRs[k] = aR * (UR1[k] - UR[k]) + FR[k]
    for k in (RO, bt1, bt2):
        FLs[k] = aL * (UL1[k] - L[k]) + FL[k]
        FRs[k] = aR * (UR1[k] - R[k]) + FR[k]

    # central states (:533-572)
    roLs = torch.sqrt(roL)
    roRs = torch.sqrt(roR)
    f1c = 1.0 / (roLs + roRs)
    sb = torch.copysign(one, Uh[bn]).detach()
    a1 = f1c * (roLs * vt1L + roRs * vt1R + (UR1[bt1] - UL1[bt1]) * sb)
    a2 = f1c * (roLs * vt2L + roRs * vt2R + (UR1[bt2] - UL1[bt2]) * sb)
    U2b1 = f1c * (roLs * UR1[bt1] + roRs * UL1[bt1] + roLs * roRs * (vt1R - vt1L) * sb)
    U2b2 = f1c * (roLs * UR1[bt2] + roRs * UL1[bt2] + roLs * roRs * (vt2R - vt2L) * sb)
    U2L = {bt1: U2b1, bt2: U2b2, RO: roL, mn: roL * aM, mt1: roL * a1, mt2: roL * a2,
           EN: UL1[EN] - roLs * (vt1L * UL1[bt1] + vt2L * UL1[bt2] - a1 * U2b1 - a2 * U2b2) * sb}
    U2R = {bt1: U2b1, bt2: U2b2, RO: roR, mn: roR * aM, mt1: roR * a1, mt2: roR * a2,
           EN: UR1[EN] + roRs * (vt1R * UR1[bt1] + vt2R * UR1[bt2] - a1 * U2b1 - a2 * U2b2) * sb}
    FLss, FRss = {}, {}
    for k in cons:
        FLss[k] = aL1 * U2L[k] - (aL1 - aL) * UL1[k] - aL * UL[k] + FL[k]
        FRss[k] = aR1 * U2R[k] - (aR1 - aR) * UR1[k] - aR * UR[k] + FR[k]
    for k in (RO, bt1, bt2):
        FLss[k] = aL1 * U2L[k] - (aL1 - aL) * UL1[k] - aL * L[k] + FL[k]
        FRss[k] = aR1 * U2R[k] - (aR1 - aR) * UR1[k] - aR * R[k] + FR[k]
    mLss = mSS & (aM >= 0)

    out = [None] * 9
    for k in (MX, MY, MZ, EN, RO, bt1, bt2):
        f = torch.where(mLss, FLss[k], FRss[k])
        f = torch.where(mRs, FRs[k], f)
        f = torch.where(mLs, FLs[k], f)
        f = torch.where(mG, FG[k], f)
        f = torch.where(mFR, FR[k], f)
        f = torch.where(mFL, FL[k], f)
        out[k] = f
    # GLM fluxes (:580-581)
    out[bn] = 0.5 * ((L[PS] + R[PS]) - ch * (R[bn] - L[bn]))
    out[PS] = 0.5 * (ch * ch * (L[bn] + R[bn]) - ch * (R[PS] - L[PS]))
    return torch.stack(out)


def _sign_vec(mask, like):
    return torch.tensor([-1.0 if (mask >> v) & 1 else 1.0 for v in range(9)], dtype=like.dtype,
                        device=like.device).view(9, 1, 1)


def bc(U, bc_kind, bc_flip):
    """Ghost fill (bc.f90): x sides, then y sides over the full rows."""
    for axis, lo, hi in ((2, 0, 1), (1, 2, 3)):
        n = U.shape[axis]
        if bc_kind[lo] == 0:
            g0, g1 = U.narrow(axis, n - 2, 1), U.narrow(axis, 1, 1)
        else:
            g0 = _sign_vec(bc_flip[lo], U) * U.narrow(axis, 1, 1)
            g1 = _sign_vec(bc_flip[hi], U) * U.narrow(axis, n - 2, 1)
        U = torch.cat([g0, U.narrow(axis, 1, n - 2), g1], axis)
    return U


def glm(U, f):
    scale = torch.ones(9, 1, 1, dtype=U.dtype, device=U.device)
    scale[PS] = f
    return U * scale


def flux_div(U, dt, ch, cfg):
    g = cfg.gamma
    w = u2v(U, g)
    out = []
    for d, axis in ((1, 2), (2, 1)):
        lo, hi = 2 * (d - 1), 2 * (d - 1) + 1
        per = cfg.bc_kind[lo] == 0
        L, R = face_states(w, axis, {"minmod": 1, "mc": 2}[cfg.limiter], per, _sign_vec(cfg.bc_flip[lo], U),
                           _sign_vec(cfg.bc_flip[hi], U))
        out.append(hlld(L, R, ch, g, d))
    F, G = out
    dtx, dty = dt / cfg.dx, dt / cfg.dy
    D = dtx * (F[:, 1:-1, :-1] - F[:, 1:-1, 1:]) + dty * (G[:, :-1, 1:-1] - G[:, 1:, 1:-1])
    return torch.nn.functional.pad(D, (1, 1, 1, 1))


def step(U, dt, ch, f, cfg):
    """One TVD-RK2 step (2D_basic/main.f90:56-188) with dt, ch and the GLM factor given."""
    Ua = glm(U, f)
    U1 = bc(Ua + flux_div(Ua, dt, ch, cfg), cfg.bc_kind, cfg.bc_flip)
    U2 = bc(0.5 * (Ua + U1 + flux_div(U1, dt, ch, cfg)), cfg.bc_kind, cfg.bc_flip)
    return glm(U2, f)


def evolve(U0, log, cfg):
    """bc of the initial state, then one step per row (dt, ch, f) of `log`."""
    U = bc(U0, cfg.bc_kind, cfg.bc_flip)
    for dt, ch, f in log:
        U = step(U, float(dt), float(ch), float(f), cfg)
    return U
