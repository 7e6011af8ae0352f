"""Gradients through time of the fused FP64 2D step (omhd_adjoint_* in the C
ABI), exposed to PyTorch as a torch.autograd.Function.

`AdjointRun` owns one omhd_adjoint handle: `forward(U0)` runs N steps with
the fused kernels and keeps a checkpoint every `checkpoint_every` steps;
`backward(gUN)` recomputes one segment of steps at a time from its checkpoint
and runs the hand-written adjoint kernels of each RK stage in reverse, giving
dJ/dU0 for the gradient dJ/dU_N of any scalar functional.  dt and ch are the
values the forward run computed (set_dt.f90), held fixed in the derivative.

`Evolve.apply(U0, run)` is the differentiable map U0 -> U_N; initial-state
builders and objectives are ordinary torch code around it, e.g.

    run = AdjointRun(cfg, nsteps=400, checkpoint_every=20)
    U0 = kh_state(base, vy)                 # differentiable in vy
    UN = Evolve.apply(U0, run)
    J = (UN[BY - 1, 1:-1, 1:-1] ** 2).sum()
    J.backward()                           # vy.grad = dJ/dvy0
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np
import torch

from . import _lib
from .solver import OmhdError, SolverConfig

NV = 9


def _check_device_array(name: str, a, shape) -> None:
    """Refuse what the adjoint kernels cannot take as it is: they read and
    write tuple(shape) float64 values at the tensor's address on the current
    device, so a smaller, strided, other-typed or other-device tensor is an
    error here, not an out-of-bounds access on the GPU."""
    if not isinstance(a, torch.Tensor) or not a.is_cuda:
        raise TypeError(f"{name} must be a CUDA tensor")
    if a.device.index != torch.cuda.current_device():
        raise ValueError(f"{name} is on cuda:{a.device.index}, not the current device cuda:{torch.cuda.current_device()}")
    if a.dtype != torch.float64 or not a.is_contiguous():
        raise TypeError(f"{name} must be a contiguous float64 tensor")
    if tuple(a.shape) != tuple(shape):
        raise ValueError(f"{name} has shape {tuple(a.shape)}, expected {tuple(shape)}")


class AdjointRun:
    def __init__(self, cfg: SolverConfig, nsteps: int, checkpoint_every: int | None = None, stream=None):
        if not torch.cuda.is_available():
            raise RuntimeError("openmhd_gb300.AdjointRun needs a CUDA device")
        if checkpoint_every is None:
            checkpoint_every = max(1, int(round(math.sqrt(nsteps))))
        self.cfg = cfg
        self.nsteps = int(nsteps)
        self.checkpoint_every = int(checkpoint_every)
        self.lib = _lib.load()
        self._h = C.c_void_p()
        ccfg = cfg.to_c()
        st = self.lib.omhd_adjoint_create(C.byref(ccfg), self.nsteps, self.checkpoint_every, C.byref(self._h))
        if st:
            raise OmhdError(st, "omhd_adjoint_create rejected the configuration")
        self.stream = stream if stream is not None else torch.cuda.Stream()
        self._check(self.lib.omhd_adjoint_set_stream(self._h, C.c_void_p(self.stream.cuda_stream)))

    def _check(self, st: int, what: str = "adjoint call failed"):
        if st:
            raise OmhdError(st, what)

    def close(self):
        if self._h:
            self.lib.omhd_adjoint_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _as_state(self, U):
        return U.detach().to(device="cuda", dtype=torch.float64).contiguous().reshape(self.cfg.shape)

    def forward(self, U0):
        """U_N of nsteps steps from U0 (bc is applied to a copy of U0)."""
        return self._run(self.lib.omhd_adjoint_forward, U0, "adjoint forward failed")

    def backward(self, gUN):
        """dJ/dU0 given dJ/dU_N (zero at ghost cells)."""
        g = self._as_state(gUN)
        out = torch.empty(self.cfg.shape, dtype=torch.float64, device="cuda")
        self.stream.wait_stream(torch.cuda.current_stream())
        self._check(self.lib.omhd_adjoint_backward(self._h, g.data_ptr(), out.data_ptr()), "adjoint backward failed")
        g.record_stream(self.stream)
        out.record_stream(self.stream)
        torch.cuda.current_stream().wait_stream(self.stream)
        return out

    def _run(self, fn, U0, what):
        src = self._as_state(U0)
        out = torch.empty(self.cfg.shape, dtype=torch.float64, device="cuda")
        self.stream.wait_stream(torch.cuda.current_stream())
        self._check(fn(self._h, src.data_ptr(), out.data_ptr()), what)
        src.record_stream(self.stream)
        out.record_stream(self.stream)
        torch.cuda.current_stream().wait_stream(self.stream)
        return out

    def record(self, U0):
        """forward(U0) that also records every step's decision tape (limiter
        selections, HLLD branches) for replay()."""
        return self._run(self.lib.omhd_adjoint_record, U0, "adjoint record failed")

    def replay(self, U0):
        """U_N from U0 with every decision and every dt, ch, GLM factor frozen
        to the last record() run: the smooth map the adjoint differentiates."""
        return self._run(self.lib.omhd_adjoint_replay, U0, "adjoint replay failed")

    def step_vjp(self, Un, U1, log3, lam_in, lam_out):
        """Adjoint of one step given its stage inputs (device tensors); lam_in is overwritten."""
        for name, a, shape in (("Un", Un, self.cfg.shape), ("U1", U1, self.cfg.shape), ("log3", log3, (3,)),
                               ("lam_in", lam_in, self.cfg.shape), ("lam_out", lam_out, self.cfg.shape)):
            _check_device_array(name, a, shape)
        self._check(self.lib.omhd_adjoint_step_vjp(self._h, Un.data_ptr(), U1.data_ptr(), log3.data_ptr(),
                                                   lam_in.data_ptr(), lam_out.data_ptr()), "step adjoint failed")

    def sync(self):
        self._check(self.lib.omhd_adjoint_sync(self._h), "a forward step reported a failure")

    def step_log(self) -> np.ndarray:
        """(nsteps, 3) array of dt, ch and the GLM factor of each forward step."""
        out = np.empty((self.nsteps, 3))
        self._check(self.lib.omhd_adjoint_step_log(self._h, out.ctypes.data))
        return out

    @property
    def memory_bytes(self) -> int:
        b = C.c_size_t()
        self._check(self.lib.omhd_adjoint_memory(self._h, C.byref(b)))
        return int(b.value)


class Evolve(torch.autograd.Function):
    """U_N = steps^N(U0) with the hand-written adjoint as its backward."""

    @staticmethod
    def forward(ctx, U0, run: AdjointRun):
        ctx.run = run
        return run.forward(U0).to(dtype=U0.dtype).reshape(U0.shape)

    @staticmethod
    def backward(ctx, gUN):
        g = ctx.run.backward(gUN)
        return g.to(dtype=gUN.dtype).reshape(gUN.shape), None


def primitive_state(U, gamma: float):
    """(rho, v(3), p, B(3), psi) of a conserved state tensor (9, ...), as torch ops."""
    ro = U[4]
    v = U[0:3] / ro
    B = U[5:8]
    p = (gamma - 1) * (U[3] - 0.5 * ((v * U[0:3]).sum(0) + (B * B).sum(0)))
    return ro, v, p, B, U[8]


def kh_state(base, vy, gamma: float = 5.0 / 3.0):
    """The state `base` (9, jx, ix) with its interior vy replaced by `vy`
    ((jx-2, ix-2), differentiable), keeping rho, vx, vz, p, B and psi: my =
    rho vy and E = p/(gamma-1) + rho v^2/2 + B^2/2 (the KH model's map from
    primitives)."""
    ro, v, p, B, ps = primitive_state(base, gamma)
    vy_full = torch.nn.functional.pad(vy, (1, 1, 1, 1)) + v[1] * _ring_mask(base)
    vx, vz = v[0], v[2]
    v2 = vx * vx + vy_full * vy_full + vz * vz
    B2 = (B * B).sum(0)
    E = 0.5 * (ro * v2 + B2) + p / (gamma - 1)
    return torch.stack([ro * vx, ro * vy_full, ro * vz, E, ro, B[0], B[1], B[2], ps])


def _ring_mask(U):
    m = torch.ones(U.shape[1:], dtype=U.dtype, device=U.device)
    m[1:-1, 1:-1] = 0
    return m
