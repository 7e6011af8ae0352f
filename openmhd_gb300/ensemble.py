"""Ensembles of independent 2D problems advanced by one persistent batched
kernel per RK stage (omhd_ensemble_* in the C ABI).

`batched_problem_set` builds the 128-member ensemble of the batched
benchmark: side lengths drawn from {128, 192, ..., 1024} with a fixed seed,
half Orszag-Tang (B amplitude in [0.5, 1.5], phase shifts in [0, 2pi)), half
Kelvin-Helmholtz (shear in [0.3, 0.8], Bx in [0.05, 0.3]), each with its own
grid, model and dt.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _lib
from .solver import ModelSpec, OmhdError, SolverConfig, kelvin_helmholtz, orszag_tang

SIDES = list(range(128, 1025, 64))


def batched_problem_set(n: int = 128, seed: int = 0, precision: str = "mixed", sides=None):
    rng = np.random.default_rng(seed)
    sides = SIDES if sides is None else sides
    cfgs, models = [], []
    two_pi = 2 * math.pi
    for i in range(n):
        nx = int(rng.choice(sides))
        ny = int(rng.choice(sides))
        if i % 2 == 0:
            cfg, m = orszag_tang(nx, ny, precision=precision, amp=float(rng.uniform(0.5, 1.5)),
                                 phase_x=float(rng.uniform(0, two_pi)), phase_y=float(rng.uniform(0, two_pi)))
        else:
            cfg, m = kelvin_helmholtz(nx, ny, precision=precision, shear=float(rng.uniform(0.3, 0.8)),
                                      bx0=float(rng.uniform(0.05, 0.3)), seed=int(rng.integers(0, 2**31)))
        cfgs.append(cfg)
        models.append(m)
    return cfgs, models


class Ensemble:
    def __init__(self, cfgs: list[SolverConfig], stream=None):
        import torch

        self.lib = _lib.load()
        self.cfgs = cfgs
        arr = (_lib.Config * len(cfgs))(*[c.to_c() for c in cfgs])
        self._h = C.c_void_p()
        st = self.lib.omhd_ensemble_create(arr, len(cfgs), C.byref(self._h))
        if st:
            raise OmhdError(st, "omhd_ensemble_create rejected the configurations")
        self.stream = stream if stream is not None else torch.cuda.Stream()
        self.lib.omhd_ensemble_set_stream(self._h, C.c_void_p(self.stream.cuda_stream))

    def close(self):
        if self._h:
            self.lib.omhd_ensemble_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def init_models(self, models: list[ModelSpec]):
        import torch

        if len(models) != len(self.cfgs):  # the library reads one model per member
            raise ValueError(f"{len(models)} models for {len(self.cfgs)} members")
        torch.cuda.current_stream().synchronize()
        arr = (_lib.Model * len(models))(*[m.to_c() for m in models])
        st = self.lib.omhd_ensemble_init_models(self._h, arr)
        if st:
            raise OmhdError(st, "model initialisation failed")
        self.sync()
        return self

    def set_tiling(self, kind: int, ctas_per_sm: int):
        st = self.lib.omhd_ensemble_set_tiling(self._h, kind, ctas_per_sm)
        if st:
            raise OmhdError(st, "bad tiling")

    def autotune(self, steps: int = 3):
        k, c, ms = C.c_int(), C.c_int(), C.c_double()
        st = self.lib.omhd_ensemble_autotune(self._h, steps, C.byref(k), C.byref(c), C.byref(ms))
        if st:
            raise OmhdError(st, "autotune failed")
        return k.value, c.value, ms.value

    def step(self, n: int = 1):
        st = self.lib.omhd_ensemble_step(self._h, n)
        if st:
            raise OmhdError(st, "ensemble step failed")
        return self

    def step_graph(self, n: int, replays: int = 1):
        st = self.lib.omhd_ensemble_step_graph(self._h, n, replays)
        if st:
            raise OmhdError(st, "ensemble graph step failed")
        return self

    def sync(self):
        infos = (_lib.StepInfo * len(self.cfgs))()
        st = self.lib.omhd_ensemble_sync(self._h, infos)
        if st:
            raise OmhdError(st, "an ensemble member failed")
        return list(infos)

    def member_state(self, i: int) -> np.ndarray:
        if not 0 <= i < len(self.cfgs):
            raise IndexError(f"member {i} of {len(self.cfgs)}")
        h = C.c_void_p()
        st = self.lib.omhd_ensemble_member(self._h, i, C.byref(h))
        if st:
            raise OmhdError(st, f"no member {i}")
        out = np.empty(self.cfgs[i].shape)
        st = self.lib.omhd_solver_get_state(h, out.ctypes.data)
        if st:
            raise OmhdError(st, "state download failed")
        return out

    @property
    def cells(self) -> int:
        return sum(c.interior_cells for c in self.cfgs)
