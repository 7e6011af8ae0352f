"""Parity at the sizes the benchmark measures: the GB300 FP64 path against the
oracle's restatement of the reference driver loop (2D_basic/main.f90:56-188)
from identical initial states.

* Kelvin-Helmholtz 4096x2048 (HLLD, minmod, GLM, TVD-RK2, zero-gradient y
  walls, CFL 0.4): the headline workload of the benchmark.  1 step within 1e-12
  and 10 steps within 1e-9 per variable, in the scaled L1 norm and in each
  variable's own relative L1 norm (the FP64 path's parity tolerances).
* Orszag-Tang 256x256 (HLLD, MC, GLM, periodic) run to t = pi, the reference
  2D_basic problem: the same step count as the reference loop (which stops at
  the first t >= tend, main.f90:73) and all 9 fields within the N-step tolerance.
* Resistive Harris sheet 64x32x64 (the 3D configuration's physics on a grid the
  serial oracle finishes in seconds): 1 step within 1e-12, 10 steps within 1e-9.

The oracle's OpenMP build runs the large grids; it is bitwise equal to the
serial build (tests/test_oracle.py)."""
import math

import numpy as np
import pytest

from helpers import assert_parity

pytestmark = pytest.mark.gpu


def _pair(cfg, model, omp=False):
    from openmhd_gb300 import Solver
    from oracle.oracle import Grid

    s = Solver(cfg).init_model(model)
    g = Grid.from_solver_config(cfg, omp=omp)
    g.U[...] = s.get_state_numpy()
    return s, g


def test_kelvin_helmholtz_4096x2048_fp64_vs_oracle(cuda_lib, oracle_mod):
    from openmhd_gb300 import kelvin_helmholtz

    cfg, model = kelvin_helmholtz(4096, 2048, precision="fp64")
    assert (cfg.ix, cfg.jx, cfg.limiter, cfg.flux, cfg.cfl) == (4098, 2050, "minmod", "hlld", 0.4)
    s, g = _pair(cfg, model, omp=True)
    s.step(1)
    info = s.sync()
    g.step(1)
    assert info.status == 0 and abs(info.dt - g.last_dt) <= 1e-14 * g.last_dt
    sc, own, li, _ = assert_parity(s.get_state_numpy(), g.U, 1e-12, "KH 4096x2048, 1 step")
    print("KH 4096x2048 1 step: scaled", sc.max(), "own", own.max(), "linf", li.max())
    s.step(9)
    info = s.sync()
    g.step(9)
    assert info.status == 0 and info.steps == 10
    assert abs(info.t - g.t) <= 1e-13 * g.t
    sc, own, li, _ = assert_parity(s.get_state_numpy(), g.U, 1e-9, "KH 4096x2048, 10 steps")
    print("KH 4096x2048 10 steps: scaled", sc.max(), "own", own.max(), "linf", li.max())


def test_orszag_tang_256_to_pi_vs_oracle(cuda_lib, oracle_mod):
    from openmhd_gb300 import orszag_tang

    cfg, model = orszag_tang(256, precision="fp64")
    assert (cfg.ix, cfg.jx, cfg.limiter, cfg.flux, cfg.tend) == (258, 258, "mc", "hlld", math.pi)
    s, g = _pair(cfg, model, omp=True)
    info = s.run_until(math.pi)
    g.run_until(math.pi)
    assert info.status == 0 and info.done == 1
    assert info.steps == g.steps, (info.steps, g.steps)
    assert g.t >= math.pi and abs(info.t - g.t) <= 1e-12 * g.t
    sc, own, li, _ = assert_parity(s.get_state_numpy(), g.U, 1e-9, f"OT 256^2 to t=pi ({g.steps} steps)")
    print(f"OT 256^2 to t=pi, {g.steps} steps: scaled", sc.max(), "own", own.max(), "linf", li.max())


def test_harris3d_64x32x64_fp64_vs_oracle(cuda_lib, oracle_mod):
    from openmhd_gb300 import harris3d

    cfg, model = harris3d(64, 32, 64, precision="fp64")
    s, g = _pair(cfg, model, omp=True)
    s.step(1)
    info = s.sync()
    g.step(1)
    assert info.status == 0 and abs(info.dt - g.last_dt) <= 1e-14 * g.last_dt
    sc, own, li, gated = assert_parity(s.get_state_numpy(), g.U, 1e-12, "Harris 64x32x64, 1 step")
    print("Harris 64x32x64 1 step: scaled", sc.max(), "own (all)", own, "gated", gated)
    s.step(9)
    info = s.sync()
    g.step(9)
    assert info.status == 0 and info.steps == 10
    sc, own, li, _ = assert_parity(s.get_state_numpy(), g.U, 1e-9, "Harris 64x32x64, 10 steps")
    print("Harris 64x32x64 10 steps: scaled", sc.max(), "own", own.max(), "linf", li.max())
