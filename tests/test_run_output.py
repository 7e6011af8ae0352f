"""Output cadence of Solver.run_with_output against the reference's main loop
(2D_basic/main.f90:41-75), on a stand-in solver with the device's stepping
semantics (steps stop at the first t >= tend), so that it runs without a GPU."""
import math
import os
from types import SimpleNamespace

import pytest

from openmhd_gb300.solver import run_with_output


class StandIn:
    """Steps through a prescribed dt sequence; stepping stops at the first t >= tend."""

    def __init__(self, dts):
        self.dts, self.k, self.t, self.tend, self.files = list(dts), 0, 0.0, math.inf, []

    def _dt(self):
        return self.dts[min(self.k, len(self.dts) - 1)]

    def sync(self):
        return SimpleNamespace(t=self.t, dt=self._dt(), done=int(self.t >= self.tend), steps=self.k)

    def set_tend(self, tend):
        self.tend = tend if tend > 0 else math.inf

    def step(self, n=1):
        for _ in range(n):
            if self.t >= self.tend:
                break
            self.t += self._dt()
            self.k += 1
        return self

    def run_until(self, tend, batch=64):
        self.set_tend(tend)
        while self.t < self.tend:
            self.step(batch)
        return self.sync()

    def write_snapshot(self, path):
        self.files.append((os.path.basename(path), self.t, self.k))


def reference_loop(dts, tend, dtout):
    """main.f90:41-75: output check, end check, one step, per iteration."""
    t, k, n_output = 0.0, 0, 0
    t_output = -dts[0] / 3.0
    out = []
    while True:
        if t >= t_output:
            out.append(("field-%05d.dat" % n_output, t, k))
            n_output += 1
            t_output += dtout
        if t >= tend:
            return out
        t += dts[min(k, len(dts) - 1)]
        k += 1


@pytest.mark.parametrize("case", ["constant", "growing", "shrinking"])
def test_files_fall_on_the_reference_steps(tmp_path, case):
    if case == "constant":
        dts, tend, dtout = [0.013], 1.0, 0.1
    elif case == "growing":  # late steps longer than dtout: one file per step, as in the reference
        dts, tend, dtout = [0.01 * 1.15**n for n in range(60)], 3.0, 0.1
    else:
        dts, tend, dtout = [0.05 / (1 + 0.1 * n) for n in range(400)], 0.7, 0.05
    s = StandIn(dts)
    paths = run_with_output(s, tend, dtout, outdir=str(tmp_path))
    assert s.files == reference_loop(dts, tend, dtout)
    assert [os.path.basename(p) for p in paths] == [f[0] for f in s.files]
    assert s.tend == tend and s.t >= tend


def test_first_dt_above_dtout_stops(tmp_path):
    with pytest.raises(ValueError):
        run_with_output(StandIn([0.2]), 1.0, 0.1, outdir=str(tmp_path))
