"""Output cadence of Solver.run_with_output against the reference's main loop
(2D_basic/main.f90:41-75), on a stand-in solver with the device's stepping
semantics (steps stop at the first t >= tend), so that it runs without a GPU."""
import json
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
        with open(path, "w") as f:
            json.dump([self.t, self.k], f)

    def read_snapshot(self, path):
        with open(path) as f:
            self.t, self.k = json.load(f)
        return self


def reference_loop(dts, tend, dtout, restart=None):
    """main.f90:41-75: output check, end check, one step, per iteration.
    restart = (n_start, t, k) continues from a file as mainp.f90:104-117 does:
    n_output = n_start + 1, t_output = t + dtout, and the restart file is not
    written again (mainp.f90:132)."""
    t, k, n_output = 0.0, 0, 0
    t_output = -dts[0] / 3.0
    if restart:
        n, t, k = restart
        n_output, t_output = n + 1, t + dtout
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


@pytest.mark.parametrize("n_start", [3, -1])
def test_restart_continues_the_reference_cadence(tmp_path, n_start):
    """Restart from file 3 (n_start = 3) or from the newest file (n_start < 0,
    searched from floor(tend/dtout) down, mainp.f90:85-101): the run reads the
    file, writes files 4, 5, ... at t_file + dtout, t_file + 2 dtout, ... and
    ends at the first t >= tend, as the reference loop does after a restart."""
    dts, tend, dtout = [0.013], 1.0, 0.1
    full = StandIn(dts)
    run_with_output(full, 0.45, dtout, outdir=str(tmp_path))  # a first run that stopped early
    names = sorted(os.listdir(tmp_path))
    assert names[-1] == "field-00004.dat"
    n = 3 if n_start > 0 else 4
    if n_start > 0:
        os.remove(tmp_path / "field-00004.dat")
        names = names[:-1]
    _, t_n, k_n = [f for f in full.files if f[0] == "field-%05d.dat" % n][0]
    s = StandIn(dts)
    paths = run_with_output(s, tend, dtout, outdir=str(tmp_path), n_start=n_start)
    assert s.files == reference_loop(dts, tend, dtout, restart=(n, t_n, k_n))
    assert s.files[0][0] == "field-%05d.dat" % (n + 1)
    assert [os.path.basename(p) for p in paths] == [f[0] for f in s.files]
    assert s.t >= tend


def test_restart_search_without_files_starts_fresh(tmp_path):
    dts, tend, dtout = [0.013], 0.5, 0.1
    s = StandIn(dts)
    run_with_output(s, tend, dtout, outdir=str(tmp_path), n_start=-1)
    assert s.files == reference_loop(dts, tend, dtout)
