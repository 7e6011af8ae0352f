"""Batched ensemble: every member of one persistent launch must evolve as the
same problem run alone by the single-grid solver.  The two are different
kernels built from the same source; with multiply-add contraction on, the
compiler may contract differently in each, so they agree to rounding (FP64
1e-12, FP32-mixed 1e-6 scaled L1), while two ensemble runs with different
launch paths (stream vs graph) agree bit for bit."""
import numpy as np
import pytest

from helpers import scaled_l1

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision,tol", [("mixed", 1e-6), ("fp64", 1e-12)])
def test_members_match_single_grid_runs(cuda_lib, precision, tol):
    from openmhd_gb300 import Solver
    from openmhd_gb300.ensemble import Ensemble, batched_problem_set

    cfgs, models = batched_problem_set(6, seed=3, precision=precision, sides=[40, 72, 96, 130])
    ens = Ensemble(cfgs).init_models(models)
    kind, cps, ms = ens.autotune(steps=1)
    assert 0 <= kind < 5 and 1 <= cps <= 4 and ms > 0
    ens.step(3)
    infos = ens.sync()
    for i, (c, m) in enumerate(zip(cfgs, models)):
        s = Solver(c).init_model(m)
        s.step(3)  # the autotuner leaves the ensemble state where it found it
        ref = s.get_state_numpy()
        info = s.sync()
        assert infos[i].steps == info.steps
        assert abs(infos[i].t - info.t) <= tol * info.t
        err = scaled_l1(ens.member_state(i)[:, 1:-1, 1:-1], ref[:, 1:-1, 1:-1])
        assert np.all(err <= tol), (i, err)


def test_graph_replay_and_per_member_dt(cuda_lib):
    from openmhd_gb300.ensemble import Ensemble, batched_problem_set

    cfgs, models = batched_problem_set(4, seed=5, precision="mixed", sides=[64, 128])
    a = Ensemble(cfgs).init_models(models)
    b = Ensemble(cfgs).init_models(models)
    a.step(6)
    b.step_graph(3, replays=2)
    ia, ib = a.sync(), b.sync()
    dts = {round(x.dt, 12) for x in ia}
    assert len(dts) > 1  # members keep their own dt
    for i in range(len(cfgs)):
        assert ia[i].steps == ib[i].steps == 6
        assert np.array_equal(a.member_state(i), b.member_state(i))


def test_autotune_leaves_state_unchanged(cuda_lib):
    """Every candidate tiling is timed from the same saved state, and the
    state, times and step counts are put back afterwards, bit for bit."""
    from openmhd_gb300.ensemble import Ensemble, batched_problem_set

    cfgs, models = batched_problem_set(5, seed=7, precision="mixed", sides=[48, 80])
    ens = Ensemble(cfgs).init_models(models)
    ens.step(2)
    before = [ens.member_state(i).copy() for i in range(len(cfgs))]
    info0 = ens.sync()
    ens.autotune(steps=2)
    info1 = ens.sync()
    for i in range(len(cfgs)):
        assert np.array_equal(ens.member_state(i), before[i])
        assert info1[i].steps == info0[i].steps and info1[i].t == info0[i].t


def test_members_at_bench_sizes_vs_oracle(cuda_lib, oracle_mod):
    """FP64 ensemble members at the batched configuration's side lengths
    (256..1024, one Orszag-Tang and one Kelvin-Helmholtz member, non-square)
    against the oracle directly, from the members' own initial states: 1 step
    within 1e-12 and 5 steps within 1e-9 per variable (scaled L1 and own-norm
    relative L1 above round-off), the FP64 tolerances of the single-grid path."""
    from helpers import assert_parity
    from openmhd_gb300.ensemble import Ensemble, batched_problem_set
    from oracle.oracle import Grid

    cfgs, models = batched_problem_set(2, seed=11, precision="fp64", sides=[256, 320, 512, 1024])
    assert all(min(c.ix, c.jx) - 2 >= 256 for c in cfgs)
    ens = Ensemble(cfgs).init_models(models)
    grids = []
    for i, c in enumerate(cfgs):
        g = Grid.from_solver_config(c, omp=True)
        g.U[...] = ens.member_state(i)
        grids.append(g)
    ens.step(1)
    infos = ens.sync()
    for i, g in enumerate(grids):
        g.step(1)
        assert infos[i].status == 0 and abs(infos[i].dt - g.last_dt) <= 1e-14 * g.last_dt
        assert_parity(ens.member_state(i), g.U, 1e-12, f"member {i}, 1 step")
    ens.step(4)
    infos = ens.sync()
    for i, g in enumerate(grids):
        g.step(4)
        assert infos[i].steps == 5
        assert_parity(ens.member_state(i), g.U, 1e-9, f"member {i}, 5 steps")
