"""TMA staging of halo tiles in the FP64 pipelined 2D stage kernel.

Tiles whose halo lies wholly inside the array are staged in shared memory by
one 3D cp.async.bulk.tensor load (producer thread 0, mbarrier completion);
edge tiles and arrays TMA cannot address (odd ix) take ordinary loads.  The
arithmetic after the load is the same, so a run with staging must equal a run
with staging switched off (omhd_set_tma_staging(0)) bit for bit, and both
must keep parity with the oracle (tests/test_gpu_fused.py,
tests/test_gpu_bench_configs.py run with staging on)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(lib, cfg, model, steps, tma):
    from openmhd_gb300 import Solver

    lib.omhd_set_tma_staging(1 if tma else 0)
    try:
        s = Solver(cfg).init_model(model)
        s.step(steps)
        info = s.sync()
        return s.get_state_numpy(), info
    finally:
        lib.omhd_set_tma_staging(1)


@pytest.mark.parametrize("case", ["kh4096x2048", "kh560x300", "ot416x280_mc", "ot_odd_ix"])
def test_staged_and_plain_loads_agree_bitwise(cuda_lib, case):
    from openmhd_gb300 import kelvin_helmholtz, orszag_tang

    steps = 3
    if case == "kh4096x2048":
        cfg, model = kelvin_helmholtz(4096, 2048, precision="fp64")
        steps = 2
    elif case == "kh560x300":
        cfg, model = kelvin_helmholtz(560, 300, precision="fp64")
    elif case == "ot416x280_mc":
        cfg, model = orszag_tang(416, 280, precision="fp64", limiter="mc")
    else:  # ix = 99: TMA cannot address the rows (odd pitch); ordinary loads throughout
        cfg, model = orszag_tang(97, 64, precision="fp64")
    a, ia = _run(cuda_lib, cfg, model, steps, True)
    b, ib = _run(cuda_lib, cfg, model, steps, False)
    assert ia.status == 0 and ib.status == 0 and ia.steps == ib.steps == steps
    assert ia.t == ib.t
    assert np.array_equal(a, b)
