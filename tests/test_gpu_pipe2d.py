"""The warp-specialised (pipelined) FP64 2D stage kernel against the one-role
FP64 2D kernel (omhd_set_2d_pipeline(0)): HLLD with minmod or MC, producer
warps loading, recovering the primitives and reconstructing tile i+1 while
consumer warps solve the faces of tile i and update it.  Cases have more tiles
than the GPU has SMs (every CTA runs several tiles through both buffers),
ragged edge tiles, walls and periodic edges; the two kernels compute the same
expressions and agree to FP64 rounding (scaled L1 <= 1e-13 after 4 steps).

The FP32-mixed path keeps one-role kernels (four 16x8-tile CTAs per SM): a
pipelined FP32-mixed variant (4 producer + 9 consumer warps, 32x8 tiles, and
variants with 2 or 6 producer warps and 32x12 or 32x16 tiles) ran 3-11 %
slower than the one-role kernel of the time on KH 4096x2048."""
import numpy as np
import pytest

from helpers import scaled_l1

pytestmark = pytest.mark.gpu


def _run(lib, cfg, model, steps, pipe=True):
    from openmhd_gb300 import Solver

    lib.omhd_set_2d_pipeline(1 if pipe else 0)
    try:
        s = Solver(cfg).init_model(model)
        s.step(steps)
        info = s.sync()
        return s.get_state_numpy(), info
    finally:
        lib.omhd_set_2d_pipeline(1)


def _case(name):
    from openmhd_gb300 import kelvin_helmholtz, orszag_tang

    if name == "kh1000x300":  # x periodic, y walls, 63 x 19 tiles of 16x16 with ragged edges
        return kelvin_helmholtz(1000, 300, precision="fp64")
    if name == "ot416x280_mc":  # periodic, MC limiter
        return orszag_tang(416, 280, precision="fp64", limiter="mc")
    return orszag_tang(97, 64, precision="fp64")  # odd ix: no TMA staging, ordinary loads


@pytest.mark.parametrize("name", ["kh1000x300", "ot416x280_mc", "ot97x64"])
def test_fp64_pipelined_matches_one_role(cuda_lib, name):
    cfg, model = _case(name)
    a, ia = _run(cuda_lib, cfg, model, 4, pipe=True)
    b, ib = _run(cuda_lib, cfg, model, 4, pipe=False)
    assert ia.status == 0 and ib.status == 0 and ia.steps == ib.steps == 4
    err = scaled_l1(a[:, 1:-1, 1:-1], b[:, 1:-1, 1:-1])
    print(f"{name}: pipelined vs one-role max scaled L1 {err.max():.3e}, bit-identical {np.array_equal(a, b)}")
    assert np.all(err <= 1e-13), err
