"""binary32 <-> binary64 conversions on the integer pipe
(openmhd_gb300/csrc/omhd_fastmath.h: narrow_f64, widen_f32), which the
FP32-mixed kernels use for every primitive they load and every face flux they
widen.  Evaluated on the GPU through omhd_probe_convert and compared bit for
bit with the host's IEEE conversions (numpy: round to nearest even):

* narrow_f64 equals float32(x) for every |x| >= 2^-126 (overflow to inf
  included); a smaller |x| gives a zero of x's sign; NaN gives NaN;
* widen_f32 equals float64(f) for every normal float, +-0 and +-inf; a
  subnormal float gives a zero of its sign; NaN gives NaN with its sign.

Arguments: uniformly random 64- and 32-bit patterns (every exponent), random
values in the ranges the solver meets, the rounding ties and their neighbours,
and the edges of the binary32 range."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TINY32 = np.float64(2.0**-126)


def _probe(lib, xd: np.ndarray, xf: np.ndarray):
    import torch

    n = max(xd.size, xf.size)
    xd = np.resize(xd, n).astype(np.float64)
    xf = np.resize(xf, n).astype(np.float32)
    td = torch.from_numpy(xd).cuda()
    tf = torch.from_numpy(xf).cuda()
    nd = torch.empty(n, dtype=torch.float32, device="cuda")
    wf = torch.empty(n, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    rc = lib.omhd_probe_convert(C.c_void_p(td.data_ptr()), C.c_void_p(nd.data_ptr()), C.c_void_p(tf.data_ptr()),
                                C.c_void_p(wf.data_ptr()), n)
    assert rc == 0
    return xd, nd.cpu().numpy(), xf, wf.cpu().numpy()


def _doubles(rng) -> np.ndarray:
    bits = rng.integers(0, 2**63, size=1 << 20, dtype=np.int64).astype(np.uint64)
    bits[: 1 << 19] |= np.uint64(1) << np.uint64(63)  # both signs
    every = bits.view(np.float64)
    solver = np.exp2(rng.uniform(-140, 130, 1 << 20)) * rng.choice([-1.0, 1.0], 1 << 20)
    # ties: a float plus exactly half its ulp (and the neighbours of that)
    f = rng.uniform(-1e3, 1e3, 1 << 16).astype(np.float32)
    half = (np.nextafter(f, np.float32(np.inf)).astype(np.float64) - f.astype(np.float64)) / 2
    ties = f.astype(np.float64) + half
    ties = np.concatenate([ties, np.nextafter(ties, np.inf), np.nextafter(ties, -np.inf)])
    fmax = np.float64(np.finfo(np.float32).max)
    ulp_top = np.float64(2.0**104)
    edges = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 1.0, -1.0, fmax, -fmax, fmax + ulp_top / 2,
                      np.nextafter(fmax + ulp_top / 2, 0), np.nextafter(fmax + ulp_top / 2, np.inf), 2.0**128,
                      TINY32, -TINY32, np.nextafter(TINY32, 0), np.nextafter(TINY32, 1), 2.0**-149, 1e-300,
                      5e-324, np.finfo(np.float64).max, 0.1, 1 / 3])
    return np.concatenate([every, solver, ties, edges, -edges])


def _floats(rng) -> np.ndarray:
    bits = rng.integers(0, 2**32, size=1 << 20, dtype=np.int64).astype(np.uint32)
    every = bits.view(np.float32)
    edges = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 1.0, np.finfo(np.float32).max,
                      np.finfo(np.float32).tiny, np.nextafter(np.finfo(np.float32).tiny, np.float32(0)),
                      np.float32(2.0**-149)], dtype=np.float32)
    return np.concatenate([every, edges, -edges]).astype(np.float32)


def test_narrow_matches_ieee_round_to_nearest(cuda_lib):
    rng = np.random.default_rng(7)
    xd, nd, _, _ = _probe(cuda_lib, _doubles(rng), np.zeros(1, np.float32))
    nan = np.isnan(xd)
    small = ~nan & (np.abs(xd) < TINY32)
    big = ~nan & ~small
    with np.errstate(over="ignore"):
        want = xd[big].astype(np.float32)
    got = nd[big]
    bad = want.view(np.uint32) != got.view(np.uint32)
    assert not bad.any(), f"{bad.sum()} mismatches, first x={xd[big][bad][:4]!r} got {got[bad][:4]!r} want {want[bad][:4]!r}"
    # below the normal binary32 range: a zero of the argument's sign
    assert np.all(nd[small] == 0) and np.all(np.signbit(nd[small]) == np.signbit(xd[small]))
    assert np.all(np.isnan(nd[nan]))
    print(f"narrow: {big.sum()} normal-range arguments bit-equal, {small.sum()} flushed, {nan.sum()} NaN")


def test_widen_is_exact(cuda_lib):
    rng = np.random.default_rng(8)
    _, _, xf, wf = _probe(cuda_lib, np.zeros(1), _floats(rng))
    nan = np.isnan(xf)
    sub = ~nan & (xf != 0) & (np.abs(xf) < np.finfo(np.float32).tiny)
    rest = ~nan & ~sub
    want = xf[rest].astype(np.float64)
    assert np.array_equal(want.view(np.uint64), wf[rest].view(np.uint64))
    assert np.all(wf[sub] == 0) and np.all(np.signbit(wf[sub]) == np.signbit(xf[sub]))
    assert np.all(np.isnan(wf[nan])) and np.all(np.signbit(wf[nan]) == np.signbit(xf[nan]))
    print(f"widen: {rest.sum()} bit-equal, {sub.sum()} subnormals flushed, {nan.sum()} NaN")
