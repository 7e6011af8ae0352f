"""Accuracy of the fast FP64 arithmetic of the performance kernels
(openmhd_gb300/csrc/omhd_fastmath.h): rcp_nr, rsqrt_nr and sqrt_nr are
refinements of the special-function unit's approximations that replace IEEE
division and square root inside every HLLD face and u2v of the FP64 stage
kernels.  Evaluated on the GPU through omhd_probe_fastmath over seeded
arguments and edge cases and compared with correctly rounded results:

* 1/x and sqrt(x): the device's IEEE division and square root (correctly
  rounded), which the probe computes beside the fast forms;
* 1/sqrt(x): the host's extended-precision 1/sqrt rounded to double.

Bound asserted: at most 1 ulp from the correctly rounded result, over the
arguments the solver uses (2^-60 .. 2^59, both signs for the reciprocal) and
over the whole domain of each function (rcp_nr: |x| in [2^-1022, 2^1022], whose
reciprocal is normal; rsqrt_nr, sqrt_nr: positive normal x).  Outside the
positive normal range rsqrt_nr and sqrt_nr take the IEEE operations, which is
checked bit for bit (0, -0, subnormals, +inf, negative numbers, NaN)."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _probe(lib, x: np.ndarray) -> np.ndarray:
    import torch

    xt = torch.from_numpy(np.ascontiguousarray(x, dtype=np.float64)).cuda()
    out = torch.empty(5 * xt.numel(), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    assert lib.omhd_probe_fastmath(C.c_void_p(xt.data_ptr()), xt.numel(), C.c_void_p(out.data_ptr())) == 0
    return out.cpu().numpy().reshape(5, -1)


def _ulps(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """Distance in units in the last place between doubles of the same sign."""
    assert np.all(np.signbit(a) == np.signbit(b)) and np.all(np.isfinite(a)) and np.all(np.isfinite(b))
    ia = np.abs(a).view(np.int64)
    ib = np.abs(b).view(np.int64)
    return np.abs(ia - ib)


def _rsqrt_ref(x: np.ndarray) -> np.ndarray:
    xl = x.astype(np.longdouble)
    return (np.longdouble(1) / np.sqrt(xl)).astype(np.float64)


def _log_uniform(rng, lo_exp, hi_exp, n):
    return np.exp2(rng.uniform(lo_exp, hi_exp, n))


def _special(lo_exp, hi_exp):
    """Powers of two, their neighbours and values next to 1 in [2^lo, 2^hi]."""
    p = np.exp2(np.arange(lo_exp, hi_exp + 1, dtype=np.float64))
    near = np.concatenate([np.nextafter(p, 0)[1:], np.nextafter(p, np.inf)[:-1]])
    one = np.array([1.0, np.nextafter(1.0, 2), np.nextafter(1.0, 0), 2.0 - 2**-52, 1.5, 3.0, 0.1, 1 / 3])
    return np.concatenate([p, near, one])


@pytest.mark.parametrize("domain", ["solver_range", "full_range"])
def test_fast_reciprocal_and_square_roots_within_one_ulp(cuda_lib, domain):
    rng = np.random.default_rng(2024 if domain == "solver_range" else 2025)
    if domain == "solver_range":
        lo, hi = -60, 59
    else:
        lo, hi = -1022, 1022
    x = np.concatenate([_log_uniform(rng, lo, hi, 1 << 20), _special(lo, hi)])
    x = x[(x >= 2.0**lo) & (x <= 2.0**hi)]
    r = _probe(cuda_lib, x)
    rcp_fast, rcp_ieee, rsq_fast, sq_fast, sq_ieee = r
    u_rcp = _ulps(rcp_fast, rcp_ieee)
    u_sq = _ulps(sq_fast, sq_ieee)
    u_rsq = _ulps(rsq_fast, _rsqrt_ref(x))
    print(f"{domain}: max ulp rcp_nr {u_rcp.max()}, sqrt_nr {u_sq.max()}, rsqrt_nr {u_rsq.max()}; "
          f"share not correctly rounded: rcp {np.mean(u_rcp > 0):.2e}, sqrt {np.mean(u_sq > 0):.2e}, "
          f"rsqrt {np.mean(u_rsq > 0):.2e}")
    assert u_rcp.max() <= 1 and u_sq.max() <= 1 and u_rsq.max() <= 1
    # the reciprocal of negative arguments (normal velocities, wave-speed
    # differences) mirrors the positive ones bit for bit
    rn = _probe(cuda_lib, -x)
    assert np.array_equal(rn[0], -rcp_fast) and np.array_equal(rn[1], -rcp_ieee)


def test_square_roots_outside_the_positive_normal_range_are_ieee(cuda_lib):
    tiny = np.array([5e-324, 1e-320, 2.2e-308, np.nextafter(2.0**-1022, 0)])
    x = np.concatenate([[0.0, -0.0, np.inf, -1.0, -2.5, -np.inf, np.nan], tiny, np.array([2.0**1023, 1.7e308])])
    r = _probe(cuda_lib, x)
    _, _, rsq_fast, sq_fast, sq_ieee = r
    with np.errstate(divide="ignore", invalid="ignore"):
        rsq_ieee = 1.0 / np.sqrt(x)
    special = ~((x >= 2.0**-1022) & np.isfinite(x))
    for got, want in ((sq_fast, sq_ieee), (rsq_fast, rsq_ieee)):
        g, w = got[special], want[special]
        assert np.array_equal(np.isnan(g), np.isnan(w))
        ok = ~np.isnan(w)
        assert np.array_equal(g[ok].view(np.int64), w[ok].view(np.int64)), (x[special][ok], g[ok], w[ok])
    # the largest normals are inside the fast range: within 1 ulp
    big = ~special
    assert _ulps(sq_fast[big], sq_ieee[big]).max() <= 1
    assert _ulps(rsq_fast[big], _rsqrt_ref(x[big])).max() <= 1
