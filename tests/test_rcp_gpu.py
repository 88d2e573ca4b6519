"""The reciprocal the FMA forms use on their serial pivot paths (rcp_nr:
rcp.approx.ftz.f64 refined by two Newton-Raphson steps), held to IEEE 1/d as
numpy computes it: at most 1 ulp apart over random operands of every binade
in its fast range, and exactly 1/d (the division) outside it."""
import numpy as np
import pytest

from nalgebra_gb300 import _lib

pytestmark = pytest.mark.gpu


def _rcp(torch, d):
    D = torch.from_numpy(np.ascontiguousarray(d, dtype=np.float64)).cuda()
    out = torch.empty_like(D)
    _lib.call("nacu_test_rcp", d.size, D.data_ptr(), out.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return out.cpu().numpy()


def _ulps(a, b):
    ia = a.view(np.int64)
    ib = b.view(np.int64)
    return np.abs(ia - ib)


def test_within_one_ulp_of_ieee(cuda):
    rng = np.random.default_rng(5)
    n = 1 << 21
    mant = 1.0 + rng.random(n)
    d = np.ldexp(mant, rng.integers(-990, 990, n)) * np.where(rng.random(n) < 0.5, -1.0, 1.0)
    got = _rcp(cuda, d)
    ref = 1.0 / d
    assert _ulps(got, ref).max() <= 1
    assert np.mean(got == ref) > 0.999  # almost always the correctly rounded value


def test_edge_operands_take_the_division(cuda):
    d = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 1e-310, -1e-305, 2.0 ** -1001, 2.0 ** 1000, 1e308, 1.0, -3.0])
    got = _rcp(cuda, d)
    with np.errstate(divide="ignore", over="ignore"):
        ref = 1.0 / d
    assert np.array_equal(got[~np.isnan(ref)], ref[~np.isnan(ref)])
    assert np.isnan(got[np.isnan(ref)]).all()
