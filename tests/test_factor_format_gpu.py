"""Device factor objects through nalgebra's serde JSON form: to_json, then
from_json, gives the same JSON and bit-identical solves; the JSON of an EXACT
factorization is the oracle's."""
import numpy as np
import pytest

import oracle as O
from nalgebra_gb300 import FLAG_EXACT, factor_format as F

pytestmark = pytest.mark.gpu


def test_mirror_round_trips(cuda):
    from nalgebra_gb300 import LU, Cholesky, ColPivQR, DeviceMatrix, FullPivLU

    rng = np.random.default_rng(9)
    n = 12
    a = rng.uniform(-100, 100, size=(n, n))
    b = rng.standard_normal((n, 2))
    for cls, make in ((LU, lambda m: m.lu(FLAG_EXACT)), (FullPivLU, lambda m: m.full_piv_lu(FLAG_EXACT)),
                      (ColPivQR, lambda m: m.col_piv_qr(FLAG_EXACT))):
        f = make(DeviceMatrix.from_numpy(a))
        s = f.to_json()
        g = cls.from_json(s, FLAG_EXACT)
        assert g.to_json() == s, cls.__name__
        x1 = f.solve(DeviceMatrix.from_numpy(b)).to_numpy()
        x2 = g.solve(DeviceMatrix.from_numpy(b)).to_numpy()
        assert np.array_equal(x1, x2), cls.__name__
    lu, ipiv = F.lu_from_json(DeviceMatrix.from_numpy(a).lu(FLAG_EXACT).to_json())
    ref, rpiv, _ = O.lu(a)
    assert np.array_equal(lu, ref) and np.array_equal(ipiv, rpiv)
    spd = a @ a.T + n * np.eye(n)
    ch = DeviceMatrix.from_numpy(spd).cholesky(flags=FLAG_EXACT)
    s = ch.to_json()
    g = Cholesky.from_json(s, FLAG_EXACT)
    assert g.to_json() == s
    assert np.array_equal(ch.solve(DeviceMatrix.from_numpy(b)).to_numpy(), g.solve(DeviceMatrix.from_numpy(b)).to_numpy())
