"""GPU checks of the size-bucketed ragged Cholesky launch and its autotuner:
every tile gives results bit-identical to the oracle in the exact form (each
element still takes its updates in nalgebra's order whatever the panel width),
the bucketed path (no caller order) equals the single launch over a caller
order, batches that span all buckets and out-of-range orders are handled, and
the autotuner returns and installs a valid table."""
import ctypes as C

import numpy as np
import pytest

import oracle as O
from nalgebra_gb300 import FLAG_EXACT, _lib, tuning
from tests.conftest import EPS64
from tests.test_chol_gpu import _posv_ragged

pytestmark = pytest.mark.gpu


def _spd_batch(ns, nrhs, seed):
    rng = np.random.default_rng(seed)
    a_parts, b_parts = [], []
    for n in ns:
        bm = rng.standard_normal((n, n))
        a = bm @ bm.T + n * np.eye(n)
        a_parts.append(np.asfortranarray(a).ravel(order="F"))
        b_parts.append(rng.standard_normal(n * nrhs))
    return np.concatenate(a_parts), np.concatenate(b_parts)


def _set_all(tile):
    lib = _lib.load()
    arr = (C.c_int32 * 8)(*([tile] * 8))
    assert lib.nacu_ragged_set_tuning(arr, 8) == 0


@pytest.fixture
def keep_tuning(cuda):
    saved = tuning.current()
    yield
    arr = (C.c_int32 * 8)(*saved)
    _lib.load().nacu_ragged_set_tuning(arr, 8)


@pytest.mark.parametrize("tile", [0, 1, 2, 3])
def test_every_tile_exact_matches_oracle(cuda, keep_tuning, tile):
    ns = np.array([1, 5, 31, 32, 33, 64, 65, 97, 128, 129, 150, 193, 256, 257, 300], dtype=np.int32)
    a_flat, b_flat = _spd_batch(ns, 3, seed=tile)
    _set_all(tile)
    A, B, info, logdet, aoff, boff = _posv_ragged(cuda, ns, a_flat, b_flat, 3, FLAG_EXACT)
    Lo, Xo, info_o, logdet_o = O.posv_ragged(ns, aoff, a_flat, boff, b_flat, 3)
    assert np.array_equal(info, info_o) and np.all(info == 0)
    assert np.array_equal(A, Lo)
    assert np.array_equal(B, Xo)


def test_bucketed_equals_single_launch(cuda):
    rng = np.random.default_rng(4)
    ns = rng.integers(1, 400, size=300).astype(np.int32)
    a_flat, b_flat = _spd_batch(ns, 4, seed=9)
    order = np.argsort(-ns, kind="stable")
    r1 = _posv_ragged(cuda, ns, a_flat, b_flat, 4, FLAG_EXACT, order=order)
    r2 = _posv_ragged(cuda, ns, a_flat, b_flat, 4, FLAG_EXACT, order=None)
    for x, y in zip(r1[:4], r2[:4]):
        assert np.array_equal(x, y)


def test_bucketed_fma_form_accuracy_and_logdet(cuda):
    rng = np.random.default_rng(5)
    ns = rng.integers(8, 257, size=400).astype(np.int32)
    a_flat, b_flat = _spd_batch(ns, 4, seed=10)
    A, B, info, logdet, aoff, boff = _posv_ragged(cuda, ns, a_flat, b_flat, 4, 0)
    Lo, Xo, info_o, logdet_o = O.posv_ragged(ns, aoff, a_flat, boff, b_flat, 4)
    assert np.all(info == 0)
    assert np.allclose(logdet, logdet_o, rtol=1e-12, atol=0)
    for s in range(0, 400, 17):
        n = ns[s]
        a = a_flat[aoff[s]:aoff[s] + n * n].reshape(n, n).T
        x = B[boff[s]:boff[s] + 4 * n].reshape(4, n).T
        b = b_flat[boff[s]:boff[s] + 4 * n].reshape(4, n).T
        assert O.backward_error(a, x, b) <= n * EPS64


def test_not_spd_and_out_of_range_in_buckets(cuda):
    ns = np.array([40, 200, 3, 300], dtype=np.int32)
    a_flat, b_flat = _spd_batch(ns, 1, seed=2)
    aoff = np.concatenate([[0], np.cumsum(ns.astype(np.int64) ** 2)[:-1]])
    # make system 1 indefinite at column 7
    n = 200
    a1 = a_flat[aoff[1]:aoff[1] + n * n].reshape(n, n).T.copy()
    a1[7, 7] = -1e6
    a_flat[aoff[1]:aoff[1] + n * n] = np.asfortranarray(a1).ravel(order="F")
    A, B, info, logdet, _, _ = _posv_ragged(cuda, ns, a_flat, b_flat, 1, FLAG_EXACT)
    _, _, info_o, _ = O.posv_ragged(ns, aoff, a_flat, np.concatenate([[0], np.cumsum(ns)[:-1]]), b_flat, 1)
    assert np.array_equal(info, info_o) and info[1] == 8 and info[0] == 0 and info[3] == 0


def test_autotune_installs_valid_table(cuda, keep_tuning):
    res = tuning.autotune(per_bucket=48, nrhs=4, save=False)
    assert len(res["table"]) == 8 and all(0 <= t < 4 for t in res["table"])
    assert all(all(m > 0 for m in row) for row in res["ms"])
    assert tuning.current() == res["table"]
    for b, row in enumerate(res["ms"]):
        assert row[res["table"][b]] == min(row)
