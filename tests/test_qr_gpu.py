"""GPU parity of the batched Householder QR / least squares against the CPU
oracle (nalgebra's QR::new, q_tr_mul and the top-n back substitution),
through the C ABI.

Bar: diag signs identical to nalgebra's (its reflect_with_sign convention);
stored factors, Q^T b and x within 1e-11 relative of the oracle; the
reference's own least-squares criterion A^T A x = A^T b within 1e-5
(nalgebra-lapack/tests/linalg/qr.rs:46-61); rank deficiency reported."""
import numpy as np
import pytest

import oracle as O
from nalgebra_gb300 import DeviceBatch, _lib
from nalgebra_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _gels(cuda, w, with_rhs=True):
    torch = cuda
    ms, n = w["ms"], w["n"]
    count = ms.size
    d = lambda x: torch.from_numpy(np.ascontiguousarray(x)).cuda()
    A, B = d(w["a_flat"]), d(w["b_flat"])
    dms, daoff, dboff = d(ms), d(w["a_offsets"]), d(w["b_offsets"])
    X = torch.full((count * n,), np.nan, dtype=torch.float64, device="cuda")
    diag = torch.zeros(count * n, dtype=torch.float64, device="cuda")
    info = torch.full((count,), -7, dtype=torch.int32, device="cuda")
    ws = torch.zeros(_lib.load().nacu_qr_workspace_bytes(count), dtype=torch.uint8, device="cuda")
    order = d(np.argsort(-ms, kind="stable").astype(np.int32))
    _lib.call("nacu_dgels_batched", count, n, int(ms.max()), dms.data_ptr(), daoff.data_ptr(), A.data_ptr(),
              dboff.data_ptr() if with_rhs else 0, B.data_ptr() if with_rhs else 0, X.data_ptr() if with_rhs else 0,
              diag.data_ptr(), info.data_ptr(), order.data_ptr(), ws.data_ptr(), ws.numel(), 0,
              torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return (A.cpu().numpy(), B.cpu().numpy(), X.cpu().numpy().reshape(count, n),
            diag.cpu().numpy().reshape(count, n), info.cpu().numpy())


def test_ls_workload_slice_parity(cuda):
    """A 300-problem slice of the 8192 x (m in [128,512], n = 64) workload."""
    w = W.ragged_ls(300, 128, 512, 64, seed=0)
    A, B, X, diag, info = _gels(cuda, w)
    qr_o, diag_o, x_o, info_o = O.gels_batched(w["ms"], 64, w["a_offsets"], w["a_flat"], w["b_offsets"], w["b_flat"])
    assert np.all(info == 0) and np.all(info_o == 0)
    assert np.array_equal(np.signbit(diag), np.signbit(diag_o))
    assert np.allclose(diag, diag_o, rtol=1e-12, atol=0)
    assert np.allclose(X, x_o, rtol=1e-10, atol=1e-12)
    scale = np.abs(w["a_flat"]).max()
    assert np.allclose(A, qr_o, rtol=1e-10, atol=1e-11 * scale)  # axes and R, nalgebra layout
    assert np.allclose(B, w["b_flat"] * 0 + _qtb_oracle(w, qr_o, diag_o), rtol=1e-10, atol=1e-11)
    for s in range(0, 300, 37):
        m = int(w["ms"][s])
        a = w["a_flat"][w["a_offsets"][s]:w["a_offsets"][s] + m * 64].reshape(64, m).T
        b = w["b_flat"][w["b_offsets"][s]:w["b_offsets"][s] + m]
        lhs, rhs = a.T @ a @ X[s], a.T @ b
        assert np.allclose(lhs, rhs, atol=1e-5), s  # nalgebra-lapack/tests/linalg/qr.rs:46-61


def _qtb_oracle(w, qr_o, diag_o):
    out = np.empty_like(w["b_flat"])
    for s, m in enumerate(w["ms"]):
        m = int(m)
        qr = qr_o[w["a_offsets"][s]:w["a_offsets"][s] + m * w["n"]].reshape(w["n"], m).T
        b = w["b_flat"][w["b_offsets"][s]:w["b_offsets"][s] + m]
        out[w["b_offsets"][s]:w["b_offsets"][s] + m] = O.qr_q_tr_mul(qr, diag_o[s], b)
    return out


@pytest.mark.parametrize("n", [1, 3, 8, 13, 64, 100, 128])
def test_shapes(cuda, n):
    w = W.ragged_ls(40, n, 3 * n + 7, n, seed=n)
    A, B, X, diag, info = _gels(cuda, w)
    qr_o, diag_o, x_o, info_o = O.gels_batched(w["ms"], n, w["a_offsets"], w["a_flat"], w["b_offsets"], w["b_flat"])
    assert np.array_equal(info, info_o)
    assert np.array_equal(np.signbit(diag), np.signbit(diag_o))
    assert np.allclose(X, x_o, rtol=1e-9, atol=1e-10)
    assert np.allclose(A, qr_o, rtol=1e-9, atol=1e-10)


def test_factor_only_and_rank_deficiency(cuda):
    w = W.ragged_ls(6, 20, 30, 8, seed=4)
    # problem 2: a zero column -> rank deficient (info = 4); problem 4: all zero
    a = w["a_flat"].copy()
    m2 = int(w["ms"][2])
    a[w["a_offsets"][2] + 3 * m2:w["a_offsets"][2] + 4 * m2] = 0.0
    m4 = int(w["ms"][4])
    a[w["a_offsets"][4]:w["a_offsets"][4] + 8 * m4] = 0.0
    w["a_flat"] = a
    A, B, X, diag, info = _gels(cuda, w)
    qr_o, diag_o, x_o, info_o = O.gels_batched(w["ms"], 8, w["a_offsets"], a, w["b_offsets"], w["b_flat"])
    assert list(info) == list(info_o)
    assert info[2] == 4 and info[4] == 1 and info[0] == 0
    A2, _, _, diag2, info2 = _gels(cuda, w, with_rhs=False)
    assert np.array_equal(A2, A) and np.array_equal(diag2, diag)


def test_device_batch_qr_api(cuda):
    w = W.ragged_ls(10, 64, 100, 16, seed=9)
    mats = [w["a_flat"][o:o + m * 16].reshape(16, m).T for o, m in zip(w["a_offsets"], w["ms"])]
    rhs = [w["b_flat"][o:o + m].reshape(m, 1) for o, m in zip(w["b_offsets"], w["ms"])]
    x = DeviceBatch.from_numpy(mats).qr().solve(DeviceBatch.from_numpy(rhs))
    for s in range(10):
        ref = np.linalg.lstsq(mats[s], rhs[s][:, 0], rcond=None)[0]
        assert np.allclose(x[s], ref, rtol=1e-10, atol=1e-12)
