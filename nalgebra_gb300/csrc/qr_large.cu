// Householder QR of one matrix of any shape: nalgebra's QR::new
// (src/linalg/qr.rs:55-76, householder::clear_column_unchecked,
// householder.rs:61-85) for the matrices the shared-memory batched kernels
// (order <= 128) do not take, wide ones (m < n, the reference's
// qr_decompose_100x500 bench shape) included; and the solve from its factors:
// QR::solve_mut (qr.rs:204-256) for a square factor, the least-squares solve
// of nalgebra-lapack (qr_util.rs:167-239) for a tall one.
//
// Factor: one launch per Householder step.  Launch i applies reflector i
// (Reflection::reflect_with_sign with bias 0, reflection.rs:70-83; skipped
// where the column was zero, which is where diag[i] == 0) to the trailing
// columns i+1 .. n-1, one warp per column: a dot with the axis, then
// y <- factor * axis + sign * y.  The warp that owns column i+1 then turns it
// into the next axis (reflection_axis_mut, householder.rs:19-53) and writes
// diag[i+1], so the next launch finds it ready: min(m, n) + 1 launches.  Each
// reads and writes the trailing matrix once (the second read for the axpy
// comes from L1/L2), 16-24 bytes per two FP64 FMAs, near the balance point of
// GB300's FP64 pipe against HBM.  EXACT rounds every operation as Rust does,
// the dots in dotx's order: bit-identical to nalgebra's factors.
//
// Solve: Q^T B by one CTA per right-hand side, each thread owning fixed rows
// of its column in registers across all steps (so B needs no barrier; the dot
// takes one per step), then R (the factor's strict upper part with |diag| on
// the diagonal) copied to the workspace and solved by the large triangular
// solve (nacu_dtrsv), which stops at the zero |diag_i| nalgebra's backward
// substitution would stop at.
#include <algorithm>

#include "common.cuh"
#include "householder.cuh"

namespace nacu {
namespace {

constexpr int kQlThreads = 256;
constexpr int kQlWarps = kQlThreads / 32;
constexpr int kQtThreads = 512;
constexpr int kQtRows = 32;  // rows per thread of the Q^T B kernel
constexpr int kQtMaxM = kQtThreads * kQtRows;

// Warp dot, FMA form: four interleaved accumulators per lane, valid in every lane.
__device__ __forceinline__ double ql_dot_fma(int len, const double* __restrict__ x, const double* __restrict__ y,
                                             int lane) {
  double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
  int e = lane;
  for (; e + 96 < len; e += 128) {
    a0 = fma(x[e], y[e], a0);
    a1 = fma(x[e + 32], y[e + 32], a1);
    a2 = fma(x[e + 64], y[e + 64], a2);
    a3 = fma(x[e + 96], y[e + 96], a3);
  }
  for (; e < len; e += 32) a0 = fma(x[e], y[e], a0);
  return warp_sum((a0 + a1) + (a2 + a3));
}

template <bool EXACT>
__device__ __forceinline__ double ql_dot(int len, const double* x, const double* y, int lane) {
  if constexpr (EXACT) return cq_dot<true>(len, x, y, lane);
  else return ql_dot_fma(len, x, y, lane);
}

// reflection_axis_mut on x[0 .. len) by one warp: x becomes the unit axis
// (where the column is not zero) and *d_out the signed diagonal entry.
template <bool EXACT>
__device__ void ql_make_axis(int len, double* x, double* d_out, int lane) {
  const double x0 = x[0];
  const double sq = cq_add<EXACT>(0.0, ql_dot<EXACT>(len, x, x, lane));  // norm_squared (norm.rs:238-250)
  const double nrm = __dsqrt_rn(sq);
  double modulus, sign;
  cq_to_exp(x0, modulus, sign);
  const double signed_norm = cq_mul<EXACT>(sign, nrm);
  const double factor = EXACT ? __dmul_rn(__dadd_rn(sq, __dmul_rn(modulus, nrm)), 2.0) : fma(modulus, nrm, sq) * 2.0;
  const double x0n = cq_add<EXACT>(x0, signed_norm);
  __syncwarp();  // every lane has read x before it changes
  const bool nz = !is_zero_bits(factor);
  if (nz) {
    if constexpr (EXACT) {
      const double sf = __dsqrt_rn(factor);
      for (int r = lane; r < len; r += 32) x[r] = __ddiv_rn(r == 0 ? x0n : x[r], sf);  // unscale_mut
      __syncwarp();
      const double n2 = __dsqrt_rn(__dadd_rn(0.0, cq_dot<true>(len, x, x, lane)));  // normalize_mut
      __syncwarp();
      for (int r = lane; r < len; r += 32) x[r] = __ddiv_rn(x[r], n2);
    } else {
      // factor = 2 (sq + |x0| nrm) is the squared norm of the updated axis, so
      // one scale by rsqrt(factor) leaves a unit vector; nalgebra's second
      // normalisation only corrects rounding
      const double rs = rsqrt(factor);
      for (int r = lane; r < len; r += 32) x[r] = (r == 0 ? x0n : x[r]) * rs;
    }
  } else if (lane == 0) {
    x[0] = x0n;  // x[0] += signed_norm happens whether or not the column was zero
  }
  if (lane == 0) *d_out = nz ? -signed_norm : signed_norm;
}

// Step i of the factorization: reflector i (i >= 0) on columns i+1 .. i+ncols,
// and the axis of column i+1 when i+1 < min(m, n).
template <bool EXACT>
__global__ void __launch_bounds__(kQlThreads)
    qr_large_step_kernel(int m, int n, double* __restrict__ A, int64_t lda, double* __restrict__ diag, int i,
                         int ncols) {
  const int lane = threadIdx.x & 31;
  const int warp = blockIdx.x * kQlWarps + (threadIdx.x >> 5);
  const int nwarps = gridDim.x * kQlWarps;
  const int mn = min(m, n);
  bool reflect = false;
  double sign = 0.0, m_two = 0.0;
  const double* axis = nullptr;
  int len = 0;
  if (i >= 0) {
    const double d = diag[i];
    reflect = !is_zero_bits(d);  // diag[i] == 0 exactly where reflection_axis_mut found a zero column
    sign = cq_signum(d);
    m_two = cq_mul<EXACT>(sign, -2.0);
    axis = A + (int64_t)i * lda + i;
    len = m - i;
  }
  for (int c = warp; c < ncols; c += nwarps) {
    const int j = i + 1 + c;
    double* col = A + (int64_t)j * lda;
    if (reflect) {
      double* y = col + i;
      const double dot = ql_dot<EXACT>(len, axis, y, lane);
      const double factor = cq_mul<EXACT>(dot, m_two);  // (dot - bias) * (sign * -2), bias 0
      __syncwarp();
      for (int r = lane; r < len; r += 32) {
        const double sy = cq_mul<EXACT>(sign, y[r]);
        y[r] = EXACT ? __dadd_rn(__dmul_rn(factor, axis[r]), sy) : fma(factor, axis[r], sy);
      }
    }
    if (j == i + 1 && j < mn) {
      __syncwarp();
      ql_make_axis<EXACT>(m - j, col + j, diag + j, lane);
    }
  }
}

// Q^T B (QR::q_tr_mul, qr.rs:157-171): column blockIdx.x of B, every reflector
// in order (q_tr_mul applies them all, a zero column's too), each with the
// sign of its diag entry; FMA form.  Thread t owns rows t + k * kQtThreads;
// a warp skips the row groups that lie wholly above the current step.
__global__ void __launch_bounds__(kQtThreads)
    qr_large_qtmul_kernel(int m, int mn, const double* __restrict__ QR, int64_t lda, const double* __restrict__ diag,
                          double* __restrict__ B, int64_t ldb) {
  __shared__ double red[2][kQtThreads / 32];
  double* b = B + (int64_t)blockIdx.x * ldb;
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  const int kmax = (m + kQtThreads - 1) / kQtThreads;
  const int wlast = w * 32 + 31;  // the warp's last row in each group
  double v[kQtRows];
#pragma unroll
  for (int k = 0; k < kQtRows; ++k) {
    const int r = t + k * kQtThreads;
    v[k] = (k < kmax && r < m) ? b[r] : 0.0;
  }
  int phase = 0;
  for (int i = 0; i < mn; ++i) {
    const double sign = cq_signum(diag[i]);
    const double* axis = QR + (int64_t)i * lda;
    double part = 0.0;
#pragma unroll
    for (int k = 0; k < kQtRows; ++k) {
      if (k < kmax && wlast + k * kQtThreads >= i) {  // warp-uniform
        const int r = t + k * kQtThreads;
        if (r >= i && r < m) part = fma(axis[r], v[k], part);
      }
    }
    part = warp_sum(part);
    double* rb = red[phase];
    phase ^= 1;
    if (lane == 0) rb[w] = part;
    __syncthreads();
    double dot = 0.0;
#pragma unroll
    for (int q = 0; q < kQtThreads / 32; ++q) dot += rb[q];
    const double factor = dot * (sign * -2.0);
#pragma unroll
    for (int k = 0; k < kQtRows; ++k) {
      if (k < kmax && wlast + k * kQtThreads >= i) {
        const int r = t + k * kQtThreads;
        if (r >= i && r < m) v[k] = fma(factor, axis[r], sign * v[k]);
      }
    }
  }
#pragma unroll
  for (int k = 0; k < kQtRows; ++k) {
    const int r = t + k * kQtThreads;
    if (k < kmax && r < m) b[r] = v[k];
  }
}

// R (n x n, leading dimension n) from the factor: its strict upper part, |diag|
// on the diagonal; the lower part is not read by the upper solve.
__global__ void qr_large_r_kernel(int n, const double* __restrict__ QR, int64_t lda, const double* __restrict__ diag,
                                  double* __restrict__ R) {
  for (int c = blockIdx.x; c < n; c += gridDim.x) {
    for (int r = threadIdx.x; r <= c; r += blockDim.x)
      R[(int64_t)c * n + r] = r == c ? fabs(diag[c]) : QR[(int64_t)c * lda + r];
  }
}

inline size_t ql_align(size_t x) { return (x + 255) & ~(size_t)255; }

template <bool EXACT>
int qr_large_factor(int m, int n, double* A, int64_t lda, double* diag, cudaStream_t s) {
  const int mn = std::min(m, n);
  const int max_blocks = sm_count() * (2048 / kQlThreads);
  for (int i = -1; i < mn; ++i) {
    const int ncols = i < 0 ? 1 : n - 1 - i;  // step -1 only forms the first axis
    if (ncols <= 0) break;
    const int blocks = std::min((ncols + kQlWarps - 1) / kQlWarps, max_blocks);
    qr_large_step_kernel<EXACT><<<blocks, kQlThreads, 0, s>>>(m, n, A, lda, diag, i, ncols);
  }
  return check_launch("nacu_dqr");
}

}  // namespace
}  // namespace nacu

extern "C" {

int nacu_dqr(int m, int n, double* A, int64_t lda, double* diag, int flags, nacu_stream_t stream) {
  using namespace nacu;
  if (m < 0) return record_arg_error(-1, "dqr: m < 0");
  if (n < 0) return record_arg_error(-2, "dqr: n < 0");
  if (m == 0 || n == 0) return NACU_SUCCESS;
  if (!A) return record_arg_error(-3, "dqr: null A");
  if (lda < m) return record_arg_error(-4, "dqr: lda < m");
  if (!diag) return record_arg_error(-5, "dqr: null diag");
  const cudaStream_t s = (cudaStream_t)stream;
  return (flags & NACU_FLAG_EXACT) ? qr_large_factor<true>(m, n, A, lda, diag, s)
                                   : qr_large_factor<false>(m, n, A, lda, diag, s);
}

size_t nacu_qr_solve_workspace_bytes(int n) {
  if (n <= 0) return 0;
  return nacu::ql_align((size_t)n * n * sizeof(double)) + nacu_trsv_workspace_bytes(n);
}

int nacu_dqr_solve(int m, int n, int nrhs, const double* QR, int64_t lda, const double* diag, double* B, int64_t ldb,
                   int32_t* info, void* workspace, size_t workspace_bytes, int flags, nacu_stream_t stream) {
  using namespace nacu;
  if (m < 0 || m > kQtMaxM) return record_arg_error(-1, "dqr_solve: m out of range [0, 16384]");
  if (n < 0 || n > m) return record_arg_error(-2, "dqr_solve: n out of range [0, m]");
  if (nrhs < 0) return record_arg_error(-3, "dqr_solve: nrhs < 0");
  if (!info) return record_arg_error(-9, "dqr_solve: null info");
  if (flags & NACU_FLAG_EXACT) return record_arg_error(-12, "dqr_solve: FMA arithmetic only (no NACU_FLAG_EXACT)");
  const cudaStream_t s = (cudaStream_t)stream;
  if (n == 0 || nrhs == 0) {
    const cudaError_t e = cudaMemsetAsync(info, 0, sizeof(int32_t), s);
    return e == cudaSuccess ? NACU_SUCCESS : record_cuda_error(e, "nacu_dqr_solve");
  }
  if (!QR) return record_arg_error(-4, "dqr_solve: null QR");
  if (lda < m) return record_arg_error(-5, "dqr_solve: lda < m");
  if (!diag) return record_arg_error(-6, "dqr_solve: null diag");
  if (!B) return record_arg_error(-7, "dqr_solve: null B");
  if (ldb < m) return record_arg_error(-8, "dqr_solve: ldb < m");
  if (!workspace || workspace_bytes < nacu_qr_solve_workspace_bytes(n))
    return record_arg_error(-11, "dqr_solve: workspace too small");
  qr_large_qtmul_kernel<<<nrhs, kQtThreads, 0, s>>>(m, n, QR, lda, diag, B, ldb);
  double* R = static_cast<double*>(workspace);
  qr_large_r_kernel<<<std::min(n, sm_count() * 8), 128, 0, s>>>(n, QR, lda, diag, R);
  int rc = check_launch("nacu_dqr_solve");
  if (rc != NACU_SUCCESS) return rc;
  char* tw = static_cast<char*>(workspace) + ql_align((size_t)n * n * sizeof(double));
  return nacu_dtrsv(n, nrhs, 1, 0, 0, 0.0, R, n, B, ldb, info, tw, nacu_trsv_workspace_bytes(n), 0, stream);
}

}  // extern "C"
