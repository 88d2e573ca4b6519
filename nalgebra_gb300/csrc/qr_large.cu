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
// columns i+1 .. n-1: a dot with the axis, then y <- factor * axis + sign * y.
// The block that owns column i+1 then turns it into the next axis
// (reflection_axis_mut, householder.rs:19-53) and writes diag[i+1], so the
// next launch finds it ready: min(m, n) + 1 launches.  Each reads and writes
// the trailing matrix once (the axpy's second read comes from L1/L2), 16-24
// bytes per two FP64 FMAs, near the balance point of GB300's FP64 pipe against
// HBM.  The FMA form gives each column a CTA of 128 threads (a thread owns
// rows t, t + 128, ...; one barrier per block-wide dot) and issues two FP64
// instructions per element: the dot's FMA and the axpy's, the +-1 sign folded
// into the FMA's operand (a multiply by it was a third).  Each warp-wide FP64
// instruction holds an SM sub-partition's FP64 unit for about 64 cycles, so
// the per-column reductions are kept short.  EXACT rounds every operation as
// Rust does, the dots in dotx's order (eight sequential accumulators), so it
// keeps one warp per column: bit-identical to nalgebra's factors.
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
constexpr int kQcThreads = 128;  // FMA form: one CTA per column
constexpr int kQcWarps = kQcThreads / 32;
constexpr int kQtThreads = 1024;
constexpr int kQtRows = 16;  // rows per thread of the Q^T B kernel
constexpr int kQtMaxM = kQtThreads * kQtRows;

// reflection_axis_mut on x[0 .. len) by one warp, EXACT form (every rounding
// as Rust's, dots in dotx's order): x becomes the unit axis (where the column
// is not zero) and *d_out the signed diagonal entry.
__device__ void ql_make_axis_exact(int len, double* x, double* d_out, int lane) {
  const double x0 = x[0];
  const double sq = __dadd_rn(0.0, cq_dot<true>(len, x, x, lane));  // norm_squared (norm.rs:238-250)
  const double nrm = __dsqrt_rn(sq);
  double modulus, sign;
  cq_to_exp(x0, modulus, sign);
  const double signed_norm = __dmul_rn(sign, nrm);
  const double factor = __dmul_rn(__dadd_rn(sq, __dmul_rn(modulus, nrm)), 2.0);
  const double x0n = __dadd_rn(x0, signed_norm);
  __syncwarp();  // every lane has read x before it changes
  const bool nz = !is_zero_bits(factor);
  if (nz) {
    const double sf = __dsqrt_rn(factor);
    for (int r = lane; r < len; r += 32) x[r] = __ddiv_rn(r == 0 ? x0n : x[r], sf);  // unscale_mut
    __syncwarp();
    const double n2 = __dsqrt_rn(__dadd_rn(0.0, cq_dot<true>(len, x, x, lane)));  // normalize_mut
    __syncwarp();
    for (int r = lane; r < len; r += 32) x[r] = __ddiv_rn(x[r], n2);
  } else if (lane == 0) {
    x[0] = x0n;  // x[0] += signed_norm happens whether or not the column was zero
  }
  if (lane == 0) *d_out = nz ? -signed_norm : signed_norm;
}

// Step i of the EXACT factorization: reflector i (i >= 0) on columns
// i+1 .. i+ncols, one warp per column, and the axis of column i+1 when
// i+1 < min(m, n).
__global__ void __launch_bounds__(kQlThreads)
    qr_large_step_exact_kernel(int m, int n, double* __restrict__ A, int64_t lda, double* __restrict__ diag, int i,
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
    m_two = __dmul_rn(sign, -2.0);
    axis = A + (int64_t)i * lda + i;
    len = m - i;
  }
  for (int c = warp; c < ncols; c += nwarps) {
    const int j = i + 1 + c;
    double* col = A + (int64_t)j * lda;
    if (reflect) {
      double* y = col + i;
      const double factor = __dmul_rn(cq_dot<true>(len, axis, y, lane), m_two);  // (dot - bias) * (sign * -2)
      __syncwarp();
      for (int r = lane; r < len; r += 32) y[r] = __dadd_rn(__dmul_rn(factor, axis[r]), __dmul_rn(sign, y[r]));
    }
    if (j == i + 1 && j < mn) {
      __syncwarp();
      ql_make_axis_exact(m - j, col + j, diag + j, lane);
    }
  }
}

// Block-wide sum for the FMA form, valid in every thread.  red holds two
// rounds of per-warp partials; consecutive calls alternate them, so one
// barrier per call suffices (a round is rewritten only two calls later, after
// every thread has passed the barrier in between).
__device__ __forceinline__ double qc_block_sum(double v, double (*red)[kQcWarps], int& phase) {
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  double* rb = red[phase];
  phase ^= 1;
  if (lane == 0) rb[w] = v;
  __syncthreads();
  double s = lane < kQcWarps ? rb[lane] : 0.0;
#pragma unroll
  for (int off = kQcWarps / 2; off >= 1; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
  return __shfl_sync(0xffffffffu, s, 0);
}

// sum_r x[r] y[r] over this thread's rows t, t + kQcThreads, ... < len: two
// accumulators, four loads in flight.  FP64 instructions are the scarce
// resource here (each warp-wide one holds an SM sub-partition's FP64 unit for
// 64 cycles), so the per-column reduction is kept short: 128 threads per
// column, one combine, warp_sum, a two-level block sum.
__device__ __forceinline__ double qc_dot_part(int len, const double* __restrict__ x, const double* __restrict__ y) {
  double a0 = 0.0, a1 = 0.0;
  int r = threadIdx.x;
  for (; r + 3 * kQcThreads < len; r += 4 * kQcThreads) {
    const double x0 = x[r], x1 = x[r + kQcThreads], x2 = x[r + 2 * kQcThreads], x3 = x[r + 3 * kQcThreads];
    const double y0 = y[r], y1 = y[r + kQcThreads], y2 = y[r + 2 * kQcThreads], y3 = y[r + 3 * kQcThreads];
    a0 = fma(x0, y0, a0);
    a1 = fma(x1, y1, a1);
    a0 = fma(x2, y2, a0);
    a1 = fma(x3, y3, a1);
  }
  for (; r < len; r += kQcThreads) a0 = fma(x[r], y[r], a0);
  return a0 + a1;
}

// y <- factor * v + s * y on this thread's rows, s = +-1 folded into the FMA's
// operand sign (no FP64 multiply); s NaN only comes with a NaN factor.
template <bool NEG>
__device__ __forceinline__ void qc_axpy(int len, double factor, const double* __restrict__ v, double* __restrict__ y) {
  int r = threadIdx.x;
  for (; r + 3 * kQcThreads < len; r += 4 * kQcThreads) {
    const double y0 = y[r], y1 = y[r + kQcThreads], y2 = y[r + 2 * kQcThreads], y3 = y[r + 3 * kQcThreads];
    const double v0 = v[r], v1 = v[r + kQcThreads], v2 = v[r + 2 * kQcThreads], v3 = v[r + 3 * kQcThreads];
    y[r] = fma(factor, v0, NEG ? -y0 : y0);
    y[r + kQcThreads] = fma(factor, v1, NEG ? -y1 : y1);
    y[r + 2 * kQcThreads] = fma(factor, v2, NEG ? -y2 : y2);
    y[r + 3 * kQcThreads] = fma(factor, v3, NEG ? -y3 : y3);
  }
  for (; r < len; r += kQcThreads) y[r] = fma(factor, v[r], NEG ? -y[r] : y[r]);
}

// reflection_axis_mut on x[0 .. len) by one CTA, FMA form (one scale by
// rsqrt(factor): factor = 2 (sq + |x0| nrm) is the squared norm of the
// updated axis, so nalgebra's second normalisation only corrects rounding).
__device__ void qc_make_axis(int len, double* x, double* d_out, double (*red)[kQcWarps], int& phase) {
  const int t = threadIdx.x;
  const double x0 = x[0];
  const double sq = qc_block_sum(qc_dot_part(len, x, x), red, phase);  // its barrier: every read of x is done
  const double nrm = __dsqrt_rn(sq);
  double modulus, sign;
  cq_to_exp(x0, modulus, sign);
  const double signed_norm = sign * nrm;
  const double factor = fma(modulus, nrm, sq) * 2.0;
  const double x0n = x0 + signed_norm;
  const bool nz = !is_zero_bits(factor);
  if (nz) {
    const double rs = rsqrt(factor);
    for (int r = t; r < len; r += kQcThreads) x[r] = (r == 0 ? x0n : x[r]) * rs;
  } else if (t == 0) {
    x[0] = x0n;
  }
  if (t == 0) *d_out = nz ? -signed_norm : signed_norm;
}

// Step i of the FMA factorization: reflector i (i >= 0) on columns
// i+1 .. i+ncols, one CTA per column, and the axis of column i+1 when
// i+1 < min(m, n).  Every branch is uniform over the CTA.
__global__ void __launch_bounds__(kQcThreads)
    qr_large_step_cta_kernel(int m, int n, double* __restrict__ A, int64_t lda, double* __restrict__ diag, int i,
                             int ncols) {
  __shared__ double red[2][kQcWarps];
  int phase = 0;
  const int mn = min(m, n);
  bool reflect = false;
  double sign = 0.0, m_two = 0.0;
  const double* axis = nullptr;
  int len = 0;
  if (i >= 0) {
    const double d = diag[i];
    reflect = !is_zero_bits(d);
    sign = cq_signum(d);
    m_two = sign * -2.0;
    axis = A + (int64_t)i * lda + i;
    len = m - i;
  }
  for (int c = blockIdx.x; c < ncols; c += gridDim.x) {
    const int j = i + 1 + c;
    double* col = A + (int64_t)j * lda;
    if (reflect) {
      double* y = col + i;
      const double factor = qc_block_sum(qc_dot_part(len, axis, y), red, phase) * m_two;
      // each thread updates the rows it read: no barrier between the dot and the axpy
      if (sign < 0.0) qc_axpy<true>(len, factor, axis, y);
      else qc_axpy<false>(len, factor, axis, y);
    }
    if (j == i + 1 && j < mn) {
      __syncthreads();  // the axis reads rows other threads just wrote
      qc_make_axis(m - j, col + j, diag + j, red, phase);
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
    // the warps' partials summed by a shuffle tree in every warp (four FP64
    // adds per warp instead of sixteen per thread)
    double s = lane < kQtThreads / 32 ? rb[lane] : 0.0;
#pragma unroll
    for (int off = kQtThreads / 64; off >= 1; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
    const double factor = __shfl_sync(0xffffffffu, s, 0) * (sign * -2.0);
    // sign * v as a flip of the sign bit on the integer pipe (sign = +-1; a NaN
    // sign comes with a NaN factor)
    const unsigned flip = sign < 0.0 ? 0x80000000u : 0u;
#pragma unroll
    for (int k = 0; k < kQtRows; ++k) {
      if (k < kmax && wlast + k * kQtThreads >= i) {
        const int r = t + k * kQtThreads;
        if (r >= i && r < m) {
          const double sv = __hiloint2double(__double2hiint(v[k]) ^ (int)flip, __double2loint(v[k]));
          v[k] = fma(factor, axis[r], sv);
        }
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

int qr_large_factor(bool exact, int m, int n, double* A, int64_t lda, double* diag, cudaStream_t s) {
  const int mn = std::min(m, n);
  const int max_blocks = sm_count() * (2048 / kQlThreads);
  for (int i = -1; i < mn; ++i) {
    const int ncols = i < 0 ? 1 : n - 1 - i;  // step -1 only forms the first axis
    if (ncols <= 0) break;
    if (exact) {
      const int blocks = std::min((ncols + kQlWarps - 1) / kQlWarps, max_blocks);
      qr_large_step_exact_kernel<<<blocks, kQlThreads, 0, s>>>(m, n, A, lda, diag, i, ncols);
    } else {
      qr_large_step_cta_kernel<<<std::min(ncols, max_blocks), kQcThreads, 0, s>>>(m, n, A, lda, diag, i, ncols);
    }
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
  return qr_large_factor((flags & NACU_FLAG_EXACT) != 0, m, n, A, lda, diag, s);
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
