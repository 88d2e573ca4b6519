// Batched updates of Cholesky factors (n <= 128), the GPU form of nalgebra's
// Cholesky::rank_one_update, remove_column and insert_column
// (src/linalg/cholesky.rs:277-449): many factors, one warp each.
//
// The rank-one update is the column recurrence of xx_rank_one_update
// (cholesky.rs:410-449): per column j, lane 0 carries the scalar chain (the new
// diagonal, beta, the two axpy coefficients) and the lanes update the rows
// below j of x and of the factor's column j, 4 rows per lane.  remove_column
// copies the factor without row and column j and updates the bottom-right
// corner by the removed column (sigma = 1); insert_column copies it with an
// empty row and column j, solves the new row with the top-left corner (the
// lower solve of solve.rs:74-101), forms the centre and the new column (gemv's
// axcpy order, blas_uninit.rs:127-176) and downdates the bottom-right corner
// (sigma = -1).  EXACT (NACU_FLAG_EXACT) rounds every operation as Rust does
// (bit-identical to the oracle's restatement); the default form contracts to
// FMA.
#include <algorithm>

#include "common.cuh"

namespace nacu {
namespace {

constexpr int kUpdWarps = 8;
constexpr int kUpdMaxN = 128;

template <bool EXACT>
__device__ __forceinline__ double mul(double a, double b) { return EXACT ? __dmul_rn(a, b) : a * b; }
template <bool EXACT>
__device__ __forceinline__ double add(double a, double b) { return EXACT ? __dadd_rn(a, b) : a + b; }
template <bool EXACT>
__device__ __forceinline__ double dvd(double a, double b) { return EXACT ? __ddiv_rn(a, b) : a / b; }

// L (m x m, lower part, leading dimension ld) becomes the factor of
// L L^T + sigma x x^T; x (the warp's shared-memory slot) is overwritten.
template <bool EXACT>
__device__ void warp_rank_one(int m, double* L, int64_t ld, double* x, double sigma, int lane) {
  double beta = 1.0;  // lane 0 only
  for (int j = 0; j < m; ++j) {
    double a1 = 0.0, a2 = 0.0, b2 = 0.0;
    int upd = 0;
    if (lane == 0) {
      const double diag = L[j + j * ld];
      const double diag2 = mul<EXACT>(diag, diag);
      const double xj = x[j];
      const double sigma_xj2 = mul<EXACT>(sigma, mul<EXACT>(xj, xj));
      const double gamma = add<EXACT>(mul<EXACT>(diag2, beta), sigma_xj2);
      const double new_diag = __dsqrt_rn(add<EXACT>(diag2, dvd<EXACT>(sigma_xj2, beta)));
      L[j + j * ld] = new_diag;
      beta = add<EXACT>(beta, dvd<EXACT>(sigma_xj2, diag2));
      a1 = dvd<EXACT>(-xj, diag);
      a2 = mul<EXACT>(dvd<EXACT>(mul<EXACT>(new_diag, sigma), gamma), xj);
      b2 = dvd<EXACT>(new_diag, diag);
      upd = (gamma != 0.0);
    }
    a1 = __shfl_sync(0xffffffffu, a1, 0);
    a2 = __shfl_sync(0xffffffffu, a2, 0);
    b2 = __shfl_sync(0xffffffffu, b2, 0);
    upd = __shfl_sync(0xffffffffu, upd, 0);
    double* col = L + (size_t)j * ld;
    for (int r = j + 1 + lane; r < m; r += 32) {
      const double lr = col[r];
      // x[j+1..] += a1 * L[j+1.., j]; then L[j+1.., j] = a2 * x[j+1..] + b2 * L[j+1.., j]
      const double xr = EXACT ? __dadd_rn(__dmul_rn(a1, lr), x[r]) : fma(a1, lr, x[r]);
      x[r] = xr;
      if (upd) col[r] = EXACT ? __dadd_rn(__dmul_rn(a2, xr), __dmul_rn(b2, lr)) : fma(a2, xr, b2 * lr);
    }
    __syncwarp();
  }
}

template <bool EXACT>
__global__ void __launch_bounds__(kUpdWarps * 32) rank1_kernel(int n, double* L, int64_t strideL, const double* X,
                                                              int64_t strideX, const double* sigma, int batch) {
  __shared__ double xs_all[kUpdWarps][kUpdMaxN];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int s = blockIdx.x * kUpdWarps + warp;
  if (s >= batch) return;
  double* xs = xs_all[warp];
  for (int r = lane; r < n; r += 32) xs[r] = X[(size_t)s * strideX + r];  // nalgebra updates a clone of x
  __syncwarp();
  warp_rank_one<EXACT>(n, L + (size_t)s * strideL, n, xs, sigma[s], lane);
}

template <bool EXACT>
__global__ void __launch_bounds__(kUpdWarps * 32) remove_kernel(int n, const double* L, int64_t strideL, int j,
                                                               double* Lout, int64_t strideOut, int batch) {
  __shared__ double xs_all[kUpdWarps][kUpdMaxN];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int s = blockIdx.x * kUpdWarps + warp;
  if (s >= batch) return;
  const double* l = L + (size_t)s * strideL;
  double* out = Lout + (size_t)s * strideOut;
  const int m = n - 1;
  for (int e = lane; e < m * m; e += 32) {
    const int c = e / m, r = e - c * m;
    out[e] = l[(r < j ? r : r + 1) + (size_t)(c < j ? c : c + 1) * n];
  }
  double* xs = xs_all[warp];
  for (int r = j + 1 + lane; r < n; r += 32) xs[r - j - 1] = l[r + (size_t)j * n];  // the removed column's tail
  __syncwarp();
  warp_rank_one<EXACT>(m - j, out + j + (size_t)j * m, m, xs, 1.0, lane);
}

template <bool EXACT>
__global__ void __launch_bounds__(kUpdWarps * 32) insert_kernel(int n, const double* L, int64_t strideL, int j,
                                                               const double* Col, int64_t strideCol, double* Lout,
                                                               int64_t strideOut, int32_t* info, int batch) {
  __shared__ double row_all[kUpdWarps][kUpdMaxN];
  __shared__ double ncol_all[kUpdWarps][kUpdMaxN];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int s = blockIdx.x * kUpdWarps + warp;
  if (s >= batch) return;
  const double* l = L + (size_t)s * strideL;
  const double* col = Col + (size_t)s * strideCol;
  double* out = Lout + (size_t)s * strideOut;
  const int m = n + 1, len = n - j;
  for (int e = lane; e < m * m; e += 32) {
    const int c = e / m, r = e - c * m;
    out[e] = (r == j || c == j) ? 0.0 : l[(r < j ? r : r - 1) + (size_t)(c < j ? c : c - 1) * n];
  }
  double* row = row_all[warp];
  double* ncol = ncol_all[warp];
  for (int r = lane; r < j; r += 32) row[r] = col[r];
  for (int r = lane; r < len; r += 32) ncol[r] = col[j + 1 + r];
  __syncwarp();
  // row j: the lower solve with the top-left corner (solve.rs:74-101)
  int fail = 0;
  for (int i = 0; i < j; ++i) {
    const double d = l[i + (size_t)i * n];
    if (d == 0.0) {
      fail = 1;
      break;
    }
    double coeff = 0.0;
    if (lane == 0) {
      coeff = dvd<EXACT>(row[i], d);
      row[i] = coeff;
    }
    coeff = __shfl_sync(0xffffffffu, coeff, 0);
    for (int r = i + 1 + lane; r < j; r += 32)
      row[r] = EXACT ? __dadd_rn(__dmul_rn(-coeff, l[r + (size_t)i * n]), row[r]) : fma(-coeff, l[r + (size_t)i * n], row[r]);
    __syncwarp();
  }
  if (fail) {
    if (lane == 0 && info) info[s] = 1;  // nalgebra's assertion
    return;
  }
  for (int k = lane; k < j; k += 32) out[j + (size_t)k * m] = row[k];
  // centre: sqrt(col_j - |row|^2), |row|^2 by dotx (blas.rs:96-165)
  double nrm2;
  if constexpr (EXACT) {
    const int nb = j >> 3;
    double acc = 0.0;
    if (lane < 8)
      for (int b = 0; b < nb; ++b) acc = __dadd_rn(acc, __dmul_rn(row[8 * b + lane], row[8 * b + lane]));
    const double pair = __dadd_rn(acc, __shfl_down_sync(0xffffffffu, acc, 4));
    double res = 0.0;
#pragma unroll
    for (int q = 0; q < 4; ++q) res = __dadd_rn(res, __shfl_sync(0xffffffffu, pair, q));
    for (int e = 8 * nb; e < j; ++e) res = __dadd_rn(res, __dmul_rn(row[e], row[e]));
    nrm2 = res;
  } else {
    double part = 0.0;
    for (int e = lane; e < j; e += 32) part = fma(row[e], row[e], part);
    nrm2 = warp_sum(part);
  }
  const double center = __dsqrt_rn(add<EXACT>(col[j], -nrm2));
  if (lane == 0) out[j + (size_t)j * m] = center;
  // new column: gemv(alpha = -1/centre, bottom-left L[j.., ..j], row, beta = 1/centre)
  const double alpha = dvd<EXACT>(-1.0, center), beta = dvd<EXACT>(1.0, center);
  if (j == 0) {
    for (int r = lane; r < len; r += 32) ncol[r] = mul<EXACT>(ncol[r], beta);
  } else {
    for (int k = 0; k < j; ++k) {
      const double* lc = l + j + (size_t)k * n;
      const double val = row[k];
      const double b = (k == 0) ? beta : 1.0;
      for (int r = lane; r < len; r += 32)
        ncol[r] = EXACT ? __dadd_rn(__dmul_rn(__dmul_rn(alpha, lc[r]), val), __dmul_rn(b, ncol[r]))
                        : fma(alpha * lc[r], val, b * ncol[r]);
    }
  }
  __syncwarp();
  for (int r = lane; r < len; r += 32) out[j + 1 + r + (size_t)j * m] = ncol[r];
  __syncwarp();
  warp_rank_one<EXACT>(len, out + (j + 1) + (size_t)(j + 1) * m, m, ncol, -1.0, lane);
  if (lane == 0 && info) info[s] = 0;
}

}  // namespace
}  // namespace nacu

using namespace nacu;

extern "C" {

int nacu_dchol_rank1_update_batched(int n, double* L, int64_t strideL, const double* X, int64_t strideX,
                                    const double* sigma, int batch, int flags, nacu_stream_t stream) {
  if (n < 0 || n > kUpdMaxN) return record_arg_error(-1, "chol rank1 update: n out of range [0, 128]");
  if (batch < 0) return record_arg_error(-7, "chol rank1 update: negative batch");
  if (batch == 0 || n == 0) return NACU_SUCCESS;
  if (!L || !X || !sigma) return record_arg_error(-2, "chol rank1 update: null L, X or sigma");
  if (strideL < (int64_t)n * n || strideX < n) return record_arg_error(-3, "chol rank1 update: stride too small");
  const int grid = (batch + kUpdWarps - 1) / kUpdWarps;
  if (flags & NACU_FLAG_EXACT)
    rank1_kernel<true><<<grid, kUpdWarps * 32, 0, (cudaStream_t)stream>>>(n, L, strideL, X, strideX, sigma, batch);
  else
    rank1_kernel<false><<<grid, kUpdWarps * 32, 0, (cudaStream_t)stream>>>(n, L, strideL, X, strideX, sigma, batch);
  return check_launch("nacu_dchol_rank1_update_batched");
}

int nacu_dchol_remove_column_batched(int n, const double* L, int64_t strideL, int j, double* Lout, int64_t strideOut,
                                     int batch, int flags, nacu_stream_t stream) {
  if (n < 1 || n > kUpdMaxN) return record_arg_error(-1, "chol remove column: n out of range [1, 128]");
  if (j < 0 || j >= n) return record_arg_error(-4, "chol remove column: j out of range [0, n)");
  if (batch < 0) return record_arg_error(-8, "chol remove column: negative batch");
  if (batch == 0) return NACU_SUCCESS;
  if (!L || (n > 1 && !Lout)) return record_arg_error(-2, "chol remove column: null L or Lout");
  if (strideL < (int64_t)n * n || strideOut < (int64_t)(n - 1) * (n - 1))
    return record_arg_error(-3, "chol remove column: stride too small");
  if (n == 1) return NACU_SUCCESS;
  const int grid = (batch + kUpdWarps - 1) / kUpdWarps;
  if (flags & NACU_FLAG_EXACT)
    remove_kernel<true><<<grid, kUpdWarps * 32, 0, (cudaStream_t)stream>>>(n, L, strideL, j, Lout, strideOut, batch);
  else
    remove_kernel<false><<<grid, kUpdWarps * 32, 0, (cudaStream_t)stream>>>(n, L, strideL, j, Lout, strideOut, batch);
  return check_launch("nacu_dchol_remove_column_batched");
}

int nacu_dchol_insert_column_batched(int n, const double* L, int64_t strideL, int j, const double* col,
                                     int64_t strideCol, double* Lout, int64_t strideOut, int32_t* info, int batch,
                                     int flags, nacu_stream_t stream) {
  if (n < 0 || n > kUpdMaxN - 1) return record_arg_error(-1, "chol insert column: n out of range [0, 127]");
  if (j < 0 || j > n) return record_arg_error(-4, "chol insert column: j out of range [0, n]");
  if (batch < 0) return record_arg_error(-10, "chol insert column: negative batch");
  if (batch == 0) return NACU_SUCCESS;
  if ((n > 0 && !L) || !col || !Lout) return record_arg_error(-2, "chol insert column: null L, col or Lout");
  if (strideL < (int64_t)n * n || strideCol < n + 1 || strideOut < (int64_t)(n + 1) * (n + 1))
    return record_arg_error(-3, "chol insert column: stride too small");
  const int grid = (batch + kUpdWarps - 1) / kUpdWarps;
  if (flags & NACU_FLAG_EXACT)
    insert_kernel<true><<<grid, kUpdWarps * 32, 0, (cudaStream_t)stream>>>(n, L, strideL, j, col, strideCol, Lout,
                                                                         strideOut, info, batch);
  else
    insert_kernel<false><<<grid, kUpdWarps * 32, 0, (cudaStream_t)stream>>>(n, L, strideL, j, col, strideCol, Lout,
                                                                          strideOut, info, batch);
  return check_launch("nacu_dchol_insert_column_batched");
}

}  // extern "C"
