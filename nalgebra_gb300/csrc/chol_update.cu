// Batched updates of Cholesky factors (n <= 128), the GPU form of nalgebra's
// Cholesky::rank_one_update, remove_column and insert_column
// (src/linalg/cholesky.rs:277-449): many factors, a group of G lanes each.
//
// The rank-one update is the column recurrence of xx_rank_one_update
// (cholesky.rs:410-449): per column j, the group's first lane carries the
// scalar chain (the new diagonal, beta, the two axpy coefficients) and the G
// lanes update the rows below j of x and of the factor's column j.
// remove_column copies the factor without row and column j and updates the
// bottom-right corner by the removed column (sigma = 1); insert_column copies
// it with an empty row and column j, solves the new row with the top-left
// corner (the lower solve of solve.rs:74-101), forms the centre and the new
// column (gemv's axcpy order, blas_uninit.rs:127-176) and downdates the
// bottom-right corner (sigma = -1).  EXACT (NACU_FLAG_EXACT) rounds every
// operation as Rust does (bit-identical to the oracle's restatement); the
// default form contracts to FMA.
//
// Why groups: the scalar chain is serial per factor (a square root and
// divisions, each on beta from the previous column), and on this part an FP64
// instruction costs the same pipe time whether one lane runs it or 32.  With
// a warp per factor the chain held most of the FP64 pipe; with G lanes per
// factor one chain instruction serves 32/G factors, while the rows' updates
// cost the same per factor and a group's loads still fill whole 32-byte
// sectors.  Measured on 4096 factors of order 128 (ms, G = 32 / 8 / 4 / 2):
// rank_one_update 1.22 / 0.73 / 1.20 / 1.63, remove_column 0.97 / 1.18 / 1.87 /
// 2.98, insert_column 1.18 / 1.57 / 2.82 / 5.52 (fewer warps hide less of the
// chain's latency and of the copies').  So rank_one_update runs G = 8 from
// kGroupMinBatch factors up and G = 32 below; remove_column and insert_column
// run G = 32.
#include <algorithm>

#include "common.cuh"

namespace nacu {
namespace {

constexpr int kUpdMaxN = 128;
constexpr int kFacPerCta = 16;  // factors per CTA: 16 G threads, 32 KB of vectors
constexpr int kGroupSmall = 8;
constexpr int kGroupMinBatch = 1024;
constexpr unsigned kFull = 0xffffffffu;

template <bool EXACT>
__device__ __forceinline__ double mul(double a, double b) { return EXACT ? __dmul_rn(a, b) : a * b; }
template <bool EXACT>
__device__ __forceinline__ double add(double a, double b) { return EXACT ? __dadd_rn(a, b) : a + b; }
template <bool EXACT>
__device__ __forceinline__ double dvd(double a, double b) { return EXACT ? __ddiv_rn(a, b) : a / b; }

__device__ __forceinline__ void prefetch_l2(const double* p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }

// Called by every lane of the warp (the loop bounds are the same for all its
// groups).  If active, the group's factor L (m x m, lower part, leading
// dimension ld) becomes the factor of L L^T + sigma x x^T; x (the group's
// shared-memory slot) is overwritten; rd (another slot) holds 1 / L_jj in the
// FMA form.  gl: the lane's index in its group.
template <bool EXACT, int G>
__device__ void group_rank_one(int m, double* L, int64_t ld, double* x, double* rd, double sigma, int gl,
                               bool active) {
  if constexpr (!EXACT) {
    // the reciprocals of the diagonal (unchanged until step j) G at a time;
    // gamma = L_jj^2 beta_{j+1} then turns the chain's remaining divisions
    // into one reciprocal of beta_{j+1}
    if (active)
      for (int j = gl; j < m; j += G) rd[j] = 1.0 / L[j + (size_t)j * ld];
    __syncwarp();
  }
  double beta = 1.0, ib = 1.0;  // the group's first lane: beta_j and 1 / beta_j
  for (int j = 0; j < m; ++j) {
    double* col = L + (size_t)j * ld;
    double a1 = 0.0, a2 = 0.0, b2 = 0.0;
    int upd = 0;
    if (active) {
      for (int r = j + 1 + 16 * gl; r < m; r += 16 * G) prefetch_l2(col + ld + r);  // column j+1, a line per lane
      if (gl == 0) {
        const double diag = col[j];
        const double xj = x[j];
        if constexpr (EXACT) {
          const double diag2 = mul<EXACT>(diag, diag);
          const double sigma_xj2 = mul<EXACT>(sigma, mul<EXACT>(xj, xj));
          const double gamma = add<EXACT>(mul<EXACT>(diag2, beta), sigma_xj2);
          const double new_diag = __dsqrt_rn(add<EXACT>(diag2, dvd<EXACT>(sigma_xj2, beta)));
          col[j] = new_diag;
          beta = add<EXACT>(beta, dvd<EXACT>(sigma_xj2, diag2));
          a1 = dvd<EXACT>(-xj, diag);
          a2 = mul<EXACT>(dvd<EXACT>(mul<EXACT>(new_diag, sigma), gamma), xj);
          b2 = dvd<EXACT>(new_diag, diag);
          upd = !is_zero_bits(gamma);
        } else {
          const double r = rd[j], r2 = r * r;
          const double sx = sigma * xj * xj;
          const double new_diag = sqrt(fma(sx, ib, diag * diag));
          const double beta1 = fma(sx, r2, beta);
          const double ib1 = rcp_nr(beta1);  // on the column chain: the short Newton form
          col[j] = new_diag;
          a1 = -xj * r;
          a2 = new_diag * sigma * xj * r2 * ib1;
          b2 = new_diag * r;
          upd = !is_zero_bits(beta1);
          beta = beta1;
          ib = ib1;
        }
      }
    }
    a1 = __shfl_sync(kFull, a1, 0, G);
    a2 = __shfl_sync(kFull, a2, 0, G);
    b2 = __shfl_sync(kFull, b2, 0, G);
    upd = __shfl_sync(kFull, upd, 0, G);
    if (active) {
      for (int r = j + 1 + gl; r < m; r += G) {
        const double lr = col[r];
        // x[j+1..] += a1 * L[j+1.., j]; then L[j+1.., j] = a2 * x[j+1..] + b2 * L[j+1.., j]
        const double xr = EXACT ? __dadd_rn(__dmul_rn(a1, lr), x[r]) : fma(a1, lr, x[r]);
        x[r] = xr;
        if (upd) col[r] = EXACT ? __dadd_rn(__dmul_rn(a2, xr), __dmul_rn(b2, lr)) : fma(a2, xr, b2 * lr);
      }
    }
    __syncwarp();
  }
}

// The first factor of this warp; a warp whose first group has no factor has
// none at all (its factors are consecutive), so it leaves at once.
template <int G>
__device__ __forceinline__ bool warp_idle(int batch) {
  return blockIdx.x * kFacPerCta + (int)(threadIdx.x >> 5) * (32 / G) >= batch;
}

template <bool EXACT, int G>
__global__ void __launch_bounds__(kFacPerCta * G) rank1_kernel(int n, double* L, int64_t strideL, const double* X,
                                                               int64_t strideX, const double* sigma, int batch) {
  __shared__ double xs_all[kFacPerCta][kUpdMaxN];
  __shared__ double rd_all[kFacPerCta][kUpdMaxN];
  if (warp_idle<G>(batch)) return;
  const int g = threadIdx.x / G, gl = threadIdx.x % G;
  const int s = blockIdx.x * kFacPerCta + g;
  const bool active = s < batch;
  double* xs = xs_all[g];
  if (active)
    for (int r = gl; r < n; r += G) xs[r] = X[(size_t)s * strideX + r];  // nalgebra updates a clone of x
  __syncwarp();
  group_rank_one<EXACT, G>(n, L + (size_t)(active ? s : 0) * strideL, n, xs, rd_all[g], active ? sigma[s] : 0.0, gl,
                           active);
}

template <bool EXACT, int G>
__global__ void __launch_bounds__(kFacPerCta * G) remove_kernel(int n, const double* L, int64_t strideL, int j,
                                                                double* Lout, int64_t strideOut, int batch) {
  __shared__ double xs_all[kFacPerCta][kUpdMaxN];
  __shared__ double rd_all[kFacPerCta][kUpdMaxN];
  if (warp_idle<G>(batch)) return;
  const int g = threadIdx.x / G, gl = threadIdx.x % G;
  const int s = blockIdx.x * kFacPerCta + g;
  const bool active = s < batch;
  const int m = n - 1;
  double* out = Lout + (size_t)(active ? s : 0) * strideOut;
  double* xs = xs_all[g];
  if (active) {
    const double* l = L + (size_t)s * strideL;
    for (int c = 0; c < m; ++c) {
      const double* src = l + (size_t)(c < j ? c : c + 1) * n;
      double* dst = out + (size_t)c * m;
      for (int r = gl; r < m; r += G) dst[r] = src[r < j ? r : r + 1];
    }
    for (int r = j + 1 + gl; r < n; r += G) xs[r - j - 1] = l[r + (size_t)j * n];  // the removed column's tail
  }
  __syncwarp();
  group_rank_one<EXACT, G>(m - j, out + j + (size_t)j * m, m, xs, rd_all[g], 1.0, gl, active);
}

template <bool EXACT, int G>
__global__ void __launch_bounds__(kFacPerCta * G) insert_kernel(int n, const double* L, int64_t strideL, int j,
                                                                const double* Col, int64_t strideCol, double* Lout,
                                                                int64_t strideOut, int32_t* info, int batch) {
  __shared__ double vs_all[kFacPerCta][kUpdMaxN];  // [0, j): the new row; [j, n): the new column below the centre
  __shared__ double rd_all[kFacPerCta][kUpdMaxN];
  if (warp_idle<G>(batch)) return;
  const int g = threadIdx.x / G, gl = threadIdx.x % G;
  const int s = blockIdx.x * kFacPerCta + g;
  const bool active = s < batch;
  const int m = n + 1, len = n - j;
  const double* l = L + (size_t)(active ? s : 0) * strideL;
  const double* col = Col + (size_t)(active ? s : 0) * strideCol;
  double* out = Lout + (size_t)(active ? s : 0) * strideOut;
  double* row = vs_all[g];
  double* ncol = vs_all[g] + j;
  if (active) {
    for (int c = 0; c < m; ++c) {
      double* dst = out + (size_t)c * m;
      if (c == j) {
        for (int r = gl; r < m; r += G) dst[r] = 0.0;
      } else {
        const double* src = l + (size_t)(c < j ? c : c - 1) * n;
        for (int r = gl; r < m; r += G) dst[r] = (r == j) ? 0.0 : src[r < j ? r : r - 1];
      }
    }
    for (int r = gl; r < n; r += G) row[r] = col[r < j ? r : r + 1];
  }
  __syncwarp();
  // row j: the lower solve with the top-left corner (solve.rs:74-101)
  bool ok = active;
  for (int i = 0; i < j; ++i) {
    const double* lc = l + (size_t)i * n;
    double coeff = 0.0;
    if (ok) {
      const double d = lc[i];  // every lane of the group reads it: the group agrees
      if (is_zero_bits(d)) {
        ok = false;  // nalgebra's assertion
      } else if (gl == 0) {
        coeff = dvd<EXACT>(row[i], d);
        row[i] = coeff;
      }
    }
    coeff = __shfl_sync(kFull, coeff, 0, G);
    if (ok)
      for (int r = i + 1 + gl; r < j; r += G)
        row[r] = EXACT ? __dadd_rn(__dmul_rn(-coeff, lc[r]), row[r]) : fma(-coeff, lc[r], row[r]);
    __syncwarp();
  }
  if (active && gl == 0 && info) info[s] = ok ? 0 : 1;
  if (ok)
    for (int k = gl; k < j; k += G) out[j + (size_t)k * m] = row[k];
  // centre: sqrt(col_j - |row|^2), |row|^2 in dotx's order (blas.rs:96-165)
  double nrm2 = 0.0;
  if constexpr (EXACT) {
    if (ok && gl == 0) {
      double a[8] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
      const int nb = j >> 3;
      for (int b = 0; b < nb; ++b)
#pragma unroll
        for (int q = 0; q < 8; ++q) a[q] = __dadd_rn(a[q], __dmul_rn(row[8 * b + q], row[8 * b + q]));
      double res = 0.0;
#pragma unroll
      for (int q = 0; q < 4; ++q) res = __dadd_rn(res, __dadd_rn(a[q], a[q + 4]));
      for (int e = 8 * nb; e < j; ++e) res = __dadd_rn(res, __dmul_rn(row[e], row[e]));
      nrm2 = res;
    }
    nrm2 = __shfl_sync(kFull, nrm2, 0, G);
  } else {
    double part = 0.0;
    if (ok)
      for (int e = gl; e < j; e += G) part = fma(row[e], row[e], part);
#pragma unroll
    for (int off = G / 2; off > 0; off >>= 1) part += __shfl_xor_sync(kFull, part, off, G);
    nrm2 = part;
  }
  const double center = __dsqrt_rn(add<EXACT>(ok ? col[j] : 1.0, -nrm2));
  if (ok && gl == 0) out[j + (size_t)j * m] = center;
  // new column: gemv(alpha = -1/centre, bottom-left L[j.., ..j], row, beta = 1/centre)
  const double alpha = dvd<EXACT>(-1.0, center), beta = dvd<EXACT>(1.0, center);
  if (ok) {
    if (j == 0) {
      for (int r = gl; r < len; r += G) ncol[r] = mul<EXACT>(ncol[r], beta);
    } else {
      for (int k = 0; k < j; ++k) {
        const double* lc = l + j + (size_t)k * n;
        const double val = row[k];
        const double b = (k == 0) ? beta : 1.0;
        for (int r = gl; r < len; r += G)
          ncol[r] = EXACT ? __dadd_rn(__dmul_rn(__dmul_rn(alpha, lc[r]), val), __dmul_rn(b, ncol[r]))
                          : fma(alpha * lc[r], val, b * ncol[r]);
      }
    }
    for (int r = gl; r < len; r += G) out[j + 1 + r + (size_t)j * m] = ncol[r];
  }
  __syncwarp();
  group_rank_one<EXACT, G>(len, out + (j + 1) + (size_t)(j + 1) * m, m, ncol, rd_all[g], -1.0, gl, ok);
}

template <int G>
void rank1_launch(bool exact, int n, double* L, int64_t strideL, const double* X, int64_t strideX,
                  const double* sigma, int batch, cudaStream_t st) {
  const int grid = (batch + kFacPerCta - 1) / kFacPerCta;
  if (exact)
    rank1_kernel<true, G><<<grid, kFacPerCta * G, 0, st>>>(n, L, strideL, X, strideX, sigma, batch);
  else
    rank1_kernel<false, G><<<grid, kFacPerCta * G, 0, st>>>(n, L, strideL, X, strideX, sigma, batch);
}

template <int G>
void remove_launch(bool exact, int n, const double* L, int64_t strideL, int j, double* Lout, int64_t strideOut,
                   int batch, cudaStream_t st) {
  const int grid = (batch + kFacPerCta - 1) / kFacPerCta;
  if (exact)
    remove_kernel<true, G><<<grid, kFacPerCta * G, 0, st>>>(n, L, strideL, j, Lout, strideOut, batch);
  else
    remove_kernel<false, G><<<grid, kFacPerCta * G, 0, st>>>(n, L, strideL, j, Lout, strideOut, batch);
}

template <int G>
void insert_launch(bool exact, int n, const double* L, int64_t strideL, int j, const double* col, int64_t strideCol,
                   double* Lout, int64_t strideOut, int32_t* info, int batch, cudaStream_t st) {
  const int grid = (batch + kFacPerCta - 1) / kFacPerCta;
  if (exact)
    insert_kernel<true, G><<<grid, kFacPerCta * G, 0, st>>>(n, L, strideL, j, col, strideCol, Lout, strideOut,
                                                             info, batch);
  else
    insert_kernel<false, G><<<grid, kFacPerCta * G, 0, st>>>(n, L, strideL, j, col, strideCol, Lout, strideOut,
                                                              info, batch);
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
  const bool exact = flags & NACU_FLAG_EXACT;
  if (batch >= kGroupMinBatch)
    rank1_launch<kGroupSmall>(exact, n, L, strideL, X, strideX, sigma, batch, (cudaStream_t)stream);
  else
    rank1_launch<32>(exact, n, L, strideL, X, strideX, sigma, batch, (cudaStream_t)stream);
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
  remove_launch<32>(flags & NACU_FLAG_EXACT, n, L, strideL, j, Lout, strideOut, batch, (cudaStream_t)stream);
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
  insert_launch<32>(flags & NACU_FLAG_EXACT, n, L, strideL, j, col, strideCol, Lout, strideOut, info, batch,
                    (cudaStream_t)stream);
  return check_launch("nacu_dchol_insert_column_batched");
}

}  // extern "C"
