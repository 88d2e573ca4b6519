// Batched triangular solves (n <= 128), the GPU form of nalgebra's standalone
// Matrix::{solve,tr_solve,ad_solve}_{lower,upper}_triangular_mut and
// solve_lower_triangular_with_diag_mut (src/linalg/solve.rs:55-442): for every
// system s, B_s (n x nrhs, column-major) <- T_s^-1 B_s or T_s^-T B_s, T_s
// lower or upper triangular (only that triangle is read).
//
// One warp per (system, right-hand-side column); the column sits in the
// warp's shared-memory slot, the triangle is read from global memory (L1/L2:
// the nrhs warps of one system share it).  Each column receives nalgebra's
// operations in nalgebra's order:
//   plain forms: the axpy sweep (coeff = b_i / T_ii, then b_j -= coeff T_ji
//     for the rows not yet solved), true division;
//   transposed forms: b_i = (b_i - dot) / T_ii with the dot of Matrix::dotx
//     (src/base/blas.rs:96-165): eight accumulators over blocks of 8, combined
//     (a0+a4), (a1+a5), (a2+a6), (a3+a7), then the tail one product at a time.
// EXACT (NACU_FLAG_EXACT) rounds every product and sum separately and divides
// at every step, as Rust does (bit-identical results); the default form
// contracts to FMA, uses a warp reduction for the dots and multiplies by the
// reciprocals of the diagonal, formed 32 at a time before the sweep: on this
// part an FP64 instruction costs the same pipe time whether one lane or 32 run
// it, and a division is a chain of them.
#include <algorithm>

#include "common.cuh"

namespace nacu {
namespace {

constexpr int kTrsvBWarps = 8;
constexpr int kTrsvBMaxN = 128;

struct TrsvBArgs {
  int n, nrhs, upper, trans, has_diag;
  double diag;
  const double* T;
  int64_t strideT;
  double* B;
  int64_t strideB;
  int32_t* info;
  int batch;
};

// sum_{e < len} x[e] * y[e], in nalgebra's dotx order (EXACT) or as a warp
// reduction (FMA form); the result is valid in every lane.
template <bool EXACT>
__device__ __forceinline__ double warp_dot(int len, const double* x, const double* y, int lane) {
  if constexpr (EXACT) {
    const int nb = len >> 3;
    double acc = 0.0;
    if (lane < 8)
      for (int b = 0; b < nb; ++b) acc = __dadd_rn(acc, __dmul_rn(x[8 * b + lane], y[8 * b + lane]));
    const double hi = __shfl_down_sync(0xffffffffu, acc, 4);
    const double pair = __dadd_rn(acc, hi);  // lanes 0..3: a_k + a_{k+4}
    const double p0 = __shfl_sync(0xffffffffu, pair, 0), p1 = __shfl_sync(0xffffffffu, pair, 1);
    const double p2 = __shfl_sync(0xffffffffu, pair, 2), p3 = __shfl_sync(0xffffffffu, pair, 3);
    double res = 0.0;
    res = __dadd_rn(res, p0);
    res = __dadd_rn(res, p1);
    res = __dadd_rn(res, p2);
    res = __dadd_rn(res, p3);
    for (int e = 8 * nb; e < len; ++e) res = __dadd_rn(res, __dmul_rn(x[e], y[e]));
    return res;
  } else {
    double part = 0.0;
    for (int e = lane; e < len; e += 32) part = fma(x[e], y[e], part);
    return warp_sum(part);
  }
}

template <bool EXACT>
__global__ void __launch_bounds__(kTrsvBWarps * 32) trsv_batched_kernel(TrsvBArgs g) {
  __shared__ double xs_all[kTrsvBWarps][kTrsvBMaxN];
  __shared__ double rd_all[kTrsvBWarps][kTrsvBMaxN];  // FMA form: 1 / T_ii
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t pair = (int64_t)blockIdx.x * kTrsvBWarps + warp;
  const int n = g.n;
  if (pair >= (int64_t)g.batch * g.nrhs) return;
  const int s = (int)(pair / g.nrhs), c = (int)(pair - (int64_t)s * g.nrhs);
  const double* t = g.T + (size_t)s * g.strideT;
  double* bcol = g.B + (size_t)s * g.strideB + (size_t)c * n;
  double* xs = xs_all[warp];
  double* rd = rd_all[warp];
  for (int j = lane; j < n; j += 32) xs[j] = bcol[j];
  if (!EXACT && !g.has_diag)  // the n divisions at once, 32 lanes per FP64 warp instruction
    for (int j = lane; j < n; j += 32) rd[j] = 1.0 / t[(size_t)j * n + j];
  __syncwarp();
  int fail = 0;  // 1-based index of the zero diagonal that stops the solve
  if (g.has_diag) {  // solve_lower_triangular_with_diag_mut: b_i is not rewritten
    if (g.diag == 0.0) fail = 1;
    for (int i = 0; i + 1 < n && !fail; ++i) {
      double coeff = 0.0;
      if (lane == 0) coeff = xs[i] / g.diag;  // one division per step, broadcast
      coeff = __shfl_sync(0xffffffffu, coeff, 0);
      const double* col = t + (size_t)i * n;
      for (int j = i + 1 + lane; j < n; j += 32) xs[j] = axpy1<EXACT>(xs[j], -coeff, col[j]);
      __syncwarp();
    }
  } else if (!g.trans) {
    for (int k = 0; k < n; ++k) {
      const int i = g.upper ? n - 1 - k : k;
      const double* col = t + (size_t)i * n;
      const double d = col[i];
      if (is_zero_bits(d)) {
        fail = i + 1;
        break;
      }
      double coeff = 0.0;
      if (lane == 0) {
        coeff = EXACT ? xs[i] / d : xs[i] * rd[i];
        xs[i] = coeff;
      }
      coeff = __shfl_sync(0xffffffffu, coeff, 0);
      const int j0 = g.upper ? 0 : i + 1, j1 = g.upper ? i : n;
      for (int j = j0 + lane; j < j1; j += 32) xs[j] = axpy1<EXACT>(xs[j], -coeff, col[j]);
      __syncwarp();
    }
  } else {
    for (int k = 0; k < n; ++k) {
      const int i = g.upper ? k : n - 1 - k;
      const double* col = t + (size_t)i * n;
      // tr lower: dot(T[i+1.., i], b[i+1..]); tr upper: dot(T[..i, i], b[..i])
      const double dt = g.upper ? warp_dot<EXACT>(i, col, xs, lane)
                                : warp_dot<EXACT>(n - i - 1, col + i + 1, xs + i + 1, lane);
      const double d = col[i];
      if (is_zero_bits(d)) {
        fail = i + 1;
        break;
      }
      if (lane == 0) xs[i] = EXACT ? __ddiv_rn(__dsub_rn(xs[i], dt), d) : (xs[i] - dt) * rd[i];
      __syncwarp();
    }
  }
  __syncwarp();
  for (int j = lane; j < n; j += 32) bcol[j] = xs[j];
  // every column of a system stops at the same diagonal: any warp reports it
  if (lane == 0 && c == 0 && g.info) g.info[s] = fail;
}

}  // namespace
}  // namespace nacu

extern "C" int nacu_dtrsv_batched(int n, int nrhs, int upper, int trans, int has_diag, double diag, const double* T,
                                  int64_t strideT, double* B, int64_t strideB, int32_t* info, int batch, int flags,
                                  nacu_stream_t stream) {
  using namespace nacu;
  const char* name = "nacu_dtrsv_batched";
  if (n < 0 || n > kTrsvBMaxN) return record_arg_error(-1, "trsv batched: n out of range [0, 128]");
  if (nrhs < 0) return record_arg_error(-2, "trsv batched: negative nrhs");
  if (has_diag && (upper || trans)) return record_arg_error(-5, "trsv batched: the diag form is lower, non-transposed");
  if (batch < 0) return record_arg_error(-12, "trsv batched: negative batch");
  if (batch == 0 || n == 0 || nrhs == 0) return NACU_SUCCESS;
  if (!T || !B) return record_arg_error(-7, "trsv batched: null T or B");
  if (strideT < (int64_t)n * n) return record_arg_error(-8, "trsv batched: strideT < n*n");
  if (strideB < (int64_t)n * nrhs) return record_arg_error(-10, "trsv batched: strideB < n*nrhs");
  TrsvBArgs g{n, nrhs, upper ? 1 : 0, trans ? 1 : 0, has_diag ? 1 : 0, diag, T, strideT, B, strideB, info, batch};
  const int64_t pairs = (int64_t)batch * nrhs;
  const int64_t grid = (pairs + kTrsvBWarps - 1) / kTrsvBWarps;
  if (grid > 0x7fffffff) return record_arg_error(-12, "trsv batched: batch * nrhs too large");
  if (flags & NACU_FLAG_EXACT) trsv_batched_kernel<true><<<(unsigned)grid, kTrsvBWarps * 32, 0, (cudaStream_t)stream>>>(g);
  else trsv_batched_kernel<false><<<(unsigned)grid, kTrsvBWarps * 32, 0, (cudaStream_t)stream>>>(g);
  return check_launch(name);
}
