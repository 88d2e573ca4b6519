// Batched LU with full pivoting (n <= 128): the GPU form of nalgebra's
// FullPivLU::new (src/linalg/full_piv_lu.rs:56-91), FullPivLU::solve_mut
// (:185-211) and, on identity right-hand sides, try_inverse (:216-233).
//
// One CTA per system; the matrix and the right-hand sides live in shared
// memory (column-major, odd leading dimension so row walks hit no bank
// conflicts).  Per step i:
//   - every warp reduces the per-warp pivot candidates (key, position, value)
//     to icamax_full's choice (src/base/min_max.rs:146-167: the largest |a| of
//     the trailing submatrix, the first in column-major order on ties, a NaN
//     only at its first position) and stops when that pivot is zero (the rest
//     of the matrix is zero: nalgebra's `break`);
//   - warp 0 rewrites columns i and q from registers (the column swap, the row
//     swap of rows i and p, the multipliers of column i in gauss_step_swap's
//     order, lu.rs:362-389) while the other warps swap rows i and p in every
//     other column, the right-hand sides included;
//   - all threads apply the rank-1 update of the trailing columns (the
//     right-hand sides ride along: the forward solve in nalgebra's order),
//     each tracking the largest |a| it wrote (the integer image of |a|, no
//     FP64 issue slots), so the next pivot search needs no pass of its own.
// Two CTA barriers per step.  The back substitution (stopping where nalgebra's
// would) and the inverse column permutation then run one warp per right-hand
// side; solving from given factors runs the permutation and the forward solve
// there too.  EXACT (NACU_FLAG_EXACT) rounds every product and sum separately
// and divides where nalgebra divides (bit-identical results); the default
// form contracts to FMA and multiplies by reciprocals.
#include <algorithm>

#include "common.cuh"

namespace nacu {
namespace {

constexpr int kFpThreads = 256;
constexpr int kFpWarps = kFpThreads / 32;
constexpr int kFpMaxN = 128;
constexpr int kFpMaxRhs = 16;

struct FpLayout {
  size_t sa, key, val, idx, piv, ipiv, jpiv, rd, total;
};

__host__ __device__ inline size_t fp_align(size_t x) { return (x + 15) & ~(size_t)15; }

__host__ __device__ inline FpLayout fp_layout(int n, int nrhs) {
  const int ld = n | 1;
  FpLayout l;
  l.sa = 0;
  l.key = fp_align(l.sa + (size_t)ld * (n + nrhs) * sizeof(double));
  l.val = fp_align(l.key + kFpWarps * sizeof(uint64_t));
  l.idx = fp_align(l.val + kFpWarps * sizeof(double));
  l.piv = fp_align(l.idx + kFpWarps * sizeof(int));
  l.ipiv = fp_align(l.piv + 4 * sizeof(int));
  l.jpiv = fp_align(l.ipiv + (size_t)n * sizeof(int));
  l.rd = fp_align(l.jpiv + (size_t)n * sizeof(int));
  l.total = fp_align(l.rd + (size_t)n * sizeof(double));
  return l;
}

// A warp's best (key, index, value) into its candidate slot.
__device__ __forceinline__ void fp_publish(uint64_t key, int idx, double val, uint64_t* s_key, int* s_idx,
                                           double* s_val, int warp, int lane) {
  uint64_t k = key;
  int i = idx;
  warp_argmax(k, i);
  const unsigned who = __ballot_sync(0xffffffffu, key == k && idx == i);
  const double v = __shfl_sync(0xffffffffu, val, __ffs(who) - 1);
  if (lane == 0) {
    s_key[warp] = k;
    s_idx[warp] = i;
    s_val[warp] = v;
  }
}

// The pivot of the step from the warps' candidates: icamax_full's choice
// (the largest key, the lowest column-major index on ties); returns its value.
__device__ __forceinline__ double fp_pick(const uint64_t* s_key, const int* s_idx, const double* s_val, int lane,
                                          int& idx) {
  const uint64_t key = lane < kFpWarps ? s_key[lane] : 0ull;
  const int id = lane < kFpWarps ? s_idx[lane] : 0x7fffffff;
  const double val = lane < kFpWarps ? s_val[lane] : 0.0;
  uint64_t k = key;
  int i = id;
  warp_argmax(k, i);
  const unsigned who = __ballot_sync(0xffffffffu, lane < kFpWarps && key == k && id == i);
  idx = i;
  return __shfl_sync(0xffffffffu, val, __ffs(who) - 1);
}

// mode: 0 = factor, 1 = factor + solve, 2 = solve from given factors.
template <bool EXACT>
__global__ void __launch_bounds__(kFpThreads, 5) fullpiv_kernel(int n, int nrhs, double* __restrict__ A, int64_t strideA,
                                                             int32_t* __restrict__ ipiv, int32_t* __restrict__ jpiv,
                                                             double* __restrict__ B, int64_t strideB,
                                                             int32_t* __restrict__ info, int batch, int mode) {
  extern __shared__ __align__(16) unsigned char fp_smem[];
  const FpLayout lay = fp_layout(n, nrhs);
  double* sa = reinterpret_cast<double*>(fp_smem + lay.sa);
  uint64_t* s_key = reinterpret_cast<uint64_t*>(fp_smem + lay.key);
  double* s_val = reinterpret_cast<double*>(fp_smem + lay.val);
  int* s_idx = reinterpret_cast<int*>(fp_smem + lay.idx);
  int* s_piv = reinterpret_cast<int*>(fp_smem + lay.piv);  // [3]: the solve's last zero U_ii from the bottom
  int* s_ipiv = reinterpret_cast<int*>(fp_smem + lay.ipiv);
  int* s_jpiv = reinterpret_cast<int*>(fp_smem + lay.jpiv);
  double* s_rd = reinterpret_cast<double*>(fp_smem + lay.rd);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int ld = n | 1;
  const int solve_cols = (mode == 0) ? 0 : nrhs;
  double* sb = sa + (size_t)ld * n;

  for (int s = blockIdx.x; s < batch; s += gridDim.x) {
    double* a = A + (size_t)s * strideA;
    for (int e = tid; e < n * n; e += kFpThreads) {
      const int c = e / n, r = e - c * n;
      sa[(size_t)c * ld + r] = a[e];
    }
    if (solve_cols > 0) {
      const double* b = B + (size_t)s * strideB;
      for (int e = tid; e < n * solve_cols; e += kFpThreads) {
        const int c = e / n, r = e - c * n;
        sb[(size_t)c * ld + r] = b[e];
      }
    }
    for (int i = tid; i < n; i += kFpThreads) {
      s_ipiv[i] = (mode == 2) ? ipiv[(size_t)s * n + i] : i;
      s_jpiv[i] = (mode == 2) ? jpiv[(size_t)s * n + i] : i;
    }
    __syncthreads();

    int inf = 0, steps = n;
    const int ncols = n + solve_cols;  // the right-hand sides ride along the elimination
    if (mode != 2) {
      // the first search, over the whole matrix
      uint64_t bkey = 0;
      int bidx = 0x7fffffff;
      double bval = 0.0;
      for (int e = tid; e < n * n; e += kFpThreads) {
        const int c = e / n, r = e - c * n;
        const double v = sa[(size_t)c * ld + r];
        const uint64_t k = pivot_key(v, e == 0);
        if (bidx == 0x7fffffff || k > bkey) {
          bkey = k;
          bidx = e;
          bval = v;
        }
      }
      fp_publish(bkey, bidx, bval, s_key, s_idx, s_val, warp, lane);
      __syncthreads();
      for (int i = 0; i < n; ++i) {
        // every warp reduces the candidates to the same pivot (no barrier)
        const int msz = n - i;
        int idx;
        const double diag = fp_pick(s_key, s_idx, s_val, lane, idx);
        if (is_zero_bits(diag)) {  // full_piv_lu.rs:73-76: the rest of the matrix is zero
          steps = i;
          break;
        }
        const int rp = i + idx % msz, cp = i + idx / msz;
        if (warp == 0) {
          // columns i and cp at once, from registers: the column swap, the
          // row swap of rows i and rp, and the multipliers of column i
          const double inv_diag = EXACT ? 1.0 / diag : rcp_nr(diag);  // gauss_step's inv_diag
          double* ci = sa + (size_t)i * ld;
          double* cq = sa + (size_t)cp * ld;
          const double a_ii = ci[i], a_rpi = ci[rp], a_icp = cq[i];
          double vi[kFpMaxN / 32], vq[kFpMaxN / 32];
#pragma unroll
          for (int q = 0; q < kFpMaxN / 32; ++q) {
            const int r = lane + 32 * q;
            if (r < n) {
              vi[q] = ci[r];
              vq[q] = cq[r];
            }
          }
          __syncwarp();
#pragma unroll
          for (int q = 0; q < kFpMaxN / 32; ++q) {
            const int r = lane + 32 * q;
            if (r < n) {
              if (cp != i) cq[r] = (r == i) ? a_rpi : (r == rp ? a_ii : vi[q]);
              double u = (r == i) ? diag : (r == rp ? a_icp : vq[q]);
              if (r > i) u = EXACT ? __dmul_rn(u, inv_diag) : u * inv_diag;
              ci[r] = u;
            }
          }
          if (lane == 0) {
            s_ipiv[i] = rp;
            s_jpiv[i] = cp;
          }
        } else if (rp != i) {
          for (int c = tid - 32; c < ncols; c += kFpThreads - 32) {
            if (c == i || c == cp) continue;
            double* col = sa + (size_t)c * ld;
            const double t = col[i];
            col[i] = col[rp];
            col[rp] = t;
          }
        }
        __syncthreads();
        // rank-1 update of rows i+1.. of columns i+1.. (right-hand sides
        // included), tracking the next pivot over the matrix columns
        const int m = n - 1 - i;
        uint64_t bk = 0;
        int bi = 0x7fffffff;
        double bv = 0.0;
        if (m > 0) {
          const int total = m * (ncols - 1 - i), mm = m * m;
          const double* lcol = sa + (size_t)i * ld + i + 1;
          int e = tid;
          int cq = e / m;
          int rr = e - cq * m;
          const int dq = kFpThreads / m, dr = kFpThreads - dq * m;
          double* base = sa + (size_t)(i + 1) * ld;
          for (; e < total; e += kFpThreads) {
            double* col = base + (size_t)cq * ld;
            const double v = axpy1<EXACT>(col[i + 1 + rr], -col[i], lcol[rr]);
            col[i + 1 + rr] = v;
            if (e < mm) {  // a matrix column: e = cq * m + rr, column-major in the next submatrix
              const uint64_t k = pivot_key(v, e == 0);
              if (bi == 0x7fffffff || k > bk) {  // e increases: the first of equal keys stays
                bk = k;
                bi = e;
                bv = v;
              }
            }
            rr += dr;
            cq += dq;
            if (rr >= m) {
              rr -= m;
              ++cq;
            }
          }
        }
        fp_publish(bk, bi, bv, s_key, s_idx, s_val, warp, lane);
        __syncthreads();
      }
      // is_invertible (full_piv_lu.rs:242-250): U[n-1][n-1] != 0; else report
      // the step at which the rest of the matrix was zero
      inf = (n == 0 || sa[(size_t)(n - 1) * ld + (n - 1)] != 0.0) ? 0 : steps + 1;
    } else if (n > 0 && sa[(size_t)(n - 1) * ld + (n - 1)] == 0.0) {
      inf = n;
      for (int i = n - 1; i >= 0; --i)
        if (sa[(size_t)i * ld + i] == 0.0) inf = i + 1;
    }

    if (solve_cols > 0 && inf == 0 && n > 0) {
      if (tid == 0) {  // the last zero U_ii from the bottom stops nalgebra's upper solve
        int z = -1;
        for (int i = n - 1; i >= 0; --i)
          if (sa[(size_t)i * ld + i] == 0.0) {
            z = i;
            break;
          }
        s_piv[3] = z;
      }
      if constexpr (!EXACT)
        for (int i = tid; i < n; i += kFpThreads) s_rd[i] = 1.0 / sa[(size_t)i * ld + i];
      __syncthreads();
      const int z = s_piv[3];
      for (int c = warp; c < solve_cols; c += kFpWarps) {
        double* bc = sb + (size_t)c * ld;
        // p.permute_rows (permutation_sequence.rs:97-104) and the unit-lower
        // solve rode along the elimination for its steps; from factors (and
        // after a stop) they run here, in nalgebra's order
        if (mode == 2 && lane == 0)
          for (int i = 0; i < n; ++i) {
            const int p = s_ipiv[i];
            if (p != i) {
              const double t = bc[i];
              bc[i] = bc[p];
              bc[p] = t;
            }
          }
        __syncwarp();
        for (int i = (mode == 2) ? 0 : steps; i + 1 < n; ++i) {  // solve_lower_triangular_with_diag_mut(b, 1)
          const double coeff = bc[i];
          const double* lc = sa + (size_t)i * ld;
          for (int r = i + 1 + lane; r < n; r += 32) bc[r] = axpy1<EXACT>(bc[r], -coeff, lc[r]);
          __syncwarp();
        }
        // solve_upper_triangular_mut(b): at a zero U_ii nalgebra returns,
        // leaving that column partly and the later columns not solved
        const int lo = (z < 0) ? 0 : (c == 0 ? z + 1 : n);
        for (int i = n - 1; i >= lo; --i) {
          const double* uc = sa + (size_t)i * ld;
          if (lane == 0) bc[i] = EXACT ? __ddiv_rn(bc[i], uc[i]) : bc[i] * s_rd[i];
          __syncwarp();
          const double coeff = bc[i];
          for (int r = lane; r < i; r += 32) bc[r] = axpy1<EXACT>(bc[r], -coeff, uc[r]);
          __syncwarp();
        }
        if (lane == 0)  // q.inv_permute_rows (permutation_sequence.rs:108-116)
          for (int k = n - 1; k >= 0; --k) {
            const int q = s_jpiv[k];
            if (q != k) {
              const double t = bc[k];
              bc[k] = bc[q];
              bc[q] = t;
            }
          }
        __syncwarp();
      }
    }
    __syncthreads();
    if (mode != 2) {
      for (int e = tid; e < n * n; e += kFpThreads) {
        const int c = e / n, r = e - c * n;
        a[e] = sa[(size_t)c * ld + r];
      }
      for (int i = tid; i < n; i += kFpThreads) {
        ipiv[(size_t)s * n + i] = s_ipiv[i];
        jpiv[(size_t)s * n + i] = s_jpiv[i];
      }
    }
    if (solve_cols > 0 && inf == 0) {  // not invertible: B stays as given (the ride-along copy is dropped)
      double* b = B + (size_t)s * strideB;
      for (int e = tid; e < n * solve_cols; e += kFpThreads) {
        const int c = e / n, r = e - c * n;
        b[e] = sb[(size_t)c * ld + r];
      }
    }
    if (tid == 0 && info) info[s] = inf;
    __syncthreads();
  }
}

int fullpiv_launch(int n, int nrhs, double* A, int64_t strideA, int32_t* ipiv, int32_t* jpiv, double* B,
                   int64_t strideB, int32_t* info, int batch, int flags, int mode, cudaStream_t stream,
                   const char* name) {
  const size_t smem = fp_layout(n, nrhs).total;
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const bool exact = flags & NACU_FLAG_EXACT;
  auto kern = exact ? fullpiv_kernel<true> : fullpiv_kernel<false>;
  if (smem > 48 * 1024) {
    const cudaError_t e = ensure_dynamic_smem(kern, smem);
    if (e != cudaSuccess) return record_cuda_error(e, name);
  }
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kFpThreads, smem);
  // persistent: as many CTAs as fit at once, each taking systems grid-stride
  const int grid = std::max(1, std::min(batch, std::max(1, per_sm) * std::max(1, nsm)));
  kern<<<grid, kFpThreads, smem, stream>>>(n, nrhs, A, strideA, ipiv, jpiv, B, strideB, info, batch, mode);
  return check_launch(name);
}

}  // namespace
}  // namespace nacu

using namespace nacu;

extern "C" {

int nacu_dfullpivlu_batched(int n, int nrhs, double* A, int64_t strideA, int32_t* ipiv, int32_t* jpiv, double* B,
                            int64_t strideB, int32_t* info, int batch, int flags, nacu_stream_t stream) {
  const char* name = "nacu_dfullpivlu_batched";
  if (n < 0 || n > kFpMaxN) return record_arg_error(-1, "full-pivot LU batched: n out of range [0, 128]");
  if (nrhs < 0 || nrhs > kFpMaxRhs) return record_arg_error(-2, "full-pivot LU batched: nrhs out of range [0, 16]");
  if (batch < 0) return record_arg_error(-10, "full-pivot LU batched: negative batch");
  if (batch == 0 || n == 0) return NACU_SUCCESS;
  if (!A || !ipiv || !jpiv || (nrhs > 0 && !B)) return record_arg_error(-3, "full-pivot LU batched: null pointer");
  if (strideA < (int64_t)n * n) return record_arg_error(-4, "full-pivot LU batched: strideA < n*n");
  if (nrhs > 0 && strideB < (int64_t)n * nrhs) return record_arg_error(-8, "full-pivot LU batched: strideB < n*nrhs");
  return fullpiv_launch(n, nrhs, A, strideA, ipiv, jpiv, B, strideB, info, batch, flags, nrhs > 0 ? 1 : 0,
                        (cudaStream_t)stream, name);
}

int nacu_dfullpivlu_solve_batched(int n, int nrhs, const double* LU, int64_t strideA, const int32_t* ipiv,
                                  const int32_t* jpiv, double* B, int64_t strideB, int32_t* info, int batch,
                                  int flags, nacu_stream_t stream) {
  const char* name = "nacu_dfullpivlu_solve_batched";
  if (n < 0 || n > kFpMaxN) return record_arg_error(-1, "full-pivot LU solve: n out of range [0, 128]");
  if (nrhs < 0 || nrhs > kFpMaxRhs) return record_arg_error(-2, "full-pivot LU solve: nrhs out of range [0, 16]");
  if (batch < 0) return record_arg_error(-10, "full-pivot LU solve: negative batch");
  if (batch == 0 || n == 0 || nrhs == 0) return NACU_SUCCESS;
  if (!LU || !ipiv || !jpiv || !B) return record_arg_error(-3, "full-pivot LU solve: null pointer");
  if (strideA < (int64_t)n * n) return record_arg_error(-4, "full-pivot LU solve: strideA < n*n");
  if (strideB < (int64_t)n * nrhs) return record_arg_error(-8, "full-pivot LU solve: strideB < n*nrhs");
  // mode 2 reads the factors and pivots and writes only B and info
  return fullpiv_launch(n, nrhs, const_cast<double*>(LU), strideA, const_cast<int32_t*>(ipiv),
                        const_cast<int32_t*>(jpiv), B, strideB, info, batch, flags, 2, (cudaStream_t)stream, name);
}

}  // extern "C"
