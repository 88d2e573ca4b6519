// Batched QR with column pivoting (n <= 128): the GPU form of nalgebra's
// ColPivQR::new (src/linalg/col_piv_qr.rs:59-92), ColPivQR::solve_mut
// (:227-247) and, on identity right-hand sides, try_inverse (:288-303).
// Without the pivot search (PIVOT = false) the same kernel is nalgebra's plain
// square QR: QR::new (src/linalg/qr.rs:55-76, the same clear_column_unchecked
// steps on the unswapped columns), QR::solve_mut (:204-256: q_tr_mul, then the
// upper solve by |diag_i|, no permutation) and QR::try_inverse (:262-279).
//
// One CTA per system; the matrix and the right-hand sides live in shared
// memory (column-major, odd leading dimension).  Per step i:
//   - warp 0 reduces the per-warp candidates to icamax_full's column (the
//     column of the trailing submatrix's largest |a|, src/base/min_max.rs:
//     146-167; not the largest column norm), swaps it with column i and turns
//     column i into the Householder axis (householder::reflection_axis_mut,
//     householder.rs:19-53: norm, sign rule, two normalisations);
//   - the reflection of the trailing columns (reflection.rs:70-83): one
//     thread per column forms its factor (a dot with the axis, sequential, so
//     no warp reductions spend FP64 adds), then all threads apply the axpys
//     as one flattened update, one FMA per element with the sign folded in,
//     each tracking the largest |a| it wrote for the next step's pivot; the
//     right-hand sides ride along (q_tr_mul applies every reflection, even
//     where the column was zero).
// Three CTA barriers per step.  The upper solve (divide by |diag_i|, stopping
// where nalgebra's would) and the inverse column permutation then run one
// warp per right-hand side.  EXACT (NACU_FLAG_EXACT) rounds every operation
// as Rust does, the dots in dotx's order (src/base/blas.rs:96-165):
// bit-identical factors, pivots and solutions.  The default form contracts to
// FMA and reduces the dots across the warp.
#include <algorithm>

#include "common.cuh"
#include "householder.cuh"

namespace nacu {
namespace {

constexpr int kCqThreads = 256;
constexpr int kCqWarps = kCqThreads / 32;
constexpr int kCqMaxN = 128;
constexpr int kCqMaxRhs = 16;

struct CqLayout {
  size_t sa, key, idx, diag, rd, f, jpiv, flag, total;
};

__host__ __device__ inline size_t cq_align(size_t x) { return (x + 15) & ~(size_t)15; }

__host__ __device__ inline CqLayout cq_layout(int n, int nrhs) {
  const int ld = n | 1;
  CqLayout l;
  l.sa = 0;
  l.key = cq_align((size_t)ld * (n + nrhs) * sizeof(double));
  l.idx = cq_align(l.key + kCqWarps * sizeof(uint64_t));
  l.diag = cq_align(l.idx + kCqWarps * sizeof(int));
  l.rd = cq_align(l.diag + (size_t)n * sizeof(double));
  l.f = cq_align(l.rd + (size_t)n * sizeof(double));
  l.jpiv = cq_align(l.f + (size_t)(n + nrhs) * sizeof(double));
  l.flag = cq_align(l.jpiv + (size_t)n * sizeof(int));
  l.total = cq_align(l.flag + 4 * sizeof(int));
  return l;
}

// mode: 0 = factor, 1 = factor + solve, 2 = solve from given factors.
// PIVOT = false: no column search or swap, no pivots read or written.
template <bool EXACT, bool PIVOT>
__global__ void __launch_bounds__(kCqThreads) colpivqr_kernel(int n, int nrhs, double* __restrict__ A, int64_t strideA,
                                                              double* __restrict__ diag, int32_t* __restrict__ jpiv,
                                                              double* __restrict__ B, int64_t strideB,
                                                              int32_t* __restrict__ info, int batch, int mode) {
  extern __shared__ __align__(16) unsigned char cq_smem[];
  const CqLayout lay = cq_layout(n, nrhs);
  double* sa = reinterpret_cast<double*>(cq_smem + lay.sa);
  uint64_t* s_key = reinterpret_cast<uint64_t*>(cq_smem + lay.key);
  int* s_idx = reinterpret_cast<int*>(cq_smem + lay.idx);
  double* s_diag = reinterpret_cast<double*>(cq_smem + lay.diag);
  double* s_rd = reinterpret_cast<double*>(cq_smem + lay.rd);
  double* s_f = reinterpret_cast<double*>(cq_smem + lay.f);  // the step's reflection factor per trailing column
  int* s_jpiv = reinterpret_cast<int*>(cq_smem + lay.jpiv);
  int* s_flag = reinterpret_cast<int*>(cq_smem + lay.flag);  // [0] the step's reflection is not empty
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int ld = n | 1;
  const int solve_cols = (mode == 0) ? 0 : nrhs;
  const int ncols = n + ((mode == 1) ? nrhs : 0);  // right-hand sides ride along the factorization
  double* sb = sa + (size_t)ld * n;

  for (int s = blockIdx.x; s < batch; s += gridDim.x) {
    double* a = A + (size_t)s * strideA;
    for (int e = tid; e < n * n; e += kCqThreads) {
      const int c = e / n, r = e - c * n;
      sa[(size_t)c * ld + r] = a[e];
    }
    if (solve_cols > 0) {
      const double* b = B + (size_t)s * strideB;
      for (int e = tid; e < n * solve_cols; e += kCqThreads) {
        const int c = e / n, r = e - c * n;
        sb[(size_t)c * ld + r] = b[e];
      }
    }
    if (mode == 2)
      for (int i = tid; i < n; i += kCqThreads) {
        s_diag[i] = diag[(size_t)s * n + i];
        s_jpiv[i] = PIVOT ? jpiv[(size_t)s * n + i] : i;
      }
    __syncthreads();

    if (mode != 2) {
      uint64_t bkey = 0;
      int bidx = 0x7fffffff;
      for (int e = PIVOT ? tid : n * n; e < n * n; e += kCqThreads) {  // the first search, over the whole matrix
        const int c = e / n, r = e - c * n;
        const uint64_t k = pivot_key(sa[(size_t)c * ld + r], e == 0);
        if (bidx == 0x7fffffff || k > bkey) {
          bkey = k;
          bidx = e;
        }
      }
      warp_argmax(bkey, bidx);
      if (lane == 0) {
        s_key[warp] = bkey;
        s_idx[warp] = bidx;
      }
      __syncthreads();
      for (int i = 0; i < n; ++i) {
        const int L = n - i;
        if (warp == 0) {
          int cp = i;
          if constexpr (PIVOT) {
            uint64_t key = lane < kCqWarps ? s_key[lane] : 0ull;
            int idx = lane < kCqWarps ? s_idx[lane] : 0x7fffffff;
            warp_argmax(key, idx);
            cp = i + idx / L;
          }
          if (cp != i)  // swap_columns(i, cp)
            for (int r = lane; r < n; r += 32) {
              const double t = sa[(size_t)i * ld + r];
              sa[(size_t)i * ld + r] = sa[(size_t)cp * ld + r];
              sa[(size_t)cp * ld + r] = t;
            }
          __syncwarp();
          // reflection_axis_mut on rows i.. of column i
          double* x = sa + (size_t)i * ld + i;
          double sq, nrm, signed_norm, factor;
          if constexpr (EXACT) {
            sq = cq_add<EXACT>(0.0, cq_dot<EXACT>(L, x, x, lane));
            nrm = __dsqrt_rn(sq);
            double modulus, sign;
            cq_to_exp(x[0], modulus, sign);
            signed_norm = cq_mul<EXACT>(sign, nrm);
            factor = cq_mul<EXACT>(cq_add<EXACT>(sq, cq_mul<EXACT>(modulus, nrm)), 2.0);
          } else {
            // the same values with the sign logic on the bits (x0 >= 0 holds
            // for +-0 and fails for NaN, as to_exp's test) and one FMA: on
            // this warp every FP64 instruction is on the step's critical path
            sq = cq_dot<EXACT>(L, x, x, lane);
            nrm = __dsqrt_rn(sq);
            const long long xb = __double_as_longlong(x[0]);
            const long long mag = xb & 0x7fffffffffffffffll;
            const bool ge0 = mag == 0 || (xb >= 0 && mag <= 0x7ff0000000000000ll);
            const long long flip = ge0 ? 0ll : (long long)0x8000000000000000ull;
            const double modulus = __longlong_as_double(xb ^ flip);
            signed_norm = __longlong_as_double(__double_as_longlong(nrm) ^ flip);
            factor = fma(modulus, nrm, sq) * 2.0;
          }
          __syncwarp();
          if (lane == 0) x[0] = cq_add<EXACT>(x[0], signed_norm);
          __syncwarp();
          const bool nz = !is_zero_bits(factor);
          double rnorm = signed_norm;
          if (nz) {
            if constexpr (EXACT) {
              const double sf = __dsqrt_rn(factor);
              for (int k = lane; k < L; k += 32) x[k] = __ddiv_rn(x[k], sf);  // unscale_mut
              __syncwarp();
              const double n2 = __dsqrt_rn(cq_add<EXACT>(0.0, cq_dot<EXACT>(L, x, x, lane)));  // normalize_mut
              __syncwarp();
              for (int k = lane; k < L; k += 32) x[k] = __ddiv_rn(x[k], n2);
            } else {
              // factor = 2 (sq + |x0| nrm) is |x'|^2 for the updated axis x',
              // so one scale by rsqrt(factor) makes it a unit vector: the
              // second normalisation and the two divisions per element (each
              // a chain of FP64 instructions on this warp, the step's
              // critical path) only corrected rounding
              const double rs = rsqrt(factor);
              for (int k = lane; k < L; k += 32) x[k] *= rs;
            }
            rnorm = -signed_norm;
          }
          if (lane == 0) {
            s_diag[i] = rnorm;
            s_jpiv[i] = cp;
            s_flag[0] = nz ? 1 : 0;
          }
        }
        __syncthreads();
        // the reflection of the trailing columns (reflect_with_sign, bias 0):
        // first every column's factor (its dot with the axis, one thread per
        // column), then the axpys as one flattened update
        const bool nz = s_flag[0] != 0;
        const double sgn = cq_signum(s_diag[i]);
        const double m_two = cq_mul<EXACT>(sgn, -2.0);
        const double* v = sa + (size_t)i * ld + i;
        const int ntr = ncols - i - 1;
        for (int t = tid; t < ntr; t += kCqThreads) {
          const int c = i + 1 + t;
          double f = 0.0;
          if (nz || c >= n) f = cq_mul<EXACT>(cq_dot_seq<EXACT>(L, v, sa + (size_t)c * ld + i), m_two);
          s_f[t] = f;
        }
        __syncthreads();
        const int lm = L - 1;  // the next submatrix is lm x lm
        // the sign's case, decided once: FP64 compares run on the FP64 pipe
        const int smode = (sgn == 1.0) ? 0 : (sgn == -1.0 ? 1 : 2);
        uint64_t bk = 0;
        int bi = 0x7fffffff;
        if (ntr > 0) {
          const int total = L * ntr;
          int e = tid;
          int cq = e / L;
          int rr = e - cq * L;
          const int dq = kCqThreads / L, dr = kCqThreads - dq * L;
          for (; e < total; e += kCqThreads) {
            const int c = i + 1 + cq;
            double* col = sa + (size_t)c * ld + i;
            double val = col[rr];
            if (nz || c >= n) {
              const double f = s_f[cq];
              if constexpr (EXACT) {
                val = __dadd_rn(__dmul_rn(f, v[rr]), __dmul_rn(sgn, val));
              } else {
                // sgn * col + f * v with the sign folded into one FMA
                val = (smode == 0) ? fma(f, v[rr], val)
                                   : (smode == 1 ? neg_bits(fma(-f, v[rr], val)) : fma(f, v[rr], sgn * val));
              }
              col[rr] = val;
            }
            if (PIVOT && c < n && rr > 0) {  // rows i+1.. of the matrix columns, column-major in the next submatrix
              const int en = cq * lm + (rr - 1);  // increases with e: the first of equal keys stays
              const uint64_t kk = pivot_key(val, en == 0);
              if (bi == 0x7fffffff || kk > bk) {
                bk = kk;
                bi = en;
              }
            }
            rr += dr;
            cq += dq;
            if (rr >= L) {
              rr -= L;
              ++cq;
            }
          }
        }
        warp_argmax(bk, bi);
        if (lane == 0) {
          s_key[warp] = bk;
          s_idx[warp] = bi;
        }
        __syncthreads();
      }
    }

    // is_invertible (col_piv_qr.rs:307-320): every diag entry non-zero; info =
    // 1 + the first zero one
    int inf = 0;
    for (int i = n - 1; i >= 0; --i)
      if (s_diag[i] == 0.0) inf = i + 1;

    if (solve_cols > 0) {
      if constexpr (!EXACT)
        for (int i = tid; i < n; i += kCqThreads) s_rd[i] = 1.0 / fabs(s_diag[i]);
      __syncthreads();
      int zb = -1;  // the first zero |diag_i| from the bottom stops nalgebra's upper solve
      for (int i = 0; i < n; ++i)
        if (s_diag[i] == 0.0) zb = i;
      for (int c = warp; c < solve_cols; c += kCqWarps) {
        double* bc = sb + (size_t)c * ld;
        if (mode == 2)  // q_tr_mul (col_piv_qr.rs:180-192): every reflection
          for (int i = 0; i < n; ++i) {
            const double sgn = cq_signum(s_diag[i]);
            const double* v = sa + (size_t)i * ld + i;
            double* y = bc + i;
            const double f = cq_mul<EXACT>(cq_dot<EXACT>(n - i, v, y, lane), cq_mul<EXACT>(sgn, -2.0));
            __syncwarp();
            for (int k = lane; k < n - i; k += 32)
              y[k] = EXACT ? __dadd_rn(__dmul_rn(f, v[k]), __dmul_rn(sgn, y[k])) : fma(f, v[k], sgn * y[k]);
            __syncwarp();
          }
        const int lo = (zb < 0) ? 0 : (c == 0 ? zb + 1 : n);
        for (int i = n - 1; i >= lo; --i) {  // col_piv_qr.rs:250-285
          const double* uc = sa + (size_t)i * ld;
          if (lane == 0) bc[i] = EXACT ? __ddiv_rn(bc[i], fabs(s_diag[i])) : bc[i] * s_rd[i];
          __syncwarp();
          const double coeff = bc[i];
          for (int r = lane; r < i; r += 32) bc[r] = axpy1<EXACT>(bc[r], -coeff, uc[r]);
          __syncwarp();
        }
        if (PIVOT && lane == 0)  // p.inv_permute_rows, whatever the upper solve returned
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
      for (int e = tid; e < n * n; e += kCqThreads) {
        const int c = e / n, r = e - c * n;
        a[e] = sa[(size_t)c * ld + r];
      }
      for (int i = tid; i < n; i += kCqThreads) {
        diag[(size_t)s * n + i] = s_diag[i];
        if (PIVOT) jpiv[(size_t)s * n + i] = s_jpiv[i];
      }
    }
    if (solve_cols > 0) {  // nalgebra overwrites b even when the upper solve fails
      double* b = B + (size_t)s * strideB;
      for (int e = tid; e < n * solve_cols; e += kCqThreads) {
        const int c = e / n, r = e - c * n;
        b[e] = sb[(size_t)c * ld + r];
      }
    }
    if (tid == 0 && info) info[s] = inf;
    __syncthreads();
  }
}

int colpivqr_launch(int n, int nrhs, double* A, int64_t strideA, double* diag, int32_t* jpiv, double* B,
                    int64_t strideB, int32_t* info, int batch, int flags, int mode, cudaStream_t stream,
                    const char* name, bool pivot = true) {
  const size_t smem = cq_layout(n, nrhs).total;
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const bool exact = (flags & NACU_FLAG_EXACT) != 0;
  auto kern = pivot ? (exact ? colpivqr_kernel<true, true> : colpivqr_kernel<false, true>)
                    : (exact ? colpivqr_kernel<true, false> : colpivqr_kernel<false, false>);
  if (smem > 48 * 1024) {
    const cudaError_t e = ensure_dynamic_smem(kern, smem);
    if (e != cudaSuccess) return record_cuda_error(e, name);
  }
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kCqThreads, smem);
  // persistent: as many CTAs as fit at once, each taking systems grid-stride
  const int grid = std::max(1, std::min(batch, std::max(1, per_sm) * std::max(1, nsm)));
  kern<<<grid, kCqThreads, smem, stream>>>(n, nrhs, A, strideA, diag, jpiv, B, strideB, info, batch, mode);
  return check_launch(name);
}

}  // namespace

// qr_ls.cu: the compact-WY Householder kernel on a uniform batch
int qr_uniform_launch(int n, int count, double* A, int64_t strideA, double* diag, double* B, int64_t strideB,
                      int32_t* info, cudaStream_t s, const char* name);

}  // namespace nacu

using namespace nacu;

extern "C" {

int nacu_dcolpivqr_batched(int n, int nrhs, double* A, int64_t strideA, double* diag, int32_t* jpiv, double* B,
                           int64_t strideB, int32_t* info, int batch, int flags, nacu_stream_t stream) {
  const char* name = "nacu_dcolpivqr_batched";
  if (n < 0 || n > kCqMaxN) return record_arg_error(-1, "col-pivot QR batched: n out of range [0, 128]");
  if (nrhs < 0 || nrhs > kCqMaxRhs) return record_arg_error(-2, "col-pivot QR batched: nrhs out of range [0, 16]");
  if (batch < 0) return record_arg_error(-10, "col-pivot QR batched: negative batch");
  if (batch == 0 || n == 0) return NACU_SUCCESS;
  if (!A || !diag || !jpiv || (nrhs > 0 && !B)) return record_arg_error(-3, "col-pivot QR batched: null pointer");
  if (strideA < (int64_t)n * n) return record_arg_error(-4, "col-pivot QR batched: strideA < n*n");
  if (nrhs > 0 && strideB < (int64_t)n * nrhs) return record_arg_error(-8, "col-pivot QR batched: strideB < n*nrhs");
  return colpivqr_launch(n, nrhs, A, strideA, diag, jpiv, B, strideB, info, batch, flags, nrhs > 0 ? 1 : 0,
                         (cudaStream_t)stream, name);
}

int nacu_dcolpivqr_solve_batched(int n, int nrhs, const double* QR, int64_t strideA, const double* diag,
                                 const int32_t* jpiv, double* B, int64_t strideB, int32_t* info, int batch, int flags,
                                 nacu_stream_t stream) {
  const char* name = "nacu_dcolpivqr_solve_batched";
  if (n < 0 || n > kCqMaxN) return record_arg_error(-1, "col-pivot QR solve: n out of range [0, 128]");
  if (nrhs < 0 || nrhs > kCqMaxRhs) return record_arg_error(-2, "col-pivot QR solve: nrhs out of range [0, 16]");
  if (batch < 0) return record_arg_error(-10, "col-pivot QR solve: negative batch");
  if (batch == 0 || n == 0 || nrhs == 0) return NACU_SUCCESS;
  if (!QR || !diag || !jpiv || !B) return record_arg_error(-3, "col-pivot QR solve: null pointer");
  if (strideA < (int64_t)n * n) return record_arg_error(-4, "col-pivot QR solve: strideA < n*n");
  if (strideB < (int64_t)n * nrhs) return record_arg_error(-8, "col-pivot QR solve: strideB < n*nrhs");
  // mode 2 reads the factors, diag and pivots and writes only B and info
  return colpivqr_launch(n, nrhs, const_cast<double*>(QR), strideA, const_cast<double*>(diag),
                         const_cast<int32_t*>(jpiv), B, strideB, info, batch, flags, 2, (cudaStream_t)stream, name);
}

int nacu_dqr_batched(int n, int nrhs, double* A, int64_t strideA, double* diag, double* B, int64_t strideB,
                     int32_t* info, int batch, int flags, nacu_stream_t stream) {
  const char* name = "nacu_dqr_batched";
  if (n < 0 || n > kCqMaxN) return record_arg_error(-1, "QR batched: n out of range [0, 128]");
  if (nrhs < 0 || nrhs > kCqMaxRhs) return record_arg_error(-2, "QR batched: nrhs out of range [0, 16]");
  if (batch < 0) return record_arg_error(-9, "QR batched: negative batch");
  if (batch == 0 || n == 0) return NACU_SUCCESS;
  if (!A || !diag || (nrhs > 0 && !B)) return record_arg_error(-3, "QR batched: null pointer");
  if (strideA < (int64_t)n * n) return record_arg_error(-4, "QR batched: strideA < n*n");
  if (nrhs > 0 && strideB < (int64_t)n * nrhs) return record_arg_error(-7, "QR batched: strideB < n*nrhs");
  // the FMA form with at most one right-hand side runs on the compact-WY
  // Householder kernel of the least-squares path (same stored layout and
  // signs); EXACT and more right-hand sides keep this kernel's steps
  if (!(flags & NACU_FLAG_EXACT) && nrhs <= 1)
    return qr_uniform_launch(n, batch, A, strideA, diag, nrhs == 1 ? B : nullptr, strideB, info,
                             (cudaStream_t)stream, name);
  return colpivqr_launch(n, nrhs, A, strideA, diag, nullptr, B, strideB, info, batch, flags, nrhs > 0 ? 1 : 0,
                         (cudaStream_t)stream, name, false);
}

int nacu_dqr_solve_batched(int n, int nrhs, const double* QR, int64_t strideA, const double* diag, double* B,
                           int64_t strideB, int32_t* info, int batch, int flags, nacu_stream_t stream) {
  const char* name = "nacu_dqr_solve_batched";
  if (n < 0 || n > kCqMaxN) return record_arg_error(-1, "QR solve: n out of range [0, 128]");
  if (nrhs < 0 || nrhs > kCqMaxRhs) return record_arg_error(-2, "QR solve: nrhs out of range [0, 16]");
  if (batch < 0) return record_arg_error(-9, "QR solve: negative batch");
  if (batch == 0 || n == 0 || nrhs == 0) return NACU_SUCCESS;
  if (!QR || !diag || !B) return record_arg_error(-3, "QR solve: null pointer");
  if (strideA < (int64_t)n * n) return record_arg_error(-4, "QR solve: strideA < n*n");
  if (strideB < (int64_t)n * nrhs) return record_arg_error(-7, "QR solve: strideB < n*nrhs");
  return colpivqr_launch(n, nrhs, const_cast<double*>(QR), strideA, const_cast<double*>(diag), nullptr, B, strideB,
                         info, batch, flags, 2, (cudaStream_t)stream, name, false);
}

}  // extern "C"
