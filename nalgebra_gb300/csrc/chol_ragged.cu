// Ragged batched Cholesky factor + solve + log-determinant: the GPU form of
// nalgebra's `m.cholesky()` then `.solve(&b)` and `.ln_determinant()` over
// thousands of SPD matrices of uneven order, in ONE persistent launch.
//
// Follows src/linalg/cholesky.rs:221-272 (Cholesky::new_internal, left-looking,
// lower triangle only, upper triangle left untouched), cholesky.rs:122-143
// (solve_mut: src/linalg/solve.rs:488-519 forward in axpy form, then
// solve.rs:697-712/732-755 adjoint back solve in dot form) and
// cholesky.rs:172-185 (ln_determinant = sum ln(L_ii^2)).
//
// Design (GB300): the FP64 pipe (~1 TFLOP/s) binds, HBM does not.  Each CTA
// factors one matrix at a time, pulling matrix indices from a device work queue
// ordered largest-first (so the short tail is made of small matrices).  The
// factorization is left-looking by NB-column panels: the panel lives in shared
// memory, the update by all earlier columns is a register-tiled product whose
// operands stream from L1/L2 (the matrix was just written by this CTA and is
// hot), and the panel itself is factored in shared memory with the trailing
// panel update spread evenly over all threads.  Every element still receives
// its updates in nalgebra's order (k = 0, 1, ..., j-1), so with EXACT the
// factor is bit-identical to nalgebra's.  The triangular solves are blocked by
// 32 rows: one warp solves each diagonal block out of registers with shuffles,
// the whole CTA applies the block to the remaining rows.
#include "common.cuh"

namespace nacu {
namespace {

constexpr int kCholThreads = 128;
constexpr int kNB = 16;        // panel width
constexpr int kRhsChunk = 4;   // right-hand sides per register pass
constexpr int kRowsPerPass = 256;  // rows of the panel update held in registers per pass

struct CholArgs {
  int count;
  int n_max;
  const int32_t* ns;
  const int64_t* aoff;
  double* A;
  int nrhs;
  const int64_t* boff;
  double* B;
  int32_t* info;
  double* logdet;
  const int32_t* order;
  int32_t* counter;
  int has_subst;
  double subst;
  int do_factor;  // 0: A already holds the factor (solve only)
};

// Pivot of column j (cholesky.rs:237-268): re <= 0 -> None, else try_sqrt
// (x >= 0), NaN fails; the substitute is tried the same way.  EXACT computes the
// correctly rounded sqrt and 1/sqrt as two operations; the FMA form derives
// both from one reciprocal square root (one dependent FP64 chain instead of
// two: on this part every dependent FP64 step costs tens of cycles).
template <bool EXACT>
__device__ __forceinline__ bool chol_pivot(double d, int has_subst, double subst, double* denom, double* rcp) {
  double v;
  if (!(d <= 0.0) && d >= 0.0) v = d;
  else if (has_subst && !(subst <= 0.0) && subst >= 0.0) v = subst;
  else return false;
  if constexpr (EXACT) {
    *denom = sqrt(v);
    *rcp = 1.0 / *denom;
  } else {
    const double r = rsqrt(v);
    *rcp = r;
    *denom = v * r;
  }
  return true;
}

// Factor one n x n matrix (column-major, lda = n, global memory, in place).
// Leaves info (0 ok, j+1 first failing pivot) in *s_info and, in the FMA form,
// 1/L_ii in rdiag[i] for the solves.
template <bool EXACT>
__device__ void chol_factor_cta(int n, double* __restrict__ a, int ldp, double* __restrict__ P, double* rdiag,
                                int* s_info, double* s_scal, int has_subst, double subst) {
  const int tid = threadIdx.x;
  const int nthr = blockDim.x;
  const int warp = tid >> 5, lane = tid & 31;
  for (int J0 = 0; J0 < n; J0 += kNB) {
    const int jb = min(kNB, n - J0);
    const int rows = n - J0;
    // Phase 1+2: P = A[J0.., J0..J0+jb] - L[J0.., 0..J0] * L[J0..J0+jb, 0..J0]^T
    // (lower part).  Warp w owns columns 4w..4w+3, lanes own rows lane + 32q;
    // each element still takes its updates in order k = 0, 1, ..., J0-1.
    for (int cg = warp * 4; cg < jb; cg += (nthr >> 5) * 4) {
      for (int rb = 0; rb < rows; rb += kRowsPerPass) {
        const int qmax = min(8, (rows - rb + 31) >> 5);
        double acc[8][4];
#pragma unroll
        for (int q = 0; q < 8; ++q)
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            const int r = rb + lane + 32 * q, c = cg + j;
            acc[q][j] = (q < qmax && r < rows && c < jb && r >= c) ? a[(size_t)(J0 + c) * n + J0 + r] : 0.0;
          }
        const double* colk = a + J0;
#pragma unroll 2
        for (int k = 0; k < J0; ++k, colk += n) {
          // L[c][k]; the negation is folded into the FMA operand (a select of
          // -x would cost one FP64 instruction per load).
          double lc[4];
#pragma unroll
          for (int j = 0; j < 4; ++j) lc[j] = (cg + j < jb) ? colk[cg + j] : 0.0;
#pragma unroll
          for (int q = 0; q < 8; ++q) {
            if (q < qmax) {
              const int r = rb + lane + 32 * q;
              const double lr = (r < rows) ? colk[r] : 0.0;
#pragma unroll
              for (int j = 0; j < 4; ++j) acc[q][j] = axpy1<EXACT>(acc[q][j], -lc[j], lr);
            }
          }
        }
#pragma unroll
        for (int q = 0; q < 8; ++q)
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            const int r = rb + lane + 32 * q, c = cg + j;
            if (q < qmax && r < rows && c < jb && r >= c) P[(size_t)c * ldp + r] = acc[q][j];
          }
      }
    }
    __syncthreads();
    // Phase 3: factor the panel in shared memory, right-looking inside the panel
    // (the same per-element update order).  Thread 0 owns every diagonal
    // element of the trailing update (flattened index 0), so it computes the
    // next pivot right after its own update: two barriers per column.
    if (tid == 0) {
      double denom, rcp;
      if (chol_pivot<EXACT>(P[0], has_subst, subst, &denom, &rcp)) {
        P[0] = denom;
        s_scal[0] = denom;
        s_scal[1] = rcp;
        rdiag[J0] = rcp;
      } else {
        *s_info = J0 + 1;
      }
    }
    __syncthreads();
    for (int j = 0; j < jb; ++j) {
      if (*s_info != 0) return;
      double* pj = P + (size_t)j * ldp;
      const double denom = s_scal[0], rcp = s_scal[1];
      for (int r = j + 1 + tid; r < rows; r += nthr) {
        if constexpr (EXACT) pj[r] = pj[r] / denom;  // cholesky.rs:261-262 (col /= denom)
        else pj[r] = pj[r] * rcp;
      }
      __syncthreads();
      const int m = rows - j - 1;  // rows j+1..rows-1
      const int w = jb - j - 1;    // columns j+1..jb-1
      if (w > 0) {
        const int total = m * w;
        int e = tid;
        int cq = e / m, rr = e - cq * m;
        const int dq = nthr / m, dr = nthr - dq * m;
        for (; e < total; e += nthr) {
          const int c = j + 1 + cq, r = j + 1 + rr;
          if (r >= c) {
            double* pc = P + (size_t)c * ldp;
            pc[r] = axpy1<EXACT>(pc[r], -pj[c], pj[r]);
          }
          rr += dr;
          cq += dq;
          if (rr >= m) {
            rr -= m;
            ++cq;
          }
        }
        if (tid == 0) {  // element (j+1, j+1) was this thread's first update
          double* pn = P + (size_t)(j + 1) * ldp + (j + 1);
          double dn, rn;
          if (chol_pivot<EXACT>(*pn, has_subst, subst, &dn, &rn)) {
            *pn = dn;
            s_scal[0] = dn;
            s_scal[1] = rn;
            rdiag[J0 + j + 1] = rn;
          } else {
            *s_info = J0 + j + 2;
          }
        }
      }
      __syncthreads();
    }
    if (*s_info != 0) return;
    // Phase 4: write the finished panel back (lower part; the strict upper
    // triangle of the diagonal block was never modified).
    for (int e = tid; e < rows * jb; e += nthr) {
      const int c = e / rows, r = e - c * rows;
      if (r >= c) a[(size_t)(J0 + c) * n + J0 + r] = P[(size_t)c * ldp + r];
    }
    __syncthreads();
  }
}

// Forward solve L y = b (axpy form) for up to kRhsChunk columns of X (shared,
// column-major ldx), blocked by 32 rows.
template <bool EXACT>
__device__ void chol_forward_cta(int n, const double* __restrict__ a, double* X, int ldx, int nr,
                                 const double* rdiag) {
  const int tid = threadIdx.x, nthr = blockDim.x;
  const int warp = tid >> 5, lane = tid & 31;
  for (int I0 = 0; I0 < n; I0 += 32) {
    const int ib = min(32, n - I0);
    if (warp == 0) {
      double lrow[32];
      double b[kRhsChunk];
#pragma unroll
      for (int i = 0; i < 32; ++i) lrow[i] = (lane < ib && i <= lane) ? a[(size_t)(I0 + i) * n + I0 + lane] : 0.0;
#pragma unroll
      for (int c = 0; c < kRhsChunk; ++c) b[c] = (lane < ib && c < nr) ? X[(size_t)c * ldx + I0 + lane] : 0.0;
      const double rd = (lane < ib) ? rdiag[I0 + lane] : 0.0;
#pragma unroll
      for (int i = 0; i < 32; ++i) {
        if (i < ib) {
#pragma unroll
          for (int c = 0; c < kRhsChunk; ++c) {
            if (lane == i) {
              if constexpr (EXACT) b[c] = b[c] / lrow[i];  // solve.rs:509: b_i / L_ii
              else b[c] = b[c] * rd;
            }
            const double y = __shfl_sync(0xffffffffu, b[c], i);
            if (lane > i) b[c] = axpy1<EXACT>(b[c], -y, lrow[i]);
          }
        }
      }
#pragma unroll
      for (int c = 0; c < kRhsChunk; ++c)
        if (lane < ib && c < nr) X[(size_t)c * ldx + I0 + lane] = b[c];
    }
    __syncthreads();
    // Rows below the block: b_r -= sum_i L[r][I0+i] y_i, one thread per row
    // for all right-hand sides (one L load feeds kRhsChunk FMAs), i ascending.
    for (int r = I0 + ib + tid; r < n; r += nthr) {
      double v[kRhsChunk];
#pragma unroll
      for (int c = 0; c < kRhsChunk; ++c) v[c] = (c < nr) ? X[(size_t)c * ldx + r] : 0.0;
      const double* lp = a + (size_t)I0 * n + r;
      for (int i = 0; i < ib; ++i, lp += n) {
        const double l = *lp;
#pragma unroll
        for (int c = 0; c < kRhsChunk; ++c) v[c] = axpy1<EXACT>(v[c], -X[(size_t)c * ldx + I0 + i], l);
      }
#pragma unroll
      for (int c = 0; c < kRhsChunk; ++c)
        if (c < nr) X[(size_t)c * ldx + r] = v[c];
    }
    __syncthreads();
  }
}

// Back solve L^T x = y, FMA form: blocked from the bottom, reductions over the
// rows below each 32-row block, then a warp solve of the transposed block.
__device__ void chol_backward_fast_cta(int n, const double* __restrict__ a, double* X, int ldx, int nr,
                                       const double* rdiag) {
  const int tid = threadIdx.x, nthr = blockDim.x;
  const int warp = tid >> 5, lane = tid & 31, nwarps = nthr >> 5;
  const int nblocks = (n + 31) / 32;
  for (int bI = nblocks - 1; bI >= 0; --bI) {
    const int I0 = bI * 32;
    const int ib = min(32, n - I0);
    const int r0 = I0 + ib;
    if (r0 < n) {
      // y_i -= sum_{r >= r0} L[r][i] x_r for the block's columns i: warp w owns
      // 4 columns at a time; each lane accumulates 4 columns x 4 rhs over rows
      // r = r0+lane, r0+lane+32, ... (coalesced column loads), then a butterfly
      // reduce-scatter leaves sum k = lane & 15 in lane `lane` (16 adds per lane
      // instead of 16 separate 5-step warp reductions).
      for (int cb = warp * 4; cb < ib; cb += nwarps * 4) {
        double v[16];
#pragma unroll
        for (int k = 0; k < 16; ++k) v[k] = 0.0;
        for (int r = r0 + lane; r < n; r += 32) {
          double xr[4];
#pragma unroll
          for (int c = 0; c < 4; ++c) xr[c] = (c < nr) ? X[(size_t)c * ldx + r] : 0.0;
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            const double l = (cb + j < ib) ? a[(size_t)(I0 + cb + j) * n + r] : 0.0;
#pragma unroll
            for (int c = 0; c < 4; ++c) v[j * 4 + c] = fma(l, xr[c], v[j * 4 + c]);
          }
        }
#pragma unroll
        for (int half = 8; half >= 1; half >>= 1) {
          const bool up = (lane & half) != 0;
#pragma unroll
          for (int t = 0; t < half; ++t) {
            const double keep = up ? v[t + half] : v[t];
            const double give = up ? v[t] : v[t + half];
            v[t] = keep + __shfl_xor_sync(0xffffffffu, give, half);
          }
        }
        v[0] += __shfl_xor_sync(0xffffffffu, v[0], 16);
        const int j = (lane & 15) >> 2, c = lane & 3;
        if (lane < 16 && cb + j < ib && c < nr) X[(size_t)c * ldx + I0 + cb + j] -= v[0];
      }
      __syncthreads();
    }
    if (warp == 0) {
      double lcol[32];  // lane j holds column j of the diagonal block
#pragma unroll
      for (int i = 0; i < 32; ++i) lcol[i] = (lane < ib && i < ib && i >= lane) ? a[(size_t)(I0 + lane) * n + I0 + i] : 0.0;
      const double rd = (lane < ib) ? rdiag[I0 + lane] : 0.0;
      for (int c = 0; c < nr; ++c) {
        double y = (lane < ib) ? X[(size_t)c * ldx + I0 + lane] : 0.0;
#pragma unroll
        for (int i = 31; i >= 0; --i) {
          if (i < ib) {
            if (lane == i) y = y * rd;
            const double xi = __shfl_sync(0xffffffffu, y, i);
            if (lane < i) y = fma(-xi, lcol[i], y);
          }
        }
        if (lane < ib) X[(size_t)c * ldx + I0 + lane] = y;
      }
    }
    __syncthreads();
  }
}

// Back solve L^T x = y in nalgebra's exact order (solve.rs:732-755): for i from
// n-1 down, x_i = (y_i - dot(L[i+1.., i], x[i+1..])) / L_ii with the
// 8-accumulator dot of src/base/blas.rs:96-165.  One warp, 8 lanes per rhs.
__device__ void chol_backward_exact_cta(int n, const double* __restrict__ a, double* X, int ldx, int nr) {
  const int tid = threadIdx.x;
  if (tid < 32) {
    const int lane = tid, c = lane >> 3, k = lane & 7;
    const unsigned grp = 0xffu << (c * 8);
    double* xc = X + (size_t)(c < nr ? c : 0) * ldx;
    for (int i = n - 1; i >= 0; --i) {
      const int len = n - i - 1;
      const double* li = a + (size_t)i * n + i + 1;
      const double* xv = xc + i + 1;
      const int nb = len >> 3;
      double acc = 0.0;
      for (int b = 0; b < nb; ++b) acc = __dadd_rn(acc, __dmul_rn(li[8 * b + k], xv[8 * b + k]));
      // res += acc0 + acc4; res += acc1 + acc5; res += acc2 + acc6; res += acc3 + acc7
      const double hi = __shfl_down_sync(0xffffffffu, acc, 4, 8);
      double res = 0.0;
      double pair = __dadd_rn(acc, hi);  // valid on k < 4
      const double p0 = __shfl_sync(0xffffffffu, pair, 0, 8);
      const double p1 = __shfl_sync(0xffffffffu, pair, 1, 8);
      const double p2 = __shfl_sync(0xffffffffu, pair, 2, 8);
      const double p3 = __shfl_sync(0xffffffffu, pair, 3, 8);
      if (k == 0 && c < nr) {
        res = __dadd_rn(res, p0);
        res = __dadd_rn(res, p1);
        res = __dadd_rn(res, p2);
        res = __dadd_rn(res, p3);
        for (int t = 8 * nb; t < len; ++t) res = __dadd_rn(res, __dmul_rn(li[t], xv[t]));
        xc[i] = __ddiv_rn(__dsub_rn(xc[i], res), a[(size_t)i * n + i]);
      }
      (void)grp;
      __syncwarp();
    }
  }
  __syncthreads();
}

template <bool EXACT>
__device__ void chol_solve_one(const CholArgs& g, int s, double* P, double* X, int* s_info, double* s_scal) {
  const int tid = threadIdx.x;
  const int n = g.ns ? g.ns[s] : g.n_max;
  if (n < 0 || n > g.n_max) {
    if (tid == 0) {
      if (g.info) g.info[s] = -1;
      if (g.logdet) g.logdet[s] = __longlong_as_double(0x7ff8000000000000ll);
    }
    return;
  }
  double* a = g.A + (g.aoff ? g.aoff[s] : 0);
  if (tid == 0) *s_info = 0;
  __syncthreads();
  const int ldp = g.n_max | 1;
  double* rdiag = X + (size_t)ldp * kRhsChunk;
  if (g.do_factor) {
    chol_factor_cta<EXACT>(n, a, ldp, P, rdiag, s_info, s_scal, g.has_subst, g.subst);
  } else if (!EXACT) {
    for (int i = tid; i < n; i += blockDim.x) rdiag[i] = 1.0 / a[(size_t)i * n + i];
    __syncthreads();
  }
  const int inf = *s_info;
  if (inf == 0) {
    if (g.nrhs > 0 && g.B) {
      double* b = g.B + (g.boff ? g.boff[s] : 0);
      const int ldx = ldp;
      for (int c0 = 0; c0 < g.nrhs; c0 += kRhsChunk) {
        const int nr = min(kRhsChunk, g.nrhs - c0);
        for (int e = tid; e < n * nr; e += blockDim.x) {
          const int c = e / n, r = e - c * n;
          X[(size_t)c * ldx + r] = b[(size_t)(c0 + c) * n + r];
        }
        __syncthreads();
        chol_forward_cta<EXACT>(n, a, X, ldx, nr, rdiag);
        if constexpr (EXACT) chol_backward_exact_cta(n, a, X, ldx, nr);
        else chol_backward_fast_cta(n, a, X, ldx, nr, rdiag);
        for (int e = tid; e < n * nr; e += blockDim.x) {
          const int c = e / n, r = e - c * n;
          b[(size_t)(c0 + c) * n + r] = X[(size_t)c * ldx + r];
        }
        __syncthreads();
      }
    }
    if (g.logdet) {
      if constexpr (EXACT) {
        if (tid == 0) {
          double sum = 0.0;
          for (int i = 0; i < n; ++i) {
            const double d = a[(size_t)i * n + i];
            sum = __dadd_rn(sum, log(__dmul_rn(d, d)));
          }
          g.logdet[s] = sum;
        }
      } else {
        double part = 0.0;
        for (int i = tid; i < n; i += blockDim.x) {
          const double d = a[(size_t)i * n + i];
          part += log(d * d);
        }
        part = warp_sum(part);
        if ((tid & 31) == 0) s_scal[2 + (tid >> 5)] = part;
        __syncthreads();
        if (tid == 0) {
          double sum = 0.0;
          for (int w = 0; w < (int)(blockDim.x >> 5); ++w) sum += s_scal[2 + w];
          g.logdet[s] = sum;
        }
      }
    }
  } else if (tid == 0 && g.logdet) {
    g.logdet[s] = __longlong_as_double(0x7ff8000000000000ll);
  }
  if (tid == 0 && g.info) g.info[s] = inf;
  __syncthreads();
}

template <bool EXACT>
__global__ void __launch_bounds__(kCholThreads, 4) chol_ragged_kernel(CholArgs g) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_item;
  __shared__ int s_info;
  __shared__ double s_scal[2 + kCholThreads / 32];
  const int ldp = g.n_max | 1;
  double* P = reinterpret_cast<double*>(smem_raw);
  double* X = P + (size_t)ldp * kNB;
  for (;;) {
    if (threadIdx.x == 0) s_item = g.counter ? atomicAdd(g.counter, 1) : 0;
    __syncthreads();
    const int idx = s_item;
    __syncthreads();
    if (idx >= g.count) break;
    const int s = g.order ? g.order[idx] : idx;
    chol_solve_one<EXACT>(g, s, P, X, &s_info, s_scal);
    if (!g.counter) break;  // single-matrix launch
  }
}

size_t chol_smem_bytes(int n_max) {
  const int ldp = n_max | 1;
  return (size_t)ldp * (kNB + kRhsChunk + 1) * sizeof(double);
}

int chol_launch(CholArgs g, int flags, cudaStream_t stream, bool persistent, const char* name) {
  const bool exact = (flags & NACU_FLAG_EXACT) != 0;
  auto kern = exact ? chol_ragged_kernel<true> : chol_ragged_kernel<false>;
  const size_t smem = chol_smem_bytes(g.n_max);
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return record_cuda_error(e, name);
  int grid = 1;
  if (persistent) {
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kCholThreads, smem);
    if (e != cudaSuccess) return record_cuda_error(e, name);
    if (per_sm < 1) per_sm = 1;
    grid = sm_count() * per_sm;
    if (grid > g.count) grid = g.count;
    e = cudaMemsetAsync(g.counter, 0, sizeof(int32_t), stream);
    if (e != cudaSuccess) return record_cuda_error(e, name);
  }
  kern<<<grid, kCholThreads, smem, stream>>>(g);
  return check_launch(name);
}

}  // namespace
}  // namespace nacu

extern "C" {

size_t nacu_ragged_workspace_bytes(int count) {
  (void)count;
  return 256;  // the work-queue head (one int32, padded)
}

static int ragged_args(int count, int n_max, const int32_t* ns, const int64_t* a_offsets, double* A,
                       void* workspace, size_t workspace_bytes, const char* name) {
  using namespace nacu;
  (void)name;
  if (count < 0) return record_arg_error(-1, "ragged Cholesky: negative count");
  if (n_max < 0 || n_max > NACU_CHOL_RAGGED_MAX_N)
    return record_arg_error(-2, "ragged Cholesky: n_max out of range [0, 512]");
  if (count == 0) return 1;
  if (!ns || !a_offsets || !A) return record_arg_error(-3, "ragged Cholesky: null ns, a_offsets or A");
  if (!workspace || workspace_bytes < nacu_ragged_workspace_bytes(count))
    return record_arg_error(-12, "ragged Cholesky: workspace too small");
  return 0;
}

int nacu_dposv_ragged(int count, int n_max, const int32_t* ns, const int64_t* a_offsets, double* A, int nrhs,
                      const int64_t* b_offsets, double* B, int32_t* info, double* logdet, const int32_t* order,
                      void* workspace, size_t workspace_bytes, double substitute, int flags,
                      nacu_stream_t stream) {
  using namespace nacu;
  int rc = ragged_args(count, n_max, ns, a_offsets, A, workspace, workspace_bytes, "nacu_dposv_ragged");
  if (rc != 0) return rc > 0 ? NACU_SUCCESS : rc;
  if (nrhs < 0) return record_arg_error(-6, "dposv_ragged: negative nrhs");
  if (nrhs > 0 && (!b_offsets || !B)) return record_arg_error(-7, "dposv_ragged: null b_offsets or B");
  if (!info) return record_arg_error(-9, "dposv_ragged: null info");
  CholArgs g{count, n_max, ns, a_offsets, A, nrhs, b_offsets, B, info, logdet, order,
             reinterpret_cast<int32_t*>(workspace), (flags & NACU_FLAG_SUBSTITUTE) ? 1 : 0, substitute, 1};
  return chol_launch(g, flags, (cudaStream_t)stream, true, "nacu_dposv_ragged");
}

int nacu_dpotrf_ragged(int count, int n_max, const int32_t* ns, const int64_t* a_offsets, double* A,
                       int32_t* info, double* logdet, const int32_t* order, void* workspace,
                       size_t workspace_bytes, double substitute, int flags, nacu_stream_t stream) {
  using namespace nacu;
  int rc = ragged_args(count, n_max, ns, a_offsets, A, workspace, workspace_bytes, "nacu_dpotrf_ragged");
  if (rc != 0) return rc > 0 ? NACU_SUCCESS : rc;
  if (!info) return record_arg_error(-6, "dpotrf_ragged: null info");
  CholArgs g{count, n_max, ns, a_offsets, A, 0, nullptr, nullptr, info, logdet, order,
             reinterpret_cast<int32_t*>(workspace), (flags & NACU_FLAG_SUBSTITUTE) ? 1 : 0, substitute, 1};
  return chol_launch(g, flags, (cudaStream_t)stream, true, "nacu_dpotrf_ragged");
}

int nacu_dpotrs_ragged(int count, int n_max, const int32_t* ns, const int64_t* a_offsets, const double* L,
                       int nrhs, const int64_t* b_offsets, double* B, const int32_t* order, void* workspace,
                       size_t workspace_bytes, int flags, nacu_stream_t stream) {
  using namespace nacu;
  int rc = ragged_args(count, n_max, ns, a_offsets, const_cast<double*>(L), workspace, workspace_bytes,
                       "nacu_dpotrs_ragged");
  if (rc != 0) return rc > 0 ? NACU_SUCCESS : rc;
  if (nrhs < 0) return record_arg_error(-6, "dpotrs_ragged: negative nrhs");
  if (nrhs == 0) return NACU_SUCCESS;
  if (!b_offsets || !B) return record_arg_error(-7, "dpotrs_ragged: null b_offsets or B");
  CholArgs g{count, n_max, ns, a_offsets, const_cast<double*>(L), nrhs, b_offsets, B, nullptr, nullptr, order,
             reinterpret_cast<int32_t*>(workspace), 0, 0.0, 0};
  return chol_launch(g, flags, (cudaStream_t)stream, true, "nacu_dpotrs_ragged");
}

int nacu_dposv(int n, double* A, int nrhs, double* B, int32_t* info, double* logdet, double substitute,
               int flags, nacu_stream_t stream) {
  using namespace nacu;
  if (n < 0 || n > NACU_CHOL_RAGGED_MAX_N) return record_arg_error(-1, "dposv: n out of range [0, 512]");
  if (n == 0) return NACU_SUCCESS;
  if (!A) return record_arg_error(-2, "dposv: null A");
  if (nrhs < 0) return record_arg_error(-3, "dposv: negative nrhs");
  if (nrhs > 0 && !B) return record_arg_error(-4, "dposv: null B");
  if (!info) return record_arg_error(-5, "dposv: null info");
  // One matrix, one CTA: the plain per-matrix launch (no work queue).
  CholArgs g{1, n, nullptr, nullptr, A, nrhs, nullptr, B, info, logdet, nullptr, nullptr,
             (flags & NACU_FLAG_SUBSTITUTE) ? 1 : 0, substitute, 1};
  return chol_launch(g, flags, (cudaStream_t)stream, false, "nacu_dposv");
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Allocation-free variant of nacu_dposv_ragged.
//
// Some callers cannot allocate device memory at the point where they solve:
// code running inside a custom allocator or memory-pool callback, real-time or
// safety-certified hosts that forbid allocation after start-up, and plugins
// whose host framework owns every device allocation and hands out no scratch.
// For them this entry point keeps its scratch -- the work-queue head and the
// largest-first processing order -- in a fixed array in the library's own
// device memory (loaded with the module; every GPU that loads the library
// holds it until the process exits).  The caller still passes all inputs and
// outputs.  Calls share that one array, so two calls that overlap on the GPU
// (different streams, no ordering between them) race on it; order such calls.
// ---------------------------------------------------------------------------
namespace nacu {
namespace {

constexpr int kNoAllocMaxCount = NACU_RAGGED_NOALLOC_MAX_COUNT;

// [0]: work-queue head; [1 .. count]: processing order.
static __device__ __align__(256) int32_t g_ragged_noalloc_scratch[1 + kNoAllocMaxCount];

int32_t* g_noalloc_scratch_ptr[64] = {nullptr};

// Builds the largest-first order (a counting sort on n, one CTA) into the
// scratch and clears the queue head, so every call starts from zero.
__global__ void __launch_bounds__(1024) ragged_order_kernel(int count, int n_max, const int32_t* __restrict__ ns,
                                                            int32_t* __restrict__ scratch) {
  __shared__ int hist[NACU_CHOL_RAGGED_MAX_N + 2];
  const int nb = n_max + 1;
  for (int i = threadIdx.x; i <= nb; i += blockDim.x) hist[i] = 0;
  __syncthreads();
  for (int s = threadIdx.x; s < count; s += blockDim.x) {
    int n = ns[s];
    n = (n < 0 || n > n_max) ? 0 : n;  // out-of-range orders still get a slot (info = -1 later)
    atomicAdd(&hist[n], 1);
  }
  __syncthreads();
  if (threadIdx.x == 0) {  // exclusive prefix sum over n, largest n first
    int run = 0;
    for (int n = n_max; n >= 0; --n) {
      const int h = hist[n];
      hist[n] = run;
      run += h;
    }
    scratch[0] = 0;
  }
  __syncthreads();
  for (int s = threadIdx.x; s < count; s += blockDim.x) {
    int n = ns[s];
    n = (n < 0 || n > n_max) ? 0 : n;
    scratch[1 + atomicAdd(&hist[n], 1)] = s;
  }
}

// Device address of the scratch array for the current device, looked up once
// per device (the array's host-side name is not a device address).
int noalloc_scratch(int32_t** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return record_cuda_error(e, "nacu_dposv_ragged_noalloc: cudaGetDevice");
  if (dev < 0 || dev >= 64) return record_arg_error(-99, "nacu_dposv_ragged_noalloc: device index >= 64");
  if (g_noalloc_scratch_ptr[dev] == nullptr) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_ragged_noalloc_scratch);
    if (e != cudaSuccess) return record_cuda_error(e, "nacu_dposv_ragged_noalloc: cudaGetSymbolAddress");
    g_noalloc_scratch_ptr[dev] = static_cast<int32_t*>(p);
  }
  *out = g_noalloc_scratch_ptr[dev];
  return NACU_SUCCESS;
}

}  // namespace
}  // namespace nacu

extern "C" int nacu_dposv_ragged_noalloc(int count, int n_max, const int32_t* ns, const int64_t* a_offsets,
                                         double* A, int nrhs, const int64_t* b_offsets, double* B, int32_t* info,
                                         double* logdet, double substitute, int flags, nacu_stream_t stream) {
  using namespace nacu;
  if (count < 0) return record_arg_error(-1, "dposv_ragged_noalloc: negative count");
  if (count > kNoAllocMaxCount)
    return record_arg_error(-1, "dposv_ragged_noalloc: count exceeds NACU_RAGGED_NOALLOC_MAX_COUNT (65536); "
                                "use nacu_dposv_ragged with a caller workspace or split the batch");
  if (n_max < 0 || n_max > NACU_CHOL_RAGGED_MAX_N)
    return record_arg_error(-2, "dposv_ragged_noalloc: n_max out of range [0, 512]");
  if (count == 0) return NACU_SUCCESS;
  if (!ns || !a_offsets || !A) return record_arg_error(-3, "dposv_ragged_noalloc: null ns, a_offsets or A");
  if (nrhs < 0) return record_arg_error(-6, "dposv_ragged_noalloc: negative nrhs");
  if (nrhs > 0 && (!b_offsets || !B)) return record_arg_error(-7, "dposv_ragged_noalloc: null b_offsets or B");
  if (!info) return record_arg_error(-9, "dposv_ragged_noalloc: null info");
  int32_t* scratch = nullptr;
  int rc = noalloc_scratch(&scratch);
  if (rc != NACU_SUCCESS) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  ragged_order_kernel<<<1, 1024, 0, s>>>(count, n_max, ns, scratch);
  rc = check_launch("nacu_dposv_ragged_noalloc: order");
  if (rc != NACU_SUCCESS) return rc;
  CholArgs g{count, n_max, ns, a_offsets, A, nrhs, b_offsets, B, info, logdet, scratch + 1, scratch,
             (flags & NACU_FLAG_SUBSTITUTE) ? 1 : 0, substitute, 1};
  // The queue head was cleared by the order kernel (same stream, in order).
  const bool exact = (flags & NACU_FLAG_EXACT) != 0;
  auto kern = exact ? chol_ragged_kernel<true> : chol_ragged_kernel<false>;
  const size_t smem = chol_smem_bytes(g.n_max);
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return record_cuda_error(e, "nacu_dposv_ragged_noalloc");
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kCholThreads, smem);
  if (e != cudaSuccess) return record_cuda_error(e, "nacu_dposv_ragged_noalloc");
  if (per_sm < 1) per_sm = 1;
  int grid = sm_count() * per_sm;
  if (grid > count) grid = count;
  kern<<<grid, kCholThreads, smem, s>>>(g);
  return check_launch("nacu_dposv_ragged_noalloc");
}
