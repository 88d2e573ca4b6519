// Large dense LU with partial pivoting (one matrix, n up to tens of
// thousands) and its solve, in FP64 (the plain form of nalgebra's `m.lu()` /
// `.solve(&b)`, src/linalg/lu.rs:93-122, 221-260) and in FP32 (the factor of
// the mixed-precision form, see gesv_mixed.cu).
//
// Blocked right-looking LU, panels of NB columns:
//   1. panel factorization, partial pivoting with nalgebra's icamax rule
//      (largest |x|, first index on ties, src/base/min_max.rs:221-240; an
//      all-zero column is skipped, lu.rs:107-110), by one cooperative kernel
//      whose CTAs own row blocks of the panel and meet at two grid barriers per
//      column (candidate pivots published; pivot row swapped);
//   2. the panel's row swaps applied to the columns left and right of it;
//   3. U12 = L11^-1 A12 (unit lower triangular solve, one thread per column);
//   4. A22 -= L21 U12 by the GEMM kernels (FP64 DFMA, or the BF16-split
//      tensor-core GEMM for the FP32 factor).
// The triangular solves for the right-hand side run as one cooperative kernel
// per triangle: the diagonal block of each step is solved by CTA 0 while all
// CTAs then apply it to the remaining rows (coalesced GEMV), one grid barrier
// per phase.
#include <cooperative_groups.h>

#include "common.cuh"

namespace cg = cooperative_groups;

namespace nacu {

// ---------------------------------------------------------------------------
// panel factorization (cooperative)
// ---------------------------------------------------------------------------
template <typename T>
struct PanelArgs {
  int n;        // matrix order
  T* A;         // column-major, lda
  int64_t lda;
  int j0, nb;   // panel columns [j0, j0 + nb)
  int32_t* ipiv;        // global per-step pivots (0-based rows)
  unsigned long long* cand;  // per-CTA candidate (key << 32 | ~row) for the current column
  int32_t* info;        // first zero pivot (1-based), atomicMin
};

constexpr int kPanelThreads = 256;

template <typename T>
__global__ void __launch_bounds__(kPanelThreads) lu_panel_coop_kernel(PanelArgs<T> g) {
  cg::grid_group grid = cg::this_grid();
  __shared__ uint64_t s_key[kPanelThreads / 32];
  __shared__ int s_idx[kPanelThreads / 32];
  __shared__ T s_prow[256];
  __shared__ int s_piv;
  __shared__ T s_inv;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int G = gridDim.x;
  const int n = g.n;
  T* A = g.A;
  const int64_t lda = g.lda;
  const int rows_total = n - g.j0;
  const int chunk = (rows_total + G - 1) / G;
  const int r_begin = g.j0 + blockIdx.x * chunk;
  const int r_end = min(n, r_begin + chunk);
  for (int j = 0; j < g.nb; ++j) {
    const int c = g.j0 + j;
    T* col = A + (size_t)c * lda;
    // 1. local icamax over my rows >= c (key = |x| bits; NaN only wins at row c)
    uint64_t key = 0;
    int idx = 0x7fffffff;
    for (int r = max(r_begin, c) + tid; r < r_end; r += kPanelThreads) {
      const uint64_t k = pivot_key(col[r], r == c);
      if (idx == 0x7fffffff || k > key) {
        key = k;
        idx = r;
      }
    }
    warp_argmax(key, idx);
    if (lane == 0) {
      s_key[warp] = key;
      s_idx[warp] = idx;
    }
    __syncthreads();
    if (tid == 0) {
      uint64_t bk = 0;
      int bi = 0x7fffffff;
      for (int w = 0; w < kPanelThreads / 32; ++w)
        if (s_idx[w] != 0x7fffffff && (bi == 0x7fffffff || s_key[w] > bk || (s_key[w] == bk && s_idx[w] < bi))) {
          bk = s_key[w];
          bi = s_idx[w];
        }
      g.cand[blockIdx.x] = (bi == 0x7fffffff) ? 0ull : bk;  // |x| key (NaN at row c: all ones)
      g.cand[G + blockIdx.x] = (unsigned long long)(long long)(bi == 0x7fffffff ? -1 : bi);
    }
    grid.sync();
    // 2. every CTA reduces the G candidates the same way; CTA 0 swaps rows
    if (tid == 0) {
      uint64_t bk = 0;
      int bi = -1;
      for (int b = 0; b < G; ++b) {
        const int ri = (int)(long long)g.cand[G + b];
        if (ri < 0) continue;
        const uint64_t kk = g.cand[b];
        if (bi < 0 || kk > bk || (kk == bk && ri < bi)) {
          bk = kk;
          bi = ri;
        }
      }
      s_piv = (bi < 0 || bk == 0) ? -1 : bi;  // key 0: |pivot| == 0, the column is skipped
    }
    __syncthreads();
    // decided from the candidates alone: no CTA reads the matrix while CTA 0 swaps
    const bool skip = (s_piv < 0);  // lu.rs:107-110
    const int piv = skip ? c : s_piv;
    if (blockIdx.x == 0) {
      if (!skip && piv != c)
        for (int cc = g.j0 + tid; cc < g.j0 + g.nb; cc += kPanelThreads) {
          T* p = A + (size_t)cc * lda;
          const T t = p[c];
          p[c] = p[piv];
          p[piv] = t;
        }
      if (tid == 0) {
        g.ipiv[c] = skip ? c : piv;
        if (skip) atomicMin(g.info, c + 1);
      }
    }
    grid.sync();
    if (skip) continue;
    // 3. scale my rows of column c and update my rows of the panel's
    //    remaining columns with the pivot row
    const int w = g.j0 + g.nb - c - 1;
    for (int t = tid; t < w; t += kPanelThreads) s_prow[t] = A[(size_t)(c + 1 + t) * lda + c];
    if (tid == 0) s_inv = T(1) / A[(size_t)c * lda + c];
    __syncthreads();
    const T inv = s_inv;
    for (int r = max(r_begin, c + 1) + tid; r < r_end; r += kPanelThreads) {
      const T l = col[r] * inv;
      col[r] = l;
      for (int t = 0; t < w; ++t) {
        T* p = A + (size_t)(c + 1 + t) * lda + r;
        *p = axpy1<false>(*p, -s_prow[t], l);
      }
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// row swaps of the panel applied to the other columns; unit-lower TRSM
// ---------------------------------------------------------------------------
template <typename T>
__global__ void lu_swap_kernel(int n, T* A, int64_t lda, const int32_t* ipiv, int j0, int nb) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n || (c >= j0 && c < j0 + nb)) return;
  T* col = A + (size_t)c * lda;
  for (int i = j0; i < j0 + nb; ++i) {
    const int p = ipiv[i];
    if (p != i) {
      const T t = col[i];
      col[i] = col[p];
      col[p] = t;
    }
  }
}

// U12 = L11^-1 A12 for columns j0+nb..n-1: L11 (nb x nb, unit lower) in
// shared memory, one thread per column, the column kept in shared memory.
template <typename T>
__global__ void __launch_bounds__(64) lu_trsm_kernel(int n, T* A, int64_t lda, int j0, int nb) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* L = reinterpret_cast<T*>(smem_raw);  // nb x nb
  T* X = L + (size_t)nb * nb;             // nb x 64 (column-major per thread)
  const int tid = threadIdx.x;
  for (int e = tid; e < nb * nb; e += blockDim.x) {
    const int cc = e / nb, r = e - cc * nb;
    L[e] = A[(size_t)(j0 + cc) * lda + j0 + r];
  }
  const int c = j0 + nb + blockIdx.x * 64 + tid;
  const bool valid = c < n;
  T* col = A + (size_t)(valid ? c : j0) * lda + j0;
  for (int i = 0; i < nb; ++i) X[(size_t)i * 64 + tid] = valid ? col[i] : T(0);
  __syncthreads();
  for (int i = 1; i < nb; ++i) {
    T x = X[(size_t)i * 64 + tid];
    for (int k = 0; k < i; ++k) x = axpy1<false>(x, -L[(size_t)k * nb + i], X[(size_t)k * 64 + tid]);
    X[(size_t)i * 64 + tid] = x;
  }
  if (valid)
    for (int i = 0; i < nb; ++i) col[i] = X[(size_t)i * 64 + tid];
}

// ---------------------------------------------------------------------------
// triangular solves for one right-hand side (cooperative)
// ---------------------------------------------------------------------------
constexpr int kTrsvBlock = 128;
constexpr int kTrsvThreads = 256;

// lower = true: x <- L^-1 x (unit diagonal); lower = false: x <- U^-1 x.
template <typename T>
__global__ void __launch_bounds__(kTrsvThreads) trsv_coop_kernel(int n, const T* __restrict__ A, int64_t lda, T* x,
                                                                 int lower, int32_t* info) {
  cg::grid_group grid = cg::this_grid();
  __shared__ T xs[kTrsvBlock];
  const int tid = threadIdx.x;
  const int nblk = (n + kTrsvBlock - 1) / kTrsvBlock;
  for (int s = 0; s < nblk; ++s) {
    const int b = lower ? s : nblk - 1 - s;
    const int r0 = b * kTrsvBlock, r1 = min(n, r0 + kTrsvBlock), bs = r1 - r0;
    if (blockIdx.x == 0) {
      // diagonal block: one warp, sequential over the block's rows
      if (tid < 32) {
        if (lower) {
          for (int i = 0; i < bs; ++i) {
            const T xi = x[r0 + i];
            __syncwarp();
            for (int r = i + 1 + tid; r < bs; r += 32)
              x[r0 + r] = axpy1<false>(x[r0 + r], -xi, A[(size_t)(r0 + i) * lda + r0 + r]);
            __syncwarp();
          }
        } else {
          for (int i = bs - 1; i >= 0; --i) {
            if (tid == 0) {
              const T d = A[(size_t)(r0 + i) * lda + r0 + i];
              if (d == T(0)) atomicMin(info, r0 + i + 1);
              x[r0 + i] = x[r0 + i] / d;
            }
            __syncwarp();
            const T xi = x[r0 + i];
            for (int r = tid; r < i; r += 32)
              x[r0 + r] = axpy1<false>(x[r0 + r], -xi, A[(size_t)(r0 + i) * lda + r0 + r]);
            __syncwarp();
          }
        }
      }
    }
    grid.sync();
    // apply the solved block to the remaining rows: x[rest] -= A[rest, blk] x[blk]
    for (int i = tid; i < bs; i += kTrsvThreads) xs[i] = x[r0 + i];
    __syncthreads();
    const int rest0 = lower ? r1 : 0, rest1 = lower ? n : r0;
    for (int r = rest0 + blockIdx.x * kTrsvThreads + tid; r < rest1; r += gridDim.x * kTrsvThreads) {
      T acc = x[r];
      for (int i = 0; i < bs; ++i) acc = axpy1<false>(acc, -xs[i], A[(size_t)(r0 + i) * lda + r]);
      x[r] = acc;
    }
    grid.sync();
  }
}

// info holds a large sentinel until some pivot fails; 0 afterwards means "ok".
__global__ void info_init_kernel(int32_t* info) { *info = 0x7fffffff; }
__global__ void info_finalize_kernel(int32_t* info) {
  if (*info == 0x7fffffff) *info = 0;
}

template <typename T>
__global__ void apply_pivots_kernel(int n, const int32_t* ipiv, T* x) {
  if (blockIdx.x == 0 && threadIdx.x == 0)
    for (int i = 0; i < n; ++i) {
      const int p = ipiv[i];
      if (p != i) {
        const T t = x[i];
        x[i] = x[p];
        x[p] = t;
      }
    }
}

// ---------------------------------------------------------------------------
// host drivers
// ---------------------------------------------------------------------------
int coop_grid(const void* kern, int threads, size_t smem) {
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem);
  if (per_sm < 1) per_sm = 1;
  return sm_count() * per_sm;
}

// Workspace for the panel candidates: 2 * G + 1 words, G <= 4 * SMs.
size_t getrf_ws_bytes() { return ((size_t)2 * 4 * 1024 + 16) * sizeof(unsigned long long); }

typedef int (*UpdateFn)(int m, int n, int k, const void* L21, const void* U12, void* A22, int64_t lda, void* ctx,
                        cudaStream_t s);

template <typename T>
int getrf_blocked(int n, T* A, int64_t lda, int32_t* ipiv, int32_t* info, void* ws, int nb, UpdateFn update,
                  void* ctx, cudaStream_t s, const char* name) {
  unsigned long long* cand = reinterpret_cast<unsigned long long*>(ws);
  cudaError_t e;
  info_init_kernel<<<1, 1, 0, s>>>(info);
  const void* pk = reinterpret_cast<const void*>(lu_panel_coop_kernel<T>);
  int G = coop_grid(pk, kPanelThreads, 0);
  if (G > 1024) G = 1024;
  for (int j0 = 0; j0 < n; j0 += nb) {
    const int jb = min(nb, n - j0);
    PanelArgs<T> pa{n, A, lda, j0, jb, ipiv, cand, info};
    // enough CTAs to cover the rows, at most the co-resident grid
    const int rows = n - j0;
    int g = min(G, (rows + kPanelThreads - 1) / kPanelThreads);
    if (g < 1) g = 1;
    void* args[] = {&pa};
    e = cudaLaunchCooperativeKernel(pk, g, kPanelThreads, args, 0, s);
    if (e != cudaSuccess) return record_cuda_error(e, name);
    lu_swap_kernel<T><<<(n + 255) / 256, 256, 0, s>>>(n, A, lda, ipiv, j0, jb);
    const int rest = n - j0 - jb;
    if (rest > 0) {
      const size_t smem = (size_t)jb * jb * sizeof(T) + (size_t)jb * 64 * sizeof(T);
      if (smem > 48 * 1024) {
        e = cudaFuncSetAttribute(lu_trsm_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return record_cuda_error(e, name);
      }
      lu_trsm_kernel<T><<<(rest + 63) / 64, 64, smem, s>>>(n, A, lda, j0, jb);
      int rc = update(rest, rest, jb, A + (size_t)j0 * lda + j0 + jb, A + (size_t)(j0 + jb) * lda + j0,
                      A + (size_t)(j0 + jb) * lda + j0 + jb, lda, ctx, s);
      if (rc != NACU_SUCCESS) return rc;
    }
    int rc = check_launch(name);
    if (rc != NACU_SUCCESS) return rc;
  }
  info_finalize_kernel<<<1, 1, 0, s>>>(info);
  return check_launch(name);
}

template <typename T>
int getrs_one(int n, const T* LU, int64_t lda, const int32_t* ipiv, T* x, int32_t* info, cudaStream_t s,
              const char* name) {
  info_init_kernel<<<1, 1, 0, s>>>(info);
  apply_pivots_kernel<T><<<1, 32, 0, s>>>(n, ipiv, x);
  const void* tk = reinterpret_cast<const void*>(trsv_coop_kernel<T>);
  int G = coop_grid(tk, kTrsvThreads, 0);
  const int want = (n + kTrsvThreads - 1) / kTrsvThreads;
  int g = min(G, max(1, want));
  for (int lower = 1; lower >= 0; --lower) {
    int nn = n;
    const T* a = LU;
    int64_t ld = lda;
    int lw = lower;
    void* args[] = {&nn, &a, &ld, &x, &lw, &info};
    cudaError_t e = cudaLaunchCooperativeKernel(tk, g, kTrsvThreads, args, 0, s);
    if (e != cudaSuccess) return record_cuda_error(e, name);
  }
  info_finalize_kernel<<<1, 1, 0, s>>>(info);
  return check_launch(name);
}

int update_fp64(int m, int n, int k, const void* L21, const void* U12, void* A22, int64_t lda, void*, cudaStream_t s) {
  return nacu_dgemm(m, n, k, -1.0, static_cast<const double*>(L21), lda, static_cast<const double*>(U12), lda, 1.0,
                    static_cast<double*>(A22), lda, s);
}

// ---------------------------------------------------------------------------
// mixed precision: FP32 factor (tensor-core trailing updates), FP64 refinement
// ---------------------------------------------------------------------------
struct Update32Ctx {
  void* ws;
  size_t ws_bytes;
};

int update_fp32_split(int m, int n, int k, const void* L21, const void* U12, void* A22, int64_t lda, void* ctx,
                      cudaStream_t s) {
  const Update32Ctx* c = static_cast<const Update32Ctx*>(ctx);
  return split_gemm_run<float, float>(m, n, k, -1.0, static_cast<const float*>(L21), lda,
                                      static_cast<const float*>(U12), lda, 1.0, static_cast<float*>(A22), lda, 3,
                                      c->ws, c->ws_bytes, s);
}

__global__ void to_fp32_kernel(int n, const double* __restrict__ A, int64_t lda, float* __restrict__ A32) {
  const int64_t total = (int64_t)n * n;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = e / n, r = e - c * n;
    A32[e] = (float)A[c * lda + r];
  }
}

__device__ __forceinline__ unsigned long long dabs_bits(double x) {
  return (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffull;
}

// part[cb * n + i] = sum over the column chunk cb of A[i][j] * x[j] (or |A[i][j]| when abs_mode).
constexpr int kGemvChunks = 16;
__global__ void gemv_partial_kernel(int n, const double* __restrict__ A, int64_t lda, const double* __restrict__ x,
                                    double* __restrict__ part, int abs_mode) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int chunk = (n + kGemvChunks - 1) / kGemvChunks;
  const int j0 = blockIdx.y * chunk, j1 = min(n, j0 + chunk);
  double acc = 0.0;
  int j = j0;
  for (; j + 4 <= j1; j += 4) {
    const double a0 = A[(size_t)j * lda + i], a1 = A[(size_t)(j + 1) * lda + i];
    const double a2 = A[(size_t)(j + 2) * lda + i], a3 = A[(size_t)(j + 3) * lda + i];
    if (abs_mode) acc += fabs(a0) + fabs(a1) + fabs(a2) + fabs(a3);
    else acc = fma(a3, x[j + 3], fma(a2, x[j + 2], fma(a1, x[j + 1], fma(a0, x[j], acc))));
  }
  for (; j < j1; ++j) acc = abs_mode ? acc + fabs(A[(size_t)j * lda + i]) : fma(A[(size_t)j * lda + i], x[j], acc);
  part[(size_t)blockIdx.y * n + i] = acc;
}

// r = b - sum(part) (or the row sums when abs_mode); norms (max |.|, as bits) of
// r, x and b into nrm[0..2] (atomicMax on non-negative doubles' bit images).
__global__ void residual_finish_kernel(int n, const double* __restrict__ b, const double* __restrict__ x,
                                       const double* __restrict__ part, double* __restrict__ r,
                                       unsigned long long* nrm, int abs_mode) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long rn = 0, xn = 0, bn = 0;
  if (i < n) {
    double s = 0.0;
    for (int cb = 0; cb < kGemvChunks; ++cb) s += part[(size_t)cb * n + i];
    const double v = abs_mode ? s : b[i] - s;
    if (!abs_mode) r[i] = v;
    rn = dabs_bits(v);
    xn = dabs_bits(x[i]);
    bn = dabs_bits(b[i]);
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    rn = max(rn, __shfl_xor_sync(0xffffffffu, rn, off));
    xn = max(xn, __shfl_xor_sync(0xffffffffu, xn, off));
    bn = max(bn, __shfl_xor_sync(0xffffffffu, bn, off));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMax(&nrm[0], rn);
    atomicMax(&nrm[1], xn);
    atomicMax(&nrm[2], bn);
  }
}

// d32 = (float)(src * 2^-e)
__global__ void scale_to_fp32_kernel(int n, const double* __restrict__ src, int e, float* __restrict__ d32) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) d32[i] = (float)(src[i] * __longlong_as_double((long long)(1023 - e) << 52));
}
// x += (double)d32 * 2^e; max |d| into nrm[3]
__global__ void accumulate_kernel(int n, const float* __restrict__ d32, int e, double* __restrict__ x,
                                  unsigned long long* nrm) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long dn = 0;
  if (i < n) {
    const double d = (double)d32[i] * __longlong_as_double((long long)(1023 + e) << 52);
    x[i] += d;
    dn = dabs_bits(d);
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) dn = max(dn, __shfl_xor_sync(0xffffffffu, dn, off));
  if ((threadIdx.x & 31) == 0) atomicMax(&nrm[3], dn);
}

struct MixedLuLayout {
  size_t a32, ipiv, info, cand, split, r, d32, part, nrm, a64, total;
};
inline size_t up256(size_t x) { return (x + 255) & ~(size_t)255; }
MixedLuLayout mixed_lu_layout(int n, int nb) {
  MixedLuLayout L;
  size_t o = 0;
  L.a32 = o;   o = up256(o + (size_t)n * n * 4);
  L.ipiv = o;  o = up256(o + (size_t)n * 4);
  L.info = o;  o = up256(o + 16);
  L.cand = o;  o = up256(o + getrf_ws_bytes());
  o = (o + 1023) & ~(size_t)1023;
  L.split = o; o = up256(o + nacu_gemm_split_workspace_bytes(n, n, nb));
  L.r = o;     o = up256(o + (size_t)n * 8);
  L.d32 = o;   o = up256(o + (size_t)n * 4);
  L.part = o;  o = up256(o + (size_t)kGemvChunks * n * 8);
  L.nrm = o;   o = up256(o + 8 * 8);
  L.a64 = o;   o = up256(o + (size_t)n * n * 8);
  L.total = o + 1024;  // the caller's base may need aligning to 1024
  return L;
}

int exp_of_bits(unsigned long long b) {
  const int ex = (int)((b >> 52) & 0x7ff);
  if (ex == 0 || ex == 0x7ff) return 0;
  const int e = ex - 1023;
  return e < -1000 ? -1000 : (e > 1000 ? 1000 : e);
}

}  // namespace nacu

extern "C" {

size_t nacu_gesv_mixed_workspace_bytes(int n) { return nacu::mixed_lu_layout(n, 128).total; }

int nacu_dgesv_mixed_ir(int n, const double* A, int64_t lda, const double* b, double* x, double tol_units,
                        int max_iter, int* iters_out, double* berr_out, int* fallback_out, void* workspace,
                        size_t workspace_bytes, nacu_stream_t stream) {
  using namespace nacu;
  if (n < 0) return record_arg_error(-1, "dgesv_mixed_ir: n < 0");
  if (n == 0) return NACU_SUCCESS;
  if (!A || lda < n) return record_arg_error(-2, "dgesv_mixed_ir: bad A / lda");
  if (!b || !x) return record_arg_error(-4, "dgesv_mixed_ir: null b or x");
  const int nb = 128;
  MixedLuLayout L = mixed_lu_layout(n, nb);
  if (!workspace || workspace_bytes < L.total) return record_arg_error(-11, "dgesv_mixed_ir: workspace too small");
  cudaStream_t s = (cudaStream_t)stream;
  unsigned char* base = reinterpret_cast<unsigned char*>(((uintptr_t)workspace + 1023) & ~(uintptr_t)1023);
  float* A32 = reinterpret_cast<float*>(base + L.a32);
  int32_t* ipiv = reinterpret_cast<int32_t*>(base + L.ipiv);
  int32_t* info = reinterpret_cast<int32_t*>(base + L.info);
  void* cand = base + L.cand;
  void* split_ws = base + L.split;
  double* r = reinterpret_cast<double*>(base + L.r);
  float* d32 = reinterpret_cast<float*>(base + L.d32);
  double* part = reinterpret_cast<double*>(base + L.part);
  unsigned long long* nrm = reinterpret_cast<unsigned long long*>(base + L.nrm);
  double* A64 = reinterpret_cast<double*>(base + L.a64);
  const double tol = (tol_units > 0 ? tol_units : 1.0) * n * 2.220446049250313e-16;
  if (max_iter <= 0) max_iter = 30;
  const int nblk = (n + 255) / 256;
  int iters = 0, fallback = 0;
  double berr = INFINITY;
  unsigned long long h[4];
  // ||A||_inf (FP64 row sums of |A|)
  cudaMemsetAsync(nrm, 0, 64, s);
  gemv_partial_kernel<<<dim3(nblk, kGemvChunks), 256, 0, s>>>(n, A, lda, x, part, 1);
  residual_finish_kernel<<<nblk, 256, 0, s>>>(n, b, b, part, r, nrm, 1);
  cudaMemcpyAsync(h, nrm, 32, cudaMemcpyDeviceToHost, s);
  cudaError_t e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return record_cuda_error(e, "nacu_dgesv_mixed_ir");
  const double anorm = __builtin_bit_cast(double, h[0]);
  const double bnorm = __builtin_bit_cast(double, h[2]);
  // FP32 factor
  to_fp32_kernel<<<sm_count() * 8, 256, 0, s>>>(n, A, lda, A32);
  Update32Ctx uctx{split_ws, nacu_gemm_split_workspace_bytes(n, n, nb)};
  int rc = getrf_blocked<float>(n, A32, n, ipiv, info, cand, nb, update_fp32_split, &uctx, s, "nacu_dgesv_mixed_ir");
  if (rc != NACU_SUCCESS) return rc;
  int32_t hinfo = 0;
  cudaMemcpyAsync(&hinfo, info, 4, cudaMemcpyDeviceToHost, s);
  e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return record_cuda_error(e, "nacu_dgesv_mixed_ir");
  bool converged = false;
  if (hinfo == 0) {
    // refinement: x0 = 0, r0 = b
    cudaMemsetAsync(x, 0, (size_t)n * 8, s);
    cudaMemcpyAsync(r, b, (size_t)n * 8, cudaMemcpyDeviceToDevice, s);
    double rnorm = bnorm, dprev = 0.0;
    for (int it = 0; it < max_iter; ++it) {
      // d = (LU)^-1 P r in FP32, scaled by the exponent of ||r||
      int er = 0;
      {
        const double m = rnorm;
        er = (m > 0.0 && std::isfinite(m)) ? exp_of_bits(__builtin_bit_cast(unsigned long long, m)) : 0;
      }
      scale_to_fp32_kernel<<<nblk, 256, 0, s>>>(n, r, er, d32);
      rc = getrs_one<float>(n, A32, n, ipiv, d32, info + 1, s, "nacu_dgesv_mixed_ir");
      if (rc != NACU_SUCCESS) return rc;
      cudaMemsetAsync(nrm, 0, 64, s);
      accumulate_kernel<<<nblk, 256, 0, s>>>(n, d32, er, x, nrm);
      gemv_partial_kernel<<<dim3(nblk, kGemvChunks), 256, 0, s>>>(n, A, lda, x, part, 0);
      residual_finish_kernel<<<nblk, 256, 0, s>>>(n, b, x, part, r, nrm, 0);
      cudaMemcpyAsync(h, nrm, 32, cudaMemcpyDeviceToHost, s);
      e = cudaStreamSynchronize(s);
      if (e != cudaSuccess) return record_cuda_error(e, "nacu_dgesv_mixed_ir");
      ++iters;
      rnorm = __builtin_bit_cast(double, h[0]);
      const double xnorm = __builtin_bit_cast(double, h[1]);
      const double dnorm = __builtin_bit_cast(double, h[3]);
      berr = rnorm / (anorm * xnorm + bnorm);
      if (berr <= tol) {
        converged = true;
        break;
      }
      if (!std::isfinite(berr) || (it >= 1 && dprev > 0.0 && dnorm > 0.5 * dprev)) break;  // stagnation
      dprev = dnorm;
    }
  }
  if (!converged) {
    // FP64 fallback on a copy of A
    fallback = 1;
    cudaMemcpy2DAsync(A64, (size_t)n * 8, A, (size_t)lda * 8, (size_t)n * 8, n, cudaMemcpyDeviceToDevice, s);
    rc = nacu_dgetrf(n, A64, n, ipiv, info, cand, getrf_ws_bytes(), stream);
    if (rc != NACU_SUCCESS) return rc;
    cudaMemcpyAsync(x, b, (size_t)n * 8, cudaMemcpyDeviceToDevice, s);
    rc = nacu_dgetrs(n, A64, n, ipiv, x, info + 1, stream);
    if (rc != NACU_SUCCESS) return rc;
    cudaMemsetAsync(nrm, 0, 64, s);
    gemv_partial_kernel<<<dim3(nblk, kGemvChunks), 256, 0, s>>>(n, A, lda, x, part, 0);
    residual_finish_kernel<<<nblk, 256, 0, s>>>(n, b, x, part, r, nrm, 0);
    cudaMemcpyAsync(h, nrm, 32, cudaMemcpyDeviceToHost, s);
    e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return record_cuda_error(e, "nacu_dgesv_mixed_ir");
    berr = __builtin_bit_cast(double, h[0]) / (anorm * __builtin_bit_cast(double, h[1]) + bnorm);
  }
  if (iters_out) *iters_out = iters;
  if (berr_out) *berr_out = berr;
  if (fallback_out) *fallback_out = fallback;
  return check_launch("nacu_dgesv_mixed_ir");
}

size_t nacu_getrf_workspace_bytes(int n) {
  (void)n;
  return nacu::getrf_ws_bytes();
}

int nacu_dgetrf(int n, double* A, int64_t lda, int32_t* ipiv, int32_t* info, void* workspace, size_t workspace_bytes,
                nacu_stream_t stream) {
  using namespace nacu;
  if (n < 0) return record_arg_error(-1, "dgetrf: n < 0");
  if (n == 0) return NACU_SUCCESS;
  if (!A) return record_arg_error(-2, "dgetrf: null A");
  if (lda < n) return record_arg_error(-3, "dgetrf: lda < n");
  if (!ipiv || !info) return record_arg_error(-4, "dgetrf: null ipiv or info");
  if (!workspace || workspace_bytes < getrf_ws_bytes()) return record_arg_error(-6, "dgetrf: workspace too small");
  return getrf_blocked<double>(n, A, lda, ipiv, info, workspace, 64, update_fp64, nullptr, (cudaStream_t)stream,
                               "nacu_dgetrf");
}

int nacu_dgetrs(int n, const double* LU, int64_t lda, const int32_t* ipiv, double* b, int32_t* info,
                nacu_stream_t stream) {
  using namespace nacu;
  if (n < 0) return record_arg_error(-1, "dgetrs: n < 0");
  if (n == 0) return NACU_SUCCESS;
  if (!LU || !ipiv || !b || !info) return record_arg_error(-2, "dgetrs: null argument");
  if (lda < n) return record_arg_error(-3, "dgetrs: lda < n");
  return getrs_one<double>(n, LU, lda, ipiv, b, info, (cudaStream_t)stream, "nacu_dgetrs");
}

}  // extern "C"
