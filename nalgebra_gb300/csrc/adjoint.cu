// Reverse-mode adjoint of the batched Cholesky solve and log-determinant, for
// batches of equal-order SPD matrices (n <= 128), in FP64 and FP32.
//
// Forward (nalgebra's `m.cholesky()`, `.solve(&b)`, `.ln_determinant()`,
// src/linalg/cholesky.rs:221-272, 122-143, 172-185): x = A^-1 b and
// logdet A = sum ln(L_ii^2); the factor L is written out (the "store" form)
// or discarded (the "recompute" form keeps only A).
//
// Backward, for the cotangents w = dl/dx and g = dl/dlogdet of a loss l
// (default g = 1: the loss l = sum_s w_s^T x_s + logdet A_s; nalgebra has no
// autodiff, this is the chosen differentiation form):
//   v  = A^-1 w                       (dl/db)
//   Abar = -v x^T + g A^-1            (dl/dA for an unstructured A)
// nalgebra reads only the lower triangle, so the parameters are the lower
// entries theta_ij (i >= j) with A_ij = A_ji = theta_ij; the gradient
// returned in dA's lower triangle is
//   dA_ii = Abar_ii = -v_i x_i + g (A^-1)_ii,
//   dA_ij = Abar_ij + Abar_ji = -(v_i x_j + v_j x_i) + 2 g (A^-1)_ij  (i > j),
// which is what central differences on theta_ij measure.  (Giles 2008,
// "Collected matrix derivative results for forward and reverse mode AD";
// Murray 2016, "Differentiation of the Cholesky decomposition".)
//
// Design: one CTA (256 threads) per matrix with the matrix's packed lower
// triangle in shared memory (66 KB at n = 128 in FP64, so three CTAs share an
// SM where the full square allowed one), so the factorization, the in-place
// triangular inverse L -> L^-1 and the product A^-1 = L^-T L^-1 run out of
// shared memory.  Trailing updates use a
// pair-folded index over the lower triangle (column c paired with column
// m-1-c fills an (m+1) x ceil(m/2) rectangle), so no lane idles on the
// triangle's empty half.
#include "common.cuh"

namespace nacu {
namespace {

constexpr int kAdjThreads = 256;
constexpr int kAdjMaxN = 128;

template <typename T>
__device__ __forceinline__ T fma_t(T a, T b, T c) {
  if constexpr (sizeof(T) == 8) return fma(a, b, c);
  else return fmaf(a, b, c);
}

// Pair-folded enumeration of the lower triangle (rows >= column) of an m x m
// block: rectangle index (k, q), k in [0, m+1), q in [0, ceil(m/2)).
__device__ __forceinline__ bool fold(int m, int k, int q, int* r, int* c) {
  const int len = m - q;  // column q holds rows q..m-1
  if (k < len) {
    *c = q;
    *r = q + k;
    return true;
  }
  const int c2 = m - 1 - q;
  if (c2 <= q) return false;  // odd m: the middle column appears once
  *c = c2;
  *r = c2 + (k - len);
  return *r < m;
}

// Element (r, c), r >= c, of the lower triangle in shared memory sits at
// S[cb[c] + r]: cb[c] = c * ld for a full column-major square, or
// c * n - c (c + 1) / 2 for the packed triangle (column c's rows c..n-1 follow
// column c-1's), which halves the backward kernel's shared memory.

// Right-looking Cholesky of the n x n matrix in S (lower triangle).
// Returns info (0 ok, j+1 first failing pivot) in *s_info.
template <typename T>
__device__ void chol_smem(int n, T* S, const int* cb, int* s_info, T* s_sc) {
  const int tid = threadIdx.x, nthr = blockDim.x;
  for (int j = 0; j < n; ++j) {
    T* cj = S + cb[j];
    if (tid == 0) {
      const T d = cj[j];
      if (!(d <= T(0)) && d >= T(0)) {
        const T r = rsqrt(d);  // L_jj = d * rsqrt(d), 1/L_jj = rsqrt(d): one dependent FP64 chain
        cj[j] = d * r;
        s_sc[0] = r;
      } else if (*s_info == 0) {
        *s_info = j + 1;
      }
    }
    __syncthreads();
    if (*s_info != 0) return;
    const T rcp = s_sc[0];
    for (int r = j + 1 + tid; r < n; r += nthr) cj[r] *= rcp;
    __syncthreads();
    const int m = n - j - 1;
    if (m > 0) {
      const int qn = (m + 1) >> 1, total = (m + 1) * qn;
      for (int e = tid; e < total; e += nthr) {
        const int q = e / (m + 1), k = e - q * (m + 1);
        int r, c;
        if (fold(m, k, q, &r, &c)) {
          r += j + 1;
          c += j + 1;
          S[cb[c] + r] = fma_t(-cj[r], cj[c], S[cb[c] + r]);
        }
      }
    }
    __syncthreads();
  }
}

// In place L -> L^-1 (lower), columns from right to left (LAPACK trti2 order):
// L^-1[i][j] = -(1/L_jj) * sum_{k=j+1..i} L^-1[i][k] L[k][j]  (i > j).
// Two threads per row i (k split by parity, combined by a shuffle), so all
// warps share each column's dot products; fused multiply-adds; the
// reciprocals of the diagonal (rdiag) are formed once beforehand.  Columns go
// two at a time (j and j-1 share each L^-1[i][k] load and one pair of
// barriers): with s0, s1 the sums over k > j,
//   L^-1[i][j] = -s0 / L_jj,  L^-1[i][j-1] = -(s1 + L^-1[i][j] L[j][j-1]) / L_{j-1,j-1}.
// tmp holds 2n values.
template <typename T>
__device__ void trinv_smem(int n, T* S, const int* cb, T* tmp, const T* rdiag) {
  const int tid = threadIdx.x;
  const int ri = tid >> 1, h = tid & 1;
  int j = n - 1;
  for (; j >= 1; j -= 2) {
    const T* cj = S + cb[j];
    const T* cj1 = S + cb[j - 1];
    const T ajj = rdiag[j], aj1 = rdiag[j - 1];
    const int i = j + 1 + ri;
    T s0 = T(0), s1 = T(0);
    if (i < n)
      for (int k = j + 1 + h; k <= i; k += 2) {
        const T li = S[cb[k] + i];  // L^-1[i][k]
        s0 = fma_t(li, cj[k], s0);
        s1 = fma_t(li, cj1[k], s1);
      }
    s0 += __shfl_xor_sync(0xffffffffu, s0, 1);
    s1 += __shfl_xor_sync(0xffffffffu, s1, 1);
    if (i < n && h == 0) {
      const T x0 = -ajj * s0;
      tmp[i] = x0;
      tmp[n + i] = -aj1 * fma_t(x0, cj1[j], s1);
    }
    __syncthreads();
    T* cw = S + cb[j];
    T* cw1 = S + cb[j - 1];
    for (int r = j + 1 + tid; r < n; r += blockDim.x) {
      cw[r] = tmp[r];
      cw1[r] = tmp[n + r];
    }
    if (tid == 0) {
      cw1[j] = -aj1 * (ajj * cw1[j]);  // L^-1[j][j-1] = -L[j][j-1] / (L_jj L_{j-1,j-1})
      cw[j] = ajj;
      cw1[j - 1] = aj1;
    }
    __syncthreads();
  }
  if (j == 0) {  // odd n: the first column on its own
    const T* c0 = S + cb[0];
    const T a00 = rdiag[0];
    const int i = 1 + ri;
    T acc = T(0);
    if (i < n)
      for (int k = 1 + h; k <= i; k += 2) acc = fma_t(S[cb[k] + i], c0[k], acc);
    acc += __shfl_xor_sync(0xffffffffu, acc, 1);
    if (i < n && h == 0) tmp[i] = -a00 * acc;
    __syncthreads();
    T* cw = S + cb[0];
    for (int r = 1 + tid; r < n; r += blockDim.x) cw[r] = tmp[r];
    if (tid == 0) cw[0] = a00;
    __syncthreads();
  }
}

// In place L^-1 -> A^-1 = L^-T L^-1 (lower triangle):
// (A^-1)_ij = sum_{k >= i} Linv_ki Linv_kj  (i >= j).  Given L^-1 the columns
// are independent, and column j needs only columns >= j, so four columns are
// formed per pair of barriers (each Linv_ki load feeds four FMAs) into tmp and
// written back over their L^-1 columns.  Two threads per row, k split by
// parity.  tmp holds 4n values.
template <typename T>
__device__ void inv_from_trinv_smem(int n, T* S, const int* cb, T* tmp) {
  const int tid = threadIdx.x;
  const int ri = tid >> 1, h = tid & 1;
  for (int j = 0; j < n; j += 4) {
    const int jw = min(4, n - j);
    const int i = j + ri;
    T acc[4] = {T(0), T(0), T(0), T(0)};
    if (i < n) {
      const T* ci = S + cb[i];
      const T* cju[4] = {S + cb[j], S + cb[min(j + 1, n - 1)], S + cb[min(j + 2, n - 1)], S + cb[min(j + 3, n - 1)]};
      for (int k = i + h; k < n; k += 2) {
        const T lki = ci[k];
#pragma unroll
        for (int u = 0; u < 4; ++u)
          if (u < jw && i >= j + u) acc[u] = fma_t(lki, cju[u][k], acc[u]);  // Linv[k][j+u], k >= i >= j+u
      }
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      acc[u] += __shfl_xor_sync(0xffffffffu, acc[u], 1);
      if (i < n && h == 0 && u < jw && i >= j + u) tmp[u * n + i] = acc[u];
    }
    __syncthreads();
    for (int u = 0; u < jw; ++u) {
      T* cw = S + cb[j + u];
      for (int r = j + u + tid; r < n; r += blockDim.x) cw[r] = tmp[u * n + r];
    }
    __syncthreads();
  }
}

// Forward: S <- A (lower), factor, x = A^-1 b (forward + back substitution in
// shared memory), logdet; write L (store form) or nothing.
template <typename T>
__global__ void __launch_bounds__(kAdjThreads) adj_forward_kernel(int n, const T* __restrict__ A, int64_t strideA,
                                                                  const T* __restrict__ B, T* __restrict__ X,
                                                                  T* __restrict__ Lout, T* __restrict__ logdet,
                                                                  int32_t* __restrict__ info, int batch) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_info;
  __shared__ T s_sc[2];
  __shared__ int cb[kAdjMaxN];
  T* S = reinterpret_cast<T*>(smem_raw);  // the packed lower triangle
  T* y = S + (size_t)n * (n + 1) / 2;
  const int tid = threadIdx.x;
  for (int c = tid; c < n; c += blockDim.x) cb[c] = c * n - c * (c + 1) / 2;
  __syncthreads();  // every column base is set before any thread stores through it
  for (int s = blockIdx.x; s < batch; s += gridDim.x) {
    const T* a = A + (size_t)s * strideA;
    for (int e = tid; e < n * n; e += blockDim.x) {
      const int c = e / n, r = e - c * n;
      if (r >= c) S[cb[c] + r] = a[e];
    }
    for (int i = tid; i < n; i += blockDim.x) y[i] = B[(size_t)s * n + i];
    if (tid == 0) s_info = 0;
    __syncthreads();
    chol_smem<T>(n, S, cb, &s_info, s_sc);
    const int inf = s_info;
    if (inf == 0) {
      // L y = b then L^T x = y; one warp (n <= 128: four rows per lane)
      if (tid < 32) {
        for (int i = 0; i < n; ++i) {
          if (tid == 0) y[i] = y[i] / S[cb[i] + i];
          __syncwarp();
          const T yi = y[i];
          for (int r = i + 1 + tid; r < n; r += 32) y[r] = fma_t(-yi, S[cb[i] + r], y[r]);
          __syncwarp();
        }
        for (int i = n - 1; i >= 0; --i) {
          T sacc = T(0);
          for (int r = i + 1 + tid; r < n; r += 32) sacc = fma_t(S[cb[i] + r], y[r], sacc);
          sacc = warp_sum(sacc);
          if (tid == 0) y[i] = (y[i] - sacc) / S[cb[i] + i];
          __syncwarp();
        }
      }
      __syncthreads();
      for (int i = tid; i < n; i += blockDim.x) X[(size_t)s * n + i] = y[i];
      if (tid == 0) {
        T sum = T(0);
        for (int i = 0; i < n; ++i) {
          const T d = S[cb[i] + i];
          sum += log(d * d);
        }
        logdet[s] = sum;
      }
      if (Lout)
        for (int e = tid; e < n * n; e += blockDim.x) {
          const int c = e / n, r = e - c * n;
          Lout[(size_t)s * strideA + e] = (r >= c) ? S[cb[c] + r] : T(0);
        }
    }
    if (tid == 0 && info) info[s] = inf;
    __syncthreads();
  }
}

// Backward: from L (store form) or A (recompute form) build A^-1 in shared
// memory, then db = v = A^-1 w and the lower-triangle gradient dA.
template <typename T>
__global__ void __launch_bounds__(kAdjThreads) adj_backward_kernel(int n, const T* __restrict__ AL, int64_t strideA,
                                                                   int recompute, const T* __restrict__ X,
                                                                   const T* __restrict__ Wt,
                                                                   const T* __restrict__ Glog, T* __restrict__ dA,
                                                                   T* __restrict__ db, int32_t* __restrict__ info,
                                                                   int batch) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_info;
  __shared__ T s_sc[2];
  __shared__ int cb[kAdjMaxN];
  T* S = reinterpret_cast<T*>(smem_raw);  // the packed lower triangle, n (n + 1) / 2 entries
  T* tmp = S + (size_t)n * (n + 1) / 2;
  T* v = tmp + n;
  T* xs = v + n;
  T* ws = xs + n;
  T* rdiag = ws + n;
  const int tid = threadIdx.x;
  for (int c = tid; c < n; c += blockDim.x) cb[c] = c * n - c * (c + 1) / 2;
  __syncthreads();
  for (int s = blockIdx.x; s < batch; s += gridDim.x) {
    const T* a = AL + (size_t)s * strideA;
    for (int e = tid; e < n * n; e += blockDim.x) {
      const int c = e / n, r = e - c * n;
      if (r >= c) S[cb[c] + r] = a[e];
    }
    if (tid == 0) s_info = 0;
    __syncthreads();
    if (recompute) chol_smem<T>(n, S, cb, &s_info, s_sc);  // refactor instead of storing L
    const int inf = s_info;
    if (inf == 0) {
      for (int i = tid; i < n; i += blockDim.x) rdiag[i] = T(1) / S[cb[i] + i];
      __syncthreads();
      trinv_smem<T>(n, S, cb, tmp, rdiag);     // tmp, v: 2n of scratch
      inv_from_trinv_smem<T>(n, S, cb, tmp);   // tmp, v, xs, ws: 4n of scratch
      for (int i = tid; i < n; i += blockDim.x) {
        xs[i] = X[(size_t)s * n + i];
        ws[i] = Wt[(size_t)s * n + i];
      }
      __syncthreads();
      // v = A^-1 w from the lower triangle of the symmetric A^-1
      for (int i = tid; i < n; i += blockDim.x) {
        T acc = T(0);
        for (int k = 0; k <= i; ++k) acc = fma_t(S[cb[k] + i], ws[k], acc);
        for (int k = i + 1; k < n; ++k) acc = fma_t(S[cb[i] + k], ws[k], acc);
        v[i] = acc;
      }
      __syncthreads();
      for (int i = tid; i < n; i += blockDim.x) db[(size_t)s * n + i] = v[i];
      T* g = dA + (size_t)s * strideA;
      const T gl = Glog ? Glog[s] : T(1);
      const T gl2 = T(2) * gl;
      for (int e = tid; e < n * n; e += blockDim.x) {
        const int c = e / n, r = e - c * n;
        T val = T(0);
        if (r == c) val = fma_t(-v[r], xs[r], gl * S[cb[c] + r]);
        else if (r > c) val = fma_t(-v[r], xs[c], fma_t(-v[c], xs[r], gl2 * S[cb[c] + r]));
        g[e] = val;
      }
    }
    if (tid == 0 && info) info[s] = inf;
    __syncthreads();
  }
}

template <typename T>
int adj_launch_forward(int n, const T* A, int64_t strideA, const T* B, T* X, T* Lout, T* logdet, int32_t* info,
                       int batch, cudaStream_t stream, const char* name) {
  if (n < 1 || n > kAdjMaxN) return record_arg_error(-1, "posv_logdet_forward: n out of range [1, 128]");
  if (batch < 0) return record_arg_error(-9, "posv_logdet_forward: negative batch");
  if (batch == 0) return NACU_SUCCESS;
  if (!A || !B || !X || !logdet) return record_arg_error(-2, "posv_logdet_forward: null A, B, X or logdet");
  if (strideA < (int64_t)n * n) return record_arg_error(-3, "posv_logdet_forward: strideA < n*n");
  const size_t smem = ((size_t)n * (n + 1) / 2 + n) * sizeof(T);
  cudaError_t e = ensure_dynamic_smem(adj_forward_kernel<T>, smem);
  if (e != cudaSuccess) return record_cuda_error(e, name);
  adj_forward_kernel<T><<<batch, kAdjThreads, smem, stream>>>(n, A, strideA, B, X, Lout, logdet, info, batch);
  return check_launch(name);
}

template <typename T>
int adj_launch_backward(int n, const T* AL, int64_t strideA, int recompute, const T* X, const T* W, const T* G, T* dA,
                        T* db, int32_t* info, int batch, cudaStream_t stream, const char* name) {
  if (n < 1 || n > kAdjMaxN) return record_arg_error(-1, "posv_logdet_backward: n out of range [1, 128]");
  if (batch < 0) return record_arg_error(-10, "posv_logdet_backward: negative batch");
  if (batch == 0) return NACU_SUCCESS;
  if (!AL || !X || !W || !dA || !db) return record_arg_error(-2, "posv_logdet_backward: null argument");
  if (strideA < (int64_t)n * n) return record_arg_error(-3, "posv_logdet_backward: strideA < n*n");
  const size_t smem = ((size_t)n * (n + 1) / 2 + 5 * (size_t)n) * sizeof(T);
  cudaError_t e = ensure_dynamic_smem(adj_backward_kernel<T>, smem);
  if (e != cudaSuccess) return record_cuda_error(e, name);
  adj_backward_kernel<T><<<batch, kAdjThreads, smem, stream>>>(n, AL, strideA, recompute, X, W, G, dA, db, info,
                                                               batch);
  return check_launch(name);
}

}  // namespace
}  // namespace nacu

extern "C" {

int nacu_dposv_logdet_forward(int n, const double* A, int64_t strideA, const double* B, double* X, double* L,
                              double* logdet, int32_t* info, int batch, nacu_stream_t stream) {
  using namespace nacu;
  if (L == nullptr)  // recompute form: no factor buffer, the shared-memory kernel keeps nothing
    return adj_launch_forward<double>(n, A, strideA, B, X, L, logdet, info, batch, (cudaStream_t)stream,
                                      "nacu_dposv_logdet_forward");
  // store form: the factor is built in L by the FP64 batched Cholesky kernel
  // (factor + solve + log-det in place on copies of A and b)
  if (n < 1 || n > kAdjMaxN) return record_arg_error(-1, "posv_logdet_forward: n out of range [1, 128]");
  if (batch < 0) return record_arg_error(-9, "posv_logdet_forward: negative batch");
  if (batch == 0) return NACU_SUCCESS;
  if (!A || !B || !X || !logdet || !info)
    return record_arg_error(-2, "posv_logdet_forward: null A, B, X, logdet or info");
  if (strideA < (int64_t)n * n) return record_arg_error(-3, "posv_logdet_forward: strideA < n*n");
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = cudaMemcpyAsync(L, A, (size_t)batch * strideA * sizeof(double), cudaMemcpyDeviceToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(X, B, (size_t)batch * n * sizeof(double), cudaMemcpyDeviceToDevice, s);
  if (e != cudaSuccess) return record_cuda_error(e, "nacu_dposv_logdet_forward");
  return chol_uniform_posv(n, L, strideA, 1, X, n, info, logdet, batch, s, "nacu_dposv_logdet_forward");
}
int nacu_sposv_logdet_forward(int n, const float* A, int64_t strideA, const float* B, float* X, float* L,
                              float* logdet, int32_t* info, int batch, nacu_stream_t stream) {
  return nacu::adj_launch_forward<float>(n, A, strideA, B, X, L, logdet, info, batch, (cudaStream_t)stream,
                                         "nacu_sposv_logdet_forward");
}
int nacu_dposv_logdet_backward(int n, const double* AL, int64_t strideA, int recompute, const double* X,
                               const double* W, const double* G, double* dA, double* db, int32_t* info, int batch,
                               nacu_stream_t stream) {
  return nacu::adj_launch_backward<double>(n, AL, strideA, recompute, X, W, G, dA, db, info, batch,
                                           (cudaStream_t)stream, "nacu_dposv_logdet_backward");
}
int nacu_sposv_logdet_backward(int n, const float* AL, int64_t strideA, int recompute, const float* X,
                               const float* W, const float* G, float* dA, float* db, int32_t* info, int batch,
                               nacu_stream_t stream) {
  return nacu::adj_launch_backward<float>(n, AL, strideA, recompute, X, W, G, dA, db, info, batch,
                                          (cudaStream_t)stream, "nacu_sposv_logdet_backward");
}

}  // extern "C"
