// Batched LU with partial pivoting and the fused solve, for many small dense
// systems (n <= 128): the GPU form of nalgebra's `m.lu()` then `.solve(&b)`.
//
// Follows src/linalg/lu.rs:93-122 (LU::new), lu.rs:337-389 (gauss_step /
// gauss_step_swap), src/base/min_max.rs:221-240 (icamax) and lu.rs:242-260 with
// src/linalg/solve.rs:106-182 (solve_mut).
//
// Design (GB300): FP64 runs at ~1/74 of the FP32 rate on this part, so the
// kernel is bound by the FP64 pipe, not HBM.  One CTA owns one system, the
// augmented matrix [A | B] lives in shared memory (column-major, odd leading
// dimension so row walks are bank-conflict free), and every elimination step
// spreads the (n-1-i) x (n-1-i+nrhs) trailing update evenly over all threads
// (a flattened index), so no lane idles on finished rows.  Comparisons for the
// pivot search are done on the integer image of |x| and cost no FP64 issue
// slots.  The forward solve rides along as extra columns of the elimination
// (bit-identical to nalgebra's permute-then-forward-substitute order); the back
// substitution runs in shared memory afterwards.
//
// EXACT = true reproduces nalgebra's arithmetic exactly (reciprocal multiply,
// separately rounded multiply and add, true division in the back solve), so
// factors, pivots and solutions are bit-identical to nalgebra's CPU results.
// EXACT = false contracts each update to one FMA (half the FP64 issue slots).
#include <algorithm>

#include "common.cuh"

namespace nacu {
namespace {

constexpr int kLuThreads = 256;

// Pivot of column c (icamax over rows c..n-1, one warp): s_piv[c] (c itself
// for an all-zero column, which is skipped: lu.rs:107-110), and in s_rcp:
// [0] = 1/pivot, [n+1] = the pivot, [n+2] = the old diagonal a[c][c].  Each
// lane scans the rows it updated itself (r = c + lane + 32k), so the scan
// needs no barrier after that update.
template <typename T, bool EXACT>
__device__ __forceinline__ void lu_find_pivot(int n, int c, const T* colc, int* s_piv, T* s_rcp, int lane) {
  uint64_t key = 0;
  int idx = 0x7fffffff;
  for (int r = c + lane; r < n; r += 32) {
    const uint64_t k = pivot_key(colc[r], r == c);
    if (idx == 0x7fffffff || k > key) {
      key = k;
      idx = r;
    }
  }
  warp_argmax(key, idx);
  __syncwarp();
  if (lane == 0) {
    const T d = colc[idx];
    const bool zero = is_zero_bits(d);
    s_piv[c] = zero ? c : idx;
    // one reciprocal per step, not per thread; it sits on warp 0's look-ahead
    // chain, so the FMA form of the FP64 kernel takes the short Newton form
    if constexpr (EXACT || sizeof(T) != 8) s_rcp[0] = zero ? T(0) : T(1) / d;
    else s_rcp[0] = zero ? T(0) : (T)rcp_nr((double)d);
    s_rcp[n + 1] = d;
    s_rcp[n + 2] = colc[c];
  }
}

template <typename T, bool EXACT>
__device__ void lu_system(int n, int nrhs, int ld, T* sa, int* s_piv, int* s_info, T* s_rcp, bool factor) {
  const int tid = threadIdx.x;
  const int nthr = blockDim.x;
  const int ncols = n + nrhs;
  const int warp = tid >> 5, lane = tid & 31;
  if (factor) {
    // Two barriers per step.  Phase A swaps rows i and piv in every column but
    // i and writes column i as [pivot; multipliers].  Phase B is the rank-1
    // update: warp 0 updates column i+1 and at once finds its pivot for the
    // next step (look-ahead), the other warps update columns i+2.. (the
    // right-hand sides included).  Every element still receives nalgebra's
    // operations in nalgebra's order.
    if (warp == 0 && n > 0) lu_find_pivot<T, EXACT>(n, 0, sa, s_piv, s_rcp, lane);
    __syncthreads();
    for (int i = 0; i < n; ++i) {
      T* coli = sa + (size_t)i * ld;
      const int piv = s_piv[i];
      const T diag = s_rcp[n + 1];
      const T inv_diag = s_rcp[0];
      const T old_ii = s_rcp[n + 2];
      const bool skip = is_zero_bits(diag);  // lu.rs:107-110: all-zero column, no elimination
      if (!skip) {
        if (piv != i) {
          for (int c = tid; c < ncols; c += nthr) {
            if (c == i) continue;
            T* col = sa + (size_t)c * ld;
            const T t = col[i];
            col[i] = col[piv];
            col[piv] = t;
          }
        }
        for (int r = i + 1 + tid; r < n; r += nthr) {
          const T v = (r == piv) ? old_ii : coli[r];
          if constexpr (EXACT) {
            coli[r] = (sizeof(T) == 8) ? (T)__dmul_rn((double)v, (double)inv_diag)
                                       : (T)__fmul_rn((float)v, (float)inv_diag);
          } else {
            coli[r] = v * inv_diag;
          }
        }
        if (tid == 0) coli[i] = diag;
      }
      __syncthreads();
      const int m = n - 1 - i;
      if (m > 0) {
        T* coln = sa + (size_t)(i + 1) * ld;
        if (!skip) {
          const T* lcol = coli + i + 1;
          if (warp == 0) {
            const T u = coln[i];
            for (int r = lane; r < m; r += 32) coln[i + 1 + r] = axpy1<EXACT>(coln[i + 1 + r], -u, lcol[r]);
          } else {
            // a[r][c] += (-a[i][c]) * l[r] for columns i+2.., one flattened
            // index per element over warps 1..
            const int w = ncols - 2 - i;
            const int total = m * w;
            const int nt = nthr - 32;
            int e = tid - 32;
            int cq = e / m;
            int rr = e - cq * m;
            const int dq = nt / m;
            const int dr = nt - dq * m;
            T* base = sa + (size_t)(i + 2) * ld;
            for (; e < total; e += nt) {
              T* col = base + (size_t)cq * ld;
              const T u = col[i];
              col[i + 1 + rr] = axpy1<EXACT>(col[i + 1 + rr], -u, lcol[rr]);
              rr += dr;
              cq += dq;
              if (rr >= m) {
                rr -= m;
                ++cq;
              }
            }
          }
        }
        if (warp == 0) lu_find_pivot<T, EXACT>(n, i + 1, coln, s_piv, s_rcp, lane);
      }
      __syncthreads();
    }
  } else {
    // Solve only: apply the recorded row swaps to the right-hand sides
    // (permutation_sequence.rs:97-104), then the unit-lower forward solve in
    // nalgebra's axpy order (solve.rs:106-133).
    for (int c = tid; c < nrhs; c += nthr) {
      T* col = sa + (size_t)(n + c) * ld;
      for (int i = 0; i < n; ++i) {
        const int p = s_piv[i];
        if (p != i) {
          T t = col[i];
          col[i] = col[p];
          col[p] = t;
        }
      }
    }
    __syncthreads();
    for (int i = 0; i + 1 < n; ++i) {
      const T* lcol = sa + (size_t)i * ld;
      const int m = n - 1 - i;
      for (int e = tid; e < m * nrhs; e += nthr) {
        const int c = e / m, r = i + 1 + (e - c * m);
        T* bcol = sa + (size_t)(n + c) * ld;
        bcol[r] = axpy1<EXACT>(bcol[r], -bcol[i], lcol[r]);
      }
      __syncthreads();
    }
  }
  // Singular check (LAPACK getrf convention: first zero U_ii, 1-based).
  if (tid == 0) {
    int inf = 0;
    for (int i = 0; i < n; ++i)
      if (is_zero_bits(sa[(size_t)i * ld + i])) {
        inf = i + 1;
        break;
      }
    *s_info = inf;
  }
  __syncthreads();
  if (nrhs == 0 || *s_info != 0) return;
  // Back substitution (solve.rs:155-182), one warp per right-hand side:
  // coeff = b[i] / U_ii (true division), then b[0..i] += (-coeff) * U[0..i][i].
  if constexpr (!EXACT) {
    for (int i = tid; i < n; i += nthr) s_rcp[1 + i] = T(1) / sa[(size_t)i * ld + i];
    __syncthreads();
  }
  for (int c = warp; c < nrhs; c += (nthr >> 5)) {
    T* bcol = sa + (size_t)(n + c) * ld;
    for (int i = n - 1; i >= 0; --i) {
      const T* ucol = sa + (size_t)i * ld;
      if (lane == 0) {
        if constexpr (EXACT) bcol[i] = bcol[i] / ucol[i];
        else bcol[i] = bcol[i] * s_rcp[1 + i];
      }
      __syncwarp();
      const T coeff = bcol[i];
      for (int r = lane; r < i; r += 32) bcol[r] = axpy1<EXACT>(bcol[r], -coeff, ucol[r]);
      __syncwarp();
    }
  }
  __syncthreads();
}

// One CTA per system, grid-stride over the batch.  mode: 0 = factor only,
// 1 = factor + solve, 2 = solve from given factors.
template <typename T, bool EXACT>
__global__ void __launch_bounds__(kLuThreads) lu_batched_kernel(int n, int nrhs, T* __restrict__ A,
                                                                 int64_t strideA, int32_t* __restrict__ ipiv,
                                                                 T* __restrict__ B, int64_t strideB,
                                                                 int32_t* __restrict__ info, int batch,
                                                                 int mode, int write_factors) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int ld = n | 1;
  const int ncols = n + nrhs;
  T* sa = reinterpret_cast<T*>(smem_raw);
  T* s_rcp = sa + (size_t)ld * ncols;  // [0]: 1/pivot, [n+1], [n+2]: the step's scalars; [1+i]: 1/U_ii
  int* s_piv = reinterpret_cast<int*>(s_rcp + n + 3);
  int* s_info = s_piv + n;
  const int tid = threadIdx.x;
  for (int s = blockIdx.x; s < batch; s += gridDim.x) {
    const T* a = A + (size_t)s * strideA;
    for (int e = tid; e < n * n; e += blockDim.x) {
      const int c = e / n, r = e - c * n;
      sa[(size_t)c * ld + r] = a[e];
    }
    if (nrhs > 0) {
      const T* b = B + (size_t)s * strideB;
      for (int e = tid; e < n * nrhs; e += blockDim.x) {
        const int c = e / n, r = e - c * n;
        sa[(size_t)(n + c) * ld + r] = b[(size_t)c * n + r];
      }
    }
    if (mode == 2)
      for (int i = tid; i < n; i += blockDim.x) s_piv[i] = ipiv[(size_t)s * n + i];
    __syncthreads();
    lu_system<T, EXACT>(n, nrhs, ld, sa, s_piv, s_info, s_rcp, mode != 2);
    if (mode != 2) {
      if (write_factors) {
        T* aw = A + (size_t)s * strideA;
        for (int e = tid; e < n * n; e += blockDim.x) {
          const int c = e / n, r = e - c * n;
          aw[e] = sa[(size_t)c * ld + r];
        }
      }
      for (int i = tid; i < n; i += blockDim.x) ipiv[(size_t)s * n + i] = s_piv[i];
    }
    if (nrhs > 0) {
      T* b = B + (size_t)s * strideB;
      for (int e = tid; e < n * nrhs; e += blockDim.x) {
        const int c = e / n, r = e - c * n;
        b[(size_t)c * n + r] = sa[(size_t)(n + c) * ld + r];
      }
    }
    if (tid == 0 && info) info[s] = *s_info;
    __syncthreads();
  }
}

template <typename T>
size_t lu_smem_bytes(int n, int nrhs) {
  const int ld = n | 1;
  return (size_t)ld * (n + nrhs) * sizeof(T) + (size_t)(n + 3) * sizeof(T) + (size_t)(n + 1) * sizeof(int);
}

template <typename T>
int lu_launch(int n, int nrhs, T* A, int64_t strideA, int32_t* ipiv, T* B, int64_t strideB, int32_t* info,
              int batch, int mode, int flags, cudaStream_t stream, const char* name) {
  if (n < 0 || n > NACU_LU_BATCHED_MAX_N) return record_arg_error(-1, "lu batched: n out of range [0, 128]");
  if (nrhs < 0 || nrhs > NACU_LU_BATCHED_MAX_NRHS) return record_arg_error(-2, "lu batched: nrhs out of range [0, 16]");
  if (batch < 0) return record_arg_error(-9, "lu batched: negative batch");
  if (batch == 0 || n == 0) return NACU_SUCCESS;
  if (A == nullptr || ipiv == nullptr) return record_arg_error(-3, "lu batched: null A or ipiv");
  if (nrhs > 0 && B == nullptr) return record_arg_error(-6, "lu batched: null B");
  if (strideA < (int64_t)n * n) return record_arg_error(-4, "lu batched: strideA < n*n");
  if (nrhs > 0 && strideB < (int64_t)n * nrhs) return record_arg_error(-7, "lu batched: strideB < n*nrhs");
  const size_t smem = lu_smem_bytes<T>(n, nrhs);
  const bool exact = (flags & NACU_FLAG_EXACT) != 0;
  auto kern = exact ? lu_batched_kernel<T, true> : lu_batched_kernel<T, false>;
  if (smem > 48 * 1024) {
    cudaError_t e = ensure_dynamic_smem(kern, smem);
    if (e != cudaSuccess) return record_cuda_error(e, name);
  }
  const int grid = batch;  // one CTA per system; the hardware scheduler refills SMs
  const int write_factors = (flags & NACU_FLAG_NO_FACTORS) ? 0 : 1;
  kern<<<grid, kLuThreads, smem, stream>>>(n, nrhs, A, strideA, ipiv, B, strideB, info, batch, mode,
                                           write_factors);
  return check_launch(name);
}

// X_s = I for every system (the right-hand sides of the inverse).
__global__ void identity_batched_kernel(int n, double* X, int64_t stride, int batch) {
  const int64_t nn = (int64_t)n * n, total = nn * batch;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t sys = e / nn, rem = e - sys * nn;
    const int c = (int)(rem / n), r = (int)(rem - (int64_t)c * n);
    X[sys * stride + rem] = (r == c) ? 1.0 : 0.0;
  }
}

}  // namespace
}  // namespace nacu

using nacu::lu_launch;

extern "C" {

int nacu_dgetrf_batched(int n, double* A, int64_t strideA, int32_t* ipiv, int32_t* info, int batch, int flags,
                        nacu_stream_t stream) {
  return lu_launch<double>(n, 0, A, strideA, ipiv, nullptr, 0, info, batch, 0, flags & ~NACU_FLAG_NO_FACTORS,
                           (cudaStream_t)stream, "nacu_dgetrf_batched");
}

int nacu_dgetrs_batched(int n, int nrhs, double* LU, int64_t strideA, int32_t* ipiv, double* B, int64_t strideB,
                        int32_t* info, int batch, int flags, nacu_stream_t stream) {
  return lu_launch<double>(n, nrhs, LU, strideA, ipiv, B, strideB, info, batch, 2, flags, (cudaStream_t)stream,
                           "nacu_dgetrs_batched");
}

// LU::try_inverse (src/linalg/lu.rs:266-297): out = I, then solve_mut(out),
// NACU_LU_BATCHED_MAX_NRHS columns of the identity per solve launch.
int nacu_dgetri_batched(int n, const double* LU, int64_t strideA, const int32_t* ipiv, double* Ainv,
                        int64_t strideInv, int32_t* info, int batch, int flags, nacu_stream_t stream) {
  using namespace nacu;
  const char* name = "nacu_dgetri_batched";
  if (n < 0 || n > NACU_LU_BATCHED_MAX_N) return record_arg_error(-1, "getri batched: n out of range [0, 128]");
  if (batch < 0) return record_arg_error(-8, "getri batched: negative batch");
  if (batch == 0 || n == 0) return NACU_SUCCESS;
  if (!LU || !ipiv || !Ainv || !info) return record_arg_error(-2, "getri batched: null LU, ipiv, Ainv or info");
  if (strideA < (int64_t)n * n) return record_arg_error(-3, "getri batched: strideA < n*n");
  if (strideInv < (int64_t)n * n) return record_arg_error(-6, "getri batched: strideInv < n*n");
  cudaStream_t s = (cudaStream_t)stream;
  const int64_t total = (int64_t)n * n * batch;
  const int grid = (int)std::min<int64_t>((total + 255) / 256, (int64_t)sm_count() * 8);
  identity_batched_kernel<<<grid, 256, 0, s>>>(n, Ainv, strideInv, batch);
  int rc = check_launch(name);
  for (int c0 = 0; c0 < n && rc == NACU_SUCCESS; c0 += NACU_LU_BATCHED_MAX_NRHS) {
    const int nr = std::min(NACU_LU_BATCHED_MAX_NRHS, n - c0);
    rc = lu_launch<double>(n, nr, const_cast<double*>(LU), strideA, const_cast<int32_t*>(ipiv), Ainv + (size_t)c0 * n,
                           strideInv, info, batch, 2, flags, s, name);
  }
  return rc;
}

int nacu_dgesv_batched(int n, int nrhs, double* A, int64_t strideA, int32_t* ipiv, double* B, int64_t strideB,
                       int32_t* info, int batch, int flags, nacu_stream_t stream) {
  return lu_launch<double>(n, nrhs, A, strideA, ipiv, B, strideB, info, batch, 1, flags, (cudaStream_t)stream,
                           "nacu_dgesv_batched");
}

int nacu_sgesv_batched(int n, int nrhs, float* A, int64_t strideA, int32_t* ipiv, float* B, int64_t strideB,
                       int32_t* info, int batch, int flags, nacu_stream_t stream) {
  return lu_launch<float>(n, nrhs, A, strideA, ipiv, B, strideB, info, batch, 1, flags, (cudaStream_t)stream,
                          "nacu_sgesv_batched");
}

}  // extern "C"
