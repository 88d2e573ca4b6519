// Ragged batched SPD solve in mixed precision: FP32 Cholesky factor, FP64
// iterative refinement.  The chosen precision form of nalgebra's
// `m.cholesky().solve(&b)` (src/linalg/cholesky.rs:221-272, 122-143): same
// inputs and outputs as the FP64 form, solutions refined until the normwise
// backward error ||b - A x||_inf / (||A||_inf ||x||_inf + ||b||_inf) is at the
// FP64 target (n * eps64 by default).
//
// Why: on GB300 FP32 runs at ~74x the FP64 rate.  The O(n^3) factorization
// and the triangular solves move to FP32; only the O(n^2) residual
// r = b - A x, the correction accumulation x += d and the fallback stay FP64.
//
// Per matrix (one CTA, persistent grid, largest matrices first):
//   1. A's lower triangle is converted to FP32 into the caller's workspace
//      (A itself is read-only) while ||A||_inf is accumulated;
//   2. FP32 Cholesky (the same left-looking panel code as the FP64 kernel);
//   3. x0 = solve32(b), then repeat: r = b - A x in FP64 (A read from its lower
//      triangle, symmetric), stop if the backward error meets the target, else
//      d = solve32(r) (right-hand sides scaled by powers of two so FP32 never
//      under- or overflows) and x += d in FP64.  After two corrections the
//      contraction rate rho = ||d_k|| / ||d_{k-1}|| predicts the error of the
//      next iterate; when rho * ||d_k|| is far below the target the last
//      residual is skipped (NACU_FLAG_VERIFY forces it).
//   4. A matrix that is not SPD in FP32, or whose refinement stagnates
//      (rho > 1/2) or runs out of iterations, is refactored in FP64 in the
//      workspace and solved there: the per-matrix `iters` output records it.
#include "chol_device.cuh"

namespace nacu {
namespace {

constexpr double kEps64 = 2.220446049250313e-16;

struct MixedArgs {
  int count;
  int n_max;
  const int32_t* ns;
  const int64_t* aoff;
  const double* A;
  int nrhs;
  const int64_t* boff;
  const double* B;
  double* X;
  int32_t* info;
  int32_t* iters;
  const int32_t* order;
  int32_t* counter;
  double* W;  // per matrix n*n doubles at W + aoff[s]
  double tol_units;
  int max_iter;
  int verify;
  int has_subst;
  double subst;
};

__device__ __forceinline__ unsigned long long abs_bits(double x) {
  return (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffull;
}

// max over the CTA of per-thread values (non-negative doubles compared as
// integers: no FP64 instructions); red: kRhsChunk x 4 warps scratch.
__device__ __forceinline__ void block_max4(unsigned long long (&v)[kRhsChunk], unsigned long long* red) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
  for (int c = 0; c < kRhsChunk; ++c) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      const unsigned long long o = __shfl_xor_sync(0xffffffffu, v[c], off);
      v[c] = o > v[c] ? o : v[c];
    }
  }
  __syncthreads();
  if (lane == 0)
#pragma unroll
    for (int c = 0; c < kRhsChunk; ++c) red[warp * kRhsChunk + c] = v[c];
  __syncthreads();
#pragma unroll
  for (int c = 0; c < kRhsChunk; ++c) {
    unsigned long long m = 0;
    for (int w = 0; w < kCholThreads / 32; ++w) m = red[w * kRhsChunk + c] > m ? red[w * kRhsChunk + c] : m;
    v[c] = m;
  }
}

// R = B - A X for the symmetric A stored in its lower triangle (column-major,
// lda = n), nr <= 4 right-hand sides; X and R in shared memory (ld = ldx).
// Thread = row: elements left of the diagonal block come from column j (row
// i of L, coalesced), elements right of it from column i (A_ij = A_ji).
__device__ void residual_fp64(int n, const double* __restrict__ a, const double* __restrict__ b, int nr,
                              const double* Xd, double* Rd, int ldx) {
  const int tid = threadIdx.x;
  for (int rb = (tid >> 5) * 32; rb < n; rb += kCholThreads) {
    const int i = rb + (tid & 31);
    const bool valid = i < n;
    const int ii = valid ? i : n - 1;
    double acc[kRhsChunk];
#pragma unroll
    for (int c = 0; c < kRhsChunk; ++c) acc[c] = (c < nr) ? b[(size_t)c * n + ii] : 0.0;
    const int dend = min(rb + 32, n);
    for (int j = 0; j < rb; ++j) {
      const double aij = a[(size_t)j * n + ii];
#pragma unroll
      for (int c = 0; c < kRhsChunk; ++c) acc[c] = fma(-aij, Xd[(size_t)c * ldx + j], acc[c]);
    }
    for (int j = rb; j < dend; ++j) {
      const double aij = (j <= ii) ? a[(size_t)j * n + ii] : a[(size_t)ii * n + j];
#pragma unroll
      for (int c = 0; c < kRhsChunk; ++c) acc[c] = fma(-aij, Xd[(size_t)c * ldx + j], acc[c]);
    }
    const double* colii = a + (size_t)ii * n;
    for (int j = dend; j < n; ++j) {
      const double aij = colii[j];
#pragma unroll
      for (int c = 0; c < kRhsChunk; ++c) acc[c] = fma(-aij, Xd[(size_t)c * ldx + j], acc[c]);
    }
    if (valid)
#pragma unroll
      for (int c = 0; c < kRhsChunk; ++c)
        if (c < nr) Rd[(size_t)c * ldx + i] = acc[c];
  }
}

// FP32 solve with the FP32 factor: X32 <- L^-T L^-1 (src * 2^-e_c), returned
// in FP64 times 2^e_c (power-of-two scaling: exact, keeps FP32 in range).
__device__ void solve32_scaled(int n, const float* L32, const double* src, int ldsrc, int nr,
                               const unsigned long long* srcnorm, float* X32, const float* rdiag32, int ldx,
                               double* dst, bool accumulate, unsigned long long* dnorm_out,
                               unsigned long long* red) {
  const int tid = threadIdx.x;
  // scale factors 2^-e and 2^e with e = the exponent of ||src_c||_inf, built
  // from the exponent bits (no FP64 instructions)
  __shared__ double s_down[kRhsChunk], s_up[kRhsChunk];
  if (tid < kRhsChunk) {
    long long ex = (long long)((srcnorm[tid] >> 52) & 0x7ff);
    if (ex == 0 || ex == 0x7ff) ex = 1023;  // zero/denormal/inf/NaN: no scaling
    const long long e = ex - 1023;
    const long long e_dn = (e < -1000) ? -1000 : (e > 1000 ? 1000 : e);
    s_down[tid] = __longlong_as_double((1023 - e_dn) << 52);
    s_up[tid] = __longlong_as_double((1023 + e_dn) << 52);
  }
  __syncthreads();
  for (int e = tid; e < n * nr; e += kCholThreads) {
    const int c = e / n, r = e - c * n;
    X32[(size_t)c * ldx + r] = (float)(src[(size_t)c * ldsrc + r] * s_down[c]);
  }
  __syncthreads();
  chol_forward_cta<false, float>(n, L32, X32, ldx, nr, rdiag32);
  chol_backward_fast_cta<float>(n, L32, X32, ldx, nr, rdiag32);
  unsigned long long dn[kRhsChunk] = {0, 0, 0, 0};
  for (int e = tid; e < n * nr; e += kCholThreads) {
    const int c = e / n, r = e - c * n;
    const double d = (double)X32[(size_t)c * ldx + r] * s_up[c];
    const unsigned long long ab = abs_bits(d);
    dn[c] = ab > dn[c] ? ab : dn[c];
    if (accumulate) dst[(size_t)c * ldx + r] += d;
    else dst[(size_t)c * ldx + r] = d;
  }
  block_max4(dn, red);
  if (dnorm_out)
    for (int c = 0; c < kRhsChunk; ++c) dnorm_out[c] = dn[c];
}

__device__ void mixed_one(const MixedArgs& g, int s, unsigned char* smem, int* s_info, double* s_scal,
                          unsigned long long* red) {
  const int tid = threadIdx.x;
  const int n = g.ns[s];
  if (n < 0 || n > g.n_max) {
    if (tid == 0) {
      if (g.info) g.info[s] = -1;
      if (g.iters) g.iters[s] = 0;
    }
    return;
  }
  const int ldp = g.n_max | 1;
  const double* a = g.A + g.aoff[s];
  const double* b = g.B + g.boff[s];
  double* x = g.X + g.boff[s];
  // shared memory: Xd (FP64 x, ldp x 4) | union { FP32: P32, X32, rdiag32, Rd ; FP64: P64, rdiag64 }
  double* Xd = reinterpret_cast<double*>(smem);
  unsigned char* u = smem + (size_t)ldp * kRhsChunk * sizeof(double);
  float* P32 = reinterpret_cast<float*>(u);
  float* X32 = P32 + (size_t)ldp * kNB;
  float* rd32 = X32 + (size_t)ldp * kRhsChunk;
  double* Rd = reinterpret_cast<double*>(u + (((size_t)ldp * (kNB + kRhsChunk + 1) * sizeof(float) + 15) & ~(size_t)15));
  double* P64 = reinterpret_cast<double*>(u);
  double* rd64 = P64 + (size_t)ldp * kNB;
  float* W32 = reinterpret_cast<float*>(g.W + g.aoff[s]);

  // 1. convert A's lower triangle to FP32 (one conversion per element: on
  //    this part an FP64<->FP32 conversion costs an FP64 issue slot), then
  //    ||A||_inf from the FP32 copy (FP32 is enough for a norm that only scales
  //    the stopping test): thread = row, left part from column j, right part
  //    from column i of the lower triangle.
  if (tid == 0) *s_info = 0;
  for (int e = tid; e < n * n; e += kCholThreads) {
    const int c = e / n, r = e - c * n;
    if (r >= c) W32[e] = (float)a[e];
  }
  __syncthreads();
  float an = 0.f;
  for (int i = tid; i < n; i += kCholThreads) {
    float rs = 0.f;
    for (int j = 0; j <= i; ++j) rs += fabsf(W32[(size_t)j * n + i]);
    for (int j = i + 1; j < n; ++j) rs += fabsf(W32[(size_t)i * n + j]);
    an = fmaxf(an, rs);
  }
  unsigned long long bn[kRhsChunk] = {0, 0, 0, 0};
  for (int e = tid; e < n * g.nrhs; e += kCholThreads) {
    const int c = e / n;
    const unsigned long long ab = abs_bits(b[e]);
    if (c < kRhsChunk) bn[c] = ab > bn[c] ? ab : bn[c];
  }
  {
    unsigned long long av[kRhsChunk] = {(unsigned long long)__float_as_uint(an), 0, 0, 0};
    block_max4(av, red);
    an = __uint_as_float((unsigned)av[0]);
  }
  block_max4(bn, red);
  const double anorm = (double)an;
  // 2. FP32 factor.
  chol_factor_cta<false, float>(n, W32, ldp, P32, rd32, s_info, reinterpret_cast<float*>(s_scal), g.has_subst,
                                g.subst);
  int status = *s_info;  // non-zero: not SPD in FP32 -> FP64 fallback
  __syncthreads();
  int used = 0;
  bool converged = false;
  const int nr = g.nrhs;
  const double tol = g.tol_units * (double)(n > 0 ? n : 1) * kEps64;
  if (status == 0 && n > 0) {
    // 3. x0 = solve32(b), then refinement with FP64 residuals.
    solve32_scaled(n, W32, b, n, nr, bn, X32, rd32, ldp, Xd, false, nullptr, red);
    unsigned long long dprev[kRhsChunk] = {0, 0, 0, 0};
    for (int it = 0; it < g.max_iter; ++it) {
      __syncthreads();
      residual_fp64(n, a, b, nr, Xd, Rd, ldp);
      ++used;
      __syncthreads();
      unsigned long long rn[kRhsChunk] = {0, 0, 0, 0}, xn[kRhsChunk] = {0, 0, 0, 0};
      for (int e = tid; e < n * nr; e += kCholThreads) {
        const int c = e / n, r = e - c * n;
        const unsigned long long ra = abs_bits(Rd[(size_t)c * ldp + r]);
        const unsigned long long xa = abs_bits(Xd[(size_t)c * ldp + r]);
        rn[c] = ra > rn[c] ? ra : rn[c];
        xn[c] = xa > xn[c] ? xa : xn[c];
      }
      block_max4(rn, red);
      block_max4(xn, red);
      bool ok = true, finite = true;
      for (int c = 0; c < nr; ++c) {
        if (rn[c] >= 0x7ff0000000000000ull || xn[c] >= 0x7ff0000000000000ull) finite = false;
        const double rr = __longlong_as_double((long long)rn[c]);
        const double den = anorm * __longlong_as_double((long long)xn[c]) + __longlong_as_double((long long)bn[c]);
        if (!(rr <= 0.5 * tol * den)) ok = false;
      }
      if (!finite) break;  // FP32 overflow or a non-finite input: FP64 fallback
      if (ok) {
        converged = true;
        break;
      }
      unsigned long long dn[kRhsChunk];
      solve32_scaled(n, W32, Rd, ldp, nr, rn, X32, rd32, ldp, Xd, true, dn, red);
      // contraction rate and predicted backward error of the new iterate
      bool stagnant = false, predicted = (it >= 1) && !g.verify;
      for (int c = 0; c < nr; ++c) {
        const double d = __longlong_as_double((long long)dn[c]);
        const double dp = __longlong_as_double((long long)dprev[c]);
        const double rho = (it >= 1 && dp > 0.0) ? d / dp : 1.0;
        if (it >= 1 && rho > 0.5) stagnant = true;
        const double den = anorm * __longlong_as_double((long long)xn[c]) + __longlong_as_double((long long)bn[c]);
        if (!(anorm * rho * d <= 0.125 * tol * den)) predicted = false;
        dprev[c] = dn[c];
      }
      if (stagnant) break;
      if (predicted) {
        converged = true;
        break;
      }
    }
  }
  __syncthreads();
  if (!converged && n > 0) {
    // 4. FP64 fallback in the workspace (A stays untouched).
    double* W64 = g.W + g.aoff[s];
    for (int e = tid; e < n * n; e += kCholThreads) W64[e] = a[e];
    if (tid == 0) *s_info = 0;
    __syncthreads();
    chol_factor_cta<false, double>(n, W64, ldp, P64, rd64, s_info, s_scal, g.has_subst, g.subst);
    status = *s_info;
    if (status == 0) {
      for (int e = tid; e < n * nr; e += kCholThreads) {
        const int c = e / n, r = e - c * n;
        Xd[(size_t)c * ldp + r] = b[e];
      }
      __syncthreads();
      chol_forward_cta<false, double>(n, W64, Xd, ldp, nr, rd64);
      chol_backward_fast_cta<double>(n, W64, Xd, ldp, nr, rd64);
    }
  }
  __syncthreads();
  if (status == 0)
    for (int e = tid; e < n * nr; e += kCholThreads) {
      const int c = e / n, r = e - c * n;
      x[e] = Xd[(size_t)c * ldp + r];
    }
  if (tid == 0) {
    if (g.info) g.info[s] = status;
    if (g.iters) g.iters[s] = converged ? used : -(used + 1);
  }
  __syncthreads();
}

__global__ void __launch_bounds__(kCholThreads, 4) chol_mixed_kernel(MixedArgs g) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_item;
  __shared__ int s_info;
  __shared__ double s_scal[2 + kCholThreads / 32];
  __shared__ unsigned long long red[4 * kRhsChunk];
  for (;;) {
    if (threadIdx.x == 0) s_item = atomicAdd(g.counter, 1);
    __syncthreads();
    const int idx = s_item;
    __syncthreads();
    if (idx >= g.count) break;
    const int s = g.order ? g.order[idx] : idx;
    mixed_one(g, s, smem_raw, &s_info, s_scal, red);
  }
}

size_t mixed_smem_bytes(int n_max) {
  const size_t ldp = (size_t)(n_max | 1);
  const size_t xd = ldp * kRhsChunk * sizeof(double);
  const size_t fp32 = ((ldp * (kNB + kRhsChunk + 1) * sizeof(float) + 15) & ~(size_t)15) + ldp * kRhsChunk * sizeof(double);
  const size_t fp64 = ldp * (kNB + 1) * sizeof(double);
  return xd + (fp32 > fp64 ? fp32 : fp64);
}

}  // namespace
}  // namespace nacu

extern "C" {

size_t nacu_mixed_workspace_bytes(int64_t total_matrix_elements) {
  return 256 + (size_t)total_matrix_elements * sizeof(double);
}

int nacu_dposv_ragged_mixed(int count, int n_max, const int32_t* ns, const int64_t* a_offsets, const double* A,
                            int nrhs, const int64_t* b_offsets, const double* B, double* X, int32_t* info,
                            int32_t* iters, const int32_t* order, int64_t total_matrix_elements, void* workspace,
                            size_t workspace_bytes, double tol_units, int max_iter, double substitute, int flags,
                            nacu_stream_t stream) {
  using namespace nacu;
  if (count < 0) return record_arg_error(-1, "dposv_ragged_mixed: negative count");
  if (n_max < 0 || n_max > NACU_CHOL_RAGGED_MAX_N)
    return record_arg_error(-2, "dposv_ragged_mixed: n_max out of range [0, 512]");
  if (count == 0) return NACU_SUCCESS;
  if (!ns || !a_offsets || !A) return record_arg_error(-3, "dposv_ragged_mixed: null ns, a_offsets or A");
  if (nrhs < 1 || nrhs > kRhsChunk) return record_arg_error(-6, "dposv_ragged_mixed: nrhs out of range [1, 4]");
  if (!b_offsets || !B || !X) return record_arg_error(-7, "dposv_ragged_mixed: null b_offsets, B or X");
  if (!info) return record_arg_error(-10, "dposv_ragged_mixed: null info");
  if (total_matrix_elements < 0) return record_arg_error(-13, "dposv_ragged_mixed: negative total_matrix_elements");
  if (!workspace || workspace_bytes < nacu_mixed_workspace_bytes(total_matrix_elements))
    return record_arg_error(-14, "dposv_ragged_mixed: workspace too small");
  if (flags & NACU_FLAG_EXACT) return record_arg_error(-19, "dposv_ragged_mixed: NACU_FLAG_EXACT does not apply");
  MixedArgs g{count, n_max, ns, a_offsets, A, nrhs, b_offsets, B, X, info, iters, order,
              reinterpret_cast<int32_t*>(workspace),
              reinterpret_cast<double*>(static_cast<unsigned char*>(workspace) + 256),
              tol_units > 0.0 ? tol_units : 1.0, max_iter > 0 ? max_iter : 10,
              (flags & NACU_FLAG_VERIFY) ? 1 : 0, (flags & NACU_FLAG_SUBSTITUTE) ? 1 : 0, substitute};
  const size_t smem = mixed_smem_bytes(n_max);
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = cudaFuncSetAttribute(chol_mixed_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return record_cuda_error(e, "nacu_dposv_ragged_mixed");
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, chol_mixed_kernel, kCholThreads, smem);
  if (e != cudaSuccess) return record_cuda_error(e, "nacu_dposv_ragged_mixed");
  if (per_sm < 1) per_sm = 1;
  int grid = sm_count() * per_sm;
  if (grid > count) grid = count;
  e = cudaMemsetAsync(workspace, 0, sizeof(int32_t), s);
  if (e != cudaSuccess) return record_cuda_error(e, "nacu_dposv_ragged_mixed");
  chol_mixed_kernel<<<grid, kCholThreads, smem, s>>>(g);
  return check_launch("nacu_dposv_ragged_mixed");
}

}  // extern "C"
