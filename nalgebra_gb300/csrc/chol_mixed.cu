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
//      (A itself is read-only); ||A||_inf comes from the first FP64 residual;
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

__device__ __forceinline__ unsigned long long abs_bits(double x) { return abs_bits_f64(x); }

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
__device__ __noinline__ void residual_fp64(int n, const double* __restrict__ a, const double* __restrict__ b, int nr,
                              const double* Xd, double* Rd, int ldx, bool with_norm, float* rowmax) {
  constexpr int U = 8;  // independent loads in flight per thread
  const int tid = threadIdx.x;
  float my_rowmax = 0.0f;
  for (int rb = (tid >> 5) * 32; rb < n; rb += kCholThreads) {
    const int i = rb + (tid & 31);
    const bool valid = i < n;
    const int ii = valid ? i : n - 1;
    double acc[kRhsChunk];
#pragma unroll
    for (int c = 0; c < kRhsChunk; ++c) acc[c] = (c < nr) ? b[(size_t)c * n + ii] : 0.0;
    float rs = 0.0f;  // sum |A_ij| over the row in FP32 (first residual only; off the FP64 pipe)
    const int dend = min(rb + 32, n);
    const double* colii = a + (size_t)ii * n;
    // element (ii, j): column j (left of / in the diagonal block, j <= ii) or
    // column ii (right of it), both from the lower triangle
    for (int j0 = 0; j0 < n; j0 += U) {
      double av[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int j = j0 + u;
        av[u] = (j < n) ? ((j <= ii && j < dend) ? a[(size_t)j * n + ii] : colii[j]) : 0.0;
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int j = j0 + u;
        if (j < n) {
          if (with_norm) rs += abs_f32_lower(av[u]);
#pragma unroll
          for (int c = 0; c < kRhsChunk; ++c) acc[c] = fma(-av[u], Xd[(size_t)c * ldx + j], acc[c]);
        }
      }
    }
    if (valid && rs > my_rowmax) my_rowmax = rs;
    if (valid)
#pragma unroll
      for (int c = 0; c < kRhsChunk; ++c)
        if (c < nr) Rd[(size_t)c * ldx + i] = acc[c];
  }
  if (with_norm) *rowmax = my_rowmax;
}

// block_max4 whose result goes to shared memory (out[0..kRhsChunk)), so the
// norms do not occupy registers across the solves.
__device__ __forceinline__ void block_max4_to(unsigned long long (&v)[kRhsChunk], unsigned long long* red,
                                              unsigned long long* out) {
  block_max4(v, red);
  if (threadIdx.x < kRhsChunk) out[threadIdx.x] = v[threadIdx.x & (kRhsChunk - 1)];
  __syncthreads();
}

// FP32 solve with the FP32 factor: X32 <- L^-T L^-1 (src * 2^-e_c), returned
// in FP64 times 2^e_c (power-of-two scaling: exact, keeps FP32 in range).
__device__ __noinline__ void solve32_scaled(int n, const float* L32, const double* src, int ldsrc, int nr,
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
  for (int c = 0; c < nr; ++c)
    for (int r = tid; r < n; r += kCholThreads) X32[(size_t)c * ldx + r] = (float)(src[(size_t)c * ldsrc + r] * s_down[c]);
  __syncthreads();
  chol_forward_cta<false, float>(n, L32, X32, ldx, nr, rdiag32);
  chol_backward_fast_cta<float>(n, L32, X32, ldx, nr, rdiag32);
  unsigned long long dn[kRhsChunk] = {0, 0, 0, 0};
#pragma unroll
  for (int c = 0; c < kRhsChunk; ++c)
    if (c < nr)
      for (int r = tid; r < n; r += kCholThreads) {
        const double d = (double)X32[(size_t)c * ldx + r] * s_up[c];
        const unsigned long long ab = abs_bits(d);
        dn[c] = ab > dn[c] ? ab : dn[c];
        if (accumulate) dst[(size_t)c * ldx + r] += d;
        else dst[(size_t)c * ldx + r] = d;
      }
  if (dnorm_out) block_max4_to(dn, red, dnorm_out);
}

// FP32 left-looking Cholesky for the refinement form.  Same panel structure as
// chol_factor_cta, but the panel itself is factored by warp 0 alone
// (warp-synchronous, no CTA barriers per column): in FP32 the arithmetic is
// cheap and the per-column barriers, not the math, set the time.
// Lb: kKB staged columns of L with leading dimension ldl (a multiple of 4 that
// covers n_max + kRowsPerPass padding: float4 reads past `rows` stay inside the
// buffer and only feed discarded accumulators).
__device__ __noinline__ void chol_factor32_cta(int n, float* __restrict__ a, int ldp, float* __restrict__ P, float* Lb,
                                  int ldl, float* Hs, float* rdiag, int* s_info, int has_subst, double subst) {
  constexpr int kKB = 8;  // columns of L staged per block
  const int tid = threadIdx.x;
  const int nthr = blockDim.x;
  const int warp = tid >> 5, lane = tid & 31;
  for (int J0 = 0; J0 < n; J0 += kNB) {
    const int jb = min(kNB, n - J0);
    const int rows = n - J0;
    // P = A[J0.., J0..J0+jb] - L[J0.., 0..J0] L[J0..J0+jb, 0..J0]^T: the
    // earlier columns are staged kKB at a time in shared memory (one batch of
    // independent coalesced loads per block instead of a dependent load per k).
    const int cg = warp * 4;  // 4 warps x 4 columns = kNB
    for (int rb = 0; rb < rows; rb += kRowsPerPass) {
      // lane owns rows rb + 4*lane + 128*h + {0..3}, h = 0, 1
      float acc[2][4][4];  // [h][row][col]
#pragma unroll
      for (int h = 0; h < 2; ++h)
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            const int r = rb + 4 * lane + 128 * h + i, c = cg + j;
            acc[h][i][j] = (r < rows && c < jb && r >= c) ? a[(size_t)(J0 + c) * n + J0 + r] : 0.f;
          }
      for (int kb = 0; kb < J0; kb += kKB) {
        const int kw = min(kKB, J0 - kb);
        __syncthreads();
        {  // stage L[J0.., kb..kb+kw): a warp per column, eight coalesced
           // loads in flight per lane, then the shared stores.  No index
           // division per element: the staged elements number the panel's
           // FMAs / 16, and an integer division costs ~20 instructions.
          for (int c = warp; c < kw; c += nthr >> 5) {
            const float* src = a + (size_t)(kb + c) * n + J0;
            float* dst = Lb + (size_t)c * ldl;
            for (int r0 = 0; r0 < rows; r0 += 8 * 32) {
              float v[8];
#pragma unroll
              for (int u = 0; u < 8; ++u) {
                const int r = r0 + u * 32 + lane;
                v[u] = (r < rows) ? src[r] : 0.f;
              }
#pragma unroll
              for (int u = 0; u < 8; ++u) {
                const int r = r0 + u * 32 + lane;
                if (r < rows) dst[r] = v[u];
              }
            }
          }
        }
        __syncthreads();
        if (cg < jb) {
#pragma unroll 2
          for (int k = 0; k < kw; ++k) {
            const float* lk = Lb + (size_t)k * ldl;
            const float4 lc = *reinterpret_cast<const float4*>(lk + cg);  // L[cg..cg+3][k]
            float4 lr[2];
#pragma unroll
            for (int h = 0; h < 2; ++h)
              lr[h] = (rb + 4 * lane + 128 * h < rows) ? *reinterpret_cast<const float4*>(lk + rb + 4 * lane + 128 * h)
                                                       : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
            for (int h = 0; h < 2; ++h) {
              const float rv[4] = {lr[h].x, lr[h].y, lr[h].z, lr[h].w};
              const float cv[4] = {lc.x, lc.y, lc.z, lc.w};
#pragma unroll
              for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[h][i][j] = fmaf(-cv[j], rv[i], acc[h][i][j]);
            }
          }
        }
      }
#pragma unroll
      for (int h = 0; h < 2; ++h)
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            const int r = rb + 4 * lane + 128 * h + i, c = cg + j;
            if (r < rows && c < jb && r >= c) P[(size_t)c * ldp + r] = acc[h][i][j];
          }
    }
    __syncthreads();
    // Panel, without CTA barriers per column: every warp factors the jb x jb
    // head of the panel redundantly (lanes 0..jb-1 hold its rows in
    // registers), keeps L_head and 1/L_jj in its own shared scratch, then
    // updates its share of the rows below the head, each row entirely in
    // registers.
    {
      float* hl = Hs + warp * (kNB * kNB + kNB);  // L_head[c][j] at hl[j*kNB + c], 1/L_jj at hl[kNB*kNB + j]
      float v[kNB];
#pragma unroll
      for (int c = 0; c < kNB; ++c) v[c] = (lane < jb && c <= lane && c < jb) ? P[(size_t)c * ldp + lane] : 0.f;
      bool fail = false;
#pragma unroll
      for (int j = 0; j < kNB; ++j) {
        if (j < jb && !fail) {
          const float d = __shfl_sync(0xffffffffu, v[j], j);
          float denom, rcp;
          if (!chol_pivot<false, float>(d, has_subst, subst, &denom, &rcp)) {
            fail = true;
            if (warp == 0 && lane == 0) *s_info = J0 + j + 1;
          } else {
            if (lane == j) v[j] = denom;
            else if (lane > j) v[j] *= rcp;
            if (lane == 0) hl[kNB * kNB + j] = rcp;
#pragma unroll
            for (int c = j + 1; c < kNB; ++c) {
              const float lcj = __shfl_sync(0xffffffffu, v[j], c);  // L[c][j]
              if (c < jb && lane >= c) v[c] = fmaf(-v[j], lcj, v[c]);
            }
          }
        }
      }
      if (lane < jb)
#pragma unroll
        for (int j = 0; j < kNB; ++j) hl[j * kNB + lane] = v[j];  // row `lane` of L_head
      __syncwarp();
      if (!fail) {
        if (warp == 0 && lane < jb) {
#pragma unroll
          for (int c = 0; c < kNB; ++c)
            if (c <= lane && c < jb) P[(size_t)c * ldp + lane] = v[c];
          rdiag[J0 + lane] = hl[kNB * kNB + lane];
        }
        for (int r = jb + warp * 32 + lane; r < rows; r += nthr) {
          float w[kNB];
#pragma unroll
          for (int c = 0; c < kNB; ++c) w[c] = (c < jb) ? P[(size_t)c * ldp + r] : 0.f;
#pragma unroll
          for (int j = 0; j < kNB; ++j) {
            w[j] *= hl[kNB * kNB + j];  // L[r][j]; zero columns stay zero
#pragma unroll
            for (int c = j + 1; c < kNB; ++c) w[c] = fmaf(-w[j], hl[j * kNB + c], w[c]);
            // keep the compiler from hoisting all 136 head loads into registers
            asm volatile("" ::: "memory");
          }
#pragma unroll
          for (int c = 0; c < kNB; ++c)
            if (c < jb) P[(size_t)c * ldp + r] = w[c];
        }
      }
    }
    __syncthreads();
    if (*s_info != 0) return;
    for (int c = warp; c < jb; c += nthr >> 5)
      for (int r = c + lane; r < rows; r += 32) a[(size_t)(J0 + c) * n + J0 + r] = P[(size_t)c * ldp + r];
    __syncthreads();
  }
}

// Dynamic shared memory of the refinement kernel (byte offsets):
//   X32  (ldp x 4 floats)  FP32 right-hand sides / solutions
//   rd32 (ldp floats)      1 / L_ii of the FP32 factor
//   u    union { P32 panel (ldp x kNB floats) ; Rd residual (ldp x 4 doubles) }
//   xd   union { staged L columns (ldl x 8 floats) during the factor ;
//                Xd, the FP64 iterate (ldp x 4 doubles) }
struct MixedSmem {
  size_t x32, rd32, u, xd, total;
  int ldl;
};
constexpr int kHeadFloats = (kCholThreads / 32) * (kNB * kNB + kNB);
__host__ __device__ inline MixedSmem mixed_smem_layout(int n_max) {
  MixedSmem L;
  const size_t ldp = (size_t)(n_max | 1);
  L.ldl = ((n_max + 3 + 3) / 4) * 4;  // float4 reads may run 3 past the last row
  auto up16 = [](size_t x) { return (x + 15) & ~(size_t)15; };
  L.x32 = 0;
  // X32 is idle during the factor: the per-warp 16 x 16 heads of the FP32
  // panel share its space (no static shared memory for them)
  const size_t x32 = ldp * kRhsChunk * sizeof(float), heads = (size_t)kHeadFloats * sizeof(float);
  L.rd32 = up16(L.x32 + (x32 > heads ? x32 : heads));
  L.u = up16(L.rd32 + ldp * sizeof(float));
  const size_t p32 = ldp * kNB * sizeof(float), rd = ldp * kRhsChunk * sizeof(double);
  L.xd = up16(L.u + (p32 > rd ? p32 : rd));
  const size_t xd = ldp * kRhsChunk * sizeof(double), lb = (size_t)L.ldl * 8 * sizeof(float);
  L.total = up16(L.xd + (xd > lb ? xd : lb));
  return L;
}

// Norms kept in shared memory (indices into nrm[]).
constexpr int kBn = 0, kRn = 4, kXn = 8, kDn = 12, kDprev = 16, kNrmSize = 20;

__device__ void mixed_one(const MixedArgs& g, int s, unsigned char* smem, int* s_info, double* s_scal,
                          unsigned long long* red, float* hs, unsigned long long* nrm) {
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
  // shared memory: Xd (FP64 x, ldp x 4) | X32 (ldp x 4) | rdiag32 (ldp) |
  // { P32 (ldp x kNB floats) during the factor, Rd (ldp x 4 doubles) after }
  MixedSmem L = mixed_smem_layout(g.n_max);
  float* X32 = reinterpret_cast<float*>(smem + L.x32);
  float* rd32 = reinterpret_cast<float*>(smem + L.rd32);
  float* P32 = reinterpret_cast<float*>(smem + L.u);
  double* Rd = reinterpret_cast<double*>(smem + L.u);
  double* Xd = reinterpret_cast<double*>(smem + L.xd);
  float* lb32 = reinterpret_cast<float*>(smem + L.xd);  // staged L columns during the factor
  const int ldl = L.ldl;
  float* W32 = reinterpret_cast<float*>(g.W + g.aoff[s]);

  // 1. convert A's lower triangle to FP32 (one conversion per element: on
  //    this part a hardware FP64<->FP32 conversion costs an FP64 issue slot,
  //    so the normal-range conversion is done with integer instructions).
  //    Only the lower triangle is read: warp w takes the column pairs
  //    (c, n-1-c), c = w, w + 4, ..., whose n + 1 rows are one run of
  //    coalesced 32-row chunks, up to 9 loads in flight per lane.
  //    ||A||_inf is accumulated by the first FP64 residual pass.
  if (tid == 0) *s_info = 0;
  {
    constexpr int U = 9;
    const int warp = tid >> 5, lane = tid & 31;
    for (int c = warp; c < (n + 1) / 2; c += kCholThreads / 32) {
      const int c2 = n - 1 - c;
      const int len1 = n - c;                             // rows c..n-1 of column c
      const int len = (c2 == c) ? len1 : len1 + (c + 1);  // and rows c2..n-1 of column c2
      for (int k0 = 0; k0 < len; k0 += U * 32) {
        double v[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int k = k0 + u * 32 + lane;
          const int idx = (k < len1) ? c * n + c + k : c2 * n + c2 + (k - len1);  // n*n < 2^31
          v[u] = (k < len) ? a[idx] : 0.0;
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int k = k0 + u * 32 + lane;
          const int idx = (k < len1) ? c * n + c + k : c2 * n + c2 + (k - len1);
          if (k < len) W32[idx] = f64_to_f32_rn(v[u]);
        }
      }
    }
  }
  {
    unsigned long long bv[kRhsChunk] = {0, 0, 0, 0};
#pragma unroll
    for (int c = 0; c < kRhsChunk; ++c)
      if (c < g.nrhs)
        for (int r = tid; r < n; r += kCholThreads) {
          const unsigned long long ab = abs_bits(b[(size_t)c * n + r]);
          bv[c] = ab > bv[c] ? ab : bv[c];
        }
    block_max4_to(bv, red, nrm + kBn);
  }
  double anorm = 0.0;
  // 2. FP32 factor.
  chol_factor32_cta(n, W32, ldp, P32, lb32, ldl, hs, rd32, s_info, g.has_subst, g.subst);
  int status = *s_info;  // non-zero: not SPD in FP32 -> FP64 fallback
  __syncthreads();
  int used = 0;
  bool converged = false;
  const int nr = g.nrhs;
  const double tol = g.tol_units * (double)(n > 0 ? n : 1) * kEps64;
  if (status == 0 && n > 0) {
    // 3. x0 = solve32(b), then refinement with FP64 residuals.
    solve32_scaled(n, W32, b, n, nr, nrm + kBn, X32, rd32, ldp, Xd, false, nullptr, red);
    if (tid < kRhsChunk) nrm[kDprev + tid] = 0;
    for (int it = 0; it < g.max_iter; ++it) {
      __syncthreads();
      float rowmax = 0.0f;
      residual_fp64(n, a, b, nr, Xd, Rd, ldp, it == 0, &rowmax);
      ++used;
      __syncthreads();
      if (it == 0) {  // ||A||_inf: max over the CTA (integer compare on the bits)
        unsigned long long av[kRhsChunk] = {(unsigned long long)__float_as_uint(rowmax), 0, 0, 0};
        block_max4(av, red);
        anorm = (double)__uint_as_float((unsigned)av[0]);  // FP32 row sums; inf only past FLT_MAX
      }
      {
        unsigned long long rn[kRhsChunk] = {0, 0, 0, 0}, xn[kRhsChunk] = {0, 0, 0, 0};
#pragma unroll
        for (int c = 0; c < kRhsChunk; ++c)
          if (c < nr)
            for (int r = tid; r < n; r += kCholThreads) {
              const unsigned long long ra = abs_bits(Rd[(size_t)c * ldp + r]);
              const unsigned long long xa = abs_bits(Xd[(size_t)c * ldp + r]);
              rn[c] = ra > rn[c] ? ra : rn[c];
              xn[c] = xa > xn[c] ? xa : xn[c];
            }
        block_max4_to(rn, red, nrm + kRn);
        block_max4_to(xn, red, nrm + kXn);
      }
      bool ok = true, finite = !isinf(anorm);  // ||A||_inf beyond FP32: the FP64 form takes over
      for (int c = 0; c < nr; ++c) {
        if (nrm[kRn + c] >= 0x7ff0000000000000ull || nrm[kXn + c] >= 0x7ff0000000000000ull) finite = false;
        const double rr = __longlong_as_double((long long)nrm[kRn + c]);
        const double den = anorm * __longlong_as_double((long long)nrm[kXn + c]) +
                           __longlong_as_double((long long)nrm[kBn + c]);
        if (!(rr <= 0.5 * tol * den)) ok = false;
      }
      if (!finite) break;  // FP32 overflow or a non-finite input: FP64 fallback
      if (ok) {
        converged = true;
        break;
      }
      solve32_scaled(n, W32, Rd, ldp, nr, nrm + kRn, X32, rd32, ldp, Xd, true, nrm + kDn, red);
      // contraction rate and predicted backward error of the new iterate
      bool stagnant = false, predicted = (it >= 1) && !g.verify;
      for (int c = 0; c < nr; ++c) {
        const double d = __longlong_as_double((long long)nrm[kDn + c]);
        const double dp = __longlong_as_double((long long)nrm[kDprev + c]);
        const double rho = (it >= 1 && dp > 0.0) ? d / dp : 1.0;
        if (it >= 1 && rho > 0.5) stagnant = true;
        const double den = anorm * __longlong_as_double((long long)nrm[kXn + c]) +
                           __longlong_as_double((long long)nrm[kBn + c]);
        if (!(anorm * rho * d <= 0.125 * tol * den)) predicted = false;
      }
      __syncthreads();
      if (tid < kRhsChunk) nrm[kDprev + tid] = nrm[kDn + tid];
      if (stagnant) break;
      if (predicted) {
        converged = true;
        break;
      }
    }
  }
  __syncthreads();
  if (!converged && n > 0) {
    // 4. queue the matrix for the FP64 fallback kernel (runs after this one)
    if (tid == 0) {
      const int slot = atomicAdd(g.counter + 1, 1);
      g.counter[4 + slot] = s;
      if (g.info) g.info[s] = 0;
      if (g.iters) g.iters[s] = -(used + 1);
    }
    __syncthreads();
    return;
  }
  if (status == 0)
    for (int c = 0; c < nr; ++c)
      for (int r = tid; r < n; r += kCholThreads) x[(size_t)c * n + r] = Xd[(size_t)c * ldp + r];
  if (tid == 0) {
    if (g.info) g.info[s] = status;
    if (g.iters) g.iters[s] = used;
  }
  __syncthreads();
}

// FP64 fallback for the matrices the refinement kernel queued: factor a copy
// of A in the workspace and solve, exactly the FP64 form's arithmetic.
__global__ void __launch_bounds__(kCholThreads, 4) chol_mixed_fallback_kernel(MixedArgs g) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_item;
  __shared__ int s_info;
  __shared__ double s_scal[2 + kCholThreads / 32];
  const int tid = threadIdx.x;
  const int ldp = g.n_max | 1;
  double* P64 = reinterpret_cast<double*>(smem_raw);
  double* Xd = P64 + (size_t)ldp * kNB;
  double* rd64 = Xd + (size_t)ldp * kRhsChunk;
  for (;;) {
    if (tid == 0) s_item = atomicAdd(g.counter + 2, 1);
    __syncthreads();
    const int idx = s_item;
    __syncthreads();
    if (idx >= g.counter[1]) break;
    const int s = g.counter[4 + idx];
    const int n = g.ns[s];
    const int nr = g.nrhs;
    const double* a = g.A + g.aoff[s];
    const double* b = g.B + g.boff[s];
    double* x = g.X + g.boff[s];
    double* W64 = g.W + g.aoff[s];
    for (int e = tid; e < n * n; e += kCholThreads) W64[e] = a[e];
    if (tid == 0) s_info = 0;
    __syncthreads();
    chol_factor_cta<false, double>(n, W64, ldp, P64, rd64, &s_info, s_scal, g.has_subst, g.subst);
    const int status = s_info;
    if (status == 0) {
      for (int e = tid; e < n * nr; e += kCholThreads) {
        const int c = e / n, r = e - c * n;
        Xd[(size_t)c * ldp + r] = b[e];
      }
      __syncthreads();
      chol_forward_cta<false, double>(n, W64, Xd, ldp, nr, rd64);
      chol_backward_fast_cta<double>(n, W64, Xd, ldp, nr, rd64);
      for (int e = tid; e < n * nr; e += kCholThreads) {
        const int c = e / n, r = e - c * n;
        x[e] = Xd[(size_t)c * ldp + r];
      }
    }
    if (tid == 0 && g.info) g.info[s] = status;
    __syncthreads();
  }
}

__global__ void __launch_bounds__(kCholThreads, 7) chol_mixed_kernel(MixedArgs g) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_item;
  __shared__ int s_info;
  __shared__ double s_scal[2 + kCholThreads / 32];
  __shared__ unsigned long long red[4 * kRhsChunk];
  __shared__ unsigned long long nrm[kNrmSize];
  float* hs = reinterpret_cast<float*>(smem_raw + mixed_smem_layout(g.n_max).x32);
  for (;;) {
    if (threadIdx.x == 0) s_item = atomicAdd(g.counter, 1);
    __syncthreads();
    const int idx = s_item;
    __syncthreads();
    if (idx >= g.count) break;
    const int s = g.order ? g.order[idx] : idx;
    mixed_one(g, s, smem_raw, &s_info, s_scal, red, hs, nrm);
  }
}

size_t mixed_smem_bytes(int n_max) { return mixed_smem_layout(n_max).total; }

size_t fallback_smem_bytes(int n_max) {
  const size_t ldp = (size_t)(n_max | 1);
  return ldp * (kNB + kRhsChunk + 1) * sizeof(double);
}

}  // namespace
}  // namespace nacu

extern "C" {

// Workspace: [0,16): queue heads; [16, 16 + 4*count): fallback list, rounded
// up to 256; then 8 bytes per matrix element (FP32 factor or FP64 fallback).
static size_t mixed_head_bytes(int count) { return ((size_t)16 + 4 * (size_t)count + 255) & ~(size_t)255; }

size_t nacu_mixed_workspace_bytes(int count, int64_t total_matrix_elements) {
  return mixed_head_bytes(count) + (size_t)total_matrix_elements * sizeof(double);
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
  if (!workspace || workspace_bytes < nacu_mixed_workspace_bytes(count, total_matrix_elements))
    return record_arg_error(-14, "dposv_ragged_mixed: workspace too small");
  if (flags & NACU_FLAG_EXACT) return record_arg_error(-19, "dposv_ragged_mixed: NACU_FLAG_EXACT does not apply");
  MixedArgs g{count, n_max, ns, a_offsets, A, nrhs, b_offsets, B, X, info, iters, order,
              reinterpret_cast<int32_t*>(workspace),
              reinterpret_cast<double*>(static_cast<unsigned char*>(workspace) + mixed_head_bytes(count)),
              tol_units > 0.0 ? tol_units : 1.0, max_iter > 0 ? max_iter : 10,
              (flags & NACU_FLAG_VERIFY) ? 1 : 0, (flags & NACU_FLAG_SUBSTITUTE) ? 1 : 0, substitute};
  const size_t smem = mixed_smem_bytes(n_max);
  const size_t smem_fb = fallback_smem_bytes(n_max);
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = ensure_dynamic_smem(chol_mixed_kernel, smem);
  if (e == cudaSuccess)
    e = ensure_dynamic_smem(chol_mixed_fallback_kernel, smem_fb);
  if (e != cudaSuccess) return record_cuda_error(e, "nacu_dposv_ragged_mixed");
  int per_sm = 0, per_sm_fb = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, chol_mixed_kernel, kCholThreads, smem);
  if (e == cudaSuccess)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_fb, chol_mixed_fallback_kernel, kCholThreads, smem_fb);
  if (e != cudaSuccess) return record_cuda_error(e, "nacu_dposv_ragged_mixed");
  int grid = sm_count() * (per_sm < 1 ? 1 : per_sm);
  if (grid > count) grid = count;
  int grid_fb = sm_count() * (per_sm_fb < 1 ? 1 : per_sm_fb);
  if (grid_fb > count) grid_fb = count;
  e = cudaMemsetAsync(workspace, 0, 16, s);
  if (e != cudaSuccess) return record_cuda_error(e, "nacu_dposv_ragged_mixed");
  chol_mixed_kernel<<<grid, kCholThreads, smem, s>>>(g);
  int rc = check_launch("nacu_dposv_ragged_mixed");
  if (rc != NACU_SUCCESS) return rc;
  // Runs after the refinement kernel on the same stream; exits at once when
  // no matrix was queued.
  chol_mixed_fallback_kernel<<<grid_fb, kCholThreads, smem_fb, s>>>(g);
  return check_launch("nacu_dposv_ragged_mixed: fallback");
}

}  // extern "C"
