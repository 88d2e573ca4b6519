// Batched Householder QR and least squares for tall-skinny systems
// (m >= n, n <= 64): the GPU form of nalgebra's `m.qr()`
// (src/linalg/qr.rs:55-76, householder.rs:19-85, geometry/reflection.rs:70-83),
// `q_tr_mul` (qr.rs:157-171) and the least-squares solve of nalgebra-lapack
// (nalgebra-lapack/src/qr_util.rs:167-239: Q^T b, then the upper-triangular
// solve with R[0:n, 0:n], dividing by |diag_i| as qr.rs:224-256 does).
//
// Sign convention.  nalgebra applies each reflection with a sign,
// c <- s_i * (I - 2 v v^T) c with s_i = signum(diag_i) (householder.rs:75-82).
// Writing D_i for the diagonal matrix that is s_i on rows >= i and 1 above,
// nalgebra's transform is D_{n-1} H_{n-1} ... D_0 H_0, and every D_i commutes
// with the later H_j (H_j touches rows >= j > i, where D_i is a scalar), so it
// equals D H_{n-1} ... H_0 with D = diag(d_r), d_r = prod_{i <= min(r, n-1)} s_i.
// The reflections themselves do not depend on the signs (a reflection axis is
// defined up to sign).  So the kernel runs plain Householder QR in compact-WY
// blocks, then one sign sweep gives nalgebra's stored factors exactly:
//   diag_i  = P_i * diag_std_i   (P_i = prod_{j<i} s_j, s_i = signum(diag_i)),
//   axis_i  = P_i * v_i          (the stored unit axis),
//   R[r][c] = d_r * R_std[r][c]  (strict upper part), Q^T b rows likewise,
// and the least-squares solution does not change at all (D cancels).
//
// Design (GB300): FP64-pipe bound like the other solvers.  One CTA (128
// threads) per problem; problems are pulled from a work queue (largest first).
// The matrix stays in global memory (L2-resident while the CTA works on it);
// each 8-column panel is factored in shared memory, then the trailing columns
// and the right-hand side take the block reflector I - V T^T V^T, one warp per
// four columns: one pass computes V^T a (8 partial dots per column and lane,
// one butterfly reduce-scatter for the 32 sums), one pass applies
// a -= V (T^T V^T a); each shared-memory axis value feeds four FMAs.
#include "common.cuh"

namespace nacu {
namespace {

constexpr int kQrThreads = 128;
constexpr int kQrNB = 8;
constexpr int kQrMaxN = 128;
// s_t layout: T (NB x NB) | tau (NB) | scratch (128) | V^T V strict upper part (28, padded to 32)
constexpr int kTOff = 0;
constexpr int kTauOff = kQrNB * kQrNB;
constexpr int kGOff = kTauOff + kQrNB;            // scratch (1 / |diag_i| of the back substitution)
constexpr int kGSumOff = kGOff + 4 * 32;           // 28 reduced pairs (i < j)
constexpr int kSTSize = kGSumOff + 32;

struct QrArgs {
  int count;
  int n;
  int m_max;
  const int32_t* ms;    // null: every problem is m_uni x n
  const int64_t* aoff;  // null: problem s at A + s * strideA
  double* A;
  const int64_t* boff;  // null with B set: b of problem s at B + s * strideB
  double* B;            // nullable: factor only
  double* X;      // n per problem, nullable
  double* diag;   // n per problem
  int32_t* info;
  const int32_t* order;
  int32_t* counter;     // null: problems taken grid-stride (no queue)
  int m_uni;
  int64_t strideA, strideB;
  int x_in_b;           // the square form: the solution overwrites b (QR::solve_mut)
};

// Butterfly reduce-scatter of N (a power of two <= 32) per-lane values: lane L
// ends with the warp-wide sum of value (L mod N) in v[0]; N-1 adds per lane
// plus log2(32/N) more, instead of N separate 5-step warp reductions.
template <int N>
__device__ __forceinline__ void warp_reduce_scatter(double (&v)[N]) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int half = N / 2; half >= 1; half >>= 1) {
    const bool up = (lane & half) != 0;
#pragma unroll
    for (int t = 0; t < half; ++t) {
      const double keep = up ? v[t + half] : v[t];
      const double give = up ? v[t] : v[t + half];
      v[t] = keep + __shfl_xor_sync(0xffffffffu, give, half);
    }
  }
#pragma unroll
  for (int off = N; off < 32; off <<= 1) v[0] += __shfl_xor_sync(0xffffffffu, v[0], off);
}

// c <- c - V T^T V^T c for G columns by one warp (V: the panel's jb axes in
// shared memory, ld ldp, zero above their diagonal; T: the kQrNB x kQrNB
// upper-triangular factor in s_t).  Pass 1 forms V^T c for the G columns (8
// partial dots per column and lane, then one reduce-scatter over all G x 8
// sums); lane (g, k) forms (T^T w_g)_k; pass 2 applies c -= V w'.
template <int G>
__device__ __forceinline__ void qr_apply_reflector(double* const (&cols)[G], int rows, const double* P, int ldp,
                                                   int jb, const double* s_t, int lane) {
  constexpr int N = G * kQrNB;
  double w[N];
#pragma unroll
  for (int e = 0; e < N; ++e) w[e] = 0.0;
  for (int r = lane; r < rows; r += 32) {
    double v[kQrNB];
#pragma unroll
    for (int c = 0; c < kQrNB; ++c) v[c] = (c < jb && r >= c) ? P[(size_t)c * ldp + r] : 0.0;
#pragma unroll
    for (int g = 0; g < G; ++g) {
      const double x = cols[g][r];
#pragma unroll
      for (int c = 0; c < kQrNB; ++c) w[g * kQrNB + c] = fma(v[c], x, w[g * kQrNB + c]);
    }
  }
  warp_reduce_scatter<N>(w);  // lane L holds the sum of value L mod N = (g, c)
  const int idx = lane % N, gq = idx / kQrNB, k = idx % kQrNB;
  double wk = 0.0;
#pragma unroll
  for (int j = 0; j < kQrNB; ++j) {
    const double wj = __shfl_sync(0xffffffffu, w[0], gq * kQrNB + j);
    if (j <= k) wk = fma(s_t[kTOff + j * kQrNB + k], wj, wk);
  }
  double wp[N];
#pragma unroll
  for (int e = 0; e < N; ++e) wp[e] = __shfl_sync(0xffffffffu, wk, e);
  for (int r = lane; r < rows; r += 32) {
    double v[kQrNB];
#pragma unroll
    for (int c = 0; c < kQrNB; ++c) v[c] = (c < jb && r >= c) ? P[(size_t)c * ldp + r] : 0.0;
#pragma unroll
    for (int g = 0; g < G; ++g) {
      double x = cols[g][r];
#pragma unroll
      for (int c = 0; c < kQrNB; ++c) x = fma(-v[c], wp[g * kQrNB + c], x);
      cols[g][r] = x;
    }
  }
}

// CTA sum, valid in thread 0 only (the one thread that uses it: the other
// threads add nothing, which saves the FP64 issue slots of 127 redundant sums).
__device__ __forceinline__ double block_sum_to0(double v, double* red) {
  v = warp_sum(v);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
#pragma unroll
    for (int w = 0; w < kQrThreads / 32; ++w) s += red[w];
  return s;
}

// A full panel (kQrNB columns, rows x kQrNB in P) in kQrNB Householder steps,
// each ONE pass over the rows with ONE CTA reduction: the pass of step j
// scales axis j, updates the later columns and accumulates, from the updated
// values, the sums step j+1 needs (|x_{j+1}|^2 and x_{j+1} . P_c for every
// other column c, x_{j+1} unscaled and unmodified); step j+1 then corrects
// them for the modified diagonal entry and the axis scale by scalars.  The
// steps are unrolled, so each pass issues only the FMAs of its live columns:
// on this part an FP64 instruction with its lanes predicated off still costs
// its issue slot.  Same reflections as the generic steps (householder.rs:
// 19-53 without the sign step); the sums are formed in a different order.
__device__ void qr_panel_full(double* P, int ldp, int rows, int J0, double* s_t, double* s_dstd, double* s_red) {
  constexpr int NB = kQrNB;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  double* s_sum = s_red + 4;           // 4 warps x NB partial sums
  double* s_par = s_red + 4 + 4 * NB;  // slot j: the axis scale; slots c > j: the column coefficients
  {
    double acc[NB];
#pragma unroll
    for (int c = 0; c < NB; ++c) acc[c] = 0.0;
    for (int r = tid; r < rows; r += kQrThreads) {
      const double x = P[r];
      acc[0] = fma(x, x, acc[0]);
#pragma unroll
      for (int c = 1; c < NB; ++c) acc[c] = fma(x, P[(size_t)c * ldp + r], acc[c]);
    }
    warp_reduce_scatter<NB>(acc);
    if (lane < NB) s_sum[warp * NB + lane] = acc[0];
  }
  __syncthreads();
#pragma unroll
  for (int j = 0; j < NB; ++j) {
    double* pj = P + (size_t)j * ldp;
    if (tid < NB) {  // lanes 0..NB-1 of warp 0: the scalars (redundantly), then column tid's term
      double sq = 0.0, dc = 0.0;
#pragma unroll
      for (int w = 0; w < kQrThreads / 32; ++w) {
        sq += s_sum[w * NB + j];
        dc += s_sum[w * NB + tid];
      }
      const double nrm = sqrt(sq);
      const double x0 = pj[j];
      const double mod = (x0 >= 0.0) ? x0 : -x0;
      const double sgn = (x0 >= 0.0) ? 1.0 : -1.0;  // simba to_exp
      const double signed_norm = sgn * nrm;
      const double factor = (sq + mod * nrm) * 2.0;
      const bool nz = factor != 0.0;
      const double scale = nz ? rsqrt(factor) : 0.0, tau = nz ? 2.0 : 0.0;
      // v . P_c with v = scale * x', x' = x but x'_j = x0 + signed_norm
      const double dv = fma(signed_norm, P[(size_t)tid * ldp + j], dc) * scale;
      if (tid == j) {
        s_dstd[J0 + j] = nz ? -signed_norm : signed_norm;  // R_std[j][j]
        s_t[kTauOff + j] = tau;
        s_par[j] = scale;
      } else if (tid > j) {
        s_par[tid] = -tau * dv;
      } else {
        s_t[kGSumOff + tid * NB - tid * (tid + 1) / 2 + (j - tid - 1)] = dv;  // G[tid][j] = v_tid . v_j
      }
      __syncwarp(0xffu);
      if (tid == j && nz) pj[j] = x0 + signed_norm;
    }
    __syncthreads();
    const double scale = s_par[j];
    double coef[NB];
#pragma unroll
    for (int c = 0; c < NB; ++c) coef[c] = (c > j) ? s_par[c] : 0.0;
    double acc[NB];
#pragma unroll
    for (int c = 0; c < NB; ++c) acc[c] = 0.0;
    for (int r = j + tid; r < rows; r += kQrThreads) {
      const double v = pj[r] * scale;
      pj[r] = v;
      double pc[NB];
#pragma unroll
      for (int c = j + 1; c < NB; ++c) {
        pc[c] = fma(coef[c], v, P[(size_t)c * ldp + r]);
        P[(size_t)c * ldp + r] = pc[c];
      }
      if (j + 1 < NB && r > j) {  // step j+1's sums over rows > j
        const double y = pc[j + 1];
#pragma unroll
        for (int c = 0; c < NB; ++c) {
          if (c == j + 1) acc[c] = fma(y, y, acc[c]);
          else if (c == j) acc[c] = fma(y, v, acc[c]);
          else if (c < j) acc[c] = fma(y, P[(size_t)c * ldp + r], acc[c]);
          else acc[c] = fma(y, pc[c], acc[c]);
        }
      }
    }
    if (j + 1 < NB) {
      warp_reduce_scatter<NB>(acc);
      if (lane < NB) s_sum[warp * NB + lane] = acc[0];
    }
    __syncthreads();
  }
}

// One problem.  P: panel buffer (ldp x kQrNB), V^T V and T in s_t, per-column
// standard diagonals in s_dstd, reductions in s_red.
__device__ void qr_one(const QrArgs& g, int s, double* P, int ldp, double* s_t, double* s_dstd,
                       double* s_red, double* s_misc) {
  const int tid = threadIdx.x;
  const int warp = tid >> 5, lane = tid & 31;
  const int n = g.n;
  const int m = g.ms ? g.ms[s] : g.m_uni;
  if (m < n || m > g.m_max) {
    if (tid == 0 && g.info) g.info[s] = -1;
    return;
  }
  double* a = g.A + (g.aoff ? g.aoff[s] : (int64_t)s * g.strideA);
  double* b = g.B ? g.B + (g.boff ? g.boff[s] : (int64_t)s * g.strideB) : nullptr;
  double* s_coef = s_red + 4 + 4 * kQrNB;
  for (int J0 = 0; J0 < n; J0 += kQrNB) {
    const int jb = min(kQrNB, n - J0);
    const int rows = m - J0;
    for (int e = tid; e < rows * jb; e += kQrThreads) {
      const int c = e / rows, r = e - c * rows;
      P[(size_t)c * ldp + r] = a[(size_t)(J0 + c) * m + J0 + r];
    }
    __syncthreads();
    // ---- panel: jb Householder steps in shared memory ----
    if (jb == kQrNB) qr_panel_full(P, ldp, rows, J0, s_t, s_dstd, s_red);
    else for (int j = 0; j < jb; ++j) {
      double* pj = P + (size_t)j * ldp;
      double part = 0.0;
      for (int r = j + tid; r < rows; r += kQrThreads) part = fma(pj[r], pj[r], part);
      const double sq = block_sum_to0(part, s_red);
      if (tid == 0) {
        // householder.rs:19-53 (reflection_axis_mut) without the sign step
        const double nrm = sqrt(sq);
        const double x0 = pj[j];
        const double mod = (x0 >= 0.0) ? x0 : -x0;
        const double sgn = (x0 >= 0.0) ? 1.0 : -1.0;  // simba to_exp
        const double signed_norm = sgn * nrm;
        const double factor = (sq + mod * nrm) * 2.0;
        if (factor != 0.0) {
          pj[j] = x0 + signed_norm;
          s_misc[0] = rsqrt(factor);
          s_misc[1] = 2.0;                // tau: v is unit length
          s_dstd[J0 + j] = -signed_norm;  // R_std[j][j]
        } else {
          s_misc[0] = 0.0;
          s_misc[1] = 0.0;  // no reflection (zero column)
          s_dstd[J0 + j] = signed_norm;
        }
        s_t[kTauOff + j] = s_misc[1];
      }
      __syncthreads();
      const double scale = s_misc[0], tau = s_misc[1];
      // v = x * scale; dots of v with the remaining panel columns (c > j) and
      // with the earlier reflection axes (c < j: the entries G[c][j] = v_c . v_j
      // of V^T V that the T factor needs, v_j being zero above row j)
      double dots[kQrNB];
#pragma unroll
      for (int c = 0; c < kQrNB; ++c) dots[c] = 0.0;
      for (int r = j + tid; r < rows; r += kQrThreads) {
        const double v = pj[r] * scale;
        pj[r] = v;
#pragma unroll
        for (int c = 0; c < kQrNB; ++c)
          if (c != j && c < jb) dots[c] = fma(v, P[(size_t)c * ldp + r], dots[c]);
      }
      // reduce the dots (at most 7) across the CTA
      warp_reduce_scatter<kQrNB>(dots);
      if (lane < kQrNB) s_red[4 + warp * kQrNB + lane] = dots[0];
      __syncthreads();
      // coef_c = -tau * (v^T P_c), formed once per column by kQrNB threads
      // (every thread forming all of them cost more FP64 issue slots than the
      // panel update itself); zero outside columns j+1..jb-1
      if (tid < kQrNB) {
        double d = 0.0;
#pragma unroll
        for (int w = 0; w < kQrThreads / 32; ++w) d += s_red[4 + w * kQrNB + tid];
        s_coef[tid] = (tid > j && tid < jb) ? -tau * d : 0.0;
        if (tid < j) s_t[kGSumOff + tid * kQrNB - tid * (tid + 1) / 2 + (j - tid - 1)] = d;  // G[tid][j]
      }
      __syncthreads();
      double coef[kQrNB];
#pragma unroll
      for (int c = 0; c < kQrNB; ++c) coef[c] = s_coef[c];
      for (int r = j + tid; r < rows; r += kQrThreads) {
        const double v = pj[r];
#pragma unroll
        for (int c = 0; c < kQrNB; ++c)
          if (c > j && c < jb) P[(size_t)c * ldp + r] = fma(coef[c], v, P[(size_t)c * ldp + r]);
      }
      __syncthreads();
    }
    // ---- T (forward, columnwise): T_jj = tau_j, T[0:j, j] = -tau_j T[0:j,0:j] V^T v_j ----
    // G = V^T V (strict upper part) was formed by the panel steps; lanes
    // 0..NB-1 of warp 0 run the small T recurrence in shared memory, lane i
    // forming row i of each new column (a column costs j FP64 steps on the
    // warp instead of j(j+1)/2 on one thread).
    if (tid < kQrNB) {
      const int i = tid;
#pragma unroll
      for (int j = 0; j < kQrNB; ++j) s_t[kTOff + i * kQrNB + j] = 0.0;
      __syncwarp(0xffu);
      for (int j = 0; j < jb; ++j) {
        const double tj = s_t[kTauOff + j];
        if (i < j) {
          double acc = 0.0;
          for (int l = i; l < j; ++l)
            acc = fma(s_t[kTOff + i * kQrNB + l], s_t[kGSumOff + l * kQrNB - l * (l + 1) / 2 + (j - l - 1)], acc);
          s_t[kTOff + i * kQrNB + j] = -tj * acc;
        } else if (i == j) {
          s_t[kTOff + j * kQrNB + j] = tj;
        }
        __syncwarp(0xffu);
      }
    }
    __syncthreads();
    // ---- trailing columns and the right-hand side: c <- c - V T^T V^T c ----
    // four columns per warp at a time (each shared-memory axis value feeds
    // four FMAs), the columns left over one at a time
    const int ntrail = n - J0 - jb;
    const int ncol = ntrail + (b ? 1 : 0);
    auto colptr = [&](int t) { return (t < ntrail) ? a + (size_t)(J0 + jb + t) * m + J0 : b + J0; };
    const int nfull = ncol / 4;
    for (int q = warp; q < nfull; q += kQrThreads / 32) {
      double* cols[4] = {colptr(4 * q), colptr(4 * q + 1), colptr(4 * q + 2), colptr(4 * q + 3)};
      qr_apply_reflector<4>(cols, rows, P, ldp, jb, s_t, lane);
    }
    for (int t = 4 * nfull + warp; t < ncol; t += kQrThreads / 32) {
      double* cols[1] = {colptr(t)};
      qr_apply_reflector<1>(cols, rows, P, ldp, jb, s_t, lane);
    }
    __syncthreads();
    // ---- write the factored panel back ----
    for (int e = tid; e < rows * jb; e += kQrThreads) {
      const int c = e / rows, r = e - c * rows;
      a[(size_t)(J0 + c) * m + J0 + r] = P[(size_t)c * ldp + r];
    }
    __syncthreads();
  }
  // ---- sign sweep (nalgebra's reflect_with_sign convention) ----
  // s_misc[2 + i] = P_i (axis sign), s_misc[2 + kQrMaxN + i] = d_i (row sign).
  if (tid == 0) {
    double pi = 1.0;
    int inf = 0;
    for (int i = 0; i < n; ++i) {
      const double di = pi * s_dstd[i];
      const double si = signbit(di) ? -1.0 : 1.0;  // Rust f64::signum (diag is never NaN here unless input is)
      s_misc[2 + i] = pi;
      pi *= si;
      s_misc[2 + kQrMaxN + i] = pi;
      s_dstd[i] = di;
      if (di == 0.0 && inf == 0) inf = i + 1;
    }
    s_misc[1] = (double)inf;
  }
  __syncthreads();
  const int inf = (int)s_misc[1];
  // |diag_i|^-1 for the back substitution (computed in parallel, once).
  for (int i = tid; i < n; i += kQrThreads) s_t[kGOff + i] = 1.0 / fabs(s_dstd[i]);
  __syncthreads();
  // The least-squares solution.  With R_nal = D R_std and (Q^T b)_nal = D (Q^T b)_std
  // the signs cancel; the solve uses nalgebra's R (rows scaled by d_r, diagonal
  // |diag_i|) exactly as qr.rs:224-256 restricted to the top n rows.
  if (b && (g.X || g.x_in_b) && inf == 0 && warp == 0) {
    constexpr int KR = kQrMaxN / 32;  // rows per lane
    double* x = g.x_in_b ? b : g.X + (size_t)s * n;
    double yv[KR];
#pragma unroll
    for (int k = 0; k < KR; ++k) {
      const int r = lane + 32 * k;
      yv[k] = (r < n) ? b[r] * s_misc[2 + kQrMaxN + r] : 0.0;
    }
    for (int i = n - 1; i >= 0; --i) {
      double own = yv[0];
#pragma unroll
      for (int k = 1; k < KR; ++k)
        if ((i >> 5) == k) own = yv[k];
      const double yi = __shfl_sync(0xffffffffu, own, i & 31);
      const double xi = yi * s_t[kGOff + i];
#pragma unroll
      for (int k = 0; k < KR; ++k)
        if (lane == (i & 31) && (i >> 5) == k) yv[k] = xi;
#pragma unroll
      for (int k = 0; k < KR; ++k) {
        const int r = lane + 32 * k;
        if (r < i) {  // R[r][i] times the row sign d_r = +-1: a sign-bit flip, no FP64 multiply
          const unsigned long long sm =
              (unsigned long long)__double_as_longlong(s_misc[2 + kQrMaxN + r]) & 0x8000000000000000ull;
          const double rri = __longlong_as_double(__double_as_longlong(a[(size_t)i * m + r]) ^ sm);
          yv[k] = fma(-xi, rri, yv[k]);
        }
      }
    }
    __syncwarp();
#pragma unroll
    for (int k = 0; k < KR; ++k) {
      const int r = lane + 32 * k;
      if (r < n) x[r] = yv[k];
    }
  }
  __syncthreads();
  // Apply the signs (+-1: a sign-bit flip, no FP64 work) to the stored
  // factors and to Q^T b.
  for (int e = tid; e < m * n; e += kQrThreads) {
    const int c = e / m, r = e - c * m;
    double* p = a + (size_t)c * m + r;
    const double f = (r >= c) ? s_misc[2 + c] : s_misc[2 + kQrMaxN + r];  // axis_c *= P_c, R[r][c] *= d_r
    const unsigned long long mask = (unsigned long long)__double_as_longlong(f) & 0x8000000000000000ull;
    *p = __longlong_as_double(__double_as_longlong(*p) ^ mask);
  }
  if (b && !(g.x_in_b && inf == 0))  // Q^T b in nalgebra's signs (the square form's solved b is x)
    for (int r = tid; r < m; r += kQrThreads) {
      const double f = s_misc[2 + kQrMaxN + min(r, n - 1)];
      const unsigned long long mask = (unsigned long long)__double_as_longlong(f) & 0x8000000000000000ull;
      b[r] = __longlong_as_double(__double_as_longlong(b[r]) ^ mask);
    }
  for (int i = tid; i < n; i += kQrThreads) g.diag[(size_t)s * n + i] = s_dstd[i];
  if (tid == 0 && g.info) g.info[s] = inf;
  __syncthreads();
}

__global__ void __launch_bounds__(kQrThreads, 4) qr_batched_kernel(QrArgs g) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ double s_t[kSTSize];
  __shared__ double s_dstd[kQrMaxN];
  __shared__ double s_red[4 + 5 * kQrNB];  // block sums | 4 warps x NB dots | NB panel coefficients
  __shared__ double s_misc[2 + 2 * kQrMaxN];
  __shared__ int s_item;
  const int ldp = g.m_max | 1;
  double* P = reinterpret_cast<double*>(smem_raw);
  if (!g.counter) {  // uniform batch: problems grid-stride
    for (int s = blockIdx.x; s < g.count; s += gridDim.x) qr_one(g, s, P, ldp, s_t, s_dstd, s_red, s_misc);
    return;
  }
  for (;;) {
    if (threadIdx.x == 0) s_item = atomicAdd(g.counter, 1);
    __syncthreads();
    const int idx = s_item;
    __syncthreads();
    if (idx >= g.count) break;
    const int s = g.order ? g.order[idx] : idx;
    qr_one(g, s, P, ldp, s_t, s_dstd, s_red, s_misc);
  }
}

}  // namespace

// The square QR's FMA form on this kernel: count uniform n x n problems
// (n <= kQrMaxN) at A + s * strideA, nalgebra's QR layout and signs in place,
// diag and info out; with B (one right-hand side per problem at B + s *
// strideB) QR::solve_mut overwrites b with x.
int qr_uniform_launch(int n, int count, double* A, int64_t strideA, double* diag, double* B, int64_t strideB,
                      int32_t* info, cudaStream_t s, const char* name) {
  QrArgs g{count, n, n, nullptr, nullptr, A, nullptr, B, nullptr, diag, info, nullptr, nullptr, n, strideA, strideB,
           1};
  const size_t smem = (size_t)(n | 1) * kQrNB * sizeof(double);
  cudaError_t e = ensure_dynamic_smem(qr_batched_kernel, smem);
  if (e != cudaSuccess) return record_cuda_error(e, name);
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, qr_batched_kernel, kQrThreads, smem);
  if (e != cudaSuccess) return record_cuda_error(e, name);
  if (per_sm < 1) per_sm = 1;
  int grid = sm_count() * per_sm;
  if (grid > count) grid = count;
  qr_batched_kernel<<<grid, kQrThreads, smem, s>>>(g);
  return check_launch(name);
}

}  // namespace nacu

extern "C" {

size_t nacu_qr_workspace_bytes(int count) {
  (void)count;
  return 256;
}

int nacu_dgels_batched(int count, int n, int m_max, const int32_t* ms, const int64_t* a_offsets, double* A,
                       const int64_t* b_offsets, double* B, double* X, double* diag, int32_t* info,
                       const int32_t* order, void* workspace, size_t workspace_bytes, int flags,
                       nacu_stream_t stream) {
  using namespace nacu;
  if (count < 0) return record_arg_error(-1, "dgels_batched: negative count");
  if (n < 1 || n > kQrMaxN) return record_arg_error(-2, "dgels_batched: n out of range [1, 128]");
  if (m_max < n || m_max > NACU_QR_MAX_M) return record_arg_error(-3, "dgels_batched: m_max out of range [n, 2048]");
  if (count == 0) return NACU_SUCCESS;
  if (!ms || !a_offsets || !A) return record_arg_error(-4, "dgels_batched: null ms, a_offsets or A");
  if ((b_offsets == nullptr) != (B == nullptr)) return record_arg_error(-7, "dgels_batched: b_offsets and B must both be set or both null");
  if (!diag) return record_arg_error(-10, "dgels_batched: null diag");
  if (!workspace || workspace_bytes < nacu_qr_workspace_bytes(count))
    return record_arg_error(-14, "dgels_batched: workspace too small");
  if (flags & NACU_FLAG_EXACT) return record_arg_error(-15, "dgels_batched: NACU_FLAG_EXACT is not available for QR");
  QrArgs g{count, n, m_max, ms, a_offsets, A, b_offsets, B, X, diag, info, order,
           reinterpret_cast<int32_t*>(workspace), 0, 0, 0, 0};
  const size_t smem = (size_t)(m_max | 1) * kQrNB * sizeof(double);
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = ensure_dynamic_smem(qr_batched_kernel, smem);
  if (e != cudaSuccess) return record_cuda_error(e, "nacu_dgels_batched");
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, qr_batched_kernel, kQrThreads, smem);
  if (e != cudaSuccess) return record_cuda_error(e, "nacu_dgels_batched");
  if (per_sm < 1) per_sm = 1;
  int grid = sm_count() * per_sm;
  if (grid > count) grid = count;
  e = cudaMemsetAsync(workspace, 0, sizeof(int32_t), s);
  if (e != cudaSuccess) return record_cuda_error(e, "nacu_dgels_batched");
  qr_batched_kernel<<<grid, kQrThreads, smem, s>>>(g);
  return check_launch("nacu_dgels_batched");
}

}  // extern "C"
