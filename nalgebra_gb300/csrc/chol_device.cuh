// Device building blocks of the Cholesky kernels, shared by the FP64 ragged
// kernel (chol_ragged.cu) and the FP32-factor / FP64-refinement kernel
// (chol_mixed.cu): templated on the scalar type, see chol_ragged.cu for the
// algorithm and the reference citations.
#pragma once
#include "common.cuh"

namespace nacu {
namespace {

constexpr int kCholThreads = 128;
constexpr int kNB = 16;        // panel width
constexpr int kRhsChunk = 4;   // right-hand sides per register pass
constexpr int kRowsPerPass = 256;  // rows of the panel update held in registers per pass

// Pivot of column j (cholesky.rs:237-268): re <= 0 -> None, else try_sqrt
// (x >= 0), NaN fails; the substitute is tried the same way.  EXACT computes the
// correctly rounded sqrt and 1/sqrt as two operations; the FMA form derives
// both from one reciprocal square root (one dependent FP64 chain instead of
// two: on this part every dependent FP64 step costs tens of cycles).
// d in (0, +inf], NaN excluded (the test !(d <= 0) && d >= 0), on the bits:
// an FP64 compare costs a warp-wide FP64 issue slot.
__device__ __forceinline__ bool pos_or_inf(double d) {
  const long long b = __double_as_longlong(d);
  return b > 0 && b <= 0x7ff0000000000000ll;
}
__device__ __forceinline__ bool pos_or_inf(float d) {
  const int b = __float_as_int(d);
  return b > 0 && b <= 0x7f800000;
}

template <bool EXACT, typename T>
__device__ __forceinline__ bool chol_pivot(T d, int has_subst, double subst, T* denom, T* rcp) {
  T v;
  if (pos_or_inf(d)) v = d;
  else if (has_subst && !(subst <= 0.0) && subst >= 0.0) v = (T)subst;
  else return false;
  if constexpr (EXACT) {
    *denom = sqrt(v);
    *rcp = T(1) / *denom;
  } else {
    const T r = rsqrt(v);
    *rcp = r;
    *denom = v * r;
  }
  return true;
}

// Factor one n x n matrix (column-major, lda = n, global memory, in place).
// Leaves info (0 ok, j+1 first failing pivot) in *s_info and, in the FMA form,
// 1/L_ii in rdiag[i] for the solves.
template <bool EXACT, typename T, int NB = kNB>
__device__ void chol_factor_cta(int n, T* __restrict__ a, int ldp, T* __restrict__ P, T* rdiag,
                                int* s_info, T* s_scal, int has_subst, double subst) {
  const int tid = threadIdx.x;
  const int nthr = blockDim.x;
  const int warp = tid >> 5, lane = tid & 31;
  for (int J0 = 0; J0 < n; J0 += NB) {
    const int jb = min(NB, n - J0);
    const int rows = n - J0;
    // Phase 1+2: P = A[J0.., J0..J0+jb] - L[J0.., 0..J0] * L[J0..J0+jb, 0..J0]^T
    // (lower part); each element still takes its updates in order k = 0, 1,
    // ..., J0-1.  On this part a warp-wide FP64 instruction costs its full
    // pipe time whatever lanes are masked, so the lanes are laid out to waste
    // few: a warp instruction covers NB/4 column groups of 4 x R = 128/NB rows
    // (rows below the panel's head, in R-row slabs spread over the warps), and
    // the head's lower triangle (c <= r < jb) is a flat list of elements, one
    // per thread.  With 32 rows per column group and the head as a square,
    // 26% of the lanes of the ragged workload's updates were idle; now 10%.
    {
      constexpr int G = NB / 4;  // column groups per warp instruction
      constexpr int R = 32 / G;  // rows per warp instruction
      constexpr int QMAX = 8;    // slabs per thread and pass
      static_assert(NB % 4 == 0 && 32 % G == 0 && G <= 32, "panel width");
      const int nw = nthr >> 5;
      const int g4 = (lane / R) * 4, rl = lane % R;
      const int nslab = (rows - jb + R - 1) / R;
      for (int sb = 0; sb < nslab; sb += QMAX * nw) {
        T acc[QMAX][4];
#pragma unroll
        for (int i = 0; i < QMAX; ++i) {
          const int r = jb + (sb + warp + nw * i) * R + rl;
#pragma unroll
          for (int j = 0; j < 4; ++j)
            acc[i][j] = (r < rows && g4 + j < jb) ? a[(size_t)(J0 + g4 + j) * n + J0 + r] : T(0);
        }
        const T* colk = a + J0;
#pragma unroll 2
        for (int k = 0; k < J0; ++k, colk += n) {
          // L[c][k]; the negation is folded into the FMA operand (a select of
          // -x would cost one FP64 instruction per load).
          T lc[4];
#pragma unroll
          for (int j = 0; j < 4; ++j) lc[j] = (g4 + j < jb) ? colk[g4 + j] : T(0);
#pragma unroll
          for (int i = 0; i < QMAX; ++i) {
            if (sb + warp + nw * i < nslab) {  // warp-uniform
              const int r = jb + (sb + warp + nw * i) * R + rl;
              const T lr = (r < rows) ? colk[r] : T(0);
#pragma unroll
              for (int j = 0; j < 4; ++j) acc[i][j] = axpy1<EXACT>(acc[i][j], -lc[j], lr);
            }
          }
        }
#pragma unroll
        for (int i = 0; i < QMAX; ++i) {
          const int r = jb + (sb + warp + nw * i) * R + rl;
#pragma unroll
          for (int j = 0; j < 4; ++j)
            if (sb + warp + nw * i < nslab && r < rows && g4 + j < jb) P[(size_t)(g4 + j) * ldp + r] = acc[i][j];
        }
      }
      // the head: element e = r(r+1)/2 + c of the lower triangle
      const int H = jb * (jb + 1) / 2;
      for (int e0 = 0; e0 < H; e0 += nthr) {
        const int e = e0 + tid;
        int r = 0;
        while ((r + 1) * (r + 2) / 2 <= e) ++r;  // at most NB steps, integer only
        const int c = e - r * (r + 1) / 2;
        const bool on = e < H;
        T acc = on ? a[(size_t)(J0 + c) * n + J0 + r] : T(0);
        const T* colk = a + J0;
#pragma unroll 4
        for (int k = 0; k < J0; ++k, colk += n) {
          const T lrk = on ? colk[r] : T(0), lck = on ? colk[c] : T(0);
          acc = axpy1<EXACT>(acc, -lck, lrk);
        }
        if (on) P[(size_t)c * ldp + r] = acc;
      }
    }
    __syncthreads();
    // Phase 3: factor the panel in shared memory, right-looking inside the panel
    // (the same per-element update order).  Thread 0 owns every diagonal
    // element of the trailing update (flattened index 0), so it computes the
    // next pivot right after its own update: two barriers per column.
    if (tid == 0) {
      T denom, rcp;
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
      T* pj = P + (size_t)j * ldp;
      const T denom = s_scal[0], rcp = s_scal[1];
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
            T* pc = P + (size_t)c * ldp;
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
          T* pn = P + (size_t)(j + 1) * ldp + (j + 1);
          T dn, rn;
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
    for (int c = warp; c < jb; c += nthr >> 5)
      for (int r = c + lane; r < rows; r += 32) a[(size_t)(J0 + c) * n + J0 + r] = P[(size_t)c * ldp + r];
    __syncthreads();
  }
}

// Forward solve L y = b (axpy form) for up to kRhsChunk columns of X (shared,
// column-major ldx), blocked by 32 rows.
template <bool EXACT, typename T>
__device__ void chol_forward_cta(int n, const T* __restrict__ a, T* X, int ldx, int nr, const T* rdiag) {
  const int tid = threadIdx.x, nthr = blockDim.x;
  const int warp = tid >> 5, lane = tid & 31;
  for (int I0 = 0; I0 < n; I0 += 32) {
    const int ib = min(32, n - I0);
    if (warp == 0) {
      T lrow[32];
      T b[kRhsChunk];
#pragma unroll
      for (int i = 0; i < 32; ++i) lrow[i] = (lane < ib && i <= lane) ? a[(size_t)(I0 + i) * n + I0 + lane] : T(0);
#pragma unroll
      for (int c = 0; c < kRhsChunk; ++c) b[c] = (lane < ib && c < nr) ? X[(size_t)c * ldx + I0 + lane] : T(0);
      const T rd = (lane < ib) ? rdiag[I0 + lane] : T(0);
      if constexpr (EXACT || sizeof(T) != 8) {  // EXACT, and FP32 (latency-bound: the short chain)
#pragma unroll
        for (int i = 0; i < 32; ++i) {
          if (i < ib) {
#pragma unroll
            for (int c = 0; c < kRhsChunk; ++c) {
              if (lane == i) {
                if constexpr (EXACT) b[c] = b[c] / lrow[i];  // solve.rs:509: b_i / L_ii
                else b[c] = b[c] * rd;
              }
              const T y = __shfl_sync(0xffffffffu, b[c], i);
              if (lane > i) b[c] = axpy1<EXACT>(b[c], -y, lrow[i]);
            }
          }
        }
      } else {
        // L's columns pre-scaled by 1/L_ii, so the chain broadcasts the
        // unscaled b_i and each step is one FMA per right-hand side (a
        // one-lane scale per step would cost a warp-wide FP64 slot); the
        // rows are scaled once at the end.
#pragma unroll
        for (int i = 0; i < 32; ++i) lrow[i] *= (i < ib) ? rdiag[I0 + i] : T(0);
#pragma unroll
        for (int i = 0; i < 32; ++i) {
          if (i < ib) {
#pragma unroll
            for (int c = 0; c < kRhsChunk; ++c) {
              const T y = __shfl_sync(0xffffffffu, b[c], i);
              if (lane > i) b[c] = fma(-y, lrow[i], b[c]);
            }
          }
        }
#pragma unroll
        for (int c = 0; c < kRhsChunk; ++c) b[c] *= rd;
      }
#pragma unroll
      for (int c = 0; c < kRhsChunk; ++c)
        if (lane < ib && c < nr) X[(size_t)c * ldx + I0 + lane] = b[c];
    }
    __syncthreads();
    // Rows below the block: b_r -= sum_i L[r][I0+i] y_i, one thread per row
    // for all right-hand sides (one L load feeds kRhsChunk FMAs), i ascending.
    for (int r = I0 + ib + tid; r < n; r += nthr) {
      T v[kRhsChunk];
#pragma unroll
      for (int c = 0; c < kRhsChunk; ++c) v[c] = (c < nr) ? X[(size_t)c * ldx + r] : T(0);
      const T* lp = a + (size_t)I0 * n + r;
      for (int i0 = 0; i0 < ib; i0 += 8) {  // 8 independent loads in flight
        T l8[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) l8[u] = (i0 + u < ib) ? lp[(size_t)(i0 + u) * n] : T(0);
#pragma unroll
        for (int u = 0; u < 8; ++u)
          if (i0 + u < ib)
#pragma unroll
            for (int c = 0; c < kRhsChunk; ++c)
              v[c] = axpy1<EXACT>(v[c], -X[(size_t)c * ldx + I0 + i0 + u], l8[u]);
      }
#pragma unroll
      for (int c = 0; c < kRhsChunk; ++c)
        if (c < nr) X[(size_t)c * ldx + r] = v[c];
    }
    __syncthreads();
  }
}

// Back solve L^T x = y, FMA form, FP32: blocked from the bottom, reductions
// over the rows below each 32-row block (16 sums per lane, one 32-lane
// reduce-scatter), then a warp solve of the transposed block.
template <typename T>
__device__ void chol_backward_fast32_cta(int n, const T* __restrict__ a, T* X, int ldx, int nr, const T* rdiag) {
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
        T v[16];
#pragma unroll
        for (int k = 0; k < 16; ++k) v[k] = T(0);
        for (int r0l = r0 + lane; r0l < n; r0l += 64) {  // two rows per step: 8 loads in flight
          T l2[2][4];
#pragma unroll
          for (int h = 0; h < 2; ++h)
#pragma unroll
            for (int j = 0; j < 4; ++j) {
              const int r = r0l + 32 * h;
              l2[h][j] = (cb + j < ib && r < n) ? a[(size_t)(I0 + cb + j) * n + r] : T(0);
            }
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            const int r = r0l + 32 * h;
            T xr[4];
#pragma unroll
            for (int c = 0; c < 4; ++c) xr[c] = (c < nr && r < n) ? X[(size_t)c * ldx + r] : T(0);
#pragma unroll
            for (int j = 0; j < 4; ++j)
#pragma unroll
              for (int c = 0; c < 4; ++c) v[j * 4 + c] = fma(l2[h][j], xr[c], v[j * 4 + c]);
          }
        }
#pragma unroll
        for (int half = 8; half >= 1; half >>= 1) {
          const bool up = (lane & half) != 0;
#pragma unroll
          for (int t = 0; t < half; ++t) {
            const T keep = up ? v[t + half] : v[t];
            const T give = up ? v[t] : v[t + half];
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
      T lcol[32];  // lane j holds column j of the diagonal block
#pragma unroll
      for (int i = 0; i < 32; ++i) lcol[i] = (lane < ib && i < ib && i >= lane) ? a[(size_t)(I0 + lane) * n + I0 + i] : T(0);
      const T rd = (lane < ib) ? rdiag[I0 + lane] : T(0);
      for (int c = 0; c < nr; ++c) {
        T y = (lane < ib) ? X[(size_t)c * ldx + I0 + lane] : T(0);
#pragma unroll
        for (int i = 31; i >= 0; --i) {
          if (i < ib) {
            if (lane == i) y = y * rd;
            const T xi = __shfl_sync(0xffffffffu, y, i);
            if (lane < i) y = fma(-xi, lcol[i], y);
          }
        }
        if (lane < ib) X[(size_t)c * ldx + I0 + lane] = y;
      }
    }
    __syncthreads();
  }
}

// The same in FP64 with fewer warp-wide FP64 instructions: blocked from the
// bottom, reductions over the rows below each 32-row block, then a warp solve
// of the transposed block.
template <typename T>
__device__ void chol_backward_fast64_cta(int n, const T* __restrict__ a, T* X, int ldx, int nr, const T* rdiag) {
  const int tid = threadIdx.x, nthr = blockDim.x;
  const int warp = tid >> 5, lane = tid & 31, nwarps = nthr >> 5;
  const int nblocks = (n + 31) / 32;
  for (int bI = nblocks - 1; bI >= 0; --bI) {
    const int I0 = bI * 32;
    const int ib = min(32, n - I0);
    const int r0 = I0 + ib;
    if (r0 < n) {
      // y_i -= sum_{r >= r0} L[r][i] x_r for the block's columns i: warp w
      // owns 4 columns at a time, lane = 8 column-lane x 4 + row-lane: lane
      // (cc, rho) accumulates column cb + cc over rows r0 + rho + 8t for the
      // 4 right-hand sides (8 consecutive rows per column load), then a
      // reduce-scatter over the 8 row-lanes (4 adds per lane instead of the
      // 31 of a 32-lane reduction of 16 sums: each is a warp-wide FP64 slot).
      const int rho = lane & 7, cc = lane >> 3;
      for (int cb = warp * 4; cb < ib; cb += nwarps * 4) {
        const bool colok = cb + cc < ib;
        const T* lcol = a + (size_t)(I0 + cb + (colok ? cc : 0)) * n;
        T v[4] = {T(0), T(0), T(0), T(0)};
        for (int rr = r0 + rho; rr < n; rr += 32) {  // four rows per lane and step: 4 loads in flight
          T l4[4];
#pragma unroll
          for (int h = 0; h < 4; ++h) {
            const int r = rr + 8 * h;
            l4[h] = (colok && r < n) ? lcol[r] : T(0);
          }
#pragma unroll
          for (int h = 0; h < 4; ++h) {
            const int r = rr + 8 * h;
#pragma unroll
            for (int c = 0; c < 4; ++c) {
              const T xr = (c < nr && r < n) ? X[(size_t)c * ldx + r] : T(0);
              v[c] = fma(l4[h], xr, v[c]);
            }
          }
        }
        // reduce-scatter over lane bits 0..2: lane keeps right-hand side
        // c = 2 * bit2 + bit1 (lanes differing in bit 0 hold the same sum)
        {
          const bool up4 = (lane & 4) != 0;
#pragma unroll
          for (int t = 0; t < 2; ++t) {
            const T keep = up4 ? v[t + 2] : v[t];
            const T give = up4 ? v[t] : v[t + 2];
            v[t] = keep + __shfl_xor_sync(0xffffffffu, give, 4);
          }
          const bool up2 = (lane & 2) != 0;
          const T keep = up2 ? v[1] : v[0];
          const T give = up2 ? v[0] : v[1];
          v[0] = keep + __shfl_xor_sync(0xffffffffu, give, 2);
          v[0] += __shfl_xor_sync(0xffffffffu, v[0], 1);
        }
        const int c = ((lane >> 2) & 1) * 2 + ((lane >> 1) & 1);
        if ((lane & 1) == 0 && colok && c < nr) X[(size_t)c * ldx + I0 + cb + cc] -= v[0];
      }
      __syncthreads();
    }
    if (warp == 0) {
      // lane j holds column j of the diagonal block, pre-scaled by 1/L_ii
      // (row i), so the chain broadcasts the unscaled y_i: one FMA per step
      T lcol[32];
#pragma unroll
      for (int i = 0; i < 32; ++i)
        lcol[i] = (lane < ib && i < ib && i >= lane) ? a[(size_t)(I0 + lane) * n + I0 + i] * rdiag[I0 + i] : T(0);
      const T rd = (lane < ib) ? rdiag[I0 + lane] : T(0);
      T y[kRhsChunk];
#pragma unroll
      for (int c = 0; c < kRhsChunk; ++c) y[c] = (lane < ib && c < nr) ? X[(size_t)c * ldx + I0 + lane] : T(0);
#pragma unroll
      for (int i = 31; i >= 0; --i) {
        if (i < ib) {
#pragma unroll
          for (int c = 0; c < kRhsChunk; ++c) {
            const T yi = __shfl_sync(0xffffffffu, y[c], i);
            if (lane < i) y[c] = fma(-yi, lcol[i], y[c]);
          }
        }
      }
#pragma unroll
      for (int c = 0; c < kRhsChunk; ++c)
        if (lane < ib && c < nr) X[(size_t)c * ldx + I0 + lane] = y[c] * rd;
    }
    __syncthreads();
  }
}

// Back solve L^T x = y, FMA form.  The FP64 variant is bound by the FP64
// pipe and minimises its warp-wide FP64 instructions; the FP32 variant (the
// refinement form's solves) is bound by L2 latency and keeps more loads in
// flight per lane.
template <typename T>
__device__ __forceinline__ void chol_backward_fast_cta(int n, const T* __restrict__ a, T* X, int ldx, int nr,
                                                       const T* rdiag) {
  if constexpr (sizeof(T) == 8) chol_backward_fast64_cta<T>(n, a, X, ldx, nr, rdiag);
  else chol_backward_fast32_cta<T>(n, a, X, ldx, nr, rdiag);
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

}  // namespace
}  // namespace nacu
