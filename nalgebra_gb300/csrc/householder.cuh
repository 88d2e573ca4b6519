// Device helpers shared by the Householder kernels (col_piv_qr.cu, qr_large.cu):
// simba's to_exp and Rust's signum on reals, dotx's summation order
// (src/base/blas.rs:96-165) for the EXACT forms, and a sign flip on the bits.
#pragma once

#include "common.cuh"

namespace nacu {

template <bool EXACT>
__device__ __forceinline__ double cq_mul(double a, double b) { return EXACT ? __dmul_rn(a, b) : a * b; }
template <bool EXACT>
__device__ __forceinline__ double cq_add(double a, double b) { return EXACT ? __dadd_rn(a, b) : a + b; }

// simba's to_exp for a real: (x, 1) when x >= 0, else (-x, -1) (NaN: -1).
__device__ __forceinline__ void cq_to_exp(double x, double& modulus, double& sign) {
  if (x >= 0.0) {
    modulus = x;
    sign = 1.0;
  } else {
    modulus = -x;
    sign = -1.0;
  }
}

// Rust's f64::signum: +1 for +0 and positives, -1 for -0 and negatives, NaN for NaN.
__device__ __forceinline__ double cq_signum(double x) { return isnan(x) ? x : (signbit(x) ? -1.0 : 1.0); }

// sum_{e < len} x[e] y[e] in dotx's order (EXACT: eight accumulators over
// blocks of 8, combined (a0+a4), (a1+a5), (a2+a6), (a3+a7) into 0, then the
// tail one product at a time) or as a warp reduction; valid in every lane.
template <bool EXACT>
__device__ double cq_dot(int len, const double* x, const double* y, int lane) {
  if constexpr (EXACT) {
    const int nb = len >> 3;
    double acc = 0.0;
    if (lane < 8)
      for (int b = 0; b < nb; ++b) acc = __dadd_rn(acc, __dmul_rn(x[8 * b + lane], y[8 * b + lane]));
    const double pair = __dadd_rn(acc, __shfl_down_sync(0xffffffffu, acc, 4));
    double res = 0.0;
#pragma unroll
    for (int q = 0; q < 4; ++q) res = __dadd_rn(res, __shfl_sync(0xffffffffu, pair, q));
    for (int e = 8 * nb; e < len; ++e) res = __dadd_rn(res, __dmul_rn(x[e], y[e]));
    return res;
  } else {
    double part = 0.0;
    for (int e = lane; e < len; e += 32) part = fma(x[e], y[e], part);
    return warp_sum(part);
  }
}

// The same sum by one thread: dotx's order in EXACT, four interleaved
// accumulators otherwise.
template <bool EXACT>
__device__ __forceinline__ double cq_dot_seq(int len, const double* x, const double* y) {
  if constexpr (EXACT) {
    double a[8] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    const int nb = len >> 3;
    for (int b = 0; b < nb; ++b)
#pragma unroll
      for (int q = 0; q < 8; ++q) a[q] = __dadd_rn(a[q], __dmul_rn(x[8 * b + q], y[8 * b + q]));
    double res = 0.0;
#pragma unroll
    for (int q = 0; q < 4; ++q) res = __dadd_rn(res, __dadd_rn(a[q], a[q + 4]));
    for (int e = 8 * nb; e < len; ++e) res = __dadd_rn(res, __dmul_rn(x[e], y[e]));
    return res;
  } else {
    double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
    int e = 0;
    for (; e + 4 <= len; e += 4) {
      a0 = fma(x[e], y[e], a0);
      a1 = fma(x[e + 1], y[e + 1], a1);
      a2 = fma(x[e + 2], y[e + 2], a2);
      a3 = fma(x[e + 3], y[e + 3], a3);
    }
    for (; e < len; ++e) a0 = fma(x[e], y[e], a0);
    return (a0 + a1) + (a2 + a3);
  }
}

// -x by flipping the sign bit with integer instructions (no FP64 slot).
__device__ __forceinline__ double neg_bits(double x) {
  unsigned lo, hi;
  asm("mov.b64 {%0, %1}, %2;" : "=r"(lo), "=r"(hi) : "d"(x));
  hi ^= 0x80000000u;
  double r;
  asm("mov.b64 %0, {%1, %2};" : "=d"(r) : "r"(lo), "r"(hi));
  return r;
}

}  // namespace nacu
