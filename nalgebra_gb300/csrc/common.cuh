// Shared device helpers for the nalgebra-cuda kernels (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/nalgebra_cuda.h"

namespace nacu {

// BF16-split tensor-core GEMM (gemm_split.cu): C = alpha A B + beta C.
template <typename TI, typename TO>
int split_gemm_run(int m, int n, int k, double alpha, const TI* A, int64_t lda, const TI* B, int64_t ldb, double beta,
                   TO* C, int64_t ldc, int slices, void* workspace, size_t workspace_bytes, cudaStream_t stream);

// Equal-order batched Cholesky factor + solve + log-determinant in place, FP64
// (chol_ragged.cu).
int chol_uniform_posv(int n, double* A, int64_t strideA, int nrhs, double* B, int64_t strideB, int32_t* info,
                      double* logdet, int batch, cudaStream_t s, const char* name);

// Processing order of a ragged batch, largest order first (a counting sort
// over n = 0..n_max on the device; chol_ragged.cu).  scratch: at least
// ragged_order_scratch_bytes() bytes, 256-byte aligned.
size_t ragged_order_scratch_bytes();
int ragged_order_desc(int count, int n_max, const int32_t* ns, int32_t* order, void* scratch, cudaStream_t s,
                      const char* name);

// Records a CUDA error (from a launch or a runtime call) for nacu_last_error().
int record_cuda_error(cudaError_t e, const char* where);
// Records an argument error message; returns `code`.
int record_arg_error(int code, const char* msg);

inline int check_launch(const char* where) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return record_cuda_error(e, where);
  return NACU_SUCCESS;
}

// Raises a kernel's dynamic shared-memory limit to at least `bytes`, never
// lowering it.  A kernel node recorded in a CUDA graph keeps the size it was
// captured with, while the function attribute is read again when the node is
// launched on its own (a profiler replaying a graph node by node does this).
// Setting the attribute to each call's own size let a later, smaller call on
// the same kernel push it below an earlier node's size, and that node's
// launch then failed.
template <typename K>
inline cudaError_t ensure_dynamic_smem(K kern, size_t bytes) {
  cudaFuncAttributes a;
  cudaError_t e = cudaFuncGetAttributes(&a, reinterpret_cast<const void*>(kern));
  if (e != cudaSuccess) return e;
  if ((size_t)a.maxDynamicSharedSizeBytes >= bytes) return cudaSuccess;
  return cudaFuncSetAttribute(reinterpret_cast<const void*>(kern), cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)bytes);
}

inline int sm_count() {
  static int count = 0;
  if (count == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&count, cudaDevAttrMultiProcessorCount, dev);
    if (count <= 0) count = 1;
  }
  return count;
}

// One element of nalgebra's axpy (src/base/blas_uninit.rs:32-53 with c = beta = 1):
// y + a*x.  EXACT keeps nalgebra's two roundings (fl(fl(a*x) + y)); otherwise one FMA.
template <bool EXACT, typename T>
__device__ __forceinline__ T axpy1(T y, T a, T x) {
  if constexpr (EXACT) {
    if constexpr (sizeof(T) == 8) return __dadd_rn(__dmul_rn(a, x), y);
    else return __fadd_rn(__fmul_rn(a, x), y);
  } else {
    if constexpr (sizeof(T) == 8) return fma(a, x, y);
    else return fmaf(a, x, y);
  }
}

// Pivot key for icamax (src/base/min_max.rs:221-240): |x| compared as an
// unsigned integer (valid for non-negative IEEE values); a NaN wins only at
// the first position of the scan (where nalgebra's running max starts), and is
// ignored elsewhere.  Ties resolve to the lowest index by the reduction.
// |x| as its bit image (for non-negative doubles the integer order is the
// numeric order), taken through an opaque mov: a plain mask of the
// reinterpreted bits is recognised as fabs and then costs an FP64 add.
__device__ __forceinline__ unsigned long long abs_bits_f64(double x) {
  unsigned lo, hi;
  asm("mov.b64 {%0, %1}, %2;" : "=r"(lo), "=r"(hi) : "d"(x));
  return ((unsigned long long)(hi & 0x7fffffffu) << 32) | lo;
}

// x == 0 (either sign) from the bit image, on the integer pipe: an FP64
// compare issues on the FP64 pipe, which on this part takes a warp-wide
// instruction every 64 cycles per sub-partition, so a test every thread makes
// once per elimination step costs as much as a sixth of the step's FMAs.
__device__ __forceinline__ bool is_zero_bits(double x) { return (abs_bits_f64(x) == 0ull); }
__device__ __forceinline__ bool is_zero_bits(float x) {
  unsigned u;
  asm("mov.b32 %0, %1;" : "=r"(u) : "f"(x));
  return (u & 0x7fffffffu) == 0u;
}

// The bit image is taken through an opaque mov: a plain mask of the
// reinterpreted bits is recognised as fabs and then costs an FP64 add (an
// FP64 pipe slot) per key, where the key is taken for every updated element.
__device__ __forceinline__ uint64_t pivot_key(double x, bool first) {
  const uint64_t b = abs_bits_f64(x);
  if (b > 0x7ff0000000000000ull) return first ? ~0ull : 0ull;
  return b;
}
__device__ __forceinline__ uint64_t pivot_key(float x, bool first) {
  unsigned u;
  asm("mov.b32 %0, %1;" : "=r"(u) : "f"(x));
  const uint32_t b = u & 0x7fffffffu;
  if (b > 0x7f800000u) return first ? ~0ull : 0ull;
  return (uint64_t)b;
}

// Warp argmax of (key, idx): larger key wins, equal keys keep the lower index;
// every lane receives the result.  Three warp-wide reductions (redux.sync:
// max of the key's high word, max of the low word among the lanes holding
// that high word, min of the index among the lanes holding the whole key)
// instead of a five-round shuffle butterfly of three values: the pivot search
// sits on the critical path of every elimination step.
__device__ __forceinline__ void warp_argmax(uint64_t& key, int& idx) {
  const unsigned hi = (unsigned)(key >> 32), lo = (unsigned)key;
  const unsigned mh = __reduce_max_sync(0xffffffffu, hi);
  const unsigned ml = __reduce_max_sync(0xffffffffu, hi == mh ? lo : 0u);
  const bool win = (hi == mh && lo == ml);
  const unsigned mi = __reduce_min_sync(0xffffffffu, win ? (unsigned)idx : 0xffffffffu);
  key = ((uint64_t)mh << 32) | ml;
  idx = (int)mi;
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
  return v;
}

// binary64 -> binary32, round to nearest even, from the IEEE 754 bit fields
// with integer instructions: where the result is a normal binary32 number
// (biased binary64 exponent 897..1150) the exponent is re-biased by
// 1023 - 127 = 896, the top 23 of the 52 fraction bits are kept and the 29
// dropped bits round (ties to even; a carry into the exponent is the correct
// rounding, up to infinity).  Zero, subnormal results, overflow, inf and NaN
// take the hardware conversion.  Bit-identical to (float)x, and keeps the
// conversion off the FP64 pipe, which the residuals need.
__device__ __forceinline__ float f64_to_f32_rn(double x) {
  const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
  const unsigned ah = hi & 0x7fffffffu;
  if (ah >= 0x38100000u && ah < 0x47f00000u) {
    unsigned m = __funnelshift_l(lo, ah, 3) - (896u << 23);  // exponent and 23 fraction bits (mod 2^32)
    const unsigned rest = lo & 0x1fffffffu;
    m += (rest > 0x10000000u || (rest == 0x10000000u && (m & 1u))) ? 1u : 0u;
    return __uint_as_float(m | (hi & 0x80000000u));
  }
  return (float)x;
}

// 1/d for the FMA forms: the hardware's approximate reciprocal
// (rcp.approx.ftz.f64) refined by two Newton-Raphson steps for 1/d,
// e = 1 - d r, r <- r + r e (quadratic convergence), four FP64 instructions
// after the approximation where an IEEE division takes a longer dependent
// chain.  Within a few ulps of 1/d (not always correctly rounded; the EXACT
// forms divide).  For |d| outside [2^-1000, 2^1000], zero, infinities and NaN
// it takes the division.
__device__ __forceinline__ double rcp_nr(double d) {
  const long long b = __double_as_longlong(d) & 0x7fffffffffffffffll;
  if (b < 0x0170000000000000ll || b >= 0x7e70000000000000ll) return 1.0 / d;
  double r;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(d));
  double e = fma(-d, r, 1.0);
  r = fma(r, e, r);
  e = fma(-d, r, 1.0);
  return fma(r, e, r);
}

// A lower bound of |x| in binary32 for norm sums, from the high word alone:
// the fraction truncated to 20 bits, magnitudes below 2^-127 counted as 0 and
// above the binary32 range clamped just under FLT_MAX (a smaller ||A|| only
// tightens the stopping test).
__device__ __forceinline__ float abs_f32_lower(double x) {
  unsigned h = (unsigned)__double2hiint(x) & 0x7fffffffu;
  h = min(max(h, 0x38000000u), 0x47efffffu);
  return __uint_as_float((h - 0x38000000u) << 3);
}

}  // namespace nacu
