// Split-precision GEMM on the tensor cores: C = alpha * A * B + beta * C for
// FP64 column-major A (m x k), B (k x n), C (m x n), the precision form of
// nalgebra's `Matrix::gemm` (src/base/blas.rs:729-746).
//
// Method (an error-free-transformation style split, Ozaki et al. 2012, cut to
// BF16 slices with FP32 accumulation):
//   1. each row i of A is scaled by 2^-e_i and each column j of B by 2^-f_j
//      (e_i, f_j = exponent of the row / column max: exact power-of-two scaling,
//      so rows and columns of wildly different magnitude -- entries N(0,1) 2^k,
//      k in [-20, 20] -- keep their full relative precision);
//   2. the scaled values are split into s BF16 slices, x = x1 + x2 + x3 + r
//      (8 significant bits each: together the 24 bits of an FP32);
//   3. the slice products p + q <= s + 1 (6 for s = 3) are accumulated in FP32
//      by tcgen05.mma (kind::f16, BF16 x BF16 -> FP32) into one TMEM tile;
//   4. C_ij = alpha * 2^(e_i + f_j) * acc_ij + beta * C_ij in FP64 (beta == 0:
//      C is not read).
// The result is FP32-class accurate (the error against the exact product is
// reported against a compensated FP64 oracle); the work runs at tensor-core
// speed instead of the ~1 TFLOP/s FP64 pipe.
//
// Kernel: persistent, one CTA per SM looping over 128 x 256 output tiles,
// 192 threads.  Warp 0 / lane 0 issues TMA loads (cp.async.bulk.tensor.2d,
// 64-byte swizzle) of every slice tile of a 32-deep k-block -- s A tiles
// (128 x 32 BF16) and s B tiles (256 x 32 BF16) -- into one stage of a
// 3-stage shared-memory ring, so each slice tile crosses L2 once; the ring
// runs on across tiles.  Warp 1 / lane 0 issues the k-block's slice products
// as tcgen05.mma 128 x 256 x 16 from that stage into one of two 256-column
// FP32 TMEM accumulators (tiles alternate) and releases the stage with
// tcgen05.commit.  Warps 2-5 are the epilogue: warp w reads TMEM lanes
// 32 (w mod 4) .. + 31 (rows) of a finished accumulator with tcgen05.ld,
// writes C, and hands the accumulator back -- while the MMAs of the next tile
// already run in the other one.  Every mbarrier wait is bounded: on time-out
// the kernel records an error flag and finishes without further waiting.
#include <cuda.h>
#include <cuda_bf16.h>

#include "common.cuh"

namespace nacu {
namespace {

constexpr int kTM = 128, kTN = 256, kTK = 64;  // output tile; K padding of the slice buffers
// One ring stage holds every slice tile of a 32-deep k-block (64-byte rows,
// 64-byte swizzle): each slice tile crosses L2 once per k-block, and all the
// slice products of that k-block are issued from the one stage.
constexpr int kKB = 32;
constexpr int kStages = 3;
constexpr int kSplitThreads = 192;  // producer, MMA issuer, four epilogue warps
constexpr uint32_t kSliceA = kTM * kKB * 2;  // 8 KB
constexpr uint32_t kSliceB = kTN * kKB * 2;  // 16 KB
constexpr uint32_t kStageBytes = 3 * (kSliceA + kSliceB);  // 72 KB (three slices)
constexpr uint32_t kTmemCols = 512;  // two 256-column accumulators
constexpr long long kWaitLimit = 1ll << 26;

__device__ int g_split_error;

// ---------------------------------------------------------------- PTX helpers
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
// Bounded wait for the phase with parity `parity`; false on time-out.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  const uint32_t a = smem_u32(bar);
  for (long long it = 0; it < kWaitLimit; ++it) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  atomicExch(&g_split_error, 1);
  return false;
}
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          smem_u32(dst)),
      "l"(map), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}
// tcgen05 shared-memory matrix descriptor: K-major, 64-byte swizzle, 8-row
// core-matrix groups 512 bytes apart, descriptor version 1.
__device__ __forceinline__ uint64_t smem_desc_sw64(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3ffff) >> 4);  // start address
  d |= (uint64_t)1 << 16;                   // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)(512 >> 4) << 32;          // stride byte offset: 8 rows x 64 B
  d |= (uint64_t)1 << 46;                   // version
  d |= (uint64_t)4 << 61;                   // swizzle: 64B
  return d;
}
// Instruction descriptor, kind::f16: D = F32, A = B = BF16, both K-major.
__host__ __device__ constexpr uint32_t idesc_bf16_f32(int m, int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}
__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t da, uint64_t db, uint32_t idesc, uint32_t accum) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(da), "l"(db), "r"(idesc), "r"(accum));
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

// ---------------------------------------------------------------- preprocessing
__device__ __forceinline__ int exp_of(double x) {  // unbiased exponent of |x| (0 for 0 / subnormal)
  const int e = (int)((__double_as_longlong(x) >> 52) & 0x7ff);
  return e == 0 ? 0 : e - 1023;
}
// 2^e as a double for e in [-1022, 1023]
__device__ __forceinline__ double pow2(int e) { return __longlong_as_double((long long)(e + 1023) << 52); }
// Scaling exponent of a row / column: its max exponent clamped to [-1000, 1000]
// (0 for an all-zero row, whose recorded max stays at the fill value).
__device__ __forceinline__ int scale_exp(int e) { return (e < -1100) ? 0 : max(min(e, 1000), -1000); }

// (double)f * 2^e built from the bits with integer arithmetic (exact: a power-of-
// two scaling), for normal f whose scaled exponent stays normal; zero keeps its
// sign.  Other cases (FP32 subnormal/inf/NaN, FP64 over/underflow) take the FP64
// multiply.  Costs no FP64-pipe instruction on the common path.
__device__ __forceinline__ double f32_scaled_to_f64(float f, int e) {
  const uint32_t u = __float_as_uint(f);
  if ((u & 0x7fffffffu) == 0u) return __longlong_as_double((long long)((uint64_t)(u >> 31) << 63));
  const int ex = (int)((u >> 23) & 0xffu);
  const int dex = ex - 127 + 1023 + e;
  if (ex == 0 || ex == 0xff || dex <= 0 || dex >= 2047) return (double)f * pow2(max(min(e, 1000), -1000));
  const uint64_t bits = ((uint64_t)(u >> 31) << 63) | ((uint64_t)dex << 52) | ((uint64_t)(u & 0x7fffffu) << 29);
  return __longlong_as_double((long long)bits);
}

// Per-row max exponent of A (column-major m x k), atomicMax into rexp (init INT_MIN).
constexpr int kRowExpChunk = 32;  // columns per thread: k / 32 CTAs along K
template <typename TI>
__global__ void row_exp_kernel(int m, int k, const TI* __restrict__ A, int64_t lda, int* __restrict__ rexp) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  const int c0 = blockIdx.y * kRowExpChunk, c1 = min(k, c0 + kRowExpChunk);
  int e = INT_MIN;
  for (int c = c0; c < c1; ++c) {
    const TI x = A[(size_t)c * lda + i];
    if constexpr (sizeof(TI) == 4) {  // FP32: the exponent from the bits (no FP64 conversion)
      const uint32_t b = __float_as_uint((float)x) & 0x7fffffffu;
      if (b == 0u) continue;
      const int ex = (int)(b >> 23);
      e = max(e, ex != 0 ? ex - 127 : exp_of((double)x));
    } else {
      const double v = (double)x;
      if (v != 0.0) e = max(e, exp_of(v));
    }
  }
  if (e != INT_MIN) atomicMax(&rexp[i], e);
}
// Split one scaled value into `slices` BF16 parts (FP32 arithmetic: the
// scaled value is first rounded to FP32, whose 24 bits three slices cover).
__device__ __forceinline__ void split3(double v, int slices, __nv_bfloat16* out) {
  float x = (float)v;
  for (int s = 0; s < 3; ++s) {
    const __nv_bfloat16 h = __float2bfloat16_rn(x);
    out[s] = (s < slices) ? h : __float2bfloat16_rn(0.f);
    x -= __bfloat162float(h);
  }
}

// A (m x k column-major) -> slices [s][mp][kp] (row-major: K contiguous),
// 32 x 32 tiles transposed through shared memory; the grid covers the padded
// mp x kp extent and writes its zeros too, so the buffer needs no memset.
template <typename TI>
__global__ void split_a_kernel(int m, int k, const TI* __restrict__ A, int64_t lda, const int* __restrict__ rexp,
                               int mp, int kp, int slices, __nv_bfloat16* __restrict__ out) {
  __shared__ double t[32][33];
  const int i0 = blockIdx.y * 32, c0 = blockIdx.x * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8 threads
  for (int r = ty; r < 32; r += 8) {
    const int i = i0 + tx, c = c0 + r;
    double v = 0.0;
    if (i < m && c < k) v = (double)A[(size_t)c * lda + i] * pow2(-scale_exp(rexp[i]));
    t[r][tx] = v;  // t[k][m]
  }
  __syncthreads();
  for (int r = ty; r < 32; r += 8) {
    const int i = i0 + r, c = c0 + tx;  // write row i, column c (K contiguous)
    __nv_bfloat16 h[3];
    split3(t[tx][r], slices, h);
    for (int s = 0; s < 3; ++s) out[((size_t)s * mp + i) * kp + c] = h[s];
  }
}
// B (k x n column-major: column j contiguous over K) -> slices [s][np][kp],
// one CTA per (padded) column: the column's max exponent (cexp[j], 0 for an
// all-zero or padding column) first, then the split, reading the column a
// second time from L2.
template <typename TI>
__global__ void __launch_bounds__(256) split_b_kernel(int k, int n, const TI* __restrict__ B, int64_t ldb,
                                                      int* __restrict__ cexp, int np, int kp, int slices,
                                                      __nv_bfloat16* __restrict__ out) {
  __shared__ int s_e[8];
  const int j = blockIdx.x;
  const TI* col = B + (size_t)j * ldb;
  int e = INT_MIN;
  if (j < n)
    for (int c = threadIdx.x; c < k; c += blockDim.x) {
      const double v = (double)col[c];
      if (v != 0.0) e = max(e, exp_of(v));
    }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) e = max(e, __shfl_xor_sync(0xffffffffu, e, off));
  if ((threadIdx.x & 31) == 0) s_e[threadIdx.x >> 5] = e;
  __syncthreads();
  int ce = INT_MIN;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) ce = max(ce, s_e[w]);
  ce = (ce == INT_MIN) ? 0 : ce;
  if (threadIdx.x == 0 && j < np) cexp[j] = ce;
  const double sc = pow2(-scale_exp(ce));
  for (int c = threadIdx.x; c < kp; c += blockDim.x) {
    double v = 0.0;
    if (j < n && c < k) v = (double)col[c] * sc;
    __nv_bfloat16 h[3];
    split3(v, slices, h);
    for (int s = 0; s < 3; ++s) out[((size_t)s * np + j) * kp + c] = h[s];
  }
}

// ---------------------------------------------------------------- the GEMM
struct SplitArgs {
  int m, n, k;
  int mp, np, kp;
  int npairs, slices;
  int pa[6], pb[6];  // slice pairs
  double alpha, beta;
  void* C;
  int64_t ldc;
  const int* rexp;
  const int* cexp;
};

template <typename TO>
__global__ void __launch_bounds__(kSplitThreads, 1)
    split_gemm_kernel(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB,
                      const SplitArgs g) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  // 1024-byte aligned stage ring (every slice tile starts on a 512-byte swizzle pattern)
  unsigned char* smem = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
  __shared__ __align__(8) uint64_t full_bar[kStages], empty_bar[kStages], acc_full[2], acc_empty[2];
  __shared__ uint32_t tmem_base_sh;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int kblocks = (g.npairs > 0) ? g.kp / kKB : 0;  // k-blocks per tile
  const int tiles_m = g.mp / kTM;
  const int ntiles = tiles_m * (g.np / kTN);
  const uint32_t stage_tx = (uint32_t)g.slices * (kSliceA + kSliceB);

  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(&full_bar[s], 1);
      mbar_init(&empty_bar[s], 1);
    }
    for (int a = 0; a < 2; ++a) {
      mbar_init(&acc_full[a], 1);
      mbar_init(&acc_empty[a], 4);  // one arrival per epilogue warp
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {  // TMEM: 128 lanes x 512 FP32 columns = two accumulators
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base_sh)),
                 "r"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_base_sh;

  if (warp == 0 && lane == 0) {
    // producer: TMA loads of every slice tile of A and B, k-block after
    // k-block, tile after tile (the ring's position runs on across tiles)
    int gk = 0;
    bool ok = true;
    for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
      const int m0 = (t % tiles_m) * kTM, n0 = (t / tiles_m) * kTN;
      for (int it = 0; it < kblocks; ++it, ++gk) {
        const int s = gk % kStages;
        const uint32_t ph = (uint32_t)(gk / kStages) & 1u;
        if (!mbar_wait(&empty_bar[s], ph ^ 1u)) {
          ok = false;
          break;
        }
        unsigned char* sa = smem + (size_t)s * kStageBytes;
        unsigned char* sb = sa + 3 * kSliceA;
        mbar_expect_tx(&full_bar[s], stage_tx);
        for (int p = 0; p < g.slices; ++p) tma_load_2d(sa + p * kSliceA, &mapA, it * kKB, p * g.mp + m0, &full_bar[s]);
        for (int q = 0; q < g.slices; ++q) tma_load_2d(sb + q * kSliceB, &mapB, it * kKB, q * g.np + n0, &full_bar[s]);
      }
    }
  } else if (warp == 1 && lane == 0) {
    // MMA issuer: tile j into accumulator j & 1, once the epilogue has emptied it
    constexpr uint32_t idesc = idesc_bf16_f32(kTM, kTN);
    int gk = 0;
    bool ok = true;
    for (int t = blockIdx.x, j = 0; t < ntiles && ok; t += gridDim.x, ++j) {
      const int slot = j & 1;
      const uint32_t use = (uint32_t)(j >> 1) & 1u;
      if (!mbar_wait(&acc_empty[slot], use ^ 1u)) break;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t acc = tmem + (uint32_t)slot * kTN;
      for (int it = 0; it < kblocks; ++it, ++gk) {
        const int s = gk % kStages;
        const uint32_t ph = (uint32_t)(gk / kStages) & 1u;
        if (!mbar_wait(&full_bar[s], ph)) {
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t sa = smem_u32(smem + (size_t)s * kStageBytes);
        const uint32_t sb = sa + 3 * kSliceA;
        for (int pr = 0; pr < g.npairs; ++pr) {
          const uint32_t ta = sa + (uint32_t)g.pa[pr] * kSliceA, tb = sb + (uint32_t)g.pb[pr] * kSliceB;
#pragma unroll
          for (int kk = 0; kk < kKB / 16; ++kk)  // K = 16 per instruction: +32 bytes in the swizzled row
            mma_bf16(acc, smem_desc_sw64(ta + kk * 32), smem_desc_sw64(tb + kk * 32), idesc,
                     (it > 0 || pr > 0 || kk > 0) ? 1u : 0u);
        }
        mma_commit(&empty_bar[s]);  // stage free once these MMAs have read it
      }
      if (ok) mma_commit(&acc_full[slot]);  // accumulator complete
    }
  } else if (warp >= 2) {
    // epilogue: warp w reads TMEM lanes 32 (w mod 4) .. + 31 (the tile's rows)
    const int q = warp & 3;
    const float falpha = (float)g.alpha, fbeta = (float)g.beta;
    const bool plain = (g.alpha == 1.0 && g.beta == 0.0);  // C = A B: no FP64 arithmetic in the epilogue
    for (int t = blockIdx.x, j = 0; t < ntiles; t += gridDim.x, ++j) {
      const int slot = j & 1;
      const uint32_t use = (uint32_t)(j >> 1) & 1u;
      const int m0 = (t % tiles_m) * kTM, n0 = (t / tiles_m) * kTN;
      if (g.beta != 0.0) {
        // bring the C tile this epilogue reads into L2 while the tile's
        // products run (one 128-byte line per prefetch, valid elements only)
        constexpr int kLineElems = 128 / (int)sizeof(TO);
        constexpr int lines_per_col = kTM / kLineElems;
        for (int e = threadIdx.x - 64; e < kTN * lines_per_col; e += 128) {
          const int col = n0 + e / lines_per_col;
          const int r = m0 + (e % lines_per_col) * kLineElems;
          if (col < g.n && r < g.m) {
            const TO* cp = static_cast<const TO*>(g.C) + (size_t)col * g.ldc + r;
            asm volatile("prefetch.global.L2 [%0];" ::"l"(cp));
          }
        }
      }
      if (!mbar_wait(&acc_full[slot], use)) break;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const int row = m0 + q * 32 + lane;
      const double srow = (row < g.m) ? pow2(scale_exp(g.rexp[row])) : 0.0;
      const int erow = (row < g.m) ? scale_exp(g.rexp[row]) : 0;
      for (int c0 = 0; c0 < kTN; c0 += 16) {
        uint32_t v[16];
        const uint32_t taddr = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)slot * kTN + (uint32_t)c0;
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
            : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
              "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
            : "r"(taddr));
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        if (row >= g.m) continue;
#pragma unroll
        for (int jj = 0; jj < 16; ++jj) {
          const int col = n0 + c0 + jj;
          if (col < g.n) {
            TO* cp = static_cast<TO*>(g.C) + (size_t)col * g.ldc + row;
            if constexpr (sizeof(TO) == 8) {
              if (plain) {
                *cp = f32_scaled_to_f64(__uint_as_float(v[jj]), erow + scale_exp(g.cexp[col]));
              } else {
                const double val = (double)__uint_as_float(v[jj]) * srow * pow2(scale_exp(g.cexp[col]));
                *cp = (g.beta == 0.0) ? g.alpha * val : fma(g.alpha, val, g.beta * *cp);
              }
            } else {  // FP32 output: integer exponent arithmetic and FP32 only
              const float val = ldexpf(__uint_as_float(v[jj]), erow + scale_exp(g.cexp[col]));
              *cp = (fbeta == 0.f) ? falpha * val : fmaf(falpha, val, fbeta * *cp);
            }
          }
        }
      }
      // the accumulator's columns are read: hand it back to the MMA issuer
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncwarp();
      if (lane == 0) mbar_arrive(&acc_empty[slot]);
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols));
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPoint("cuTensorMapEncodeTiled", &p, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  }
  return fn;
}

int make_map(CUtensorMap* map, void* base, uint64_t rows, uint64_t kp, uint32_t box_rows) {
  EncodeTiledFn f = encode_fn();
  if (!f) return record_arg_error(-100, "split gemm: cuTensorMapEncodeTiled unavailable");
  const cuuint64_t dims[2] = {kp, rows};
  const cuuint64_t strides[1] = {kp * 2};
  const cuuint32_t box[2] = {(cuuint32_t)kKB, box_rows};
  const cuuint32_t estr[2] = {1, 1};
  CUresult r = f(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, base, dims, strides, box, estr,
                 CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                 CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return record_arg_error(-101, "split gemm: cuTensorMapEncodeTiled failed");
  return NACU_SUCCESS;
}

size_t round_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

struct SplitLayout {
  int mp, np, kp;
  size_t a_off, b_off, rexp_off, cexp_off, total;
};
SplitLayout split_layout(int m, int n, int k) {
  SplitLayout L;
  L.mp = (int)round_up((size_t)(m > 0 ? m : 1), kTM);
  L.np = (int)round_up((size_t)(n > 0 ? n : 1), kTN);
  L.kp = (int)round_up((size_t)(k > 0 ? k : 1), kTK);
  L.a_off = 0;
  L.b_off = round_up(L.a_off + (size_t)3 * L.mp * L.kp * 2, 1024);
  L.rexp_off = round_up(L.b_off + (size_t)3 * L.np * L.kp * 2, 256);
  L.cexp_off = round_up(L.rexp_off + (size_t)L.mp * 4, 256);
  L.total = round_up(L.cexp_off + (size_t)L.np * 4, 256);
  return L;
}

}  // namespace
}  // namespace nacu

extern "C" {

size_t nacu_gemm_split_workspace_bytes(int m, int n, int k) { return nacu::split_layout(m, n, k).total; }

int nacu_split_gemm_error(int* flag_out) {
  int v = 0;
  cudaError_t e = cudaMemcpyFromSymbol(&v, nacu::g_split_error, sizeof(int));
  if (e != cudaSuccess) return nacu::record_cuda_error(e, "nacu_split_gemm_error");
  if (flag_out) *flag_out = v;
  return NACU_SUCCESS;
}

}  // extern "C"

namespace nacu {

template <typename TI, typename TO>
int split_gemm_run(int m, int n, int k, double alpha, const TI* A, int64_t lda, const TI* B, int64_t ldb, double beta,
                   TO* C, int64_t ldc, int slices, void* workspace, size_t workspace_bytes, cudaStream_t stream) {
  if (m < 0) return record_arg_error(-1, "dgemm_split_bf16: m < 0");
  if (n < 0) return record_arg_error(-2, "dgemm_split_bf16: n < 0");
  if (k < 0) return record_arg_error(-3, "dgemm_split_bf16: k < 0");
  if (m == 0 || n == 0) return NACU_SUCCESS;
  if (k > 0 && (!A || lda < (m > 1 ? m : 1))) return record_arg_error(-5, "dgemm_split_bf16: bad A / lda");
  if (k > 0 && (!B || ldb < (k > 1 ? k : 1))) return record_arg_error(-7, "dgemm_split_bf16: bad B / ldb");
  if (!C || ldc < (m > 1 ? m : 1)) return record_arg_error(-10, "dgemm_split_bf16: bad C / ldc");
  if (slices < 1 || slices > 3) return record_arg_error(-12, "dgemm_split_bf16: slices out of range [1, 3]");
  const SplitLayout L = split_layout(m, n, k);
  if (!workspace || workspace_bytes < L.total) return record_arg_error(-13, "dgemm_split_bf16: workspace too small");
  if ((reinterpret_cast<uintptr_t>(workspace) & 1023) != 0)
    return record_arg_error(-13, "dgemm_split_bf16: workspace must be 1024-byte aligned");
  cudaStream_t s = stream;
  unsigned char* ws = static_cast<unsigned char*>(workspace);
  __nv_bfloat16* as = reinterpret_cast<__nv_bfloat16*>(ws + L.a_off);
  __nv_bfloat16* bs = reinterpret_cast<__nv_bfloat16*>(ws + L.b_off);
  int* rexp = reinterpret_cast<int*>(ws + L.rexp_off);
  int* cexp = reinterpret_cast<int*>(ws + L.cexp_off);
  // INT_MIN the row exponents (0x80 bytes give 0x80808080 < any real
  // exponent); the split kernels write every element of the padded slice
  // buffers, zeros included
  cudaError_t e = cudaMemsetAsync(rexp, 0x80, (size_t)L.mp * 4, s);
  if (e != cudaSuccess) return record_cuda_error(e, "nacu_dgemm_split_bf16");
  if (k > 0) {
    row_exp_kernel<TI><<<dim3((m + 255) / 256, (k + kRowExpChunk - 1) / kRowExpChunk), 256, 0, s>>>(m, k, A, lda,
                                                                                                 rexp);
    split_a_kernel<TI><<<dim3(L.kp / 32, L.mp / 32), 256, 0, s>>>(m, k, A, lda, rexp, L.mp, L.kp, slices, as);
    split_b_kernel<TI><<<L.np, 256, 0, s>>>(k, n, B, ldb, cexp, L.np, L.kp, slices, bs);
    int rc = check_launch("nacu_dgemm_split_bf16: split");
    if (rc != NACU_SUCCESS) return rc;
  } else {
    e = cudaMemsetAsync(cexp, 0, (size_t)L.np * 4, s);
    if (e != cudaSuccess) return record_cuda_error(e, "nacu_dgemm_split_bf16");
  }
  CUtensorMap mapA, mapB;
  int rc = make_map(&mapA, as, (uint64_t)3 * L.mp, L.kp, kTM);
  if (rc == NACU_SUCCESS) rc = make_map(&mapB, bs, (uint64_t)3 * L.np, L.kp, kTN);
  if (rc != NACU_SUCCESS) return rc;
  SplitArgs g{};
  g.m = m;
  g.n = n;
  g.k = k;
  g.mp = L.mp;
  g.np = L.np;
  g.kp = L.kp;
  // slice pairs (p, q) with p + q <= slices - 1 (0-based), largest terms first
  int np_ = 0;
  for (int sum = 0; sum < slices; ++sum)
    for (int p = 0; p <= sum; ++p) {
      g.pa[np_] = p;
      g.pb[np_] = sum - p;
      ++np_;
    }
  g.npairs = (k > 0) ? np_ : 0;
  g.slices = slices;
  g.alpha = alpha;
  g.beta = beta;
  g.C = C;
  g.ldc = ldc;
  g.rexp = rexp;
  g.cexp = cexp;
  const size_t smem = (size_t)kStages * kStageBytes + 1024;
  e = ensure_dynamic_smem(split_gemm_kernel<TO>, smem);
  if (e != cudaSuccess) return record_cuda_error(e, "nacu_dgemm_split_bf16");
  const int ntiles = (L.mp / kTM) * (L.np / kTN);
  // FP64 output (the public GEMM): persistent, one CTA per SM looping over the
  // tiles.  FP32 output (the large LU's trailing updates): one CTA per tile, so
  // that the look-ahead's concurrent update on the other stream still finds
  // SMs (persistent CTAs would hold every SM until the bulk update ends).
  const int grid = (sizeof(TO) == 8 && ntiles > sm_count()) ? sm_count() : ntiles;
  if (g.npairs == 0) {  // k == 0: C = beta * C
    if constexpr (sizeof(TO) == 8)
      return nacu_dgemm(m, n, 0, alpha, nullptr, m > 1 ? m : 1, nullptr, 1, beta, C, ldc, stream);
    else
      return record_arg_error(-3, "split gemm: k == 0 is not supported for FP32 output");
  }
  split_gemm_kernel<TO><<<grid, kSplitThreads, smem, s>>>(mapA, mapB, g);
  return check_launch("nacu_dgemm_split_bf16");
}


template int split_gemm_run<float, float>(int, int, int, double, const float*, int64_t, const float*, int64_t,
                                           double, float*, int64_t, int, void*, size_t, cudaStream_t);
}  // namespace nacu

extern "C" int nacu_dgemm_split_bf16(int m, int n, int k, double alpha, const double* A, int64_t lda, const double* B,
                                     int64_t ldb, double beta, double* C, int64_t ldc, int slices, void* workspace,
                                     size_t workspace_bytes, nacu_stream_t stream) {
  return nacu::split_gemm_run<double, double>(m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, slices, workspace,
                                              workspace_bytes, (cudaStream_t)stream);
}
