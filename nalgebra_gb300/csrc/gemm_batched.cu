// Batched small GEMM: C_s = alpha * A_s * B_s + beta * C_s for many
// independent column-major FP64 products in one launch -- the GPU form of
// nalgebra's `&a * &b` (src/base/ops.rs:566-570, `gemm_uninit` with alpha = 1,
// beta = 0) and of `Matrix::gemm` (src/base/blas.rs:729-746) over a batch.
//
// nalgebra computes a product in one of two orders (gemm_uninit,
// src/base/blas_uninit.rs:187-333): Dyn matrices with every dimension above 5
// go to matrixmultiply::dgemm, whose blocking and summation order are not in
// the reference; everything else (a dimension <= 5, or static sizes) runs
// gemv_uninit per output column, i.e. for each output element the sequential
// sum over l = 0..k-1 of fl(fl(alpha * A_il) * B_lj), the first term added to
// fl(beta * C_ij) (or standing alone when beta == 0), each step rounded
// separately (array_axcpy / array_axc, blas_uninit.rs:32-78, 127-176).
// NACU_FLAG_EXACT reproduces that order bit for bit; the default form
// contracts each step to one FMA and applies alpha and beta once at the end.
//
// Design (GB300): the FP64 pipe (one warp-wide DFMA per 64 cycles on each SM
// sub-partition) bounds the kernel, so lane utilisation decides the speed.
// Each CTA computes one tile of one product; the tile's sides are chosen per
// call as the smallest multiples of 4 (<= 64) that split m and n into equal
// tiles (100 x 100 -> four 52 x 52 tiles, 92% of the padded area used, where
// 64 x 64 tiles would use 61%), and the threads of the tile's 4 x 4 register
// blocks are numbered densely so only the last warp is partial; threads past
// the tile idle.  K runs in 16-deep slices staged in shared memory with the
// next slice prefetched into registers, and the last slice stops at k.
#include "common.cuh"

namespace nacu {
namespace {

constexpr int kBK = 16, kMaxT = 64, kBatchedThreads = 256;

template <bool EXACT>
__global__ void __launch_bounds__(kBatchedThreads, 3)
    gemm_batched_kernel(int M, int N, int K, double alpha, const double* __restrict__ A, int64_t lda, int64_t sA,
                        const double* __restrict__ B, int64_t ldb, int64_t sB, double beta, double* __restrict__ C,
                        int64_t ldc, int64_t sC, int batch, int TM, int TN, int tiles_m) {
  __shared__ __align__(16) double As[2][kBK][kMaxT];
  __shared__ __align__(16) double Bs[2][kBK][kMaxT];
  const int tid = threadIdx.x;
  const int tx_n = TN >> 2;                      // register blocks per tile row
  const int nblk = (TM >> 2) * tx_n;             // blocks of the tile
  const bool active = tid < nblk;
  const int ty = active ? tid / tx_n : 0, tx = active ? tid - (tid / tx_n) * tx_n : 0;
  const int tm = blockIdx.x % tiles_m, tn = blockIdx.x / tiles_m;
  const int m0 = tm * TM, n0 = tn * TN;
  const int mlim = min(M - m0, TM), nlim = min(N - n0, TN);  // rows / columns of C in this tile
  // loaders: A slice (TM x 16, rows contiguous), B slice (16 x TN, K contiguous)
  const int ar = tid & 63, ak = tid >> 6;  // rows ar, k = ak + 4u
  const int bk = tid & 15, bc = tid >> 4;  // k = bk, columns bc + 16u
  const bool alpha_one = alpha == 1.0;
  for (int s = blockIdx.y; s < batch; s += gridDim.y) {
    const double* a = A + (size_t)s * sA;
    const double* b = B + (size_t)s * sB;
    double* c = C + (size_t)s * sC;
    double ra[4], rb[4];
    auto load = [&](int k0) {
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int kk = k0 + ak + 4 * u;
        ra[u] = (ar < mlim && kk < K) ? a[(size_t)kk * lda + m0 + ar] : 0.0;
        const int cc = bc + 16 * u, kb = k0 + bk;
        rb[u] = (cc < nlim && kb < K) ? b[(size_t)(n0 + cc) * ldb + kb] : 0.0;
      }
    };
    auto store = [&](int buf) {
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        As[buf][ak + 4 * u][ar] = ra[u];
        Bs[buf][bk][bc + 16 * u] = rb[u];
      }
    };
    double acc[4][4];
    if constexpr (EXACT) {
      // gemv's first column step adds fl(beta * C) (array_axcpy), or nothing
      // when beta == 0 (array_axc): -0.0 is the exact neutral start, since
      // fl(t + -0) = t for every t, signed zeros included.
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const int r = 4 * ty + i, q = 4 * tx + j;
          acc[i][j] = (beta != 0.0 && active && r < mlim && q < nlim)
                          ? __dmul_rn(beta, c[(size_t)(n0 + q) * ldc + m0 + r]) : -0.0;
        }
    } else {
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = 0.0;
    }
    __syncthreads();  // the previous product's last slice is consumed
    if (K > 0) {
      load(0);
      store(0);
    }
    __syncthreads();
    int buf = 0;
    const bool work = active && 4 * ty < mlim && 4 * tx < nlim;
    for (int k0 = 0; k0 < K; k0 += kBK) {
      const bool more = k0 + kBK < K;
      if (more) load(k0 + kBK);  // prefetch the next slice into registers
      if (work) {
        const int kmax = min(kBK, K - k0);
#pragma unroll
        for (int kk = 0; kk < kBK; ++kk) {
          if (kk < kmax) {
            const double2 a01 = *reinterpret_cast<const double2*>(&As[buf][kk][4 * ty]);
            const double2 a23 = *reinterpret_cast<const double2*>(&As[buf][kk][4 * ty + 2]);
            const double2 b01 = *reinterpret_cast<const double2*>(&Bs[buf][kk][4 * tx]);
            const double2 b23 = *reinterpret_cast<const double2*>(&Bs[buf][kk][4 * tx + 2]);
            double av[4] = {a01.x, a01.y, a23.x, a23.y};
            const double bv[4] = {b01.x, b01.y, b23.x, b23.y};
            if constexpr (EXACT) {
              if (!alpha_one)
#pragma unroll
                for (int i = 0; i < 4; ++i) av[i] = __dmul_rn(alpha, av[i]);
#pragma unroll
              for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = __dadd_rn(__dmul_rn(av[i], bv[j]), acc[i][j]);
            } else {
#pragma unroll
              for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fma(av[i], bv[j], acc[i][j]);
            }
          }
        }
      }
      if (more) {
        store(buf ^ 1);
        __syncthreads();
        buf ^= 1;
      }
    }
    if (active) {
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int q = 4 * tx + j;
        if (q >= nlim) continue;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const int r = 4 * ty + i;
          if (r >= mlim) continue;
          double* cp = c + (size_t)(n0 + q) * ldc + m0 + r;
          if (K == 0) {  // gemv_uninit with ncols == 0: y = 0 or y *= beta
            *cp = (beta == 0.0) ? 0.0 : *cp * beta;
          } else if constexpr (EXACT) {
            *cp = acc[i][j];
          } else {
            *cp = (beta == 0.0) ? alpha * acc[i][j] : fma(alpha, acc[i][j], beta * *cp);
          }
        }
      }
    }
  }
}

// Smallest multiple of 4 (<= kMaxT) that splits `dim` into equal tiles.
int tile_side(int dim) {
  if (dim <= 0) return 4;
  const int tiles = (dim + kMaxT - 1) / kMaxT;
  const int per = (dim + tiles - 1) / tiles;
  return (per + 3) & ~3;
}

}  // namespace
}  // namespace nacu

extern "C" int nacu_dgemm_batched(int m, int n, int k, double alpha, const double* A, int64_t lda, int64_t strideA,
                                  const double* B, int64_t ldb, int64_t strideB, double beta, double* C, int64_t ldc,
                                  int64_t strideC, int batch, int flags, nacu_stream_t stream) {
  using namespace nacu;
  if (m < 0) return record_arg_error(-1, "dgemm_batched: m < 0");
  if (n < 0) return record_arg_error(-2, "dgemm_batched: n < 0");
  if (k < 0) return record_arg_error(-3, "dgemm_batched: k < 0");
  if (batch < 0) return record_arg_error(-15, "dgemm_batched: negative batch");
  if (m == 0 || n == 0 || batch == 0) return NACU_SUCCESS;
  if (k > 0 && !A) return record_arg_error(-5, "dgemm_batched: null A");
  if (lda < (m > 1 ? m : 1)) return record_arg_error(-6, "dgemm_batched: lda < max(1, m)");
  if (batch > 1 && k > 0 && strideA < lda * k) return record_arg_error(-7, "dgemm_batched: strideA < lda * k");
  if (k > 0 && !B) return record_arg_error(-8, "dgemm_batched: null B");
  if (ldb < (k > 1 ? k : 1)) return record_arg_error(-9, "dgemm_batched: ldb < max(1, k)");
  if (batch > 1 && k > 0 && strideB < ldb * n) return record_arg_error(-10, "dgemm_batched: strideB < ldb * n");
  if (!C) return record_arg_error(-12, "dgemm_batched: null C");
  if (ldc < (m > 1 ? m : 1)) return record_arg_error(-13, "dgemm_batched: ldc < max(1, m)");
  if (batch > 1 && strideC < ldc * n) return record_arg_error(-14, "dgemm_batched: strideC < ldc * n");
  const int TM = tile_side(m), TN = tile_side(n);
  const int tiles_m = (m + TM - 1) / TM, tiles_n = (n + TN - 1) / TN;
  const int64_t tiles = (int64_t)tiles_m * tiles_n;
  if (tiles > 0x7fffffff) return record_arg_error(-2, "dgemm_batched: too many tiles for one launch");
  dim3 grid((unsigned)tiles, (unsigned)(batch < 65535 ? batch : 65535));
  const bool exact = (flags & NACU_FLAG_EXACT) != 0;
  cudaStream_t s = (cudaStream_t)stream;
  if (exact)
    gemm_batched_kernel<true><<<grid, kBatchedThreads, 0, s>>>(m, n, k, alpha, A, lda, strideA, B, ldb, strideB, beta,
                                                               C, ldc, strideC, batch, TM, TN, tiles_m);
  else
    gemm_batched_kernel<false><<<grid, kBatchedThreads, 0, s>>>(m, n, k, alpha, A, lda, strideA, B, ldb, strideB, beta,
                                                                C, ldc, strideC, batch, TM, TN, tiles_m);
  return check_launch("nacu_dgemm_batched");
}
