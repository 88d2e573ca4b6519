// Plain FP64 GEMM: C = alpha * A * B + beta * C, column-major, the GPU form of
// nalgebra's `Matrix::gemm` (src/base/blas.rs:729-746 -> gemm_uninit,
// src/base/blas_uninit.rs:187-333, which hands Dyn f64 matrices to
// matrixmultiply::dgemm).  As in nalgebra, beta == 0 means C is never read.
//
// Design (GB300): FP64 is bound by the FP64 pipe (~1 TFLOP/s), so the kernel
// only has to keep that pipe fed: 64 x 64 CTA tiles, 256 threads, a 4 x 4
// register tile per thread (16 independent DFMA chains), 16-deep K slices
// staged in shared memory with the next slice prefetched into registers while
// the current one is consumed.  Loads of A (column-major: rows contiguous) and
// B (columns contiguous along K) are coalesced; edges are zero-filled.
#include "common.cuh"

namespace nacu {
namespace {

constexpr int kBM = 64, kBN = 64, kBK = 16, kGemmThreads = 256;

__global__ void __launch_bounds__(kGemmThreads, 3)
    dgemm_kernel(int M, int N, int K, double alpha, const double* __restrict__ A, int64_t lda,
                 const double* __restrict__ B, int64_t ldb, double beta, double* __restrict__ C, int64_t ldc) {
  __shared__ __align__(16) double As[2][kBK][kBM];
  __shared__ __align__(16) double Bs[2][kBK][kBN + 2];  // +2: conflict-free column writes
  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;
  const int m0 = blockIdx.x * kBM, n0 = blockIdx.y * kBN;
  // loader mapping: A slice (64 x 16): 4 elements per thread, rows contiguous
  const int ar = tid & 63, ak = tid >> 6;   // rows ar, k = ak + 4*u
  // B slice (16 x 64): k contiguous within a column
  const int bk = tid & 15, bc = tid >> 4;   // k = bk, columns bc + 16*u
  double ra[4], rb[4];
  auto load = [&](int k0) {
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int k = k0 + ak + 4 * u, r = m0 + ar;
      ra[u] = (r < M && k < K) ? A[(size_t)k * lda + r] : 0.0;
      const int c = n0 + bc + 16 * u, kb = k0 + bk;
      rb[u] = (c < N && kb < K) ? B[(size_t)c * ldb + kb] : 0.0;
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
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = 0.0;
  load(0);
  store(0);
  __syncthreads();
  int buf = 0;
  for (int k0 = 0; k0 < K; k0 += kBK) {
    const bool more = k0 + kBK < K;
    if (more) load(k0 + kBK);  // prefetch the next slice into registers
#pragma unroll
    for (int k = 0; k < kBK; ++k) {
      const double2 a01 = *reinterpret_cast<const double2*>(&As[buf][k][ty * 4]);
      const double2 a23 = *reinterpret_cast<const double2*>(&As[buf][k][ty * 4 + 2]);
      const double a[4] = {a01.x, a01.y, a23.x, a23.y};
      double b[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[buf][k][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
    }
    if (more) {
      store(buf ^ 1);
      __syncthreads();
      buf ^= 1;
    }
  }
  // epilogue: thread (ty, tx) owns rows m0 + 4ty + i, columns n0 + tx + 16j
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int c = n0 + tx + 16 * j;
    if (c >= N) continue;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int r = m0 + ty * 4 + i;
      if (r >= M) continue;
      double* cp = C + (size_t)c * ldc + r;
      *cp = (beta == 0.0) ? alpha * acc[i][j] : fma(alpha, acc[i][j], beta * *cp);
    }
  }
}

}  // namespace
}  // namespace nacu

extern "C" int nacu_dgemm(int m, int n, int k, double alpha, const double* A, int64_t lda, const double* B,
                          int64_t ldb, double beta, double* C, int64_t ldc, nacu_stream_t stream) {
  using namespace nacu;
  if (m < 0) return record_arg_error(-1, "dgemm: m < 0");
  if (n < 0) return record_arg_error(-2, "dgemm: n < 0");
  if (k < 0) return record_arg_error(-3, "dgemm: k < 0");
  if (m == 0 || n == 0) return NACU_SUCCESS;
  if (k > 0 && !A) return record_arg_error(-5, "dgemm: null A");
  if (lda < (m > 1 ? m : 1)) return record_arg_error(-6, "dgemm: lda < max(1, m)");
  if (k > 0 && !B) return record_arg_error(-7, "dgemm: null B");
  if (ldb < (k > 1 ? k : 1)) return record_arg_error(-8, "dgemm: ldb < max(1, k)");
  if (!C) return record_arg_error(-10, "dgemm: null C");
  if (ldc < (m > 1 ? m : 1)) return record_arg_error(-11, "dgemm: ldc < max(1, m)");
  dim3 grid((m + kBM - 1) / kBM, (n + kBN - 1) / kBN);
  if (grid.y > 65535) return record_arg_error(-2, "dgemm: n too large for one launch");
  dgemm_kernel<<<grid, kGemmThreads, 0, (cudaStream_t)stream>>>(m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
  return check_launch("nacu_dgemm");
}
