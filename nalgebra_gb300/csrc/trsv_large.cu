// Triangular solves of one large matrix (any n): the GPU form of nalgebra's
// Matrix::{solve,tr_solve,ad_solve}_{lower,upper}_triangular_mut and
// solve_lower_triangular_with_diag_mut (src/linalg/solve.rs:55-442) past the
// batched kernel's n <= 128, e.g. the reference's 1000 x 1000 solve benches
// (benches/linalg/solve.rs).  Each right-hand-side column is one launch.
//
// The solve is bound by reading the triangle once (n^2/2 doubles per column),
// so the kernel streams it at HBM rate with as much of it in flight as the
// dependency chain allows: the rows are cut into 64-row blocks and each CTA
// takes one block in ticket order (tickets are drawn when the CTA starts, so a
// CTA only ever waits for blocks whose CTAs are already running).  A CTA first
// loads its diagonal block into shared memory; then, for every block solved
// before it, it prefetches its tile of the triangle into registers, waits for
// that block's flag (bounded: after kTrsvLPollLimit polls it records a timeout
// in info and returns) and applies the tile; then it solves its diagonal block
// 32 rows at a time (one warp, shuffles) and raises its own flag.
//
// The solved system is M x = b with M = T (trans = 0) or T^T (trans = 1),
// T lower or upper; M is lower (forward, blocks top-down) when T is lower and
// not transposed or upper and transposed.  For trans = 0 a thread owns one row
// of a tile and a quarter of its columns (column-major T: coalesced over the
// rows); for trans = 1 the tile of M is a tile of T read across, so a thread
// owns one column of the tile and a quarter of its rows, keeps 16 partial
// sums and the two warps of each quarter reduce them once at the end.
// Arithmetic: FMA, and the reciprocal of each diagonal entry (the batched
// kernel's EXACT form is the bit-identical one).  with_diag (lower, trans = 0,
// solve.rs:106-134) propagates the coefficients b_i / diag but leaves each b_i
// undivided, i.e. returns diag * z where z solves the system whose diagonal is
// `diag`: the kernel solves for z, and a final pass scales it by diag.
#include "common.cuh"

namespace nacu {
namespace {

constexpr int kTrsvLThreads = 256;
constexpr int kTrsvLBS = 64;                                   // rows per block
constexpr int kTrsvLNC = kTrsvLThreads / kTrsvLBS;             // parts per tile
constexpr int kTrsvLCW = kTrsvLBS / kTrsvLNC;                  // columns (rows) per part
constexpr int kTrsvLLD = kTrsvLBS + 1;
constexpr int kTrsvLPollLimit = 1 << 22;  // with the 64 ns back-off: seconds, far above any block's solve
constexpr int kTrsvLInfoTimeout = -1000;

struct TrsvLArgs {
  int n;
  const double* A;
  int64_t lda;
  double* x;
  int fwd;        // M lower: blocks top-down
  int diag_mode;  // 0: T's diagonal; 1: the value dval (with_diag)
  double dval;
  int32_t* info;
  int* sync;  // [0] ticket, [1] timeout flag, [2 + b] block b solved (zeroed before the launch)
  int poll_limit;
};

__device__ __forceinline__ int trsvl_ld_acquire(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void trsvl_st_release(int* p, int v) {
  asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

template <bool TRANS>
__global__ void __launch_bounds__(kTrsvLThreads) trsv_large_kernel(TrsvLArgs g) {
  constexpr int BS = kTrsvLBS, NC = kTrsvLNC, CW = kTrsvLCW, LD = kTrsvLLD;
  extern __shared__ __align__(16) double trsvl_ts[];  // Ts[k * LD + i] = M(r0 + i, r0 + k)
  double* Ts = trsvl_ts;
  __shared__ double xs[BS];
  __shared__ double rd[BS];
  __shared__ double part[NC][BS];
  __shared__ int s_ticket, s_abort;
  const int tid = threadIdx.x;
  const int n = g.n, fwd = g.fwd;
  const int nblk = (n + BS - 1) / BS;
  if (tid == 0) {
    s_ticket = atomicAdd(&g.sync[0], 1);
    s_abort = 0;
  }
  __syncthreads();
  const int t = s_ticket;
  if (t >= nblk) return;
  const int kb = fwd ? t : nblk - 1 - t;
  const int r0 = kb * BS, bs = min(BS, n - r0);
  const double* A = g.A;
  const int64_t lda = g.lda;
  // the strict triangle of M's diagonal block (M(i, k) = T(k, i) when TRANS),
  // column k pre-scaled by 1 / M_kk: the diagonal solve then broadcasts each
  // unscaled value and takes one FMA per step (a one-lane scale per step held
  // the chain for a second warp-wide FP64 instruction); the values are scaled
  // once when the block is stored.  Done before this CTA's turn comes.
  for (int i = tid; i < bs; i += kTrsvLThreads)
    rd[i] = 1.0 / (g.diag_mode == 0 ? A[(size_t)(r0 + i) * lda + r0 + i] : g.dval);
  __syncthreads();
  for (int e = tid; e < bs * bs; e += kTrsvLThreads) {
    const int hi = e / bs, lo = e - hi * bs;  // coalesced: lo runs along T's columns
    const int i = TRANS ? hi : lo, k = TRANS ? lo : hi;
    if (fwd ? (i > k) : (i < k)) Ts[k * LD + i] = A[(size_t)(r0 + hi) * lda + r0 + lo] * rd[k];
  }

  if constexpr (!TRANS) {
    const int tr = tid % BS, tc = tid / BS;
    double acc = (tc == 0 && tr < bs) ? g.x[r0 + tr] : 0.0;
    for (int q = 0; q < t; ++q) {
      const int jb = fwd ? q : nblk - 1 - q;
      const int c0 = jb * BS, cs = min(BS, n - c0);
      double a[CW];
#pragma unroll
      for (int u = 0; u < CW; ++u) {
        const int col = tc * CW + u;
        a[u] = (tr < bs && col < cs) ? A[(size_t)(c0 + col) * lda + r0 + tr] : 0.0;
      }
      if (tid == 0) {
        int polls = 0;
        while (trsvl_ld_acquire(&g.sync[2 + jb]) == 0) {
          if (++polls > g.poll_limit) {
            s_abort = 1;
            atomicExch(&g.sync[1], 1);
            atomicMin(g.info, kTrsvLInfoTimeout);
            break;
          }
          __nanosleep(64);
        }
      }
      __syncthreads();
      if (s_abort) return;
      // the whole of xs: a short last block leaves entries past cs that meet zero
      // tile entries, and shared memory still holds an earlier kernel's values
      // there (inf or NaN after a solve that met a zero diagonal: NaN * 0)
      if (tid < BS) xs[tid] = tid < cs ? __ldcg(&g.x[c0 + tid]) : 0.0;
      __syncthreads();
#pragma unroll
      for (int u = 0; u < CW; ++u) acc = fma(-xs[tc * CW + u], a[u], acc);
      __syncthreads();
    }
    part[tc][tr] = acc;
    __syncthreads();
    if (tid < bs) {
      double y = part[0][tid];
#pragma unroll
      for (int c = 1; c < NC; ++c) y += part[c][tid];
      xs[tid] = y;
    }
  } else {
    const int tcol = tid % BS, trp = tid / BS;  // rows r0 + trp * CW + u of the tile, column c0 + tcol
    double acc[CW];
#pragma unroll
    for (int u = 0; u < CW; ++u) acc[u] = 0.0;
    for (int q = 0; q < t; ++q) {
      const int jb = fwd ? q : nblk - 1 - q;
      const int c0 = jb * BS, cs = min(BS, n - c0);
      double a[CW];
#pragma unroll
      for (int u = 0; u < CW; ++u) {
        const int row = trp * CW + u;
        a[u] = (row < bs && tcol < cs) ? A[(size_t)(r0 + row) * lda + c0 + tcol] : 0.0;
      }
      if (tid == 0) {
        int polls = 0;
        while (trsvl_ld_acquire(&g.sync[2 + jb]) == 0) {
          if (++polls > g.poll_limit) {
            s_abort = 1;
            atomicExch(&g.sync[1], 1);
            atomicMin(g.info, kTrsvLInfoTimeout);
            break;
          }
          __nanosleep(64);
        }
      }
      __syncthreads();
      if (s_abort) return;
      // the whole of xs: a short last block leaves entries past cs that meet zero
      // tile entries, and shared memory still holds an earlier kernel's values
      // there (inf or NaN after a solve that met a zero diagonal: NaN * 0)
      if (tid < BS) xs[tid] = tid < cs ? __ldcg(&g.x[c0 + tid]) : 0.0;
      __syncthreads();
      const double xv = xs[tcol];
#pragma unroll
      for (int u = 0; u < CW; ++u) acc[u] = fma(-a[u], xv, acc[u]);
      __syncthreads();
    }
    // reduce the CW sums of each thread over the tile's BS columns: within
    // each warp a butterfly reduce-scatter leaves the sum of row k = lane % CW
    // in the lanes congruent to k; the BS / 32 warps of a row part meet in part[]
    constexpr int WP = BS / 32;
    const int lane = tid & 31, half = (tid >> 5) % WP;
#pragma unroll
    for (int h = CW / 2; h >= 1; h >>= 1) {
      const bool up = (lane & h) != 0;
#pragma unroll
      for (int u = 0; u < h; ++u) {
        const double keep = up ? acc[u + h] : acc[u];
        const double give = up ? acc[u] : acc[u + h];
        acc[u] = keep + __shfl_xor_sync(0xffffffffu, give, h);
      }
    }
#pragma unroll
    for (int off = CW; off < 32; off <<= 1) acc[0] += __shfl_xor_sync(0xffffffffu, acc[0], off);
    if (lane < CW) part[half][trp * CW + lane] = acc[0];
    __syncthreads();
    if (tid < bs) {
      double y = part[0][tid];
#pragma unroll
      for (int h = 1; h < WP; ++h) y += part[h][tid];
      xs[tid] = g.x[r0 + tid] + y;
    }
  }
  __syncthreads();
  // the diagonal block, 32 rows at a time: warp 0 solves the 32 x 32 piece
  // with shuffles, then all threads apply it to the block's remaining rows
  const int warp = tid >> 5, lane = tid & 31;
  const int nsub = (bs + 31) / 32;
  for (int q = 0; q < nsub; ++q) {
    const int sb = fwd ? q * 32 : (nsub - 1 - q) * 32;
    const int sw = min(32, bs - sb);
    if (warp == 0) {
      double v = lane < sw ? xs[sb + lane] : 0.0;
      if (fwd) {
#pragma unroll
        for (int kk = 0; kk < 32; ++kk) {
          if (kk < sw) {
            const double xk = __shfl_sync(0xffffffffu, v, kk);
            if (lane > kk && lane < sw) v = fma(-Ts[(sb + kk) * LD + sb + lane], xk, v);
          }
        }
      } else {
#pragma unroll
        for (int kk = 31; kk >= 0; --kk) {
          if (kk < sw) {
            const double xk = __shfl_sync(0xffffffffu, v, kk);
            if (lane < kk) v = fma(-Ts[(sb + kk) * LD + sb + lane], xk, v);
          }
        }
      }
      if (lane < sw) xs[sb + lane] = v;  // unscaled
    }
    __syncthreads();
    // the block's rows on the far side of the piece (at most 32) take its
    // contribution: warp w sums terms 4w..4w+3 for row i0 + lane, then one
    // thread per row adds the 8 partial sums (8 dependent FP64 steps on the
    // chain instead of 32)
    const int i0 = fwd ? sb + sw : 0, i1 = fwd ? bs : sb;
    if (i1 > i0) {
      double* pp = &part[0][0];  // 8 warps x 32 rows (the tile sums are consumed)
      double acc = 0.0;
      if (i0 + lane < i1)
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int k = 4 * warp + u;
          if (k < sw) acc = fma(-Ts[(sb + k) * LD + i0 + lane], xs[sb + k], acc);
        }
      pp[warp * 32 + lane] = acc;
      __syncthreads();
      if (tid < i1 - i0) {
        double y = xs[i0 + tid];
#pragma unroll
        for (int w = 0; w < kTrsvLThreads / 32; ++w) y += pp[w * 32 + tid];
        xs[i0 + tid] = y;
      }
    }
    __syncthreads();
  }
  if (tid < bs) g.x[r0 + tid] = xs[tid] * rd[tid];
  // the barrier orders the block's stores before thread 0's release, which is
  // cumulative over them: a CTA that acquires the flag sees x (no fence needed)
  __syncthreads();
  if (tid == 0) trsvl_st_release(&g.sync[2 + kb], 1);
}

__global__ void trsv_large_set_info_kernel(int32_t* info, int v) { *info = v; }

// with_diag's last pass: x <- diag * x.
__global__ void trsv_large_scale_kernel(int n, double* x, double d) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) x[i] *= d;
}

// info: the zero diagonal that stops nalgebra's solve, in its solve order
// (forward: the first; backward: the last), 1-based; 0 when none.
__global__ void __launch_bounds__(256) trsv_large_info_kernel(int n, const double* __restrict__ A, int64_t lda,
                                                             int fwd, int32_t* info) {
  __shared__ int best;
  if (threadIdx.x == 0) best = fwd ? 0x7fffffff : -1;
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x)
    if (A[(size_t)i * lda + i] == 0.0) {
      if (fwd) atomicMin(&best, i);
      else atomicMax(&best, i);
    }
  __syncthreads();
  if (threadIdx.x == 0) *info = (best == 0x7fffffff || best < 0) ? 0 : best + 1;
}

}  // namespace
}  // namespace nacu

extern "C" size_t nacu_trsv_workspace_bytes(int n) {
  const int nb = n > 0 ? (n + nacu::kTrsvLBS - 1) / nacu::kTrsvLBS : 0;
  return (size_t)(nb + 2) * sizeof(int);
}

namespace nacu {
namespace {
int trsv_large_run(int n, int nrhs, int upper, int trans, int has_diag, double diag, const double* T, int64_t lda,
                   double* B, int64_t ldb, int32_t* info, void* workspace, int poll_limit, cudaStream_t s) {
  const char* name = "nacu_dtrsv";
  const int fwd = (upper == 0) != (trans != 0);
  const size_t smem = (size_t)kTrsvLBS * kTrsvLLD * sizeof(double);
  auto kern = trans ? trsv_large_kernel<true> : trsv_large_kernel<false>;
  cudaError_t e = ensure_dynamic_smem(kern, smem);
  if (e != cudaSuccess) return record_cuda_error(e, name);
  if (has_diag) {
    e = cudaMemsetAsync(info, 0, sizeof(int32_t), s);  // with_diag never reads T's diagonal
    if (e != cudaSuccess) return record_cuda_error(e, name);
  } else {
    trsv_large_info_kernel<<<1, 256, 0, s>>>(n, T, lda, fwd, info);
  }
  const int nblk = (n + kTrsvLBS - 1) / kTrsvLBS;
  int* sync = static_cast<int*>(workspace);
  for (int c = 0; c < nrhs; ++c) {
    double* x = B + (size_t)c * ldb;
    e = cudaMemsetAsync(sync, 0, (size_t)(nblk + 2) * sizeof(int), s);
    if (e != cudaSuccess) return record_cuda_error(e, name);
    TrsvLArgs a{n, T, lda, x, fwd, has_diag ? 1 : 0, diag, info, sync, poll_limit};
    kern<<<nblk, kTrsvLThreads, smem, s>>>(a);
    if (has_diag) trsv_large_scale_kernel<<<(n + 255) / 256, 256, 0, s>>>(n, x, diag);
  }
  return check_launch(name);
}
}  // namespace
}  // namespace nacu

extern "C" int nacu_dtrsv(int n, int nrhs, int upper, int trans, int has_diag, double diag, const double* T,
                          int64_t lda, double* B, int64_t ldb, int32_t* info, void* workspace,
                          size_t workspace_bytes, int flags, nacu_stream_t stream) {
  using namespace nacu;
  if (n < 0) return record_arg_error(-1, "dtrsv: n < 0");
  if (nrhs < 0) return record_arg_error(-2, "dtrsv: nrhs < 0");
  if (has_diag && (upper || trans)) return record_arg_error(-5, "dtrsv: has_diag is the lower, trans = 0 form");
  if (n == 0 || nrhs == 0) return NACU_SUCCESS;
  if (!T) return record_arg_error(-7, "dtrsv: null T");
  if (lda < n) return record_arg_error(-8, "dtrsv: lda < n");
  if (!B) return record_arg_error(-9, "dtrsv: null B");
  if (ldb < n) return record_arg_error(-10, "dtrsv: ldb < n");
  if (!info) return record_arg_error(-11, "dtrsv: null info");
  if (!workspace || workspace_bytes < nacu_trsv_workspace_bytes(n))
    return record_arg_error(-12, "dtrsv: workspace too small");
  if (flags & NACU_FLAG_EXACT) return record_arg_error(-14, "dtrsv: NACU_FLAG_EXACT is the batched form's (n <= 128)");
  if (has_diag && diag == 0.0) {  // solve.rs:115-117: false, inputs untouched
    trsv_large_set_info_kernel<<<1, 1, 0, (cudaStream_t)stream>>>(info, 1);
    return check_launch("nacu_dtrsv");
  }
  return trsv_large_run(n, nrhs, upper, trans, has_diag, diag, T, lda, B, ldb, info, workspace, kTrsvLPollLimit,
                        (cudaStream_t)stream);
}
