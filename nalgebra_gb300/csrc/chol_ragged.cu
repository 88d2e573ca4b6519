// Ragged batched Cholesky factor + solve + log-determinant: the GPU form of
// nalgebra's `m.cholesky()` then `.solve(&b)` and `.ln_determinant()` over
// thousands of SPD matrices of uneven order, in ONE persistent launch.
//
// Follows src/linalg/cholesky.rs:221-272 (Cholesky::new_internal, left-looking,
// lower triangle only, upper triangle left untouched), cholesky.rs:122-143
// (solve_mut: src/linalg/solve.rs:488-519 forward in axpy form, then
// solve.rs:697-712/732-755 adjoint back solve in dot form) and
// cholesky.rs:172-185 (ln_determinant = sum ln(L_ii^2)).
//
// Design (GB300): the FP64 pipe (~1 TFLOP/s) binds, HBM does not.  Each CTA
// factors one matrix at a time, pulling matrix indices from a device work queue
// ordered largest-first (so the short tail is made of small matrices).  The
// factorization is left-looking by NB-column panels: the panel lives in shared
// memory, the update by all earlier columns is a register-tiled product whose
// operands stream from L1/L2 (the matrix was just written by this CTA and is
// hot), and the panel itself is factored in shared memory with the trailing
// panel update spread evenly over all threads.  Every element still receives
// its updates in nalgebra's order (k = 0, 1, ..., j-1), so with EXACT the
// factor is bit-identical to nalgebra's.  The triangular solves are blocked by
// 32 rows: one warp solves each diagonal block out of registers with shuffles,
// the whole CTA applies the block to the remaining rows.
#include <atomic>
#include <algorithm>
#include <vector>

#include "chol_device.cuh"

namespace nacu {
namespace {

struct CholArgs {
  int count;
  int n_max;
  const int32_t* ns;
  const int64_t* aoff;
  double* A;
  int nrhs;
  const int64_t* boff;
  double* B;
  int32_t* info;
  double* logdet;
  const int32_t* order;
  int32_t* counter;
  int has_subst;
  double subst;
  int do_factor;         // 0: A already holds the factor (solve only)
  const int32_t* range;  // [start, end) of this launch within `order` (device), or null: [0, count)
  int64_t astride, bstride;  // equal-order batches without offset tables: system s at s * stride
};

template <bool EXACT, int NB>
__device__ void chol_solve_one(const CholArgs& g, int s, double* P, double* X, int* s_info, double* s_scal) {
  const int tid = threadIdx.x;
  const int n = g.ns ? g.ns[s] : g.n_max;
  if (n < 0 || n > g.n_max) {
    if (tid == 0) {
      if (g.info) g.info[s] = -1;
      if (g.logdet) g.logdet[s] = __longlong_as_double(0x7ff8000000000000ll);
    }
    return;
  }
  double* a = g.A + (g.aoff ? g.aoff[s] : (int64_t)s * g.astride);
  if (tid == 0) *s_info = 0;
  __syncthreads();
  const int ldp = g.n_max | 1;
  double* rdiag = X + (size_t)ldp * kRhsChunk;
  if (g.do_factor) {
    chol_factor_cta<EXACT, double, NB>(n, a, ldp, P, rdiag, s_info, s_scal, g.has_subst, g.subst);
  } else if (!EXACT) {
    for (int i = tid; i < n; i += blockDim.x) rdiag[i] = 1.0 / a[(size_t)i * n + i];
    __syncthreads();
  }
  const int inf = *s_info;
  if (inf == 0) {
    if (g.nrhs > 0 && g.B) {
      double* b = g.B + (g.boff ? g.boff[s] : (int64_t)s * g.bstride);
      const int ldx = ldp;
      for (int c0 = 0; c0 < g.nrhs; c0 += kRhsChunk) {
        const int nr = min(kRhsChunk, g.nrhs - c0);
        for (int e = tid; e < n * nr; e += blockDim.x) {
          const int c = e / n, r = e - c * n;
          X[(size_t)c * ldx + r] = b[(size_t)(c0 + c) * n + r];
        }
        __syncthreads();
        chol_forward_cta<EXACT, double>(n, a, X, ldx, nr, rdiag);
        if constexpr (EXACT) chol_backward_exact_cta(n, a, X, ldx, nr);
        else chol_backward_fast_cta<double>(n, a, X, ldx, nr, rdiag);
        for (int e = tid; e < n * nr; e += blockDim.x) {
          const int c = e / n, r = e - c * n;
          b[(size_t)(c0 + c) * n + r] = X[(size_t)c * ldx + r];
        }
        __syncthreads();
      }
    }
    if (g.logdet) {
      if constexpr (EXACT) {
        if (tid == 0) {
          double sum = 0.0;
          for (int i = 0; i < n; ++i) {
            const double d = a[(size_t)i * n + i];
            sum = __dadd_rn(sum, log(__dmul_rn(d, d)));
          }
          g.logdet[s] = sum;
        }
      } else {
        double part = 0.0;
        for (int i = tid; i < n; i += blockDim.x) {
          const double d = a[(size_t)i * n + i];
          part += log(d * d);
        }
        part = warp_sum(part);
        if ((tid & 31) == 0) s_scal[2 + (tid >> 5)] = part;
        __syncthreads();
        if (tid == 0) {
          double sum = 0.0;
          for (int w = 0; w < (int)(blockDim.x >> 5); ++w) sum += s_scal[2 + w];
          g.logdet[s] = sum;
        }
      }
    }
  } else if (tid == 0 && g.logdet) {
    g.logdet[s] = __longlong_as_double(0x7ff8000000000000ll);
  }
  if (tid == 0 && g.info) g.info[s] = inf;
  __syncthreads();
}

// One tile of the ragged kernel: THREADS threads per matrix, NB-column panels.
template <bool EXACT, int THREADS, int NB, int MINB>
__global__ void __launch_bounds__(THREADS, MINB) chol_ragged_kernel(CholArgs g) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_item;
  __shared__ int s_info;
  __shared__ double s_scal[2 + THREADS / 32];
  const int ldp = g.n_max | 1;
  double* P = reinterpret_cast<double*>(smem_raw);
  double* X = P + (size_t)ldp * NB;
  const int start = g.range ? g.range[0] : 0;
  const int end = g.range ? g.range[1] : g.count;
  for (;;) {
    if (threadIdx.x == 0) s_item = g.counter ? atomicAdd(g.counter, 1) : (int)blockIdx.x;  // no queue: one system per CTA
    __syncthreads();
    const int idx = start + s_item;
    __syncthreads();
    if (idx >= end) break;
    const int s = g.order ? g.order[idx] : idx;
    chol_solve_one<EXACT, NB>(g, s, P, X, &s_info, s_scal);
    if (!g.counter) break;  // single-matrix launch
  }
}

// The tiles the autotuner chooses from (threads per matrix, panel width).
struct CholTile {
  int threads, nb;
};
constexpr CholTile kCholTiles[NACU_RAGGED_TILES] = {{64, 8}, {128, 16}, {128, 32}, {256, 32}};
constexpr int kDefaultTile = 1;
// Upper order of each size bucket; bucket b holds (kBucketHi[b-1], kBucketHi[b]].
constexpr int kBucketHi[NACU_RAGGED_BUCKETS] = {32, 64, 96, 128, 192, 256, 384, 512};
__device__ __forceinline__ int bucket_hi_dev(int b) {
  constexpr int hi[NACU_RAGGED_BUCKETS] = {32, 64, 96, 128, 192, 256, 384, 512};
  return hi[b];
}
// Measured on GB300 by nacu_ragged_autotune (FP64 form, 4 right-hand sides,
// 2500 systems per bucket); replaced by nacu_ragged_set_tuning / autotune.
int g_tuning[NACU_RAGGED_BUCKETS] = {0, 0, 0, 0, 0, 1, 3, 3};

typedef void (*CholKernel)(CholArgs);
CholKernel chol_kernel(bool exact, int tile) {
  switch (tile) {
    case 0: return exact ? chol_ragged_kernel<true, 64, 8, 8> : chol_ragged_kernel<false, 64, 8, 8>;
    case 2: return exact ? chol_ragged_kernel<true, 128, 32, 4> : chol_ragged_kernel<false, 128, 32, 4>;
    case 3: return exact ? chol_ragged_kernel<true, 256, 32, 2> : chol_ragged_kernel<false, 256, 32, 2>;
    default: return exact ? chol_ragged_kernel<true, 128, 16, 4> : chol_ragged_kernel<false, 128, 16, 4>;
  }
}

size_t chol_smem_bytes(int n_max, int nb = kNB) {
  const int ldp = n_max | 1;
  return (size_t)ldp * (nb + kRhsChunk + 1) * sizeof(double);
}

// One launch of one tile over g.range (or the whole batch).
int chol_launch_tile(CholArgs g, int tile, bool exact, cudaStream_t stream, bool persistent, const char* name) {
  if (tile < 0 || tile >= NACU_RAGGED_TILES) tile = kDefaultTile;
  CholKernel kern = chol_kernel(exact, tile);
  const int threads = kCholTiles[tile].threads;
  const size_t smem = chol_smem_bytes(g.n_max, kCholTiles[tile].nb);
  cudaError_t e = ensure_dynamic_smem(kern, smem);
  if (e != cudaSuccess) return record_cuda_error(e, name);
  int grid = 1;
  if (persistent) {
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem);
    if (e != cudaSuccess) return record_cuda_error(e, name);
    if (per_sm < 1) per_sm = 1;
    grid = sm_count() * per_sm;
    if (grid > g.count) grid = g.count;
  }
  kern<<<grid, threads, smem, stream>>>(g);
  return check_launch(name);
}

int chol_launch(CholArgs g, int flags, cudaStream_t stream, bool persistent, const char* name) {
  if (persistent) {
    cudaError_t e = cudaMemsetAsync(g.counter, 0, sizeof(int32_t), stream);
    if (e != cudaSuccess) return record_cuda_error(e, name);
  }
  return chol_launch_tile(g, kDefaultTile, (flags & NACU_FLAG_EXACT) != 0, stream, persistent, name);
}

// ---- size-bucketed launches ------------------------------------------------
// Workspace: [0] per-bucket queue heads, [256] per-bucket [start, end) pairs,
// [512] histogram / scatter cursors over n = 0..512, then the order.
constexpr size_t kWsRanges = 256, kWsHist = 512;
constexpr size_t kWsOrder = kWsHist + (((size_t)(NACU_CHOL_RAGGED_MAX_N + 2) * 4 + 255) & ~(size_t)255);

__global__ void ragged_hist_kernel(int count, int n_max, const int32_t* __restrict__ ns, int32_t* hist) {
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < count; s += gridDim.x * blockDim.x) {
    int n = ns[s];
    n = (n < 0 || n > n_max) ? 0 : n;  // out-of-range orders land in bucket 0 (info = -1 there)
    atomicAdd(&hist[n], 1);
  }
}

// hist -> scatter cursors (largest n first) and the bucket ranges; clears the
// queue heads.
__global__ void ragged_scan_kernel(int count, int n_max, int32_t* hist, int32_t* ranges, int32_t* heads) {
  __shared__ int above[NACU_CHOL_RAGGED_MAX_N + 2];  // above[n] = items with order > n
  if (threadIdx.x == 0) {
    int run = 0;
    for (int n = n_max; n >= 0; --n) {
      above[n] = run;
      const int h = hist[n];
      hist[n] = run;
      run += h;
    }
    for (int b = 0; b < NACU_RAGGED_BUCKETS; ++b) {
      const int hi = bucket_hi_dev(b), lo = b ? bucket_hi_dev(b - 1) : -1;
      ranges[2 * b] = hi >= n_max ? 0 : above[hi];
      ranges[2 * b + 1] = lo < 0 ? count : (lo >= n_max ? 0 : above[lo]);
      heads[b] = 0;
    }
  }
}

__global__ void ragged_scatter_kernel(int count, int n_max, const int32_t* __restrict__ ns, int32_t* cursor,
                                      int32_t* order) {
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < count; s += gridDim.x * blockDim.x) {
    int n = ns[s];
    n = (n < 0 || n > n_max) ? 0 : n;
    order[atomicAdd(&cursor[n], 1)] = s;
  }
}

// Internal streams for the concurrent bucket launches (per device, created on
// first use): the bucket kernels fork from the caller's stream after the
// order is built and join back before the call returns, so the tail of one
// bucket overlaps the next one and a stream capture sees a fork/join graph.
struct ForkStreams {
  cudaStream_t st[NACU_RAGGED_BUCKETS] = {};
  cudaEvent_t fork = nullptr;
  cudaEvent_t join[NACU_RAGGED_BUCKETS] = {};
  bool ready = false;
};
ForkStreams g_fork[64];

int fork_streams(ForkStreams** out, const char* name) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return record_cuda_error(e, name);
  if (dev < 0 || dev >= 64) return record_arg_error(-99, "ragged Cholesky: device index >= 64");
  ForkStreams& f = g_fork[dev];
  if (!f.ready) {
    e = cudaEventCreateWithFlags(&f.fork, cudaEventDisableTiming);
    for (int b = 0; b < NACU_RAGGED_BUCKETS && e == cudaSuccess; ++b) {
      e = cudaStreamCreateWithFlags(&f.st[b], cudaStreamNonBlocking);
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&f.join[b], cudaEventDisableTiming);
    }
    if (e != cudaSuccess) return record_cuda_error(e, name);
    f.ready = true;
  }
  *out = &f;
  return NACU_SUCCESS;
}

// Builds the bucketed order in the workspace, then one persistent launch per
// bucket that can hold orders of this batch (largest bucket first), each with
// its tuned tile and shared memory sized for the bucket's largest order.
int chol_launch_bucketed(CholArgs g, int flags, cudaStream_t s, const char* name) {
  unsigned char* ws = reinterpret_cast<unsigned char*>(g.counter);
  int32_t* heads = reinterpret_cast<int32_t*>(ws);
  int32_t* ranges = reinterpret_cast<int32_t*>(ws + kWsRanges);
  int32_t* hist = reinterpret_cast<int32_t*>(ws + kWsHist);
  int32_t* order = reinterpret_cast<int32_t*>(ws + kWsOrder);
  cudaError_t e = cudaMemsetAsync(hist, 0, (size_t)(NACU_CHOL_RAGGED_MAX_N + 2) * 4, s);
  if (e != cudaSuccess) return record_cuda_error(e, name);
  const int blocks = std::min(sm_count() * 4, (g.count + 255) / 256);
  ragged_hist_kernel<<<blocks, 256, 0, s>>>(g.count, g.n_max, g.ns, hist);
  ragged_scan_kernel<<<1, 32, 0, s>>>(g.count, g.n_max, hist, ranges, heads);
  ragged_scatter_kernel<<<blocks, 256, 0, s>>>(g.count, g.n_max, g.ns, hist, order);
  int rc = check_launch(name);
  if (rc != NACU_SUCCESS) return rc;
  const bool exact = (flags & NACU_FLAG_EXACT) != 0;
  int active[NACU_RAGGED_BUCKETS], na = 0;
  for (int b = NACU_RAGGED_BUCKETS - 1; b >= 0; --b) {
    const int lo = b ? kBucketHi[b - 1] : -1;
    if (b > 0 && lo >= g.n_max) continue;  // no order of this batch falls in the bucket
    active[na++] = b;
  }
  ForkStreams* f = nullptr;
  if (na > 1) {
    rc = fork_streams(&f, name);
    if (rc != NACU_SUCCESS) return rc;
    e = cudaEventRecord(f->fork, s);
    if (e != cudaSuccess) return record_cuda_error(e, name);
  }
  for (int i = 0; i < na; ++i) {
    const int b = active[i];
    cudaStream_t sb = s;
    if (f) {
      sb = f->st[i];
      e = cudaStreamWaitEvent(sb, f->fork, 0);
      if (e != cudaSuccess) return record_cuda_error(e, name);
    }
    CholArgs gb = g;
    gb.n_max = std::min(g.n_max, kBucketHi[b]);
    gb.order = order;
    gb.counter = heads + b;
    gb.range = ranges + 2 * b;
    rc = chol_launch_tile(gb, g_tuning[b], exact, sb, true, name);
    if (rc != NACU_SUCCESS) return rc;
    if (f) {
      e = cudaEventRecord(f->join[i], sb);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(s, f->join[i], 0);
      if (e != cudaSuccess) return record_cuda_error(e, name);
    }
  }
  return NACU_SUCCESS;
}

// Either the caller's processing order (one launch, default tile) or the
// library's bucketed order with the tuned tiles.
int chol_launch_ragged(CholArgs g, int flags, cudaStream_t s, const char* name) {
  if (g.order) return chol_launch(g, flags, s, true, name);
  return chol_launch_bucketed(g, flags, s, name);
}

}  // namespace

size_t ragged_order_scratch_bytes() { return kWsOrder; }

int ragged_order_desc(int count, int n_max, const int32_t* ns, int32_t* order, void* scratch, cudaStream_t s,
                      const char* name) {
  if (count <= 0) return NACU_SUCCESS;
  unsigned char* ws = static_cast<unsigned char*>(scratch);
  int32_t* heads = reinterpret_cast<int32_t*>(ws);
  int32_t* ranges = reinterpret_cast<int32_t*>(ws + kWsRanges);
  int32_t* hist = reinterpret_cast<int32_t*>(ws + kWsHist);
  cudaError_t e = cudaMemsetAsync(hist, 0, (size_t)(NACU_CHOL_RAGGED_MAX_N + 2) * 4, s);
  if (e != cudaSuccess) return record_cuda_error(e, name);
  const int blocks = std::min(sm_count() * 4, (count + 255) / 256);
  ragged_hist_kernel<<<blocks, 256, 0, s>>>(count, n_max, ns, hist);
  ragged_scan_kernel<<<1, 32, 0, s>>>(count, n_max, hist, ranges, heads);
  ragged_scatter_kernel<<<blocks, 256, 0, s>>>(count, n_max, ns, hist, order);
  return check_launch(name);
}

// Equal-order batch (system s at A + s*strideA, B + s*strideB), one CTA per
// system, factor + solve + log-determinant in place with the tuned tile of
// the order's size bucket (used by the adjoint's forward pass).
int chol_uniform_posv(int n, double* A, int64_t strideA, int nrhs, double* B, int64_t strideB, int32_t* info,
                      double* logdet, int batch, cudaStream_t s, const char* name) {
  if (batch <= 0) return NACU_SUCCESS;
  int b = 0;
  while (b < NACU_RAGGED_BUCKETS - 1 && n > kBucketHi[b]) ++b;
  CholArgs g{batch, n, nullptr, nullptr, A, nrhs, nullptr, B, info, logdet, nullptr, nullptr, 0, 0.0, 1, nullptr,
             strideA, strideB};
  int tile = g_tuning[b];
  if (tile < 0 || tile >= NACU_RAGGED_TILES) tile = kDefaultTile;
  CholKernel kern = chol_kernel(false, tile);
  const size_t smem = chol_smem_bytes(n, kCholTiles[tile].nb);
  cudaError_t e = ensure_dynamic_smem(kern, smem);
  if (e != cudaSuccess) return record_cuda_error(e, name);
  kern<<<batch, kCholTiles[tile].threads, smem, s>>>(g);
  return check_launch(name);
}

namespace {

}  // namespace
}  // namespace nacu

extern "C" {

size_t nacu_ragged_workspace_bytes(int count) {
  // queue heads, bucket ranges, histogram, and the bucketed order
  return nacu::kWsOrder + (((size_t)(count > 0 ? count : 0) * 4 + 255) & ~(size_t)255);
}

static int ragged_args(int count, int n_max, const int32_t* ns, const int64_t* a_offsets, double* A,
                       void* workspace, size_t workspace_bytes, const char* name) {
  using namespace nacu;
  (void)name;
  if (count < 0) return record_arg_error(-1, "ragged Cholesky: negative count");
  if (n_max < 0 || n_max > NACU_CHOL_RAGGED_MAX_N)
    return record_arg_error(-2, "ragged Cholesky: n_max out of range [0, 512]");
  if (count == 0) return 1;
  if (!ns || !a_offsets || !A) return record_arg_error(-3, "ragged Cholesky: null ns, a_offsets or A");
  if (!workspace || workspace_bytes < nacu_ragged_workspace_bytes(count))
    return record_arg_error(-12, "ragged Cholesky: workspace too small");
  return 0;
}

int nacu_dposv_ragged(int count, int n_max, const int32_t* ns, const int64_t* a_offsets, double* A, int nrhs,
                      const int64_t* b_offsets, double* B, int32_t* info, double* logdet, const int32_t* order,
                      void* workspace, size_t workspace_bytes, double substitute, int flags,
                      nacu_stream_t stream) {
  using namespace nacu;
  int rc = ragged_args(count, n_max, ns, a_offsets, A, workspace, workspace_bytes, "nacu_dposv_ragged");
  if (rc != 0) return rc > 0 ? NACU_SUCCESS : rc;
  if (nrhs < 0) return record_arg_error(-6, "dposv_ragged: negative nrhs");
  if (nrhs > 0 && (!b_offsets || !B)) return record_arg_error(-7, "dposv_ragged: null b_offsets or B");
  if (!info) return record_arg_error(-9, "dposv_ragged: null info");
  CholArgs g{count, n_max, ns, a_offsets, A, nrhs, b_offsets, B, info, logdet, order,
             reinterpret_cast<int32_t*>(workspace), (flags & NACU_FLAG_SUBSTITUTE) ? 1 : 0, substitute, 1, nullptr};
  return chol_launch_ragged(g, flags, (cudaStream_t)stream, "nacu_dposv_ragged");
}

int nacu_dpotrf_ragged(int count, int n_max, const int32_t* ns, const int64_t* a_offsets, double* A,
                       int32_t* info, double* logdet, const int32_t* order, void* workspace,
                       size_t workspace_bytes, double substitute, int flags, nacu_stream_t stream) {
  using namespace nacu;
  int rc = ragged_args(count, n_max, ns, a_offsets, A, workspace, workspace_bytes, "nacu_dpotrf_ragged");
  if (rc != 0) return rc > 0 ? NACU_SUCCESS : rc;
  if (!info) return record_arg_error(-6, "dpotrf_ragged: null info");
  CholArgs g{count, n_max, ns, a_offsets, A, 0, nullptr, nullptr, info, logdet, order,
             reinterpret_cast<int32_t*>(workspace), (flags & NACU_FLAG_SUBSTITUTE) ? 1 : 0, substitute, 1, nullptr};
  return chol_launch_ragged(g, flags, (cudaStream_t)stream, "nacu_dpotrf_ragged");
}

int nacu_dpotrs_ragged(int count, int n_max, const int32_t* ns, const int64_t* a_offsets, const double* L,
                       int nrhs, const int64_t* b_offsets, double* B, const int32_t* order, void* workspace,
                       size_t workspace_bytes, int flags, nacu_stream_t stream) {
  using namespace nacu;
  int rc = ragged_args(count, n_max, ns, a_offsets, const_cast<double*>(L), workspace, workspace_bytes,
                       "nacu_dpotrs_ragged");
  if (rc != 0) return rc > 0 ? NACU_SUCCESS : rc;
  if (nrhs < 0) return record_arg_error(-6, "dpotrs_ragged: negative nrhs");
  if (nrhs == 0) return NACU_SUCCESS;
  if (!b_offsets || !B) return record_arg_error(-7, "dpotrs_ragged: null b_offsets or B");
  CholArgs g{count, n_max, ns, a_offsets, const_cast<double*>(L), nrhs, b_offsets, B, nullptr, nullptr, order,
             reinterpret_cast<int32_t*>(workspace), 0, 0.0, 0, nullptr};
  return chol_launch_ragged(g, flags, (cudaStream_t)stream, "nacu_dpotrs_ragged");
}

int nacu_dposv(int n, double* A, int nrhs, double* B, int32_t* info, double* logdet, double substitute,
               int flags, nacu_stream_t stream) {
  using namespace nacu;
  if (n < 0 || n > NACU_CHOL_RAGGED_MAX_N) return record_arg_error(-1, "dposv: n out of range [0, 512]");
  if (n == 0) return NACU_SUCCESS;
  if (!A) return record_arg_error(-2, "dposv: null A");
  if (nrhs < 0) return record_arg_error(-3, "dposv: negative nrhs");
  if (nrhs > 0 && !B) return record_arg_error(-4, "dposv: null B");
  if (!info) return record_arg_error(-5, "dposv: null info");
  // One matrix, one CTA: the plain per-matrix launch (no work queue).
  CholArgs g{1, n, nullptr, nullptr, A, nrhs, nullptr, B, info, logdet, nullptr, nullptr,
             (flags & NACU_FLAG_SUBSTITUTE) ? 1 : 0, substitute, 1, nullptr};
  return chol_launch(g, flags, (cudaStream_t)stream, false, "nacu_dposv");
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Allocation-free variant of nacu_dposv_ragged.
//
// Some callers cannot allocate device memory at the point where they solve:
// code running inside a custom allocator or memory-pool callback, real-time or
// safety-certified hosts that forbid allocation after start-up, and plugins
// whose host framework owns every device allocation and hands out no scratch.
// For them this entry point keeps its scratch -- the work-queue head and the
// largest-first processing order -- in a fixed array in the library's own
// device memory (loaded with the module; every GPU that loads the library
// holds it until the process exits).  The caller still passes all inputs and
// outputs.  Calls share that one array, so two calls that overlap on the GPU
// (different streams, no ordering between them) race on it; order such calls.
// ---------------------------------------------------------------------------
namespace nacu {
namespace {

constexpr int kNoAllocMaxCount = NACU_RAGGED_NOALLOC_MAX_COUNT;

// [0]: work-queue head; [1 .. count]: processing order.
static __device__ __align__(256) int32_t g_ragged_noalloc_scratch[1 + kNoAllocMaxCount];

// Per-device cache of the array's device address.  Atomic: two host threads
// making a first call at once both look it up and store the same value.
std::atomic<int32_t*> g_noalloc_scratch_ptr[64] = {};

// Builds the largest-first order (a counting sort on n, one CTA) into the
// scratch and clears the queue head, so every call starts from zero.
__global__ void __launch_bounds__(1024) ragged_order_kernel(int count, int n_max, const int32_t* __restrict__ ns,
                                                            int32_t* __restrict__ scratch) {
  __shared__ int hist[NACU_CHOL_RAGGED_MAX_N + 2];
  const int nb = n_max + 1;
  for (int i = threadIdx.x; i <= nb; i += blockDim.x) hist[i] = 0;
  __syncthreads();
  for (int s = threadIdx.x; s < count; s += blockDim.x) {
    int n = ns[s];
    n = (n < 0 || n > n_max) ? 0 : n;  // out-of-range orders still get a slot (info = -1 later)
    atomicAdd(&hist[n], 1);
  }
  __syncthreads();
  if (threadIdx.x == 0) {  // exclusive prefix sum over n, largest n first
    int run = 0;
    for (int n = n_max; n >= 0; --n) {
      const int h = hist[n];
      hist[n] = run;
      run += h;
    }
    scratch[0] = 0;
  }
  __syncthreads();
  for (int s = threadIdx.x; s < count; s += blockDim.x) {
    int n = ns[s];
    n = (n < 0 || n > n_max) ? 0 : n;
    scratch[1 + atomicAdd(&hist[n], 1)] = s;
  }
}

// Device address of the scratch array for the current device, looked up once
// per device (the array's host-side name is not a device address).
int noalloc_scratch(int32_t** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return record_cuda_error(e, "nacu_dposv_ragged_noalloc: cudaGetDevice");
  if (dev < 0 || dev >= 64) return record_arg_error(-99, "nacu_dposv_ragged_noalloc: device index >= 64");
  int32_t* cached = g_noalloc_scratch_ptr[dev].load(std::memory_order_acquire);
  if (cached == nullptr) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_ragged_noalloc_scratch);
    if (e != cudaSuccess) return record_cuda_error(e, "nacu_dposv_ragged_noalloc: cudaGetSymbolAddress");
    cached = static_cast<int32_t*>(p);
    g_noalloc_scratch_ptr[dev].store(cached, std::memory_order_release);
  }
  *out = cached;
  return NACU_SUCCESS;
}

}  // namespace
}  // namespace nacu

extern "C" int nacu_dposv_ragged_noalloc(int count, int n_max, const int32_t* ns, const int64_t* a_offsets,
                                         double* A, int nrhs, const int64_t* b_offsets, double* B, int32_t* info,
                                         double* logdet, double substitute, int flags, nacu_stream_t stream) {
  using namespace nacu;
  if (count < 0) return record_arg_error(-1, "dposv_ragged_noalloc: negative count");
  if (count > kNoAllocMaxCount)
    return record_arg_error(-1, "dposv_ragged_noalloc: count exceeds NACU_RAGGED_NOALLOC_MAX_COUNT (65536); "
                                "use nacu_dposv_ragged with a caller workspace or split the batch");
  if (n_max < 0 || n_max > NACU_CHOL_RAGGED_MAX_N)
    return record_arg_error(-2, "dposv_ragged_noalloc: n_max out of range [0, 512]");
  if (count == 0) return NACU_SUCCESS;
  if (!ns || !a_offsets || !A) return record_arg_error(-3, "dposv_ragged_noalloc: null ns, a_offsets or A");
  if (nrhs < 0) return record_arg_error(-6, "dposv_ragged_noalloc: negative nrhs");
  if (nrhs > 0 && (!b_offsets || !B)) return record_arg_error(-7, "dposv_ragged_noalloc: null b_offsets or B");
  if (!info) return record_arg_error(-9, "dposv_ragged_noalloc: null info");
  int32_t* scratch = nullptr;
  int rc = noalloc_scratch(&scratch);
  if (rc != NACU_SUCCESS) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  ragged_order_kernel<<<1, 1024, 0, s>>>(count, n_max, ns, scratch);
  rc = check_launch("nacu_dposv_ragged_noalloc: order");
  if (rc != NACU_SUCCESS) return rc;
  CholArgs g{count, n_max, ns, a_offsets, A, nrhs, b_offsets, B, info, logdet, scratch + 1, scratch,
             (flags & NACU_FLAG_SUBSTITUTE) ? 1 : 0, substitute, 1, nullptr};
  // The queue head was cleared by the order kernel (same stream, in order).
  return chol_launch_tile(g, kDefaultTile, (flags & NACU_FLAG_EXACT) != 0, s, true, "nacu_dposv_ragged_noalloc");
}

// ---------------------------------------------------------------------------
// Autotuner of the bucketed launch: per size bucket, every tile is timed on a
// synthetic batch of that bucket (CUDA events, best of three after a warm-up)
// and the fastest becomes the bucket's tile.
// ---------------------------------------------------------------------------
namespace nacu {
namespace {

__device__ __forceinline__ uint32_t mix32(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7feb352du;
  x ^= x >> 15;
  x *= 0x846ca68bu;
  x ^= x >> 16;
  return x;
}

// Diagonally dominant SPD matrices: symmetric off-diagonal entries in
// [-0.5, 0.5) hashed from (system, i, j), diagonal n + 1; right-hand sides 1.
__global__ void tune_fill_kernel(const int32_t* __restrict__ ns, const int64_t* __restrict__ aoff, double* A,
                                 int nrhs, const int64_t* __restrict__ boff, double* B) {
  const int s = blockIdx.x;
  const int n = ns[s];
  double* a = A + aoff[s];
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
    const int j = e / n, i = e - j * n;
    const int lo = min(i, j), hi = max(i, j);
    const uint32_t h = mix32((uint32_t)s * 0x9e3779b9u ^ mix32((uint32_t)lo * 1024u + (uint32_t)hi));
    a[e] = (i == j) ? (double)(n + 1) : ((double)(h >> 8) * (1.0 / 16777216.0) - 0.5);
  }
  double* b = B + boff[s];
  for (int e = threadIdx.x; e < n * nrhs; e += blockDim.x) b[e] = 1.0;
}

struct TuneBuffers {
  int32_t* ns = nullptr;
  int64_t* aoff = nullptr;
  int64_t* boff = nullptr;
  double* A = nullptr;
  double* B = nullptr;
  int32_t* info = nullptr;
  int32_t* head = nullptr;
  ~TuneBuffers() {
    cudaFree(ns);
    cudaFree(aoff);
    cudaFree(boff);
    cudaFree(A);
    cudaFree(B);
    cudaFree(info);
    cudaFree(head);
  }
};

}  // namespace
}  // namespace nacu

extern "C" {

int nacu_ragged_tuning_layout(int32_t* bucket_hi, int32_t* tile_threads, int32_t* tile_nb) {
  for (int b = 0; b < NACU_RAGGED_BUCKETS; ++b)
    if (bucket_hi) bucket_hi[b] = nacu::kBucketHi[b];
  for (int t = 0; t < NACU_RAGGED_TILES; ++t) {
    if (tile_threads) tile_threads[t] = nacu::kCholTiles[t].threads;
    if (tile_nb) tile_nb[t] = nacu::kCholTiles[t].nb;
  }
  return NACU_SUCCESS;
}

int nacu_ragged_set_tuning(const int32_t* table, int nbuckets) {
  using namespace nacu;
  if (!table || nbuckets != NACU_RAGGED_BUCKETS)
    return record_arg_error(-1, "ragged_set_tuning: need NACU_RAGGED_BUCKETS entries");
  for (int b = 0; b < NACU_RAGGED_BUCKETS; ++b)
    if (table[b] < 0 || table[b] >= NACU_RAGGED_TILES)
      return record_arg_error(-1, "ragged_set_tuning: tile index out of range");
  for (int b = 0; b < NACU_RAGGED_BUCKETS; ++b) g_tuning[b] = table[b];
  return NACU_SUCCESS;
}

int nacu_ragged_get_tuning(int32_t* table, int nbuckets) {
  using namespace nacu;
  if (!table || nbuckets != NACU_RAGGED_BUCKETS)
    return record_arg_error(-1, "ragged_get_tuning: need NACU_RAGGED_BUCKETS entries");
  for (int b = 0; b < NACU_RAGGED_BUCKETS; ++b) table[b] = g_tuning[b];
  return NACU_SUCCESS;
}

int nacu_ragged_autotune(int per_bucket, int nrhs, int flags, int32_t* table_out, double* ms_out,
                         nacu_stream_t stream) {
  using namespace nacu;
  if (per_bucket < 1 || per_bucket > 1000000) return record_arg_error(-1, "ragged_autotune: per_bucket out of range");
  if (nrhs < 0 || nrhs > 64) return record_arg_error(-2, "ragged_autotune: nrhs out of range [0, 64]");
  cudaStream_t s = (cudaStream_t)stream;
  const bool exact = (flags & NACU_FLAG_EXACT) != 0;
  int32_t table[NACU_RAGGED_BUCKETS];
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  if (e != cudaSuccess) return record_cuda_error(e, "nacu_ragged_autotune");
  int rc = NACU_SUCCESS;
  for (int b = 0; b < NACU_RAGGED_BUCKETS && rc == NACU_SUCCESS; ++b) {
    const int hi = kBucketHi[b], lo = b ? kBucketHi[b - 1] : 0;
    std::vector<int32_t> ns(per_bucket);
    std::vector<int64_t> aoff(per_bucket), boff(per_bucket);
    uint32_t st = 12345u + 977u * (uint32_t)b;
    int64_t ta = 0, tb = 0;
    for (int i = 0; i < per_bucket; ++i) {
      st = st * 1664525u + 1013904223u;
      ns[i] = lo + 1 + (int)((st >> 8) % (uint32_t)(hi - lo));
      aoff[i] = ta;
      boff[i] = tb;
      ta += (int64_t)ns[i] * ns[i];
      tb += (int64_t)ns[i] * nrhs;
    }
    TuneBuffers buf;
    e = cudaMalloc(&buf.ns, per_bucket * sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMalloc(&buf.aoff, per_bucket * sizeof(int64_t));
    if (e == cudaSuccess) e = cudaMalloc(&buf.boff, per_bucket * sizeof(int64_t));
    if (e == cudaSuccess) e = cudaMalloc(&buf.A, (size_t)ta * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&buf.B, (size_t)std::max<int64_t>(tb, 1) * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&buf.info, per_bucket * sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMalloc(&buf.head, 256);
    if (e == cudaSuccess) e = cudaMemcpyAsync(buf.ns, ns.data(), per_bucket * 4, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(buf.aoff, aoff.data(), per_bucket * 8, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(buf.boff, boff.data(), per_bucket * 8, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) {
      rc = record_cuda_error(e, "nacu_ragged_autotune");
      break;
    }
    double best = 1e300;
    table[b] = kDefaultTile;
    for (int t = 0; t < NACU_RAGGED_TILES && rc == NACU_SUCCESS; ++t) {
      float tbest = 1e30f;
      for (int rep = 0; rep < 4 && rc == NACU_SUCCESS; ++rep) {
        tune_fill_kernel<<<per_bucket, 256, 0, s>>>(buf.ns, buf.aoff, buf.A, nrhs, buf.boff, buf.B);
        e = cudaMemsetAsync(buf.head, 0, 4, s);
        if (e != cudaSuccess) {
          rc = record_cuda_error(e, "nacu_ragged_autotune");
          break;
        }
        CholArgs g{per_bucket, hi, buf.ns, buf.aoff, buf.A, nrhs, buf.boff, buf.B, buf.info, nullptr, nullptr,
                   buf.head, 0, 0.0, 1, nullptr};
        cudaEventRecord(e0, s);
        rc = chol_launch_tile(g, t, exact, s, true, "nacu_ragged_autotune");
        cudaEventRecord(e1, s);
        e = cudaEventSynchronize(e1);
        if (e != cudaSuccess) rc = record_cuda_error(e, "nacu_ragged_autotune");
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms < tbest) tbest = ms;
      }
      if (rc != NACU_SUCCESS) break;
      // every system must have factored (the inputs are SPD)
      std::vector<int32_t> info(per_bucket);
      e = cudaMemcpy(info.data(), buf.info, per_bucket * 4, cudaMemcpyDeviceToHost);
      if (e != cudaSuccess) {
        rc = record_cuda_error(e, "nacu_ragged_autotune");
        break;
      }
      for (int i = 0; i < per_bucket; ++i)
        if (info[i] != 0) {
          rc = record_arg_error(-100, "ragged_autotune: a tile failed to factor an SPD test matrix");
          break;
        }
      if (ms_out) ms_out[b * NACU_RAGGED_TILES + t] = tbest;
      if (tbest < best) {
        best = tbest;
        table[b] = t;
      }
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc != NACU_SUCCESS) return rc;
  for (int b = 0; b < NACU_RAGGED_BUCKETS; ++b) {
    g_tuning[b] = table[b];
    if (table_out) table_out[b] = table[b];
  }
  return NACU_SUCCESS;
}

}  // extern "C"
