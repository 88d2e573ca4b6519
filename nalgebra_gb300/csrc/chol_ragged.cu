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
  int do_factor;  // 0: A already holds the factor (solve only)
};

template <bool EXACT>
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
  double* a = g.A + (g.aoff ? g.aoff[s] : 0);
  if (tid == 0) *s_info = 0;
  __syncthreads();
  const int ldp = g.n_max | 1;
  double* rdiag = X + (size_t)ldp * kRhsChunk;
  if (g.do_factor) {
    chol_factor_cta<EXACT, double>(n, a, ldp, P, rdiag, s_info, s_scal, g.has_subst, g.subst);
  } else if (!EXACT) {
    for (int i = tid; i < n; i += blockDim.x) rdiag[i] = 1.0 / a[(size_t)i * n + i];
    __syncthreads();
  }
  const int inf = *s_info;
  if (inf == 0) {
    if (g.nrhs > 0 && g.B) {
      double* b = g.B + (g.boff ? g.boff[s] : 0);
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

template <bool EXACT>
__global__ void __launch_bounds__(kCholThreads, 4) chol_ragged_kernel(CholArgs g) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_item;
  __shared__ int s_info;
  __shared__ double s_scal[2 + kCholThreads / 32];
  const int ldp = g.n_max | 1;
  double* P = reinterpret_cast<double*>(smem_raw);
  double* X = P + (size_t)ldp * kNB;
  for (;;) {
    if (threadIdx.x == 0) s_item = g.counter ? atomicAdd(g.counter, 1) : 0;
    __syncthreads();
    const int idx = s_item;
    __syncthreads();
    if (idx >= g.count) break;
    const int s = g.order ? g.order[idx] : idx;
    chol_solve_one<EXACT>(g, s, P, X, &s_info, s_scal);
    if (!g.counter) break;  // single-matrix launch
  }
}

size_t chol_smem_bytes(int n_max) {
  const int ldp = n_max | 1;
  return (size_t)ldp * (kNB + kRhsChunk + 1) * sizeof(double);
}

int chol_launch(CholArgs g, int flags, cudaStream_t stream, bool persistent, const char* name) {
  const bool exact = (flags & NACU_FLAG_EXACT) != 0;
  auto kern = exact ? chol_ragged_kernel<true> : chol_ragged_kernel<false>;
  const size_t smem = chol_smem_bytes(g.n_max);
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return record_cuda_error(e, name);
  int grid = 1;
  if (persistent) {
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kCholThreads, smem);
    if (e != cudaSuccess) return record_cuda_error(e, name);
    if (per_sm < 1) per_sm = 1;
    grid = sm_count() * per_sm;
    if (grid > g.count) grid = g.count;
    e = cudaMemsetAsync(g.counter, 0, sizeof(int32_t), stream);
    if (e != cudaSuccess) return record_cuda_error(e, name);
  }
  kern<<<grid, kCholThreads, smem, stream>>>(g);
  return check_launch(name);
}

}  // namespace
}  // namespace nacu

extern "C" {

size_t nacu_ragged_workspace_bytes(int count) {
  (void)count;
  return 256;  // the work-queue head (one int32, padded)
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
             reinterpret_cast<int32_t*>(workspace), (flags & NACU_FLAG_SUBSTITUTE) ? 1 : 0, substitute, 1};
  return chol_launch(g, flags, (cudaStream_t)stream, true, "nacu_dposv_ragged");
}

int nacu_dpotrf_ragged(int count, int n_max, const int32_t* ns, const int64_t* a_offsets, double* A,
                       int32_t* info, double* logdet, const int32_t* order, void* workspace,
                       size_t workspace_bytes, double substitute, int flags, nacu_stream_t stream) {
  using namespace nacu;
  int rc = ragged_args(count, n_max, ns, a_offsets, A, workspace, workspace_bytes, "nacu_dpotrf_ragged");
  if (rc != 0) return rc > 0 ? NACU_SUCCESS : rc;
  if (!info) return record_arg_error(-6, "dpotrf_ragged: null info");
  CholArgs g{count, n_max, ns, a_offsets, A, 0, nullptr, nullptr, info, logdet, order,
             reinterpret_cast<int32_t*>(workspace), (flags & NACU_FLAG_SUBSTITUTE) ? 1 : 0, substitute, 1};
  return chol_launch(g, flags, (cudaStream_t)stream, true, "nacu_dpotrf_ragged");
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
             reinterpret_cast<int32_t*>(workspace), 0, 0.0, 0};
  return chol_launch(g, flags, (cudaStream_t)stream, true, "nacu_dpotrs_ragged");
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
             (flags & NACU_FLAG_SUBSTITUTE) ? 1 : 0, substitute, 1};
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

int32_t* g_noalloc_scratch_ptr[64] = {nullptr};

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
  if (g_noalloc_scratch_ptr[dev] == nullptr) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_ragged_noalloc_scratch);
    if (e != cudaSuccess) return record_cuda_error(e, "nacu_dposv_ragged_noalloc: cudaGetSymbolAddress");
    g_noalloc_scratch_ptr[dev] = static_cast<int32_t*>(p);
  }
  *out = g_noalloc_scratch_ptr[dev];
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
             (flags & NACU_FLAG_SUBSTITUTE) ? 1 : 0, substitute, 1};
  // The queue head was cleared by the order kernel (same stream, in order).
  const bool exact = (flags & NACU_FLAG_EXACT) != 0;
  auto kern = exact ? chol_ragged_kernel<true> : chol_ragged_kernel<false>;
  const size_t smem = chol_smem_bytes(g.n_max);
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return record_cuda_error(e, "nacu_dposv_ragged_noalloc");
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kCholThreads, smem);
  if (e != cudaSuccess) return record_cuda_error(e, "nacu_dposv_ragged_noalloc");
  if (per_sm < 1) per_sm = 1;
  int grid = sm_count() * per_sm;
  if (grid > count) grid = count;
  kern<<<grid, kCholThreads, smem, s>>>(g);
  return check_launch("nacu_dposv_ragged_noalloc");
}
