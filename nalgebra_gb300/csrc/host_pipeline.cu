// Ragged mixed-precision SPD solve from host memory, pipelined: the batch is
// cut into chunks of about equal bytes; while chunk k is solved on the GPU,
// chunk k+1's matrices and right-hand sides are copied in and chunk k-1's
// solutions copied out, on three internal streams (copy-in, solve, copy-out)
// through a two-stage staging ring in the caller's device workspace.  It is
// the form a host-resident caller (nalgebra's own users: matrices in host
// memory) calls in place of `m.cholesky()` + `.solve(&b)` per matrix
// (src/linalg/cholesky.rs:221-272, 122-143): the same packed ragged layout as
// nacu_dposv_ragged_mixed, but every array is a host array.
//
// Each chunk runs the unchanged device path (nacu_dposv_ragged_mixed) on its
// systems in largest-first order, so every system's result is bit-identical
// to a single device call over the whole batch.
#include <algorithm>
#include <cstring>

#include "common.cuh"

namespace nacu {
namespace {

constexpr int kMaxChunks = 64;

struct ChunkPlan {
  int nchunks;
  int s0[kMaxChunks + 1];                    // chunk c: systems s0[c] .. s0[c+1]-1
  int64_t a_lo[kMaxChunks], a_hi[kMaxChunks];  // element spans of A and of B / X
  int64_t b_lo[kMaxChunks], b_hi[kMaxChunks];
  int max_count;
  int64_t max_a, max_b;
};

// Chunks of about equal A bytes.  Offsets must be non-decreasing (each chunk
// then is one contiguous span of A and of B).  Returns 0 or a negative code.
int plan_chunks(int count, int n_max, const int32_t* ns, const int64_t* aoff, const int64_t* boff, int nrhs,
                int chunks, ChunkPlan* p) {
  if (chunks < 1) chunks = 8;
  if (chunks > kMaxChunks) chunks = kMaxChunks;
  if (chunks > count) chunks = count;
  int64_t total = 0;
  for (int s = 0; s < count; ++s) {
    const int n = ns[s];
    if (n < 0 || n > n_max) return -2;
    if (s > 0 && (aoff[s] < aoff[s - 1] || boff[s] < boff[s - 1])) return -4;
    if (aoff[s] < 0 || boff[s] < 0) return -4;
    total += (int64_t)n * n;
  }
  p->nchunks = 0;
  p->max_count = 0;
  p->max_a = p->max_b = 0;
  int64_t acc = 0;
  int start = 0;
  for (int s = 0; s < count; ++s) {
    acc += (int64_t)ns[s] * ns[s];
    const int c = p->nchunks;
    const bool last = (s == count - 1);
    // cut when the running total passes the next equal share (or at the end)
    if (last || (c < chunks - 1 && acc * chunks >= total * (int64_t)(c + 1))) {
      p->s0[c] = start;
      int64_t alo = aoff[start], ahi = alo, blo = boff[start], bhi = blo;
      for (int q = start; q <= s; ++q) {
        ahi = std::max(ahi, aoff[q] + (int64_t)ns[q] * ns[q]);
        bhi = std::max(bhi, boff[q] + (int64_t)ns[q] * nrhs);
      }
      p->a_lo[c] = alo;
      p->a_hi[c] = ahi;
      p->b_lo[c] = blo;
      p->b_hi[c] = bhi;
      p->max_count = std::max(p->max_count, s + 1 - start);
      p->max_a = std::max(p->max_a, ahi - alo);
      p->max_b = std::max(p->max_b, bhi - blo);
      p->nchunks = c + 1;
      start = s + 1;
    }
  }
  p->s0[p->nchunks] = count;
  return 0;
}

size_t up256(size_t x) { return (x + 255) & ~(size_t)255; }

struct HostLayout {
  size_t ns, order, info, iters, aoff, boff, sort, stage_a[2], stage_b[2], stage_x[2], solver, total;
};

HostLayout host_layout(int count, const ChunkPlan& p) {
  HostLayout L;
  size_t o = 0;
  L.ns = o; o = up256(o + (size_t)count * 4);
  L.order = o; o = up256(o + (size_t)count * 4);
  L.info = o; o = up256(o + (size_t)count * 4);
  L.iters = o; o = up256(o + (size_t)count * 4);
  L.aoff = o; o = up256(o + (size_t)count * 8);
  L.boff = o; o = up256(o + (size_t)count * 8);
  L.sort = o; o = up256(o + ragged_order_scratch_bytes());
  for (int st = 0; st < 2; ++st) {
    L.stage_a[st] = o; o = up256(o + (size_t)p.max_a * 8);
    L.stage_b[st] = o; o = up256(o + (size_t)p.max_b * 8);
    L.stage_x[st] = o; o = up256(o + (size_t)p.max_b * 8);
  }
  L.solver = o; o = up256(o + nacu_mixed_workspace_bytes(p.max_count, p.max_a));
  L.total = o;
  return L;
}

// Offsets relative to their chunk's first element: a chunk's arrays start at
// its staging buffers.
struct RebaseArgs {
  int nchunks;
  int s0[kMaxChunks + 1];
  int64_t a_lo[kMaxChunks], b_lo[kMaxChunks];
};
__global__ void rebase_kernel(int count, int64_t* aoff, int64_t* boff, const RebaseArgs r) {
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < count; s += gridDim.x * blockDim.x) {
    int lo = 0, hi = r.nchunks - 1;  // the chunk c with s0[c] <= s < s0[c+1]
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (r.s0[mid] <= s) lo = mid;
      else hi = mid - 1;
    }
    aoff[s] -= r.a_lo[lo];
    boff[s] -= r.b_lo[lo];
  }
}

// Internal streams and events (per device, created on first use).
struct HostPipe {
  cudaStream_t in = nullptr, comp = nullptr, out = nullptr;
  cudaEvent_t fork = nullptr, in_done[2] = {}, comp_done[2] = {}, out_done[2] = {}, join[3] = {};
  bool ready = false;
};
HostPipe g_pipe[64];

int host_pipe(HostPipe** out, const char* name) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return record_cuda_error(e, name);
  if (dev < 0 || dev >= 64) return record_arg_error(-99, "host pipeline: device index >= 64");
  HostPipe& P = g_pipe[dev];
  if (!P.ready) {
    e = cudaStreamCreateWithFlags(&P.in, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&P.comp, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&P.out, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&P.fork, cudaEventDisableTiming);
    for (int i = 0; i < 2 && e == cudaSuccess; ++i) {
      e = cudaEventCreateWithFlags(&P.in_done[i], cudaEventDisableTiming);
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&P.comp_done[i], cudaEventDisableTiming);
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&P.out_done[i], cudaEventDisableTiming);
    }
    for (int i = 0; i < 3 && e == cudaSuccess; ++i) e = cudaEventCreateWithFlags(&P.join[i], cudaEventDisableTiming);
    if (e != cudaSuccess) return record_cuda_error(e, name);
    P.ready = true;
  }
  *out = &P;
  return NACU_SUCCESS;
}

}  // namespace
}  // namespace nacu

extern "C" {

size_t nacu_mixed_host_workspace_bytes(int count, int n_max, const int32_t* ns, const int64_t* a_offsets,
                                       const int64_t* b_offsets, int nrhs, int chunks) {
  using namespace nacu;
  if (count <= 0 || !ns || !a_offsets || !b_offsets || nrhs < 1) return 0;
  ChunkPlan p;
  if (plan_chunks(count, n_max, ns, a_offsets, b_offsets, nrhs, chunks, &p) != 0) return 0;
  return host_layout(count, p).total;
}

int nacu_dposv_ragged_mixed_host(int count, int n_max, const int32_t* ns, const int64_t* a_offsets, const double* A,
                                 int nrhs, const int64_t* b_offsets, const double* B, double* X, int32_t* info,
                                 int32_t* iters, int chunks, void* workspace, size_t workspace_bytes,
                                 double tol_units, int max_iter, double substitute, int flags, nacu_stream_t stream) {
  using namespace nacu;
  const char* name = "nacu_dposv_ragged_mixed_host";
  if (count < 0) return record_arg_error(-1, "dposv_ragged_mixed_host: negative count");
  if (count == 0) return NACU_SUCCESS;
  if (n_max < 0 || n_max > NACU_CHOL_RAGGED_MAX_N)
    return record_arg_error(-2, "dposv_ragged_mixed_host: n_max out of range [0, 512]");
  if (!ns || !a_offsets || !A) return record_arg_error(-3, "dposv_ragged_mixed_host: null ns, a_offsets or A");
  if (nrhs < 1 || nrhs > 4) return record_arg_error(-6, "dposv_ragged_mixed_host: nrhs out of range [1, 4]");
  if (!b_offsets || !B || !X) return record_arg_error(-7, "dposv_ragged_mixed_host: null b_offsets, B or X");
  if (!info) return record_arg_error(-10, "dposv_ragged_mixed_host: null info");
  ChunkPlan p;
  const int prc = plan_chunks(count, n_max, ns, a_offsets, b_offsets, nrhs, chunks, &p);
  if (prc == -2) return record_arg_error(-2, "dposv_ragged_mixed_host: an order is outside [0, n_max]");
  if (prc != 0) return record_arg_error(-4, "dposv_ragged_mixed_host: offsets must be non-negative and non-decreasing");
  const HostLayout L = host_layout(count, p);
  if (!workspace || workspace_bytes < L.total) return record_arg_error(-14, "dposv_ragged_mixed_host: workspace too small");
  if ((reinterpret_cast<uintptr_t>(workspace) & 255) != 0)
    return record_arg_error(-14, "dposv_ragged_mixed_host: workspace must be 256-byte aligned");
  unsigned char* ws = static_cast<unsigned char*>(workspace);
  int32_t* d_ns = reinterpret_cast<int32_t*>(ws + L.ns);
  int32_t* d_order = reinterpret_cast<int32_t*>(ws + L.order);
  int32_t* d_info = reinterpret_cast<int32_t*>(ws + L.info);
  int32_t* d_iters = reinterpret_cast<int32_t*>(ws + L.iters);
  int64_t* d_aoff = reinterpret_cast<int64_t*>(ws + L.aoff);
  int64_t* d_boff = reinterpret_cast<int64_t*>(ws + L.boff);

  HostPipe* P = nullptr;
  int rc = host_pipe(&P, name);
  if (rc != NACU_SUCCESS) return rc;
  const cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = cudaEventRecord(P->fork, s);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(P->in, P->fork, 0);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(P->comp, P->fork, 0);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(P->out, P->fork, 0);
  // the orders and offsets (small), then offsets relative to their chunk
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_ns, ns, (size_t)count * 4, cudaMemcpyHostToDevice, P->in);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_aoff, a_offsets, (size_t)count * 8, cudaMemcpyHostToDevice, P->in);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_boff, b_offsets, (size_t)count * 8, cudaMemcpyHostToDevice, P->in);
  if (e != cudaSuccess) return record_cuda_error(e, name);
  {
    RebaseArgs r;
    std::memset(&r, 0, sizeof(r));
    r.nchunks = p.nchunks;
    for (int c = 0; c <= p.nchunks; ++c) r.s0[c] = p.s0[c];
    for (int c = 0; c < p.nchunks; ++c) {
      r.a_lo[c] = p.a_lo[c];
      r.b_lo[c] = p.b_lo[c];
    }
    rebase_kernel<<<std::min(sm_count() * 4, (count + 255) / 256), 256, 0, P->in>>>(count, d_aoff, d_boff, r);
    rc = check_launch(name);
    if (rc != NACU_SUCCESS) return rc;
  }
  for (int c = 0; c < p.nchunks; ++c) {
    const int st = c & 1;
    const int s0 = p.s0[c], cnt = p.s0[c + 1] - s0;
    double* sa = reinterpret_cast<double*>(ws + L.stage_a[st]);
    double* sb = reinterpret_cast<double*>(ws + L.stage_b[st]);
    double* sx = reinterpret_cast<double*>(ws + L.stage_x[st]);
    const int64_t na = p.a_hi[c] - p.a_lo[c], nb = p.b_hi[c] - p.b_lo[c];
    // copy in: the stage is free once chunk c-2's solve has read it
    if (c >= 2) e = cudaStreamWaitEvent(P->in, P->comp_done[st], 0);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(sa, A + p.a_lo[c], (size_t)na * 8, cudaMemcpyHostToDevice, P->in);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(sb, B + p.b_lo[c], (size_t)nb * 8, cudaMemcpyHostToDevice, P->in);
    if (e == cudaSuccess) e = cudaEventRecord(P->in_done[st], P->in);
    // solve: after the copy in, and once chunk c-2's solutions have left sx
    if (e == cudaSuccess) e = cudaStreamWaitEvent(P->comp, P->in_done[st], 0);
    if (e == cudaSuccess && c >= 2) e = cudaStreamWaitEvent(P->comp, P->out_done[st], 0);
    if (e != cudaSuccess) return record_cuda_error(e, name);
    rc = ragged_order_desc(cnt, n_max, d_ns + s0, d_order + s0, ws + L.sort, P->comp, name);
    if (rc != NACU_SUCCESS) return rc;
    rc = nacu_dposv_ragged_mixed(cnt, n_max, d_ns + s0, d_aoff + s0, sa, nrhs, d_boff + s0, sb, sx, d_info + s0,
                                 d_iters + s0, d_order + s0, na, ws + L.solver, L.total - L.solver, tol_units,
                                 max_iter, substitute, flags, (nacu_stream_t)P->comp);
    if (rc != NACU_SUCCESS) return rc;
    e = cudaEventRecord(P->comp_done[st], P->comp);
    // copy out
    if (e == cudaSuccess) e = cudaStreamWaitEvent(P->out, P->comp_done[st], 0);
    if (e == cudaSuccess) e = cudaMemcpyAsync(X + p.b_lo[c], sx, (size_t)nb * 8, cudaMemcpyDeviceToHost, P->out);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(info + s0, d_info + s0, (size_t)cnt * 4, cudaMemcpyDeviceToHost, P->out);
    if (e == cudaSuccess && iters)
      e = cudaMemcpyAsync(iters + s0, d_iters + s0, (size_t)cnt * 4, cudaMemcpyDeviceToHost, P->out);
    if (e == cudaSuccess) e = cudaEventRecord(P->out_done[st], P->out);
    if (e != cudaSuccess) return record_cuda_error(e, name);
  }
  // join every internal stream back to the caller's stream
  e = cudaEventRecord(P->join[0], P->in);
  if (e == cudaSuccess) e = cudaEventRecord(P->join[1], P->comp);
  if (e == cudaSuccess) e = cudaEventRecord(P->join[2], P->out);
  for (int i = 0; i < 3 && e == cudaSuccess; ++i) e = cudaStreamWaitEvent(s, P->join[i], 0);
  if (e != cudaSuccess) return record_cuda_error(e, name);
  return NACU_SUCCESS;
}

}  // extern "C"
