// Library-level entry points: version, error reporting, the FP64 roofline probe.
#include <algorithm>
#include <cstdio>
#include <cstring>

#include "common.cuh"

namespace nacu {

namespace {
thread_local char g_last_error[512] = "";
}

int record_cuda_error(cudaError_t e, const char* where) {
  std::snprintf(g_last_error, sizeof(g_last_error), "%s: CUDA error %d (%s)", where, (int)e, cudaGetErrorString(e));
  return NACU_ERR_CUDA;
}

int record_arg_error(int code, const char* msg) {
  std::snprintf(g_last_error, sizeof(g_last_error), "%s (argument %d)", msg, -code);
  return code;
}

namespace {

__device__ double g_probe_sink;

// Sixteen independent DFMA chains per thread, two warps per SM sub-partition
// (the FP64 unit needs little latency hiding but every issue slot must carry a
// DFMA); the result is stored only when it equals an impossible value, so the
// chains are live but nothing is written.
__global__ void __launch_bounds__(256) fp64_probe_kernel(int iters, double s) {
  double a[16];
#pragma unroll
  for (int i = 0; i < 16; ++i) a[i] = threadIdx.x * 1e-3 + i;
  const double m = 0.999999;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int i = 0; i < 16; ++i) a[i] = fma(a[i], m, s);
  }
  double r = 0.0;
#pragma unroll
  for (int i = 0; i < 16; ++i) r += a[i];
  if (r == -12345.678) g_probe_sink = r;
}

__global__ void rcp_test_kernel(int n, const double* __restrict__ d, double* __restrict__ out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) out[i] = rcp_nr(d[i]);
}

}  // namespace
}  // namespace nacu

extern "C" {

const char* nacu_version(void) { return "0.1.0"; }

int nacu_test_rcp(int n, const double* d, double* out, nacu_stream_t stream) {
  using namespace nacu;
  if (n < 0) return record_arg_error(-1, "test_rcp: n < 0");
  if (n == 0) return NACU_SUCCESS;
  if (!d || !out) return record_arg_error(-2, "test_rcp: null pointer");
  const int blocks = std::min((n + 255) / 256, sm_count() * 8);
  rcp_test_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(n, d, out);
  return check_launch("nacu_test_rcp");
}

const char* nacu_last_error(void) { return nacu::g_last_error; }

int nacu_device_arch(void) {
#if defined(NACU_ARCH)
  return NACU_ARCH;
#else
  return 103;
#endif
}

int nacu_probe_fp64_peak(double* flops) {
  using namespace nacu;
  if (!flops) return record_arg_error(-1, "probe_fp64_peak: null output");
  const int blocks = sm_count() * 2, threads = 256, iters = 4000;
  cudaEvent_t e0, e1;
  cudaError_t e = cudaEventCreate(&e0);
  if (e != cudaSuccess) return record_cuda_error(e, "probe_fp64_peak");
  cudaEventCreate(&e1);
  double best = 0.0;
  for (int rep = 0; rep < 4; ++rep) {
    cudaEventRecord(e0, 0);
    fp64_probe_kernel<<<blocks, threads>>>(iters, 1e-9);
    cudaEventRecord(e1, 0);
    e = cudaEventSynchronize(e1);
    if (e != cudaSuccess) {
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      return record_cuda_error(e, "probe_fp64_peak");
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    const double f = 2.0 * 16.0 * (double)blocks * threads * iters / (ms * 1e-3);
    if (rep > 0 && f > best) best = f;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *flops = best;
  return check_launch("probe_fp64_peak");
}

}  // extern "C"
