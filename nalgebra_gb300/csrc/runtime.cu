// Device memory, copies, streams and CUDA-graph capture for hosts that have
// no CUDA binding of their own (the Python mirror, a Rust crate without the
// cuda-runtime crate).  They are thin: each is one CUDA runtime call with the
// library's error convention (NACU_ERR_CUDA and a message for
// nacu_last_error), so a host needs this one library and nothing else to move
// matrices to the GPU, run the kernels and read the results back.
#include "common.cuh"

extern "C" {

int nacu_device_count(int* count) {
  using namespace nacu;
  if (!count) return record_arg_error(-1, "device_count: null output");
  const cudaError_t e = cudaGetDeviceCount(count);
  if (e != cudaSuccess) {
    *count = 0;
    (void)cudaGetLastError();
    return record_cuda_error(e, "nacu_device_count");
  }
  return NACU_SUCCESS;
}

int nacu_malloc(void** ptr, size_t bytes) {
  using namespace nacu;
  if (!ptr) return record_arg_error(-1, "malloc: null output");
  *ptr = nullptr;
  if (bytes == 0) return NACU_SUCCESS;
  const cudaError_t e = cudaMalloc(ptr, bytes);
  if (e != cudaSuccess) {
    *ptr = nullptr;
    (void)cudaGetLastError();
    return record_cuda_error(e, "nacu_malloc");
  }
  return NACU_SUCCESS;
}

int nacu_free(void* ptr) {
  using namespace nacu;
  if (!ptr) return NACU_SUCCESS;
  const cudaError_t e = cudaFree(ptr);
  return e == cudaSuccess ? NACU_SUCCESS : record_cuda_error(e, "nacu_free");
}

int nacu_host_alloc(void** ptr, size_t bytes) {
  using namespace nacu;
  if (!ptr) return record_arg_error(-1, "host_alloc: null output");
  *ptr = nullptr;
  if (bytes == 0) return NACU_SUCCESS;
  const cudaError_t e = cudaMallocHost(ptr, bytes);
  if (e != cudaSuccess) {
    *ptr = nullptr;
    (void)cudaGetLastError();
    return record_cuda_error(e, "nacu_host_alloc");
  }
  return NACU_SUCCESS;
}

int nacu_host_free(void* ptr) {
  using namespace nacu;
  if (!ptr) return NACU_SUCCESS;
  const cudaError_t e = cudaFreeHost(ptr);
  return e == cudaSuccess ? NACU_SUCCESS : record_cuda_error(e, "nacu_host_free");
}

int nacu_memcpy(void* dst, const void* src, size_t bytes, nacu_stream_t stream) {
  using namespace nacu;
  if (bytes == 0) return NACU_SUCCESS;
  if (!dst) return record_arg_error(-1, "memcpy: null destination");
  if (!src) return record_arg_error(-2, "memcpy: null source");
  // The direction follows from the unified address space.
  const cudaError_t e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, (cudaStream_t)stream);
  return e == cudaSuccess ? NACU_SUCCESS : record_cuda_error(e, "nacu_memcpy");
}

int nacu_memset(void* ptr, int value, size_t bytes, nacu_stream_t stream) {
  using namespace nacu;
  if (bytes == 0) return NACU_SUCCESS;
  if (!ptr) return record_arg_error(-1, "memset: null pointer");
  const cudaError_t e = cudaMemsetAsync(ptr, value, bytes, (cudaStream_t)stream);
  return e == cudaSuccess ? NACU_SUCCESS : record_cuda_error(e, "nacu_memset");
}

int nacu_stream_create(nacu_stream_t* stream) {
  using namespace nacu;
  if (!stream) return record_arg_error(-1, "stream_create: null output");
  cudaStream_t s = nullptr;
  const cudaError_t e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  if (e != cudaSuccess) return record_cuda_error(e, "nacu_stream_create");
  *stream = (nacu_stream_t)s;
  return NACU_SUCCESS;
}

int nacu_stream_destroy(nacu_stream_t stream) {
  using namespace nacu;
  if (!stream) return NACU_SUCCESS;
  const cudaError_t e = cudaStreamDestroy((cudaStream_t)stream);
  return e == cudaSuccess ? NACU_SUCCESS : record_cuda_error(e, "nacu_stream_destroy");
}

int nacu_stream_synchronize(nacu_stream_t stream) {
  using namespace nacu;
  const cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
  return e == cudaSuccess ? NACU_SUCCESS : record_cuda_error(e, "nacu_stream_synchronize");
}

int nacu_stream_wait(nacu_stream_t waiting, nacu_stream_t on) {
  using namespace nacu;
  cudaEvent_t ev;
  cudaError_t e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
  if (e != cudaSuccess) return record_cuda_error(e, "nacu_stream_wait");
  e = cudaEventRecord(ev, (cudaStream_t)on);
  if (e == cudaSuccess) e = cudaStreamWaitEvent((cudaStream_t)waiting, ev, 0);
  const cudaError_t e2 = cudaEventDestroy(ev);
  if (e == cudaSuccess) e = e2;
  return e == cudaSuccess ? NACU_SUCCESS : record_cuda_error(e, "nacu_stream_wait");
}

int nacu_device_synchronize(void) {
  using namespace nacu;
  const cudaError_t e = cudaDeviceSynchronize();
  return e == cudaSuccess ? NACU_SUCCESS : record_cuda_error(e, "nacu_device_synchronize");
}

int nacu_graph_begin_capture(nacu_stream_t stream) {
  using namespace nacu;
  if (!stream) return record_arg_error(-1, "graph_begin_capture: capture needs a created stream, not the default");
  const cudaError_t e = cudaStreamBeginCapture((cudaStream_t)stream, cudaStreamCaptureModeThreadLocal);
  return e == cudaSuccess ? NACU_SUCCESS : record_cuda_error(e, "nacu_graph_begin_capture");
}

int nacu_graph_end_capture(nacu_stream_t stream, void** graph_exec) {
  using namespace nacu;
  if (!stream) return record_arg_error(-1, "graph_end_capture: null stream");
  if (!graph_exec) return record_arg_error(-2, "graph_end_capture: null output");
  *graph_exec = nullptr;
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamEndCapture((cudaStream_t)stream, &g);
  if (e != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    return record_cuda_error(e, "nacu_graph_end_capture");
  }
  cudaGraphExec_t x = nullptr;
  e = cudaGraphInstantiate(&x, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return record_cuda_error(e, "nacu_graph_end_capture (instantiate)");
  *graph_exec = (void*)x;
  return NACU_SUCCESS;
}

int nacu_graph_launch(void* graph_exec, nacu_stream_t stream) {
  using namespace nacu;
  if (!graph_exec) return record_arg_error(-1, "graph_launch: null graph");
  const cudaError_t e = cudaGraphLaunch((cudaGraphExec_t)graph_exec, (cudaStream_t)stream);
  return e == cudaSuccess ? NACU_SUCCESS : record_cuda_error(e, "nacu_graph_launch");
}

int nacu_graph_destroy(void* graph_exec) {
  using namespace nacu;
  if (!graph_exec) return NACU_SUCCESS;
  const cudaError_t e = cudaGraphExecDestroy((cudaGraphExec_t)graph_exec);
  return e == cudaSuccess ? NACU_SUCCESS : record_cuda_error(e, "nacu_graph_destroy");
}

}  // extern "C"
