//! The few CUDA runtime calls the crate makes itself: device memory, copies
//! and stream synchronisation (the kernels are reached through `ffi`).
use std::os::raw::{c_int, c_void};

pub type CudaError = c_int;
pub const MEMCPY_HOST_TO_DEVICE: c_int = 1;
pub const MEMCPY_DEVICE_TO_HOST: c_int = 2;
pub const MEMCPY_DEVICE_TO_DEVICE: c_int = 3;

extern "C" {
    pub fn cudaMalloc(ptr: *mut *mut c_void, size: usize) -> CudaError;
    pub fn cudaFree(ptr: *mut c_void) -> CudaError;
    pub fn cudaMemcpy(dst: *mut c_void, src: *const c_void, count: usize, kind: c_int) -> CudaError;
    pub fn cudaMemset(ptr: *mut c_void, value: c_int, count: usize) -> CudaError;
    pub fn cudaStreamSynchronize(stream: *mut c_void) -> CudaError;
}

pub fn check(e: CudaError, what: &str) {
    if e != 0 {
        panic!("{what}: CUDA error {e}");
    }
}
