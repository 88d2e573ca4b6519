//! Device memory, copies and stream synchronisation for the crate, through
//! the library's own plumbing entry points (`nacu_malloc`, `nacu_memcpy`, ...
//! in include/nalgebra_cuda.h): the crate links libnalgebra_cuda and nothing
//! else of CUDA.
use std::os::raw::c_int;

pub use crate::ffi::{nacu_free, nacu_malloc, nacu_memcpy, nacu_memset, nacu_stream_synchronize};

pub fn check(rc: c_int, what: &str) {
    if rc != 0 {
        let msg = unsafe { std::ffi::CStr::from_ptr(crate::ffi::nacu_last_error()) };
        panic!("{what} failed with code {rc}: {}", msg.to_string_lossy());
    }
}
