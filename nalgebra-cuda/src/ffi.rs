//! Raw bindings of `libnalgebra_cuda.so` (the C ABI declared in
//! `include/nalgebra_cuda.h`).  Device pointers are plain pointers; `Stream`
//! is a `cudaStream_t` (null: the legacy default stream).  Every entry point
//! returns 0 on success, `-k` when argument k is invalid, or a CUDA error
//! code; `nacu_last_error` holds the message.
use std::os::raw::{c_char, c_int, c_void};
pub type Stream = *mut c_void; // cudaStream_t
pub const NACU_FLAG_EXACT: c_int = 1;
pub const NACU_FLAG_NO_FACTORS: c_int = 2;
pub const NACU_FLAG_SUBSTITUTE: c_int = 4;
pub const NACU_FLAG_VERIFY: c_int = 8;

#[link(name = "nalgebra_cuda")]
extern "C" {
    pub fn nacu_last_error() -> *const c_char;
    // device memory, copies, streams, graphs (the crate's DeviceBuffer uses these)
    pub fn nacu_device_count(count: *mut c_int) -> c_int;
    pub fn nacu_malloc(ptr: *mut *mut c_void, bytes: usize) -> c_int;
    pub fn nacu_free(ptr: *mut c_void) -> c_int;
    pub fn nacu_host_alloc(ptr: *mut *mut c_void, bytes: usize) -> c_int;
    pub fn nacu_host_free(ptr: *mut c_void) -> c_int;
    pub fn nacu_memcpy(dst: *mut c_void, src: *const c_void, bytes: usize, s: Stream) -> c_int;
    pub fn nacu_memset(ptr: *mut c_void, value: c_int, bytes: usize, s: Stream) -> c_int;
    pub fn nacu_stream_create(s: *mut Stream) -> c_int;
    pub fn nacu_stream_destroy(s: Stream) -> c_int;
    pub fn nacu_stream_synchronize(s: Stream) -> c_int;
    pub fn nacu_stream_wait(waiting: Stream, on: Stream) -> c_int;
    pub fn nacu_device_synchronize() -> c_int;
    pub fn nacu_graph_begin_capture(s: Stream) -> c_int;
    pub fn nacu_graph_end_capture(s: Stream, graph_exec: *mut *mut c_void) -> c_int;
    pub fn nacu_graph_launch(graph_exec: *mut c_void, s: Stream) -> c_int;
    pub fn nacu_graph_destroy(graph_exec: *mut c_void) -> c_int;
    // LU, batched (n <= 128) and large
    pub fn nacu_dgetrf_batched(n: c_int, a: *mut f64, stride_a: i64, ipiv: *mut i32,
                               info: *mut i32, batch: c_int, flags: c_int, s: Stream) -> c_int;
    pub fn nacu_dgetrs_batched(n: c_int, nrhs: c_int, lu: *mut f64, stride_a: i64, ipiv: *mut i32,
                               b: *mut f64, stride_b: i64, info: *mut i32, batch: c_int,
                               flags: c_int, s: Stream) -> c_int;
    pub fn nacu_dgesv_batched(n: c_int, nrhs: c_int, a: *mut f64, stride_a: i64, ipiv: *mut i32,
                              b: *mut f64, stride_b: i64, info: *mut i32, batch: c_int,
                              flags: c_int, s: Stream) -> c_int;
    // Matrix::{solve,tr_solve,ad_solve}_{lower,upper}_triangular_mut (solve.rs:55-442)
    pub fn nacu_dtrsv_batched(n: c_int, nrhs: c_int, upper: c_int, trans: c_int, has_diag: c_int,
                              diag: f64, t: *const f64, stride_t: i64, b: *mut f64, stride_b: i64,
                              info: *mut i32, batch: c_int, flags: c_int, s: Stream) -> c_int;
    // the same solves for one matrix of any order
    pub fn nacu_trsv_workspace_bytes(n: c_int) -> usize;
    pub fn nacu_dtrsv(n: c_int, nrhs: c_int, upper: c_int, trans: c_int, has_diag: c_int, diag: f64,
                      t: *const f64, lda: i64, b: *mut f64, ldb: i64, info: *mut i32, ws: *mut c_void,
                      ws_bytes: usize, flags: c_int, s: Stream) -> c_int;
    // LU::try_inverse (lu.rs:266-297) from getrf factors
    pub fn nacu_dgetri_batched(n: c_int, lu: *const f64, stride_a: i64, ipiv: *const i32,
                               a_inv: *mut f64, stride_inv: i64, info: *mut i32, batch: c_int,
                               flags: c_int, s: Stream) -> c_int;
    // Cholesky::{rank_one_update, remove_column, insert_column} (cholesky.rs:277-449)
    pub fn nacu_dchol_rank1_update_batched(n: c_int, l: *mut f64, stride_l: i64, x: *const f64,
                                           stride_x: i64, sigma: *const f64, batch: c_int,
                                           flags: c_int, s: Stream) -> c_int;
    pub fn nacu_dchol_remove_column_batched(n: c_int, l: *const f64, stride_l: i64, j: c_int,
                                            l_out: *mut f64, stride_out: i64, batch: c_int,
                                            flags: c_int, s: Stream) -> c_int;
    pub fn nacu_dchol_insert_column_batched(n: c_int, l: *const f64, stride_l: i64, j: c_int,
                                            col: *const f64, stride_col: i64, l_out: *mut f64,
                                            stride_out: i64, info: *mut i32, batch: c_int,
                                            flags: c_int, s: Stream) -> c_int;
    // FullPivLU::new and solve_mut (full_piv_lu.rs:56-91, 185-211)
    pub fn nacu_dfullpivlu_batched(n: c_int, nrhs: c_int, a: *mut f64, stride_a: i64, ipiv: *mut i32,
                                   jpiv: *mut i32, b: *mut f64, stride_b: i64, info: *mut i32,
                                   batch: c_int, flags: c_int, s: Stream) -> c_int;
    pub fn nacu_dfullpivlu_solve_batched(n: c_int, nrhs: c_int, lu: *const f64, stride_a: i64,
                                         ipiv: *const i32, jpiv: *const i32, b: *mut f64, stride_b: i64,
                                         info: *mut i32, batch: c_int, flags: c_int, s: Stream) -> c_int;
    // ColPivQR::new and solve_mut (col_piv_qr.rs:59-92, 227-247)
    pub fn nacu_dcolpivqr_batched(n: c_int, nrhs: c_int, a: *mut f64, stride_a: i64, diag: *mut f64,
                                  jpiv: *mut i32, b: *mut f64, stride_b: i64, info: *mut i32,
                                  batch: c_int, flags: c_int, s: Stream) -> c_int;
    pub fn nacu_dcolpivqr_solve_batched(n: c_int, nrhs: c_int, qr: *const f64, stride_a: i64,
                                        diag: *const f64, jpiv: *const i32, b: *mut f64, stride_b: i64,
                                        info: *mut i32, batch: c_int, flags: c_int, s: Stream) -> c_int;
    // QR::new and solve_mut for square matrices (qr.rs:55-76, 204-256)
    pub fn nacu_dqr_batched(n: c_int, nrhs: c_int, a: *mut f64, stride_a: i64, diag: *mut f64, b: *mut f64,
                            stride_b: i64, info: *mut i32, batch: c_int, flags: c_int, s: Stream) -> c_int;
    pub fn nacu_dqr_solve_batched(n: c_int, nrhs: c_int, qr: *const f64, stride_a: i64, diag: *const f64,
                                  b: *mut f64, stride_b: i64, info: *mut i32, batch: c_int, flags: c_int,
                                  s: Stream) -> c_int;
    // QR::new of one matrix of any shape, and its square / least-squares solve
    pub fn nacu_dqr(m: c_int, n: c_int, a: *mut f64, lda: i64, diag: *mut f64, flags: c_int, s: Stream) -> c_int;
    pub fn nacu_qr_solve_workspace_bytes(n: c_int) -> usize;
    pub fn nacu_dqr_solve(m: c_int, n: c_int, nrhs: c_int, qr: *const f64, lda: i64, diag: *const f64,
                          b: *mut f64, ldb: i64, info: *mut i32, ws: *mut c_void, ws_bytes: usize, flags: c_int,
                          s: Stream) -> c_int;
    pub fn nacu_getrf_workspace_bytes(n: c_int) -> usize;
    pub fn nacu_dgetrf(n: c_int, a: *mut f64, lda: i64, ipiv: *mut i32, info: *mut i32,
                       ws: *mut c_void, ws_bytes: usize, s: Stream) -> c_int;
    pub fn nacu_dgetrs(n: c_int, lu: *const f64, lda: i64, ipiv: *const i32, b: *mut f64,
                       info: *mut i32, ws: *mut c_void, ws_bytes: usize, s: Stream) -> c_int;
    // Cholesky, ragged batch
    pub fn nacu_ragged_workspace_bytes(count: c_int) -> usize;
    pub fn nacu_dposv_ragged(count: c_int, n_max: c_int, ns: *const i32, a_off: *const i64,
                             a: *mut f64, nrhs: c_int, b_off: *const i64, b: *mut f64,
                             info: *mut i32, logdet: *mut f64, order: *const i32,
                             ws: *mut c_void, ws_bytes: usize, substitute: f64, flags: c_int,
                             s: Stream) -> c_int;
    pub fn nacu_dpotrf_ragged(count: c_int, n_max: c_int, ns: *const i32, a_off: *const i64,
                              a: *mut f64, info: *mut i32, logdet: *mut f64, order: *const i32,
                              ws: *mut c_void, ws_bytes: usize, substitute: f64, flags: c_int,
                              s: Stream) -> c_int;
    pub fn nacu_dpotrs_ragged(count: c_int, n_max: c_int, ns: *const i32, a_off: *const i64,
                              l: *const f64, nrhs: c_int, b_off: *const i64, b: *mut f64,
                              order: *const i32, ws: *mut c_void, ws_bytes: usize, flags: c_int,
                              s: Stream) -> c_int;
    pub fn nacu_dposv(n: c_int, a: *mut f64, nrhs: c_int, b: *mut f64, info: *mut i32,
                      logdet: *mut f64, substitute: f64, flags: c_int, s: Stream) -> c_int;
    // QR least squares, GEMM
    pub fn nacu_qr_workspace_bytes(count: c_int) -> usize;
    pub fn nacu_dgels_batched(count: c_int, n: c_int, m_max: c_int, ms: *const i32,
                              a_off: *const i64, a: *mut f64, b_off: *const i64, b: *mut f64,
                              x: *mut f64, diag: *mut f64, info: *mut i32, order: *const i32,
                              ws: *mut c_void, ws_bytes: usize, flags: c_int, s: Stream) -> c_int;
    pub fn nacu_dgemm(m: c_int, n: c_int, k: c_int, alpha: f64, a: *const f64, lda: i64,
                      b: *const f64, ldb: i64, beta: f64, c: *mut f64, ldc: i64, s: Stream) -> c_int;
    pub fn nacu_dgemm_batched(m: c_int, n: c_int, k: c_int, alpha: f64, a: *const f64, lda: i64, stride_a: i64,
                              b: *const f64, ldb: i64, stride_b: i64, beta: f64, c: *mut f64, ldc: i64,
                              stride_c: i64, batch: c_int, flags: c_int, s: Stream) -> c_int;
    // chosen forms
    pub fn nacu_mixed_workspace_bytes(count: c_int, total_matrix_elements: i64) -> usize;
    pub fn nacu_dposv_ragged_mixed(count: c_int, n_max: c_int, ns: *const i32, a_off: *const i64,
                                   a: *const f64, nrhs: c_int, b_off: *const i64, b: *const f64,
                                   x: *mut f64, info: *mut i32, iters: *mut i32, order: *const i32,
                                   total_matrix_elements: i64, ws: *mut c_void, ws_bytes: usize,
                                   tol_units: f64, max_iter: c_int, substitute: f64, flags: c_int,
                                   s: Stream) -> c_int;
    // the same solve with every array in host memory (page-locked for overlap)
    pub fn nacu_mixed_host_workspace_bytes(count: c_int, n_max: c_int, ns: *const i32, a_off: *const i64,
                                           b_off: *const i64, nrhs: c_int, chunks: c_int) -> usize;
    pub fn nacu_dposv_ragged_mixed_host(count: c_int, n_max: c_int, ns: *const i32, a_off: *const i64,
                                        a: *const f64, nrhs: c_int, b_off: *const i64, b: *const f64,
                                        x: *mut f64, info: *mut i32, iters: *mut i32, chunks: c_int,
                                        ws: *mut c_void, ws_bytes: usize, tol_units: f64,
                                        max_iter: c_int, substitute: f64, flags: c_int,
                                        s: Stream) -> c_int;
    pub fn nacu_gesv_mixed_workspace_bytes(n: c_int) -> usize;
    pub fn nacu_dgesv_mixed_ir(n: c_int, a: *const f64, lda: i64, b: *const f64, x: *mut f64,
                               tol_units: f64, max_iter: c_int, iters: *mut c_int, berr: *mut f64,
                               fallback: *mut c_int, ws: *mut c_void, ws_bytes: usize,
                               s: Stream) -> c_int;
    pub fn nacu_gemm_split_workspace_bytes(m: c_int, n: c_int, k: c_int) -> usize;
    pub fn nacu_dgemm_split_bf16(m: c_int, n: c_int, k: c_int, alpha: f64, a: *const f64, lda: i64,
                                 b: *const f64, ldb: i64, beta: f64, c: *mut f64, ldc: i64,
                                 slices: c_int, ws: *mut c_void, ws_bytes: usize, s: Stream) -> c_int;
    pub fn nacu_dposv_logdet_forward(n: c_int, a: *const f64, stride_a: i64, b: *const f64,
                                     x: *mut f64, l: *mut f64, logdet: *mut f64, info: *mut i32,
                                     batch: c_int, s: Stream) -> c_int;
    pub fn nacu_dposv_logdet_backward(n: c_int, al: *const f64, stride_a: i64, recompute: c_int,
                                      x: *const f64, x_bar: *const f64, logdet_bar: *const f64,
                                      da: *mut f64, db: *mut f64, info: *mut i32, batch: c_int,
                                      s: Stream) -> c_int;
    pub fn nacu_ragged_autotune(per_bucket: c_int, nrhs: c_int, flags: c_int, table: *mut i32,
                                ms: *mut f64, s: Stream) -> c_int;
    pub fn nacu_ragged_set_tuning(table: *const i32, nbuckets: c_int) -> c_int;
    // allocation-free ragged Cholesky (scratch in the library's own device array)
    pub fn nacu_dposv_ragged_noalloc(count: c_int, n_max: c_int, ns: *const i32, a_off: *const i64,
                                     a: *mut f64, nrhs: c_int, b_off: *const i64, b: *mut f64,
                                     info: *mut i32, logdet: *mut f64, substitute: f64, flags: c_int,
                                     s: Stream) -> c_int;
    pub fn nacu_sgesv_batched(n: c_int, nrhs: c_int, a: *mut f32, stride_a: i64, ipiv: *mut i32,
                              b: *mut f32, stride_b: i64, info: *mut i32, batch: c_int,
                              flags: c_int, s: Stream) -> c_int;
    pub fn nacu_sposv_logdet_forward(n: c_int, a: *const f32, stride_a: i64, b: *const f32,
                                     x: *mut f32, l: *mut f32, logdet: *mut f32, info: *mut i32,
                                     batch: c_int, s: Stream) -> c_int;
    pub fn nacu_sposv_logdet_backward(n: c_int, al: *const f32, stride_a: i64, recompute: c_int,
                                      x: *const f32, x_bar: *const f32, logdet_bar: *const f32,
                                      da: *mut f32, db: *mut f32, info: *mut i32, batch: c_int,
                                      s: Stream) -> c_int;
    pub fn nacu_split_gemm_error(flag_out: *mut c_int) -> c_int;
    pub fn nacu_version() -> *const c_char;
    pub fn nacu_device_arch() -> c_int;
    pub fn nacu_ragged_tuning_layout(bucket_hi: *mut i32, tile_threads: *mut i32, tile_nb: *mut i32) -> c_int;
    pub fn nacu_ragged_get_tuning(table: *mut i32, nbuckets: c_int) -> c_int;
    pub fn nacu_probe_fp64_peak(flops: *mut f64) -> c_int;
    // test hook: the triangular solve's bounded flag wait made to run out
    pub fn nacu_test_rcp(n: c_int, d: *const f64, out: *mut f64, s: Stream) -> c_int;
    pub fn nacu_test_dgetrs_flag_timeout(n: c_int, lu: *const f64, lda: i64, ipiv: *const i32, b: *mut f64,
                                         info: *mut i32, skip_block: c_int, poll_limit: c_int, ws: *mut c_void,
                                         ws_bytes: usize, s: Stream) -> c_int;
}
