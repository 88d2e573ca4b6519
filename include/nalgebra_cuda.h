/*
 * nalgebra-cuda: C ABI of the GB300 (sm_103a) dense linear-algebra library.
 *
 * This is the drop-in boundary for nalgebra's dense solve path: the calls a
 * `nalgebra-cuda` crate (or any other host) binds over FFI in place of
 * nalgebra's CPU `LU` / `Cholesky` / `QR` / `Matrix::gemm`.  Every reference
 * function each entry point replaces is cited (file:line inside the nalgebra
 * 0.35 source tree).
 *
 * Conventions (shared by every entry point):
 *  - Matrices are column-major and contiguous, element (r, c) at a[r + c*lda],
 *    exactly nalgebra's VecStorage (src/base/vec_storage.rs:28-32).
 *  - All matrix / vector / info pointers are DEVICE pointers owned by the
 *    caller.  Factorizations overwrite their input in place, as nalgebra's
 *    consume-and-factor constructors do (src/linalg/lu.rs:93,
 *    src/linalg/cholesky.rs:221, src/linalg/qr.rs:55).
 *  - Every call is asynchronous on the given CUDA stream (`nacu_stream_t` is a
 *    `cudaStream_t`; NULL = the legacy default stream) and does not
 *    synchronize.  No call allocates device memory; scratch is passed in by the
 *    caller (sizes from the *_workspace_bytes queries, the LAPACK lwork idiom,
 *    nalgebra-lapack/src/qr.rs:79-100).
 *  - Return value: NACU_SUCCESS (0); -i when argument i (1-based) is invalid
 *    (LAPACK xerbla convention); NACU_ERR_CUDA when a CUDA call or launch
 *    failed.  nacu_last_error() returns a message for the last failure on the
 *    calling thread.
 *  - Per-matrix numerical status goes to a device `int32_t info[]`: 0 = ok,
 *    k > 0 = the 1-based index of the failing pivot (LU: first zero U_kk;
 *    Cholesky: first non-positive or NaN pivot; least squares: a zero R_kk),
 *    as nalgebra-lapack's info (nalgebra-lapack/src/lapack_error.rs:14-20).
 *    A host binding maps info != 0 to nalgebra's None / false.
 *  - Pivots are 0-based per step: ipiv[i] = the row swapped with row i at
 *    elimination step i (ipiv[i] == i: no swap).  The (i, ipiv[i]) pairs with
 *    ipiv[i] != i, in order, are nalgebra's PermutationSequence
 *    (src/linalg/permutation_sequence.rs:84-93); their count's parity is the
 *    determinant sign (permutation_sequence.rs:158-164).
 */
#ifndef NALGEBRA_CUDA_H
#define NALGEBRA_CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef void* nacu_stream_t;

#define NACU_SUCCESS 0
#define NACU_ERR_CUDA 1
#define NACU_ERR_UNSUPPORTED 2

/* flags (bitwise or) */
/* Reproduce nalgebra's arithmetic exactly: no FMA contraction, reciprocal
 * multiply / true division exactly where nalgebra uses them, nalgebra's
 * 8-accumulator dot order.  Factors and solutions then match nalgebra's CPU
 * results bit for bit (log-determinants to a few ulps: CUDA's log is not
 * correctly rounded).  Costs about twice the FP64 issue slots. */
#define NACU_FLAG_EXACT 1
/* gesv: do not write the LU factors back (solutions, pivots and info only). */
#define NACU_FLAG_NO_FACTORS 2
/* Cholesky: replace a failing pivot by the `substitute` argument, as
 * Cholesky::new_with_substitute does (src/linalg/cholesky.rs:216-218). */
#define NACU_FLAG_SUBSTITUTE 4
/* Mixed precision: always confirm convergence with a final FP64 residual
 * instead of accepting an iterate whose predicted error is far below the
 * target. */
#define NACU_FLAG_VERIFY 8

#define NACU_LU_BATCHED_MAX_N 128
#define NACU_LU_BATCHED_MAX_NRHS 16
#define NACU_CHOL_RAGGED_MAX_N 512
#define NACU_QR_MAX_N 128
#define NACU_QR_MAX_M 2048

/* ---- library ------------------------------------------------------------- */

/* Library version, e.g. "0.1.0". */
const char* nacu_version(void);
/* Message for the last failed call on this host thread ("" if none). */
const char* nacu_last_error(void);
/* Compiled device architecture, e.g. 103 for sm_103a. */
int nacu_device_arch(void);

/* ---- device memory, copies, streams, graphs -------------------------------
 * Plumbing for hosts without a CUDA binding of their own (nalgebra's side of
 * the FFI has none: a `DMatrix` is host memory).  Each is one CUDA runtime
 * call under the library's error convention.  nalgebra counterpart: none; a
 * `nalgebra-cuda` `DeviceMatrix::from(&DMatrix)` / `to_host()` is
 * nacu_malloc + nacu_memcpy. */

/* Number of visible CUDA devices (0 and NACU_ERR_CUDA when there is none). */
int nacu_device_count(int* count);
/* Device memory; bytes == 0 gives NULL.  nacu_free(NULL) is a no-op.
 * nacu_free synchronizes the device (cudaFree). */
int nacu_malloc(void** ptr, size_t bytes);
int nacu_free(void* ptr);
/* Page-locked host memory (lets nacu_memcpy and the *_host entry points
 * overlap copies with kernels). */
int nacu_host_alloc(void** ptr, size_t bytes);
int nacu_host_free(void* ptr);
/* Asynchronous copy on `stream`, any direction (unified addressing decides:
 * host->device, device->host, device->device).  A copy to pageable host
 * memory returns when it is complete. */
int nacu_memcpy(void* dst, const void* src, size_t bytes, nacu_stream_t stream);
/* Asynchronous byte fill on `stream`. */
int nacu_memset(void* ptr, int value, size_t bytes, nacu_stream_t stream);
/* A non-blocking stream; destroy(NULL) is a no-op. */
int nacu_stream_create(nacu_stream_t* stream);
int nacu_stream_destroy(nacu_stream_t stream);
int nacu_stream_synchronize(nacu_stream_t stream);
/* Work queued on `waiting` after this call starts after the work queued on
 * `on` before it. */
int nacu_stream_wait(nacu_stream_t waiting, nacu_stream_t on);
int nacu_device_synchronize(void);
/* CUDA-graph capture of the calls queued on `stream` (a created stream, not
 * NULL) between begin and end; *graph_exec is the instantiated graph, run by
 * nacu_graph_launch on any stream.  No call of this library allocates or
 * synchronizes inside its compute entry points, so every one of them can be
 * captured. */
int nacu_graph_begin_capture(nacu_stream_t stream);
int nacu_graph_end_capture(nacu_stream_t stream, void** graph_exec);
int nacu_graph_launch(void* graph_exec, nacu_stream_t stream);
int nacu_graph_destroy(void* graph_exec);

/* ---- LU with partial pivoting (batched, n <= 128) ------------------------- */

/* Factor `batch` n x n matrices A + s*strideA in place into nalgebra's packed
 * L\U form, with per-step pivots ipiv[s*n + i] and info[s].
 * Replaces LU::new (src/linalg/lu.rs:93-122) with icamax
 * (src/base/min_max.rs:221-240) and gauss_step(_swap) (lu.rs:337-389). */
int nacu_dgetrf_batched(int n, double* A, int64_t strideA, int32_t* ipiv, int32_t* info, int batch,
                        int flags, nacu_stream_t stream);

/* Solve A X = B from getrf factors; B + s*strideB (n x nrhs) becomes X.
 * Replaces LU::solve_mut (src/linalg/lu.rs:242-260: permute_rows,
 * solve_lower_triangular_with_diag_mut solve.rs:106-133,
 * solve_upper_triangular_mut solve.rs:137-182).  info[s] = first zero U_kk. */
int nacu_dgetrs_batched(int n, int nrhs, double* LU, int64_t strideA, int32_t* ipiv, double* B,
                        int64_t strideB, int32_t* info, int batch, int flags, nacu_stream_t stream);

/* ---- LU with full pivoting (batched, n <= 128) ------------------------------ */

/* FullPivLU::new (src/linalg/full_piv_lu.rs:56-91) on A + s*strideA (n x n,
 * in place: the packed L\U factors), and with nrhs > 0 (<= 16)
 * FullPivLU::solve_mut (:185-211) on B + s*strideB (n x nrhs).  ipiv[s*n+i]
 * / jpiv[s*n+i]: the row / column swapped with i at step i (i when none);
 * the pairs with ipiv[i] != i (jpiv[i] != i), in order, are nalgebra's p (q).
 * Steps stop where the remaining submatrix is zero, as nalgebra's do.
 * info[s] = 0 when U[n-1][n-1] != 0 (is_invertible, :242-250; B solved),
 * else 1 + the step that found the remaining submatrix zero (B untouched).
 * NACU_FLAG_EXACT: factors, pivots and solutions bit-identical to nalgebra. */
int nacu_dfullpivlu_batched(int n, int nrhs, double* A, int64_t strideA, int32_t* ipiv, int32_t* jpiv, double* B,
                            int64_t strideB, int32_t* info, int batch, int flags, nacu_stream_t stream);

/* FullPivLU::solve_mut from factors written by nacu_dfullpivlu_batched (read
 * only); `lu.try_inverse()` (:216-233) with B = the identity, 16 columns per
 * call.  info[s] = 0 (solved) or 1 + the first zero U_ii (not invertible: B
 * untouched). */
int nacu_dfullpivlu_solve_batched(int n, int nrhs, const double* LU, int64_t strideA, const int32_t* ipiv,
                                  const int32_t* jpiv, double* B, int64_t strideB, int32_t* info, int batch,
                                  int flags, nacu_stream_t stream);

/* ---- QR with column pivoting (batched, n <= 128) --------------------------- */

/* ColPivQR::new (src/linalg/col_piv_qr.rs:59-92) on A + s*strideA (n x n, in
 * place: the Householder axes at and below the diagonal, R above it),
 * diag[s*n+i] (QR::new's signed diagonal; R's is |diag|), jpiv[s*n+i] (the
 * column swapped with i at step i: the column of the trailing submatrix's
 * largest |a|); with nrhs > 0 (<= 16) ColPivQR::solve_mut (:227-247) on B +
 * s*strideB (n x nrhs; written even when the solve fails, as nalgebra's b
 * is).  info[s] = 0 when every diag entry is non-zero (is_invertible,
 * :307-320; B solved), else 1 + the first zero one.  NACU_FLAG_EXACT:
 * factors, pivots and solutions bit-identical to nalgebra. */
int nacu_dcolpivqr_batched(int n, int nrhs, double* A, int64_t strideA, double* diag, int32_t* jpiv, double* B,
                           int64_t strideB, int32_t* info, int batch, int flags, nacu_stream_t stream);

/* ColPivQR::solve_mut from factors written by nacu_dcolpivqr_batched (read
 * only); `qr.try_inverse()` (:288-303) with B = the identity, 16 columns per
 * call.  info as above. */
int nacu_dcolpivqr_solve_batched(int n, int nrhs, const double* QR, int64_t strideA, const double* diag,
                                 const int32_t* jpiv, double* B, int64_t strideB, int32_t* info, int batch, int flags,
                                 nacu_stream_t stream);

/* ---- square QR (batched, n <= 128) ----------------------------------------- */

/* QR::new (src/linalg/qr.rs:55-76) on A + s*strideA (n x n, in place: the
 * Householder axes at and below the diagonal, R above it) and diag[s*n+i]
 * (the signed diagonal; R's is |diag|); with nrhs > 0 (<= 16) QR::solve_mut
 * (:204-256: q_tr_mul, then the upper solve dividing by |diag_i|) on B +
 * s*strideB (n x nrhs; written even when the solve fails, as nalgebra's b
 * is).  info[s] = 0 when every diag entry is non-zero (is_invertible,
 * :281-292; B solved), else 1 + the first zero one.  NACU_FLAG_EXACT: factors
 * and solutions bit-identical to nalgebra. */
int nacu_dqr_batched(int n, int nrhs, double* A, int64_t strideA, double* diag, double* B, int64_t strideB,
                     int32_t* info, int batch, int flags, nacu_stream_t stream);

/* QR::solve_mut from factors written by nacu_dqr_batched (read only);
 * `qr.try_inverse()` (:262-279) with B = the identity, 16 columns per call.
 * info as above. */
int nacu_dqr_solve_batched(int n, int nrhs, const double* QR, int64_t strideA, const double* diag, double* B,
                           int64_t strideB, int32_t* info, int batch, int flags, nacu_stream_t stream);

/* ---- Householder QR of one matrix of any shape ------------------------------ */

/* QR::new (src/linalg/qr.rs:55-76) of one m x n matrix, any m and n (wide
 * matrices too, e.g. the reference's qr_decompose_100x500): A (lda >= m) is
 * overwritten with the unit Householder axes on and below the diagonal and R's
 * strict upper part above it; diag[0 .. min(m, n)) receives the signed
 * diagonal (R's diagonal is |diag|, qr.rs:81-89; 0 where a column was zero,
 * nalgebra's is_invertible false, qr.rs:281-292).  One launch per Householder
 * step, no workspace.  NACU_FLAG_EXACT: nalgebra's arithmetic, bit for bit. */
int nacu_dqr(int m, int n, double* A, int64_t lda, double* diag, int flags, nacu_stream_t stream);

/* Bytes of device scratch nacu_dqr_solve needs for an n-column factor. */
size_t nacu_qr_solve_workspace_bytes(int n);

/* Solve from the factors of nacu_dqr, m >= n, m <= 16384: B (m x nrhs,
 * ldb >= m) <- Q^T B (QR::q_tr_mul, qr.rs:157-171), then its top n rows <-
 * R^-1 (Q^T B)[0:n] (the upper solve by |diag_i| of qr.rs:224-256).  m == n is
 * QR::solve_mut; m > n the least-squares solution, as nalgebra-lapack's QR
 * solve (nalgebra-lapack/src/qr_util.rs:167-239).  *info (device) = the
 * 1-based index of the zero |diag_i| that stops nalgebra's backward
 * substitution (the last one; B then holds partial results), 0, or -1000 if
 * an internal wait between thread blocks ran out.  FMA arithmetic:
 * NACU_FLAG_EXACT returns -12. */
int nacu_dqr_solve(int m, int n, int nrhs, const double* QR, int64_t lda, const double* diag, double* B, int64_t ldb,
                   int32_t* info, void* workspace, size_t workspace_bytes, int flags, nacu_stream_t stream);

/* Inverse from getrf factors: `lu.try_inverse()` (src/linalg/lu.rs:266-297:
 * out = I, then solve_mut(out)), and with nacu_dgetrf_batched before it
 * `m.try_inverse()` for n > 4 (src/linalg/inverse.rs:135-137).  Ainv + s*strideInv
 * (n x n) receives the inverse; LU and ipiv are read only.  info[s] = first
 * zero U_kk + 1 (nalgebra's None; Ainv then holds garbage, as nalgebra's
 * `out` may), or 0.  NACU_FLAG_EXACT: bit-identical to nalgebra's
 * solve_mut on the identity. */
int nacu_dgetri_batched(int n, const double* LU, int64_t strideA, const int32_t* ipiv, double* Ainv,
                        int64_t strideInv, int32_t* info, int batch, int flags, nacu_stream_t stream);

/* Batched triangular solves (n <= 128): B + s*strideB (n x nrhs) <- T_s^-1 B
 * (trans = 0) or T_s^-T B (trans = 1), T_s = T + s*strideT lower (upper = 0)
 * or upper (upper = 1) triangular, only that triangle read.  Replaces
 * Matrix::solve_{lower,upper}_triangular_mut (src/linalg/solve.rs:55-101,
 * 137-181), tr_solve_*_mut and ad_solve_*_mut (:233-283, 325-372; the same for
 * real scalars, dot form :374-442).  has_diag = 1 (lower, trans = 0 only):
 * solve_lower_triangular_with_diag_mut (:106-134), the diagonal never read,
 * `diag` assumed.  info[s] (nullable) = 1-based index of the zero diagonal
 * that stops the solve (nalgebra's false; B then holds partial results), or
 * 0.  NACU_FLAG_EXACT: bit-identical to nalgebra's arithmetic. */
int nacu_dtrsv_batched(int n, int nrhs, int upper, int trans, int has_diag, double diag, const double* T,
                       int64_t strideT, double* B, int64_t strideB, int32_t* info, int batch, int flags,
                       nacu_stream_t stream);

/* Bytes of device scratch nacu_dtrsv needs for an n x n triangle (the
 * per-block completion flags). */
size_t nacu_trsv_workspace_bytes(int n);

/* Triangular solve of one matrix of any order (the batched kernel above stops
 * at n = 128): B (n x nrhs, leading dimension ldb) <- T^-1 B (trans = 0) or
 * T^-T B (trans = 1), T (lda) lower (upper = 0) or upper (upper = 1), only
 * that triangle read; has_diag = 1 (lower, trans = 0 only):
 * solve_lower_triangular_with_diag_mut, `diag` assumed for the diagonal (0:
 * info = 1 and B untouched, solve.rs:115-117).  The same nalgebra functions
 * as nacu_dtrsv_batched (src/linalg/solve.rs:55-442).  *info (device) = the
 * 1-based index of the zero diagonal that stops nalgebra's solve in its
 * order (forward: the first, backward: the last; B then holds garbage), 0,
 * or -1000 when an internal wait between thread blocks ran out (does not
 * happen in normal operation).  FMA arithmetic: NACU_FLAG_EXACT returns -14. */
int nacu_dtrsv(int n, int nrhs, int upper, int trans, int has_diag, double diag, const double* T, int64_t lda,
               double* B, int64_t ldb, int32_t* info, void* workspace, size_t workspace_bytes, int flags,
               nacu_stream_t stream);

/* Fused factor + solve in one launch: `m.lu()` then `.solve(&b)`
 * (src/linalg/decomposition.rs:48-54, src/linalg/lu.rs:221-236). */
int nacu_dgesv_batched(int n, int nrhs, double* A, int64_t strideA, int32_t* ipiv, double* B,
                       int64_t strideB, int32_t* info, int batch, int flags, nacu_stream_t stream);

/* FP32 form of nacu_dgesv_batched (the factor step of mixed precision). */
int nacu_sgesv_batched(int n, int nrhs, float* A, int64_t strideA, int32_t* ipiv, float* B,
                       int64_t strideB, int32_t* info, int batch, int flags, nacu_stream_t stream);

/* ---- autotuned tiles of the ragged Cholesky launch --------------------------
 * When nacu_dposv_ragged / nacu_dpotrf_ragged / nacu_dpotrs_ragged get no
 * processing order (order == NULL), the library sorts the batch by order into
 * NACU_RAGGED_BUCKETS size buckets (upper orders 32, 64, 96, 128, 192, 256,
 * 384, 512) and runs one persistent launch per bucket, largest first, each
 * with the bucket's tile (threads per matrix, panel width) from the tuning
 * table and shared memory sized for the bucket.  No reference counterpart
 * (nalgebra factors one matrix per call). */
#define NACU_RAGGED_BUCKETS 8
#define NACU_RAGGED_TILES 4

/* The bucket bounds (NACU_RAGGED_BUCKETS ints) and the tiles (threads per
 * matrix and panel width, NACU_RAGGED_TILES ints each); any pointer may be NULL. */
int nacu_ragged_tuning_layout(int32_t* bucket_hi, int32_t* tile_threads, int32_t* tile_nb);

/* Installs / reads the process-wide tuning table (a tile index per bucket). */
int nacu_ragged_set_tuning(const int32_t* table, int nbuckets);
int nacu_ragged_get_tuning(int32_t* table, int nbuckets);

/* Times every tile on every bucket (per_bucket synthetic diagonally dominant
 * SPD systems with orders uniform in the bucket, nrhs right-hand sides; CUDA
 * events, best of three after a warm-up), installs the fastest tile per
 * bucket and returns the table and the times (ms_out: NACU_RAGGED_BUCKETS x
 * NACU_RAGGED_TILES, may be NULL).  Allocates and frees its own test batch;
 * synchronizes the stream. */
int nacu_ragged_autotune(int per_bucket, int nrhs, int flags, int32_t* table_out, double* ms_out,
                         nacu_stream_t stream);

/* ---- Cholesky (ragged batch, one persistent launch) ------------------------ */

/* Bytes of device scratch nacu_dposv_ragged needs (the work-queue head). */
size_t nacu_ragged_workspace_bytes(int count);

/* Factor, solve and log-determinant for `count` SPD matrices of uneven order.
 * Matrix s is ns[s] x ns[s] (ns[s] <= n_max <= 512) at A + a_offsets[s]
 * (lda = ns[s]); its nrhs right-hand sides are ns[s] x nrhs at
 * B + b_offsets[s] (ldb = ns[s]) and are overwritten by X.  Only the lower
 * triangle is read and written.  info[s] as above (-1: ns[s] out of range);
 * logdet[s] (nullable) = sum ln(L_ii^2), NaN when info != 0.  `order`
 * (nullable) is the processing order (largest matrices first balances the
 * persistent CTAs).  ns, a_offsets, b_offsets and order are device arrays.
 * Replaces Cholesky::new (src/linalg/cholesky.rs:196-272), Cholesky::solve_mut
 * (cholesky.rs:122-129, solve.rs:488-519, 697-755) and ln_determinant
 * (cholesky.rs:172-185). */
int nacu_dposv_ragged(int count, int n_max, const int32_t* ns, const int64_t* a_offsets, double* A,
                      int nrhs, const int64_t* b_offsets, double* B, int32_t* info, double* logdet,
                      const int32_t* order, void* workspace, size_t workspace_bytes, double substitute,
                      int flags, nacu_stream_t stream);

/* Factor + log-determinant only (no right-hand sides), same layout as
 * nacu_dposv_ragged: `m.cholesky()` and `.ln_determinant()`. */
int nacu_dpotrf_ragged(int count, int n_max, const int32_t* ns, const int64_t* a_offsets, double* A,
                       int32_t* info, double* logdet, const int32_t* order, void* workspace,
                       size_t workspace_bytes, double substitute, int flags, nacu_stream_t stream);

/* Solve from factors written by nacu_dpotrf_ragged (only matrices whose info
 * was 0 are meaningful): `chol.solve_mut(&mut b)` (src/linalg/cholesky.rs:122-129). */
int nacu_dpotrs_ragged(int count, int n_max, const int32_t* ns, const int64_t* a_offsets, const double* L,
                       int nrhs, const int64_t* b_offsets, double* B, const int32_t* order, void* workspace,
                       size_t workspace_bytes, int flags, nacu_stream_t stream);

/* One matrix, one plain launch: `m.cholesky()`, `.solve(&b)`,
 * `.ln_determinant()` for an n x n SPD matrix (n <= 512). */
int nacu_dposv(int n, double* A, int nrhs, double* B, int32_t* info, double* logdet, double substitute,
               int flags, nacu_stream_t stream);

/* ---- Cholesky factor updates (batched, n <= 128) ---------------------------- */

/* Cholesky::rank_one_update (src/linalg/cholesky.rs:277-285, 410-449): the
 * factor L_s = L + s*strideL (n x n, lower part) becomes the factor of
 * L_s L_s^T + sigma[s] x_s x_s^T, in place; X + s*strideX (n values) is read
 * only (nalgebra updates a clone).  sigma: device array of batch values. */
int nacu_dchol_rank1_update_batched(int n, double* L, int64_t strideL, const double* X, int64_t strideX,
                                    const double* sigma, int batch, int flags, nacu_stream_t stream);

/* Cholesky::remove_column (src/linalg/cholesky.rs:365-399): Lout_s
 * ((n-1) x (n-1)) = the factor of A_s without row and column j, from L_s (its
 * strict upper part copied block by block, as nalgebra copies its views). */
int nacu_dchol_remove_column_batched(int n, const double* L, int64_t strideL, int j, double* Lout, int64_t strideOut,
                                     int batch, int flags, nacu_stream_t stream);

/* Cholesky::insert_column (src/linalg/cholesky.rs:287-357): Lout_s
 * ((n+1) x (n+1)) = the factor of A_s with col_s (n+1 values, col + s*strideCol)
 * inserted as row and column j (n <= 127).  info[s] (nullable) = 1 where the
 * lower solve of the new row meets a zero diagonal (nalgebra's assertion),
 * else 0. */
int nacu_dchol_insert_column_batched(int n, const double* L, int64_t strideL, int j, const double* col,
                                     int64_t strideCol, double* Lout, int64_t strideOut, int32_t* info, int batch,
                                     int flags, nacu_stream_t stream);

/* ---- Cholesky, mixed precision (FP32 factor, FP64 refinement) ------------- */

/* Workspace bytes of nacu_dposv_ragged_mixed: queue heads and a fallback
 * list (4 bytes per matrix), then 8 bytes per matrix element (room for the
 * FP32 factor, or for the FP64 fallback factor). */
size_t nacu_mixed_workspace_bytes(int count, int64_t total_matrix_elements);

/* The precision form of nacu_dposv_ragged: same ragged layout, but A and B
 * are read-only and the solutions go to X (X + b_offsets[s], ns[s] x nrhs,
 * nrhs <= 4).  Each matrix is factored in FP32 and its solutions refined with
 * FP64 residuals r = b - A x until the normwise backward error
 * ||r||_inf / (||A||_inf ||x||_inf + ||b||_inf) <= tol_units * n * eps64
 * (tol_units <= 0: 1.0), at most max_iter residuals (<= 0: 10).  A matrix that
 * is not SPD in FP32 or whose refinement does not converge is refactored and
 * solved in FP64 in the workspace.  info[s]: 0 ok, k = not SPD (as
 * nacu_dposv_ragged); iters[s] (nullable): residuals computed, negative when
 * the FP64 fallback was used.  total_matrix_elements = sum ns[s]^2 (the extent
 * of A).  No reference counterpart: nalgebra has no mixed precision; it
 * replaces `m.cholesky()` + `.solve(&b)` (src/linalg/cholesky.rs:221-272,
 * 122-143) where FP64-accurate solutions, not the factor, are wanted. */
int nacu_dposv_ragged_mixed(int count, int n_max, const int32_t* ns, const int64_t* a_offsets, const double* A,
                            int nrhs, const int64_t* b_offsets, const double* B, double* X, int32_t* info,
                            int32_t* iters, const int32_t* order, int64_t total_matrix_elements, void* workspace,
                            size_t workspace_bytes, double tol_units, int max_iter, double substitute, int flags,
                            nacu_stream_t stream);

/* The same solve from host memory, pipelined: every array (ns, offsets, A,
 * B, X, info, iters) is a host array in the layout of nacu_dposv_ragged_mixed,
 * with non-decreasing offsets.  The batch is cut into `chunks` parts of about
 * equal bytes (<= 0: 8; at most 64); while one part is solved on the GPU the
 * next is copied in and the previous one copied out, on internal streams of
 * the library forked from `stream` and joined back to it before the call
 * returns (the results are in host memory once `stream` has been
 * synchronized).  Page-locked host memory gives the overlap; pageable memory
 * works but serializes the copies.  Each system's results are bit-identical to
 * nacu_dposv_ragged_mixed's.  workspace: device memory of
 * nacu_mixed_host_workspace_bytes bytes (same arguments), 256-byte aligned;
 * calls must not be issued concurrently from several host threads on one
 * device.  It is the form a host-resident caller uses in place of
 * `m.cholesky()` + `.solve(&b)` per matrix (src/linalg/cholesky.rs:221-272,
 * 122-143).  Returns 0 bytes for invalid arguments. */
size_t nacu_mixed_host_workspace_bytes(int count, int n_max, const int32_t* ns, const int64_t* a_offsets,
                                       const int64_t* b_offsets, int nrhs, int chunks);
int nacu_dposv_ragged_mixed_host(int count, int n_max, const int32_t* ns, const int64_t* a_offsets, const double* A,
                                 int nrhs, const int64_t* b_offsets, const double* B, double* X, int32_t* info,
                                 int32_t* iters, int chunks, void* workspace, size_t workspace_bytes,
                                 double tol_units, int max_iter, double substitute, int flags, nacu_stream_t stream);

/* ---- Adjoint of the Cholesky solve and log-determinant (batched, n <= 128) - */

/* Forward: for `batch` SPD matrices A + s*strideA (lower triangle read),
 * X[s*n..] = A^-1 B[s*n..] and logdet[s] = sum ln(L_ii^2)
 * (src/linalg/cholesky.rs:221-272, 122-143, 172-185).  L (nullable) receives
 * the factor in its lower triangle (the FP64 form leaves A's values above the
 * diagonal, as nalgebra's factor does; the FP32 form writes zeros there): the
 * "store" form keeps it for the backward pass; pass NULL to keep nothing (the
 * "recompute" form).  info is required in the FP64 store form.  No
 * reference counterpart for the adjoint itself: nalgebra has no autodiff. */
int nacu_dposv_logdet_forward(int n, const double* A, int64_t strideA, const double* B, double* X, double* L,
                              double* logdet, int32_t* info, int batch, nacu_stream_t stream);
int nacu_sposv_logdet_forward(int n, const float* A, int64_t strideA, const float* B, float* X, float* L,
                              float* logdet, int32_t* info, int batch, nacu_stream_t stream);

/* Reverse mode: given the cotangents W = dl/dx (n per system) and G =
 * dl/dlogdet (one per system; NULL: all 1, i.e. l = sum_s w_s^T x_s +
 * logdet A_s), db[s*n..] = A^-T w = dl/db and dA's lower triangle = dl/dA with
 * respect to the lower-triangle entries that nalgebra reads
 * (dA_ii = -v_i x_i + g (A^-1)_ii, dA_ij = -(v_i x_j + v_j x_i) + 2 g (A^-1)_ij
 * for i > j, v = A^-1 w; zeros above).  AL holds the stored factor L
 * (recompute = 0) or the original A (recompute = 1: the factor is rebuilt,
 * trading n^3/3 flops for n^2 stored values per matrix). */
int nacu_dposv_logdet_backward(int n, const double* AL, int64_t strideA, int recompute, const double* X,
                               const double* W, const double* G, double* dA, double* db, int32_t* info,
                               int batch, nacu_stream_t stream);
int nacu_sposv_logdet_backward(int n, const float* AL, int64_t strideA, int recompute, const float* X,
                               const float* W, const float* G, float* dA, float* db, int32_t* info, int batch,
                               nacu_stream_t stream);

/* ---- Householder QR and least squares (batched, tall-skinny) ------------- */

/* Bytes of device scratch nacu_dgels_batched needs (the work-queue head). */
size_t nacu_qr_workspace_bytes(int count);

/* Householder QR of `count` tall matrices with n <= 128 columns and
 * ms[s] >= n rows (ms[s] <= m_max <= 2048), A + a_offsets[s] (lda = ms[s]),
 * factored in place into nalgebra's QR layout: unit reflection axes on and
 * below the diagonal, R strictly above it, and diag[s*n + i] = the signed
 * diagonal (R_ii = |diag_i|), exactly nalgebra's sign convention
 * (src/linalg/qr.rs:55-76, householder.rs:19-85, reflection.rs:70-83).
 * With b_offsets/B set, each B + b_offsets[s] (ms[s] x 1) is replaced by
 * Q^T b (qr.rs:157-171) and X + s*n receives the least-squares solution
 * argmin ||A x - b|| (R[0:n,0:n] x = (Q^T b)[0:n], as
 * nalgebra-lapack/src/qr_util.rs:167-239).  info[s] (nullable): 0 ok,
 * k = first zero R_kk (rank deficient), -1 = ms[s] out of range.
 * NACU_FLAG_EXACT is not available for QR (returns -15). */
int nacu_dgels_batched(int count, int n, int m_max, const int32_t* ms, const int64_t* a_offsets, double* A,
                       const int64_t* b_offsets, double* B, double* X, double* diag, int32_t* info,
                       const int32_t* order, void* workspace, size_t workspace_bytes, int flags,
                       nacu_stream_t stream);

/* Largest batch nacu_dposv_ragged_noalloc accepts. */
#define NACU_RAGGED_NOALLOC_MAX_COUNT 65536

/* nacu_dposv_ragged without any caller scratch, for hosts that cannot
 * allocate device memory when they solve (allocator callbacks, real-time or
 * certified hosts that allocate only at start-up, plugins whose framework owns
 * every allocation).  No counterpart in nalgebra: it exists for callers of
 * this library.  Scratch (the work-queue head and the largest-first order) is
 * a fixed array of 4 * (1 + 65536) bytes (256 KiB + 4 B) inside the
 * library's device image, held on every GPU that loads the library until the
 * process exits.  count <= 65536, else the call returns -1 with a message.
 * The first call on each device looks up the array's device address
 * (cudaGetSymbolAddress) and caches it for the process; make that first call
 * before any stream capture.  cudaDeviceReset unloads the module and leaves
 * that cached address stale: do not call this entry point on a device after
 * resetting it.  All calls share the one array: calls that overlap on
 * the GPU race on it and must be ordered by the caller.  Arguments and results
 * are those of nacu_dposv_ragged; allocates nothing. */
int nacu_dposv_ragged_noalloc(int count, int n_max, const int32_t* ns, const int64_t* a_offsets, double* A,
                              int nrhs, const int64_t* b_offsets, double* B, int32_t* info, double* logdet,
                              double substitute, int flags, nacu_stream_t stream);

/* ---- LU of one large matrix (blocked, multi-SM) ---------------------------- */

/* Workspace bytes of nacu_dgetrf and nacu_dgetrs (the panel's pivot exchange
 * area; the triangular solves' block flags). */
size_t nacu_getrf_workspace_bytes(int n);

/* LU with partial pivoting of one n x n matrix (column-major, lda), in place,
 * nalgebra's packed L\U with per-step pivots ipiv[0..n) (src/linalg/lu.rs:93-122;
 * icamax rule src/base/min_max.rs:221-240; a zero column is skipped,
 * lu.rs:107-110).  *info (device) = 0, or the first skipped column + 1.
 * Look-ahead: the work forks from `stream` onto two internal streams of the
 * library (per device; the panel chain at the highest stream priority, the
 * bulk of each trailing update concurrently) and joins back before the call
 * returns, so it is ordered like any work on `stream` and can be captured into
 * a CUDA graph.  Calls that use the internal streams (this one,
 * nacu_dgesv_mixed_ir) must not be issued concurrently from several host
 * threads on one device. */
int nacu_dgetrf(int n, double* A, int64_t lda, int32_t* ipiv, int32_t* info, void* workspace, size_t workspace_bytes,
                nacu_stream_t stream);

/* Solve A x = b in place in b from nacu_dgetrf factors
 * (src/linalg/lu.rs:242-260); *info = first zero U_kk + 1, or 0 (-1000: an
 * internal wait between thread blocks ran out; the result is not valid).
 * workspace: nacu_getrf_workspace_bytes(n) bytes, not shared with a call in
 * flight on another stream. */
int nacu_dgetrs(int n, const double* LU, int64_t lda, const int32_t* ipiv, double* b, int32_t* info, void* workspace,
                size_t workspace_bytes, nacu_stream_t stream);

/* Test hook, no counterpart in nalgebra: nacu_dgetrs in which row block
 * `skip_block` (0-based, 64 rows each) of the unit-lower solve never raises
 * its ready flag, and every flag wait gives up after `poll_limit` polls
 * (1 .. 2^22).  The blocks after it run out of their bounded wait, set *info
 * to -1000 and return, so the call ends with the context usable: the failure
 * path of the bounded waits, exercised without faulting or hanging a GPU. */
int nacu_test_dgetrs_flag_timeout(int n, const double* LU, int64_t lda, const int32_t* ipiv, double* b,
                                  int32_t* info, int skip_block, int poll_limit, void* workspace,
                                  size_t workspace_bytes, nacu_stream_t stream);

/* Test hook, no counterpart in nalgebra: out[i] = the reciprocal the FMA
 * forms use on their serial pivot paths (rcp.approx.ftz.f64 refined by two
 * Newton-Raphson steps; division outside |d| in [2^-1000, 2^1000]) for
 * d[0..n) in device memory, so a test can hold it to IEEE 1/d. */
int nacu_test_rcp(int n, const double* d, double* out, nacu_stream_t stream);

/* Workspace bytes of nacu_dgesv_mixed_ir (FP32 copy of A, split-GEMM slices,
 * vectors, and an FP64 copy of A for the fallback). */
size_t nacu_gesv_mixed_workspace_bytes(int n);

/* Mixed-precision solve of one large system A x = b (A, b read-only, FP64):
 * FP32 LU with partial pivoting (BF16-split tensor-core trailing updates),
 * then FP64 iterative refinement r = b - A x, x += (LU)^-1 r until the normwise
 * backward error ||r||_inf / (||A||_inf ||x||_inf + ||b||_inf) <= tol_units * n *
 * eps64 (tol_units <= 0: 1), at most max_iter steps (<= 0: 30).  When the
 * classical refinement stagnates (u32 * cond(A) near 1), GMRES-IR takes over
 * (Carson & Higham 2018): each correction solves M^-1 A d = M^-1 r by
 * restarted GMRES with FP64 vectors, M = the FP32 LU factors (applied in
 * FP64) as the preconditioner.  When FP32 cannot factor A, when classical
 * refinement diverges outright (u32 * cond(A) well above 1), or when GMRES-IR
 * makes no progress, A is refactored in FP64.  *fallback_out: 0 classical refinement, 2 GMRES-IR,
 * 1 FP64 refactorization; *iters_out: FP64 residuals formed.
 * Synchronous: *iters_out, *berr_out, *fallback_out are host values.  No
 * reference counterpart (nalgebra has no mixed precision); it replaces
 * `m.lu().solve(&b)` (src/linalg/lu.rs:93-122, 221-260) when an FP64-accurate
 * solution, not the factor, is wanted.  The FP32 factorization forks onto the
 * internal streams as nacu_dgetrf does. */
int nacu_dgesv_mixed_ir(int n, const double* A, int64_t lda, const double* b, double* x, double tol_units,
                        int max_iter, int* iters_out, double* berr_out, int* fallback_out, void* workspace,
                        size_t workspace_bytes, nacu_stream_t stream);

/* ---- GEMM ------------------------------------------------------------------ */

/* C = alpha * A * B + beta * C, FP64, column-major (A m x k, B k x n, C m x n),
 * `Matrix::gemm` (src/base/blas.rs:729-746, blas_uninit.rs:187-333).
 * beta == 0: C is never read. */
int nacu_dgemm(int m, int n, int k, double alpha, const double* A, int64_t lda, const double* B, int64_t ldb,
               double beta, double* C, int64_t ldc, nacu_stream_t stream);

/* Many independent products in one launch: C_s = alpha * A_s * B_s + beta *
 * C_s for s < batch, each m x k by k x n, column-major with leading dimensions
 * lda / ldb / ldc, product s at A + s*strideA, B + s*strideB, C + s*strideC.
 * The batched form of `&a * &b` (src/base/ops.rs:566-570: gemm_uninit with
 * alpha = 1, beta = 0) and of `Matrix::gemm` (src/base/blas.rs:729-746).
 * beta == 0: C is never read.  NACU_FLAG_EXACT: nalgebra's gemv order of
 * gemm_uninit (src/base/blas_uninit.rs:127-176, 320-332; the order nalgebra
 * uses when a dimension is <= 5 or the sizes are static), bit for bit;
 * default: one FMA per step, alpha and beta applied at the end.  Any m, n, k
 * (tiles of up to 64 x 64 per CTA). */
int nacu_dgemm_batched(int m, int n, int k, double alpha, const double* A, int64_t lda, int64_t strideA,
                       const double* B, int64_t ldb, int64_t strideB, double beta, double* C, int64_t ldc,
                       int64_t strideC, int batch, int flags, nacu_stream_t stream);

/* Workspace bytes of nacu_dgemm_split_bf16 (BF16 slices of A and B, padded to
 * the 128 x 256 x 64 tiles, and the row / column exponents). */
size_t nacu_gemm_split_workspace_bytes(int m, int n, int k);

/* The precision form of nacu_dgemm on the tensor cores: rows of A and columns
 * of B scaled by powers of two, split into `slices` (1..3) BF16 parts, the
 * slice products p + q < slices accumulated in FP32 by tcgen05.mma, the result
 * rescaled and combined with beta * C in FP64.  FP32-class accuracy (3 slices:
 * ~1e-7 relative to |A||B|).  No reference counterpart (nalgebra's gemm is
 * FP64 only).  workspace must be 1024-byte aligned. */
int nacu_dgemm_split_bf16(int m, int n, int k, double alpha, const double* A, int64_t lda, const double* B,
                          int64_t ldb, double beta, double* C, int64_t ldc, int slices, void* workspace,
                          size_t workspace_bytes, nacu_stream_t stream);

/* 1 when a split-GEMM kernel gave up waiting on a pipeline barrier (its
 * results are then invalid), else 0; synchronous. */
int nacu_split_gemm_error(int* flag_out);

/* ---- measurement helpers ---------------------------------------------------- */

/* FP64 FMA throughput probe: runs a fixed DFMA-chain kernel over the whole GPU
 * and returns the achieved FP64 FLOP/s through *flops (synchronous; used as
 * the FP64 roofline denominator). */
int nacu_probe_fp64_peak(double* flops);

#ifdef __cplusplus
}
#endif

#endif /* NALGEBRA_CUDA_H */
