//! nalgebra's dense solve API on one GB300 GPU.
//!
//! The types keep nalgebra's method names (`lu()`, `cholesky()`, `qr()`,
//! `solve()`, `gemm(alpha, a, b, beta)`) over device-resident column-major f64
//! matrices, and every numerical operation is a hand-written sm_103a kernel of
//! `libnalgebra_cuda` reached through its C ABI (`ffi`).  There is no CPU
//! fallback.  Conventions carried over from nalgebra:
//! - `lu()` / `cholesky()` / `qr()` consume the matrix and factor it in place
//!   (src/linalg/lu.rs:93, cholesky.rs:221, qr.rs:55);
//! - singular / non-SPD results are `None` (lu.rs:221-236, cholesky.rs:196);
//! - shape mismatches panic, as nalgebra's assertions do;
//! - the pivots come back as nalgebra's `PermutationSequence`.
//!
//! Beside the drop-in (plain FP64) form stand the chosen forms with no
//! nalgebra counterpart: the mixed-precision refined solves
//! (`DeviceMatrix::solve_refined`, `DeviceBatch::cholesky_solve_refined`), the
//! ragged batched launch (`DeviceBatch`), and the reverse-mode adjoint of the
//! batched solve + log-determinant (`SolveLogdet::forward` / `backward`).
pub mod ffi;
mod cuda;

use std::ffi::CStr;
use std::marker::PhantomData;
use std::os::raw::{c_int, c_void};

use nalgebra::{DMatrix, Dyn, PermutationSequence};

pub use ffi::{NACU_FLAG_EXACT, NACU_FLAG_NO_FACTORS, NACU_FLAG_SUBSTITUTE, NACU_FLAG_VERIFY};

fn check(rc: c_int) {
    // rc < 0: argument -rc was invalid (nalgebra panics on shape errors the same way)
    if rc != 0 {
        let msg = unsafe { CStr::from_ptr(ffi::nacu_last_error()) }.to_string_lossy().into_owned();
        panic!("nalgebra-cuda: {msg}");
    }
}

/// A device allocation of `len` values of `T` (freed on drop).
pub struct DeviceBuffer<T> {
    ptr: *mut T,
    len: usize,
    _t: PhantomData<T>,
}

impl<T: Copy> DeviceBuffer<T> {
    pub fn zeroed(len: usize) -> Self {
        let mut p: *mut c_void = std::ptr::null_mut();
        let bytes = len.max(1) * std::mem::size_of::<T>();
        unsafe {
            cuda::check(cuda::nacu_malloc(&mut p, bytes), "nacu_malloc");
            cuda::check(cuda::nacu_memset(p, 0, bytes, std::ptr::null_mut()), "nacu_memset");
        }
        DeviceBuffer { ptr: p as *mut T, len, _t: PhantomData }
    }
    pub fn from_slice(h: &[T]) -> Self {
        let b = Self::zeroed(h.len());
        unsafe {
            cuda::check(cuda::nacu_memcpy(b.ptr as *mut c_void, h.as_ptr() as *const c_void,
                                          h.len() * std::mem::size_of::<T>(), std::ptr::null_mut()),
                        "nacu_memcpy");
        }
        b
    }
    /// Synchronous copy to the host (waits for the work on the legacy stream).
    pub fn to_vec(&self) -> Vec<T> {
        let mut v: Vec<T> = Vec::with_capacity(self.len);
        unsafe {
            cuda::check(cuda::nacu_memcpy(v.as_mut_ptr() as *mut c_void, self.ptr as *const c_void,
                                          self.len * std::mem::size_of::<T>(), std::ptr::null_mut()),
                        "nacu_memcpy");
            cuda::check(cuda::nacu_stream_synchronize(std::ptr::null_mut()), "nacu_stream_synchronize");
            v.set_len(self.len);
        }
        v
    }
    pub fn clone_device(&self) -> Self {
        let b = Self::zeroed(self.len);
        unsafe {
            cuda::check(cuda::nacu_memcpy(b.ptr as *mut c_void, self.ptr as *const c_void,
                                          self.len * std::mem::size_of::<T>(), std::ptr::null_mut()),
                        "nacu_memcpy");
        }
        b
    }
    pub fn as_ptr(&self) -> *const T {
        self.ptr
    }
    pub fn as_mut_ptr(&mut self) -> *mut T {
        self.ptr
    }
    pub fn len(&self) -> usize {
        self.len
    }
}

impl<T> Drop for DeviceBuffer<T> {
    fn drop(&mut self) {
        unsafe {
            cuda::nacu_free(self.ptr as *mut c_void);
        }
    }
}

fn sync() {
    unsafe { cuda::check(cuda::nacu_stream_synchronize(std::ptr::null_mut()), "nacu_stream_synchronize") };
}

/// An nrows x ncols f64 matrix on the GPU, column-major like nalgebra's
/// `DMatrix` (src/base/vec_storage.rs:28-32).
pub struct DeviceMatrix {
    data: DeviceBuffer<f64>,
    nrows: usize,
    ncols: usize,
}

impl DeviceMatrix {
    pub fn from_dmatrix(m: &DMatrix<f64>) -> Self {
        DeviceMatrix { data: DeviceBuffer::from_slice(m.as_slice()), nrows: m.nrows(), ncols: m.ncols() }
    }
    pub fn zeros(nrows: usize, ncols: usize) -> Self {
        DeviceMatrix { data: DeviceBuffer::zeroed(nrows * ncols), nrows, ncols }
    }
    pub fn to_dmatrix(&self) -> DMatrix<f64> {
        DMatrix::from_vec(self.nrows, self.ncols, self.data.to_vec())
    }
    pub fn nrows(&self) -> usize {
        self.nrows
    }
    pub fn ncols(&self) -> usize {
        self.ncols
    }
    pub fn is_square(&self) -> bool {
        self.nrows == self.ncols
    }
    pub fn clone_owned(&self) -> Self {
        DeviceMatrix { data: self.data.clone_device(), nrows: self.nrows, ncols: self.ncols }
    }

    fn trsv(&self, b: &mut DeviceMatrix, upper: bool, trans: bool, diag: Option<f64>) -> bool {
        let n = self.nrows;
        assert!(self.is_square() && b.nrows == n, "triangular solve dimension mismatch");
        let mut info = DeviceBuffer::<i32>::zeroed(1);
        let (hd, d) = (diag.is_some() as c_int, diag.unwrap_or(0.0));
        if n <= 128 {
            check(unsafe {
                ffi::nacu_dtrsv_batched(n as c_int, b.ncols as c_int, upper as c_int, trans as c_int, hd, d,
                                        self.data.as_ptr(), (n * n) as i64, b.data.as_mut_ptr(),
                                        (n * b.ncols) as i64, info.as_mut_ptr(), 1, 0, std::ptr::null_mut())
            });
        } else {
            let bytes = unsafe { ffi::nacu_trsv_workspace_bytes(n as c_int) };
            let mut ws = DeviceBuffer::<u8>::zeroed(bytes);
            check(unsafe {
                ffi::nacu_dtrsv(n as c_int, b.ncols as c_int, upper as c_int, trans as c_int, hd, d,
                                self.data.as_ptr(), n as i64, b.data.as_mut_ptr(), n as i64, info.as_mut_ptr(),
                                ws.as_mut_ptr() as *mut c_void, bytes, 0, std::ptr::null_mut())
            });
        }
        info.to_vec()[0] == 0
    }

    /// `Matrix::solve_lower_triangular_mut` (src/linalg/solve.rs:55-101).
    pub fn solve_lower_triangular_mut(&self, b: &mut DeviceMatrix) -> bool {
        self.trsv(b, false, false, None)
    }
    /// `Matrix::solve_upper_triangular_mut` (solve.rs:137-181).
    pub fn solve_upper_triangular_mut(&self, b: &mut DeviceMatrix) -> bool {
        self.trsv(b, true, false, None)
    }
    /// `Matrix::tr_solve_lower_triangular_mut` (solve.rs:233-256); `ad_` is the same for f64.
    pub fn tr_solve_lower_triangular_mut(&self, b: &mut DeviceMatrix) -> bool {
        self.trsv(b, false, true, None)
    }
    /// `Matrix::tr_solve_upper_triangular_mut` (solve.rs:258-283).
    pub fn tr_solve_upper_triangular_mut(&self, b: &mut DeviceMatrix) -> bool {
        self.trsv(b, true, true, None)
    }
    /// `Matrix::solve_lower_triangular_with_diag_mut` (solve.rs:106-134).
    pub fn solve_lower_triangular_with_diag_mut(&self, b: &mut DeviceMatrix, diag: f64) -> bool {
        self.trsv(b, false, false, Some(diag))
    }
    /// `Matrix::solve_lower_triangular` (solve.rs:15-34): a new matrix, or None.
    pub fn solve_lower_triangular(&self, b: &DeviceMatrix) -> Option<DeviceMatrix> {
        let mut res = b.clone_owned();
        if self.solve_lower_triangular_mut(&mut res) { Some(res) } else { None }
    }
    /// `Matrix::solve_upper_triangular` (solve.rs:36-53).
    pub fn solve_upper_triangular(&self, b: &DeviceMatrix) -> Option<DeviceMatrix> {
        let mut res = b.clone_owned();
        if self.solve_upper_triangular_mut(&mut res) { Some(res) } else { None }
    }

    /// `Matrix::lu` (src/linalg/decomposition.rs:48-54): LU with partial
    /// pivoting, factors in place (the batched kernel up to n = 128, the
    /// blocked multi-SM factorization above).
    pub fn lu(mut self) -> DeviceLU {
        assert!(self.is_square(), "nalgebra-cuda: LU of a square matrix");
        let n = self.nrows as c_int;
        let mut ipiv = DeviceBuffer::<i32>::zeroed(self.nrows);
        let mut info = DeviceBuffer::<i32>::zeroed(1);
        let mut ws = None;
        if n <= 128 {
            check(unsafe {
                ffi::nacu_dgetrf_batched(n, self.data.as_mut_ptr(), (n * n) as i64, ipiv.as_mut_ptr(),
                                         info.as_mut_ptr(), 1, 0, std::ptr::null_mut())
            });
        } else {
            let bytes = unsafe { ffi::nacu_getrf_workspace_bytes(n) };
            let mut w = DeviceBuffer::<u8>::zeroed(bytes);
            check(unsafe {
                ffi::nacu_dgetrf(n, self.data.as_mut_ptr(), n as i64, ipiv.as_mut_ptr(), info.as_mut_ptr(),
                                 w.as_mut_ptr() as *mut c_void, bytes, std::ptr::null_mut())
            });
            ws = Some(w);
        }
        DeviceLU { lu: self, ipiv, info, ws }
    }

    /// `Matrix::cholesky` (src/linalg/decomposition.rs:257-262): `None` when
    /// the matrix is not SPD (cholesky.rs:237-268); n <= 512.
    pub fn cholesky(mut self) -> Option<DeviceCholesky> {
        assert!(self.is_square(), "nalgebra-cuda: Cholesky of a square matrix");
        let n = self.nrows as c_int;
        let mut info = DeviceBuffer::<i32>::zeroed(1);
        let mut logdet = DeviceBuffer::<f64>::zeroed(1);
        check(unsafe {
            ffi::nacu_dposv(n, self.data.as_mut_ptr(), 0, std::ptr::null_mut(), info.as_mut_ptr(),
                            logdet.as_mut_ptr(), 0.0, 0, std::ptr::null_mut())
        });
        if info.to_vec()[0] != 0 {
            return None;
        }
        Some(DeviceCholesky { l: self, logdet: logdet.to_vec()[0] })
    }

    /// `Matrix::qr` (src/linalg/decomposition.rs:56-62): `QR::new` in place.
    /// Square n <= 128: the shared-memory batched kernel; any other shape
    /// (larger, tall or wide): one launch per Householder step (`nacu_dqr`).
    pub fn qr(mut self) -> DeviceQR {
        let (m, n) = (self.nrows, self.ncols);
        let k = m.min(n);
        let mut diag = DeviceBuffer::<f64>::zeroed(k.max(1));
        if m == n && n <= 128 {
            let mut info = DeviceBuffer::<i32>::zeroed(1);
            check(unsafe {
                ffi::nacu_dqr_batched(n as c_int, 0, self.data.as_mut_ptr(), (n * n) as i64, diag.as_mut_ptr(),
                                      std::ptr::null_mut(), 0, info.as_mut_ptr(), 1, 0, std::ptr::null_mut())
            });
            let invertible = info.to_vec()[0] == 0;
            return DeviceQR { a: self, diag, invertible, large: false };
        }
        check(unsafe {
            ffi::nacu_dqr(m as c_int, n as c_int, self.data.as_mut_ptr(), m.max(1) as i64, diag.as_mut_ptr(), 0,
                          std::ptr::null_mut())
        });
        // qr.rs:281-292: square, and no diag entry zero
        let invertible = m == n && diag.to_vec()[..k].iter().all(|d| *d != 0.0);
        DeviceQR { a: self, diag, invertible, large: true }
    }

    /// `Matrix::gemm` (src/base/blas.rs:729-746): self = alpha a b + beta self.
    pub fn gemm(&mut self, alpha: f64, a: &DeviceMatrix, b: &DeviceMatrix, beta: f64) {
        assert!(a.ncols == b.nrows, "gemm: dimensions mismatch for multiplication.");
        assert!(self.nrows == a.nrows && self.ncols == b.ncols, "gemm: dimensions mismatch for addition.");
        let (m, n, k) = (a.nrows as c_int, b.ncols as c_int, a.ncols as c_int);
        check(unsafe {
            ffi::nacu_dgemm(m, n, k, alpha, a.data.as_ptr(), m.max(1) as i64, b.data.as_ptr(), k.max(1) as i64, beta,
                            self.data.as_mut_ptr(), m.max(1) as i64, std::ptr::null_mut())
        });
    }

    /// The precision form for one system (no nalgebra counterpart): FP32 LU
    /// with BF16-split tensor-core updates, FP64 refinement (GMRES-IR where
    /// classical refinement stalls) to backward error <= n * eps64, FP64
    /// fallback.  `self` and `b` are left unchanged.
    pub fn solve_refined(&self, b: &DeviceMatrix) -> (DeviceMatrix, RefineInfo) {
        assert!(self.is_square() && b.nrows == self.nrows && b.ncols == 1, "one n x n system, one right-hand side");
        let n = self.nrows as c_int;
        let mut x = DeviceMatrix::zeros(self.nrows, 1);
        let bytes = unsafe { ffi::nacu_gesv_mixed_workspace_bytes(n) };
        let mut ws = DeviceBuffer::<u8>::zeroed(bytes);
        let (mut iters, mut berr, mut path) = (0 as c_int, 0.0f64, 0 as c_int);
        check(unsafe {
            ffi::nacu_dgesv_mixed_ir(n, self.data.as_ptr(), n as i64, b.data.as_ptr(), x.data.as_mut_ptr(), 1.0, 0,
                                     &mut iters, &mut berr, &mut path, ws.as_mut_ptr() as *mut c_void, bytes,
                                     std::ptr::null_mut())
        });
        (x, RefineInfo { iters: iters as usize, backward_error: berr, path: path as u8 })
    }
}

/// How a refined solve ended: `path` 0 classical refinement, 2 GMRES-IR, 1 the
/// FP64 refactorization.
#[derive(Debug, Clone, Copy)]
pub struct RefineInfo {
    pub iters: usize,
    pub backward_error: f64,
    pub path: u8,
}

fn permutation_from_ipiv(ipiv: &[i32]) -> PermutationSequence<Dyn> {
    let mut p = PermutationSequence::identity(ipiv.len());
    for (i, &piv) in ipiv.iter().enumerate() {
        p.append_permutation(i, piv as usize); // nalgebra skips i == piv itself
    }
    p
}

/// `LU` (src/linalg/lu.rs:32-38) with its factors on the device.
pub struct DeviceLU {
    lu: DeviceMatrix,
    ipiv: DeviceBuffer<i32>,
    info: DeviceBuffer<i32>,
    ws: Option<DeviceBuffer<u8>>,
}

impl DeviceLU {
    /// `LU::solve_mut` (src/linalg/lu.rs:242-260): false when some U_ii == 0.
    pub fn solve_mut(&mut self, b: &mut DeviceMatrix) -> bool {
        let n = self.lu.nrows as c_int;
        assert!(b.nrows == self.lu.nrows, "LU solve matrix dimension mismatch.");
        let mut info = DeviceBuffer::<i32>::zeroed(1);
        if let Some(ws) = self.ws.as_mut() {
            let bytes = ws.len();
            for c in 0..b.ncols {
                check(unsafe {
                    ffi::nacu_dgetrs(n, self.lu.data.as_ptr(), n as i64, self.ipiv.as_ptr(),
                                     b.data.as_mut_ptr().add(c * b.nrows), info.as_mut_ptr(),
                                     ws.as_mut_ptr() as *mut c_void, bytes, std::ptr::null_mut())
                });
                if info.to_vec()[0] != 0 {
                    return false;
                }
            }
            return true;
        }
        check(unsafe {
            ffi::nacu_dgetrs_batched(n, b.ncols as c_int, self.lu.data.as_mut_ptr(), (n * n) as i64,
                                     self.ipiv.as_mut_ptr(), b.data.as_mut_ptr(), (b.nrows * b.ncols) as i64,
                                     info.as_mut_ptr(), 1, 0, std::ptr::null_mut())
        });
        info.to_vec()[0] == 0
    }
    /// `LU::solve` (src/linalg/lu.rs:221-236): `None` when singular.
    pub fn solve(&mut self, b: &DeviceMatrix) -> Option<DeviceMatrix> {
        let mut res = b.clone_owned();
        if self.solve_mut(&mut res) { Some(res) } else { None }
    }
    /// `LU::p`: nalgebra's PermutationSequence of the recorded row swaps.
    pub fn p(&self) -> PermutationSequence<Dyn> {
        permutation_from_ipiv(&self.ipiv.to_vec())
    }
    pub fn is_invertible(&self) -> bool {
        self.info.to_vec()[0] == 0
    }
    /// `LU::determinant` (src/linalg/lu.rs:301-314).
    pub fn determinant(&self) -> f64 {
        let lu = self.lu.to_dmatrix();
        let mut d = 1.0;
        for i in 0..lu.nrows() {
            d *= lu[(i, i)];
        }
        d * self.p().determinant::<f64>()
    }
    /// `LU::try_inverse` (src/linalg/lu.rs:266-297), n <= 128.
    pub fn try_inverse(&self) -> Option<DeviceMatrix> {
        let n = self.lu.nrows as c_int;
        assert!(n <= 128, "try_inverse: n <= 128 (the batched kernels)");
        let mut out = DeviceMatrix::zeros(self.lu.nrows, self.lu.nrows);
        let mut info = DeviceBuffer::<i32>::zeroed(1);
        check(unsafe {
            ffi::nacu_dgetri_batched(n, self.lu.data.as_ptr(), (n * n) as i64, self.ipiv.as_ptr(),
                                     out.data.as_mut_ptr(), (n * n) as i64, info.as_mut_ptr(), 1, 0,
                                     std::ptr::null_mut())
        });
        if info.to_vec()[0] == 0 { Some(out) } else { None }
    }
}

/// `Cholesky` (src/linalg/cholesky.rs:28-33) with its factor on the device.
pub struct DeviceCholesky {
    l: DeviceMatrix,
    logdet: f64,
}

impl DeviceCholesky {
    /// `Cholesky::solve` (src/linalg/cholesky.rs:134-143).
    pub fn solve(&self, b: &DeviceMatrix) -> DeviceMatrix {
        assert!(b.nrows == self.l.nrows, "Cholesky solve matrix dimension mismatch.");
        let n = self.l.nrows as c_int;
        let mut x = b.clone_owned();
        let ns = DeviceBuffer::from_slice(&[n]);
        let aoff = DeviceBuffer::from_slice(&[0i64]);
        let boff = DeviceBuffer::from_slice(&[0i64]);
        let bytes = unsafe { ffi::nacu_ragged_workspace_bytes(1) };
        let mut ws = DeviceBuffer::<u8>::zeroed(bytes);
        let order = DeviceBuffer::from_slice(&[0i32]);
        check(unsafe {
            ffi::nacu_dpotrs_ragged(1, n, ns.as_ptr(), aoff.as_ptr(), self.l.data.as_ptr(), b.ncols as c_int,
                                    boff.as_ptr(), x.data.as_mut_ptr(), order.as_ptr(),
                                    ws.as_mut_ptr() as *mut c_void, bytes, 0, std::ptr::null_mut())
        });
        x
    }
    /// `Cholesky::ln_determinant` (src/linalg/cholesky.rs:172-185).
    pub fn ln_determinant(&self) -> f64 {
        self.logdet
    }
    /// The factor with its strict upper part as stored (nalgebra's `l_dirty`).
    pub fn l_dirty(&self) -> DMatrix<f64> {
        self.l.to_dmatrix()
    }
    /// `Cholesky::rank_one_update` (src/linalg/cholesky.rs:277-285), in place.
    pub fn rank_one_update(&mut self, x: &DeviceMatrix, sigma: f64) {
        let n = self.l.nrows as c_int;
        let s = DeviceBuffer::from_slice(&[sigma]);
        check(unsafe {
            ffi::nacu_dchol_rank1_update_batched(n, self.l.data.as_mut_ptr(), (n * n) as i64, x.data.as_ptr(),
                                                 n as i64, s.as_ptr(), 1, 0, std::ptr::null_mut())
        });
    }
}

/// Householder QR (src/linalg/qr.rs:34-40): the axes and R in the matrix
/// buffer, the signed diagonal on the device.  `solve` / `try_inverse` for a
/// square factor; `solve_least_squares` for a tall one, as nalgebra-lapack's
/// `QrDecomposition::solve` (src/qr/abstraction.rs:46-77).
pub struct DeviceQR {
    a: DeviceMatrix,
    diag: DeviceBuffer<f64>,
    invertible: bool,
    large: bool,
}

impl DeviceQR {
    /// b <- Q^T b, then its top n rows <- R^-1 (Q^T b)[0:n]; false at a zero |diag_i|.
    fn solve_cols(&self, b: &mut DeviceMatrix) -> bool {
        let (m, n) = (self.a.nrows, self.a.ncols);
        let mut info = DeviceBuffer::<i32>::zeroed(1);
        if self.large {
            let bytes = unsafe { ffi::nacu_qr_solve_workspace_bytes(n as c_int) };
            let mut ws = DeviceBuffer::<u8>::zeroed(bytes.max(1));
            check(unsafe {
                ffi::nacu_dqr_solve(m as c_int, n as c_int, b.ncols as c_int, self.a.data.as_ptr(), m.max(1) as i64,
                                    self.diag.as_ptr(), b.data.as_mut_ptr(), m.max(1) as i64, info.as_mut_ptr(),
                                    ws.as_mut_ptr() as *mut c_void, bytes, 0, std::ptr::null_mut())
            });
            return info.to_vec()[0] == 0;
        }
        let mut ok = true;
        let mut c0 = 0;
        while c0 < b.ncols {
            let k = (b.ncols - c0).min(16);
            check(unsafe {
                ffi::nacu_dqr_solve_batched(n as c_int, k as c_int, self.a.data.as_ptr(), (n * n) as i64,
                                            self.diag.as_ptr(), b.data.as_mut_ptr().add(c0 * n), (n * k) as i64,
                                            info.as_mut_ptr(), 1, 0, std::ptr::null_mut())
            });
            ok &= info.to_vec()[0] == 0;
            c0 += k;
        }
        ok
    }

    /// `QR::solve_mut` (qr.rs:204-222): b is overwritten even when it
    /// returns false.
    pub fn solve_mut(&self, b: &mut DeviceMatrix) -> bool {
        assert!(self.a.is_square(), "The QR decomposition must be square.");
        assert!(b.nrows == self.a.nrows, "QR solve matrix dimension mismatch.");
        self.solve_cols(b)
    }

    /// `QR::solve` (qr.rs:182-198).
    pub fn solve(&self, b: &DeviceMatrix) -> Option<DeviceMatrix> {
        let mut res = b.clone_owned();
        if self.solve_mut(&mut res) { Some(res) } else { None }
    }

    /// `QR::try_inverse` (qr.rs:262-279).
    pub fn try_inverse(&self) -> Option<DeviceMatrix> {
        assert!(self.a.is_square(), "The QR decomposition must be square.");
        let n = self.a.nrows;
        let mut res = DeviceMatrix::from_dmatrix(&DMatrix::<f64>::identity(n, n));
        if self.solve_cols(&mut res) { Some(res) } else { None }
    }

    /// `QR::is_invertible` (qr.rs:281-292).
    pub fn is_invertible(&self) -> bool {
        self.invertible
    }

    /// argmin ||A x - b|| for a tall factor (m >= n, m <= 16384): the n x nrhs
    /// solution, or `Err` naming the zero |diag_k| (1-based) when A is rank
    /// deficient.
    pub fn solve_least_squares(&self, b: &DeviceMatrix) -> Result<DeviceMatrix, usize> {
        let (m, n) = (self.a.nrows, self.a.ncols);
        assert!(m >= n && b.nrows == m, "QR least squares: m >= n and an m-row right-hand side");
        let mut res = b.clone_owned();
        if !self.solve_cols(&mut res) {
            let d = self.diag.to_vec();
            let k = (0..n).rev().find(|&i| d[i] == 0.0).unwrap_or(0);
            return Err(k + 1);
        }
        let top = res.to_dmatrix().rows(0, n).into_owned();
        Ok(DeviceMatrix::from_dmatrix(&top))
    }
}

/// A ragged batch of square systems packed in one device buffer: system s is
/// ns[s] x ns[s] at a_offsets[s], its nrhs right-hand sides at b_offsets[s].
pub struct DeviceBatch {
    pub ns: Vec<i32>,
    pub a_offsets: Vec<i64>,
    pub a: DeviceBuffer<f64>,
}

impl DeviceBatch {
    /// Packs host matrices (column-major, as `DMatrix` stores them).
    pub fn from_matrices(ms: &[DMatrix<f64>]) -> Self {
        let mut ns = Vec::with_capacity(ms.len());
        let mut offs = Vec::with_capacity(ms.len());
        let mut flat = Vec::new();
        for m in ms {
            assert!(m.is_square(), "a batch of square systems");
            ns.push(m.nrows() as i32);
            offs.push(flat.len() as i64);
            flat.extend_from_slice(m.as_slice());
        }
        DeviceBatch { ns, a_offsets: offs, a: DeviceBuffer::from_slice(&flat) }
    }

    fn rhs_offsets(&self, nrhs: usize) -> Vec<i64> {
        let mut o = Vec::with_capacity(self.ns.len());
        let mut t = 0i64;
        for &n in &self.ns {
            o.push(t);
            t += n as i64 * nrhs as i64;
        }
        o
    }

    /// `m.cholesky()` then `.solve(&b)` for every system in ONE persistent
    /// launch (size-bucketed, autotuned tiles), factors in place; returns the
    /// per-system info (0: SPD, else nalgebra's `None`) and ln_determinant.
    pub fn cholesky_solve(&mut self, b: &mut DeviceBuffer<f64>, nrhs: usize) -> (Vec<i32>, Vec<f64>) {
        let count = self.ns.len() as c_int;
        let n_max = self.ns.iter().copied().max().unwrap_or(0);
        let dns = DeviceBuffer::from_slice(&self.ns);
        let daoff = DeviceBuffer::from_slice(&self.a_offsets);
        let dboff = DeviceBuffer::from_slice(&self.rhs_offsets(nrhs));
        let mut info = DeviceBuffer::<i32>::zeroed(self.ns.len());
        let mut logdet = DeviceBuffer::<f64>::zeroed(self.ns.len());
        let bytes = unsafe { ffi::nacu_ragged_workspace_bytes(count) };
        let mut ws = DeviceBuffer::<u8>::zeroed(bytes);
        check(unsafe {
            ffi::nacu_dposv_ragged(count, n_max, dns.as_ptr(), daoff.as_ptr(), self.a.as_mut_ptr(), nrhs as c_int,
                                   dboff.as_ptr(), b.as_mut_ptr(), info.as_mut_ptr(), logdet.as_mut_ptr(),
                                   std::ptr::null(), ws.as_mut_ptr() as *mut c_void, bytes, 0.0, 0,
                                   std::ptr::null_mut())
        });
        (info.to_vec(), logdet.to_vec())
    }

    /// The precision form of `cholesky_solve` (no nalgebra counterpart): FP32
    /// factor, FP64 refinement to backward error <= n * eps64, FP64 fallback
    /// per system; A and b are left unchanged, the solutions go to x.
    pub fn cholesky_solve_refined(&self, b: &DeviceBuffer<f64>, x: &mut DeviceBuffer<f64>, nrhs: usize)
                                  -> (Vec<i32>, Vec<i32>) {
        let count = self.ns.len() as c_int;
        let n_max = self.ns.iter().copied().max().unwrap_or(0);
        let total: i64 = self.ns.iter().map(|&n| n as i64 * n as i64).sum();
        let dns = DeviceBuffer::from_slice(&self.ns);
        let daoff = DeviceBuffer::from_slice(&self.a_offsets);
        let dboff = DeviceBuffer::from_slice(&self.rhs_offsets(nrhs));
        let mut order: Vec<i32> = (0..count).collect();
        order.sort_by_key(|&s| -self.ns[s as usize]);
        let dorder = DeviceBuffer::from_slice(&order);
        let mut info = DeviceBuffer::<i32>::zeroed(self.ns.len());
        let mut iters = DeviceBuffer::<i32>::zeroed(self.ns.len());
        let bytes = unsafe { ffi::nacu_mixed_workspace_bytes(count, total) };
        let mut ws = DeviceBuffer::<u8>::zeroed(bytes);
        check(unsafe {
            ffi::nacu_dposv_ragged_mixed(count, n_max, dns.as_ptr(), daoff.as_ptr(), self.a.as_ptr(), nrhs as c_int,
                                         dboff.as_ptr(), b.as_ptr(), x.as_mut_ptr(), info.as_mut_ptr(),
                                         iters.as_mut_ptr(), dorder.as_ptr(), total,
                                         ws.as_mut_ptr() as *mut c_void, bytes, 0.0, 0, 0.0, 0,
                                         std::ptr::null_mut())
        });
        (info.to_vec(), iters.to_vec())
    }
}

/// `&a[s] * &b[s]` for a batch of equal-shape products (src/base/ops.rs:566-570),
/// one launch; `exact` = nalgebra's gemv summation order, bit for bit.
pub fn mul_batched(a: &DeviceBuffer<f64>, b: &DeviceBuffer<f64>, m: usize, k: usize, n: usize, batch: usize,
                   exact: bool) -> DeviceBuffer<f64> {
    assert!(a.len() >= m * k * batch && b.len() >= k * n * batch, "mul_batched: buffers too small");
    let mut c = DeviceBuffer::<f64>::zeroed(m * n * batch);
    check(unsafe {
        ffi::nacu_dgemm_batched(m as c_int, n as c_int, k as c_int, 1.0, a.as_ptr(), m.max(1) as i64,
                                (m * k) as i64, b.as_ptr(), k.max(1) as i64, (k * n) as i64, 0.0, c.as_mut_ptr(),
                                m.max(1) as i64, (m * n) as i64, batch as c_int,
                                if exact { NACU_FLAG_EXACT } else { 0 }, std::ptr::null_mut())
    });
    c
}

/// Reverse mode of l = sum_s w_s^T x_s + g_s logdet A_s with x_s = A_s^-1 b_s
/// over a batch of n x n SPD systems (no nalgebra counterpart): `forward`
/// keeps the factors ("store") unless `recompute`, `backward` turns the
/// cotangents (x_bar, logdet_bar) into dA (lower triangle) and db.
pub struct SolveLogdet {
    n: usize,
    batch: usize,
    recompute: bool,
    a: DeviceBuffer<f64>,
    l: Option<DeviceBuffer<f64>>,
    x: DeviceBuffer<f64>,
}

impl SolveLogdet {
    pub fn forward(a: DeviceBuffer<f64>, b: &DeviceBuffer<f64>, n: usize, batch: usize, recompute: bool)
                   -> (SolveLogdet, Vec<f64>) {
        let mut x = DeviceBuffer::<f64>::zeroed(n * batch);
        let mut logdet = DeviceBuffer::<f64>::zeroed(batch);
        let mut info = DeviceBuffer::<i32>::zeroed(batch);
        let mut l = if recompute { None } else { Some(DeviceBuffer::<f64>::zeroed(n * n * batch)) };
        let lp = l.as_mut().map_or(std::ptr::null_mut(), |v| v.as_mut_ptr());
        check(unsafe {
            ffi::nacu_dposv_logdet_forward(n as c_int, a.as_ptr(), (n * n) as i64, b.as_ptr(), x.as_mut_ptr(), lp,
                                           logdet.as_mut_ptr(), info.as_mut_ptr(), batch as c_int,
                                           std::ptr::null_mut())
        });
        (SolveLogdet { n, batch, recompute, a, l, x }, logdet.to_vec())
    }

    pub fn solution(&self) -> &DeviceBuffer<f64> {
        &self.x
    }

    /// (dA, db) from (x_bar, logdet_bar); logdet_bar = None means 0.
    pub fn backward(&self, x_bar: &DeviceBuffer<f64>, logdet_bar: Option<&DeviceBuffer<f64>>)
                    -> (DeviceBuffer<f64>, DeviceBuffer<f64>) {
        let (n, batch) = (self.n, self.batch);
        let mut da = DeviceBuffer::<f64>::zeroed(n * n * batch);
        let mut db = DeviceBuffer::<f64>::zeroed(n * batch);
        let mut info = DeviceBuffer::<i32>::zeroed(batch);
        let al = if self.recompute { self.a.as_ptr() } else { self.l.as_ref().unwrap().as_ptr() };
        let gp = logdet_bar.map_or(std::ptr::null(), |g| g.as_ptr());
        check(unsafe {
            ffi::nacu_dposv_logdet_backward(n as c_int, al, (n * n) as i64, self.recompute as c_int, self.x.as_ptr(),
                                            x_bar.as_ptr(), gp, da.as_mut_ptr(), db.as_mut_ptr(), info.as_mut_ptr(),
                                            batch as c_int, std::ptr::null_mut())
        });
        sync();
        (da, db)
    }
}
