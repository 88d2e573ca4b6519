// TEST INFRASTRUCTURE ONLY — the CPU oracle.
//
// A line-by-line C++ restatement of nalgebra 0.35's dense factorization loops
// (LU with partial pivoting, Cholesky, Householder QR, triangular solves and the
// 8-accumulator dot product).  It exists to check the CUDA kernels and to time
// the CPU baseline; no product code path may call it.
//
// Build with -O2 -ffp-contract=off and without -ffast-math: Rust never contracts
// a*b+c into an FMA, so with contraction off every rounding here happens exactly
// where nalgebra's rounds, and the factors are bit-identical to nalgebra's own on
// the same inputs.
//
// Storage convention (src/base/vec_storage.rs:28-32): column-major, contiguous,
// element (r, c) of an nrows x ncols matrix at a[r + c * lda].
#pragma once
#include <cmath>
#include <vector>
#include <cstddef>
#include <cstdint>

namespace orc {

// ---------------------------------------------------------------------------
// Scalar helpers (simba 0.10 real-field semantics; simba is not vendored in the
// reference, these follow its published behaviour for f32/f64).
// ---------------------------------------------------------------------------

// simba `ComplexField::to_exp` for a real: (|x|, +1) when x >= 0, else (-x, -1).
// The comparison form means -0.0 maps to sign +1 and NaN to sign -1.
template <class T>
inline void to_exp(T x, T* modulus, T* sign) {
  if (x >= T(0)) {
    *modulus = x;
    *sign = T(1);
  } else {
    *modulus = -x;
    *sign = T(-1);
  }
}

// Rust `f64::signum`: +1 for +0.0 and positive, -1 for -0.0 and negative, NaN for NaN.
template <class T>
inline T signum(T x) {
  if (std::isnan(x)) return x;
  return std::signbit(x) ? T(-1) : T(1);
}

// simba `try_sqrt` for a real: Some(sqrt(x)) when x >= 0, else None (NaN -> None).
template <class T>
inline bool try_sqrt(T x, T* out) {
  if (x >= T(0)) {
    *out = std::sqrt(x);
    return true;
  }
  return false;
}

// ---------------------------------------------------------------------------
// BLAS-like kernels
// ---------------------------------------------------------------------------

// Matrix::dotx for one Dyn column (src/base/blas.rs:96-165): eight independent
// accumulators over blocks of 8, combined as (a0+a4), (a1+a5), (a2+a6), (a3+a7)
// into `res` (blas.rs:154-157), then the tail added one product at a time.
template <class T>
inline T dot(std::size_t n, const T* x, const T* y) {
  T res = T(0);
  T acc0 = T(0), acc1 = T(0), acc2 = T(0), acc3 = T(0);
  T acc4 = T(0), acc5 = T(0), acc6 = T(0), acc7 = T(0);
  std::size_t i = 0;
  while (n - i >= 8) {
    acc0 += x[i] * y[i];
    acc1 += x[i + 1] * y[i + 1];
    acc2 += x[i + 2] * y[i + 2];
    acc3 += x[i + 3] * y[i + 3];
    acc4 += x[i + 4] * y[i + 4];
    acc5 += x[i + 5] * y[i + 5];
    acc6 += x[i + 6] * y[i + 6];
    acc7 += x[i + 7] * y[i + 7];
    i += 8;
  }
  res += acc0 + acc4;
  res += acc1 + acc5;
  res += acc2 + acc6;
  res += acc3 + acc7;
  for (std::size_t k = i; k < n; ++k) res += x[k] * y[k];
  return res;
}

// array_axcpy with c = 1 (src/base/blas_uninit.rs:32-53):
// y[i] = a * x[i] * 1 + beta * y[i].  The two unit factors are exact, so this is
// fl(fl(a*x[i]) + fl(beta*y[i])).
template <class T>
inline void axpy(std::size_t n, T a, const T* x, T beta, T* y) {
  for (std::size_t i = 0; i < n; ++i) y[i] = a * x[i] * T(1) + beta * y[i];
}

// gemm_uninit's non-matrixmultiply path (src/base/blas_uninit.rs:187-333, the
// loop at :320-332), used by nalgebra when some dimension is <= 5 or the sizes
// are static: for each output column j, gemv_uninit (:127-176) -- with k == 0,
// y = 0 (beta == 0) or y *= beta; otherwise the first column of A through
// axcpy with beta (array_axc when beta == 0: y = alpha * a * x, else
// array_axcpy: y = alpha * a * x + beta * y, :32-78), the others with beta = 1.
// C = alpha * A * B + beta * C, column-major; C is not read when beta == 0.
template <class T>
inline void gemm_gemv_order(std::size_t m, std::size_t n, std::size_t k, T alpha, const T* a, std::size_t lda,
                            const T* b, std::size_t ldb, T beta, T* c, std::size_t ldc) {
  for (std::size_t j = 0; j < n; ++j) {
    T* y = c + j * ldc;
    const T* x = b + j * ldb;
    if (k == 0) {
      for (std::size_t i = 0; i < m; ++i) y[i] = (beta == T(0)) ? T(0) : y[i] * beta;
      continue;
    }
    for (std::size_t l = 0; l < k; ++l) {
      const T* col = a + l * lda;
      const T val = x[l];
      const T bb = (l == 0) ? beta : T(1);
      if (bb == T(0)) {
        for (std::size_t i = 0; i < m; ++i) y[i] = alpha * col[i] * val;
      } else {
        for (std::size_t i = 0; i < m; ++i) y[i] = alpha * col[i] * val + bb * y[i];
      }
    }
  }
}

// Matrix::icamax for a real column (src/base/min_max.rs:221-240): the first
// index of the largest |x|, strict `>` so ties keep the lower index; a NaN never
// wins unless it sits at index 0.
template <class T>
inline std::size_t icamax(std::size_t n, const T* x) {
  T the_max = std::fabs(x[0]);
  std::size_t the_i = 0;
  for (std::size_t i = 1; i < n; ++i) {
    T v = std::fabs(x[i]);
    if (v > the_max) {
      the_max = v;
      the_i = i;
    }
  }
  return the_i;
}

// ---------------------------------------------------------------------------
// LU with partial pivoting (src/linalg/lu.rs)
// ---------------------------------------------------------------------------

// gauss_step (lu.rs:337-357) and gauss_step_swap (lu.rs:362-389) on an m x n
// matrix at step i, with the pivot value `diag` read before any swap.
template <class T>
inline void gauss_step(std::size_t m, std::size_t n, T* a, std::size_t lda, T diag, std::size_t i,
                       std::size_t piv) {
  const T inv_diag = T(1) / diag;
  T* coeffs = a + i + i * lda;  // column i, rows i..m
  if (piv != i) {
    T t = coeffs[0];
    coeffs[0] = coeffs[piv - i];
    coeffs[piv - i] = t;
  }
  for (std::size_t r = 1; r < m - i; ++r) coeffs[r] = coeffs[r] * inv_diag;
  for (std::size_t k = i + 1; k < n; ++k) {
    T* col = a + i + k * lda;  // rows i..m of column k
    if (piv != i) {
      T t = col[0];
      col[0] = col[piv - i];
      col[piv - i] = t;
    }
    axpy(m - i - 1, -col[0], coeffs + 1, T(1), col + 1);
  }
}

// LU::new (lu.rs:93-122).  Writes the packed L\U factors in place, the full
// per-step pivot row `ipiv[i]` (== i when no swap happened) for i < min(m, n),
// and returns the number of recorded swaps (PermutationSequence::len,
// permutation_sequence.rs:84-93).  The (i, ipiv[i]) pairs with ipiv[i] != i, in
// order, are exactly nalgebra's PermutationSequence entries.
template <class T>
inline std::size_t lu_factor(std::size_t m, std::size_t n, T* a, std::size_t lda, int32_t* ipiv) {
  const std::size_t mn = m < n ? m : n;
  std::size_t len = 0;
  for (std::size_t i = 0; i < mn; ++i) {
    const std::size_t piv = icamax(m - i, a + i + i * lda) + i;
    const T diag = a[piv + i * lda];
    ipiv[i] = (int32_t)i;
    if (diag == T(0)) continue;  // lu.rs:107-110: an all-zero column is skipped
    if (piv != i) {
      ipiv[i] = (int32_t)piv;
      ++len;
      for (std::size_t c = 0; c < i; ++c) {  // columns_range_mut(..i).swap_rows(i, piv)
        T t = a[i + c * lda];
        a[i + c * lda] = a[piv + c * lda];
        a[piv + c * lda] = t;
      }
    }
    gauss_step(m, n, a, lda, diag, i, piv);
  }
  return len;
}

// ---------------------------------------------------------------------------
// LU with full pivoting (src/linalg/full_piv_lu.rs)
// ---------------------------------------------------------------------------

// Matrix::icamax_full for a real m x n matrix (src/base/min_max.rs:146-167):
// columns in order, rows within each, strict `>` from (0, 0), so ties keep the
// earlier position in that order and a NaN never wins unless it is at (0, 0).
template <class T>
inline void icamax_full(std::size_t m, std::size_t n, const T* a, std::size_t lda, std::size_t* ri,
                        std::size_t* ci) {
  T the_max = std::fabs(a[0]);
  std::size_t bi = 0, bj = 0;
  for (std::size_t j = 0; j < n; ++j)
    for (std::size_t i = 0; i < m; ++i) {
      const T v = std::fabs(a[i + j * lda]);
      if (v > the_max) {
        the_max = v;
        bi = i;
        bj = j;
      }
    }
  *ri = bi;
  *ci = bj;
}

// FullPivLU::new (full_piv_lu.rs:56-91): per step i the pivot of the trailing
// submatrix (icamax_full), a stop when it is zero (the rest of the matrix is
// zero), the column swap, then the same rows swap and gauss_step as LU::new.
// Writes ipiv[i] / jpiv[i] (the row / column swapped with i at step i, i when
// none or after the stop) and returns the number of steps taken.  The pairs
// with ipiv[i] != i (jpiv[i] != i), in order, are nalgebra's p (q).
template <class T>
inline std::size_t full_piv_lu_factor(std::size_t m, std::size_t n, T* a, std::size_t lda, int32_t* ipiv,
                                      int32_t* jpiv) {
  const std::size_t mn = m < n ? m : n;
  for (std::size_t i = 0; i < mn; ++i) ipiv[i] = jpiv[i] = (int32_t)i;
  for (std::size_t i = 0; i < mn; ++i) {
    std::size_t r, c;
    icamax_full(m - i, n - i, a + i + i * lda, lda, &r, &c);
    const std::size_t row_piv = r + i, col_piv = c + i;
    const T diag = a[row_piv + col_piv * lda];
    if (diag == T(0)) return i;
    if (col_piv != i)
      for (std::size_t k = 0; k < m; ++k) {  // swap_columns(i, col_piv)
        T t = a[k + i * lda];
        a[k + i * lda] = a[k + col_piv * lda];
        a[k + col_piv * lda] = t;
      }
    jpiv[i] = (int32_t)col_piv;
    if (row_piv != i) {
      ipiv[i] = (int32_t)row_piv;
      for (std::size_t k = 0; k < i; ++k) {  // columns_range_mut(..i).swap_rows(i, row_piv)
        T t = a[i + k * lda];
        a[i + k * lda] = a[row_piv + k * lda];
        a[row_piv + k * lda] = t;
      }
    }
    gauss_step(m, n, a, lda, diag, i, row_piv);
  }
  return mn;
}

// FullPivLU::solve_mut (full_piv_lu.rs:185-211) for an n x n factor: false (b
// untouched) unless lu[n-1][n-1] != 0 (is_invertible, :242-250); then
// p.permute_rows, the unit-lower solve, the upper solve (whose result nalgebra
// ignores: a zero U_ii stops it there, later columns of b unsolved), and
// q.inv_permute_rows (permutation_sequence.rs:108-116).
template <class T>
inline bool full_piv_lu_solve(std::size_t n, const T* lu, std::size_t lda, const int32_t* ipiv,
                              const int32_t* jpiv, T* b, std::size_t ldb, std::size_t nrhs) {
  if (n == 0) return true;
  if (lu[(n - 1) + (n - 1) * lda] == T(0)) return false;
  for (std::size_t i = 0; i < n; ++i) {
    const std::size_t p = (std::size_t)ipiv[i];
    if (p != i)
      for (std::size_t c = 0; c < nrhs; ++c) {
        T t = b[i + c * ldb];
        b[i + c * ldb] = b[p + c * ldb];
        b[p + c * ldb] = t;
      }
  }
  for (std::size_t c = 0; c < nrhs; ++c) {  // solve_lower_triangular_with_diag_mut(b, 1)
    T* bc = b + c * ldb;
    for (std::size_t i = 0; i + 1 < n; ++i) {
      const T coeff = bc[i] / T(1);
      axpy(n - i - 1, -coeff, lu + (i + 1) + i * lda, T(1), bc + i + 1);
    }
  }
  bool stop = false;
  for (std::size_t c = 0; c < nrhs && !stop; ++c) {  // solve_upper_triangular_mut(b)
    T* bc = b + c * ldb;
    for (std::size_t ii = n; ii-- > 0;) {
      const T diag = lu[ii + ii * lda];
      if (diag == T(0)) {
        stop = true;
        break;
      }
      const T coeff = bc[ii] / diag;
      bc[ii] = coeff;
      axpy(ii, -coeff, lu + ii * lda, T(1), bc);
    }
  }
  for (std::size_t k = n; k-- > 0;) {  // q.inv_permute_rows(b)
    const std::size_t q = (std::size_t)jpiv[k];
    if (q != k)
      for (std::size_t c = 0; c < nrhs; ++c) {
        T t = b[k + c * ldb];
        b[k + c * ldb] = b[q + c * ldb];
        b[q + c * ldb] = t;
      }
  }
  return true;
}

// LU::solve_mut (lu.rs:242-260): permute_rows, then the unit-lower forward
// solve (solve.rs:106-133), then the upper back substitution (solve.rs:137-182).
// Returns false when some U_ii == 0 (columns before the failing one are solved).
template <class T>
inline bool lu_solve(std::size_t n, const T* lu, std::size_t lda, const int32_t* ipiv, T* b,
                     std::size_t ldb, std::size_t nrhs) {
  for (std::size_t i = 0; i < n; ++i) {  // permutation_sequence.rs:97-104
    const std::size_t p = (std::size_t)ipiv[i];
    if (p != i)
      for (std::size_t c = 0; c < nrhs; ++c) {
        T t = b[i + c * ldb];
        b[i + c * ldb] = b[p + c * ldb];
        b[p + c * ldb] = t;
      }
  }
  if (n == 0) return true;
  for (std::size_t c = 0; c < nrhs; ++c) {  // with diag = 1
    T* bc = b + c * ldb;
    for (std::size_t i = 0; i + 1 < n; ++i) {
      const T coeff = bc[i] / T(1);
      axpy(n - i - 1, -coeff, lu + (i + 1) + i * lda, T(1), bc + i + 1);
    }
  }
  for (std::size_t c = 0; c < nrhs; ++c) {
    T* bc = b + c * ldb;
    for (std::size_t ii = n; ii-- > 0;) {
      const T diag = lu[ii + ii * lda];
      if (diag == T(0)) return false;
      const T coeff = bc[ii] / diag;
      bc[ii] = coeff;
      axpy(ii, -coeff, lu + ii * lda, T(1), bc);
    }
  }
  return true;
}

// Triangular solves of Matrix (src/linalg/solve.rs), one column of b at a time
// (the `_mut` forms loop over the columns, returning false at the first zero
// diagonal; the columns after a failing one are left as they are).
// lower = solve_lower_triangular_vector_mut (solve.rs:74-101): axpy form.
// upper = solve_upper_triangular_vector_mut (solve.rs:156-181).
// tr lower = xx_solve_lower_triangular_vector_mut (solve.rs:374-407): dot
//   form, i descending; tr upper = xx_solve_upper_triangular_vector_mut
//   (solve.rs:409-442), i ascending (ad_ = tr_ for real scalars).
// with_diag = solve_lower_triangular_with_diag_mut (solve.rs:106-134): the
//   diagonal is never read; b_i itself is not rewritten (i < n-1 only).
template <class T>
inline bool triangular_solve(std::size_t n, const T* t, std::size_t lda, T* b, std::size_t ldb, std::size_t nrhs,
                             bool upper, bool trans, bool has_diag, T diag) {
  if (has_diag) {
    if (diag == T(0)) return false;
    for (std::size_t c = 0; c < nrhs; ++c) {
      T* bc = b + c * ldb;
      for (std::size_t i = 0; i + 1 < n; ++i) {
        const T coeff = bc[i] / diag;
        axpy(n - i - 1, -coeff, t + (i + 1) + i * lda, T(1), bc + i + 1);
      }
    }
    return true;
  }
  for (std::size_t c = 0; c < nrhs; ++c) {
    T* bc = b + c * ldb;
    if (!upper && !trans) {
      for (std::size_t i = 0; i < n; ++i) {
        const T d = t[i + i * lda];
        if (d == T(0)) return false;
        const T coeff = bc[i] / d;
        bc[i] = coeff;
        axpy(n - i - 1, -coeff, t + (i + 1) + i * lda, T(1), bc + i + 1);
      }
    } else if (upper && !trans) {
      for (std::size_t i = n; i-- > 0;) {
        const T d = t[i + i * lda];
        if (d == T(0)) return false;
        const T coeff = bc[i] / d;
        bc[i] = coeff;
        axpy(i, -coeff, t + i * lda, T(1), bc);
      }
    } else if (!upper && trans) {
      for (std::size_t i = n; i-- > 0;) {
        const T dt = dot(n - i - 1, t + (i + 1) + i * lda, bc + i + 1);
        const T d = t[i + i * lda];
        if (d == T(0)) return false;
        bc[i] = (bc[i] - dt) / d;
      }
    } else {
      for (std::size_t i = 0; i < n; ++i) {
        const T dt = dot(i, t + i * lda, bc);
        const T d = t[i + i * lda];
        if (d == T(0)) return false;
        bc[i] = (bc[i] - dt) / d;
      }
    }
  }
  return true;
}

// LU::determinant (lu.rs:301-314): product of the diagonal times the sign of
// the permutation (permutation_sequence.rs:158-164).
template <class T>
inline T lu_determinant(std::size_t n, const T* lu, std::size_t lda, std::size_t len) {
  T res = T(1);
  for (std::size_t i = 0; i < n; ++i) res *= lu[i + i * lda];
  return res * ((len % 2 == 0) ? T(1) : T(-1));
}

// ---------------------------------------------------------------------------
// Cholesky (src/linalg/cholesky.rs)
// ---------------------------------------------------------------------------

// Cholesky::new_internal (cholesky.rs:221-272): left-looking, reads the lower
// triangle only, leaves the strict upper triangle untouched.  Returns 0 on
// success or j + 1 for the first column whose pivot is not > 0 (NaN included)
// and could not be replaced by `substitute` (has_substitute != 0).
template <class T>
inline int cholesky_factor(std::size_t n, T* a, std::size_t lda, int has_substitute, T substitute) {
  for (std::size_t j = 0; j < n; ++j) {
    for (std::size_t k = 0; k < j; ++k) {
      const T factor = -a[j + k * lda];
      axpy(n - j, factor, a + j + k * lda, T(1), a + j + j * lda);
    }
    const T diag = a[j + j * lda];
    T denom;
    bool ok = false;
    if (!(diag <= T(0))) ok = try_sqrt(diag, &denom);
    if (!ok && has_substitute && !(substitute <= T(0))) ok = try_sqrt(substitute, &denom);
    if (!ok) return (int)j + 1;
    a[j + j * lda] = denom;
    for (std::size_t r = j + 1; r < n; ++r) a[r + j * lda] = a[r + j * lda] / denom;
  }
  return 0;
}

// Cholesky::solve_mut (cholesky.rs:122-129): forward solve in axpy form
// (solve.rs:488-519) then the adjoint back solve in dot form (solve.rs:697-712,
// 732-755).
template <class T>
inline void cholesky_solve(std::size_t n, const T* l, std::size_t lda, T* b, std::size_t ldb,
                           std::size_t nrhs) {
  for (std::size_t c = 0; c < nrhs; ++c) {
    T* bc = b + c * ldb;
    for (std::size_t i = 0; i < n; ++i) {
      const T coeff = bc[i] / l[i + i * lda];
      bc[i] = coeff;
      axpy(n - i - 1, -coeff, l + (i + 1) + i * lda, T(1), bc + i + 1);
    }
  }
  for (std::size_t c = 0; c < nrhs; ++c) {
    T* bc = b + c * ldb;
    for (std::size_t ii = n; ii-- > 0;) {
      const T d = dot(n - ii - 1, l + (ii + 1) + ii * lda, bc + ii + 1);
      bc[ii] = (bc[ii] - d) / l[ii + ii * lda];
    }
  }
}

// Cholesky::xx_rank_one_update (cholesky.rs:410-449): L (n x n, lower part)
// becomes the factor of L L^T + sigma x x^T; x is overwritten (nalgebra works
// on a clone of the caller's vector).  Operation order as in Rust, no FMA.
template <class T>
inline void chol_rank_one_update(std::size_t n, T* l, std::size_t lda, T* x, T sigma) {
  T beta = T(1);
  for (std::size_t j = 0; j < n; ++j) {
    const T diag = l[j + j * lda];
    const T diag2 = diag * diag;
    const T xj = x[j];
    const T sigma_xj2 = sigma * (xj * xj);
    const T gamma = diag2 * beta + sigma_xj2;
    const T new_diag = std::sqrt(diag2 + sigma_xj2 / beta);
    l[j + j * lda] = new_diag;
    beta += sigma_xj2 / diag2;
    T* col = l + (j + 1) + j * lda;
    T* xp = x + j + 1;
    axpy(n - j - 1, -xj / diag, col, T(1), xp);  // x[j+1..] += (-xj / diag) L[j+1.., j]
    if (gamma != T(0)) axpy(n - j - 1, new_diag * sigma / gamma * xj, xp, new_diag / diag, col);
  }
}

// Cholesky::remove_column (cholesky.rs:365-399): out ((n-1) x (n-1), ldo) is
// L without row and column j (the strict upper part copied block by block, as
// nalgebra copies its views), then the rank-one update of the bottom-right
// corner by L[j+1.., j] with sigma = 1.
template <class T>
inline void chol_remove_column(std::size_t n, const T* l, std::size_t lda, std::size_t j, T* out, std::size_t ldo) {
  for (std::size_t c = 0; c + 1 < n; ++c)
    for (std::size_t r = 0; r + 1 < n; ++r)
      out[r + c * ldo] = l[(r < j ? r : r + 1) + (c < j ? c : c + 1) * lda];
  std::vector<T> w(l + (j + 1) + j * lda, l + n + j * lda);
  chol_rank_one_update<T>(n - 1 - j, out + j + j * ldo, ldo, w.data(), T(1));
}

// Cholesky::insert_column (cholesky.rs:287-357): out ((n+1) x (n+1), ldo)
// holds L with an empty row and column j, then row j from the lower solve of
// the top-left corner with col[..j], the centre sqrt(col[j] - |row j|^2), the
// new column (col[j+1..] - bottom-left L[j.., ..j] row_j) / centre through
// gemv's axcpy order (blas_uninit.rs:127-176), and the rank-one downdate of the
// bottom-right corner by that column.  False when the lower solve fails
// (nalgebra's assert).
template <class T>
inline bool chol_insert_column(std::size_t n, const T* l, std::size_t lda, std::size_t j, const T* col, T* out,
                               std::size_t ldo) {
  const std::size_t m = n + 1;
  for (std::size_t c = 0; c < m; ++c)
    for (std::size_t r = 0; r < m; ++r) {
      if (r == j || c == j) out[r + c * ldo] = T(0);
      else out[r + c * ldo] = l[(r < j ? r : r - 1) + (c < j ? c : c - 1) * lda];
    }
  std::vector<T> row(col, col + j);             // new_rowj_adjoint
  std::vector<T> ncol(col + j + 1, col + m);    // new_colj
  if (!triangular_solve<T>(j, l, lda, row.data(), j, 1, false, false, false, T(0))) return false;
  for (std::size_t k = 0; k < j; ++k) out[j + k * ldo] = row[k];
  const T center = std::sqrt(col[j] - dot(j, row.data(), row.data()));
  out[j + j * ldo] = center;
  // new_colj.gemm(-1/center, L[j.., ..j], row, 1/center), one output column: gemv
  const T alpha = -T(1) / center, beta = T(1) / center;
  const std::size_t len = n - j;
  if (j == 0) {
    for (std::size_t r = 0; r < len; ++r) ncol[r] *= beta;
  } else {
    for (std::size_t k = 0; k < j; ++k) {
      const T* lc = l + j + k * lda;  // column k of the bottom-left corner
      const T val = row[k];
      const T b = (k == 0) ? beta : T(1);
      for (std::size_t r = 0; r < len; ++r) ncol[r] = alpha * lc[r] * val + b * ncol[r];
    }
  }
  for (std::size_t r = 0; r < len; ++r) out[(j + 1 + r) + j * ldo] = ncol[r];
  chol_rank_one_update<T>(len, out + (j + 1) + (j + 1) * ldo, ldo, ncol.data(), T(-1));
  return true;
}

// Cholesky::ln_determinant (cholesky.rs:172-185): sum of ln(L_ii * L_ii).
template <class T>
inline T cholesky_ln_determinant(std::size_t n, const T* l, std::size_t lda) {
  T s = T(0);
  for (std::size_t i = 0; i < n; ++i) {
    const T d = l[i + i * lda];
    s += std::log(d * d);
  }
  return s;
}

// ---------------------------------------------------------------------------
// Householder QR (src/linalg/qr.rs, householder.rs, geometry/reflection.rs)
// ---------------------------------------------------------------------------

// Reflection::reflect_with_sign (reflection.rs:70-83) with bias 0 on the
// `ncols` columns of `c` (each `len` long), axis `v` of length `len`.
template <class T>
inline void reflect_with_sign(std::size_t len, const T* v, std::size_t ncols, T* c, std::size_t ldc,
                              T sign) {
  for (std::size_t j = 0; j < ncols; ++j) {
    T* cj = c + j * ldc;
    const T m_two = sign * T(-2);
    const T factor = (dot(len, v, cj) - T(0)) * m_two;
    axpy(len, factor, v, sign, cj);
  }
}

// householder::reflection_axis_mut (householder.rs:19-53).  Returns the value
// of the first component after reflection; *not_zero is false when no
// reflection was needed (a zero column).
template <class T>
inline T reflection_axis(std::size_t len, T* x, bool* not_zero) {
  const T sq = T(0) + dot(len, x, x);  // norm_squared (norm.rs:238-250)
  const T nrm = std::sqrt(sq);
  T modulus, sign;
  to_exp(x[0], &modulus, &sign);
  const T signed_norm = sign * nrm;
  const T factor = (sq + modulus * nrm) * T(2);
  x[0] += signed_norm;
  if (factor != T(0)) {
    const T sf = std::sqrt(factor);
    for (std::size_t i = 0; i < len; ++i) x[i] = x[i] / sf;  // unscale_mut
    const T n2 = std::sqrt(T(0) + dot(len, x, x));          // normalize_mut (norm.rs:505-513)
    for (std::size_t i = 0; i < len; ++i) x[i] = x[i] / n2;
    *not_zero = true;
    return -signed_norm;
  }
  *not_zero = false;
  return signed_norm;
}

// QR::new (qr.rs:55-76) via householder::clear_column_unchecked
// (householder.rs:61-85) with shift 0.  diag has min(m, n) entries.
template <class T>
inline void qr_factor(std::size_t m, std::size_t n, T* a, std::size_t lda, T* diag) {
  const std::size_t mn = m < n ? m : n;
  for (std::size_t i = 0; i < mn; ++i) {
    bool not_zero;
    T* axis = a + i + i * lda;
    const T rnorm = reflection_axis(m - i, axis, &not_zero);
    if (not_zero) reflect_with_sign(m - i, axis, n - i - 1, axis + lda, lda, signum(rnorm));
    diag[i] = rnorm;
  }
}

// QR::q_tr_mul (qr.rs:157-171): rhs <- Q^T rhs.
template <class T>
inline void qr_q_tr_mul(std::size_t m, std::size_t n, const T* qr, std::size_t lda, const T* diag,
                        T* b, std::size_t ldb, std::size_t nrhs) {
  const std::size_t mn = m < n ? m : n;
  for (std::size_t i = 0; i < mn; ++i)
    reflect_with_sign(m - i, qr + i + i * lda, nrhs, b + i, ldb, signum(diag[i]));
}

// QR::solve_mut (qr.rs:204-256) for an n x n factor: q_tr_mul (:157-171),
// then the upper solve of :224-256 (for each column, i descending: a zero
// |diag_i| returns false at once, leaving that column partly and the later
// ones not solved; else b_i / |diag_i| and the axpy with R's column above i).
template <class T>
inline bool qr_solve(std::size_t n, const T* qr, std::size_t lda, const T* diag, T* b, std::size_t ldb,
                     std::size_t nrhs) {
  qr_q_tr_mul(n, n, qr, lda, diag, b, ldb, nrhs);
  for (std::size_t c = 0; c < nrhs; ++c) {
    T* bc = b + c * ldb;
    for (std::size_t ii = n; ii-- > 0;) {
      const T d = std::fabs(diag[ii]);
      if (d == T(0)) return false;
      const T coeff = bc[ii] / d;
      bc[ii] = coeff;
      axpy(ii, -coeff, qr + ii * lda, T(1), bc);
    }
  }
  return true;
}

// ColPivQR::new (src/linalg/col_piv_qr.rs:59-92): per step the column of
// icamax_full over the trailing submatrix (its largest |a|, min_max.rs:146-167),
// the column swap, then clear_column_unchecked as QR::new.  jpiv[i] is the
// column swapped with i at step i (i when none); diag as QR::new's.
template <class T>
inline void col_piv_qr_factor(std::size_t m, std::size_t n, T* a, std::size_t lda, T* diag, int32_t* jpiv) {
  const std::size_t mn = m < n ? m : n;
  for (std::size_t i = 0; i < mn; ++i) {
    std::size_t r, c;
    icamax_full(m - i, n - i, a + i + i * lda, lda, &r, &c);
    const std::size_t col_piv = c + i;
    if (col_piv != i)
      for (std::size_t k = 0; k < m; ++k) {  // swap_columns(i, col_piv)
        T t = a[k + i * lda];
        a[k + i * lda] = a[k + col_piv * lda];
        a[k + col_piv * lda] = t;
      }
    jpiv[i] = (int32_t)col_piv;
    bool not_zero;
    T* axis = a + i + i * lda;
    const T rnorm = reflection_axis(m - i, axis, &not_zero);
    if (not_zero) reflect_with_sign(m - i, axis, n - i - 1, axis + lda, lda, signum(rnorm));
    diag[i] = rnorm;
  }
}

// ColPivQR::solve_mut (col_piv_qr.rs:227-247) for an n x n factor: q_tr_mul
// (:180-192, every reflection, with the sign of its diag entry), the upper
// solve of :250-285 (divide by |diag_i|; a zero one returns false at once,
// that column partly and the later ones not solved), then p.inv_permute_rows
// whatever the upper solve returned.  Returns the upper solve's result.
template <class T>
inline bool col_piv_qr_solve(std::size_t n, const T* qr, std::size_t lda, const T* diag, const int32_t* jpiv, T* b,
                             std::size_t ldb, std::size_t nrhs) {
  for (std::size_t i = 0; i < n; ++i)
    reflect_with_sign(n - i, qr + i + i * lda, nrhs, b + i, ldb, signum(diag[i]));
  bool solved = true;
  for (std::size_t c = 0; c < nrhs && solved; ++c) {
    T* bc = b + c * ldb;
    for (std::size_t ii = n; ii-- > 0;) {
      const T d = std::fabs(diag[ii]);
      if (d == T(0)) {
        solved = false;
        break;
      }
      const T coeff = bc[ii] / d;
      bc[ii] = coeff;
      axpy(ii, -coeff, qr + ii * lda, T(1), bc);
    }
  }
  for (std::size_t k = n; k-- > 0;) {
    const std::size_t q = (std::size_t)jpiv[k];
    if (q != k)
      for (std::size_t c = 0; c < nrhs; ++c) {
        T t = b[k + c * ldb];
        b[k + c * ldb] = b[q + c * ldb];
        b[q + c * ldb] = t;
      }
  }
  return solved;
}

// Least squares x = argmin ||A x - b|| for m >= n from the factors: Q^T b
// (qr.rs:157-171), then the back substitution of qr.rs:224-256 (divide by
// |diag_i|, axpy with the strict upper part of R) restricted to the top n rows,
// as nalgebra-lapack's qr_solve_mut_with_rank_unpermuted (qr_util.rs:167-239)
// restricts dtrtrs to R[0:n, 0:n].  b (m x nrhs) is overwritten by Q^T b; x
// (n x nrhs) receives the solution.  Returns 0, or i + 1 for the first zero
// |diag_i| (rank deficient, LAPACK trtrs info > 0).
template <class T>
inline int qr_ls_solve(std::size_t m, std::size_t n, const T* qr, std::size_t lda, const T* diag,
                       T* b, std::size_t ldb, T* x, std::size_t ldx, std::size_t nrhs) {
  qr_q_tr_mul(m, n, qr, lda, diag, b, ldb, nrhs);
  // LAPACK trtrs reports the first zero diagonal from the top (info > 0).
  for (std::size_t i = 0; i < n; ++i)
    if (std::fabs(diag[i]) == T(0)) return (int)i + 1;
  for (std::size_t c = 0; c < nrhs; ++c) {
    T* xc = x + c * ldx;
    for (std::size_t r = 0; r < n; ++r) xc[r] = b[r + c * ldb];
    for (std::size_t ii = n; ii-- > 0;) {
      const T d = std::fabs(diag[ii]);
      if (d == T(0)) return (int)ii + 1;
      const T coeff = xc[ii] / d;
      xc[ii] = coeff;
      axpy(ii, -coeff, qr + ii * lda, T(1), xc);
    }
  }
  return 0;
}

// ---------------------------------------------------------------------------
// Accurate FP64 arithmetic for the parity metrics (not a nalgebra restatement):
// TwoSum / TwoProduct compensated dot, Ogita, Rump & Oishi (2005), "Accurate
// sum and dot product", Algorithm Dot2.
// ---------------------------------------------------------------------------
inline void two_sum(double a, double b, double* s, double* e) {
  const double x = a + b;
  const double z = x - a;
  *e = (a - (x - z)) + (b - z);
  *s = x;
}
inline void two_prod(double a, double b, double* p, double* e) {
  const double x = a * b;
  *e = std::fma(a, b, -x);
  *p = x;
}

}  // namespace orc
