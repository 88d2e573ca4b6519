// TEST INFRASTRUCTURE ONLY — C entry points of the CPU oracle (nalgebra_ref.hpp)
// for the parity tests and the timed CPU baseline.  Nothing in the product
// (the CUDA library or its host mirrors) links or calls this.
//
// Batched drivers parallelise across independent systems with OpenMP, one
// system per thread, exactly as a caller would run nalgebra's single-threaded
// LU/Cholesky/QR on many matrices.
#include <omp.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "nalgebra_ref.hpp"

using orc::two_prod;
using orc::two_sum;

namespace {
void set_threads(int nthreads) {
  if (nthreads > 0) omp_set_num_threads(nthreads);
}
}  // namespace

extern "C" {

int orc_max_threads(void) { return omp_get_max_threads(); }

// ---- single-matrix restatements (f64 and f32) -------------------------------
double orc_ddot(int64_t n, const double* x, const double* y) { return orc::dot<double>(n, x, y); }

int64_t orc_dgetrf(int64_t m, int64_t n, double* a, int64_t lda, int32_t* ipiv) {
  return (int64_t)orc::lu_factor<double>(m, n, a, lda, ipiv);
}
int64_t orc_sgetrf(int64_t m, int64_t n, float* a, int64_t lda, int32_t* ipiv) {
  return (int64_t)orc::lu_factor<float>(m, n, a, lda, ipiv);
}
int orc_dgetrs(int64_t n, const double* lu, int64_t lda, const int32_t* ipiv, double* b, int64_t ldb,
               int64_t nrhs) {
  return orc::lu_solve<double>(n, lu, lda, ipiv, b, ldb, nrhs) ? 1 : 0;
}
int64_t orc_dfullpivlu(int64_t m, int64_t n, double* a, int64_t lda, int32_t* ipiv, int32_t* jpiv) {
  return (int64_t)orc::full_piv_lu_factor<double>(m, n, a, lda, ipiv, jpiv);
}
int orc_dfullpivlu_solve(int64_t n, const double* lu, int64_t lda, const int32_t* ipiv, const int32_t* jpiv,
                         double* b, int64_t ldb, int64_t nrhs) {
  return orc::full_piv_lu_solve<double>(n, lu, lda, ipiv, jpiv, b, ldb, nrhs) ? 1 : 0;
}
void orc_dcolpivqr(int64_t m, int64_t n, double* a, int64_t lda, double* diag, int32_t* jpiv) {
  orc::col_piv_qr_factor<double>(m, n, a, lda, diag, jpiv);
}
int orc_dcolpivqr_solve(int64_t n, const double* qr, int64_t lda, const double* diag, const int32_t* jpiv,
                        double* b, int64_t ldb, int64_t nrhs) {
  return orc::col_piv_qr_solve<double>(n, qr, lda, diag, jpiv, b, ldb, nrhs) ? 1 : 0;
}
double orc_dlu_determinant(int64_t n, const double* lu, int64_t lda, int64_t len) {
  return orc::lu_determinant<double>(n, lu, lda, len);
}
int orc_dpotrf(int64_t n, double* a, int64_t lda, int has_substitute, double substitute) {
  return orc::cholesky_factor<double>(n, a, lda, has_substitute, substitute);
}
int orc_spotrf(int64_t n, float* a, int64_t lda, int has_substitute, float substitute) {
  return orc::cholesky_factor<float>(n, a, lda, has_substitute, substitute);
}
void orc_dpotrs(int64_t n, const double* l, int64_t lda, double* b, int64_t ldb, int64_t nrhs) {
  orc::cholesky_solve<double>(n, l, lda, b, ldb, nrhs);
}
double orc_dpotrf_ln_det(int64_t n, const double* l, int64_t lda) {
  return orc::cholesky_ln_determinant<double>(n, l, lda);
}
void orc_dgeqrf(int64_t m, int64_t n, double* a, int64_t lda, double* diag) {
  orc::qr_factor<double>(m, n, a, lda, diag);
}
void orc_dqr_q_tr_mul(int64_t m, int64_t n, const double* qr, int64_t lda, const double* diag,
                      double* b, int64_t ldb, int64_t nrhs) {
  orc::qr_q_tr_mul<double>(m, n, qr, lda, diag, b, ldb, nrhs);
}
int orc_dqr_solve(int64_t n, const double* qr, int64_t lda, const double* diag, double* b, int64_t ldb,
                  int64_t nrhs) {
  return orc::qr_solve<double>(n, qr, lda, diag, b, ldb, nrhs) ? 1 : 0;
}
int orc_dqr_ls_solve(int64_t m, int64_t n, const double* qr, int64_t lda, const double* diag,
                     double* b, int64_t ldb, double* x, int64_t ldx, int64_t nrhs) {
  return orc::qr_ls_solve<double>(m, n, qr, lda, diag, b, ldb, x, ldx, nrhs);
}

// Triangular solve of b (n x nrhs) by t (solve.rs:55-442): uplo 0 lower / 1
// upper, trans 0 / 1 (tr_ and ad_ forms), has_diag (lower only): the
// with_diag form.  1 = solved, 0 = a zero diagonal (nalgebra's false).
int orc_dtrsv(int64_t n, const double* t, int64_t lda, double* b, int64_t ldb, int64_t nrhs, int uplo, int trans,
              int has_diag, double diag) {
  return orc::triangular_solve<double>(n, t, lda, b, ldb, nrhs, uplo != 0, trans != 0, has_diag != 0, diag) ? 1 : 0;
}

// Cholesky updates (cholesky.rs:277-449): the rank-one update in place (x is
// overwritten), remove_column into out ((n-1)^2), insert_column into out
// ((n+1)^2; 0 when the lower solve fails).
void orc_dchol_rank1(int64_t n, double* l, int64_t lda, double* x, double sigma) {
  orc::chol_rank_one_update<double>(n, l, lda, x, sigma);
}
void orc_dchol_remove_column(int64_t n, const double* l, int64_t lda, int64_t j, double* out, int64_t ldo) {
  orc::chol_remove_column<double>(n, l, lda, j, out, ldo);
}
int orc_dchol_insert_column(int64_t n, const double* l, int64_t lda, int64_t j, const double* col, double* out,
                            int64_t ldo) {
  return orc::chol_insert_column<double>(n, l, lda, j, col, out, ldo) ? 1 : 0;
}

// ---- batched drivers (the CPU baseline) -----------------------------------
// `batch` dense n x n systems packed back to back (stride n*n), one n x nrhs
// right-hand side each (stride n*nrhs).  Factor in place, solve in place.
// info[s] = 0 ok, 1 when the solve reported a zero U_ii.
void orc_dgesv_batched(int64_t batch, int64_t n, double* a, int32_t* ipiv, double* b, int64_t nrhs,
                       int32_t* info, int nthreads) {
  set_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 4)
  for (int64_t s = 0; s < batch; ++s) {
    double* as = a + s * n * n;
    int32_t* ps = ipiv + s * n;
    orc::lu_factor<double>(n, n, as, n, ps);
    info[s] = orc::lu_solve<double>(n, as, n, ps, b + s * n * nrhs, n, nrhs) ? 0 : 1;
  }
}

// Ragged Cholesky: matrix s is ns[s] x ns[s] at a + aoff[s], its RHS block
// ns[s] x nrhs at b + boff[s].  info as cholesky_factor; logdet per matrix.
void orc_dposv_ragged(int64_t count, const int32_t* ns, const int64_t* aoff, double* a,
                      const int64_t* boff, double* b, int64_t nrhs, int32_t* info, double* logdet,
                      int nthreads) {
  set_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t s = 0; s < count; ++s) {
    const int64_t n = ns[s];
    double* as = a + aoff[s];
    const int r = orc::cholesky_factor<double>(n, as, n, 0, 0.0);
    info[s] = r;
    if (r == 0) {
      orc::cholesky_solve<double>(n, as, n, b + boff[s], n, nrhs);
      if (logdet) logdet[s] = orc::cholesky_ln_determinant<double>(n, as, n);
    } else if (logdet) {
      logdet[s] = NAN;
    }
  }
}

// Batched least squares: problem s is ms[s] x n at a + aoff[s] with one m x 1
// RHS at b + boff[s]; x is n x 1 at x + s*n; diag n per problem.
void orc_dgels_batched(int64_t count, const int32_t* ms, int64_t n, const int64_t* aoff, double* a,
                       const int64_t* boff, double* b, double* diag, double* x, int32_t* info,
                       int nthreads) {
  set_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t s = 0; s < count; ++s) {
    const int64_t m = ms[s];
    double* as = a + aoff[s];
    orc::qr_factor<double>(m, n, as, m, diag + s * n);
    info[s] = orc::qr_ls_solve<double>(m, n, as, m, diag + s * n, b + boff[s], m, x + s * n, n, 1);
  }
}

// ---- accurate FP64 metrics ---------------------------------------------------

// nalgebra's gemm in its gemv order (the small / static-size path of
// gemm_uninit), batched over `batch` products at the given strides.
void orc_dgemm_gemv_order_batched(int64_t m, int64_t n, int64_t k, double alpha, const double* a, int64_t lda,
                                  int64_t sa, const double* b, int64_t ldb, int64_t sb, double beta, double* c,
                                  int64_t ldc, int64_t sc, int64_t batch, int nthreads) {
  set_threads(nthreads);
#pragma omp parallel for schedule(static)
  for (int64_t s = 0; s < batch; ++s)
    orc::gemm_gemv_order<double>(m, n, k, alpha, a + s * sa, lda, b + s * sb, ldb, beta, c + s * sc, ldc);
}

// C = alpha * A * B + beta * C with every dot product accumulated by Dot2
// (compensated), the accurate reference for the GEMM kernels.  beta == 0 means
// C is never read (blas.rs:729-746 contract).
void orc_dgemm_dot2(int64_t m, int64_t n, int64_t k, double alpha, const double* a, int64_t lda,
                    const double* b, int64_t ldb, double beta, double* c, int64_t ldc,
                    int nthreads) {
  set_threads(nthreads);
#pragma omp parallel for schedule(static)
  for (int64_t j = 0; j < n; ++j) {
    std::vector<double> arow(k);
    for (int64_t i = 0; i < m; ++i) {
      double s = 0.0, e = 0.0;
      for (int64_t p = 0; p < k; ++p) {
        double pr, pe, ss, se;
        two_prod(a[i + p * lda], b[p + j * ldb], &pr, &pe);
        two_sum(s, pr, &ss, &se);
        s = ss;
        e += pe + se;
      }
      const double ab = s + e;
      c[i + j * ldc] = (beta == 0.0) ? alpha * ab : alpha * ab + beta * c[i + j * ldc];
    }
  }
}

// Normwise backward error of x for A x = b, per RHS column, maximum over
// columns: ||b - A x||_inf / (||A||_inf ||x||_inf + ||b||_inf), residual by Dot2.
double orc_dbackward_error(int64_t n, const double* a, int64_t lda, const double* x, int64_t ldx,
                           const double* b, int64_t ldb, int64_t nrhs) {
  double anorm = 0.0;
  for (int64_t i = 0; i < n; ++i) {
    double s = 0.0;
    for (int64_t j = 0; j < n; ++j) s += std::fabs(a[i + j * lda]);
    if (s > anorm) anorm = s;
  }
  double worst = 0.0;
  for (int64_t c = 0; c < nrhs; ++c) {
    double rmax = 0.0, xmax = 0.0, bmax = 0.0;
    for (int64_t i = 0; i < n; ++i) {
      double s = b[i + c * ldb], e = 0.0;
      for (int64_t j = 0; j < n; ++j) {
        double pr, pe, ss, se;
        two_prod(-a[i + j * lda], x[j + c * ldx], &pr, &pe);
        two_sum(s, pr, &ss, &se);
        s = ss;
        e += pe + se;
      }
      const double r = std::fabs(s + e);
      if (r > rmax) rmax = r;
      if (std::fabs(b[i + c * ldb]) > bmax) bmax = std::fabs(b[i + c * ldb]);
    }
    for (int64_t j = 0; j < n; ++j)
      if (std::fabs(x[j + c * ldx]) > xmax) xmax = std::fabs(x[j + c * ldx]);
    const double den = anorm * xmax + bmax;
    const double be = den > 0.0 ? rmax / den : (rmax > 0.0 ? INFINITY : 0.0);
    if (!(be <= worst)) worst = be;
  }
  return worst;
}

// ||P A - L U||_F / (||A||_F * n * eps64) for packed factors and a per-step
// pivot list (the LU parity criterion: at most 10).
double orc_dlu_reconstruction(int64_t n, const double* a, int64_t lda, const double* lu,
                              int64_t ldlu, const int32_t* ipiv) {
  std::vector<double> pa(n * n);
  for (int64_t j = 0; j < n; ++j)
    for (int64_t i = 0; i < n; ++i) pa[i + j * n] = a[i + j * lda];
  for (int64_t i = 0; i < n; ++i) {
    const int64_t p = ipiv[i];
    if (p != i)
      for (int64_t j = 0; j < n; ++j) {
        const double t = pa[i + j * n];
        pa[i + j * n] = pa[p + j * n];
        pa[p + j * n] = t;
      }
  }
  double num = 0.0, den = 0.0;
  for (int64_t j = 0; j < n; ++j)
    for (int64_t i = 0; i < n; ++i) {
      double s = 0.0, e = 0.0;
      const int64_t kmax = i < j ? i : j;
      for (int64_t k = 0; k <= kmax; ++k) {
        const double l = (k == i) ? 1.0 : lu[i + k * ldlu];
        double pr, pe, ss, se;
        two_prod(l, lu[k + j * ldlu], &pr, &pe);
        two_sum(s, pr, &ss, &se);
        s = ss;
        e += pe + se;
      }
      const double d = pa[i + j * n] - (s + e);
      num += d * d;
      den += pa[i + j * n] * pa[i + j * n];
    }
  if (n == 0 || den == 0.0) return num == 0.0 ? 0.0 : INFINITY;
  return std::sqrt(num) / (std::sqrt(den) * (double)n * 2.220446049250313e-16);
}

// ---- accuracy metrics over whole batches (checkers, not restatements) -----

namespace {
// r = b - A x with every row's sum carried as a Dot2 pair (s, e), A given
// by columns: column j adds -A(i, j) x_j to every row i.  `sym` takes A as
// the symmetric matrix of its lower triangle (the only part the Cholesky
// solvers read, cholesky.rs:221-272).  Returns max_i |r_i| and fills
// rowabs[i] = sum_j |A(i, j)| when rowabs is given.
double residual_inf_dd(int64_t n, const double* a, int64_t lda, bool sym, const double* x, const double* b,
                       double* s, double* e, double* rowabs) {
  for (int64_t i = 0; i < n; ++i) {
    s[i] = b[i];
    e[i] = 0.0;
    if (rowabs) rowabs[i] = 0.0;
  }
  auto acc = [&](int64_t i, double aij, double xj) {
    double pr, pe, ss, se;
    two_prod(-aij, xj, &pr, &pe);
    two_sum(s[i], pr, &ss, &se);
    s[i] = ss;
    e[i] += pe + se;
  };
  for (int64_t j = 0; j < n; ++j) {
    const double* col = a + j * lda;
    const double xj = x[j];
    if (sym) {
      // lower column j: rows i >= j get A(i, j) x_j; row j gets A(i, j) x_i
      // for i > j (the mirrored upper entries A(j, i)).
      acc(j, col[j], xj);
      if (rowabs) rowabs[j] += std::fabs(col[j]);
      for (int64_t i = j + 1; i < n; ++i) {
        acc(i, col[i], xj);
        acc(j, col[i], x[i]);
        if (rowabs) {
          rowabs[i] += std::fabs(col[i]);
          rowabs[j] += std::fabs(col[i]);
        }
      }
    } else {
      for (int64_t i = 0; i < n; ++i) {
        acc(i, col[i], xj);
        if (rowabs) rowabs[i] += std::fabs(col[i]);
      }
    }
  }
  double rmax = 0.0;
  for (int64_t i = 0; i < n; ++i) {
    const double r = std::fabs(s[i] + e[i]);
    if (!(r <= rmax)) rmax = r;  // a NaN residual propagates
  }
  return rmax;
}

double normwise_berr(double rmax, double anorm, const double* x, const double* b, int64_t n) {
  double xmax = 0.0, bmax = 0.0;
  for (int64_t i = 0; i < n; ++i) {
    xmax = std::fmax(xmax, std::fabs(x[i]));
    bmax = std::fmax(bmax, std::fabs(b[i]));
  }
  const double den = anorm * xmax + bmax;
  if (rmax != rmax) return NAN;
  return den > 0.0 ? rmax / den : (rmax > 0.0 ? INFINITY : 0.0);
}
}  // namespace

// Per-system normwise backward error of a ragged batch of solves (max over
// the system's right-hand sides), A taken from its lower triangle when `sym`
// (the SPD solves) or as stored otherwise (the LU solves):
// berr[s] = max_c ||b_c - A x_c||_inf / (||A||_inf ||x_c||_inf + ||b_c||_inf),
// residuals by Dot2.  Systems run in parallel over the host threads.
void orc_dposv_ragged_backward_errors(int64_t count, const int32_t* ns, const int64_t* aoff, const double* a,
                                      const int64_t* boff, const double* b, const double* x, int64_t nrhs,
                                      int sym, double* berr, int nthreads) {
  set_threads(nthreads);
#pragma omp parallel
  {
    std::vector<double> s, e, rowabs;
#pragma omp for schedule(dynamic, 16)
    for (int64_t q = 0; q < count; ++q) {
      const int64_t n = ns[q];
      s.resize(n);
      e.resize(n);
      rowabs.resize(n);
      const double* aq = a + aoff[q];
      double worst = 0.0;
      for (int64_t c = 0; c < nrhs; ++c) {
        const double* bc = b + boff[q] + c * n;
        const double* xc = x + boff[q] + c * n;
        const double rmax = residual_inf_dd(n, aq, n, sym != 0, xc, bc, s.data(), e.data(), c ? nullptr : rowabs.data());
        double anorm = 0.0;
        for (int64_t i = 0; i < n; ++i) anorm = std::fmax(anorm, rowabs[i]);
        const double be = normwise_berr(rmax, anorm, xc, bc, n);
        if (!(be <= worst)) worst = be;
      }
      berr[q] = worst;
    }
  }
}

// Normwise backward error of one large dense system with one right-hand side,
// the residual by Dot2, rows split over the host threads (each thread walks
// every column over its own row block, so A is read by contiguous segments).
double orc_dgesv_backward_error(int64_t n, const double* a, int64_t lda, const double* x, const double* b,
                                int nthreads) {
  set_threads(nthreads);
  std::vector<double> s(n), e(n), rowabs(n, 0.0);
  for (int64_t i = 0; i < n; ++i) {
    s[i] = b[i];
    e[i] = 0.0;
  }
  const int64_t blk = 256;
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t i0 = 0; i0 < n; i0 += blk) {
    const int64_t i1 = i0 + blk < n ? i0 + blk : n;
    for (int64_t j = 0; j < n; ++j) {
      const double* col = a + j * lda;
      const double xj = x[j];
      for (int64_t i = i0; i < i1; ++i) {
        double pr, pe, ss, se;
        two_prod(-col[i], xj, &pr, &pe);
        two_sum(s[i], pr, &ss, &se);
        s[i] = ss;
        e[i] += pe + se;
        rowabs[i] += std::fabs(col[i]);
      }
    }
  }
  double rmax = 0.0, anorm = 0.0;
  for (int64_t i = 0; i < n; ++i) {
    const double r = std::fabs(s[i] + e[i]);
    if (!(r <= rmax)) rmax = r;
    anorm = std::fmax(anorm, rowabs[i]);
  }
  return normwise_berr(rmax, anorm, x, b, n);
}

}  // extern "C"
