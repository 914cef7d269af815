// TEST INFRASTRUCTURE (CPU oracle) -- not part of the shipped library.
//
// Row-major dense kernels with the semantics of the reference's MATRIX
// wrappers (src/rschol/linearalgebra/MATRIX_FAST.cpp:1095-1180 qr /
// extractQRfactor, 1758-1960 gemm / syrk, 2086-2105 cholesky, 3049-3140
// triangularSolve).  The reference calls CBLAS/LAPACKE; this oracle calls
// the Fortran BLAS/LAPACK that ships inside scipy (pointers taken from
// scipy.linalg.cython_blas / cython_lapack capsules and handed over by the
// Python side) and falls back to plain loops when no table is set.
#pragma once
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

namespace oracle {

typedef void (*dgemm_t)(const char*, const char*, const int*, const int*, const int*, const double*,
                        const double*, const int*, const double*, const int*, const double*, double*,
                        const int*);
typedef void (*dtrsm_t)(const char*, const char*, const char*, const char*, const int*, const int*,
                        const double*, const double*, const int*, double*, const int*);
typedef void (*dpotrf_t)(const char*, const int*, double*, const int*, int*);
typedef void (*dgeqrf_t)(const int*, const int*, double*, const int*, double*, double*, const int*, int*);
typedef void (*dorgqr_t)(const int*, const int*, const int*, double*, const int*, const double*, double*,
                         const int*, int*);

struct BlasTable {
  dgemm_t gemm = nullptr;
  dtrsm_t trsm = nullptr;
  dpotrf_t potrf = nullptr;
  dgeqrf_t geqrf = nullptr;
  dorgqr_t orgqr = nullptr;
};
extern BlasTable g_blas;

// C (MxN) = alpha * op(A) * op(B) + beta * C, row-major.
inline void gemm(int M, int N, int K, double alpha, const double* A, int lda, bool tA, const double* B,
                 int ldb, bool tB, double beta, double* C, int ldc) {
  if (M <= 0 || N <= 0) return;
  if (K <= 0) {
    for (int i = 0; i < M; ++i)
      for (int j = 0; j < N; ++j) C[(size_t)i * ldc + j] = beta == 0.0 ? 0.0 : beta * C[(size_t)i * ldc + j];
    return;
  }
  if (g_blas.gemm) {
    const char ta = tA ? 'T' : 'N', tb = tB ? 'T' : 'N';
    g_blas.gemm(&tb, &ta, &N, &M, &K, &alpha, B, &ldb, A, &lda, &beta, C, &ldc);
    return;
  }
  std::vector<double> row(N);
  for (int i = 0; i < M; ++i) {
    std::fill(row.begin(), row.end(), 0.0);
    for (int k = 0; k < K; ++k) {
      double a = tA ? A[(size_t)k * lda + i] : A[(size_t)i * lda + k];
      if (a == 0.0) continue;
      if (!tB) {
        const double* b = B + (size_t)k * ldb;
        for (int j = 0; j < N; ++j) row[j] += a * b[j];
      } else {
        for (int j = 0; j < N; ++j) row[j] += a * B[(size_t)j * ldb + k];
      }
    }
    double* c = C + (size_t)i * ldc;
    for (int j = 0; j < N; ++j) c[j] = alpha * row[j] + (beta == 0.0 ? 0.0 : beta * c[j]);
  }
}

// Lower Cholesky in place (row-major); returns LAPACK info (0 = ok).
inline int potrf(int n, double* A, int lda) {
  if (n <= 0) return 0;
  if (g_blas.potrf) {
    int info = 0;
    const char u = 'U';
    g_blas.potrf(&u, &n, A, &lda, &info);
    return info;
  }
  for (int j = 0; j < n; ++j) {
    double d = A[(size_t)j * lda + j];
    for (int k = 0; k < j; ++k) d -= A[(size_t)j * lda + k] * A[(size_t)j * lda + k];
    if (!(d > 0.0)) return j + 1;
    d = std::sqrt(d);
    A[(size_t)j * lda + j] = d;
    for (int i = j + 1; i < n; ++i) {
      double s = A[(size_t)i * lda + j];
      for (int k = 0; k < j; ++k) s -= A[(size_t)i * lda + k] * A[(size_t)j * lda + k];
      A[(size_t)i * lda + j] = s / d;
    }
  }
  return 0;
}

// B (m x n) := B * L^{-T}, L (n x n) lower, row-major.
inline void trsm_right_lt(int m, int n, const double* L, int ldl, double* B, int ldb) {
  if (m <= 0 || n <= 0) return;
  if (g_blas.trsm) {
    const char s = 'L', u = 'U', t = 'T', d = 'N';
    const double one = 1.0;
    g_blas.trsm(&s, &u, &t, &d, &n, &m, &one, L, &ldl, B, &ldb);
    return;
  }
  for (int i = 0; i < m; ++i) {
    double* b = B + (size_t)i * ldb;
    for (int j = 0; j < n; ++j) {
      double s = b[j];
      for (int k = 0; k < j; ++k) s -= b[k] * L[(size_t)j * ldl + k];
      b[j] = s / L[(size_t)j * ldl + j];
    }
  }
}

// B (n x k) := L^{-1} B  (trans = false)  or  L^{-T} B  (trans = true).
inline void trsm_left(int n, int k, const double* L, int ldl, bool trans, double* B, int ldb) {
  if (n <= 0 || k <= 0) return;
  if (g_blas.trsm) {
    const char s = 'R', u = 'U', t = trans ? 'T' : 'N', d = 'N';
    const double one = 1.0;
    g_blas.trsm(&s, &u, &t, &d, &k, &n, &one, L, &ldl, B, &ldb);
    return;
  }
  if (!trans) {
    for (int i = 0; i < n; ++i) {
      double* bi = B + (size_t)i * ldb;
      for (int j = 0; j < i; ++j) {
        double l = L[(size_t)i * ldl + j];
        if (l == 0.0) continue;
        const double* bj = B + (size_t)j * ldb;
        for (int c = 0; c < k; ++c) bi[c] -= l * bj[c];
      }
      double d = L[(size_t)i * ldl + i];
      for (int c = 0; c < k; ++c) bi[c] /= d;
    }
  } else {
    for (int i = n - 1; i >= 0; --i) {
      double* bi = B + (size_t)i * ldb;
      for (int j = i + 1; j < n; ++j) {
        double l = L[(size_t)j * ldl + i];
        if (l == 0.0) continue;
        const double* bj = B + (size_t)j * ldb;
        for (int c = 0; c < k; ++c) bi[c] -= l * bj[c];
      }
      double d = L[(size_t)i * ldl + i];
      for (int c = 0; c < k; ++c) bi[c] /= d;
    }
  }
}

// Thin QR: Y (n x r, row-major) is overwritten with the orthonormal factor Q
// (LAPACK geqrf + orgqr, as MATRIX::qr + MATRIX::extractQRfactor).
inline void thin_q(int n, int r, double* Y) {
  if (n <= 0 || r <= 0) return;
  std::vector<double> A((size_t)n * r), tau(r);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < r; ++j) A[(size_t)j * n + i] = Y[(size_t)i * r + j];   // column-major copy
  if (g_blas.geqrf && g_blas.orgqr) {
    int info = 0, lwork = -1;
    double wq = 0;
    g_blas.geqrf(&n, &r, A.data(), &n, tau.data(), &wq, &lwork, &info);
    lwork = std::max(1, (int)wq);
    std::vector<double> work(lwork);
    g_blas.geqrf(&n, &r, A.data(), &n, tau.data(), work.data(), &lwork, &info);
    lwork = -1;
    g_blas.orgqr(&n, &r, &r, A.data(), &n, tau.data(), &wq, &lwork, &info);
    lwork = std::max(1, (int)wq);
    work.assign(lwork, 0.0);
    g_blas.orgqr(&n, &r, &r, A.data(), &n, tau.data(), work.data(), &lwork, &info);
  } else {
    // Householder QR (Golub & Van Loan, Alg. 5.2.1) then backward accumulation.
    std::vector<std::vector<double>> vs(r);
    for (int j = 0; j < r; ++j) {
      double* a = &A[(size_t)j * n];
      double nrm = 0;
      for (int i = j; i < n; ++i) nrm += a[i] * a[i];
      nrm = std::sqrt(nrm);
      std::vector<double> v(n, 0.0);
      double alpha = a[j] >= 0 ? -nrm : nrm;
      for (int i = j; i < n; ++i) v[i] = a[i];
      v[j] -= alpha;
      double vn = 0;
      for (int i = j; i < n; ++i) vn += v[i] * v[i];
      if (vn > 0)
        for (int c = j; c < r; ++c) {
          double* ac = &A[(size_t)c * n];
          double s = 0;
          for (int i = j; i < n; ++i) s += v[i] * ac[i];
          s = 2 * s / vn;
          for (int i = j; i < n; ++i) ac[i] -= s * v[i];
        }
      vs[j] = v;
      (void)vn;
    }
    std::fill(A.begin(), A.end(), 0.0);
    for (int j = 0; j < r; ++j) A[(size_t)j * n + j] = 1.0;
    for (int j = r - 1; j >= 0; --j) {
      const std::vector<double>& v = vs[j];
      double vn = 0;
      for (int i = j; i < n; ++i) vn += v[i] * v[i];
      if (vn == 0) continue;
      for (int c = 0; c < r; ++c) {
        double* ac = &A[(size_t)c * n];
        double s = 0;
        for (int i = j; i < n; ++i) s += v[i] * ac[i];
        s = 2 * s / vn;
        for (int i = j; i < n; ++i) ac[i] -= s * v[i];
      }
    }
  }
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < r; ++j) Y[(size_t)i * r + j] = A[(size_t)j * n + i];
}

}  // namespace oracle
