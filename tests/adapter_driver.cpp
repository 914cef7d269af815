// Test driver for include/rschol_gpu_preconditioner.hpp: uses the adapter the
// way the reference's pcg_solver driver uses FactorPreconditioner
// (src/pcg_solver.cpp:98-117) -- initialize() with the driver's arguments,
// then the preconditioner only through the abstract PRECONDITIONER interface.
//
//   adapter_driver <in.bin> <out.bin> [precision]
//
// in.bin:  int32 n, int32 nnz, int32 colptr[n+1], int32 rowind[nnz],
//          float64 vals[nnz], float64 b[n]   (full symmetric CSC)
// out.bin: float64 z[n] = M^{-1} b through PRECONDITIONER::solve,
//          float64 x[n] from a host CG loop preconditioned through
//          PRECONDITIONER::solve, float64 y[n] from the adapter's device PCG,
//          int32 host iterations, int32 device iterations
// Exit status 3 with "error: <message>" on stderr when the library reports a
// failure (e.g. no CUDA device).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <exception>
#include <vector>

#include "rschol_gpu_preconditioner.hpp"

namespace {

double dot(const VECTOR &a, const VECTOR &b) {
  double s = 0;
  for (int i = 0; i < a.size(); ++i) s += a(i) * b(i);
  return s;
}

// y = A x for a full symmetric CSC matrix
void spmv(const SPARSE_MATRIX::SparseColumnMatrix &A, const VECTOR &x, VECTOR &y) {
  for (int i = 0; i < A._nrow; ++i) y[i] = 0.0;
  for (int j = 0; j < A._ncol; ++j)
    for (int p = A._p[j]; p < A._p[j + 1]; ++p) y[A._i[p]] += A._x[p] * x(j);
}

// Preconditioned CG from x = 0, stopping at ||r|| / ||b|| <= eps: the
// recurrences of PCG_SOLVER::solvePCG (PCG_SOLVER.cpp:226-363), driven
// through PRECONDITIONER::solve as the reference's solver drives it.
int host_pcg(const SPARSE_MATRIX::SparseColumnMatrix &A, PRECONDITIONER *M, VECTOR &x, VECTOR &b, double eps,
             int maxit) {
  const int n = b.size();
  x.resizeAndWipe(n);
  VECTOR r(n, b.data()), s(n), d(n), q(n);
  M->solve(d, r);
  double deltaNew = dot(r, d);
  const double bnorm = std::sqrt(dot(b, b));
  int it = 0;
  while (it < maxit && std::sqrt(dot(r, r)) > eps * bnorm) {
    spmv(A, d, q);
    const double alpha = deltaNew / dot(d, q);
    for (int i = 0; i < n; ++i) {
      x[i] += alpha * d(i);
      r[i] -= alpha * q(i);
    }
    M->solve(s, r);
    const double deltaOld = deltaNew;
    deltaNew = dot(r, s);
    const double beta = deltaNew / deltaOld;
    for (int i = 0; i < n; ++i) d[i] = s(i) + beta * d(i);
    ++it;
  }
  return it;
}

}  // namespace

int main(int argc, char **argv) {
  if (argc < 3) {
    std::fprintf(stderr, "usage: %s in.bin out.bin [precision]\n", argv[0]);
    return 2;
  }
  FILE *in = std::fopen(argv[1], "rb");
  if (!in) return 2;
  int n = 0, nnz = 0;
  if (std::fread(&n, 4, 1, in) != 1 || std::fread(&nnz, 4, 1, in) != 1) return 2;
  std::vector<int> p(n + 1), ix(nnz);
  std::vector<double> v(nnz), bv(n);
  if (std::fread(p.data(), 4, n + 1, in) != (size_t)n + 1 || std::fread(ix.data(), 4, nnz, in) != (size_t)nnz ||
      std::fread(v.data(), 8, nnz, in) != (size_t)nnz || std::fread(bv.data(), 8, n, in) != (size_t)n)
    return 2;
  std::fclose(in);

  SPARSE_MATRIX::SparseColumnMatrix A;
  A._nrow = A._ncol = n;
  A._nzmax = nnz;
  A._p = p.data();
  A._i = ix.data();
  A._x = v.data();
  Vector3Array positions(n, VEC3F(0.0, 0.0, 0.0));
  VECTOR b(n, bv.data()), z, x, y;
  int hostIt = 0, devIt = 0;
  try {
    GpuFactorPreconditioner gpu(argc > 3 ? std::atoi(argv[3]) : RSCHOL_FP64);
    gpu.initialize(A, positions, 200, 400, CHOLESKY, IN_PLACE, DECOMPOSE_TRANSPOSE, DECOMPOSE_FACTOR, false);
    PRECONDITIONER *M = &gpu;
    M->init();
    M->solve(z, b);
    hostIt = host_pcg(A, M, x, b, 1e-8, 1000);
    devIt = gpu.solvePCG(y, b, 1e-8, 1000);
  } catch (const std::exception &e) {
    std::fprintf(stderr, "error: %s\n", e.what());
    A._p = A._i = NULL;
    A._x = NULL;
    return 3;
  }
  A._p = A._i = NULL;
  A._x = NULL;
  FILE *out = std::fopen(argv[2], "wb");
  if (!out) return 2;
  std::fwrite(z.data(), 8, n, out);
  std::fwrite(x.data(), 8, n, out);
  std::fwrite(y.data(), 8, n, out);
  std::fwrite(&hostIt, 4, 1, out);
  std::fwrite(&devIt, 4, 1, out);
  std::fclose(out);
  std::printf("n=%d host_iterations=%d device_iterations=%d\n", n, hostIt, devIt);
  return 0;
}
