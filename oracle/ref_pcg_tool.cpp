// TEST INFRASTRUCTURE: the reference's own PCG loop as a checking library.
//
// Compiled where the reference sources lie (rank_structured_cholesky_gb300/
// _build.py, build_reference_tools) from src/rschol/linearalgebra/
// PCG_SOLVER.cpp, VECTOR_FAST.cpp and SPARSE_MATRIX.cpp, with the shims in
// oracle/ref_shim/ (Boost names, the CMake-written config.h, CBLAS level 1
// as plain loops), into oracle/_ref/libref_pcg.so.  Nothing here changes
// the reference's code: PCG_SOLVER::solvePCG (PCG_SOLVER.cpp:226-363) runs
// as written, with the preconditioner supplied by the caller through a
// callback (in the tests: the CPU oracle's factor), so that iteration counts
// and residuals of the oracle and of the GPU library can be checked against
// the reference's own Krylov loop.
#include <cstdlib>
#include <cstring>

#include <rschol/linearalgebra/PCG_SOLVER.h>

typedef void (*ref_apply_fn)(void *user, const double *b, double *x, int n);

namespace {

// PRECONDITIONER (src/rschol/linearalgebra/PRECONDITIONER.h:54-56) whose
// solve calls back into the caller.
class CallbackPreconditioner : public PRECONDITIONER {
 public:
  CallbackPreconditioner(ref_apply_fn fn, void *user) : _fn(fn), _user(user) {}
  virtual void init() {}
  virtual void init(SPARSE_MATRIX &) {}
  virtual void solve(VECTOR &x, VECTOR &b) {
    if (x.size() != b.size()) x.resizeAndWipe(b.size());
    _fn(_user, b.data(), x.data(), b.size());
  }

 private:
  ref_apply_fn _fn;
  void *_user;
};

}  // namespace

// Runs PCG_SOLVER(A, eps, maxit).solvePCG(x, b, M) from x = 0 on the full
// symmetric CSC matrix (colptr, rowind, vals); returns the iteration count
// and writes the final ||b - A x|| / ||b|| (the reference's closing
// residual, PCG_SOLVER.cpp:351-361) to *residual.
extern "C" __attribute__((visibility("default"))) int ref_pcg_solve(int n, const int *colptr, const int *rowind, const double *vals, const double *b,
                             double *x, double eps, int maxit, ref_apply_fn apply, void *user, double *residual) {
  SPARSE_MATRIX::SparseColumnMatrix A;
  A._nrow = A._ncol = n;
  A._nzmax = colptr[n];
  A.allocate();
  std::memcpy(A._p, colptr, sizeof(int) * (n + 1));
  std::memcpy(A._i, rowind, sizeof(int) * colptr[n]);
  std::memcpy(A._x, vals, sizeof(double) * colptr[n]);
  VECTOR bv(n, b);
  VECTOR xv(n);
  CallbackPreconditioner M(apply, user);
  PCG_SOLVER solver(A, eps, maxit);
  solver.solvePCG(xv, bv, &M);
  std::memcpy(x, xv.data(), sizeof(double) * n);
  if (residual) *residual = solver.residual().norm2() / bv.norm2();
  return (int)(solver.meanIterations() + 0.5);
}
