/*
 * rschol_gpu_preconditioner.hpp -- a PRECONDITIONER backed by the GB300
 * library, for the reference's own C++ code.
 *
 * Drop-in for FactorPreconditioner (src/rschol/solver/FactorPreconditioner.h:
 * 60-113): the same initialize() arguments, and the three pure virtuals of
 * PRECONDITIONER (src/rschol/linearalgebra/PRECONDITIONER.h:54-56), so that
 * PCG_SOLVER::solvePCG(x, b, &M) (src/rschol/linearalgebra/PCG_SOLVER.h:59)
 * and the pcg_solver driver (src/pcg_solver.cpp:98-117) run unchanged with
 * the factor and its application on the GPU.
 *
 * Build: put this directory and the reference's src/ on the include path and
 * link librschol_gb300.so.  Header-only; the reference types it uses are
 * SPARSE_MATRIX::SparseColumnMatrix {_nrow, _ncol, _p, _i, _x}, VECTOR
 * {size, data, resizeAndWipe}, Vector3Array and the factor-type enums of
 * src/rschol/TYPES.h.
 *
 * Errors: the reference aborts on a factor that stays indefinite after its
 * retries (src/rschol/solver/SparseSolver.cpp:206-207); this adapter throws
 * std::runtime_error with the library's message instead, and rejects the
 * factor variants the library does not implement (LDL, EXTENDED_VARIABLE,
 * DECOMPOSE_STANDARD, DECOMPOSE_SCHUR) with std::invalid_argument.
 */
#ifndef RSCHOL_GPU_PRECONDITIONER_HPP
#define RSCHOL_GPU_PRECONDITIONER_HPP

#include <rschol/TYPES.h>
#include <rschol/linearalgebra/PRECONDITIONER.h>
#include <rschol/linearalgebra/SPARSE_MATRIX.h>
#include <rschol/linearalgebra/VECTOR.h>

#include <iostream>
#include <stdexcept>
#include <string>
#include <vector>

#include "rschol_gpu.h"

class GpuFactorPreconditioner : public PRECONDITIONER {
 public:
  /* precision: RSCHOL_FP64 (the reference's arithmetic) or RSCHOL_MIXED
   * (FP32 factor, the PCG recurrences stay FP64) */
  explicit GpuFactorPreconditioner(int precision = RSCHOL_FP64, int device = 0) {
    rschol_default_params(&_params);
    _params.precision = precision;
    _params.device = device;
  }

  virtual ~GpuFactorPreconditioner() { release(); }

  /* FactorPreconditioner::initialize (FactorPreconditioner.h:92-103): ordering,
   * symbolic and numeric factorisation of `matrix` (full symmetric CSC).
   * meshPositions are used for the separator sub-ordering when
   * reorderSeparators is set, as in the reference. */
  void initialize(const SPARSE_MATRIX::SparseColumnMatrix &matrix, const Vector3Array &meshPositions,
                  int maxDenseBlock, int maxDiagonalBlock, ExtendedFactorType extFactorType,
                  CompressionType compressionType, DecompositionBlock blockType, DecompositionType decompType,
                  bool reorderSeparators) {
    if (extFactorType != CHOLESKY || compressionType != IN_PLACE || blockType != DECOMPOSE_TRANSPOSE ||
        decompType != DECOMPOSE_FACTOR)
      throw std::invalid_argument(
          "GpuFactorPreconditioner: only CHOLESKY, IN_PLACE, DECOMPOSE_TRANSPOSE, DECOMPOSE_FACTOR are implemented");
    if (matrix._nrow != matrix._ncol || matrix._p == NULL)
      throw std::invalid_argument("GpuFactorPreconditioner: the matrix must be square CSC");
    release();
    _params.max_dense_block = maxDenseBlock;
    _params.max_diag_block = maxDiagonalBlock;
    _params.reorder_separators = reorderSeparators ? 1 : 0;
    _ctx = rschol_create(&_params);
    if (_ctx == NULL) throw std::runtime_error("GpuFactorPreconditioner: rschol_create failed");
    std::vector<double> xyz;
    if (reorderSeparators && (int)meshPositions.size() >= matrix._nrow) {
      xyz.resize(3 * (size_t)matrix._nrow);
      for (int i = 0; i < matrix._nrow; ++i)
        for (int d = 0; d < 3; ++d) xyz[3 * (size_t)i + d] = meshPositions[i][d];
    }
    const int st = rschol_factor_create(_ctx, matrix._nrow, matrix._p, matrix._i, matrix._x,
                                        xyz.empty() ? NULL : xyz.data(), &_factor);
    if (st != RSCHOL_OK) fail("rschol_factor_create", st);
  }

  /* New values with the same pattern (numeric factorisation only). */
  void refactor(const SPARSE_MATRIX::SparseColumnMatrix &matrix) {
    require_factor("refactor");
    const int st = rschol_refactor(_factor, matrix._x);
    if (st != RSCHOL_OK) fail("rschol_refactor", st);
  }

  /* PRECONDITIONER::init() -- as FactorPreconditioner, the factor is built by
   * initialize() outside the PCG solver, so there is nothing to do here. */
  virtual void init() {}

  /* PRECONDITIONER::init(SPARSE_MATRIX &) -- not implemented by the
   * reference's FactorPreconditioner either (FactorPreconditioner.h:107-111),
   * which prints the same notice. */
  virtual void init(SPARSE_MATRIX &matrix) {
    (void)matrix;
    std::cerr << "GpuFactorPreconditioner::init(SPARSE_MATRIX &) not implemented" << std::endl;
  }

  /* PRECONDITIONER::solve: x = M^{-1} b (FactorPreconditioner::solve,
   * FactorPreconditioner.cpp:135-162), permutation included. */
  virtual void solve(VECTOR &x, VECTOR &b) {
    require_factor("solve");
    if (x.size() != b.size()) x.resizeAndWipe(b.size());
    const int st = rschol_precond_apply(_factor, b.data(), x.data(), 1);
    if (st != RSCHOL_OK) fail("rschol_precond_apply", st);
  }

  /* The whole PCG on the device (PCG_SOLVER::solvePCG's recurrences, x0 = 0,
   * stop at ||r|| / ||b|| <= eps): one call instead of `iterations` host round
   * trips through solve().  Returns the iteration count. */
  int solvePCG(VECTOR &x, VECTOR &b, double eps, int iterations, rschol_pcg_info *info = NULL) {
    require_factor("solvePCG");
    if (x.size() != b.size()) x.resizeAndWipe(b.size());
    rschol_pcg_info local;
    const int st = rschol_pcg(_factor, b.data(), x.data(), 1, eps, iterations, info ? info : &local);
    if (st != RSCHOL_OK && st != RSCHOL_E_BREAKDOWN) fail("rschol_pcg", st);
    return (info ? info : &local)->iterations;
  }

  rschol_factor *factor() { return _factor; }

 private:
  void require_factor(const char *what) const {
    if (_factor == NULL)
      throw std::runtime_error(std::string("GpuFactorPreconditioner::") + what + " before initialize()");
  }

  void fail(const char *what, int status) {
    const std::string msg = std::string("GpuFactorPreconditioner: ") + what + " returned status " +
                            std::to_string(status) + ": " + (_ctx ? rschol_last_error(_ctx) : "");
    throw std::runtime_error(msg);
  }

  void release() {
    if (_factor) rschol_factor_free(_factor);
    if (_ctx) rschol_destroy(_ctx);
    _factor = NULL;
    _ctx = NULL;
  }

  GpuFactorPreconditioner(const GpuFactorPreconditioner &);
  GpuFactorPreconditioner &operator=(const GpuFactorPreconditioner &);

  rschol_params _params;
  rschol_ctx *_ctx = NULL;
  rschol_factor *_factor = NULL;
};

#endif /* RSCHOL_GPU_PRECONDITIONER_HPP */
