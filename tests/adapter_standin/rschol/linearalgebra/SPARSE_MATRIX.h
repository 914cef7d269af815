// Stand-in for the reference's SPARSE_MATRIX (src/rschol/linearalgebra/
// SPARSE_MATRIX.h:57, 187-300): the class name and the CSC fields of its
// nested SparseColumnMatrix, same names and types.
#ifndef STANDIN_SPARSE_MATRIX_H
#define STANDIN_SPARSE_MATRIX_H
#include <cstddef>
#include <rschol/TYPES.h>
#include <rschol/linearalgebra/VECTOR.h>

class SPARSE_MATRIX {
 public:
  struct SparseColumnMatrix {
    SparseColumnMatrix() : _nrow(0), _ncol(0), _nzmax(0), _p(NULL), _i(NULL), _x(NULL) {}
    virtual ~SparseColumnMatrix() {}
    int _nrow;
    int _ncol;
    int _nzmax;
    int *_p;
    int *_i;
    Real *_x;
  };
};
#endif
