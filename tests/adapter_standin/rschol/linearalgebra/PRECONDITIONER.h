// Stand-in for the reference's PRECONDITIONER (src/rschol/linearalgebra/
// PRECONDITIONER.h:49-57): the same three pure virtuals.
#ifndef STANDIN_PRECONDITIONER_H
#define STANDIN_PRECONDITIONER_H
#include <rschol/linearalgebra/SPARSE_MATRIX.h>

class PRECONDITIONER {
 public:
  PRECONDITIONER() {}
  virtual ~PRECONDITIONER() {}
  virtual void init() = 0;
  virtual void init(SPARSE_MATRIX &matrix) = 0;
  virtual void solve(VECTOR &x, VECTOR &b) = 0;
};
#endif
