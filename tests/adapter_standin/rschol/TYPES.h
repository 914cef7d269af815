// Stand-in for the reference's src/rschol/TYPES.h (and SETTINGS.h): only the
// declarations the GPU preconditioner adapter uses, with the reference's
// names and types (Real = double, SETTINGS.h:62-66; Vector3Array,
// TYPES.h:58; the factor-type enums, TYPES.h:135-160).  Test scaffolding for
// compiling include/rschol_gpu_preconditioner.hpp without the reference's
// Boost-dependent headers.
#ifndef STANDIN_TYPES_H
#define STANDIN_TYPES_H
#include <vector>

typedef double Real;

struct VEC3F {
  Real v[3];
  VEC3F(Real x = 0, Real y = 0, Real z = 0) { v[0] = x; v[1] = y; v[2] = z; }
  Real operator[](int i) const { return v[i]; }
  Real &operator[](int i) { return v[i]; }
};
typedef std::vector<VEC3F> Vector3Array;

enum ExtendedFactorType { CHOLESKY = 0, LDL };
enum CompressionType { EXTENDED_VARIABLE = 0, IN_PLACE };
enum DecompositionBlock { DECOMPOSE_STANDARD = 0, DECOMPOSE_TRANSPOSE };
enum DecompositionType { DECOMPOSE_SCHUR = 0, DECOMPOSE_FACTOR };
#endif
