// Synthetic SPD systems with the shapes and value distributions of the
// workloads this library is measured on.  The reference ships a constant
// coefficient finite-difference generator (src/rschol/geometry/
// FiniteDifference.cpp:54) and an uncompiled Q1 hex element
// (src/rschol/mesh/IsoHexElement.cpp:283); these generators are written
// fresh: variable-coefficient cell-centred diffusion with harmonic-mean
// faces, and trilinear hexahedral linear elasticity.
//
// Every random value comes from one MT19937 stream seeded with the problem
// seed, drawn with the reference's randNorm / randExc conventions: first the
// cell coefficients (natural cell order), then the right-hand sides
// (column by column).
#pragma once
#include <cstdint>
#include <vector>

namespace rschol {

struct Problem {
  int n = 0;                     // number of unknowns
  std::vector<int> colptr;       // CSC, full symmetric storage, sorted rows
  std::vector<int> rowind;
  std::vector<double> vals;
  std::vector<double> xyz;       // 3 coordinates per unknown
  int nrhs = 0;
  std::vector<double> rhs;       // n * nrhs, column-major
};

// 2D 5-point (d=2) or 3D 7-point (d=3) cell-centred diffusion on an
// nx*ny*nz interior grid with Dirichlet boundary, h = 1.  Cell coefficients
// kappa = exp(sigma * N(0,1)) (sigma = 0 gives the constant-coefficient
// Poisson matrix).  Interior faces use the harmonic mean of the two cells,
// boundary faces use the cell's own coefficient.
Problem make_diffusion(int dim, int nx, int ny, int nz, double sigma,
                       uint32_t seed, int nrhs);

// Trilinear (Q1) hexahedral linear elasticity on an ne^3 unit-cube mesh
// (h = 1/ne), Young's modulus E, Poisson ratio nu, 2x2x2 Gauss quadrature,
// the x = 0 face clamped (its dofs eliminated).  Right-hand sides are
// nodal loads uniform in [-1, 1].
Problem make_elasticity(int ne, double E, double nu, uint32_t seed, int nrhs);

}  // namespace rschol
