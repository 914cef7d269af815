// Host-only entry points of the C ABI: synthetic problem generators and the
// symbolic summary used by benchmarks and tests (declared in
// include/rschol_gpu.h).
#include <cstring>
#include <exception>
#include <string>

#include "ordering.h"
#include "problems.h"
#include "rng.h"
#include "symbolic.h"

extern "C" {

void* rschol_problem_diffusion(int dim, int nx, int ny, int nz, double sigma, unsigned seed, int nrhs) {
  try {
    return new rschol::Problem(rschol::make_diffusion(dim, nx, ny, nz, sigma, seed, nrhs));
  } catch (const std::exception&) {
    return nullptr;
  }
}

void* rschol_problem_elasticity(int ne, double E, double nu, unsigned seed, int nrhs) {
  try {
    return new rschol::Problem(rschol::make_elasticity(ne, E, nu, seed, nrhs));
  } catch (const std::exception&) {
    return nullptr;
  }
}

int rschol_problem_n(const void* p) { return ((const rschol::Problem*)p)->n; }
long long rschol_problem_nnz(const void* p) { return (long long)((const rschol::Problem*)p)->rowind.size(); }
int rschol_problem_nrhs(const void* p) { return ((const rschol::Problem*)p)->nrhs; }

void rschol_problem_get(const void* p, int* colptr, int* rowind, double* vals, double* xyz, double* rhs) {
  const rschol::Problem& P = *(const rschol::Problem*)p;
  if (colptr) std::memcpy(colptr, P.colptr.data(), sizeof(int) * P.colptr.size());
  if (rowind) std::memcpy(rowind, P.rowind.data(), sizeof(int) * P.rowind.size());
  if (vals) std::memcpy(vals, P.vals.data(), sizeof(double) * P.vals.size());
  if (xyz) std::memcpy(xyz, P.xyz.data(), sizeof(double) * P.xyz.size());
  if (rhs) std::memcpy(rhs, P.rhs.data(), sizeof(double) * P.rhs.size());
}

void rschol_problem_free(void* p) { delete (rschol::Problem*)p; }

// MT19937 draws with the reference's conventions, for known-answer tests.
void rschol_mt_draws(unsigned seed, long long count, unsigned* out) {
  rschol::MT19937 g(seed);
  g.rawDraws(count, out);
}

void rschol_mt_gaussians(unsigned seed, long long count, double* out) {
  rschol::MT19937 g(seed);
  g.gaussianMatrix(count, out);
}

}  // extern "C"
