// TEST INFRASTRUCTURE: known-answer generator built against the reference's
// own MERSENNETWISTER class (src/rschol/util/MERSENNETWISTER.h), compiled
// where the reference sources lie (recipe: rank_structured_cholesky_gb300/
// _build.py build_reference_tools, output in oracle/_ref/).
//
// Prints, for a seed, N raw randInt() draws, then N randNorm(0, 1) values
// from a freshly seeded generator (exactly what MathUtil::randomGaussianMatrix
// consumes, src/rschol/util/MathUtil.cpp:100-111), as text with %.17g.
#include <cstdio>
#include <cstdlib>

#include "MERSENNETWISTER.h"

int main(int argc, char** argv) {
  unsigned long seed = argc > 1 ? std::strtoul(argv[1], nullptr, 10) : 152;
  long n = argc > 2 ? std::strtol(argv[2], nullptr, 10) : 16;
  MERSENNETWISTER a(seed);
  for (long i = 0; i < n; ++i) std::printf("%lu\n", (unsigned long)a.randInt());
  MERSENNETWISTER b(seed);
  for (long i = 0; i < n; ++i) std::printf("%.17g\n", b.randNorm(0.0, 1.0));
  return 0;
}
