// Mersenne Twister MT19937 with the draw conventions of the reference's
// MERSENNETWISTER class (src/rschol/util/MERSENNETWISTER.h:69-330) and the
// Gaussian matrix fill of MathUtil::randomGaussianMatrix
// (src/rschol/util/MathUtil.cpp:100-111).
//
// The generator is the published Matsumoto-Nishimura MT19937 with the
// 2002 "init_genrand" seeding (multiplier 1812433253).  On top of the raw
// 32-bit stream the reference defines:
//   randExc()    = u * 2^-32                      in [0,1)
//   randDblExc() = (u + 0.5) * 2^-32              in (0,1)
//   randNorm(m,v)= m + sqrt(-2 log(1 - randDblExc())) * v * cos(2 pi randExc())
// (the reference multiplies by the *variance*, which equals the standard
// deviation for the unit variance used on the factorisation path).  Each
// Gaussian consumes exactly two 32-bit draws, first for the radius and then
// for the angle; the sketch matrices are filled row-major, one draw per entry.
#pragma once
#include <cmath>
#include <cstdint>

namespace rschol {

class MT19937 {
 public:
  static constexpr int N = 624;
  static constexpr int M = 397;

  explicit MT19937(uint32_t s = 152u) { seed(s); }

  void seed(uint32_t s) {
    state_[0] = s;
    for (int i = 1; i < N; ++i)
      state_[i] = 1812433253u * (state_[i - 1] ^ (state_[i - 1] >> 30)) + (uint32_t)i;
    reload();
  }

  uint32_t randInt() {
    if (left_ == 0) reload();
    --left_;
    uint32_t y = state_[next_++];
    y ^= (y >> 11);
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    return y ^ (y >> 18);
  }

  double randExc() { return double(randInt()) * (1.0 / 4294967296.0); }
  double randDblExc() { return (double(randInt()) + 0.5) * (1.0 / 4294967296.0); }

  double randNorm(double mean = 0.0, double variance = 1.0) {
    double r = std::sqrt(-2.0 * std::log(1.0 - randDblExc())) * variance;
    double phi = 2.0 * 3.14159265358979323846264338328 * randExc();
    return mean + r * std::cos(phi);
  }

  // Fill nRows x nCols row-major with unit Gaussians, in the reference's order.
  void gaussianMatrix(long long count, double* out) {
    for (long long i = 0; i < count; ++i) out[i] = randNorm(0.0, 1.0);
  }

  // Raw 32-bit draws (two per Gaussian) for a device-side Box-Muller transform:
  // the same stream as count calls of randInt(), tempered a whole state
  // block at a time.
  void rawDraws(long long count, uint32_t* out) {
    while (count > 0) {
      if (left_ == 0) reload();
      const int k = (int)(count < left_ ? count : left_);
      const uint32_t* src = state_ + next_;
      for (int i = 0; i < k; ++i) {
        uint32_t y = src[i];
        y ^= (y >> 11);
        y ^= (y << 7) & 0x9d2c5680u;
        y ^= (y << 15) & 0xefc60000u;
        out[i] = y ^ (y >> 18);
      }
      next_ += k;
      left_ -= k;
      out += k;
      count -= k;
    }
  }

 private:
  static uint32_t twist(uint32_t m, uint32_t s0, uint32_t s1) {
    uint32_t mix = (s0 & 0x80000000u) | (s1 & 0x7fffffffu);
    return m ^ (mix >> 1) ^ ((0u - (s1 & 1u)) & 0x9908b0dfu);
  }
  void reload() {
    int i = 0;
    for (; i < N - M; ++i) state_[i] = twist(state_[i + M], state_[i], state_[i + 1]);
    for (; i < N - 1; ++i) state_[i] = twist(state_[i + M - N], state_[i], state_[i + 1]);
    state_[N - 1] = twist(state_[M - 1], state_[N - 1], state_[0]);
    left_ = N;
    next_ = 0;
  }

  uint32_t state_[N];
  int left_ = 0;
  int next_ = 0;
};

}  // namespace rschol
