// The Wang-Landau acceptance u < min(1, exp(d)) (wl.cu:1113-1116) decided in
// FP32 where that is provably the reference's FP64 answer.
//
// u is the float uniform of a 32-bit draw x (curand_uniform: in (0, 1]) and
// d = log g(E) - log g(E') is known only as an FP32 estimate df with
// |df - d| <= eps.  For u < 1 the test equals log u < d, and log u depends on
// the draw alone, so it is formed off the walker's serial path; after df the
// decision costs one subtraction and one comparison.  The reference rounds
// exp(d) to double before comparing, which can matter only within ~2^-52 of
// the boundary, far inside the band left to the exact FP64 test.
#pragma once

#include <cstdint>

#include "wlg_rng.cuh"

namespace wlg {

// Bound on |__logf(u) - log(u)| over every float u in [2^-33, 1] (all values
// a uniform can take), checked exhaustively against FP64 log on the device.
constexpr float kLogAbsErr = 4.0e-6f;

__device__ __forceinline__ float log_uniform(uint32_t x) { return __logf(unit_float(x)); }

struct Decision {
  bool acc;    // the reference's answer, when known
  bool known;  // false: |log u - d| may be below the error bounds; decide in FP64
};

// same: the proposal keeps the energy (d = 0 exactly).  lu = log_uniform(x).
__device__ __forceinline__ Decision decide(uint32_t x, float lu, float df, float eps, bool same)
{
  const bool one = x >= 0xFFFFFF80u;  // u rounds to 1: never below min(1, .)
  // |lu - df| > eps + kLogAbsErr separates log u from d; the computed
  // difference is within 2^-24 of the true one, hence the (1 + 2^-23)
  const float m = eps * (1.0f + 0x1p-23f) + kLogAbsErr * (1.0f + 0x1p-23f);
  const float diff = lu - df;
  Decision r;
  r.acc = !one && (same || diff < 0.0f);
  r.known = one || same || fabsf(diff) > m;
  return r;
}

}  // namespace wlg
