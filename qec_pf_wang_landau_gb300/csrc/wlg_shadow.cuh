// Float shadows of FP64 log g differences, formed with integer arithmetic.
//
// The main-run sweep decides acceptances from FP32 copies ("shadows") of
// each walker's log g relative to a per-sweep base.  Forming a shadow as
// float(g - base) costs an FP64 subtraction and an FP64->FP32 conversion,
// both on GB300's narrow FP64 pipe; on every change of energy bin that
// pair sat on the walker's serial path.  Splitting each double into a float
// of its leading 24 significand bits and a float of the rest (bit
// operations) gives the difference from three float subtractions and adds.
#pragma once

#include <cstdint>

namespace wlg {

// g = hi + lo for a double g >= 0: hi = g with its significand truncated to
// float precision (exact), lo = the remaining 29 significand bits as a float
// (one rounding, |error| <= 2^-47 g).  Integer operations only.  Below
// 2^-74 lo is 0 (error < 2^-97), below 2^-126 both are (error < 2^-126); g
// must be below 2^128.
struct Split {
  float hi, lo;
};

__device__ __forceinline__ Split split_float(double g)
{
  const long long b = __double_as_longlong(g);
  const int e = static_cast<int>(b >> 52);
  const uint32_t hw = static_cast<uint32_t>(b >> 32), lw = static_cast<uint32_t>(b);
  const float hi = __uint_as_float((static_cast<uint32_t>(e - 896) << 23) | ((hw & 0xFFFFFu) << 3) | (lw >> 29));
  const float lo = __uint2float_rn(lw & 0x1FFFFFFFu) * __uint_as_float(static_cast<uint32_t>(max(e - 948, 0)) << 23);
  const bool tiny = e < 897;
  return Split{tiny ? 0.0f : hi, tiny ? 0.0f : lo};
}

// float(g - base) from the splits: (hi - base.hi) + (lo - base.lo).  Error
// <= 2^-23 |result| + 2^-44 (g + base): the hi difference is exact when the
// values are within a factor 2 (else one rounding of it), the lo terms are
// below 2^-22 of the values, and the sum is rounded once.
__device__ __forceinline__ float shadow_split(double g, const Split& base)
{
  const Split a = split_float(g);
  return (a.hi - base.hi) + (a.lo - base.lo);
}

}  // namespace wlg
