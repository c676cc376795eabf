// Float shadows of FP64 log g differences, formed with integer arithmetic.
//
// The main-run sweep decides acceptances from FP32 copies ("shadows") of
// each walker's log g relative to a per-sweep base.  Forming a shadow as
// float(g - base) costs an FP64 subtraction and an FP64->FP32 conversion,
// both on GB300's narrow FP64 pipe; on every change of energy bin that
// pair sat on the walker's serial path.  On a common grid the difference of
// two doubles is an integer, so the shadow needs only integer operations and
// one int->float rounding.
#pragma once

#include <cstdint>

namespace wlg {

// Exponent field and 53-bit significand of a non-negative double (zero and
// subnormals give a zero significand).
struct Bits {
  int e;
  long long m;
};

__device__ __forceinline__ Bits split_bits(double g)
{
  const long long b = __double_as_longlong(g);
  const int e = static_cast<int>(b >> 52);
  return Bits{e, e == 0 ? 0ll : (b & 0xFFFFFFFFFFFFFll) | 0x10000000000000ll};
}

__device__ __forceinline__ long long shift_signed(long long m, int k)  // m 2^k, truncated; m >= 0, k <= 10
{
  return k >= 0 ? (m << k) : (k <= -63 ? 0ll : (m >> -k));
}

// float(g - base) for non-negative doubles without FP64 arithmetic.  Both
// significands are put on the grid 2^(emax - 1085), emax the larger
// exponent: the larger operand becomes an integer below 2^63 exactly, a
// smaller one more than ten binades down loses bits below the grid (< 1 unit,
// while |difference| >= 2^61 units then).  The top 31 bits of the integer
// difference are converted (one rounding) and scaled by a power of two.
// Relative error <= 2^-24 + 2^-30 (+ 2^-61), i.e. one float rounding of the
// exact difference.  Two values both below 2^-63 give 0 (absolute error
// < 2^-63); a value of 2^77 or more gives NaN.
__device__ __forceinline__ float shadow_of(double g, const Bits& base)
{
  const Bits a = split_bits(g);
  const int emax = max(a.e, base.e);
  const int qe = emax - 10;
  const long long D = shift_signed(a.m, a.e - qe) - shift_signed(base.m, base.e - qe);
  const unsigned long long mag = static_cast<unsigned long long>(D < 0 ? -D : D);
  const int sh = max(0, 33 - __clzll(static_cast<long long>(mag)));
  const int hi = static_cast<int>(D >> sh);
  const float v = __int2float_rn(hi) * __int_as_float((emax - 958 + sh) << 23);  // 2^(qe - 1075 + sh)
  return emax > 1100 ? __int_as_float(0x7FC00000) : (emax < 959 ? 0.0f : v);
}

}  // namespace wlg
