// Counter-based random streams for the Wang-Landau engine.
//
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel Random Numbers: As Easy
// as 1, 2, 3", SC'11): a 128-bit counter and a 64-bit key give four 32-bit
// outputs.  The reference draws from cuRAND's Philox4_32_10 generator with
// curand_init(seed, subsequence, offset) and curand_uniform (wl.cu:63, :380,
// :448, :505, :796, :875, :1074).  A stream here is the same object: draw t of
// subsequence s under key k is word (t mod 4) of Philox(counter = s*2^64 + t/4,
// key = k), and a uniform is the centre of the draw's 2^-32 cell rounded to
// float, in (0, 1].  The GPU tests pin these draws against cuRAND itself.
//
// A walker keeps only (key, subsequence, position) plus the block of four
// outputs it is consuming, so a stream costs six registers and one Philox
// evaluation per four draws; positions persist across launches exactly like
// the reference's d_offset_iter.
#pragma once

#include <cstdint>

#include "wlg_keys.h"

namespace wlg {

constexpr uint32_t kPhiloxMulA = 0xD2511F53u;
constexpr uint32_t kPhiloxMulB = 0xCD9E8D57u;
constexpr uint32_t kPhiloxWeylA = 0x9E3779B9u;
constexpr uint32_t kPhiloxWeylB = 0xBB67AE85u;

// kRounds Philox4x32 rounds applied to the state c, the first of them under
// the key (k0, k1); the key advances by the Weyl constants every round.
template <int kRounds>
__device__ __forceinline__ uint4 philox_rounds(uint4 c, uint32_t k0, uint32_t k1)
{
#pragma unroll
  for (int r = 0; r < kRounds; ++r) {
    const uint64_t pa = static_cast<uint64_t>(kPhiloxMulA) * c.x;
    const uint64_t pb = static_cast<uint64_t>(kPhiloxMulB) * c.z;
    const uint32_t n0 = static_cast<uint32_t>(pb >> 32) ^ c.y ^ k0;
    const uint32_t n2 = static_cast<uint32_t>(pa >> 32) ^ c.w ^ k1;
    c.y = static_cast<uint32_t>(pb);
    c.w = static_cast<uint32_t>(pa);
    c.x = n0;
    c.z = n2;
    k0 += kPhiloxWeylA;
    k1 += kPhiloxWeylB;
  }
  return c;
}

__device__ __forceinline__ uint4 philox10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0,
                                          uint32_t k1)
{
  return philox_rounds<10>(make_uint4(c0, c1, c2, c3), k0, k1);
}

// (0, 1] float of a 32-bit draw.  The product is exact (power-of-two scale),
// so a fused multiply-add rounds identically to the separate operations.
__device__ __forceinline__ float unit_float(uint32_t x)
{
  return __fmaf_rn(__uint2float_rn(x), 0x1p-32f, 0x1p-33f);
}

struct Stream {
  uint32_t k0, k1;  // key
  uint32_t s0, s1;  // subsequence: upper half of the counter
  uint64_t pos;     // draws consumed
  uint4 blk;        // outputs of counter pos/4

  __device__ __forceinline__ void refill()
  {
    const uint64_t c = pos >> 2;
    blk = philox10(static_cast<uint32_t>(c), static_cast<uint32_t>(c >> 32), s0, s1, k0, k1);
  }

  __device__ __forceinline__ void init(uint64_t key, uint64_t subseq, uint64_t position)
  {
    k0 = static_cast<uint32_t>(key);
    k1 = static_cast<uint32_t>(key >> 32);
    s0 = static_cast<uint32_t>(subseq);
    s1 = static_cast<uint32_t>(subseq >> 32);
    pos = position;
    refill();
  }

  __device__ __forceinline__ uint32_t raw()
  {
    const uint32_t q = static_cast<uint32_t>(pos) & 3u;
    const uint32_t v = (q == 0) ? blk.x : (q == 1) ? blk.y : (q == 2) ? blk.z : blk.w;
    ++pos;
    if (q == 3) refill();
    return v;
  }

  __device__ __forceinline__ float uniform() { return unit_float(raw()); }
};

}  // namespace wlg
