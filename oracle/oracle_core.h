// ORACLE internals — test infrastructure only (see oracle.cpp).
// Philox4x32-10 stream, spin-flip proposal and lattice energy shared by the
// oracle's translation units.
#pragma once

#include <cmath>
#include <cstdint>

namespace orc {

// ---------------------------------------------------------------- Philox ---

constexpr uint32_t kMulA = 0xD2511F53u;
constexpr uint32_t kMulB = 0xCD9E8D57u;
constexpr uint32_t kWeylA = 0x9E3779B9u;
constexpr uint32_t kWeylB = 0xBB67AE85u;

struct Quad {
  uint32_t w[4];
};

// Philox4x32 with 10 rounds (Salmon et al. 2011, section 4.2).
inline Quad philox10(uint64_t ctr_lo, uint64_t ctr_hi, uint64_t key)
{
  uint32_t c0 = static_cast<uint32_t>(ctr_lo), c1 = static_cast<uint32_t>(ctr_lo >> 32);
  uint32_t c2 = static_cast<uint32_t>(ctr_hi), c3 = static_cast<uint32_t>(ctr_hi >> 32);
  uint32_t k0 = static_cast<uint32_t>(key), k1 = static_cast<uint32_t>(key >> 32);
  for (int r = 0; r < 10; ++r) {
    const uint64_t pa = static_cast<uint64_t>(kMulA) * c0;
    const uint64_t pb = static_cast<uint64_t>(kMulB) * c2;
    const uint32_t n0 = static_cast<uint32_t>(pb >> 32) ^ c1 ^ k0;
    const uint32_t n2 = static_cast<uint32_t>(pa >> 32) ^ c3 ^ k1;
    c1 = static_cast<uint32_t>(pb);
    c3 = static_cast<uint32_t>(pa);
    c0 = n0;
    c2 = n2;
    k0 += kWeylA;
    k1 += kWeylB;
  }
  return {{c0, c1, c2, c3}};
}

// (0, 1] float from one 32-bit output: the centre of the 2^-32 cell,
// rounded to float (x = 2^32 - 1 rounds to exactly 1.0f).
inline float to_unit(uint32_t x)
{
  const float fx = static_cast<float>(x);
  return fx * 0x1p-32f + 0x1p-33f;
}

// One counter-based stream: draw t of subsequence s is word (t mod 4) of
// Philox(counter = s * 2^64 + t / 4, key).
struct Stream {
  uint64_t key;
  uint64_t subseq;
  uint64_t pos;  // number of 32-bit outputs consumed so far
  uint64_t cached = ~0ull;
  Quad blk{};

  Stream(uint64_t k, uint64_t s, uint64_t off) : key(k), subseq(s), pos(off) {}

  uint32_t raw()
  {
    const uint64_t b = pos >> 2;
    if (b != cached) {
      blk = philox10(b, subseq, key);
      cached = b;
    }
    return blk.w[pos++ & 3];
  }
  float uniform() { return to_unit(raw()); }
};

// The reference forms the 64-bit Philox seed from `seed + sample` with three
// different integer promotions (see the cited lines); they differ only for
// negative seeds.
inline uint64_t key_u32(int seed, uint64_t k)  // unsigned int arithmetic
{
  return static_cast<uint32_t>(static_cast<uint32_t>(seed) + static_cast<uint32_t>(k));
}
inline uint64_t key_i32(int seed, uint64_t k)  // int arithmetic, sign-extended
{
  return static_cast<uint64_t>(static_cast<int64_t>(
    static_cast<int32_t>(static_cast<uint32_t>(seed) + static_cast<uint32_t>(k))));
}
inline uint64_t key_size(int seed, uint64_t k)  // size_t arithmetic
{
  return static_cast<uint64_t>(static_cast<int64_t>(seed)) + k;
}

// ------------------------------------------------------ spin-flip proposal ---

struct Proposal {
  int new_energy;
  int site;
};

// wl.cu:52-156: random site from one uniform, dE from the four neighbours.
// Couplings: right bond of (i,j) at i*Y+j, down bond of (i,j) at N+i*Y+j.
inline Proposal propose(Stream& rng, const int8_t* s, const int8_t* J, int E, int X, int Y, int boundary)
{
  const int N = X * Y;
  double u = rng.uniform();
  u *= (N - 1 + 0.999999);
  const int site = static_cast<int>(std::trunc(u));
  const int i = site / Y;
  const int j = site % Y;
  const int ip = (i + 1 < X) ? i + 1 : 0;
  const int im = (i - 1 >= 0) ? i - 1 : X - 1;
  const int jp = (j + 1 < Y) ? j + 1 : 0;
  const int jm = (j - 1 >= 0) ? j - 1 : Y - 1;
  int up = s[im * Y + j] * J[N + im * Y + j];
  int left = s[i * Y + jm] * J[i * Y + jm];
  int down = s[ip * Y + j] * J[N + i * Y + j];
  int right = s[i * Y + jp] * J[i * Y + j];
  if (boundary == 1) {  // wl.cu:137-149
    if (i == 0) up = 0;
    if (i + 1 == X) down = 0;
    if (j == Y - 1) right = 0;
    if (j == 0) left = 0;
  }
  const int dE = -2 * s[site] * (up + left + down + right);
  return {E - dE, site};
}

inline int energy_of(const int8_t* s, const int8_t* J, int X, int Y, int boundary)
{
  const int N = X * Y;
  int acc = 0;
  for (int i = 0; i < X; ++i) {
    for (int j = 0; j < Y; ++j) {
      const int im = (i - 1 >= 0) ? i - 1 : X - 1;
      const int jm = (j - 1 >= 0) ? j - 1 : Y - 1;
      int up = s[im * Y + j] * J[N + im * Y + j];
      int left = s[i * Y + jm] * J[i * Y + jm];
      if (boundary == 1) {  // wl.cu:324-335: no wrap terms
        if (i == 0) up = 0;
        if (j == 0) left = 0;
      }
      acc += s[i * Y + j] * (up + left);
    }
  }
  return -acc;
}


}  // namespace orc
