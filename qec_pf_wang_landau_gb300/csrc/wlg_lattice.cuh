// Spin-flip proposal and lattice energy on the reference's int8 layout,
// shared by the operator kernels and the batched pre-run.
#pragma once

#include <cstdint>

#include "wlg_rng.cuh"

namespace wlg {

struct Move {
  int new_energy;
  int site;
};

// wl.cu:52-208: one uniform picks the site (double arithmetic exactly as the
// reference), dE from the four neighbours; open boundaries drop the bonds
// that would wrap.  Couplings: right bond of (i,j) at i*Y+j, down bond at
// N+i*Y+j.
// Energy after flipping `site` of the int8 lattice s (wl.cu:52-156).
// magic: ceil(2^20 / Y) when site * magic >> 20 == site / Y for every site
// (checked by the caller), 0 to divide.
__device__ __forceinline__ Move move_i8(const int8_t* __restrict__ s, const int8_t* __restrict__ J, int E, int X,
                                        int Y, int site, int boundary, uint32_t magic = 0)
{
  const int N = X * Y;
  const int i = magic != 0 ? static_cast<int>((static_cast<uint32_t>(site) * magic) >> 20) : site / Y;
  const int j = site - i * Y;
  const int ip = (i + 1 < X) ? i + 1 : 0;
  const int im = (i - 1 >= 0) ? i - 1 : X - 1;
  const int jp = (j + 1 < Y) ? j + 1 : 0;
  const int jm = (j - 1 >= 0) ? j - 1 : Y - 1;
  int up = s[im * Y + j] * J[N + im * Y + j];
  int left = s[i * Y + jm] * J[i * Y + jm];
  int down = s[ip * Y + j] * J[N + i * Y + j];
  int right = s[i * Y + jp] * J[i * Y + j];
  if (boundary == 1) {
    up = (i == 0) ? 0 : up;
    down = (i + 1 == X) ? 0 : down;
    right = (j == Y - 1) ? 0 : right;
    left = (j == 0) ? 0 : left;
  }
  const int dE = -2 * s[site] * (up + left + down + right);
  return {E - dE, site};
}

// A uniform site and its flipped energy (wl.cu:60-66 then :52-156).
__device__ __forceinline__ Move propose_i8(Stream& rng, const int8_t* __restrict__ s, const int8_t* __restrict__ J,
                                           int E, int X, int Y, double site_scale, int boundary)
{
  double u = rng.uniform();
  u *= site_scale;
  return move_i8(s, J, E, X, Y, static_cast<int>(trunc(u)), boundary);
}

// wl.cu:261-340.
__device__ __forceinline__ int energy_i8(const int8_t* __restrict__ s, const int8_t* __restrict__ J, int X, int Y,
                                         int boundary)
{
  const int N = X * Y;
  int acc = 0;
  for (int i = 0; i < X; ++i) {
    const int im = (i - 1 >= 0) ? i - 1 : X - 1;
    for (int j = 0; j < Y; ++j) {
      const int jm = (j - 1 >= 0) ? j - 1 : Y - 1;
      int up = s[im * Y + j] * J[N + im * Y + j];
      int left = s[i * Y + jm] * J[i * Y + jm];
      if (boundary == 1) {
        up = (i == 0) ? 0 : up;
        left = (j == 0) ? 0 : left;
      }
      acc += s[i * Y + j] * (up + left);
    }
  }
  return -acc;
}

}  // namespace wlg
