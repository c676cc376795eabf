// Syndromes of bond patterns: the decoding front-end of the serving API.
//
// The reference draws every bond pattern itself (wl.cu:364-386); a decoder
// is given a syndrome instead.  In the random-bond Ising model of the code,
// the syndrome is the set of frustrated plaquettes of the spin lattice, and
// any bond pattern with those plaquettes frustrated serves as the reference
// error: its four error classes (prerun.cu:56-75) then give the probability
// of each logical class relative to it.
//
// Bond layout (wl.cu:77-87): right bond of spin (i, j) at [i*Y + j] joins
// (i, j) and (i, j+1); down bond at [N + i*Y + j] joins (i, j) and (i+1, j)
// (indices mod X, Y; open lattices leave the wrap-around bonds unused).

#include <cstdint>
#include <vector>

#include "../../include/wlg.h"
#include "wlg_internal.h"

namespace {

constexpr int kMaxSpins = 1 << 22;

bool valid_shape(int X, int Y, int boundary)
{
  return X >= 2 && Y >= 2 && (boundary == 0 || boundary == 1) && static_cast<long long>(X) * Y <= kMaxSpins;
}

int right(int X, int Y, int i, int j) { return (i % X) * Y + (j % Y); }
int down(int X, int Y, int i, int j) { return X * Y + (i % X) * Y + (j % Y); }

}  // namespace

extern "C" {

wlg_status wlg_frustration(int X, int Y, int boundary, const signed char* couplings, unsigned char* syndrome)
{
  return wlg::guarded([&]() -> wlg_status {
    if (!valid_shape(X, Y, boundary) || couplings == nullptr || syndrome == nullptr) return WLG_ERR_INVALID;
    const int PX = boundary == 0 ? X : X - 1, PY = boundary == 0 ? Y : Y - 1;
    for (int i = 0; i < PX; ++i)
      for (int j = 0; j < PY; ++j) {
        const int prod = couplings[right(X, Y, i, j)] * couplings[right(X, Y, i + 1, j)] *
                         couplings[down(X, Y, i, j)] * couplings[down(X, Y, i, j + 1)];
        syndrome[i * PY + j] = prod < 0 ? 1 : 0;
      }
    return WLG_OK;
  });
}

wlg_status wlg_couplings_from_syndrome(int X, int Y, int boundary, const unsigned char* syndrome,
                                       signed char* couplings)
{
  return wlg::guarded([&]() -> wlg_status {
    if (!valid_shape(X, Y, boundary) || couplings == nullptr || syndrome == nullptr) return WLG_ERR_INVALID;
    const int N = X * Y;
    const int PX = boundary == 0 ? X : X - 1, PY = boundary == 0 ? Y : Y - 1;
    std::vector<uint8_t> flip(static_cast<size_t>(2 * N), 0);
    int defects = 0;
    for (int i = 0; i < PX; ++i)
      for (int j = 0; j < PY; ++j) {
        if (syndrome[i * PY + j] > 1) return WLG_ERR_INVALID;
        if (syndrome[i * PY + j] == 0) continue;
        ++defects;
        // plaquettes (i, c) and (i, c-1) share the down bond of (i, c); on an
        // open lattice the one of (i, 0) leads out across the left edge
        for (int c = j; c >= (boundary == 0 ? 1 : 0); --c) flip[down(X, Y, i, c)] ^= 1;
        if (boundary == 0)  // plaquettes (r, 0) and (r-1, 0) share the right bond of (r, 0)
          for (int r = i; r >= 1; --r) flip[right(X, Y, r, 0)] ^= 1;
      }
    if (boundary == 0 && defects % 2 != 0) return WLG_ERR_INVALID;
    for (int q = 0; q < 2 * N; ++q) couplings[q] = flip[q] ? -1 : 1;
    return WLG_OK;
  });
}

}  // extern "C"
