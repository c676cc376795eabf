// Philox keys of the reference's streams.  The reference forms the 64-bit
// key from `seed + sample` with three different integer promotions; they
// agree for non-negative seeds that do not overflow.
#pragma once

#include <cstdint>

#if defined(__CUDACC__)
#define WLG_KEYS_HD __host__ __device__ __forceinline__
#else
#define WLG_KEYS_HD inline
#endif

namespace wlg {

WLG_KEYS_HD uint64_t key_u32(int seed, uint64_t k)  // unsigned int arithmetic: wl.cu:448, :505, :1074
{
  return static_cast<uint32_t>(static_cast<uint32_t>(seed) + static_cast<uint32_t>(k));
}

WLG_KEYS_HD uint64_t key_i32(int seed, uint64_t k)  // int arithmetic, sign-extended: wl.cu:796, :875
{
  return static_cast<uint64_t>(
    static_cast<int64_t>(static_cast<int32_t>(static_cast<uint32_t>(seed) + static_cast<uint32_t>(k))));
}

WLG_KEYS_HD uint64_t key_size(int seed, uint64_t k)  // size_t arithmetic: wl.cu:380
{
  return static_cast<uint64_t>(static_cast<int64_t>(seed)) + k;
}

}  // namespace wlg
