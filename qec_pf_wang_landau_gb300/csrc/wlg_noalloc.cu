// Fixed device scratch for wlg_solve_raw_noalloc().
//
// Some callers cannot allocate device memory: code that runs while a
// framework owns the whole device pool (cudaMalloc would fail or fragment
// it), latency-critical loops where an allocation's implicit
// synchronisation is not acceptable, or hosts whose policy forbids
// allocating after start-up.  For them the engine keeps one file-scope
// arena of kNoAllocBytes (8 MiB) in device memory; every GPU that loads this
// library holds it until the process exits.  The no-allocation entry point
// carves all of its device buffers out of this arena.
//
// The arena is shared by every call on a device and keeps the contents of
// the last call; the entry point clears what must start at zero.  Calls
// that overlap on the GPU (from several host threads or streams) race on
// it; serialise them.

#include <cuda_runtime.h>

#include <cstddef>
#include <mutex>

#include "../../include/wlg.h"

namespace wlg {
constexpr size_t kNoAllocBytes = size_t{8} << 20;
}

static __device__ __align__(256) unsigned char g_noalloc_arena[wlg::kNoAllocBytes];

namespace wlg {

// Device address of the arena on the current device.  Host code may not use
// the symbol itself (on the host it names a stand-in, not device memory), so
// the address is looked up with cudaGetSymbolAddress once per device, with
// that device current, on the first call that needs it.
wlg_status noalloc_arena(void** out, size_t* bytes)
{
  constexpr int kMaxDevices = 64;
  static std::mutex mu;
  static void* addr[kMaxDevices] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return WLG_ERR_CUDA;
  std::lock_guard<std::mutex> lock(mu);
  if (addr[dev] == nullptr) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_arena) != cudaSuccess || p == nullptr) return WLG_ERR_CUDA;
    addr[dev] = p;
  }
  *out = addr[dev];
  *bytes = kNoAllocBytes;
  return WLG_OK;
}

}  // namespace wlg
