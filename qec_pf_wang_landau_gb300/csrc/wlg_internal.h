// Shared helpers of the engine's translation units (not part of the ABI).
#pragma once

#include <cuda_runtime.h>

#include <new>

#include "../../include/wlg.h"

namespace wlg {

inline cudaStream_t as_stream(wlg_stream s) { return static_cast<cudaStream_t>(s); }

// Status of the launches just issued (configuration errors surface here;
// faults inside a kernel surface at the next synchronising call).
inline wlg_status launch_status()
{
  return cudaGetLastError() == cudaSuccess ? WLG_OK : WLG_ERR_CUDA;
}

inline wlg_status cuda_status(cudaError_t e)
{
  if (e == cudaSuccess) return WLG_OK;
  if (e == cudaErrorMemoryAllocation) return WLG_ERR_OOM;
  return WLG_ERR_CUDA;
}

// Runs an entry point's body so that no C++ exception crosses the C ABI:
// allocation failures become WLG_ERR_OOM, anything else WLG_ERR_INVALID.
template <typename F>
wlg_status guarded(F&& body) noexcept
{
  try {
    return body();
  } catch (const std::bad_alloc&) {
    return WLG_ERR_OOM;
  } catch (...) {
    return WLG_ERR_INVALID;
  }
}

}  // namespace wlg
