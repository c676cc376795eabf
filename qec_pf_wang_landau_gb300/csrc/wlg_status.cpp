// Status strings and version of the C ABI.
#include "../../include/wlg.h"

extern "C" {

const char* wlg_status_string(wlg_status s)
{
  switch (s) {
    case WLG_OK: return "ok";
    case WLG_ERR_INVALID: return "invalid argument";
    case WLG_ERR_CUDA: return "CUDA error";
    case WLG_ERR_NEW_ENERGY: return "found new energy outside the pre-run spectrum";
    case WLG_ERR_ENERGY_RANGE: return "start energy outside its window";
    case WLG_ERR_NO_LATTICE: return "no pre-run lattice inside a window";
    case WLG_ERR_OOM: return "out of device memory or over budget";
    case WLG_ERR_TIMEOUT: return "iteration or time limit reached";
    case WLG_ERR_STITCH: return "windows could not be stitched";
    case WLG_ERR_CAPACITY: return "output buffer too small";
    case WLG_ERR_EMPTY_WINDOW: return "window construction produced an empty window";
    default: return "unknown status";
  }
}

const char* wlg_version(void) { return "wlg-gb300 0.1.0 (sm_103a)"; }

}  // extern "C"
