// Test infrastructure, not part of the product: the reference's own host
// code for window construction (src/interval.cpp) and result stitching
// (src/result_handling.cpp), compiled from the reference's sources where
// they lie (the build recipe passes -I <reference>/src) and driven through
// plain C entry points, so that the oracle's restatements of both can be
// checked against the reference itself.
//
// The two translation units are included whole (their helpers live in an
// anonymous namespace); the reference's HDF5 writer (src/utils.cpp,
// wl::write_results) is replaced by a capture of exactly the data it would
// write, flattened the way it flattens it (utils.cpp:144-149).
//
// result_handling.cpp:125-126 dereferences std::next(it) at the last key
// two windows share, which is the end of the first window's map.  With
// libstdc++ that reads the map's header as a node: key = the map's element
// count, value = the 8 bytes after the map object, i.e. the start of the next
// map in the std::vector (or the heap beyond it), which the reference never
// initialises.  Its stitch energies therefore depend on what that memory
// held.  This harness makes the memory deterministic: the library replaces
// operator new for its own code (linked with -Bsymbolic-functions, so no
// other library in the process is affected) by a zero-filling allocation,
// so the value read is 0 — the case the engine's reference stitching mode
// reproduces.

#include <cstdlib>
#include <new>

#include "interval.cpp"
#include "result_handling.cpp"

void* operator new(std::size_t n)
{
  void* p = std::calloc(1, n != 0 ? n : 1);
  if (p == nullptr) throw std::bad_alloc();
  return p;
}
void operator delete(void* p) noexcept { std::free(p); }
void operator delete(void* p, std::size_t) noexcept { std::free(p); }

namespace wl::git {
const char* const version = "reference harness";
}

namespace {
std::vector<std::map<int, double>> g_written;
}

void wl::write_results(const std::vector<std::map<int, double>>& result_data, const mainrun_options&, int,
                       const std::string_view, const std::string_view, const std::string_view)
{
  g_written = result_data;
}

extern "C" {

// interval.cpp:5-41.  Returns 0, or 1 when the constructor throws.
int ref_interval(int e_min, int e_max, unsigned int n_int, int walkers, float overlap, int* start, int* end,
                 long long* total, int* len)
{
  try {
    const wl::interval_results r(e_min, e_max, n_int, walkers, overlap);
    for (unsigned int i = 0; i < n_int; ++i) {
      start[i] = r.h_start[i];
      end[i] = r.h_end[i];
    }
    *total = r.len_histogram_over_all_walkers;
    *len = r.len_interval;
    return 0;
  } catch (const std::exception&) {
    return 1;
  }
}

// result_handling.cpp:368-431 on a dense per-window log g layout (walker
// after walker inside each window, mainrun.cu).  Returns 0, 2 when it
// throws, 3 when cap is too small; (E_out, g_out) the pairs it would write.
int ref_stitch(const double* logG, long long n, const int* start, const int* end, int n_int, int W, int X, int Y,
               int* E_out, double* g_out, int cap, int* n_out)
{
  wl::mainrun_options o{};
  o.X = X;
  o.Y = Y;
  o.num_intervals = n_int;
  o.walker_per_interval = W;
  g_written.clear();
  try {
    wl::result_handling_stitched_histogram(o, std::vector<double>(logG, logG + n),
                                           std::vector<int>(start, start + n_int), std::vector<int>(end, end + n_int),
                                           "", "", "", 0);
  } catch (const std::exception&) {
    return 2;
  }
  int k = 0;
  for (const auto& m : g_written)
    for (const auto& [key, value] : m) {
      if (k >= cap) return 3;
      E_out[k] = key;
      g_out[k] = value;
      ++k;
    }
  *n_out = k;
  return 0;
}

}  // extern "C"
