// Test infrastructure, not part of the product: the reference's own host
// code for window construction (src/interval.cpp), result stitching
// (src/result_handling.cpp) and the pre-run -> main-run hand-off
// (src/file_io.cpp:558-659), compiled from the reference's sources where
// they lie (the build recipe passes -I <reference>/src) and driven through
// plain C entry points, so that the oracle's restatements of both can be
// checked against the reference itself.
//
// The translation units are included whole (their helpers live in an
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
// file_io.cpp compiles against the test-only HDF5 declarations of
// oracle/h5stub (the recipe puts that directory first on the include path);
// only its in-memory hand-off functions are called
#include "file_io.cpp"
#include "h5stub.inc"

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

// The hand-off of mainrun.cu:60-172: file_io.cpp:558-597 (spectrum from the
// pre-run's binary histograms), interval.cpp per sample, file_io.cpp:618-659
// (the lowest-energy stored lattice inside each window, for every walker),
// on the in-memory pre-run outputs of samples 0..R-1 that its HDF5 readers
// would return (file_io.cpp:218-556): per sample the binary histogram over
// [-2N, 2N], and a map from energy to each stored lattice (found[k*pre_i+q]
// != 0).  Outputs: the trimmed spectrum of every sample, concatenated
// (off_spec/len_spec per sample, at most spec_cap entries), E_min and E_max
// per sample, the window bounds [R*I], and the start lattice of every
// walker [R*I*W][N].  Returns 0, 2 when the reference throws, 3 when
// spec_cap is too small.
int ref_handoff(int X, int Y, int R, int pre_i, int I, int W, float overlap, const unsigned char* seen,
                const int* found, const int* found_energy, const signed char* lattices, signed char* spectrum,
                int* off_spec, int* len_spec, int* e_min, int* e_max, int* start, int* end,
                signed char* start_lattices, long long spec_cap)
{
  const std::size_t N = static_cast<std::size_t>(X) * Y, L = 4 * N + 1;
  std::map<int, std::vector<unsigned char>> hist;
  std::map<int, std::map<int, std::vector<signed char>>> lat;
  for (int k = 0; k < R; ++k) {
    hist[k].assign(seen + k * L, seen + (k + 1) * L);
    for (int q = 0; q < pre_i; ++q)
      if (found[k * pre_i + q] != 0) {
        const signed char* l = lattices + (static_cast<std::size_t>(k) * pre_i + q) * N;
        lat[k][found_energy[k * pre_i + q]] = std::vector<signed char>(l, l + N);
      }
  }
  wl::mainrun_options o{};
  o.X = X;
  o.Y = Y;
  o.num_interactions = R;
  o.num_intervals = I;
  o.walker_per_interval = W;
  o.overlap_decimal = overlap;
  try {
    std::vector<signed char> spec;
    std::vector<int> offs, lens, lo, hi, s_all, e_all;
    wl::get_energy_spectrum_information_from_prerun_results(spec, offs, lens, lo, hi, 0, hist, o);
    for (int k = 0; k < R; ++k) {
      const wl::interval_results r{lo[k], hi[k], static_cast<unsigned int>(I), W, overlap};
      s_all.insert(s_all.end(), r.h_start.begin(), r.h_start.end());
      e_all.insert(e_all.end(), r.h_end.begin(), r.h_end.end());
    }
    std::vector<std::int8_t> starts;
    wl::get_lattice_from_prerun_results(starts, lat, s_all, e_all, o);
    if (static_cast<long long>(spec.size()) > spec_cap) return 3;
    std::copy(spec.begin(), spec.end(), spectrum);
    for (int k = 0; k < R; ++k) {
      off_spec[k] = offs[k];
      len_spec[k] = lens[k];
      e_min[k] = lo[k];
      e_max[k] = hi[k];
    }
    std::copy(s_all.begin(), s_all.end(), start);
    std::copy(e_all.begin(), e_all.end(), end);
    std::copy(starts.begin(), starts.end(), start_lattices);
    return 0;
  } catch (const std::exception&) {
    return 2;
  }
}

}  // extern "C"
