// Reference harness — test/benchmark infrastructure only.
//
// Runs the reference's OWN CUDA kernels (src/wl.cu of
// dfki-ric-quantum/qec_pf_wang_landau, compiled unmodified into a cubin by
// oracle/ref_build.py) on the GPU, in the launch order and geometry of its
// drivers src/prerun.cu:36-154 and src/mainrun.cu:115-383.  The drivers
// themselves need Boost and HDF5, so this harness restates their host logic:
// the HDF5 hand-off becomes an in-memory copy, thrust::max_element and
// cub::DeviceSegmentedReduce become the small kernels below (each followed by
// the same device synchronisation), everything else is the reference's.
// Kernels are found in the cubin by their demangled names.

#include <cuda.h>
#include <cuda_runtime.h>
#include <cxxabi.h>

#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <map>
#include <numbers>
#include <string>
#include <vector>

namespace {

CUmodule g_mod = nullptr;
std::map<std::string, CUfunction> g_fn;

const char* kNames[] = {"wl::init_interactions(",
                        "wl::apply_x_horizontal_error(",
                        "wl::apply_x_vertical_error(",
                        "wl::init_lattice(",
                        "wl::init_offsets_lattice(",
                        "wl::calc_energy_periodic_boundary(",
                        "wl::calc_energy_open_boundary(",
                        "wl::wang_landau_pre_run(",
                        "wl::check_energy_ranges(",
                        "wl::init_indices(",
                        "wl::reset_d_cond(",
                        "wl::init_offsets_histogram(",
                        "wl::calc_average_log_g(",
                        "wl::replica_exchange(",
                        "wl::check_histogram(",
                        "wl::redistribute_g_values(",
                        "wl::wang_landau(",
                        "check_all_intervals_finished("};

int launch(const char* name, unsigned grid, unsigned block, std::vector<void*> args)
{
  auto it = g_fn.find(name);
  if (it == g_fn.end()) return 10;
  if (grid == 0) return 0;
  return cuLaunchKernel(it->second, grid, 1, 1, block, 1, 1, 0, nullptr, args.data(), nullptr) == CUDA_SUCCESS ? 0
                                                                                                                 : 11;
}

// thrust::max_element replacements (mainrun.cu:221-224, :273-276, :342-344)
__global__ void h_max_i32(const int* in, size_t n, int* out)
{
  for (size_t q = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; q < n;
       q += static_cast<size_t>(gridDim.x) * blockDim.x)
    atomicMax(out, in[q]);
}
__global__ void h_max_i8(const int8_t* in, size_t n, int* out)
{
  for (size_t q = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; q < n;
       q += static_cast<size_t>(gridDim.x) * blockDim.x)
    atomicMax(out, static_cast<int>(in[q]));
}
__global__ void h_max_f64(const double* in, size_t n, unsigned long long* out)
{
  for (size_t q = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; q < n;
       q += static_cast<size_t>(gridDim.x) * blockDim.x)
    atomicMax(out, static_cast<unsigned long long>(__double_as_longlong(in[q])));
}
// cub::DeviceSegmentedReduce::Sum of cond per sample (wl.cu:685-703)
__global__ void h_segsum(const int8_t* cond, int n_int, int R, int* out)
{
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= R) return;
  int s = 0;
  for (int b = 0; b < n_int; ++b) s += cond[k * n_int + b];
  out[k] = s;
}

struct Dev {
  std::vector<void*> p;
  ~Dev()
  {
    for (void* x : p) cudaFree(x);
  }
  template <typename T>
  T* zeros(size_t n)
  {
    void* x = nullptr;
    cudaMalloc(&x, std::max<size_t>(n, 1) * sizeof(T));
    cudaMemset(x, 0, std::max<size_t>(n, 1) * sizeof(T));
    p.push_back(x);
    return static_cast<T*>(x);
  }
  template <typename T>
  T* from(const std::vector<T>& h)
  {
    T* d = zeros<T>(h.size());
    cudaMemcpy(d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice);
    return d;
  }
};

// interval.cpp:5-41
bool windows(int e_min, int e_max, unsigned n, int walkers, float o, std::vector<int>& s, std::vector<int>& e,
             long long& total, int& len)
{
  if (o > 1 || o < 0) return false;
  const int range = e_max - e_min + 1;
  len = static_cast<int>(static_cast<float>(range) / (1.0F + o * static_cast<float>(n - 1)));
  const int step = static_cast<int>(o * static_cast<float>(len));
  s.assign(n, 0);
  e.assign(n, 0);
  total = 0;
  int st = e_min;
  for (unsigned b = 0; b < n; ++b) {
    s[b] = st;
    if (b + 1 < n) {
      e[b] = st + len - 1;
      total += static_cast<long long>(walkers) * len;
    } else {
      e[b] = e_max;
      total += static_cast<long long>(walkers) * (e_max - st + 1);
    }
    if (s[b] >= e[b]) return false;
    st += step;
  }
  return true;
}

double ms_since(std::chrono::steady_clock::time_point t0)
{
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

}  // namespace

extern "C" {

// Loads the cubin and resolves every reference kernel; 0 on success.
int refh_open(const char* cubin)
{
  cudaFree(nullptr);  // create the runtime's primary context
  if (g_mod != nullptr) return 0;
  if (cuModuleLoad(&g_mod, cubin) != CUDA_SUCCESS) return 1;
  unsigned count = 0;
  if (cuModuleGetFunctionCount(&count, g_mod) != CUDA_SUCCESS) return 2;
  std::vector<CUfunction> fns(count);
  if (cuModuleEnumerateFunctions(fns.data(), count, g_mod) != CUDA_SUCCESS) return 3;
  for (CUfunction f : fns) {
    const char* mangled = nullptr;
    if (cuFuncGetName(&mangled, f) != CUDA_SUCCESS || mangled == nullptr) continue;
    int st = 0;
    char* dem = abi::__cxa_demangle(mangled, nullptr, nullptr, &st);
    const std::string name = (st == 0 && dem != nullptr) ? dem : mangled;
    std::free(dem);
    for (const char* want : kNames) {
      const std::string w(want);
      if (name.rfind(w, 0) == 0 || name.find("::" + w) != std::string::npos || name.find(" " + w) != std::string::npos)
        g_fn[want] = f;
    }
  }
  for (const char* want : kNames)
    if (g_fn.find(want) == g_fn.end()) return 4;
  return 0;
}

}  // extern "C"

namespace {

// Host copies of what prerun.cu writes to prerun_results.h5 for R samples
// (file_io.cpp:23-192): the binary histogram [R][4N+1], the couplings
// [R][2N], the stored lattices [R][pre_i][N] (all zero where none was
// stored) and their energies.
struct PreOut {
  std::vector<unsigned long long> hist;
  std::vector<int8_t> J, found;
  std::vector<int> energy;
};

// prerun.cu:23-146 on the reference's kernels.
int run_prerun(int X, int Y, int boundary, float prob, char cls, int seed, int R, int pre_w, int pre_i, int pre_n,
               PreOut& po)
{
  const int N = X * Y;
  unsigned int bnd = static_cast<unsigned>(boundary);
  Dev dv;
  const int e_min = -2 * N, e_max = -e_min;
  std::vector<int> ps, pe;
  long long ptot = 0;
  int len_interval = 0;
  if (!windows(e_min, e_max, static_cast<unsigned>(pre_i), 1, 1.0F, ps, pe, ptot, len_interval)) return 2;
  const unsigned total_walker = static_cast<unsigned>(R * pre_w);
  const unsigned total_intervals = static_cast<unsigned>(R) * pre_i;
  const unsigned len_histogram = static_cast<unsigned>(e_max - e_min + 1);
  const unsigned total_histogram = static_cast<unsigned>(R) * len_histogram;
  auto* d_histogram = dv.zeros<unsigned long long>(total_histogram);
  auto* d_seed_offset = dv.zeros<unsigned long>(total_walker);
  auto* d_lattice = dv.zeros<int8_t>(static_cast<size_t>(total_walker) * N);
  auto* d_probs = dv.zeros<float>(total_walker);
  auto* d_J = dv.zeros<int8_t>(static_cast<size_t>(R) * N * 2);
  auto* d_energy = dv.zeros<int>(total_walker);
  auto* d_found = dv.zeros<int8_t>(static_cast<size_t>(total_intervals) * N);
  auto* d_flag = dv.zeros<int>(total_intervals);
  auto* d_ienergy = dv.zeros<int>(total_intervals);
  auto* d_off_w = dv.zeros<int>(total_walker);
  auto* d_off_i = dv.zeros<int>(total_intervals);
  const unsigned T = 128;
  const unsigned B_INIT = (total_walker * N * 2 + T - 1) / T;
  const unsigned B_EN = (total_walker + T - 1) / T;
  const unsigned B_INT = (total_intervals + T - 1) / T;
  size_t lsz = static_cast<size_t>(N), nl = total_walker, ni = total_intervals;
  int rc = 0;
  rc |= launch("wl::init_interactions(", B_INIT, T, {&d_J, &lsz, &R, &seed, &prob});
  if (cls == 'h' || cls == 'c') rc |= launch("wl::apply_x_horizontal_error(", B_INIT, T, {&d_J, &X, &Y, &R});
  if (cls == 'v' || cls == 'c') rc |= launch("wl::apply_x_vertical_error(", B_INIT, T, {&d_J, &X, &Y, &R});
  rc |= launch("wl::init_lattice(", B_INIT, T, {&d_lattice, &d_probs, &X, &Y, &nl, &seed, &pre_w});
  rc |= launch("wl::init_offsets_lattice(", B_EN, T, {&d_off_w, &X, &Y, &nl});
  rc |= launch("wl::init_offsets_lattice(", B_INT, T, {&d_off_i, &X, &Y, &ni});
  const char* energy_fn = boundary == 1 ? "wl::calc_energy_open_boundary(" : "wl::calc_energy_periodic_boundary(";
  rc |= launch(energy_fn, B_EN, T, {&d_energy, &d_lattice, &d_J, &d_off_w, &X, &Y, &nl, &pre_w});
  unsigned pre_iu = static_cast<unsigned>(pre_i);
  rc |= launch("wl::wang_landau_pre_run(", B_EN, T,
               {&d_energy, &d_flag, &d_lattice, &d_found, &d_histogram, &d_seed_offset, &d_J, &d_off_w,
                const_cast<int*>(&e_min), const_cast<int*>(&e_max), &pre_n, &X, &Y, &seed, &pre_iu, &len_interval, &nl,
                &pre_w, &bnd});
  rc |= launch(energy_fn, B_INT, T, {&d_ienergy, &d_found, &d_J, &d_off_i, &X, &Y, &ni, &pre_i});
  if (rc != 0) return 10;
  po.energy.assign(total_intervals, 0);
  po.J.assign(static_cast<size_t>(R) * N * 2, 0);
  po.found.assign(static_cast<size_t>(total_intervals) * N, 0);
  po.hist.assign(total_histogram, 0);
  cudaMemcpy(po.energy.data(), d_ienergy, po.energy.size() * 4, cudaMemcpyDeviceToHost);
  cudaMemcpy(po.J.data(), d_J, po.J.size(), cudaMemcpyDeviceToHost);
  cudaMemcpy(po.found.data(), d_found, po.found.size(), cudaMemcpyDeviceToHost);
  cudaMemcpy(po.hist.data(), d_histogram, po.hist.size() * 8, cudaMemcpyDeviceToHost);
  if (cudaDeviceSynchronize() != cudaSuccess) return 12;
  return 0;
}

// The hand-off (file_io.cpp:558-659) and mainrun.cu:42-383 on the
// reference's kernels, from pre-run outputs.  Outputs as refh_run.
int run_mainrun(int X, int Y, int boundary, int seed, int R, int pre_i, const PreOut& po, int I, int W, float overlap,
                double alpha, double beta, int n_iter, int xc, long long max_outer, double* t_main,
                long long* outer_out, int* starts, int* ends, double* raw, long long raw_cap)
{
  const int N = X * Y;
  unsigned int bnd = static_cast<unsigned>(boundary);
  Dev dv;
  const int e_min = -2 * N;
  const unsigned len_histogram = static_cast<unsigned>(4 * N + 1);
  const char* energy_fn = boundary == 1 ? "wl::calc_energy_open_boundary(" : "wl::calc_energy_periodic_boundary(";
  const std::vector<unsigned long long>& h_hist = po.hist;
  const std::vector<int8_t>& h_J = po.J;
  const std::vector<int8_t>& h_found = po.found;
  const std::vector<int>& h_ienergy = po.energy;
  int rc = 0;
  auto t0 = std::chrono::steady_clock::now();
  // ------------------------------------------------ mainrun.cu:42-228
  const int total_walker_m = R * I * W, total_intervals_m = R * I, wpi = I * W;
  std::vector<int8_t> spectrum;
  std::vector<int> off_spec, h_start, h_end, len_hist_k;
  long long total_len = 0;
  for (int k = 0; k < R; ++k) {  // file_io.cpp:558-597 on the binary histogram
    const unsigned long long* h = h_hist.data() + static_cast<size_t>(k) * len_histogram;
    int first = -1, last = -1;
    for (unsigned i = 0; i < len_histogram; ++i)
      if (h[i] != 0) {
        if (first < 0) first = static_cast<int>(i);
        last = static_cast<int>(i);
      }
    if (first < 0) return 2;
    off_spec.push_back(static_cast<int>(spectrum.size()));
    for (int i = first; i <= last; ++i) spectrum.push_back(h[i] != 0 ? 1 : 0);
    std::vector<int> s, e;
    long long tot = 0;
    int len = 0;
    if (!windows(e_min + first, e_min + last, static_cast<unsigned>(I), W, overlap, s, e, tot, len)) return 2;
    h_start.insert(h_start.end(), s.begin(), s.end());
    h_end.insert(h_end.end(), e.begin(), e.end());
    len_hist_k.push_back(static_cast<int>(tot));
    total_len += tot;
  }
  std::vector<long long> off_shared;
  long long size_shared = 0;
  for (int q = 0; q < total_intervals_m; ++q) {
    off_shared.push_back(size_shared);
    size_shared += h_end[q] - h_start[q] + 1;
  }
  std::vector<int> off_intervals(static_cast<size_t>(R) + 1);
  for (int k = 0; k <= R; ++k) off_intervals[k] = k * I;
  std::vector<int8_t> lattices;  // file_io.cpp:618-659: lowest-energy stored lattice per window
  for (int k = 0; k < R; ++k) {
    std::map<int, const int8_t*> by_e;
    for (int q = 0; q < pre_i; ++q) {
      const int8_t* l = h_found.data() + (static_cast<size_t>(k) * pre_i + q) * N;
      if (l[0] != 0) by_e.emplace(h_ienergy[k * pre_i + q], l);  // file_io.cpp:151
    }
    for (int b = 0; b < I; ++b) {
      const int8_t* pick = nullptr;
      for (const auto& [en, l] : by_e)
        if (en >= h_start[k * I + b] && en <= h_end[k * I + b]) {
          pick = l;
          break;
        }
      if (pick == nullptr) return 2;
      for (int w = 0; w < W; ++w) lattices.insert(lattices.end(), pick, pick + N);
    }
  }
  auto* dm_off_spec = dv.from(off_spec);
  auto* dm_len_hist = dv.from(len_hist_k);
  auto* dm_start = dv.from(h_start);
  auto* dm_end = dv.from(h_end);
  auto* dm_H = dv.zeros<unsigned long long>(static_cast<size_t>(total_len));
  auto* dm_logG = dv.zeros<double>(static_cast<size_t>(total_len));
  auto* dm_shared = dv.zeros<double>(static_cast<size_t>(size_shared));
  auto* dm_off_shared = dv.from(off_shared);
  // one entry more than walkers: calc_average_log_g and redistribute_g_values
  // read d_offset_histogram[R*I*W] while looking up the last sample (wl.cu:737, :1001)
  auto* dm_off_hist = dv.zeros<int>(static_cast<size_t>(total_walker_m) + 1);
  auto* dm_off_lat = dv.zeros<int>(static_cast<size_t>(total_walker_m));
  auto* dm_off_iter = dv.zeros<unsigned long>(static_cast<size_t>(total_walker_m));
  auto* dm_factor = dv.from(std::vector<double>(static_cast<size_t>(total_walker_m), std::numbers::e));
  auto* dm_indices = dv.zeros<int>(static_cast<size_t>(total_walker_m));
  auto* dm_lattice = dv.from(lattices);
  auto* dm_J = dv.from(h_J);
  auto* dm_energy = dv.zeros<int>(static_cast<size_t>(total_walker_m));
  auto* dm_flag_check = dv.zeros<int8_t>(static_cast<size_t>(total_walker_m));
  auto* dm_spectrum = dv.from(spectrum);
  auto* dm_newE = dv.zeros<int>(static_cast<size_t>(total_walker_m));
  auto* dm_found = dv.zeros<int>(static_cast<size_t>(total_walker_m));
  auto* dm_cond = dv.zeros<int8_t>(static_cast<size_t>(total_intervals_m));
  auto* dm_ci = dv.zeros<int>(static_cast<size_t>(R));
  auto* dm_red = dv.zeros<unsigned long long>(1);
  unsigned tim = static_cast<unsigned>(total_intervals_m), wu = static_cast<unsigned>(W);
  size_t twm = static_cast<size_t>(total_walker_m);
  int tw_int = total_walker_m;
  rc |= launch("wl::init_offsets_lattice(", tim, wu, {&dm_off_lat, &X, &Y, &twm});
  rc |= launch("wl::init_offsets_histogram(", tim, wu, {&dm_off_hist, &dm_start, &dm_end, &dm_len_hist, &I, &tw_int});
  rc |= launch("wl::init_indices(", tim, wu, {&dm_indices, &twm});
  rc |= launch(energy_fn, tim, wu, {&dm_energy, &dm_lattice, &dm_J, &dm_off_lat, &X, &Y, &twm, const_cast<int*>(&wpi)});
  rc |= launch("wl::check_energy_ranges(", tim, wu, {&dm_flag_check, &dm_energy, &dm_start, &dm_end, &twm});
  if (rc != 0) return 10;
  int hmax = 0;
  cudaMemset(dm_red, 0, 8);
  h_max_i8<<<64, 256>>>(dm_flag_check, twm, reinterpret_cast<int*>(dm_red));
  cudaMemcpy(&hmax, dm_red, 4, cudaMemcpyDeviceToHost);
  if (hmax == 1) return 2;

  // ------------------------------------------------ mainrun.cu:235-383
  double max_factor = std::numbers::e;
  const long long counter = 1;  // never incremented (mainrun.cu:241, :346)
  const int block_count = static_cast<int>((total_len + 127) / 128);
  int tlh = static_cast<int>(total_len);
  long long outer = 0;
  int status = 0;
  while (max_factor - std::exp(beta) > 1e-10) {
    if (max_outer > 0 && outer >= max_outer) {
      status = 3;
      break;
    }
    ++outer;
    rc |= launch("wl::wang_landau(", tim, wu,
                 {&dm_lattice, &dm_J, &dm_H, &dm_logG, &dm_factor, &dm_energy, &dm_newE, &dm_off_iter, &dm_found,
                  &dm_start, &dm_end, &dm_off_hist, &dm_off_lat, &dm_cond, &dm_spectrum, &dm_off_spec, &dm_ci, &X, &Y,
                  &n_iter, &tw_int, &I, const_cast<int*>(&wpi), &seed, &bnd});
    cudaMemset(dm_red, 0, 8);
    h_max_i32<<<64, 256>>>(dm_found, twm, reinterpret_cast<int*>(dm_red));
    cudaMemcpy(&hmax, dm_red, 4, cudaMemcpyDeviceToHost);
    if (hmax != 0) {
      status = 1;
      break;
    }
    rc |= launch("wl::check_histogram(", tim, wu,
                 {&dm_H, &dm_factor, &dm_cond, &dm_off_hist, &dm_end, &dm_start, &dm_spectrum, &dm_off_spec, &dm_ci,
                  &alpha, &tw_int, const_cast<int*>(&wpi), &I});
    rc |= launch("wl::calc_average_log_g(", static_cast<unsigned>(block_count), 128,
                 {&dm_shared, &dm_len_hist, &dm_logG, &dm_start, &dm_end, &dm_spectrum, &dm_cond, &dm_off_hist,
                  &dm_off_spec, &dm_off_shared, &dm_ci, &R, &W, &I, &tlh});
    rc |= launch("wl::redistribute_g_values(", static_cast<unsigned>(block_count), 128,
                 {&dm_logG, &dm_shared, &dm_len_hist, &dm_start, &dm_end, &dm_ci, &dm_off_hist, &dm_cond,
                  &dm_off_shared, &I, &W, &R, &tlh});
    cudaMemset(dm_shared, 0, static_cast<size_t>(size_shared) * 8);
    int tim_i = total_intervals_m;
    rc |= launch("wl::reset_d_cond(", static_cast<unsigned>(R), static_cast<unsigned>(I),
                 {&dm_cond, &dm_factor, &tim_i, &beta, &W});
    h_segsum<<<(R + 127) / 128, 128>>>(dm_cond, I, R, dm_ci);
    cudaDeviceSynchronize();
    rc |= launch("check_all_intervals_finished(", static_cast<unsigned>(R), 1, {&dm_ci, &I, &R});
    cudaDeviceSynchronize();
    cudaMemset(dm_red, 0, 8);
    h_max_f64<<<64, 256>>>(dm_factor, twm, dm_red);
    unsigned long long bits = 0;
    cudaMemcpy(&bits, dm_red, 8, cudaMemcpyDeviceToHost);
    std::memcpy(&max_factor, &bits, 8);
    if (counter % xc == 0) {
      for (int even = 1; even >= 0; --even) {
        bool ev = even == 1;
        rc |= launch("wl::replica_exchange(", tim, wu,
                     {&dm_off_lat, &dm_energy, &dm_indices, &dm_off_iter, &dm_start, &dm_end, &dm_off_hist, &dm_ci,
                      &dm_logG, &ev, &seed, &I, const_cast<int*>(&wpi)});
      }
    }
    if (rc != 0) return 10;
  }
  if (cudaDeviceSynchronize() != cudaSuccess) return 12;
  *t_main = ms_since(t0);
  *outer_out = outer;
  if (raw != nullptr) {
    std::vector<double> h_logG(static_cast<size_t>(total_len));
    std::vector<int> h_off_hist(static_cast<size_t>(total_walker_m));
    cudaMemcpy(h_logG.data(), dm_logG, h_logG.size() * 8, cudaMemcpyDeviceToHost);
    cudaMemcpy(h_off_hist.data(), dm_off_hist, h_off_hist.size() * 4, cudaMemcpyDeviceToHost);
    long long pos = 0;
    for (int q = 0; q < total_intervals_m; ++q) {
      starts[q] = h_start[q];
      ends[q] = h_end[q];
      const int len = h_end[q] - h_start[q] + 1;
      if (pos + len > raw_cap) return 13;
      std::memcpy(raw + pos, h_logG.data() + h_off_hist[static_cast<size_t>(q) * W], static_cast<size_t>(len) * 8);
      pos += len;
    }
  }
  return status;
}

}  // namespace

extern "C" {

// prerun.cu then mainrun.cu for R samples of one error class, exactly as
// the reference runs them (its exchange counter never advances, so
// replica exchange runs only when xc == 1).  Outputs: pre-run and main-run
// wall time (ms, device-synchronised), outer iterations, a status (0
// converged, 1 new energy, 2 hand-off error, 3 iteration cap, >= 10 launch
// error) and, when raw != nullptr, walker 0's dense log g of every window
// (sample after sample) with the window bounds.
int refh_run(int X, int Y, int boundary, float prob, char cls, int seed, int R, int pre_w, int pre_i, int pre_n, int I,
             int W, float overlap, double alpha, double beta, int n_iter, int xc, long long max_outer, double* t_pre,
             double* t_main, long long* outer_out, int* starts, int* ends, double* raw, long long raw_cap)
{
  if (g_mod == nullptr) return 20;
  PreOut po;
  const auto t0 = std::chrono::steady_clock::now();
  const int rc = run_prerun(X, Y, boundary, prob, cls, seed, R, pre_w, pre_i, pre_n, po);
  if (rc != 0) return rc;
  *t_pre = ms_since(t0);
  return run_mainrun(X, Y, boundary, seed, R, pre_i, po, I, W, overlap, alpha, beta, n_iter, xc, max_outer, t_main,
                     outer_out, starts, ends, raw, raw_cap);
}

// mainrun.cu alone, on the reference's kernels, from given pre-run outputs
// of R samples (samples 0..R-1 of a run seeded `seed`) in the layout the
// reference writes to prerun_results.h5: seen [R][4N+1] (nonzero where the
// pre-run visited energy -2N + i), couplings [R][2N], stored lattices
// [R][pre_i][N] (all zero where none was stored) and their energies
// [R][pre_i].  Outputs as refh_run.
int refh_mainrun(int X, int Y, int boundary, int seed, int R, int pre_i, const unsigned char* seen,
                 const int8_t* couplings, const int8_t* lattices, const int* lattice_energy, int I, int W,
                 float overlap, double alpha, double beta, int n_iter, int xc, long long max_outer, double* t_main,
                 long long* outer_out, int* starts, int* ends, double* raw, long long raw_cap)
{
  if (g_mod == nullptr) return 20;
  const size_t N = static_cast<size_t>(X) * Y;
  PreOut po;
  po.hist.assign(seen, seen + R * (4 * N + 1));
  po.J.assign(couplings, couplings + R * 2 * N);
  po.found.assign(lattices, lattices + static_cast<size_t>(R) * pre_i * N);
  po.energy.assign(lattice_energy, lattice_energy + static_cast<size_t>(R) * pre_i);
  return run_mainrun(X, Y, boundary, seed, R, pre_i, po, I, W, overlap, alpha, beta, n_iter, xc, max_outer, t_main,
                     outer_out, starts, ends, raw, raw_cap);
}

}  // extern "C"

// ---------------------------------------------------------------------------
// One reference kernel at a time on caller-owned device state in the
// reference's layout, launched with the geometry of its drivers.  Every
// pointer is a device address; each call synchronises the device and returns
// 0, 10/11 on a missing kernel or failed launch, 12 on a device error.

namespace {

int finish(int rc)
{
  if (rc != 0) return rc;
  return cudaDeviceSynchronize() == cudaSuccess ? 0 : 12;
}

unsigned blocks128(size_t n) { return static_cast<unsigned>((n + 127) / 128); }

}  // namespace

extern "C" {

// wl::init_interactions then the class's chains, prerun.cu:52-75.
int refh_k_init_interactions(void* J, int X, int Y, int R, int seed, float prob, char cls)
{
  size_t lsz = static_cast<size_t>(X) * Y;
  const unsigned g = blocks128(lsz * 2 * R);
  int rc = launch("wl::init_interactions(", g, 128, {&J, &lsz, &R, &seed, &prob});
  if (cls == 'h' || cls == 'c') rc |= launch("wl::apply_x_horizontal_error(", g, 128, {&J, &X, &Y, &R});
  if (cls == 'v' || cls == 'c') rc |= launch("wl::apply_x_vertical_error(", g, 128, {&J, &X, &Y, &R});
  return finish(rc);
}

// wl::calc_energy_periodic_boundary / wl::calc_energy_open_boundary (wl.cu:261-340).
int refh_k_calc_energy(int boundary, void* energy, void* lattice, void* J, void* off_lat, int X, int Y,
                       size_t num_lattices, int wpi)
{
  const char* fn = boundary == 1 ? "wl::calc_energy_open_boundary(" : "wl::calc_energy_periodic_boundary(";
  return finish(launch(fn, blocks128(num_lattices), 128, {&energy, &lattice, &J, &off_lat, &X, &Y, &num_lattices, &wpi}));
}

// wl::wang_landau_pre_run (wl.cu:473-560), prerun.cu:103 geometry.
int refh_k_pre_run(void* energy, void* flag_found, void* lattice, void* found_lattice, void* histogram,
                   void* seed_offset, void* J, void* off_lat, int e_min, int e_max, int n_iter, int X, int Y, int seed,
                   unsigned num_intervals, int len_interval, size_t num_walkers, int wpi, int boundary)
{
  unsigned bnd = static_cast<unsigned>(boundary);
  return finish(launch("wl::wang_landau_pre_run(", blocks128(num_walkers), 128,
                       {&energy, &flag_found, &lattice, &found_lattice, &histogram, &seed_offset, &J, &off_lat, &e_min,
                        &e_max, &n_iter, &X, &Y, &seed, &num_intervals, &len_interval, &num_walkers, &wpi, &bnd}));
}

// wl::init_offsets_histogram (wl.cu:615-652), mainrun.cu:177 geometry:
// grid = windows, block = walkers per window.
int refh_k_init_offsets_histogram(void* off_hist, void* start, void* end, void* len_hist, int I, int W,
                                  int total_walkers)
{
  return finish(launch("wl::init_offsets_histogram(", static_cast<unsigned>(total_walkers / W),
                       static_cast<unsigned>(W), {&off_hist, &start, &end, &len_hist, &I, &total_walkers}));
}

// wl::wang_landau (wl.cu:1033-1175), mainrun.cu:245 geometry.
int refh_k_wang_landau(void* lattice, void* J, void* H, void* logG, void* factor, void* energy, void* new_energy,
                       void* offset_iter, void* found, void* start, void* end, void* off_hist, void* off_lat, void* cond,
                       void* spectrum, void* off_spec, void* cond_inter, int X, int Y, int n_iter, int num_lattices,
                       int I, int wpi, int seed, int boundary)
{
  unsigned bnd = static_cast<unsigned>(boundary);
  const int W = wpi / I;
  return finish(launch("wl::wang_landau(", static_cast<unsigned>(num_lattices / W), static_cast<unsigned>(W),
                       {&lattice, &J, &H, &logG, &factor, &energy, &new_energy, &offset_iter, &found, &start, &end,
                        &off_hist, &off_lat, &cond, &spectrum, &off_spec, &cond_inter, &X, &Y, &n_iter, &num_lattices,
                        &I, &wpi, &seed, &bnd}));
}

// wl::check_histogram (wl.cu:892-967), mainrun.cu:285 geometry.
int refh_k_check_histogram(void* H, void* factor, void* cond, void* off_hist, void* end, void* start, void* spectrum,
                           void* off_spec, void* cond_inter, double alpha, int num_walkers, int wpi, int I)
{
  const int W = wpi / I;
  return finish(launch("wl::check_histogram(", static_cast<unsigned>(num_walkers / W), static_cast<unsigned>(W),
                       {&H, &factor, &cond, &off_hist, &end, &start, &spectrum, &off_spec, &cond_inter, &alpha,
                        &num_walkers, &wpi, &I}));
}

// wl::calc_average_log_g then wl::redistribute_g_values (wl.cu:710-783,
// :969-1031), mainrun.cu:299-329: the scratch arrays the reference's driver
// keeps (per-sample histogram lengths, per-window offsets into the shared
// log g buffer, the zeroed buffer itself) are built here from start/end.
int refh_k_average_log_g(void* logG, void* start, void* end, void* spectrum, void* cond, void* off_hist,
                         void* off_spec, void* cond_inter, int R, int W, int I)
{
  const int nwin = R * I;
  std::vector<int> h_start(static_cast<size_t>(nwin)), h_end(static_cast<size_t>(nwin));
  cudaMemcpy(h_start.data(), start, h_start.size() * 4, cudaMemcpyDeviceToHost);
  cudaMemcpy(h_end.data(), end, h_end.size() * 4, cudaMemcpyDeviceToHost);
  std::vector<int> len_hist(static_cast<size_t>(R), 0);
  std::vector<long long> off_shared(static_cast<size_t>(nwin));
  long long size_shared = 0, total = 0;
  for (int q = 0; q < nwin; ++q) {
    const int len = h_end[q] - h_start[q] + 1;
    off_shared[q] = size_shared;
    size_shared += len;
    len_hist[q / I] += W * len;
    total += static_cast<long long>(W) * len;
  }
  Dev dv;
  auto* d_len = dv.from(len_hist);
  auto* d_off_shared = dv.from(off_shared);
  auto* d_shared = dv.zeros<double>(static_cast<size_t>(size_shared));
  // the walker offsets plus one entry: both kernels read index R*I*W (wl.cu:737, :1001)
  auto* d_off_hist = dv.zeros<int>(static_cast<size_t>(nwin) * W + 1);
  cudaMemcpy(d_off_hist, off_hist, static_cast<size_t>(nwin) * W * 4, cudaMemcpyDeviceToDevice);
  int tlh = static_cast<int>(total);
  const unsigned g = blocks128(static_cast<size_t>(total));
  int rc = launch("wl::calc_average_log_g(", g, 128,
                  {&d_shared, &d_len, &logG, &start, &end, &spectrum, &cond, &d_off_hist, &off_spec, &d_off_shared,
                   &cond_inter, &R, &W, &I, &tlh});
  rc |= launch("wl::redistribute_g_values(", g, 128,
               {&logG, &d_shared, &d_len, &start, &end, &cond_inter, &d_off_hist, &cond, &d_off_shared, &I, &W, &R,
                &tlh});
  return finish(rc);
}

// wl::reset_d_cond (wl.cu:596-613), mainrun.cu:331 geometry.
int refh_k_reset_cond(void* cond, void* factor, int total_intervals, double beta, int W, int R, int I)
{
  return finish(launch("wl::reset_d_cond(", static_cast<unsigned>(R), static_cast<unsigned>(I),
                       {&cond, &factor, &total_intervals, &beta, &W}));
}

// wl::check_interactions_finished (wl.cu:662-708): the segmented sum of cond
// per sample, then the reference's check_all_intervals_finished kernel.
int refh_k_check_finished(void* cond_inter, void* cond, int I, int R)
{
  h_segsum<<<(R + 127) / 128, 128>>>(static_cast<const int8_t*>(cond), I, R, static_cast<int*>(cond_inter));
  if (cudaDeviceSynchronize() != cudaSuccess) return 12;
  return finish(launch("check_all_intervals_finished(", static_cast<unsigned>(R), 1, {&cond_inter, &I, &R}));
}

// wl::replica_exchange with its Fisher-Yates shuffle (wl.cu:785-890), one
// parity, mainrun.cu:347-371 geometry.
int refh_k_replica_exchange(void* off_lat, void* energy, void* indices, void* offset_iter, void* start, void* end,
                            void* off_hist, void* cond_inter, void* logG, int even, int seed, int I, int wpi,
                            int total_intervals)
{
  bool ev = even != 0;
  const int W = wpi / I;
  return finish(launch("wl::replica_exchange(", static_cast<unsigned>(total_intervals), static_cast<unsigned>(W),
                       {&off_lat, &energy, &indices, &offset_iter, &start, &end, &off_hist, &cond_inter, &logG, &ev,
                        &seed, &I, &wpi}));
}

}  // extern "C"
