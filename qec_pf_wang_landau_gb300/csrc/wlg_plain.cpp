// Plain form of the engine: the reference's own structure (prerun.cu:36-154,
// mainrun.cu:115-421) executed with this library's operator kernels — one
// launch per operation, one thread per walker, state in global memory, the
// outer loop on the host with a device->host check every iteration.  It
// processes problems that share every parameter except the sample index as
// one run of R samples, exactly like one prerun/mainrun invocation.

#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <numbers>
#include <tuple>
#include <vector>

#include "../../include/wlg.h"
#include "wlg_internal.h"

namespace wlg {
wlg_status make_windows(int e_min, int e_max, int n, float overlap, std::vector<int>& start, std::vector<int>& end);
wlg_status stitch_windows(std::vector<std::map<int, double>> windows, int X, int Y,
                          std::vector<std::pair<int, double>>& out, int mode);
}  // namespace wlg

namespace {

struct Dev {
  std::vector<void*> ptrs;
  ~Dev()
  {
    for (void* p : ptrs) cudaFree(p);
  }
  template <typename T>
  T* alloc(size_t n)
  {
    void* p = nullptr;
    if (cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess) return nullptr;
    ptrs.push_back(p);
    return static_cast<T*>(p);
  }
  template <typename T>
  T* put(const std::vector<T>& h, cudaStream_t s)
  {
    T* d = alloc<T>(h.size());
    if (d != nullptr && !h.empty()) cudaMemcpyAsync(d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, s);
    return d;
  }
};

template <typename T>
void get(std::vector<T>& h, const T* d, cudaStream_t s)
{
  if (!h.empty()) cudaMemcpyAsync(h.data(), d, h.size() * sizeof(T), cudaMemcpyDeviceToHost, s);
}

#define WLG_TRY(x)                          \
  do {                                      \
    const wlg_status st_ = (x);             \
    if (st_ != WLG_OK) return st_;          \
  } while (0)

// One run: R samples (0..R-1) of the same parameters.
wlg_status run_plain(const wlg_problem& q, int R, cudaStream_t s, std::vector<wlg_result>& res,
                     std::vector<std::vector<std::pair<int, double>>>& curves, long long& launches)
{
  const int X = q.X, Y = q.Y, N = X * Y;
  const int seed = q.seed;
  Dev dv;
  // ---------------- pre-run (prerun.cu:23-133)
  const int e_min = -2 * N, e_max = 2 * N;
  std::vector<int> ps, pe;
  WLG_TRY(wlg::make_windows(e_min, e_max, q.pre_intervals, 1.0F, ps, pe));
  const int len_int = pe[0] - ps[0] + 1;
  const int pw = q.pre_walkers, pI = q.pre_intervals;
  const size_t T0 = static_cast<size_t>(R) * pw;
  int8_t* J = dv.alloc<int8_t>(static_cast<size_t>(R) * 2 * N);
  int8_t* lat0 = dv.alloc<int8_t>(T0 * N);
  int* E0 = dv.alloc<int>(T0);
  unsigned long long* H0 = dv.alloc<unsigned long long>(static_cast<size_t>(R) * (4 * N + 1));
  uint64_t* so = dv.alloc<uint64_t>(T0);
  int8_t* flat = dv.alloc<int8_t>(static_cast<size_t>(R) * pI * N);
  int* fflag = dv.alloc<int>(static_cast<size_t>(R) * pI);
  int* fen = dv.alloc<int>(static_cast<size_t>(R) * pI);
  if (fen == nullptr) return WLG_ERR_OOM;
  std::vector<int> off0(T0), offf(static_cast<size_t>(R) * pI);
  for (size_t t = 0; t < T0; ++t) off0[t] = static_cast<int>(t * N);
  for (size_t t = 0; t < offf.size(); ++t) offf[t] = static_cast<int>(t * N);
  int* doff0 = dv.put(off0, s);
  int* dofff = dv.put(offf, s);
  cudaMemsetAsync(H0, 0, static_cast<size_t>(R) * (4 * N + 1) * 8, s);
  cudaMemsetAsync(so, 0, T0 * 8, s);
  cudaMemsetAsync(flat, 0, static_cast<size_t>(R) * pI * N, s);
  cudaMemsetAsync(fflag, 0, static_cast<size_t>(R) * pI * 4, s);
  WLG_TRY(wlg_init_interactions(J, static_cast<size_t>(N), R, seed, q.prob, s));
  WLG_TRY(wlg_apply_error_class(J, X, Y, R, q.error_class, s));
  WLG_TRY(wlg_init_lattice(lat0, X, Y, T0, seed, pw, s));
  WLG_TRY(wlg_calc_energy(q.boundary, E0, lat0, J, doff0, X, Y, T0, pw, s));
  WLG_TRY(wlg_wang_landau_pre_run(E0, fflag, lat0, flat, H0, so, J, doff0, e_min, e_max, q.pre_iterations, X, Y, seed,
                                  static_cast<unsigned>(pI), len_int, T0, pw, q.boundary, s));
  WLG_TRY(wlg_calc_energy(q.boundary, fen, flat, J, dofff, X, Y, offf.size(), pI, s));
  launches += 6 + ((q.error_class == 'c') ? 2 : (q.error_class == 'h' || q.error_class == 'v') ? 1 : 0);
  std::vector<unsigned long long> hH(static_cast<size_t>(R) * (4 * N + 1));
  std::vector<int8_t> hJ(static_cast<size_t>(R) * 2 * N), hflat(static_cast<size_t>(R) * pI * N);
  std::vector<int> hflag(static_cast<size_t>(R) * pI), hfen(static_cast<size_t>(R) * pI);
  get(hH, H0, s);
  get(hJ, J, s);
  get(hflat, flat, s);
  get(hflag, fflag, s);
  get(hfen, fen, s);
  if (cudaStreamSynchronize(s) != cudaSuccess) return WLG_ERR_CUDA;

  // ---------------- hand-off (file_io.cpp:558-659, mainrun.cu:79-113)
  const int I = q.intervals, W = q.walkers_per_interval, wpi = I * W;
  std::vector<int8_t> spectrum;
  std::vector<int> off_spec, start, end;
  for (int k = 0; k < R; ++k) {
    const unsigned long long* h = hH.data() + static_cast<size_t>(k) * (4 * N + 1);
    int first = -1, last = -1;
    for (int i = 0; i <= 4 * N; ++i)
      if (h[i] != 0) {
        if (first < 0) first = i;
        last = i;
      }
    if (first < 0) return WLG_ERR_NO_LATTICE;
    off_spec.push_back(static_cast<int>(spectrum.size()));
    for (int i = first; i <= last; ++i) spectrum.push_back(h[i] != 0 ? 1 : 0);
    std::vector<int> ws, we;
    WLG_TRY(wlg::make_windows(e_min + first, e_min + last, I, q.overlap, ws, we));
    start.insert(start.end(), ws.begin(), ws.end());
    end.insert(end.end(), we.begin(), we.end());
  }
  const size_t T = static_cast<size_t>(R) * wpi;
  std::vector<int> off_hist(T), off_lat(T), perm(T);
  long long acc = 0;
  for (size_t t = 0; t < T; ++t) {
    const size_t b = t / W;
    off_hist[t] = static_cast<int>(acc);
    acc += end[b] - start[b] + 1;
    off_lat[t] = static_cast<int>(t * N);
    perm[t] = static_cast<int>(t % W);
  }
  std::vector<int8_t> lat(T * N);
  for (int k = 0; k < R; ++k) {
    std::map<int, int> by_energy;
    for (int b = 0; b < pI; ++b)
      if (hflag[k * pI + b] != 0) by_energy.emplace(hfen[k * pI + b], b);
    for (int b = 0; b < I; ++b) {
      int pick = -1;
      for (const auto& [en, idx] : by_energy)
        if (en >= start[k * I + b] && en <= end[k * I + b]) {
          pick = idx;
          break;
        }
      if (pick < 0) return WLG_ERR_NO_LATTICE;
      for (int w = 0; w < W; ++w)
        std::memcpy(lat.data() + ((static_cast<size_t>(k) * I + b) * W + w) * N,
                    hflat.data() + (static_cast<size_t>(k) * pI + pick) * N, static_cast<size_t>(N));
    }
  }
  int8_t* dlat = dv.put(lat, s);
  int* doff_lat = dv.put(off_lat, s);
  int* doff_hist = dv.put(off_hist, s);
  int* dperm = dv.put(perm, s);
  int* dstart = dv.put(start, s);
  int* dend = dv.put(end, s);
  int8_t* dspec = dv.put(spectrum, s);
  int* doff_spec = dv.put(off_spec, s);
  int* dE = dv.alloc<int>(T);
  int* dnewE = dv.alloc<int>(T);
  int* dfound = dv.alloc<int>(T);
  unsigned long long* dH = dv.alloc<unsigned long long>(static_cast<size_t>(acc));
  double* dG = dv.alloc<double>(static_cast<size_t>(acc));
  std::vector<double> factor(T, std::numbers::e);
  double* dfac = dv.put(factor, s);
  uint64_t* doff_iter = dv.alloc<uint64_t>(T);
  int8_t* dcond = dv.alloc<int8_t>(static_cast<size_t>(R) * I);
  int* dci = dv.alloc<int>(static_cast<size_t>(R));
  int* dmax = dv.alloc<int>(1);
  double* dfmax = dv.alloc<double>(1);
  if (dfmax == nullptr) return WLG_ERR_OOM;
  cudaMemsetAsync(dfound, 0, T * 4, s);
  cudaMemsetAsync(dH, 0, static_cast<size_t>(acc) * 8, s);
  cudaMemsetAsync(dG, 0, static_cast<size_t>(acc) * 8, s);
  cudaMemsetAsync(doff_iter, 0, T * 8, s);
  cudaMemsetAsync(dcond, 0, static_cast<size_t>(R) * I, s);
  cudaMemsetAsync(dci, 0, static_cast<size_t>(R) * 4, s);
  WLG_TRY(wlg_calc_energy(q.boundary, dE, dlat, J, doff_lat, X, Y, T, wpi, s));
  ++launches;

  // ---------------- main loop (mainrun.cu:235-383)
  double max_factor = std::numbers::e;
  long long counter = 1;
  std::vector<long long> outer(static_cast<size_t>(R), 0);
  std::vector<int> ci(static_cast<size_t>(R), 0);
  int status = WLG_OK;
  long long it = 0;
  while (max_factor - std::exp(q.beta) > 1e-10) {
    if (q.max_outer > 0 && it >= q.max_outer) {
      status = WLG_ERR_TIMEOUT;
      break;
    }
    for (int k = 0; k < R; ++k)
      if (ci[k] != -1) ++outer[k];
    ++it;
    WLG_TRY(wlg_wang_landau(dlat, J, dH, dG, dfac, dE, dnewE, doff_iter, dfound, dstart, dend, doff_hist, doff_lat,
                            dcond, dspec, doff_spec, dci, X, Y, q.iterations, static_cast<int>(T), I, wpi, seed,
                            q.boundary, s));
    WLG_TRY(wlg_max_int(dfound, T, dmax, s));
    int hmax = 0;
    cudaMemcpyAsync(&hmax, dmax, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) return WLG_ERR_CUDA;
    launches += 3;
    if (hmax != 0) {
      status = WLG_ERR_NEW_ENERGY;
      break;
    }
    WLG_TRY(wlg_check_histogram(dH, dfac, dcond, doff_hist, dend, dstart, dspec, doff_spec, dci, q.alpha,
                                static_cast<int>(T), wpi, I, s));
    WLG_TRY(wlg_average_log_g(dG, dstart, dend, dspec, doff_spec, dcond, doff_hist, dci, R, W, I, s));
    WLG_TRY(wlg_reset_cond(dcond, dfac, R * I, q.beta, W, s));
    WLG_TRY(wlg_check_finished(dci, dcond, I, R, s));
    WLG_TRY(wlg_max_f64_nonneg(dfac, T, dfmax, s));
    cudaMemcpyAsync(&max_factor, dfmax, sizeof(double), cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(ci.data(), dci, static_cast<size_t>(R) * sizeof(int), cudaMemcpyDeviceToHost, s);
    launches += 5;
    if (counter % q.exchange_every == 0) {
      const int gp = q.global_parity ? 1 : 0;
      WLG_TRY(wlg_replica_exchange(doff_lat, dE, dperm, doff_iter, dstart, dend, doff_hist, dci, dG, 1, seed, I, wpi,
                                   R * I, gp, s));
      WLG_TRY(wlg_replica_exchange(doff_lat, dE, dperm, doff_iter, dstart, dend, doff_hist, dci, dG, 0, seed, I, wpi,
                                   R * I, gp, s));
      launches += 2;
    }
    if (q.exchange_mode == 1) ++counter;
    if (cudaStreamSynchronize(s) != cudaSuccess) return WLG_ERR_CUDA;
  }
  std::vector<double> hG(static_cast<size_t>(acc));
  get(hG, dG, s);
  if (cudaStreamSynchronize(s) != cudaSuccess) return WLG_ERR_CUDA;
  res.assign(static_cast<size_t>(R), wlg_result{});
  curves.assign(static_cast<size_t>(R), {});
  for (int k = 0; k < R; ++k) {
    wlg_result& r = res[k];
    r.outer_iterations = outer[k];
    r.flips = outer[k] * static_cast<long long>(wpi) * q.iterations;
    r.pre_flips = static_cast<long long>(pw) * q.pre_iterations;
    if (status != WLG_OK) {
      r.status = status;
      continue;
    }
    if (ci[k] != -1) {
      r.status = WLG_ERR_TIMEOUT;
      continue;
    }
    std::vector<std::map<int, double>> wins(static_cast<size_t>(I));
    for (int b = 0; b < I; ++b) {
      const int gb = k * I + b;
      const int o = off_hist[static_cast<size_t>(gb) * W];
      for (int e = start[gb]; e <= end[gb]; ++e)
        if (hG[o + e - start[gb]] != 0) wins[b].emplace(e, hG[o + e - start[gb]]);
    }
    r.status = wlg::stitch_windows(std::move(wins), X, Y, curves[k], WLG_STITCH_REFERENCE);
  }
  return WLG_OK;
}

}  // namespace

extern "C" {

/* Declared in wlg.h. */
wlg_status wlg_solve_plain(const wlg_problem* problems, int n, wlg_result* results, int* energies, double* log_g,
                           long long capacity, wlg_stream stream, long long* kernel_launches)
{
  return wlg::guarded([&]() -> wlg_status {
    if (n < 0 || (n > 0 && (problems == nullptr || results == nullptr))) return WLG_ERR_INVALID;
    cudaStream_t s = wlg::as_stream(stream);
    // group problems that differ only in the sample index; each group must hold
    // samples 0..R-1 (one reference run)
    std::map<std::vector<double>, std::vector<int>> groups;
    for (int p = 0; p < n; ++p) {
      const wlg_problem& q = problems[p];
      std::vector<double> key = {static_cast<double>(q.X), static_cast<double>(q.Y), static_cast<double>(q.boundary),
                                 q.prob, static_cast<double>(q.error_class == 'I' ? 'i' : q.error_class),
                                 static_cast<double>(q.seed), static_cast<double>(q.pre_walkers),
                                 static_cast<double>(q.pre_intervals), static_cast<double>(q.pre_iterations),
                                 static_cast<double>(q.intervals), static_cast<double>(q.walkers_per_interval),
                                 q.overlap, q.alpha, q.beta, static_cast<double>(q.iterations),
                                 static_cast<double>(q.exchange_every), static_cast<double>(q.exchange_mode),
                                 static_cast<double>(q.global_parity), static_cast<double>(q.max_outer)};
      groups[key].push_back(p);
    }
    long long pos = 0, launches = 0;
    for (auto& [key, idx] : groups) {
      std::sort(idx.begin(), idx.end(), [&](int a, int b) { return problems[a].sample < problems[b].sample; });
      for (size_t i = 0; i < idx.size(); ++i)
        if (problems[idx[i]].sample != static_cast<int>(i)) return WLG_ERR_INVALID;
      std::vector<wlg_result> res;
      std::vector<std::vector<std::pair<int, double>>> curves;
      WLG_TRY(run_plain(problems[idx[0]], static_cast<int>(idx.size()), s, res, curves, launches));
      for (size_t i = 0; i < idx.size(); ++i) {
        wlg_result r = res[i];
        r.offset = pos;
        r.n_energies = 0;
        if (r.status == WLG_OK) {
          if (pos + static_cast<long long>(curves[i].size()) > capacity) return WLG_ERR_CAPACITY;
          for (size_t k = 0; k < curves[i].size(); ++k) {
            energies[pos + static_cast<long long>(k)] = curves[i][k].first;
            log_g[pos + static_cast<long long>(k)] = curves[i][k].second;
          }
          r.n_energies = static_cast<int>(curves[i].size());
          pos += r.n_energies;
        }
        results[idx[i]] = r;
      }
    }
    if (kernel_launches != nullptr) *kernel_launches = launches;
    return WLG_OK;
  });
}

}  // extern "C"
