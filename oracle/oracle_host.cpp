// ORACLE — test infrastructure only (see oracle.cpp for the contract).
//
// Pipeline-level restatement of the reference: the pre-run driver
// (src/prerun.cu:15-167), the spectrum / start-lattice hand-off
// (src/file_io.cpp:558-659), the main-run outer loop (src/mainrun.cu:235-383),
// result stitching (src/result_handling.cpp:26-431), plus checkers the
// reference does not have: exact density of states by transfer matrix and
// Nishimori-temperature class log-probabilities.  A threaded runner drives
// whole problems for the CPU baseline.

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <map>
#include <numbers>
#include <thread>
#include <tuple>
#include <vector>

#include "oracle_core.h"

extern "C" {
int orc_interval_results(int e_min, int e_max, unsigned n_int, int walkers, float overlap, int* h_start, int* h_end,
                         long long* len_all, int* len_interval);
void orc_init_interactions(int8_t* J, size_t N, int R, int seed, float prob);
void orc_apply_error_class(int8_t* J, int X, int Y, int R, char cls);
void orc_init_lattice(int8_t* lat, int X, int Y, size_t num_lattices, int seed, int wpi);
void orc_calc_energy(int boundary, int* E, const int8_t* lat, const int8_t* J, const int* off_lat, int X, int Y,
                     size_t num_lattices, int wpi);
void orc_wang_landau_pre_run(int* E, int* flag_found, int8_t* lat, int8_t* found_lat, unsigned long long* H,
                             uint64_t* seed_off, const int8_t* J, const int* off_lat, int E_min, int E_max, int n_iter,
                             int X, int Y, int seed, unsigned n_int, int len_int, size_t total_walker, int wpi,
                             int boundary);
int orc_wang_landau(int8_t* lat, const int8_t* J, unsigned long long* H, double* logG, const double* factor, int* E,
                    int* newE, uint64_t* off_iter, int* found, const int* start, const int* end, const int* off_hist,
                    const int* off_lat, const int8_t* cond, const int8_t* spectrum, const int* off_spec,
                    const int* cond_inter, int X, int Y, int n_iter, int num_lattices, int n_int, int wpi, int seed,
                    int boundary);
void orc_check_histogram(unsigned long long* H, double* factor, int8_t* cond, const int* off_hist, const int* end,
                         const int* start, const int8_t* spectrum, const int* off_spec, const int* cond_inter,
                         double alpha, int num_walker_total, int wpi, int n_int);
void orc_average_log_g(double* logG, const int* start, const int* end, const int8_t* spectrum, const int* off_spec,
                       const int8_t* cond, const int* off_hist, const int* cond_inter, int R, int W, int n_int);
void orc_reset_cond(int8_t* cond, const double* factor, int total_intervals, double beta, int W);
void orc_check_finished(int* cond_inter, const int8_t* cond, int n_int, int R);
void orc_replica_exchange(int* off_lat, int* E, int* perm, uint64_t* off_iter, const int* start, const int* end,
                          const int* off_hist, const int* cond_inter, const double* logG, int even, int seed,
                          int n_int, int wpi, int total_intervals, int global_parity);
}

namespace {

// ------------------------------------------------------------- pre-run -----

struct PrerunOut {
  std::vector<uint8_t> seen;       // [R][4N+1] histogram != 0
  std::vector<int8_t> J;           // [R][2N]
  std::vector<int8_t> found_lat;   // [R][I_pre][N]
  std::vector<int> found_flag;     // [R][I_pre]
  std::vector<int> found_energy;   // [R][I_pre]
};

// prerun.cu:23-133 for R samples of one (X, Y, p, class).
PrerunOut run_prerun(int X, int Y, int boundary, float prob, char cls, int seed, int R, int walkers, int n_int,
                     int n_iter)
{
  const int N = X * Y;
  const int e_min = -2 * N, e_max = 2 * N;
  std::vector<int> hs(static_cast<size_t>(n_int)), he(static_cast<size_t>(n_int));
  long long tot = 0;
  int len_int = 0;
  const int irc =
    orc_interval_results(e_min, e_max, static_cast<unsigned>(n_int), 1, 1.0F, hs.data(), he.data(), &tot, &len_int);

  const size_t total_walker = static_cast<size_t>(R) * walkers;
  PrerunOut out;
  if (irc != 0) {  // prerun.cu:23-35: interval_results throws (empty coarse bins); nothing runs
    out.J.assign(static_cast<size_t>(R) * 2 * N, 0);
    out.seen.assign(static_cast<size_t>(R) * (4 * N + 1), 0);
    out.found_flag.assign(static_cast<size_t>(R) * n_int, 0);
    out.found_lat.assign(static_cast<size_t>(R) * n_int * N, 0);
    out.found_energy.assign(static_cast<size_t>(R) * n_int, 0);
    return out;
  }
  out.J.assign(static_cast<size_t>(R) * 2 * N, 0);
  orc_init_interactions(out.J.data(), static_cast<size_t>(N), R, seed, prob);
  orc_apply_error_class(out.J.data(), X, Y, R, cls);

  std::vector<int8_t> lat(total_walker * N);
  orc_init_lattice(lat.data(), X, Y, total_walker, seed, walkers);
  std::vector<int> off_lat(total_walker);
  for (size_t t = 0; t < total_walker; ++t) off_lat[t] = static_cast<int>(t * N);
  std::vector<int> E(total_walker);
  orc_calc_energy(boundary, E.data(), lat.data(), out.J.data(), off_lat.data(), X, Y, total_walker, walkers);

  const int len_hist = e_max - e_min + 1;
  std::vector<unsigned long long> H(static_cast<size_t>(R) * len_hist, 0);
  std::vector<uint64_t> seed_off(total_walker, 0);
  out.found_flag.assign(static_cast<size_t>(R) * n_int, 0);
  out.found_lat.assign(static_cast<size_t>(R) * n_int * N, 0);
  orc_wang_landau_pre_run(E.data(), out.found_flag.data(), lat.data(), out.found_lat.data(), H.data(), seed_off.data(),
                          out.J.data(), off_lat.data(), e_min, e_max, n_iter, X, Y, seed, static_cast<unsigned>(n_int),
                          len_int, total_walker, walkers, boundary);

  std::vector<int> off_found(static_cast<size_t>(R) * n_int);
  for (size_t t = 0; t < off_found.size(); ++t) off_found[t] = static_cast<int>(t * N);
  out.found_energy.assign(off_found.size(), 0);
  orc_calc_energy(boundary, out.found_energy.data(), out.found_lat.data(), out.J.data(), off_found.data(), X, Y,
                  off_found.size(), n_int);
  out.seen.resize(H.size());
  for (size_t t = 0; t < H.size(); ++t) out.seen[t] = H[t] != 0 ? 1 : 0;
  return out;
}

// ------------------------------------------------------------- main run ----

struct MainrunIn {
  int X, Y, boundary;
  int R, n_int, W;
  float overlap;
  double alpha, beta;
  int n_iter, exchange_every, exchange_mode, global_parity, seed;
  long long max_outer;
};

struct MainrunOut {
  int status = 0;  // 0 converged, 1 new energy, 2 bad input, 3 outer-iteration cap
  long long outer = 0;
  long long flips = 0;
  std::vector<int> start, end;
  std::vector<int> off_hist;
  std::vector<double> logG;
  std::vector<int> cond_inter;
};

// file_io.cpp:558-597 + mainrun.cu:79-113 + file_io.cpp:618-659 + the loop
// of mainrun.cu:235-383.
MainrunOut run_mainrun(const MainrunIn& a, const uint8_t* seen, const int8_t* J, const int8_t* found_lat,
                       const int* found_flag, const int* found_energy, int n_int_pre)
{
  MainrunOut o;
  const int N = a.X * a.Y;
  const int len_full = 4 * N + 1;
  const int R = a.R, I = a.n_int, W = a.W;
  const int wpi = I * W;
  const size_t total_walker = static_cast<size_t>(R) * wpi;

  std::vector<int8_t> spectrum;
  std::vector<int> off_spec(static_cast<size_t>(R));
  std::vector<int> e_lo(static_cast<size_t>(R)), e_hi(static_cast<size_t>(R));
  for (int k = 0; k < R; ++k) {
    const uint8_t* h = seen + static_cast<size_t>(k) * len_full;
    int first = -1, last = -1;
    for (int i = 0; i < len_full; ++i)
      if (h[i] == 1) {
        if (first < 0) first = i;
        last = i;
      }
    if (first < 0) {
      o.status = 2;
      return o;
    }
    e_lo[k] = -2 * N + first;
    e_hi[k] = -2 * N + last;
    off_spec[k] = static_cast<int>(spectrum.size());
    spectrum.insert(spectrum.end(), h + first, h + last + 1);
  }

  std::vector<int> len_hist_k(static_cast<size_t>(R));
  long long total_len = 0;
  for (int k = 0; k < R; ++k) {
    std::vector<int> hs(static_cast<size_t>(I)), he(static_cast<size_t>(I));
    long long tot = 0;
    int len_int = 0;
    if (orc_interval_results(e_lo[k], e_hi[k], static_cast<unsigned>(I), W, a.overlap, hs.data(), he.data(), &tot,
                             &len_int) != 0) {
      o.status = 2;
      return o;
    }
    o.start.insert(o.start.end(), hs.begin(), hs.end());
    o.end.insert(o.end.end(), he.begin(), he.end());
    len_hist_k[k] = static_cast<int>(tot);
    total_len += tot;
  }

  // Per-walker slice offsets (wl.cu:615-652): walkers of a sample follow one
  // another window by window.
  o.off_hist.resize(total_walker);
  {
    int acc = 0;
    for (int k = 0; k < R; ++k)
      for (int b = 0; b < I; ++b) {
        const int len = o.end[k * I + b] - o.start[k * I + b] + 1;
        for (int w = 0; w < W; ++w) {
          o.off_hist[(static_cast<size_t>(k) * I + b) * W + w] = acc;
          acc += len;
        }
      }
  }

  // Start lattices: the lowest-energy stored lattice inside each window.
  std::vector<int8_t> lat(total_walker * N);
  for (int k = 0; k < R; ++k) {
    std::map<int, const int8_t*> by_energy;
    for (int q = 0; q < n_int_pre; ++q)
      if (found_flag[k * n_int_pre + q] != 0)
        by_energy.emplace(found_energy[k * n_int_pre + q], found_lat + (static_cast<size_t>(k) * n_int_pre + q) * N);
    for (int b = 0; b < I; ++b) {
      const int s = o.start[k * I + b], e = o.end[k * I + b];
      const int8_t* pick = nullptr;
      for (const auto& [energy, l] : by_energy)
        if (energy >= s && energy <= e) {
          pick = l;
          break;
        }
      if (pick == nullptr) {
        o.status = 2;
        return o;
      }
      for (int w = 0; w < W; ++w)
        std::memcpy(lat.data() + ((static_cast<size_t>(k) * I + b) * W + w) * N, pick, static_cast<size_t>(N));
    }
  }

  std::vector<int> off_lat(total_walker), E(total_walker), perm(total_walker), newE(total_walker, 0),
    found(total_walker, 0);
  for (size_t t = 0; t < total_walker; ++t) {
    off_lat[t] = static_cast<int>(t * N);
    perm[t] = static_cast<int>(t % W);
  }
  orc_calc_energy(a.boundary, E.data(), lat.data(), J, off_lat.data(), a.X, a.Y, total_walker, wpi);
  for (size_t t = 0; t < total_walker; ++t) {
    const size_t b = t / W;
    if (E[t] < o.start[b] || E[t] > o.end[b]) {
      o.status = 2;
      return o;
    }
  }

  std::vector<unsigned long long> H(static_cast<size_t>(total_len), 0);
  o.logG.assign(static_cast<size_t>(total_len), 0.0);
  std::vector<double> factor(total_walker, std::numbers::e);
  std::vector<uint64_t> off_iter(total_walker, 0);
  std::vector<int8_t> cond(static_cast<size_t>(R) * I, 0);
  o.cond_inter.assign(static_cast<size_t>(R), 0);

  double max_factor = std::numbers::e;
  long long counter = 1;
  const double lim = std::exp(a.beta);
  while (max_factor - lim > 1e-10) {
    if (a.max_outer > 0 && o.outer >= a.max_outer) {
      o.status = 3;
      return o;
    }
    for (int k = 0; k < R; ++k)
      if (o.cond_inter[k] != -1) o.flips += static_cast<long long>(wpi) * a.n_iter;
    const int n_new = orc_wang_landau(lat.data(), J, H.data(), o.logG.data(), factor.data(), E.data(), newE.data(),
                                      off_iter.data(), found.data(), o.start.data(), o.end.data(), o.off_hist.data(),
                                      off_lat.data(), cond.data(), spectrum.data(), off_spec.data(),
                                      o.cond_inter.data(), a.X, a.Y, a.n_iter, static_cast<int>(total_walker), I, wpi,
                                      a.seed, a.boundary);
    ++o.outer;
    if (n_new > 0) {
      o.status = 1;
      return o;
    }
    orc_check_histogram(H.data(), factor.data(), cond.data(), o.off_hist.data(), o.end.data(), o.start.data(),
                        spectrum.data(), off_spec.data(), o.cond_inter.data(), a.alpha, static_cast<int>(total_walker),
                        wpi, I);
    orc_average_log_g(o.logG.data(), o.start.data(), o.end.data(), spectrum.data(), off_spec.data(), cond.data(),
                      o.off_hist.data(), o.cond_inter.data(), R, W, I);
    orc_reset_cond(cond.data(), factor.data(), R * I, a.beta, W);
    orc_check_finished(o.cond_inter.data(), cond.data(), I, R);
    max_factor = *std::max_element(factor.begin(), factor.end());
    if (counter % a.exchange_every == 0) {
      orc_replica_exchange(off_lat.data(), E.data(), perm.data(), off_iter.data(), o.start.data(), o.end.data(),
                           o.off_hist.data(), o.cond_inter.data(), o.logG.data(), 1, a.seed, I, wpi, R * I,
                           a.global_parity);
      orc_replica_exchange(off_lat.data(), E.data(), perm.data(), off_iter.data(), o.start.data(), o.end.data(),
                           o.off_hist.data(), o.cond_inter.data(), o.logG.data(), 0, a.seed, I, wpi, R * I,
                           a.global_parity);
    }
    if (a.exchange_mode == 1) ++counter;
  }
  return o;
}

// ------------------------------------------------------------ stitching ----

using Curve = std::map<int, double>;

// Slope towards the successor key (result_handling.cpp:125-126).  The
// reference takes std::next of a map's last node too: with libstdc++ that
// lands on the map header, read as a node whose key is the element count
// and whose value is the following 8 bytes (~0 in practice).  mode 0
// (reference) uses that phantom successor (count, 0.0); mode 1 (defined)
// gives keys without a successor no slope, so they are skipped.
bool slope_to_next(const Curve& c, Curve::const_iterator a, int mode, double& out)
{
  const auto an = std::next(a);
  if (an != c.end()) {
    out = (an->second - a->second) / (an->first - a->first);
    return true;
  }
  if (mode != 0) return false;
  out = (0.0 - a->second) / (static_cast<int>(c.size()) - a->first);
  return true;
}

// result_handling.cpp:115-143.
std::tuple<int, double> stitch_key(const Curve& cur, const Curve& nxt, int mode)
{
  int best_key = std::numeric_limits<int>::max();
  double best = std::numeric_limits<double>::max();
  auto a = cur.begin();
  auto b = nxt.begin();
  while (a != cur.end() && b != nxt.end()) {
    if (a->first == b->first) {
      double da = 0, db = 0;
      if (slope_to_next(cur, a, mode, da) && slope_to_next(nxt, b, mode, db)) {
        const double d = std::abs(da - db);
        if (d < best) {
          best = d;
          best_key = a->first;
        }
      }
      ++a;
      ++b;
    } else if (a->first < b->first) {
      ++a;
    } else {
      ++b;
    }
  }
  return {best_key, best};
}

Curve keep_below(const Curve& c, int t, bool below)
{
  Curve out;
  for (const auto& [k, v] : c)
    if ((below && k < t) || (!below && k >= t)) out[k] = v;
  return out;
}

// result_handling.cpp:368-431 (with helpers :26-366).  Returns 0 or a
// nonzero code when a stitch energy is missing from a window.
int stitch(const double* logG, const int* start, const int* end, int n_int, int W, int X, int Y,
           std::vector<std::pair<int, double>>& result, int mode)
{
  const auto I = static_cast<size_t>(n_int);
  std::vector<Curve> data(I);
  size_t pos = 0;
  for (size_t i = 0; i < I; ++i) {  // walker 0 of each window, nonzero bins only
    const int len = end[i] - start[i] + 1;
    for (int k = 0; k < len; ++k)
      if (logG[pos + k] != 0) data[i][start[i] + k] = logG[pos + k];
    pos += static_cast<size_t>(len) * W;
  }
  for (auto& c : data) {  // shift each window's minimum to 0
    double mn = std::numeric_limits<double>::max();
    for (const auto& kv : c) mn = std::min(mn, kv.second);
    if (mn == std::numeric_limits<double>::max()) mn = 0;
    for (auto& kv : c) kv.second -= mn;
  }
  std::vector<std::tuple<int, int>> keys;  // (window index, energy)
  for (size_t i = 0; i + 1 < I; ++i) {
    int best_key = std::numeric_limits<int>::max();
    double best = std::numeric_limits<double>::max();
    int best_win = std::numeric_limits<int>::max();
    for (size_t j = i + 1; j < I; ++j) {
      const auto [key, d] = stitch_key(data[i], data[j], mode);
      if (key < std::numeric_limits<int>::max()) {
        if (d < best) {
          best_key = key;
          best = d;
          best_win = static_cast<int>(j);
        }
      } else {
        break;
      }
    }
    if (best_win < std::numeric_limits<int>::max()) keys.emplace_back(best_win, best_key);
  }
  std::vector<std::tuple<int, int>> real;
  for (size_t i = 0; i < keys.size(); ++i) {
    bool keep = true;
    for (size_t j = i + 1; j < keys.size(); ++j)
      if (std::get<1>(keys[j]) <= std::get<1>(keys[i])) keep = false;
    if (keep) real.push_back(keys[i]);
  }
  if (real.empty()) {
    // A single window: nothing to stitch.
    if (I != 1) return 1;
    real.clear();
  }
  std::vector<std::tuple<int, int>> smallest;
  if (!real.empty()) {
    int cur_k = std::get<0>(real[0]);
    int cur_v = std::get<1>(real[0]);
    for (const auto& [k, v] : real) {
      if (k != cur_k) {
        smallest.emplace_back(cur_k, cur_v);
        cur_k = k;
        cur_v = v;
      } else if (v < cur_v) {
        cur_v = v;
      }
    }
    smallest.emplace_back(cur_k, cur_v);
  }
  // result_handling.cpp:202-234
  for (size_t i = 0; i < smallest.size(); ++i) {
    const int e = std::get<1>(smallest[i]);
    const auto nxt = static_cast<size_t>(std::get<0>(smallest[i]));
    const size_t prev = (i == 0) ? 0 : static_cast<size_t>(std::get<0>(smallest[i - 1]));
    const auto ip = data[prev].find(e);
    const auto in = data[nxt].find(e);
    if (ip == data[prev].end() || in == data[nxt].end()) return 2;
    const double shift = ip->second - in->second;
    for (auto& kv : data[nxt]) kv.second += shift;
  }
  // result_handling.cpp:270-306
  std::vector<Curve> cut;
  if (smallest.empty()) {
    cut.push_back(data[0]);
  } else {
    auto f = keep_below(data[0], std::get<1>(smallest[0]), true);
    if (!f.empty()) cut.push_back(f);
    for (size_t i = 1; i < smallest.size(); ++i) {
      const int e = std::get<1>(smallest[i]);
      const int ep = std::get<1>(smallest[i - 1]);
      auto m = keep_below(data[static_cast<size_t>(std::get<0>(smallest[i - 1]))], e, true);
      m = keep_below(m, ep, false);
      if (!m.empty()) cut.push_back(m);
    }
    auto l = keep_below(data[static_cast<size_t>(std::get<0>(smallest.back()))], std::get<1>(smallest.back()), false);
    if (!l.empty()) cut.push_back(l);
  }
  // result_handling.cpp:319-365: logsumexp normalised to N ln 2
  double mx = -std::numeric_limits<double>::infinity();
  for (const auto& c : cut)
    for (const auto& kv : c) mx = std::max(mx, kv.second);
  double se = 0.0;
  for (const auto& c : cut)
    for (const auto& kv : c) se += std::exp(kv.second - mx);
  const double off = mx + std::log(se);
  const double l2 = std::log(2) * static_cast<double>(X) * static_cast<double>(Y);
  result.clear();
  for (const auto& c : cut)
    for (const auto& kv : c) result.emplace_back(kv.first, kv.second + l2 - off);
  return 0;
}

}  // namespace

extern "C" {

// Pre-run for R samples (prerun.cu:23-133); outputs in the layout the
// pre-run file stores: seen [R][4N+1], J [R][2N], found lattices
// [R][I_pre][N] with flags and energies [R][I_pre].
void orc_prerun(int X, int Y, int boundary, float prob, char cls, int seed, int R, int walkers, int n_int, int n_iter,
                uint8_t* seen, int8_t* J, int8_t* found_lat, int* found_flag, int* found_energy)
{
  PrerunOut p = run_prerun(X, Y, boundary, prob, cls, seed, R, walkers, n_int, n_iter);
  std::memcpy(seen, p.seen.data(), p.seen.size());
  std::memcpy(J, p.J.data(), p.J.size());
  std::memcpy(found_lat, p.found_lat.data(), p.found_lat.size());
  std::memcpy(found_flag, p.found_flag.data(), p.found_flag.size() * sizeof(int));
  std::memcpy(found_energy, p.found_energy.data(), p.found_energy.size() * sizeof(int));
}

// Main run for R samples of one lattice shape from pre-run outputs.
// Writes the per-window start/end energies [R*I], the per-walker slice
// offsets [R*I*W] and the dense log g of all walkers (length returned in
// *len_logG; pass logG = nullptr to query).  Returns the status of
// MainrunOut.
int orc_mainrun(int X, int Y, int boundary, int R, int n_int, int W, float overlap, double alpha, double beta,
                int n_iter, int exchange_every, int exchange_mode, int global_parity, int seed, long long max_outer,
                const uint8_t* seen, const int8_t* J, const int8_t* found_lat, const int* found_flag,
                const int* found_energy, int n_int_pre, int* start, int* end, int* off_hist, double* logG,
                long long* len_logG, int* cond_inter, long long* outer, long long* flips)
{
  MainrunIn a{X, Y, boundary, R, n_int, W, overlap, alpha, beta, n_iter, exchange_every, exchange_mode,
              global_parity, seed, max_outer};
  MainrunOut o = run_mainrun(a, seen, J, found_lat, found_flag, found_energy, n_int_pre);
  *outer = o.outer;
  *flips = o.flips;
  if (!o.start.empty()) {
    std::memcpy(start, o.start.data(), o.start.size() * sizeof(int));
    std::memcpy(end, o.end.data(), o.end.size() * sizeof(int));
  }
  if (!o.off_hist.empty()) std::memcpy(off_hist, o.off_hist.data(), o.off_hist.size() * sizeof(int));
  *len_logG = static_cast<long long>(o.logG.size());
  if (logG != nullptr && !o.logG.empty()) std::memcpy(logG, o.logG.data(), o.logG.size() * sizeof(double));
  if (!o.cond_inter.empty()) std::memcpy(cond_inter, o.cond_inter.data(), o.cond_inter.size() * sizeof(int));
  return o.status;
}

// Stitch one sample's windows into a normalised log g (result_handling.cpp).
// `logG` is the sample's dense slice (walkers of window 0, then window 1...).
// Returns 0 and the number of (E, log g) pairs in *n_out, or a nonzero code.
int orc_stitch(const double* logG, const int* start, const int* end, int n_int, int W, int X, int Y, int* E_out,
               double* g_out, int cap, int* n_out, int mode)
{
  std::vector<std::pair<int, double>> r;
  const int rc = stitch(logG, start, end, n_int, W, X, Y, r, mode);
  if (rc != 0) return rc;
  *n_out = static_cast<int>(r.size());
  if (static_cast<int>(r.size()) > cap) return 3;
  for (size_t i = 0; i < r.size(); ++i) {
    E_out[i] = r[i].first;
    g_out[i] = r[i].second;
  }
  return 0;
}

// Exact number of states per energy, E in [-2N, 2N], of one coupling set
// (reference layout), by a site-by-site transfer matrix over a front of Y
// spins: adding spin (i, j) replaces spin (i-1, j) in the front.  counts[]
// has 4N+1 entries; values are exact up to 2^53 and within rounding of the
// count beyond.
//
// A partial energy made of b bond terms (each +-1) lies in [-b, b] with the
// parity of b, so each front configuration holds b+1 bins, bin t standing
// for energy -b + 2t, and adding a spin that brings nb - b more terms moves
// bin t to bin t + (de + nb - b) / 2.  Each new front configuration g is
// gathered from its two predecessors (g with spin j up, then down) in one
// contiguous pass that vectorises: bins are stored with kPad zero slots on
// either side, so the shifted reads never leave a front's slice.
//
// Periodic lattices: the down wrap of the last row needs row 0, so the first
// row is fixed and walked over; flipping every spin maps the states with
// first row r0 onto those with first row ~r0 at the same energy, so only
// first rows with spin Y-1 up are walked and the total is doubled.  First
// rows are split into fixed blocks of kRowsPerBlock, walked by all host
// threads, each block summed in row order and the blocks summed in block
// order, so the result does not depend on the number of threads.
// Open lattices: no bond reaches back to row 0, so one pass starts from all
// first rows at once.
namespace {

constexpr size_t kRowsPerBlock = 8;
constexpr int kPad = 4;  // a spin adds at most 4 terms, so a bin moves by at most 4

struct ExactLattice {
  const int8_t* J;
  int X, Y, N, boundary;
  size_t S;      // front configurations, 2^Y
  size_t Lc;     // slots per front configuration: kPad, 2N + 1 bins, kPad
  static int spin(size_t cfg, int j) { return ((cfg >> j) & 1) ? -1 : 1; }
  int Jr(int i, int j) const { return static_cast<int>(J[i * Y + j]); }
  int Jd(int i, int j) const { return static_cast<int>(J[N + i * Y + j]); }

  // bond terms and energy of a first row; a periodic lattice of one row
  // also holds each spin's down bond to itself (a constant -J)
  int row0_terms() const { return (boundary == 0 ? Y : Y - 1) + (boundary == 0 && X == 1 ? Y : 0); }
  int row0_energy(size_t r0) const
  {
    int e = 0;
    for (int j = 0; j + 1 < Y; ++j) e -= Jr(0, j) * spin(r0, j) * spin(r0, j + 1);
    if (boundary == 0) e -= Jr(0, Y - 1) * spin(r0, Y - 1) * spin(r0, 0);
    if (boundary == 0 && X == 1)
      for (int j = 0; j < Y; ++j) e -= Jd(0, j);
    return e;
  }

  // Rows 1..X-1 added to the fronts in cur (b terms so far); r0 is the first
  // row for the periodic down wrap.  Returns the final number of terms.
  int add_rows(size_t r0, int b, std::vector<double>& cur, std::vector<double>& nxt) const
  {
    for (int i = 1; i < X; ++i) {
      for (int j = 0; j < Y; ++j) {
        // terms added with spin (i, j): up, left, right wrap, down wrap
        const bool rwrap = j == Y - 1 && boundary == 0, dwrap = i == X - 1 && boundary == 0;
        const int nb = b + 1 + (j > 0) + rwrap + dwrap;
        const size_t bit = static_cast<size_t>(1) << j;
        for (size_t g = 0; g < S; ++g) {
          const int s = spin(g, j);
          const double* src[2];
          for (int u = 0; u < 2; ++u) {
            const size_t f = u ? (g | bit) : (g & ~bit);
            int de = -Jd(i - 1, j) * s * spin(f, j);                        // up bond
            if (j > 0) de -= Jr(i, j - 1) * s * spin(f, j - 1);              // left bond
            if (rwrap) de -= Jr(i, j) * s * ((j == 0) ? s : spin(f, 0));     // right wrap
            if (dwrap) de -= Jd(i, j) * s * spin(r0, j);                     // down wrap to row 0
            // de has the parity of nb - b and |de| <= nb - b <= kPad: new bin t
            // reads old bin t - (de + nb - b) / 2, in [-kPad, b + kPad]
            src[u] = &cur[f * Lc + kPad] - (de + nb - b) / 2;
          }
          const double* __restrict s0 = src[0];
          const double* __restrict s1 = src[1];
          double* __restrict d = &nxt[g * Lc + kPad];
          for (int t = 0; t <= nb; ++t) d[t] = s0[t] + s1[t];
          std::fill(d + nb + 1, d + nb + 1 + kPad, 0.0);  // upper pad for the next step
        }
        std::swap(cur, nxt);
        b = nb;
      }
    }
    return b;
  }

  void accumulate(int b, const std::vector<double>& cur, double* out) const
  {
    for (size_t f = 0; f < S; ++f)
      for (int t = 0; t <= b; ++t) out[2 * N - b + 2 * t] += cur[f * Lc + kPad + t];
  }
};

void exact_counts_rows(const ExactLattice& lat, size_t r_begin, size_t r_end, std::vector<double>& cur,
                       std::vector<double>& nxt, double* out)
{
  const int b0 = lat.row0_terms();
  for (size_t r0 = r_begin; r0 < r_end; ++r0) {
    for (size_t f = 0; f < lat.S; ++f) std::fill(&cur[f * lat.Lc], &cur[f * lat.Lc] + b0 + 1 + 2 * kPad, 0.0);
    cur[r0 * lat.Lc + kPad + (lat.row0_energy(r0) + b0) / 2] = 1.0;
    lat.accumulate(lat.add_rows(r0, b0, cur, nxt), cur, out);
  }
}

}  // namespace

void orc_exact_counts(const int8_t* J, int X, int Y, int boundary, double* counts)
{
  const int N = X * Y;
  const size_t L = static_cast<size_t>(4 * N + 1);
  const size_t S = static_cast<size_t>(1) << Y;
  const ExactLattice lat{J, X, Y, N, boundary, S, static_cast<size_t>(2 * N + 1 + 2 * kPad)};
  std::fill(counts, counts + L, 0.0);
  if (boundary != 0) {
    std::vector<double> cur(S * lat.Lc, 0.0), nxt(S * lat.Lc, 0.0);
    const int b0 = lat.row0_terms();
    for (size_t r0 = 0; r0 < S; ++r0) cur[r0 * lat.Lc + kPad + (lat.row0_energy(r0) + b0) / 2] = 1.0;
    lat.accumulate(lat.add_rows(0, b0, cur, nxt), cur, counts);
    return;
  }
  const size_t rows = S / 2;  // first rows with spin Y-1 up
  const size_t blocks = (rows + kRowsPerBlock - 1) / kRowsPerBlock;
  std::vector<double> part(blocks * L, 0.0);
  std::atomic<size_t> next{0};
  auto work = [&] {
    std::vector<double> cur(S * lat.Lc, 0.0), nxt(S * lat.Lc, 0.0);
    for (size_t k; (k = next.fetch_add(1)) < blocks;)
      exact_counts_rows(lat, k * kRowsPerBlock, std::min(rows, (k + 1) * kRowsPerBlock), cur, nxt, &part[k * L]);
  };
  const size_t threads = std::min<size_t>(blocks, std::max(1u, std::thread::hardware_concurrency()));
  std::vector<std::thread> pool;
  for (size_t t = 1; t < threads; ++t) pool.emplace_back(work);
  work();
  for (std::thread& t : pool) t.join();
  for (size_t k = 0; k < blocks; ++k)
    for (size_t e = 0; e < L; ++e) counts[e] += part[k * L + e];
  for (size_t e = 0; e < L; ++e) counts[e] *= 2.0;
}

// Brute-force enumeration of the same counts (small N), a check on the
// transfer matrix.
void orc_enumerate_counts(const int8_t* J, int X, int Y, int boundary, double* counts)
{
  const int N = X * Y;
  const int L = 4 * N + 1;
  std::fill(counts, counts + L, 0.0);
  std::vector<int8_t> s(static_cast<size_t>(N));
  for (uint64_t c = 0; c < (1ull << N); ++c) {
    for (int q = 0; q < N; ++q) s[q] = ((c >> q) & 1) ? -1 : 1;
    counts[orc::energy_of(s.data(), J, X, Y, boundary) + 2 * N] += 1.0;
  }
}

// log Z(beta) = logsumexp_E(log g(E) - beta E) over entries with finite g.
double orc_log_partition(const int* E, const double* logg, int n, double beta)
{
  double mx = -std::numeric_limits<double>::infinity();
  for (int i = 0; i < n; ++i) mx = std::max(mx, logg[i] - beta * E[i]);
  double s = 0;
  for (int i = 0; i < n; ++i) s += std::exp(logg[i] - beta * E[i] - mx);
  return mx + std::log(s);
}

// Whole problems for the CPU baseline: each problem is one (disorder sample,
// error class) pre-run + main run with R = 1 and seed' = seed + sample, which
// reproduces the reference's per-sample Philox keys.  Problems are spread
// over `threads` host threads.  Per problem: status, outer iterations,
// main-run flips; returns the total main-run flips.
struct OrcProblem {
  int X, Y, boundary;
  float prob;
  int error_class;
  int seed, sample;
  int pre_walkers, pre_intervals, pre_iterations;
  int n_int, W;
  float overlap;
  double alpha, beta;
  int n_iter, exchange_every, exchange_mode;
  long long max_outer;
};

long long orc_run_problems(const OrcProblem* probs, int n, int threads, int* status, long long* outer,
                           long long* flips)
{
  std::atomic<int> next{0};
  auto worker = [&]() {
    for (;;) {
      const int p = next.fetch_add(1);
      if (p >= n) return;
      const OrcProblem& q = probs[p];
      const int s = q.seed + q.sample;
      PrerunOut pr = run_prerun(q.X, q.Y, q.boundary, q.prob, static_cast<char>(q.error_class), s, 1, q.pre_walkers,
                                q.pre_intervals, q.pre_iterations);
      MainrunIn a{q.X, q.Y, q.boundary, 1, q.n_int, q.W, q.overlap, q.alpha, q.beta, q.n_iter, q.exchange_every,
                  q.exchange_mode, 0, s, q.max_outer};
      MainrunOut o = run_mainrun(a, pr.seen.data(), pr.J.data(), pr.found_lat.data(), pr.found_flag.data(),
                                 pr.found_energy.data(), q.pre_intervals);
      status[p] = o.status;
      outer[p] = o.outer;
      flips[p] = o.flips;
    }
  };
  std::vector<std::thread> pool;
  for (int t = 0; t < std::max(1, threads); ++t) pool.emplace_back(worker);
  for (auto& th : pool) th.join();
  long long tot = 0;
  for (int p = 0; p < n; ++p) tot += flips[p];
  return tot;
}

}  // extern "C"
