// ORACLE — test infrastructure only.
//
// A plain C++ restatement of the reference's replica-exchange Wang-Landau path
// (dfki-ric-quantum/qec_pf_wang_landau, src/wl.cu, src/interval.cpp,
// src/file_io.cpp, src/result_handling.cpp), used by tests/, by
// __graft_entry__.smoke() and by bench.py's CPU-baseline leg, to compare the
// engine's results with.
// It is never linked into, loaded by or called from the product library.
//
// Every function works on the reference's own data layout (int8 spins and
// couplings, per-walker offsets into dense u64 histograms and f64 log g
// slices) and cites the reference line it restates.
//
// Parity anchors:
//   * RNG: Philox4x32-10 is restated from Salmon, Moraes, Dror, Shaw,
//     "Parallel Random Numbers: As Easy as 1, 2, 3" (SC'11).  The mapping of
//     the reference's (seed, subsequence, offset) triples onto the Philox
//     counter is the documented counter-based one: the subsequence is the
//     upper 64 bits of the 128-bit counter, the offset counts 32-bit outputs
//     (four per counter value).  The tests pin this against the device
//     cuRAND draws.
//   * Known-answer tests of the reference's test/ directory are re-expressed
//     in tests/test_oracle_golden.py.
//
// Where the reference is nondeterministic (lattice init CAS, shared pre-run
// histogram, first-come lattice store, FP64 atomic averaging) this file
// fixes one deterministic order and the CUDA engine implements the same one.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <map>
#include <thread>
#include <vector>

#include "oracle_core.h"

using namespace orc;


extern "C" {

// ------------------------------------------------------------------- RNG ----

void orc_philox_raw(uint64_t key, uint64_t subseq, uint64_t offset, int n, uint32_t* out)
{
  Stream st(key, subseq, offset);
  for (int t = 0; t < n; ++t) out[t] = st.raw();
}

void orc_uniform(uint64_t key, uint64_t subseq, uint64_t offset, int n, float* out)
{
  Stream st(key, subseq, offset);
  for (int t = 0; t < n; ++t) out[t] = st.uniform();
}

float orc_raw_to_uniform(uint32_t x) { return to_unit(x); }

// ------------------------------------------------------ energy windows -----
// interval.cpp:5-41.  Returns 0, or 1 for an overlap outside [0,1], or 2 for
// an empty window.
int orc_interval_results(int e_min, int e_max, unsigned n_int, int walkers, float overlap, int* h_start, int* h_end,
                         long long* len_all, int* len_interval)
{
  if (overlap > 1 || overlap < 0) return 1;
  const int range = e_max - e_min + 1;
  const int len = static_cast<int>(static_cast<float>(range) / (1.0F + overlap * static_cast<float>(n_int - 1)));
  const int step = static_cast<int>(overlap * static_cast<float>(len));
  long long total = 0;
  int s = e_min;
  for (unsigned b = 0; b < n_int; ++b) {
    h_start[b] = s;
    if (b + 1 < n_int) {
      h_end[b] = s + len - 1;
      total += static_cast<long long>(walkers) * len;
    } else {
      h_end[b] = e_max;
      total += static_cast<long long>(walkers) * (e_max - s + 1);
    }
    if (h_start[b] >= h_end[b]) return 2;
    s += step;
  }
  *len_all = total;
  *len_interval = len;
  return 0;
}

// ------------------------------------------------------------ disorder -----
// wl.cu:364-386: bond b of sample k is -1 iff the first draw of stream
// (seed+k, 0, b) is below p.
void orc_init_interactions(int8_t* J, size_t N, int R, int seed, float prob)
{
  for (int k = 0; k < R; ++k) {
    for (size_t b = 0; b < 2 * N; ++b) {
      Stream st(key_size(seed, static_cast<uint64_t>(k)), 0, b);
      const double u = st.uniform();
      J[static_cast<size_t>(k) * 2 * N + b] = (u < prob) ? -1 : 1;
    }
  }
}

// wl.cu:388-407 (class h): negate the down bonds of row 0.
void orc_apply_horizontal_error(int8_t* J, int X, int Y, int R)
{
  const size_t N = static_cast<size_t>(X) * Y;
  for (int k = 0; k < R; ++k)
    for (int col = 0; col < Y; ++col) J[k * 2 * N + N + col] = static_cast<int8_t>(-J[k * 2 * N + N + col]);
}

// wl.cu:409-428 (class v): negate the right bonds of column 0.
void orc_apply_vertical_error(int8_t* J, int X, int Y, int R)
{
  const size_t N = static_cast<size_t>(X) * Y;
  for (int k = 0; k < R; ++k)
    for (int row = 0; row < X; ++row) J[k * 2 * N + row * Y] = static_cast<int8_t>(-J[k * 2 * N + row * Y]);
}

// prerun.cu:56-75 dispatch: 'h', 'v', 'c' (both); anything else is trivial.
void orc_apply_error_class(int8_t* J, int X, int Y, int R, char cls)
{
  if (cls == 'h' || cls == 'c') orc_apply_horizontal_error(J, X, Y, R);
  if (cls == 'v' || cls == 'c') orc_apply_vertical_error(J, X, Y, R);
}

// wl.cu:430-457.  Every spin thread of a lattice reads stream
// (seed+k, 1, site): its first draw is a candidate for the lattice's
// probability p0 (installed by a float CAS, first writer wins), its second
// draw sets the spin.  Which thread wins the CAS is unordered in the
// reference; this restatement fixes the winner to site 0, so
// p0 = draw 0 and spin s = (draw s+1 < p0) ? -1 : +1.
void orc_init_lattice(int8_t* lat, int X, int Y, size_t num_lattices, int seed, int wpi)
{
  const size_t N = static_cast<size_t>(X) * Y;
  for (size_t l = 0; l < num_lattices; ++l) {
    const uint64_t k = l / static_cast<size_t>(wpi);
    Stream st(key_u32(seed, k), 1, 0);
    std::vector<float> d(N + 1);
    for (size_t t = 0; t <= N; ++t) d[t] = st.uniform();
    const float p0 = d[0];
    for (size_t s = 0; s < N; ++s) {
      const double u = d[s + 1];
      lat[l * N + s] = (u < p0) ? -1 : 1;
    }
  }
}

// ---------------------------------------------------------------- energy ---
// wl.cu:261-362.
void orc_calc_energy(int boundary, int* E, const int8_t* lat, const int8_t* J, const int* off_lat, int X, int Y,
                     size_t num_lattices, int wpi)
{
  const size_t N = static_cast<size_t>(X) * Y;
  for (size_t t = 0; t < num_lattices; ++t) {
    const size_t k = t / static_cast<size_t>(wpi);
    E[t] = energy_of(lat + off_lat[t], J + k * 2 * N, X, Y, boundary);
  }
}

// ------------------------------------------------------------- pre-run -----
// wl.cu:473-560 with store_lattice wl.cu:227-257.  The reference's walkers of
// one sample share one histogram that they read without synchronisation; the
// restatement runs them round-synchronously: in round `it` every walker
// decides against the histogram as it stood after round it-1, then all
// increments of the round land, then each still-empty coarse bin takes the
// lattice of the lowest-index walker that accepted a move into it.
// Each round consumes two draws per walker (site, acceptance).
void orc_wang_landau_pre_run(int* E, int* flag_found, int8_t* lat, int8_t* found_lat, unsigned long long* H,
                             uint64_t* seed_off, const int8_t* J, const int* off_lat, int E_min, int E_max, int n_iter,
                             int X, int Y, int seed, unsigned n_int, int len_int, size_t total_walker, int wpi,
                             int boundary)
{
  const int N = X * Y;
  const int len_hist = E_max - E_min + 1;
  const size_t R = total_walker / static_cast<size_t>(wpi);
  std::vector<int> accepted(static_cast<size_t>(wpi));
  std::vector<int> idx_hit(static_cast<size_t>(wpi));
  for (size_t k = 0; k < R; ++k) {
    std::vector<Stream> rng;
    rng.reserve(static_cast<size_t>(wpi));
    for (int w = 0; w < wpi; ++w) {
      const size_t t = k * wpi + w;
      rng.emplace_back(key_u32(seed, k), 2 + static_cast<uint64_t>(w), seed_off[t]);
    }
    const int8_t* Jk = J + k * 2 * N;
    unsigned long long* Hk = H + k * len_hist;
    std::vector<char> live(static_cast<size_t>(wpi));
    for (int w = 0; w < wpi; ++w) {
      const int e = E[k * wpi + w];
      live[w] = e >= E_min && e <= E_max;
    }
    for (int it = 0; it < n_iter; ++it) {
      for (int w = 0; w < wpi; ++w) {
        const size_t t = k * wpi + w;
        accepted[w] = 0;
        idx_hit[w] = -1;
        if (!live[w]) continue;
        int8_t* s = lat + off_lat[t];
        const Proposal p = propose(rng[w], s, Jk, E[t], X, Y, boundary);
        if (p.new_energy > E_max || p.new_energy < E_min) {  // wl.cu:522-529: the walker stops
          E[t] = p.new_energy;
          live[w] = 0;
          continue;
        }
        const int io = E[t] - E_min;
        const int in = p.new_energy - E_min;
        const double prob = std::exp(static_cast<double>(Hk[io]) - static_cast<double>(Hk[in]));
        const double u = rng[w].uniform();
        if (u < prob) {
          s[p.site] = static_cast<int8_t>(-s[p.site]);
          E[t] = p.new_energy;
          accepted[w] = 1;
          idx_hit[w] = in;
        } else {
          accepted[w] = 0;
          idx_hit[w] = io;
        }
      }
      for (int w = 0; w < wpi; ++w)
        if (idx_hit[w] >= 0) Hk[idx_hit[w]] += 1;
      for (int w = 0; w < wpi; ++w) {
        if (!accepted[w]) continue;
        const size_t t = k * wpi + w;
        const int q = (E[t] - E_min) / len_int;
        const unsigned bin = (q < static_cast<int>(n_int)) ? static_cast<unsigned>(q) : n_int - 1;
        int& flag = flag_found[k * n_int + bin];
        if (flag != 0) continue;
        flag = 1;
        std::memcpy(found_lat + (k * n_int + bin) * N, lat + off_lat[t], static_cast<size_t>(N));
      }
    }
    for (int w = 0; w < wpi; ++w) seed_off[k * wpi + w] = rng[w].pos;
  }
}

// ------------------------------------------------------ main WL sweep ------
// wl.cu:1033-1175.  Returns the number of walkers that proposed an energy
// outside the pre-run spectrum (their found flag is tid+1 and newE holds the
// energy, wl.cu:1091-1104).  Windows with cond == 1 walk with frozen
// histogram and log g; the reference's test there (wl.cu:1161) is `<= end ||
// >= start`, which is always true and reads log g outside the walker's own
// window; the restatement keeps the walker inside its window (`&&`).
int orc_wang_landau(int8_t* lat, const int8_t* J, unsigned long long* H, double* logG, const double* factor, int* E,
                    int* newE, uint64_t* off_iter, int* found, const int* start, const int* end, const int* off_hist,
                    const int* off_lat, const int8_t* cond, const int8_t* spectrum, const int* off_spec,
                    const int* cond_inter, int X, int Y, int n_iter, int num_lattices, int n_int, int wpi, int seed,
                    int boundary)
{
  const int N = X * Y;
  const int W = wpi / n_int;
  int n_new = 0;
  for (int t = 0; t < num_lattices; ++t) {
    const int k = t / wpi;
    const int b = t / W;
    if (cond_inter[k] == -1) continue;
    Stream rng(key_u32(seed, static_cast<uint64_t>(k)), static_cast<uint64_t>(t % wpi), off_iter[t]);
    int8_t* s = lat + off_lat[t];
    const int8_t* Jk = J + static_cast<size_t>(k) * 2 * N;
    const int e0 = start[k * n_int];
    const int e_last = end[k * n_int + n_int - 1];
    const double lnf = std::log(factor[t]);
    for (int it = 0; it < n_iter; ++it) {
      const Proposal p = propose(rng, s, Jk, E[t], X, Y, boundary);
      // An energy outside the sample's spectrum range counts as new as well
      // (the reference reads the mask out of bounds there, wl.cu:1091).
      if (p.new_energy < e0 || p.new_energy > e_last || spectrum[off_spec[k] + p.new_energy - e0] != 1) {
        found[t] = t + 1;
        newE[t] = p.new_energy;
        ++n_new;
        break;
      }
      found[t] = 0;
      const int io = off_hist[t] + E[t] - start[b];
      const bool inside = p.new_energy <= end[b] && p.new_energy >= start[b];
      if (cond[b] == 0) {
        if (!inside) {
          H[io] += 1;
          logG[io] += lnf;
          continue;
        }
        const int in = off_hist[t] + p.new_energy - start[b];
        const double prob = std::min(1.0, std::exp(logG[io] - logG[in]));
        const double u = rng.uniform();
        if (u < prob) {
          s[p.site] = static_cast<int8_t>(-s[p.site]);
          H[in] += 1;
          logG[in] += lnf;
          E[t] = p.new_energy;
        } else {
          H[io] += 1;
          logG[io] += lnf;
        }
      } else {
        if (!inside) continue;
        const int in = off_hist[t] + p.new_energy - start[b];
        const double prob = std::min(1.0, std::exp(logG[io] - logG[in]));
        const double u = rng.uniform();
        if (u < prob) {
          s[p.site] = static_cast<int8_t>(-s[p.site]);
          E[t] = p.new_energy;
        }
      }
    }
    off_iter[t] = rng.pos;
  }
  return n_new;
}

// ------------------------------------------------------------ flatness -----
// wl.cu:892-967.  A window (cond == 0, sample not finished) is flat when
// every walker has min H >= alpha * mean H over the window's spectrum bins;
// then cond = 1, its histograms are cleared and every walker's f -> sqrt(f).
void orc_check_histogram(unsigned long long* H, double* factor, int8_t* cond, const int* off_hist, const int* end,
                         const int* start, const int8_t* spectrum, const int* off_spec, const int* cond_inter,
                         double alpha, int num_walker_total, int wpi, int n_int)
{
  const int W = wpi / n_int;
  const int n_windows = num_walker_total / W;
  for (int b = 0; b < n_windows; ++b) {
    const int k = (b * W) / wpi;
    if (cond[b] == 1 || cond_inter[k] == -1) continue;
    const int len = end[b] - start[b] + 1;
    int flat = 0;
    for (int w = 0; w < W; ++w) {
      const int t = b * W + w;
      unsigned long long mn = 2147483647ull;  // INT_MAX, wl.cu:923
      double sum = 0;
      int cnt = 0;
      for (int i = 0; i < len; ++i) {
        if (spectrum[off_spec[k] + start[b] + i - start[k * n_int]] != 1) continue;
        const unsigned long long h = H[off_hist[t] + i];
        if (h < mn) mn = h;
        sum += static_cast<double>(h);
        ++cnt;
      }
      if (cnt > 0) {
        const double avg = sum / cnt;
        if (static_cast<double>(mn) >= alpha * avg) ++flat;
      }
    }
    if (flat == W) {
      cond[b] = 1;
      for (int w = 0; w < W; ++w) {
        const int t = b * W + w;
        for (int i = 0; i < len; ++i) H[off_hist[t] + i] = 0;
        factor[t] = std::sqrt(factor[t]);
      }
    }
  }
}

// ----------------------------------------------- window log g averaging ----
// wl.cu:710-783 followed by wl.cu:969-1031: for every window with cond == 1
// (sample not finished) each spectrum bin becomes the mean over the window's
// W walkers, summed in walker order as ((0 + g0/W) + g1/W) + ...; bins outside
// the spectrum become 0.  (The reference sums with FP64 atomics in an
// unspecified order.)
void orc_average_log_g(double* logG, const int* start, const int* end, const int8_t* spectrum, const int* off_spec,
                       const int8_t* cond, const int* off_hist, const int* cond_inter, int R, int W, int n_int)
{
  for (int k = 0; k < R; ++k) {
    if (cond_inter[k] == -1) continue;
    for (int bl = 0; bl < n_int; ++bl) {
      const int b = k * n_int + bl;
      if (cond[b] != 1) continue;
      const int len = end[b] - start[b] + 1;
      for (int i = 0; i < len; ++i) {
        double avg = 0.0;
        if (spectrum[off_spec[k] + start[b] + i - start[k * n_int]] == 1) {
          for (int w = 0; w < W; ++w) avg += logG[off_hist[b * W + w] + i] / W;
        }
        for (int w = 0; w < W; ++w) logG[off_hist[b * W + w] + i] = avg;
      }
    }
  }
}

// wl.cu:596-613: reopen a flat window unless its f reached exp(beta).
void orc_reset_cond(int8_t* cond, const double* factor, int total_intervals, double beta, int W)
{
  const double lim = std::exp(beta);
  for (int t = 0; t < total_intervals; ++t)
    if (cond[t] == 1 && factor[static_cast<size_t>(t) * W] > lim) cond[t] = 0;
}

// wl.cu:662-708: per sample, the number of windows with cond == 1, or -1
// when all of them are.
void orc_check_finished(int* cond_inter, const int8_t* cond, int n_int, int R)
{
  for (int k = 0; k < R; ++k) {
    int s = 0;
    for (int b = 0; b < n_int; ++b) s += cond[k * n_int + b];
    cond_inter[k] = (s == n_int) ? -1 : s;
  }
}

// ---------------------------------------------------- replica exchange -----
// wl.cu:785-890.  Window b (not the last of its sample, right parity) pairs
// walker t with walker perm[t] of window b+1; walker 0 of window b first
// shuffles perm[] in place with W-1 draws of its own stream (Fisher-Yates).
// `global_parity` selects the reference's parity on the global window index
// (wl.cu:830); 0 uses the window's index inside its sample.
void orc_replica_exchange(int* off_lat, int* E, int* perm, uint64_t* off_iter, const int* start, const int* end,
                          const int* off_hist, const int* cond_inter, const double* logG, int even, int seed,
                          int n_int, int wpi, int total_intervals, int global_parity)
{
  const int W = wpi / n_int;
  for (int b = 0; b < total_intervals; ++b) {
    if (b % n_int == n_int - 1) continue;
    const int par = global_parity ? b : (b % n_int);
    if ((even && par % 2 != 0) || (!even && par % 2 == 0)) continue;
    const int k = (b * W) / wpi;
    if (cond_inter[k] == -1) continue;
    {
      const int t0 = b * W;
      Stream st(key_i32(seed, static_cast<uint64_t>(k)), static_cast<uint64_t>(t0 % wpi), off_iter[t0]);
      for (int i = W - 1; i > 0; --i) {
        double u = st.uniform();
        u *= (i + 0.999999);
        const int r = static_cast<int>(std::trunc(u));
        std::swap(perm[t0 + i], perm[t0 + r]);
      }
      off_iter[t0] = st.pos;
    }
    for (int w = 0; w < W; ++w) {
      const int t = b * W + w;
      const int o = W * (b + 1) + perm[t];
      if (E[t] > end[b + 1] || E[t] < start[b + 1]) continue;
      if (E[o] > end[b] || E[o] < start[b]) continue;
      const double gi_x = logG[off_hist[t] + E[t] - start[b]];
      const double gi_y = logG[off_hist[t] + E[o] - start[b]];
      const double gj_y = logG[off_hist[o] + E[o] - start[b + 1]];
      const double gj_x = logG[off_hist[o] + E[t] - start[b + 1]];
      const double prob = std::min(1.0, std::exp(gi_x - gi_y) * std::exp(gj_y - gj_x));
      Stream st(key_i32(seed, static_cast<uint64_t>(k)), static_cast<uint64_t>(t % wpi), off_iter[t]);
      if (st.uniform() < prob) {
        std::swap(off_lat[t], off_lat[o]);
        std::swap(E[t], E[o]);
      }
      off_iter[t] = st.pos;
    }
  }
}

}  // extern "C"

extern "C" {

// Host exp/log of the oracle (glibc), for comparison with CUDA's.
void orc_exp_log(const double* x, double* e, double* l, int n)
{
  for (int q = 0; q < n; ++q) {
    e[q] = std::exp(x[q]);
    l[q] = std::log(x[q]);
  }
}

// The modification-factor chain of the main run: f_0 = x0, f_{k+1} =
// sqrt(f_k) (wl.cu:965) and ln f_k (wl.cu:1110).
void orc_sqrt_chain(double x0, int n, double* f, double* lf)
{
  double x = x0;
  for (int q = 0; q < n; ++q) {
    f[q] = x;
    lf[q] = std::log(x);
    x = std::sqrt(x);
  }
}

}  // extern "C"
