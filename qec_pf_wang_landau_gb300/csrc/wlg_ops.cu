// Operator layer: one sm_103a kernel per device operation of the reference's
// kernel library (src/wl.cu of dfki-ric-quantum/qec_pf_wang_landau), on the
// reference's data layout, behind the extern "C" entry points of wlg.h.
//
// Layout (shared with the reference): spins int8 +-1, lattice t at
// d_offset_lattice[t]; couplings int8 [sample][2N] with the right bond of
// site (i,j) at i*Y+j and its down bond at N+i*Y+j; per-walker dense
// histogram / log g slices starting at d_offset_histogram[t], indexed by
// E - start[window]; walker t belongs to window t / W and sample t / (I*W).

#include <cuda_runtime.h>

#include <climits>
#include <cstdint>
#include <algorithm>
#include <cstdio>

#include "../../include/wlg.h"
#include "wlg_internal.h"
#include "wlg_lattice.cuh"
#include "wlg_rng.cuh"

namespace wlg {
namespace {

constexpr int kThreads = 128;

// -------------------------------------------------------------- disorder ----

__global__ void k_init_interactions(int8_t* __restrict__ J, size_t N, int R, int seed, float prob)
{
  const size_t t = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= 2 * N * static_cast<size_t>(R)) return;
  const size_t k = t / (2 * N);
  Stream st;
  st.init(key_size(seed, k), 0, t % (2 * N));
  const double u = st.uniform();
  J[t] = (u < prob) ? -1 : 1;
}

// which: 0 = horizontal chain (down bonds of row 0), 1 = vertical chain
// (right bonds of column 0).
__global__ void k_apply_chain(int8_t* __restrict__ J, int X, int Y, int R, int which)
{
  const int len = which == 0 ? Y : X;
  const long long t = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= static_cast<long long>(len) * R) return;
  const size_t N = static_cast<size_t>(X) * Y;
  const size_t k = static_cast<size_t>(t / len);
  const int q = static_cast<int>(t % len);
  const size_t idx = k * 2 * N + (which == 0 ? N + q : static_cast<size_t>(q) * Y);
  J[idx] = static_cast<int8_t>(-J[idx]);
}

__global__ void k_init_lattice(int8_t* __restrict__ lat, int X, int Y, size_t num_lattices, int seed, int wpi)
{
  const size_t t = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  const size_t N = static_cast<size_t>(X) * Y;
  if (t >= N * num_lattices) return;
  const size_t l = t / N;
  const size_t s = t % N;
  const uint64_t key = key_u32(seed, l / static_cast<size_t>(wpi));
  Stream st;
  st.init(key, 1, 0);
  const float p0 = st.uniform();
  st.init(key, 1, s + 1);
  const double u = st.uniform();
  lat[t] = (u < p0) ? -1 : 1;
}

// ---------------------------------------------------------------- energy ----

__global__ void k_calc_energy(int boundary, int* __restrict__ E, const int8_t* __restrict__ lat,
                              const int8_t* __restrict__ J, const int* __restrict__ off_lat, int X, int Y,
                              size_t num_lattices, int wpi)
{
  const size_t t = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= num_lattices) return;
  const size_t N = static_cast<size_t>(X) * Y;
  E[t] = energy_i8(lat + off_lat[t], J + (t / static_cast<size_t>(wpi)) * 2 * N, X, Y, boundary);
}

// --------------------------------------------------------------- pre-run ----
// One CTA per sample, one thread per walker, the sample's histogram and
// coarse-bin claims in shared memory.  Round-synchronous: decisions of round
// r read the histogram after round r-1; barrier; increments and claims;
// barrier; the lowest claimant of a still-empty bin stores its lattice.
__global__ void k_prerun(int* __restrict__ E, int* __restrict__ flag_found, int8_t* __restrict__ lat,
                         int8_t* __restrict__ found_lat, unsigned long long* __restrict__ H,
                         uint64_t* __restrict__ seed_off, const int8_t* __restrict__ J,
                         const int* __restrict__ off_lat, int E_min, int E_max, int n_iter, int X, int Y, int seed,
                         unsigned n_int, int len_int, int wpi, int boundary)
{
  extern __shared__ unsigned long long sm[];
  const int len_hist = E_max - E_min + 1;
  unsigned long long* hist = sm;
  int* claim = reinterpret_cast<int*>(hist + len_hist);
  int* found = claim + n_int;

  const int k = blockIdx.x;
  const int w = threadIdx.x;
  const int N = X * Y;
  const bool live = w < wpi;
  const size_t t = static_cast<size_t>(k) * wpi + w;

  for (int q = threadIdx.x; q < len_hist; q += blockDim.x) hist[q] = H[static_cast<size_t>(k) * len_hist + q];
  for (int q = threadIdx.x; q < static_cast<int>(n_int); q += blockDim.x) {
    claim[q] = INT_MAX;
    found[q] = flag_found[static_cast<size_t>(k) * n_int + q];
  }

  Stream rng;
  int energy = 0;
  int8_t* s = nullptr;
  bool ok = true;
  if (live) {
    rng.init(key_u32(seed, static_cast<uint64_t>(k)), 2 + static_cast<uint64_t>(w), seed_off[t]);
    energy = E[t];
    s = lat + off_lat[t];
    ok = energy >= E_min && energy <= E_max;  // a walker outside the range never indexes the histogram
  }
  const int8_t* Jk = J + static_cast<size_t>(k) * 2 * N;
  const double site_scale = (N - 1 + 0.999999);
  __syncthreads();

  for (int it = 0; it < n_iter; ++it) {
    int hit = -1;
    bool acc = false;
    if (live && ok) {
      const Move m = propose_i8(rng, s, Jk, energy, X, Y, site_scale, boundary);
      if (m.new_energy > E_max || m.new_energy < E_min) {  // wl.cu:522-529: the walker stops
        energy = m.new_energy;                               // and keeps the offending energy
        ok = false;
      } else {
        const int io = energy - E_min;
        const int in = m.new_energy - E_min;
        const double prob = exp(static_cast<double>(hist[io]) - static_cast<double>(hist[in]));
        const double u = rng.uniform();
        if (u < prob) {
          s[m.site] = static_cast<int8_t>(-s[m.site]);
          energy = m.new_energy;
          acc = true;
          hit = in;
        } else {
          hit = io;
        }
      }
    }
    __syncthreads();
    int bin = -1;
    if (hit >= 0) atomicAdd(&hist[hit], 1ull);
    if (acc) {
      const int q = (energy - E_min) / len_int;
      bin = (q < static_cast<int>(n_int)) ? q : static_cast<int>(n_int) - 1;
      if (found[bin] == 0) atomicMin(&claim[bin], w);
      else bin = -1;
    }
    __syncthreads();
    if (bin >= 0 && claim[bin] == w && found[bin] == 0) {
      found[bin] = 1;
      int8_t* dst = found_lat + (static_cast<size_t>(k) * n_int + bin) * N;
      for (int q = 0; q < N; ++q) dst[q] = s[q];
    }
  }
  __syncthreads();
  for (int q = threadIdx.x; q < len_hist; q += blockDim.x) H[static_cast<size_t>(k) * len_hist + q] = hist[q];
  for (int q = threadIdx.x; q < static_cast<int>(n_int); q += blockDim.x)
    flag_found[static_cast<size_t>(k) * n_int + q] = found[q];
  if (live) {
    E[t] = energy;
    seed_off[t] = rng.pos;
  }
}

// ------------------------------------------------------- main WL sweep -----
// wl.cu:1033-1175, one thread per walker.
__global__ void k_wang_landau(int8_t* __restrict__ lat, const int8_t* __restrict__ J,
                              unsigned long long* __restrict__ H, double* __restrict__ logG,
                              const double* __restrict__ factor, int* __restrict__ E, int* __restrict__ newE,
                              uint64_t* __restrict__ off_iter, int* __restrict__ found, const int* __restrict__ start,
                              const int* __restrict__ end, const int* __restrict__ off_hist,
                              const int* __restrict__ off_lat, const int8_t* __restrict__ cond,
                              const int8_t* __restrict__ spectrum, const int* __restrict__ off_spec,
                              const int* __restrict__ cond_inter, int X, int Y, int n_iter, int num_lattices,
                              int n_int, int wpi, int seed, int boundary)
{
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= num_lattices) return;
  const int W = wpi / n_int;
  const int k = t / wpi;
  const int b = t / W;
  if (cond_inter[k] == -1) return;
  const int N = X * Y;
  Stream rng;
  rng.init(key_u32(seed, static_cast<uint64_t>(k)), static_cast<uint64_t>(t % wpi), off_iter[t]);
  int8_t* s = lat + off_lat[t];
  const int8_t* Jk = J + static_cast<size_t>(k) * 2 * N;
  const int8_t* mask = spectrum + off_spec[k] - start[k * n_int];
  const int e_first = start[k * n_int], e_last = end[k * n_int + n_int - 1];
  const int lo = start[b], hi = end[b];
  unsigned long long* Hw = H + off_hist[t] - lo;
  double* Gw = logG + off_hist[t] - lo;
  const double lnf = log(factor[t]);
  const double site_scale = (N - 1 + 0.999999);
  const bool frozen = cond[b] != 0;
  int energy = E[t];
  int flag = 0;
  for (int it = 0; it < n_iter; ++it) {
    const Move m = propose_i8(rng, s, Jk, energy, X, Y, site_scale, boundary);
    // wl.cu:1091-1104; an energy outside the sample's spectrum range counts
    // as new too (the reference reads the mask out of bounds there).
    if (m.new_energy < e_first || m.new_energy > e_last || mask[m.new_energy] != 1) {
      flag = t + 1;
      newE[t] = m.new_energy;
      break;
    }
    const bool inside = m.new_energy <= hi && m.new_energy >= lo;
    if (!frozen) {
      if (!inside) {
        Hw[energy] += 1;
        Gw[energy] += lnf;
        continue;
      }
      const double prob = fmin(1.0, exp(Gw[energy] - Gw[m.new_energy]));
      const double u = rng.uniform();
      if (u < prob) {
        s[m.site] = static_cast<int8_t>(-s[m.site]);
        energy = m.new_energy;
      }
      Hw[energy] += 1;
      Gw[energy] += lnf;
    } else if (inside) {
      const double prob = fmin(1.0, exp(Gw[energy] - Gw[m.new_energy]));
      const double u = rng.uniform();
      if (u < prob) {
        s[m.site] = static_cast<int8_t>(-s[m.site]);
        energy = m.new_energy;
      }
    }
  }
  if (n_iter > 0) found[t] = flag;
  E[t] = energy;
  off_iter[t] = rng.pos;
}

// -------------------------------------------------------------- flatness ----
// wl.cu:892-967, one block per window, one thread per walker.
__global__ void k_check_histogram(unsigned long long* __restrict__ H, double* __restrict__ factor,
                                  int8_t* __restrict__ cond, const int* __restrict__ off_hist,
                                  const int* __restrict__ end, const int* __restrict__ start,
                                  const int8_t* __restrict__ spectrum, const int* __restrict__ off_spec,
                                  const int* __restrict__ cond_inter, double alpha, int W, int wpi, int n_int)
{
  const int b = blockIdx.x;
  const int w = threadIdx.x;
  const int k = (b * W) / wpi;
  if (cond[b] == 1 || cond_inter[k] == -1) return;
  const int len = end[b] - start[b] + 1;
  const int8_t* mask = spectrum + off_spec[k] + start[b] - start[k * n_int];
  int flat = 0;
  if (w < W) {
    const unsigned long long* h = H + off_hist[b * W + w];
    unsigned long long mn = 2147483647ull;
    unsigned long long sum = 0;  // exact: the reference's double sum of integers is exact below 2^53
    int cnt = 0;
    for (int i = 0; i < len; ++i) {
      if (mask[i] != 1) continue;
      const unsigned long long v = h[i];
      mn = v < mn ? v : mn;
      sum += v;
      ++cnt;
    }
    if (cnt > 0) {
      const double avg = static_cast<double>(sum) / cnt;
      flat = static_cast<double>(mn) >= alpha * avg ? 1 : 0;
    }
  }
  const int n_flat = __syncthreads_count(flat);
  if (n_flat == W && w < W) {
    unsigned long long* h = H + off_hist[b * W + w];
    for (int i = 0; i < len; ++i) h[i] = 0;
    factor[b * W + w] = sqrt(factor[b * W + w]);
    if (w == 0) cond[b] = 1;
  }
}

// ------------------------------------------------------- log g averaging ----
// wl.cu:710-783 + :969-1031 fused; one block per window, threads over bins.
__global__ void k_average_log_g(double* __restrict__ logG, const int* __restrict__ start,
                                const int* __restrict__ end, const int8_t* __restrict__ spectrum,
                                const int* __restrict__ off_spec, const int8_t* __restrict__ cond,
                                const int* __restrict__ off_hist, const int* __restrict__ cond_inter, int R, int W,
                                int n_int)
{
  const int total = R * n_int;
  for (int b = blockIdx.x; b < total; b += gridDim.x) {
    const int k = b / n_int;
    if (cond[b] != 1 || cond_inter[k] == -1) continue;
    const int len = end[b] - start[b] + 1;
    const int8_t* mask = spectrum + off_spec[k] + start[b] - start[k * n_int];
    for (int i = threadIdx.x; i < len; i += blockDim.x) {
      double avg = 0.0;
      if (mask[i] == 1) {
        for (int w = 0; w < W; ++w) avg += logG[off_hist[b * W + w] + i] / W;
      }
      for (int w = 0; w < W; ++w) logG[off_hist[b * W + w] + i] = avg;
    }
  }
}

__global__ void k_reset_cond(int8_t* __restrict__ cond, const double* __restrict__ factor, int total, double beta,
                             int W)
{
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= total) return;
  if (cond[t] == 1 && factor[static_cast<size_t>(t) * W] > exp(beta)) cond[t] = 0;
}

__global__ void k_check_finished(int* __restrict__ cond_inter, const int8_t* __restrict__ cond, int n_int, int R)
{
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= R) return;
  int s = 0;
  for (int b = 0; b < n_int; ++b) s += cond[k * n_int + b];
  cond_inter[k] = (s == n_int) ? -1 : s;
}

// ------------------------------------------------------ replica exchange ----
// wl.cu:785-890, one block per window, one thread per walker.
__global__ void k_replica_exchange(int* __restrict__ off_lat, int* __restrict__ E, int* __restrict__ perm,
                                   uint64_t* __restrict__ off_iter, const int* __restrict__ start,
                                   const int* __restrict__ end, const int* __restrict__ off_hist,
                                   const int* __restrict__ cond_inter, const double* __restrict__ logG, int even,
                                   int seed, int n_int, int W, int wpi, int global_parity)
{
  const int b = blockIdx.x;
  if (b % n_int == n_int - 1) return;
  const int par = global_parity ? b : (b % n_int);
  if ((even && par % 2 != 0) || (!even && par % 2 == 0)) return;
  const int k = (b * W) / wpi;
  if (cond_inter[k] == -1) return;
  const int w = threadIdx.x;
  const int t0 = b * W;
  if (w == 0) {
    Stream st;
    st.init(key_i32(seed, static_cast<uint64_t>(k)), static_cast<uint64_t>(t0 % wpi), off_iter[t0]);
    for (int i = W - 1; i > 0; --i) {
      double u = st.uniform();
      u *= (i + 0.999999);
      const int r = static_cast<int>(trunc(u));
      const int tmp = perm[t0 + i];
      perm[t0 + i] = perm[t0 + r];
      perm[t0 + r] = tmp;
    }
    off_iter[t0] = st.pos;
  }
  __syncthreads();
  if (w >= W) return;
  const int t = t0 + w;
  const int o = W * (b + 1) + perm[t];
  const int et = E[t], eo = E[o];
  if (et > end[b + 1] || et < start[b + 1]) return;
  if (eo > end[b] || eo < start[b]) return;
  const double gi_x = logG[off_hist[t] + et - start[b]];
  const double gi_y = logG[off_hist[t] + eo - start[b]];
  const double gj_y = logG[off_hist[o] + eo - start[b + 1]];
  const double gj_x = logG[off_hist[o] + et - start[b + 1]];
  const double prob = fmin(1.0, exp(gi_x - gi_y) * exp(gj_y - gj_x));
  Stream st;
  st.init(key_i32(seed, static_cast<uint64_t>(k)), static_cast<uint64_t>(t % wpi), off_iter[t]);
  if (st.uniform() < prob) {
    const int tmp = off_lat[t];
    off_lat[t] = off_lat[o];
    off_lat[o] = tmp;
    E[t] = eo;
    E[o] = et;
  }
  off_iter[t] = st.pos;
}

// ------------------------------------------------------------ reductions ----

__global__ void k_max_int(const int* __restrict__ in, size_t n, int* __restrict__ out)
{
  int m = INT_MIN;
  for (size_t q = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x; q < n;
       q += static_cast<size_t>(gridDim.x) * blockDim.x)
    m = max(m, in[q]);
  for (int d = 16; d > 0; d >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, d));
  if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

// Maximum of non-negative doubles through their bit patterns, which order
// like the values.
__global__ void k_max_f64_nonneg(const double* __restrict__ in, size_t n, unsigned long long* __restrict__ out)
{
  unsigned long long m = 0;
  for (size_t q = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x; q < n;
       q += static_cast<size_t>(gridDim.x) * blockDim.x) {
    const unsigned long long v = static_cast<unsigned long long>(__double_as_longlong(in[q]));
    m = v > m ? v : m;
  }
  for (int d = 16; d > 0; d >>= 1) {
    const unsigned long long o = __shfl_xor_sync(0xffffffffu, m, d);
    m = o > m ? o : m;
  }
  if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

__global__ void k_fill_int(int* out, int v) { *out = v; }

inline int blocks_for(size_t n) { return static_cast<int>((n + kThreads - 1) / kThreads); }

}  // namespace
}  // namespace wlg

using namespace wlg;

// ------------------------------------------------------------ C ABI -------

extern "C" {

wlg_status wlg_init_interactions(int8_t* d_J, size_t lattice_size, int num_samples, int seed, float prob,
                                 wlg_stream stream)
{
  if (d_J == nullptr || lattice_size == 0 || num_samples <= 0) return WLG_ERR_INVALID;
  const size_t n = 2 * lattice_size * static_cast<size_t>(num_samples);
  k_init_interactions<<<blocks_for(n), kThreads, 0, as_stream(stream)>>>(d_J, lattice_size, num_samples, seed, prob);
  return launch_status();
}

wlg_status wlg_apply_error_class(int8_t* d_J, int X, int Y, int num_samples, char error_class, wlg_stream stream)
{
  if (d_J == nullptr || X <= 0 || Y <= 0 || num_samples <= 0) return WLG_ERR_INVALID;
  cudaStream_t s = as_stream(stream);
  if (error_class == 'h' || error_class == 'c')
    k_apply_chain<<<blocks_for(static_cast<size_t>(Y) * num_samples), kThreads, 0, s>>>(d_J, X, Y, num_samples, 0);
  if (error_class == 'v' || error_class == 'c')
    k_apply_chain<<<blocks_for(static_cast<size_t>(X) * num_samples), kThreads, 0, s>>>(d_J, X, Y, num_samples, 1);
  return launch_status();
}

wlg_status wlg_init_lattice(int8_t* d_lattice, int X, int Y, size_t num_lattices, int seed, int walker_per_sample,
                            wlg_stream stream)
{
  if (d_lattice == nullptr || X <= 0 || Y <= 0 || walker_per_sample <= 0) return WLG_ERR_INVALID;
  if (num_lattices == 0) return WLG_OK;
  const size_t n = static_cast<size_t>(X) * Y * num_lattices;
  k_init_lattice<<<blocks_for(n), kThreads, 0, as_stream(stream)>>>(d_lattice, X, Y, num_lattices, seed,
                                                                     walker_per_sample);
  return launch_status();
}

wlg_status wlg_calc_energy(int boundary, int* d_energy, const int8_t* d_lattice, const int8_t* d_J,
                           const int* d_offset_lattice, int X, int Y, size_t num_lattices, int walker_per_sample,
                           wlg_stream stream)
{
  if ((boundary != 0 && boundary != 1) || X <= 0 || Y <= 0 || walker_per_sample <= 0) return WLG_ERR_INVALID;
  if (num_lattices == 0) return WLG_OK;
  k_calc_energy<<<blocks_for(num_lattices), kThreads, 0, as_stream(stream)>>>(
    boundary, d_energy, d_lattice, d_J, d_offset_lattice, X, Y, num_lattices, walker_per_sample);
  return launch_status();
}

wlg_status wlg_wang_landau_pre_run(int* d_energy, int* d_flag_found_interval, int8_t* d_lattice,
                                   int8_t* d_found_interval_lattice, unsigned long long* d_histogram,
                                   uint64_t* d_seed_offset, const int8_t* d_J, const int* d_offset_lattice, int E_min,
                                   int E_max, int num_iterations, int X, int Y, int seed, unsigned num_intervals,
                                   int len_interval, size_t num_total_walker, int walker_per_sample, int boundary,
                                   wlg_stream stream)
{
  if ((boundary != 0 && boundary != 1) || X <= 0 || Y <= 0 || walker_per_sample <= 0 || walker_per_sample > 1024 ||
      num_intervals == 0 || len_interval <= 0 || E_max < E_min || num_total_walker % walker_per_sample != 0)
    return WLG_ERR_INVALID;
  const int R = static_cast<int>(num_total_walker / walker_per_sample);
  if (R == 0 || num_iterations <= 0) return WLG_OK;
  const int len_hist = E_max - E_min + 1;
  const size_t smem = static_cast<size_t>(len_hist) * sizeof(unsigned long long) + 2 * sizeof(int) * num_intervals;
  if (smem > 200 * 1024) return WLG_ERR_INVALID;
  cudaStream_t s = as_stream(stream);
  if (smem > 48 * 1024) {
    if (cudaFuncSetAttribute(k_prerun, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)) !=
        cudaSuccess)
      return WLG_ERR_CUDA;
  }
  const int threads = (walker_per_sample + 31) / 32 * 32;
  k_prerun<<<R, threads, smem, s>>>(d_energy, d_flag_found_interval, d_lattice, d_found_interval_lattice, d_histogram,
                                    d_seed_offset, d_J, d_offset_lattice, E_min, E_max, num_iterations, X, Y, seed,
                                    num_intervals, len_interval, walker_per_sample, boundary);
  return launch_status();
}

wlg_status wlg_wang_landau(int8_t* d_lattice, const int8_t* d_J, unsigned long long* d_H, double* d_logG,
                           const double* d_factor, int* d_energy, int* d_new_energy, uint64_t* d_offset_iter,
                           int* d_found, const int* d_start, const int* d_end, const int* d_offset_histogram,
                           const int* d_offset_lattice, const int8_t* d_cond, const int8_t* d_spectrum,
                           const int* d_offset_spectrum, const int* d_cond_sample, int X, int Y, int num_iterations,
                           int num_lattices, int num_intervals, int walker_per_sample, int seed, int boundary,
                           wlg_stream stream)
{
  if ((boundary != 0 && boundary != 1) || X <= 0 || Y <= 0 || num_intervals <= 0 || walker_per_sample <= 0 ||
      walker_per_sample % num_intervals != 0 || num_lattices < 0)
    return WLG_ERR_INVALID;
  if (num_lattices == 0) return WLG_OK;
  k_wang_landau<<<blocks_for(static_cast<size_t>(num_lattices)), kThreads, 0, as_stream(stream)>>>(
    d_lattice, d_J, d_H, d_logG, d_factor, d_energy, d_new_energy, d_offset_iter, d_found, d_start, d_end,
    d_offset_histogram, d_offset_lattice, d_cond, d_spectrum, d_offset_spectrum, d_cond_sample, X, Y, num_iterations,
    num_lattices, num_intervals, walker_per_sample, seed, boundary);
  return launch_status();
}

wlg_status wlg_check_histogram(unsigned long long* d_H, double* d_factor, int8_t* d_cond,
                               const int* d_offset_histogram, const int* d_end, const int* d_start,
                               const int8_t* d_spectrum, const int* d_offset_spectrum, const int* d_cond_sample,
                               double alpha, int num_walker_total, int walker_per_sample, int num_intervals,
                               wlg_stream stream)
{
  if (num_intervals <= 0 || walker_per_sample <= 0 || walker_per_sample % num_intervals != 0) return WLG_ERR_INVALID;
  const int W = walker_per_sample / num_intervals;
  if (W > 1024 || num_walker_total % W != 0) return WLG_ERR_INVALID;
  const int windows = num_walker_total / W;
  if (windows == 0) return WLG_OK;
  k_check_histogram<<<windows, (W + 31) / 32 * 32, 0, as_stream(stream)>>>(
    d_H, d_factor, d_cond, d_offset_histogram, d_end, d_start, d_spectrum, d_offset_spectrum, d_cond_sample, alpha, W,
    walker_per_sample, num_intervals);
  return launch_status();
}

wlg_status wlg_average_log_g(double* d_logG, const int* d_start, const int* d_end, const int8_t* d_spectrum,
                             const int* d_offset_spectrum, const int8_t* d_cond, const int* d_offset_histogram,
                             const int* d_cond_sample, int num_samples, int walker_per_interval, int num_intervals,
                             wlg_stream stream)
{
  if (num_samples < 0 || walker_per_interval <= 0 || num_intervals <= 0) return WLG_ERR_INVALID;
  const int total = num_samples * num_intervals;
  if (total == 0) return WLG_OK;
  const int grid = total < 65535 ? total : 65535;
  k_average_log_g<<<grid, kThreads, 0, as_stream(stream)>>>(d_logG, d_start, d_end, d_spectrum, d_offset_spectrum,
                                                             d_cond, d_offset_histogram, d_cond_sample, num_samples,
                                                             walker_per_interval, num_intervals);
  return launch_status();
}

wlg_status wlg_reset_cond(int8_t* d_cond, const double* d_factor, int total_intervals, double beta,
                          int walker_per_interval, wlg_stream stream)
{
  if (total_intervals < 0 || walker_per_interval <= 0) return WLG_ERR_INVALID;
  if (total_intervals == 0) return WLG_OK;
  k_reset_cond<<<blocks_for(static_cast<size_t>(total_intervals)), kThreads, 0, as_stream(stream)>>>(
    d_cond, d_factor, total_intervals, beta, walker_per_interval);
  return launch_status();
}

wlg_status wlg_check_finished(int* d_cond_sample, const int8_t* d_cond, int num_intervals, int num_samples,
                              wlg_stream stream)
{
  if (num_intervals <= 0 || num_samples < 0) return WLG_ERR_INVALID;
  if (num_samples == 0) return WLG_OK;
  k_check_finished<<<blocks_for(static_cast<size_t>(num_samples)), kThreads, 0, as_stream(stream)>>>(
    d_cond_sample, d_cond, num_intervals, num_samples);
  return launch_status();
}

wlg_status wlg_replica_exchange(int* d_offset_lattice, int* d_energy, int* d_replica_indices,
                                uint64_t* d_offset_iter, const int* d_start, const int* d_end,
                                const int* d_offset_histogram, const int* d_cond_sample, const double* d_logG,
                                int even, int seed, int num_intervals, int walker_per_sample, int total_intervals,
                                int global_parity, wlg_stream stream)
{
  if (num_intervals <= 0 || walker_per_sample <= 0 || walker_per_sample % num_intervals != 0 || total_intervals < 0)
    return WLG_ERR_INVALID;
  const int W = walker_per_sample / num_intervals;
  if (W > 1024) return WLG_ERR_INVALID;
  if (total_intervals == 0) return WLG_OK;
  k_replica_exchange<<<total_intervals, (W + 31) / 32 * 32, 0, as_stream(stream)>>>(
    d_offset_lattice, d_energy, d_replica_indices, d_offset_iter, d_start, d_end, d_offset_histogram, d_cond_sample,
    d_logG, even, seed, num_intervals, W, walker_per_sample, global_parity);
  return launch_status();
}

wlg_status wlg_max_int(const int* d_in, size_t n, int* d_out, wlg_stream stream)
{
  if (d_in == nullptr || d_out == nullptr) return WLG_ERR_INVALID;
  cudaStream_t s = as_stream(stream);
  k_fill_int<<<1, 1, 0, s>>>(d_out, INT_MIN);
  if (n > 0) {
    const int blocks = static_cast<int>(std::min<size_t>((n + kThreads - 1) / kThreads, 1024));
    k_max_int<<<blocks, kThreads, 0, s>>>(d_in, n, d_out);
  }
  return launch_status();
}

wlg_status wlg_max_f64_nonneg(const double* d_in, size_t n, double* d_out, wlg_stream stream)
{
  if (d_in == nullptr || d_out == nullptr) return WLG_ERR_INVALID;
  cudaStream_t s = as_stream(stream);
  if (cudaMemsetAsync(d_out, 0, sizeof(double), s) != cudaSuccess) return WLG_ERR_CUDA;
  if (n > 0) {
    const int blocks = static_cast<int>(std::min<size_t>((n + kThreads - 1) / kThreads, 1024));
    k_max_f64_nonneg<<<blocks, kThreads, 0, s>>>(d_in, n, reinterpret_cast<unsigned long long*>(d_out));
  }
  return launch_status();
}

}  // extern "C"

// ------------------------------------------------------------ diagnostics ---

namespace wlg {
namespace {
__global__ void k_uniforms(uint64_t key, uint64_t subseq, uint64_t offset, int n, float* out)
{
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  Stream st;
  st.init(key, subseq, offset);
  for (int q = 0; q < n; ++q) out[q] = st.uniform();
}
}  // namespace
}  // namespace wlg

extern "C" wlg_status wlg_uniforms(uint64_t key, uint64_t subseq, uint64_t offset, int n, float* d_out,
                                   wlg_stream stream)
{
  if (n < 0 || (n > 0 && d_out == nullptr)) return WLG_ERR_INVALID;
  if (n == 0) return WLG_OK;
  wlg::k_uniforms<<<1, 32, 0, wlg::as_stream(stream)>>>(key, subseq, offset, n, d_out);
  return wlg::launch_status();
}
