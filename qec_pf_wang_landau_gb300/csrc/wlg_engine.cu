// Batched Wang-Landau engine for sm_103a.
//
// k_pre_batch:  one CTA per problem runs the whole pre-run of the reference
//               (prerun.cu:52-133) — disorder, error chain, lattice init,
//               energy, histogram-biased walk, stored lattices — with the
//               sample's histogram in shared memory.
// k_main_batch: persistent kernel.  A team of threads (one per walker, a
//               multiple of 32) takes a problem from a global work counter
//               and runs the reference's whole main-run loop
//               (mainrun.cu:243-383) for it without leaving the GPU: WL
//               sweeps, flatness vote, window averaging, reset, convergence
//               and replica exchange, then takes the next problem.
//
// Walker state never leaves the SM during a run:
//   * spins bit-packed (one u64 register for N <= 64, else 32-bit words in
//     shared memory), couplings bit-packed (registers / shared memory);
//   * histogram (u32) and log g (f64) in shared memory, interleaved
//     [bin][walker] so a warp's 32 walkers hit 32 distinct banks, and only
//     over energies the lattice can reach (every 2nd or 4th value);
//   * the current bin's log g and count cached in registers, written back
//     only when the walker changes energy.
// Acceptance u < min(1, exp(dlogg)) is decided as log u < dlogg with FP32
// values and proven error bounds (float shadows of log g, __logf of the
// uniform); inside the band, and for the site pick near a bin edge, the exact
// FP64 expression of the reference decides, so every decision equals the
// reference's.

#include <cuda_runtime.h>

#include <climits>
#include <cstdint>

#include "../../include/wlg.h"
#include "wlg_engine.h"
#include "wlg_internal.h"
#include "wlg_lattice.cuh"
#include "wlg_accept.cuh"
#include "wlg_rng.cuh"
#include "wlg_shadow.cuh"

namespace wlg {
namespace {

constexpr double kE = 2.718281828459045;  // std::numbers::e, mainrun.cu:56

// ------------------------------------------------------------ pre-run -----

__device__ __noinline__ int site_exact(uint32_t x, double scale);

__global__ void __launch_bounds__(1024) k_pre_batch(const PreDesc* __restrict__ descs, int n,
                                                    int8_t* __restrict__ Jpool, uint8_t* __restrict__ seen_pool,
                                                    int8_t* __restrict__ found_pool, int* __restrict__ fflag_pool)
{
  const int p = blockIdx.x;
  if (p >= n) return;
  const PreDesc d = descs[p];
  const int N = d.N, X = d.X, Y = d.Y;
  const int L = 4 * N + 1;
  const int e_min = -2 * N;
  extern __shared__ __align__(16) unsigned char smem[];
  unsigned long long* hist = reinterpret_cast<unsigned long long*>(smem);
  int* claim = reinterpret_cast<int*>(hist + L);
  int* found = claim + d.n_int;
  int* misc = found + d.n_int;  // [0] start energy
  int8_t* J = reinterpret_cast<int8_t*>(misc + 4);
  int8_t* lat = J + 2 * N;  // [walkers][N]

  const int tid = threadIdx.x;
  // disorder (wl.cu:364-386), or the caller's pattern, and the error chain
  // (wl.cu:388-428, prerun.cu:56-75)
  for (int q = tid; q < 2 * N; q += blockDim.x) {
    if (d.given_J) {
      J[q] = Jpool[d.off_J + q];
      continue;
    }
    Stream st;
    st.init(key_size(d.seed, static_cast<uint64_t>(d.sample)), 0, static_cast<uint64_t>(q));
    const double u = st.uniform();
    J[q] = (u < d.prob) ? -1 : 1;
  }
  for (int q = tid; q < L; q += blockDim.x) hist[q] = 0;
  for (int q = tid; q < d.n_int; q += blockDim.x) {
    claim[q] = INT_MAX;
    found[q] = 0;
  }
  __syncthreads();
  if (d.error_class == 'h' || d.error_class == 'c')
    for (int q = tid; q < Y; q += blockDim.x) J[N + q] = static_cast<int8_t>(-J[N + q]);
  if (d.error_class == 'v' || d.error_class == 'c')
    for (int q = tid; q < X; q += blockDim.x) J[q * Y] = static_cast<int8_t>(-J[q * Y]);
  // lattice (wl.cu:430-457, CAS winner fixed to site 0)
  const uint64_t key_l = key_u32(d.seed, static_cast<uint64_t>(d.sample));
  for (int q = tid; q < N; q += blockDim.x) {
    Stream st;
    st.init(key_l, 1, 0);
    const float p0 = st.uniform();
    st.init(key_l, 1, static_cast<uint64_t>(q) + 1);
    const double u = st.uniform();
    lat[q] = (u < p0) ? -1 : 1;
  }
  __syncthreads();
  for (int q = tid; q < 2 * N; q += blockDim.x) Jpool[d.off_J + q] = J[q];
  const int w = tid;
  const bool live = w < d.walkers;
  int8_t* s = lat + static_cast<size_t>(w) * N;
  if (live && w > 0)
    for (int q = 0; q < N; ++q) s[q] = lat[q];
  if (tid == 0) misc[0] = energy_i8(lat, J, X, Y, d.boundary);
  __syncthreads();

  // histogram-biased walk (wl.cu:473-560), round-synchronous
  Stream rng;
  int energy = misc[0];
  if (live) rng.init(key_u32(d.seed, static_cast<uint64_t>(d.sample)), 2 + static_cast<uint64_t>(w), 0);
  const double site_scale = (N - 1 + 0.999999);
  const uint32_t site_thr = static_cast<uint32_t>(N) * 2048u + 16384u;  // as MainDesc::site_thr
  // u < exp(H[old] - H[new]) (wl.cu:536-537) for an integer count difference
  // dd: always for dd >= 1 (exp(dd) > 1 >= u); never for dd <= -25
  // (exp(dd) < 2^-33 <= u); else x < acc_thr[-dd], the least draw whose
  // uniform reaches the device's exp(dd) (uniforms are monotone in the draw)
  __shared__ uint32_t acc_thr[25];
  if (tid < 25) {
    const double e = exp(static_cast<double>(-tid));
    unsigned long long lo = 0, hi = 1ull << 32;
    while (lo < hi) {
      const unsigned long long mid = (lo + hi) >> 1;
      if (static_cast<double>(unit_float(static_cast<uint32_t>(mid))) >= e) hi = mid;
      else lo = mid + 1;
    }
    acc_thr[tid] = static_cast<uint32_t>(lo);  // <= 2^32 - 128: u reaches 1 there
  }
  __syncthreads();
  bool ok = live;
  for (int it = 0; it < d.n_iter; ++it) {
    int hit = -1;
    bool acc = false;
    if (ok) {
      // site trunc(u (N - 1 + 0.999999)) (wl.cu:60-66): floor(x N / 2^32)
      // unless x N lies next to a multiple of 2^32 (see the main run)
      const uint32_t xs = rng.raw();
      const uint32_t lo_s = xs * static_cast<uint32_t>(N);
      int site = static_cast<int>(__umulhi(xs, static_cast<uint32_t>(N)));
      if (lo_s < site_thr || lo_s > ~site_thr) site = site_exact(xs, site_scale);  // out of line: FP64
      const Move m = move_i8(s, J, energy, X, Y, site, d.boundary, d.site_magic);
      const int io = energy - e_min;
      const int in = m.new_energy - e_min;
      const long long dd = static_cast<long long>(hist[io]) - static_cast<long long>(hist[in]);
      const uint32_t xa = rng.raw();
      const int ti = static_cast<int>(min(max(-dd, 0ll), 24ll));
      acc = dd >= 1 || (dd >= -24 && xa < acc_thr[ti]);
      if (acc) s[m.site] = static_cast<int8_t>(-s[m.site]);
      energy = acc ? m.new_energy : energy;
      hit = acc ? in : io;
    }
    __syncthreads();
    int bin = -1;
    {
      // warp-aggregated histogram update: walkers sit on few energies (all
      // start on one), so lanes with the same bin add their count once
      const unsigned on = __ballot_sync(0xFFFFFFFFu, hit >= 0);
      if (hit >= 0) {
        const unsigned same = __match_any_sync(on, hit);
        if (static_cast<int>(threadIdx.x & 31u) == __ffs(same) - 1)
          atomicAdd(&hist[hit], static_cast<unsigned long long>(__popc(same)));
      }
    }
    if (acc) {
      const int q = (energy - e_min) / d.len_int;
      bin = (q < d.n_int) ? q : d.n_int - 1;
      if (found[bin] == 0) atomicMin(&claim[bin], w);
      else bin = -1;
    }
    __syncthreads();
    if (bin >= 0 && claim[bin] == w && found[bin] == 0) {
      found[bin] = 1;
      int8_t* dst = found_pool + d.off_found + static_cast<long long>(bin) * N;
      for (int q = 0; q < N; ++q) dst[q] = s[q];
    }
  }
  __syncthreads();
  for (int q = tid; q < L; q += blockDim.x) seen_pool[d.off_seen + q] = hist[q] != 0 ? 1 : 0;
  // energies of the stored lattices (prerun.cu:123-133)
  for (int q = tid; q < d.n_int; q += blockDim.x) {
    fflag_pool[d.off_fflag + q] = found[q];
    int e = 0;
    if (found[q]) e = energy_i8(found_pool + d.off_found + static_cast<long long>(q) * N, J, X, Y, d.boundary);
    fflag_pool[d.off_fflag + d.n_int + q] = e;
  }
}

// ----------------------------------------------------------- main run -----

struct Team {
  int size;  // threads
  int id;    // barrier id (1..15) or 0 for a single warp
  __device__ __forceinline__ void sync() const
  {
    if (size == 32) {
      __syncwarp();
    } else {
      asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(size) : "memory");
    }
  }
};

// Site of a draw: trunc(double(u) * ((N-1) + 0.999999)) (wl.cu:63-65).  With
// f = x / 2^32 the reference's product lies within N*2^-23 + 1e-6 of f*N, so
// floor(f*N) = umulhi(x, N) is exact unless the fraction x*N mod 2^32 lies
// within site_thr (= 2^32 (N 2^-21 + 2^-18), >= 4x that bound) of an
// integer; there the reference's own float/double expression below decides.
// No int<->float conversion on the common path (they share GB300's slow
// FP64 pipe).  Out of line: inlined, its FP64 multiply and conversions would
// be scheduled into every step.
__device__ __noinline__ int site_exact(uint32_t x, double scale)
{
  return static_cast<int>(trunc(static_cast<double>(unit_float(x)) * scale));
}

// The reference's acceptance u < min(1, exp(g - g_new)) (wl.cu:1113-1116)
// in FP64, out of line (rare path; see site_exact).
__device__ __noinline__ bool accept_exact(uint32_t x2, double g, const double* g_new)
{
  return static_cast<double>(unit_float(x2)) < fmin(1.0, exp(g - *g_new));
}

struct Lat {
  uint64_t r;           // spins in a register (N <= 64)
  uint32_t* s;          // or shared-memory words, stride P
  int P;
};

template <bool kReg>
__device__ __forceinline__ uint32_t spin_bit(const Lat& l, int q)
{
  if constexpr (kReg) {
    return static_cast<uint32_t>(l.r >> q) & 1u;
  } else {
    return (l.s[(q >> 5) * l.P] >> (q & 31)) & 1u;
  }
}

template <bool kReg>
__device__ __forceinline__ void flip_spin(Lat& l, int q, bool doit)
{
  if constexpr (kReg) {
    l.r ^= static_cast<uint64_t>(doit) << q;
  } else {
    if (doit) l.s[(q >> 5) * l.P] ^= 1u << (q & 31);
  }
}

template <bool kReg>
__device__ __forceinline__ uint32_t bond_bit(uint64_t reg, const uint32_t* sm, int q)
{
  if constexpr (kReg) {
    return static_cast<uint32_t>(reg >> q) & 1u;
  } else {
    return (sm[q >> 5] >> (q & 31)) & 1u;
  }
}

struct Nbr {
  int up, dn, lf, rt, i, j;
};

__device__ __forceinline__ Nbr neighbours(int site, const MainDesc& d)
{
  Nbr n;
  n.i = static_cast<int>((static_cast<uint32_t>(site) * d.site_magic) >> 20);
  n.j = site - n.i * d.Y;
  n.up = (n.i == 0 ? d.X - 1 : n.i - 1) * d.Y + n.j;
  n.dn = (n.i == d.X - 1 ? 0 : n.i + 1) * d.Y + n.j;
  n.lf = n.i * d.Y + (n.j == 0 ? d.Y - 1 : n.j - 1);
  n.rt = n.i * d.Y + (n.j == d.Y - 1 ? 0 : n.j + 1);
  return n;
}

// Energy after flipping `site` (wl.cu:52-156 on bits: a neighbour term
// s_nb * J is -1 exactly when its spin bit and bond bit differ).
template <bool kReg>
__device__ __forceinline__ int energy_after_flip(const Lat& l, uint64_t JR, uint64_t JD, const uint32_t* Jr_s,
                                                 const uint32_t* Jd_s, int site, int E, const MainDesc& d)
{
  const Nbr n = neighbours(site, d);
  const int t_up = static_cast<int>(spin_bit<kReg>(l, n.up) ^ bond_bit<kReg>(JD, Jd_s, n.up));
  const int t_lf = static_cast<int>(spin_bit<kReg>(l, n.lf) ^ bond_bit<kReg>(JR, Jr_s, n.lf));
  const int t_dn = static_cast<int>(spin_bit<kReg>(l, n.dn) ^ bond_bit<kReg>(JD, Jd_s, site));
  const int t_rt = static_cast<int>(spin_bit<kReg>(l, n.rt) ^ bond_bit<kReg>(JR, Jr_s, site));
  int sigma;
  if (d.boundary == 0) {
    sigma = 4 - 2 * (t_up + t_lf + t_dn + t_rt);
  } else {
    sigma = (n.i > 0 ? 1 - 2 * t_up : 0) + (n.j > 0 ? 1 - 2 * t_lf : 0) + (n.i < d.X - 1 ? 1 - 2 * t_dn : 0) +
            (n.j < d.Y - 1 ? 1 - 2 * t_rt : 0);
  }
  const int s = 1 - 2 * static_cast<int>(spin_bit<kReg>(l, site));
  return E + 2 * s * sigma;
}

// Energy after flipping `site` on the row layout (lattice_rows), the same
// arithmetic as wl.cu:52-156: with r, ru, rd the rows of the site and of the
// rows above and below, a bond is unsatisfied (s_a s_b J = -1) exactly when
// the two spin bits and the coupling bit have odd parity, and flipping the
// site changes the energy by 2 (deg - 2 unsat) over its deg bonds.  Without
// a branch on the boundary: a horizontal bond belongs to the column on its
// left and is missing on an open lattice exactly when that is the last
// column (hedge clears its bit), a vertical bond is missing at the first or
// last row (wl.cu:134-137).  Also returns the offset of the site's row word
// and that word with the site flipped.
__device__ __forceinline__ int energy_after_flip_rows(const Lat& l, const uint32_t* Jr_s, const uint32_t* Jd_s,
                                                      int site, int E, const MainDesc& d, uint32_t hedge, bool open,
                                                      int& row_off, uint32_t& row_new)
{
  const int i = static_cast<int>((static_cast<uint32_t>(site) * d.site_magic) >> 20);
  const int j = site - i * d.Y;
  const int iu = i == 0 ? d.X - 1 : i - 1;
  const int id = i == d.X - 1 ? 0 : i + 1;
  row_off = i * l.P;
  const uint32_t r = l.s[row_off], ru = l.s[iu * l.P], rd = l.s[id * l.P];
  const uint32_t mj = 1u << j;
  const uint32_t mjl = j == 0 ? 1u << (d.Y - 1) : mj >> 1;
  const uint32_t rr = (r >> 1) | ((r & 1u) << (d.Y - 1));  // bit c: spin (i, c + 1 mod Y)
  const uint32_t h = r ^ rr ^ Jr_s[i];                     // bit c: bond (i, c)-(i, c + 1) unsatisfied
  const bool up = !open || i != 0, dn = !open || i != d.X - 1;
  const uint32_t vu = up ? (r ^ ru ^ Jd_s[iu]) & mj : 0u;  // bond (i - 1, j)-(i, j) unsatisfied
  const uint32_t vd = dn ? (r ^ rd ^ Jd_s[i]) & mj : 0u;   // bond (i, j)-(i + 1, j) unsatisfied
  const uint32_t hm = (mj | mjl) & hedge;
  row_new = r ^ mj;
  const int unsat = __popc(h & hm) + __popc(vu) + __popc(vd);
  const int deg = __popc(hm) + (up ? 1 : 0) + (dn ? 1 : 0);
  return E + 2 * (deg - 2 * unsat);
}

__device__ __forceinline__ bool mask_has(const uint32_t* mask, int c) { return (mask[c >> 5] >> (c & 31)) & 1u; }

// Draws q and q + 1 of the words of A then B (q in [0, 3]); the three
// compares serve both picks.
__device__ __forceinline__ void pick_pair(const uint4& A, const uint4& B, int q, uint32_t& x1, uint32_t& x2)
{
  const bool q1 = q == 1, q2 = q == 2, q3 = q == 3;
  x1 = q3 ? A.w : (q2 ? A.z : (q1 ? A.y : A.x));
  x2 = q3 ? B.x : (q2 ? A.w : (q1 ? A.z : A.y));
}

__device__ __forceinline__ long long device_clock_ns()
{
  long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

template <bool kReg, bool kTable, bool kGlobalG, bool kRows>
__device__ void run_problem(const MainDesc& d, int p, const Team& team, int t, unsigned char* base, double* gslot,
                            const uint32_t* __restrict__ Jpool, const uint32_t* __restrict__ latpool,
                            const int* __restrict__ winpool, const uint32_t* __restrict__ maskpool,
                            double* __restrict__ outpool, MainResult* __restrict__ results,
                            unsigned char* __restrict__ statepool)
{
  const int P = team.size;
  // start time straight into the result slot: a value kept live through the
  // sweep costs the step registers (measured 3 % on one-warp teams)
  if (t == 0) results[p].t_start = device_clock_ns();
  // resumable run: state saved at the end of a launch, restored at the start
  unsigned char* const st = d.off_state >= 0 ? statepool + d.off_state : nullptr;
  const StateLayout sl = state_layout(P, d.I, d.nwL, d.L);
  const TeamLayout lay = team_layout(P, d.L, d.nwL, d.nwM, d.I, kReg ? 2 : d.nwL, kTable ? d.N : 0, !kGlobalG);
  // FP64 log g: in the team's shared memory, or (large problems) in this
  // resident team's slice of a global pool, L2-resident and touched only on
  // bin changes, averaging and exchange
  double* G = kGlobalG ? (st != nullptr ? reinterpret_cast<double*>(st + sl.off_G) : gslot)
                       : reinterpret_cast<double*>(base + lay.off_G);
  float* Gf = reinterpret_cast<float*>(base + lay.off_Gf);
  uint32_t* H = reinterpret_cast<uint32_t*>(base + lay.off_H);
  uint32_t* lat_s = reinterpret_cast<uint32_t*>(base + lay.off_lat);
  int* E_s = reinterpret_cast<int*>(base + lay.off_E);
  int* perm = reinterpret_cast<int*>(base + lay.off_perm);
  uint32_t* mask = reinterpret_cast<uint32_t*>(base + lay.off_mask);
  uint32_t* Js = reinterpret_cast<uint32_t*>(base + lay.off_J);
  ulonglong2* nbt = reinterpret_cast<ulonglong2*>(base + lay.off_nbt);
  double* fwin = reinterpret_cast<double*>(base + lay.off_f);
  double* lnfw = fwin + d.I;  // log(f) of each window, recomputed only when f changes
  int* cond = reinterpret_cast<int*>(base + lay.off_cond);
  int* flat = reinterpret_cast<int*>(base + lay.off_flat);
  // A finished window (cond stays 1) is frozen: its walkers no longer change
  // log g, so once an averaging pass leaves every value as it was, every
  // later pass would too; such windows are skipped (stab).  Not saved with a
  // suspended run: a resumed one recomputes one pass, with the same result.
  int* stab = reinterpret_cast<int*>(base + lay.off_stab);
  int* chg = stab + d.I;
  int* win = reinterpret_cast<int*>(base + lay.off_win);  // start, end, base, Lb, E0
  int* misc = reinterpret_cast<int*>(base + lay.off_misc);
  const int I = d.I, W = d.W;
  int* w_start = win;
  int* w_end = win + I;
  int* w_base = win + 2 * I;
  int* w_len = win + 3 * I;

  // ---- load the problem
  for (int q = t; q < d.nwM; q += P) mask[q] = maskpool[d.off_mask + q];
  for (int q = t; q < 2 * d.nwL; q += P) Js[q] = Jpool[d.off_J + q];
  for (int q = t; q < 5 * I; q += P) win[q] = winpool[d.off_win + q];
  for (int q = t; q < I; q += P) {
    fwin[q] = kE;
    lnfw[q] = log(kE);
    cond[q] = 0;
    flat[q] = 0;
    stab[q] = 0;
    chg[q] = 0;
  }
  const bool resumed = st != nullptr && reinterpret_cast<const int*>(st)[4] != 0;
  for (int c = 0; c < d.L; ++c) {
    if (!resumed || !kGlobalG) G[c * P + t] = 0.0;
    Gf[c * P + t] = 0.0f;
    H[c * P + t] = 0u;
  }
  if (t < 8) misc[t] = 0;
  const bool live = t < d.nwalk;
  const int b = live ? t / W : 0;
  const int w = t - b * W;
  perm[t] = w;
  team.sync();

  uint64_t JR = 0, JD = 0;
  if constexpr (kReg) {
    JR = Js[0] | (d.nwL > 1 ? static_cast<uint64_t>(Js[1]) << 32 : 0ull);
    JD = Js[d.nwL] | (d.nwL > 1 ? static_cast<uint64_t>(Js[d.nwL + 1]) << 32 : 0ull);
  }
  const uint32_t* Jr_s = Js;
  const uint32_t* Jd_s = Js + d.nwL;
  if constexpr (kTable) {
    // neighbour table: bits of the neighbours of each site, and of those
    // whose connecting bond is -1 (X, Y >= 3, so the 4 neighbours differ)
    for (int site = t; site < d.N; site += P) {
      const Nbr n = neighbours(site, d);
      uint64_t m = 0, bnd = 0;
      const bool has_up = d.boundary == 0 || n.i > 0, has_dn = d.boundary == 0 || n.i < d.X - 1;
      const bool has_lf = d.boundary == 0 || n.j > 0, has_rt = d.boundary == 0 || n.j < d.Y - 1;
      if (has_up) {
        m |= 1ull << n.up;
        bnd |= static_cast<uint64_t>((JD >> n.up) & 1ull) << n.up;
      }
      if (has_lf) {
        m |= 1ull << n.lf;
        bnd |= static_cast<uint64_t>((JR >> n.lf) & 1ull) << n.lf;
      }
      if (has_dn) {
        m |= 1ull << n.dn;
        bnd |= static_cast<uint64_t>((JD >> site) & 1ull) << n.dn;
      }
      if (has_rt) {
        m |= 1ull << n.rt;
        bnd |= static_cast<uint64_t>((JR >> site) & 1ull) << n.rt;
      }
      nbt[site] = make_ulonglong2(m, bnd);
    }
  }
  Lat lt;
  lt.P = P;
  lt.s = lat_s + t;
  lt.r = 0;
  if (live) {
    const uint32_t* src = latpool + d.off_lat + static_cast<long long>(b) * d.nwL;
    if constexpr (kReg) {
      lt.r = src[0] | (d.nwL > 1 ? static_cast<uint64_t>(src[1]) << 32 : 0ull);
    } else {
      for (int q = 0; q < d.nwL; ++q) lat_s[q * P + t] = src[q];
    }
  }
  int E = live ? win[4 * I + b] : 0;
  Stream rng;
  rng.init(d.key_wl, static_cast<uint64_t>(t), 0);
  const bool keys_differ = d.key_ex != static_cast<uint64_t>(d.key_wl);
  const double reset_lim = exp(d.beta);  // wl.cu:609
  const int lo = live ? w_start[b] : 0, hi = live ? w_end[b] : 0, bb = live ? w_base[b] : 0;
  const int step_mask = (1 << d.lg) - 1;
  const int span = d.e_max - d.e_min;
  // row layout: open lattices have no bond right of the last column
  const bool open_bc = d.boundary != 0;
  const uint32_t hedge = open_bc ? ~(1u << (d.Y - 1)) : 0xFFFFFFFFu;
  const int Lm1 = d.L - 1;

  long long outer = 0;
  long long counter = 1;
  int status = WLG_OK;
  if (resumed) {
    const long long* hdr = reinterpret_cast<const long long*>(st);
    outer = hdr[0];
    counter = hdr[1];
    if (t < I) {
      fwin[t] = reinterpret_cast<const double*>(st + sl.off_f)[t];
      lnfw[t] = log(fwin[t]);
      cond[t] = reinterpret_cast<const int*>(st + sl.off_cond)[t];
    }
    perm[t] = reinterpret_cast<const int*>(st + sl.off_perm)[t];
    if (live) {
      E = reinterpret_cast<const int*>(st + sl.off_E)[t];
      rng.init(d.key_wl, static_cast<uint64_t>(t), reinterpret_cast<const unsigned long long*>(st + sl.off_pos)[t]);
      const uint32_t* ls = reinterpret_cast<const uint32_t*>(st + sl.off_lat);
      if constexpr (kReg) {
        lt.r = ls[t] | (d.nwL > 1 ? static_cast<uint64_t>(ls[P + t]) << 32 : 0ull);
      } else {
        for (int q = 0; q < d.nwL; ++q) lat_s[q * P + t] = ls[q * P + t];
      }
    }
    const uint32_t* hs = reinterpret_cast<const uint32_t*>(st + sl.off_H);
    const double* gs = reinterpret_cast<const double*>(st + sl.off_G);
    for (int c = 0; c < d.L; ++c) {
      H[c * P + t] = hs[c * P + t];
      if constexpr (!kGlobalG) G[c * P + t] = gs[c * P + t];
    }
  }
  int launch_outer = 0;  // outer iterations of this launch
  bool suspended = false;
  team.sync();

  for (;;) {
    if (d.max_outer > 0 && outer >= d.max_outer) {
      status = WLG_ERR_TIMEOUT;
      break;
    }
    // ---- WL sweep (wl.cu:1077-1175).  The step body has no divergent
    // branch: every state update is predicated on `commit`.  The two FP64
    // decisions of the reference that FP32 cannot always settle (a site pick
    // next to a cell boundary, an acceptance inside the FP32 error band) are
    // made for the few lanes that need them in a warp-uniform block at the
    // end of the body, after which those lanes replay the same step (same
    // draws) with the exact answer.  Each lane counts its own steps; the warp
    // loops until all of its live lanes are done.  The acceptance draw is
    // peeked and consumed only for in-window proposals, and the Philox block
    // after next is computed speculatively every step.
    const unsigned wmask = __ballot_sync(0xFFFFFFFFu, live);
    if (live) {
      const bool frozen = cond[b] != 0;
      const double lnf = lnfw[b];  // log(f) (wl.cu:1124)
      const float lnf_f = static_cast<float>(lnf);
      int c_cur = (E - bb) >> d.lg;
      double g_cur = G[c_cur * P + t];
      // float shadows of this walker's log g relative to gbase: differences
      // inside a window stay small while absolute values reach 1e4, so the
      // relative shadow keeps the FP32 error bound (and the FP64 fallback
      // rate) small
      const double gbase = g_cur;
      const Split gbase_split = split_float(gbase);
      for (int c = 0; c < d.L; ++c) Gf[c * P + t] = shadow_split(G[c * P + t], gbase_split);
      // one rounding of a double of size |g| <= |gbase| + (small shadow terms)
      const float ulp_g = static_cast<float>((fabs(gbase) + 1.0) * 0x1p-51);
      float gfb = 0.0f;               // float of g_cur - gbase at the last change of bin
      uint32_t h_cur = H[c_cur * P + t];
      float kf = 0.0f;                // ln f increments since then (exact below 2^24)
      // ln f owed to g_cur by the previous step (wl.cu:1124), added one step
      // late so the FP64 addition overlaps the next step's decision instead
      // of waiting on a shared-memory load; same additions, same order
      double owed = 0.0;
      // Draws: A and B hold the outputs of counters blk and blk + 1; C is
      // Philox of counter blk + 2, advanced five rounds per step (phase
      // 0, 1: rounds done 0, 5; 2: complete).  A step consumes at most two
      // draws, so after C is restarted two steps pass before B runs out
      // and C, complete by then, replaces it.
      const uint64_t pos = rng.pos;
      const uint64_t blk = pos >> 2;
      uint4 A = philox10(static_cast<uint32_t>(blk), static_cast<uint32_t>(blk >> 32), rng.s0, rng.s1, rng.k0, rng.k1);
      uint4 B = philox10(static_cast<uint32_t>(blk + 1), static_cast<uint32_t>((blk + 1) >> 32), rng.s0, rng.s1,
                         rng.k0, rng.k1);
      uint4 Cb = philox10(static_cast<uint32_t>(blk + 2), static_cast<uint32_t>((blk + 2) >> 32), rng.s0, rng.s1,
                          rng.k0, rng.k1);
      int phase = 2;
      const uint32_t k5a = rng.k0 + 5u * kPhiloxWeylA, k5b = rng.k1 + 5u * kPhiloxWeylB;  // key of round 5
      const uint32_t nN = static_cast<uint32_t>(d.N);
      int it = 0;
      bool stopped = false;
      int ovr_site = -1;  // exact site of the step being replayed
      int ovr_acc = -1;   // exact acceptance of the step being replayed
      int q = static_cast<int>(pos - (blk << 2));  // draw offset in block A, 0..3
      uint64_t nc = blk + 2;                        // counter of the block being built in C
      // For the first n_iter warp iterations no live lane has finished (a
      // lane finishes after n_iter committed steps), so the warp votes on
      // continuing only after that, when lanes that replayed catch up.
      for (int k = 0;; ++k) {
        const bool act = it < d.n_iter && !stopped;
        if (k >= d.n_iter && !__any_sync(wmask, act)) break;
        {
          const uint4 half = philox_rounds<5>(Cb, phase == 0 ? rng.k0 : k5a, phase == 0 ? rng.k1 : k5b);
          Cb = phase < 2 ? half : Cb;
          phase = min(phase + 1, 2);
        }
        uint32_t x1, x2;
        pick_pair(A, B, q, x1, x2);
        const float lu = log_uniform(x2);  // depends on the draw only: off the serial path
        // site trunc(u (N - 1 + 0.999999)) (wl.cu:60-66) as floor(x N / 2^32)
        // unless x N lies within site_thr of a multiple of 2^32
        const uint32_t lo_s = x1 * nN;
        const bool need_site = act && ovr_site < 0 && (lo_s < d.site_thr || lo_s > ~d.site_thr);
        const int site = ovr_site >= 0 ? ovr_site : static_cast<int>(__umulhi(x1, nN));
        int En;
        int row_off = 0;       // row layout: offset of the site's row word,
        uint32_t row_new = 0;  // and that word with the site flipped
        if constexpr (kTable) {
          const ulonglong2 nt = nbt[site];
          const int unsat = __popcll((lt.r ^ nt.y) & nt.x);
          const int deg = __popcll(nt.x);
          const int sb = static_cast<int>((lt.r >> site) & 1ull);
          En = E + 2 * (1 - 2 * sb) * (deg - 2 * unsat);
        } else if constexpr (kRows) {
          En = energy_after_flip_rows(lt, Jr_s, Jd_s, site, E, d, hedge, open_bc, row_off, row_new);
        } else {
          En = energy_after_flip<kReg>(lt, JR, JD, Jr_s, Jd_s, site, E, d);
        }
        const int rel = En - d.e_min;
        const int relc = min(max(rel, 0), span);
        const bool bad = rel != relc || (rel & step_mask) != 0 || !mask_has(mask, relc >> d.lg);
        const bool inside = En >= lo && En <= hi;
        const int c_new = min(max((En - bb) >> d.lg, 0), Lm1);
        const bool same = c_new == c_cur;
        const float gfn = Gf[c_new * P + t];
        const uint32_t h_new = H[c_new * P + t];
        const double g_new = kGlobalG ? 0.0 : G[c_new * P + t];
        // u < min(1, exp(g_cur - g_new)) (wl.cu:1113-1116) decided from FP32
        // values with a proven error bound eps on the exponent; the
        // reference's FP64 expression decides whenever the bound does not.
        const float kl = kf * lnf_f;
        const float df = (gfb - gfn) + kl;
        // |df - (g_cur - g_new)|: the shadows' relative errors (<= 2^-23)
        // and the float roundings of kl and df (2^-22 = 2x and 4x them); the k
        // sequential double additions in g_cur and the double differences,
        // each <= one rounding at |g| (k + 4 ulp_g); the shadows' absolute
        // error 2^-44 (g + gbase) each (<= 512 ulp_g for both)
        const float eps_b = fmaf(0x1p-22f, fabsf(gfb) + kl, (kf + 516.0f) * ulp_g);  // before the load of gfn
        const float eps = fmaf(0x1p-22f, fabsf(gfn) + fabsf(df), eps_b);
        const Decision dec = decide(x2, lu, df, eps, same);
        const bool fast_acc = dec.acc;
        const bool known = dec.known;
        const bool need_acc = act && !need_site && !bad && inside && ovr_acc < 0 && !known;
        g_cur += owed;  // g >= +0, so adding +0 (frozen, first step) is exact
        owed = 0.0;
        const bool stop_now = act && !need_site && bad;  // wl.cu:1091-1104: a new energy stops the problem
        if (stop_now) {
          misc[1] = 1;
          misc[2] = En;
        }
        const bool commit = act && !need_site && !need_acc && !bad;
        const bool acc = commit && inside && (ovr_acc >= 0 ? ovr_acc != 0 : fast_acc);
        if constexpr (kRows) {
          if (acc) lt.s[row_off] = row_new;
        } else {
          flip_spin<kReg>(lt, site, acc);
        }
        E = acc ? En : E;
        // leaving c_cur: write back its log g, shadow and visit count
        const bool chg = acc && !same;
        const float sh = shadow_split(g_cur, gbase_split);
        if (chg && !frozen) {
          G[c_cur * P + t] = g_cur;
          Gf[c_cur * P + t] = sh;
          H[c_cur * P + t] = h_cur;
        }
        if constexpr (kGlobalG) {
          if (chg) g_cur = G[c_new * P + t];
        } else {
          g_cur = chg ? g_new : g_cur;
        }
        h_cur = chg ? h_new : h_cur;
        gfb = chg ? gfn : gfb;
        kf = chg ? 0.0f : kf;
        c_cur = chg ? c_new : c_cur;
        const bool upd = commit && !frozen;
        owed = upd ? lnf : 0.0;
        h_cur += upd ? 1u : 0u;
        kf += upd ? 1.0f : 0.0f;
        const int used = commit ? (inside ? 2 : 1) : (stop_now ? 1 : 0);  // draws consumed
        q += used;
        it += commit ? 1 : 0;
        stopped = stopped || stop_now;
        ovr_site = commit || stop_now ? -1 : ovr_site;
        ovr_acc = commit || stop_now ? -1 : ovr_acc;
        const bool adv = q >= 4;
        q = adv ? q - 4 : q;
        A = adv ? B : A;
        B = adv ? Cb : B;
        nc += adv ? 1u : 0u;  // restart C on the counter after the new B
        Cb = adv ? make_uint4(static_cast<uint32_t>(nc), static_cast<uint32_t>(nc >> 32), rng.s0, rng.s1) : Cb;
        phase = adv ? 0 : phase;
        if (__any_sync(wmask, need_site || need_acc)) {  // rare
          if (need_site) ovr_site = site_exact(x1, d.site_scale);
          if (need_acc) ovr_acc = accept_exact(x2, g_cur, G + c_new * P + t) ? 1 : 0;
        }
      }
      g_cur += owed;
      if (!frozen) {
        G[c_cur * P + t] = g_cur;
        H[c_cur * P + t] = h_cur;
      }
      rng.pos = ((nc - 2) << 2) + static_cast<uint64_t>(q);  // draws consumed: block A's offset plus q
      rng.refill();
    }
    team.sync();
    ++outer;
    if (misc[1] != 0) {
      status = WLG_ERR_NEW_ENERGY;
      break;
    }
    // ---- flatness (wl.cu:892-967)
    if (live && cond[b] == 0) {
      const int cb = (bb - d.e_min) >> d.lg;
      uint32_t mn = 2147483647u;
      unsigned long long sum = 0;
      int cnt = 0;
      for (int c = 0; c < w_len[b]; ++c) {
        if (!mask_has(mask, cb + c)) continue;
        const uint32_t v = H[c * P + t];
        mn = v < mn ? v : mn;
        sum += v;
        ++cnt;
      }
      if (cnt > 0 && static_cast<double>(mn) >= d.alpha * (static_cast<double>(sum) / cnt)) atomicAdd(&flat[b], 1);
    }
    team.sync();
    if (live && cond[b] == 0 && flat[b] == W) {
      for (int c = 0; c < d.L; ++c) H[c * P + t] = 0u;
    }
    team.sync();
    if (t < I && cond[t] == 0 && flat[t] == W) {
      fwin[t] = sqrt(fwin[t]);
      lnfw[t] = log(fwin[t]);
      cond[t] = 1;
    }
    team.sync();
    // ---- window averages (wl.cu:710-783 + :969-1031)
    for (int q = t; q < I * d.L; q += P) {
      const int wb = q / d.L;
      const int c = q - wb * d.L;
      if (cond[wb] != 1 || stab[wb] != 0 || c >= w_len[wb]) continue;
      double avg = 0.0;
      if (mask_has(mask, ((w_base[wb] - d.e_min) >> d.lg) + c)) {
        for (int v = 0; v < W; ++v) avg += G[c * P + wb * W + v] / W;
      }
      bool same = true;
      for (int v = 0; v < W; ++v) {
        same = same && __double_as_longlong(G[c * P + wb * W + v]) == __double_as_longlong(avg);
        G[c * P + wb * W + v] = avg;
      }
      if (!same) chg[wb] = 1;
    }
    team.sync();
    // ---- reset and convergence (wl.cu:596-613, :662-708, mainrun.cu:243, :342-344)
    if (t < I) {
      if (cond[t] == 1 && fwin[t] > reset_lim) cond[t] = 0;
      stab[t] = cond[t] == 1 && (stab[t] != 0 || chg[t] == 0) ? 1 : 0;
      chg[t] = 0;
      flat[t] = 0;
    }
    team.sync();
    bool done = true;
    double fmax = 0.0;
    for (int q = 0; q < I; ++q) {
      done = done && cond[q] == 1;
      fmax = fmax > fwin[q] ? fmax : fwin[q];
    }
    const bool stop = !(fmax - d.loop_lim > 1e-10);
    // ---- replica exchange (wl.cu:785-890)
    if (!done && counter % d.exch_every == 0) {
      if (live) {
        E_s[t] = E;
        if constexpr (kReg) {
          lat_s[t] = static_cast<uint32_t>(lt.r);
          lat_s[P + t] = static_cast<uint32_t>(lt.r >> 32);
        }
        if (keys_differ) rng.init(d.key_ex, static_cast<uint64_t>(t), rng.pos);
      }
      const int nw = kReg ? 2 : d.nwL;
      for (int pass = 0; pass < 2; ++pass) {
        const int even = pass == 0;
        team.sync();
        const int par = (b + d.parity_base) & 1;
        const bool active = live && b < I - 1 && ((even && par == 0) || (!even && par == 1));
        if (active && w == 0) {  // Fisher-Yates by the window's first walker
          for (int i = W - 1; i > 0; --i) {
            double u = rng.uniform();
            u *= (i + 0.999999);
            const int r = static_cast<int>(trunc(u));
            const int tmp = perm[t + i];
            perm[t + i] = perm[t + r];
            perm[t + r] = tmp;
          }
        }
        team.sync();
        if (active) {
          const int o = (b + 1) * W + perm[t];
          const int et = E_s[t], eo = E_s[o];
          if (et >= w_start[b + 1] && et <= w_end[b + 1] && eo >= w_start[b] && eo <= w_end[b]) {
            const int nb = w_base[b + 1];
            const double gi_x = G[((et - bb) >> d.lg) * P + t];
            const double gi_y = G[((eo - bb) >> d.lg) * P + t];
            const double gj_y = G[((eo - nb) >> d.lg) * P + o];
            const double gj_x = G[((et - nb) >> d.lg) * P + o];
            const double prob = fmin(1.0, exp(gi_x - gi_y) * exp(gj_y - gj_x));
            if (rng.uniform() < prob) {
              E_s[t] = eo;
              E_s[o] = et;
              for (int q = 0; q < nw; ++q) {
                const uint32_t a = lat_s[q * P + t];
                lat_s[q * P + t] = lat_s[q * P + o];
                lat_s[q * P + o] = a;
              }
            }
          }
        }
      }
      team.sync();
      if (live) {
        E = E_s[t];
        if constexpr (kReg) lt.r = lat_s[t] | static_cast<uint64_t>(lat_s[P + t]) << 32;
        if (keys_differ) rng.init(d.key_wl, static_cast<uint64_t>(t), rng.pos);
      }
    }
    if (d.exch_mode == 1) ++counter;
    team.sync();
    if (stop) break;
    if (st != nullptr && d.epoch_outer > 0 && ++launch_outer >= d.epoch_outer) {
      suspended = true;
      break;
    }
  }

  if (suspended) {  // save the state; the next launch resumes from it
    if (t == 0) {
      long long* hdr = reinterpret_cast<long long*>(st);
      hdr[0] = outer;
      hdr[1] = counter;
      reinterpret_cast<int*>(st)[4] = 1;
    }
    if (t < I) {
      reinterpret_cast<double*>(st + sl.off_f)[t] = fwin[t];
      reinterpret_cast<int*>(st + sl.off_cond)[t] = cond[t];
    }
    reinterpret_cast<int*>(st + sl.off_perm)[t] = perm[t];
    if (live) {
      reinterpret_cast<int*>(st + sl.off_E)[t] = E;
      reinterpret_cast<unsigned long long*>(st + sl.off_pos)[t] = rng.pos;
      uint32_t* ls = reinterpret_cast<uint32_t*>(st + sl.off_lat);
      for (int q = 0; q < d.nwL; ++q) {
        if constexpr (kReg) {
          ls[q * P + t] = static_cast<uint32_t>(lt.r >> (32 * q));
        } else {
          ls[q * P + t] = lat_s[q * P + t];
        }
      }
    }
    uint32_t* hs = reinterpret_cast<uint32_t*>(st + sl.off_H);
    double* gs = reinterpret_cast<double*>(st + sl.off_G);
    for (int c = 0; c < d.L; ++c) {
      hs[c * P + t] = H[c * P + t];
      if constexpr (!kGlobalG) gs[c * P + t] = G[c * P + t];
    }
    if (t == 0) {
      MainResult r{};
      r.status = WLG_OK;
      r.outer = outer;
      r.flips = outer * static_cast<long long>(d.nwalk) * d.n_iter;
      r.done = 0;
      r.t_start = results[p].t_start;
      r.t_end = device_clock_ns();
      results[p] = r;
    }
    team.sync();
    return;
  }

  // ---- results
  if (live && w == 0) {
    for (int c = 0; c < d.L; ++c) outpool[d.off_out + static_cast<long long>(b) * d.L + c] = G[c * P + t];
  }
  if (t == 0) {
    MainResult r{};
    r.status = status;
    r.new_energy = misc[2];
    r.outer = outer;
    r.flips = outer * static_cast<long long>(d.nwalk) * d.n_iter;
    r.done = 1;
    r.t_start = results[p].t_start;
    r.t_end = device_clock_ns();
    results[p] = r;
  }
  team.sync();
}

template <bool kReg, bool kTable, bool kGlobalG, bool kRows, int kMaxThreads>
__global__ void __launch_bounds__(kMaxThreads) k_main_batch(const MainDesc* __restrict__ descs, const int* __restrict__ order,
                                                     int n, int team_size, int team_bytes, int* __restrict__ next,
                                                     double* __restrict__ gpool, long long gslot_doubles,
                                                     const uint32_t* __restrict__ Jpool,
                                                     const uint32_t* __restrict__ latpool,
                                                     const int* __restrict__ winpool,
                                                     const uint32_t* __restrict__ maskpool,
                                                     double* __restrict__ outpool, MainResult* __restrict__ results,
                                                     unsigned char* __restrict__ statepool)
{
  extern __shared__ __align__(16) unsigned char smem[];
  const int tix = threadIdx.x / team_size;
  Team team{team_size, team_size == 32 ? 0 : 1 + tix};
  const int t = threadIdx.x - tix * team_size;
  unsigned char* base = smem + static_cast<size_t>(tix) * team_bytes;
  int* slot = reinterpret_cast<int*>(base + team_bytes - 16);
  for (;;) {
    if (t == 0) *slot = atomicAdd(next, 1);
    team.sync();
    const int q = *slot;
    team.sync();
    if (q >= n) return;
    const int p = order[q];
    const MainDesc d = descs[p];
    if (d.off_state >= 0 && results[p].done != 0) continue;  // resumable run that finished in an earlier launch
    double* gslot = kGlobalG ? gpool + (static_cast<long long>(blockIdx.x) * (blockDim.x / team_size) + tix) * gslot_doubles
                             : nullptr;
    run_problem<kReg, kTable, kGlobalG, kRows>(d, p, team, t, base, gslot, Jpool, latpool, winpool, maskpool, outpool,
                                               results, statepool);
  }
}

}  // namespace

// ------------------------------------------------------------ launchers ----

wlg_status launch_pre_batch(const PreDesc* d_descs, int n, int threads, int smem, int8_t* Jpool, uint8_t* seen_pool,
                            int8_t* found_pool, int* fflag_pool, cudaStream_t s)
{
  if (n == 0) return WLG_OK;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(k_pre_batch, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return WLG_ERR_CUDA;
  }
  k_pre_batch<<<n, threads, smem, s>>>(d_descs, n, Jpool, seen_pool, found_pool, fflag_pool);
  return launch_status();
}

using MainFn = void (*)(const MainDesc*, const int*, int, int, int, int*, double*, long long, const uint32_t*,
                        const uint32_t*, const int*, const uint32_t*, double*, MainResult*, unsigned char*);

// variant (kernel_variant): form 0 = spins and log g in shared memory,
// 1 = spins in a register, 2 = register spins + neighbour table, 3 = spins
// in shared memory, FP64 log g in a global pool (problems too large for one
// SM's shared memory); plus kKernelRows (4) for lattices one row per word
// (forms 0 and 3)
template <int kMaxThreads>
MainFn main_fn_for(int variant)
{
  switch (variant) {
    case 1: return &k_main_batch<true, false, false, false, kMaxThreads>;
    case 2: return &k_main_batch<true, true, false, false, kMaxThreads>;
    case 3: return &k_main_batch<false, false, true, false, kMaxThreads>;
    case 0 | kKernelRows: return &k_main_batch<false, false, false, true, kMaxThreads>;
    case 3 | kKernelRows: return &k_main_batch<false, false, true, true, kMaxThreads>;
    default: return &k_main_batch<false, false, false, false, kMaxThreads>;
  }
}

MainFn main_fn(int variant, int cta_threads)
{
  if (cta_threads <= 256) return main_fn_for<256>(variant);
  if (cta_threads <= 512) return main_fn_for<512>(variant);
  return main_fn_for<1024>(variant);
}

// Returns the number of resident CTAs the launch may use (0 if the
// configuration does not fit).
int main_batch_capacity(int variant, int cta_threads, int smem)
{
  MainFn fn = main_fn(variant, cta_threads);
  int per_sm = 0;
  if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess) return 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, cta_threads, smem) != cudaSuccess) return 0;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return per_sm * sms;
}

wlg_status launch_main_batch(int variant, const MainDesc* d_descs, const int* d_order, int n, int team_size,
                             int team_bytes, int teams_per_cta, int grid, int* d_next, double* gpool,
                             long long gslot_doubles, const uint32_t* Jpool,
                             const uint32_t* latpool, const int* winpool, const uint32_t* maskpool, double* outpool,
                             MainResult* results, unsigned char* statepool, cudaStream_t s)
{
  if (n == 0) return WLG_OK;
  const int threads = team_size * teams_per_cta;
  const int smem = team_bytes * teams_per_cta;
  MainFn fn = main_fn(variant, threads);
  if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess) return WLG_ERR_CUDA;
  fn<<<grid, threads, smem, s>>>(d_descs, d_order, n, team_size, team_bytes, d_next, gpool, gslot_doubles, Jpool,
                                 latpool, winpool, maskpool, outpool, results, statepool);
  return launch_status();
}

}  // namespace wlg
