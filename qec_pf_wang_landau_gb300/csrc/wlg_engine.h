// Batched engine: descriptors shared by the device kernels (wlg_engine.cu)
// and the host pipeline (wlg_engine_host.cpp).  Not part of the C ABI.
//
// A "problem" is one disorder sample of one error class: the reference runs
// R of them per invocation of prerun/mainrun, keyed by `seed + sample`.  The
// engine runs thousands of heterogeneous problems per launch.
#pragma once

#include <cstdint>

#if defined(__CUDACC__)
#define WLG_HD __host__ __device__
#else
#define WLG_HD
#endif

namespace wlg {

// ------------------------------------------------------------ pre-run -----
// One CTA per problem: disorder, error chain, lattice init, energy,
// histogram-biased walk, stored lattices and their energies, fused.
struct PreDesc {
  int X, Y, N, boundary;
  float prob;
  int error_class;  // 'i', 'h', 'v', 'c'
  int seed, sample;
  int walkers;      // <= 1024
  int n_int;        // coarse bins for stored lattices
  int len_int;      // coarse bin width (interval.cpp with overlap 1)
  int n_iter;
  int given_J;          // 1: the class-'i' couplings are read from off_J instead of drawn
  uint32_t site_magic;  // ceil(2^20 / Y) when it divides every site exactly, else 0
  long long off_J;      // int8 [2N]
  long long off_seen;   // uint8 [4N+1]
  long long off_found;  // int8 [n_int][N]
  long long off_fflag;  // int [n_int] flags, then int [n_int] energies
  int smem;             // dynamic shared memory of the CTA
};

// ----------------------------------------------------------- main run -----
// Bit-packed lattices and couplings.  Lattices of more than 64 sites whose
// rows fit a 32-bit word (2 <= Y <= 32) are kept one row per word: bit j of
// word i is site (i, j), so a site's four neighbours lie in three words
// (its row and the rows above and below).  Others are packed linearly: bit
// q & 31 of word q >> 5 is site q = i*Y + j.  A set bit is a -1 spin or a
// -1 coupling; right bonds (site, site + 1 in the row) and down bonds (site,
// site + Y) are packed the same way as the sites that own them.
WLG_HD inline bool lattice_rows(int X, int Y) { return X * Y > 64 && Y >= 2 && Y <= 32; }
// bit of a main-run kernel variant (kernel_variant) for the row layout
constexpr int kKernelRows = 4;
WLG_HD inline int lattice_words(int X, int Y) { return lattice_rows(X, Y) ? X : (X * Y + 31) / 32; }
// word and bit of site q (q = i*Y + j)
WLG_HD inline void lattice_bit(int X, int Y, int q, int& word, int& bit)
{
  if (lattice_rows(X, Y)) {
    word = q / Y;
    bit = q - word * Y;
  } else {
    word = q >> 5;
    bit = q & 31;
  }
}

// One team of threads per problem (one thread per walker, team size a
// multiple of 32).  Walker state lives in registers and the team's shared
// memory for the whole run.
struct MainDesc {
  int X, Y, N, boundary;
  int I, W, nwalk, team;
  int e_min, e_max, lg;   // spectrum range and log2 of the energy step
  int L;                  // compact bins per walker (max over windows)
  int n_iter, exch_every, exch_mode, parity_base;
  double alpha, beta, loop_lim;  // loop_lim: exp(beta) as the host computes it
  uint32_t key_wl;               // Philox key of the WL sweeps (wl.cu:1074)
  uint64_t key_ex;               // Philox key of the exchange (wl.cu:796, :875)
  uint32_t site_magic;           // ceil(2^20 / Y): site / Y = site * magic >> 20
  uint32_t site_thr;             // 2^32 * (N 2^-21 + 2^-18): site pick needs the exact path within this
  double site_scale;             // (N - 1) + 0.999999, wl.cu:64
  long long max_outer;           // 0 = no cap
  int nwL;                       // 32-bit words per lattice (lattice_words)
  int nwM;                       // 32-bit words of the compact spectrum mask
  long long off_J;               // words: right bonds [nwL], down bonds [nwL]
  long long off_lat;             // words: start lattice of each window [I][nwL]
  long long off_win;             // ints: start[I], end[I], base[I], Lb[I], E0[I]
  long long off_mask;            // words [nwM]
  long long off_out;             // doubles: [I][L] walker-0 log g (compact)
  long long off_state;           // bytes: saved state (state_layout) of a resumable run, -1 = run to the end
  int epoch_outer;               // resumable runs: outer iterations per launch before the state is saved
  int rows;                      // 1: one row per word (lattice_rows)
};

// Per-problem result of the main run (of one launch, for resumable runs).
struct MainResult {
  int status;  // WLG_OK, WLG_ERR_NEW_ENERGY, WLG_ERR_TIMEOUT
  int new_energy;
  long long outer;
  long long flips;
  int done;    // 1: finished (status final, log g written); 0: suspended
  int pad;
  // device clock (%globaltimer, ns) when this launch started the problem and
  // when it finished or suspended it
  long long t_start, t_end;
};

// Saved state of a suspended problem (resumable runs), byte offsets: a
// header (outer iterations, exchange counter, started flag), per window
// f and cond, per walker the exchange permutation, energy, RNG position,
// lattice words, compact histogram [L] and FP64 log g [L] (interleaved
// [bin][walker] like the team's shared memory).
struct StateLayout {
  long long off_f, off_cond, off_perm, off_E, off_pos, off_lat, off_H, off_G, bytes;
};

WLG_HD inline long long align8(long long x) { return (x + 7) & ~7ll; }

WLG_HD inline StateLayout state_layout(int P, int I, int nwL, int L)
{
  StateLayout s{};
  long long o = 32;  // header: long long outer, long long counter, int started
  s.off_f = o;
  o += 8ll * I;
  s.off_cond = o;
  o = align8(o + 4ll * I);
  s.off_perm = o;
  o = align8(o + 4ll * P);
  s.off_E = o;
  o = align8(o + 4ll * P);
  s.off_pos = o;
  o += 8ll * P;
  s.off_lat = o;
  o = align8(o + 4ll * nwL * P);
  s.off_H = o;
  o = align8(o + 4ll * L * P);
  s.off_G = o;
  o += 8ll * L * P;
  s.bytes = o;
  return s;
}

// Team shared-memory layout of a problem (bytes, 16-byte aligned pieces).
struct TeamLayout {
  int off_G, off_Gf, off_H, off_lat, off_E, off_perm, off_mask, off_J, off_nbt, off_f, off_cond, off_flat, off_stab,
    off_win, off_misc;
  int bytes;
};

WLG_HD inline int align16(int x) { return (x + 15) & ~15; }

// reg_lattice: spins in a register (N <= 64); nbt_sites: sites of the
// neighbour table (0 when the table is not used); g_in_smem: FP64 log g in
// shared memory (else in a global pool).
// lat_words: 32-bit words per walker of the lattice area (the lattice
// itself, or the exchange staging of a register lattice); nbt_entries:
// 16-byte neighbour-table entries.
WLG_HD inline TeamLayout team_layout(int team, int L, int nwL, int nwM, int I, int lat_words, int nbt_entries,
                                     bool g_in_smem = true)
{
  TeamLayout t{};
  int o = 0;
  t.off_G = o;
  o = align16(o + (g_in_smem ? 8 * L * team : 0));
  t.off_Gf = o;
  o = align16(o + 4 * L * team);
  t.off_H = o;
  o = align16(o + 4 * L * team);
  t.off_lat = o;
  o = align16(o + 4 * lat_words * team);
  t.off_E = o;
  o = align16(o + 4 * team);
  t.off_perm = o;
  o = align16(o + 4 * team);
  t.off_mask = o;
  o = align16(o + 4 * nwM);
  t.off_J = o;
  o = align16(o + 4 * 2 * nwL);
  t.off_nbt = o;
  o = align16(o + 16 * nbt_entries);
  t.off_f = o;  // f [I], then ln f [I]
  o = align16(o + 16 * I);
  t.off_cond = o;
  o = align16(o + 4 * I);
  t.off_flat = o;
  o = align16(o + 4 * I);
  t.off_stab = o;  // per window: averaging is a fixed point [I], then changed-in-this-pass [I]
  o = align16(o + 8 * I);
  t.off_win = o;
  o = align16(o + 4 * 5 * I);
  t.off_misc = o;
  o = align16(o + 4 * 8);
  t.bytes = o;
  return t;
}

}  // namespace wlg
