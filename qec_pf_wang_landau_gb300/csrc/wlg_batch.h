// Batch pipeline internals shared by the batch entry points
// (wlg_engine_host.cpp) and the serving loop (wlg_server.cpp): where a batch
// runs, the pre-run -> main-run hand-off, the kernel launchers and result
// stitching.  Not part of the C ABI.
#pragma once

#include <cuda_runtime.h>

#include <map>
#include <string>
#include <utility>
#include <vector>

#include "../../include/wlg.h"
#include "wlg_engine.h"
#include "wlg_pool.h"

namespace wlg {

// ---- kernels (wlg_engine.cu)
wlg_status launch_pre_batch(const PreDesc* d_descs, int n, int threads, int smem, int8_t* Jpool, uint8_t* seen_pool,
                            int8_t* found_pool, int* fflag_pool, cudaStream_t s);
// variant: kernel_variant (form | kKernelRows)
int main_batch_capacity(int variant, int cta_threads, int smem);
wlg_status launch_main_batch(int variant, const MainDesc* d_descs, const int* d_order, int n, int team_size,
                             int team_bytes, int teams_per_cta, int grid, int* d_next, double* gpool,
                             long long gslot_doubles, const uint32_t* Jpool, const uint32_t* latpool,
                             const int* winpool, const uint32_t* maskpool, double* outpool, MainResult* results,
                             unsigned char* statepool, cudaStream_t s);

// ---- windows and stitching (interval.cpp, result_handling.cpp)
wlg_status make_windows(int e_min, int e_max, int n, float overlap, std::vector<int>& start, std::vector<int>& end);
using Curve = std::map<int, double>;
// mode: WLG_STITCH_REFERENCE or WLG_STITCH_DEFINED (wlg_context_set_stitching).
wlg_status stitch_windows(std::vector<Curve> windows, int X, int Y, std::vector<std::pair<int, double>>& out,
                          int mode = WLG_STITCH_REFERENCE);

// Stitched, normalised (E, log g) of one finished problem from its compact
// walker-0 output out[I][L] and its windows win[5 I] (start, end, base, Lb, E0).
wlg_status stitched_curve(const MainDesc& d, const double* out, const int* win,
                          std::vector<std::pair<int, double>>& res, int mode = WLG_STITCH_REFERENCE);

// ---- where a batch runs
// Device buffers of one batch, by role.
enum Slot {
  kPreDesc,
  kJ8,
  kSeen,
  kFound,
  kFflag,
  kMainDesc,
  kOrder,
  kNext,
  kJw,
  kLatw,
  kWin,
  kMask,
  kOut,
  kRes,
  kGpool,
  kState,
  kSlots
};

// A stream, a provider of device buffers, optional timing events, and what
// the batch did.
struct Exec {
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t* ev = nullptr;  // 4 events, or nullptr for no timing
  float t_pre = 0, t_main = 0;
  double t_handoff = 0;
  long long h2d = 0, d2h = 0;
  int launches = 0;
  int main_forms = 0;  // bit v: a main-run launch of form v
  // per problem of the batch: when its main run started and ended (ms from
  // the first start, device clock); -1 for problems without a main run
  std::vector<double> p_start_ms, p_end_ms;
  std::string err;
  // teams per CTA chosen by an autotuner, by (form, team size); nullptr or
  // no entry: the built-in rule
  const std::map<std::pair<int, int>, int>* per_cta = nullptr;
  WorkerPool* pool = nullptr;  // host threads for the per-problem phases; nullptr: the calling thread
  // streams on which the main-run launches of different groups run side by
  // side (fork/join through aux_ev: [0] fork, [1 + a] join of aux[a]);
  // n_aux = 0: all on `stream`, one after another
  cudaStream_t* aux = nullptr;
  cudaEvent_t* aux_ev = nullptr;
  int n_aux = 0;
  virtual ~Exec() = default;
  // device buffer for `slot` of at least `bytes` bytes
  virtual wlg_status buffer(Slot slot, size_t bytes, void** out) = 0;
};

inline wlg_status fail(Exec& ex, wlg_status st, const std::string& msg)
{
  ex.err = msg;
  return st;
}

template <typename T>
wlg_status upload(Exec& ex, Slot slot, const std::vector<T>& h, void** dptr)
{
  const size_t bytes = h.size() * sizeof(T);
  wlg_status st = ex.buffer(slot, bytes, dptr);
  if (st != WLG_OK || bytes == 0) return st;
  const cudaError_t e = cudaMemcpyAsync(*dptr, h.data(), bytes, cudaMemcpyHostToDevice, ex.stream);
  ex.h2d += static_cast<long long>(bytes);
  return e == cudaSuccess ? WLG_OK : fail(ex, WLG_ERR_CUDA, cudaGetErrorString(e));
}

template <typename T>
wlg_status download(Exec& ex, const void* dptr, std::vector<T>& h)
{
  if (h.empty()) return WLG_OK;
  const cudaError_t e = cudaMemcpyAsync(h.data(), dptr, h.size() * sizeof(T), cudaMemcpyDeviceToHost, ex.stream);
  ex.d2h += static_cast<long long>(h.size() * sizeof(T));
  return e == cudaSuccess ? WLG_OK : fail(ex, WLG_ERR_CUDA, cudaGetErrorString(e));
}

inline int round32(int x) { return (x + 31) / 32 * 32; }

wlg_status check_problem(const wlg_problem& q);

struct Prepared {
  std::vector<MainDesc> main;                  // problems that reach the main run
  std::vector<int> main_problem;               // index into the batch
  std::vector<std::vector<int>> starts, ends;  // per batch problem
  std::vector<int> lg;                         // per main entry: log2 of the energy step
};

// Main-run inputs of a prepared batch, on the host: packed couplings, start
// lattices, spectrum masks (32-bit words), windows, and the size of the
// walker-0 output; MainDesc offsets index these arrays.
struct Handoff {
  std::vector<uint32_t> Jw, latw, maskw;
  std::vector<int> win;
  long long n_out = 0;
};

// Pre-run outputs on the host, concatenated in problem order with the
// offsets of each PreDesc: couplings J8 [2N], visited energies seen [4N+1]
// (0/1), stored lattices found [n_int][N] (+-1, 0 where none), and fflag
// [n_int] found flags followed by [n_int] their energies.
struct PreOut {
  std::vector<PreDesc> pd;
  std::vector<int8_t> J8, found;
  std::vector<uint8_t> seen;
  std::vector<int> fflag;
};

// Validation and pre-run descriptors (sizes the PreOut arrays).
wlg_status prerun_descs(const wlg_problem* probs, int n, wlg_result* results, PreOut& po, int& threads, int& smem,
                        std::string& err);
// Validation and the pre-run of every problem (one launch).
// couplings (int8 [sum 2N], problem order): the class-'i' bond patterns of the
// problems whose given[p] != 0 (all of them when given is null); the others
// draw theirs.  Null couplings: every problem draws.
wlg_status run_prerun(Exec& ex, const wlg_problem* probs, int n, wlg_result* results, PreOut& po,
                      const int8_t* couplings = nullptr, const unsigned char* given = nullptr);
// The hand-off to the main run on the host.  Problems that cannot start the
// main run get their status in `results` and no MainDesc.
wlg_status handoff(Exec& ex, const wlg_problem* probs, int n, wlg_result* results, const PreOut& po, Prepared& prep,
                   Handoff& ho);
// run_prerun + handoff.
wlg_status prepare_batch(Exec& ex, const wlg_problem* probs, int n, wlg_result* results, Prepared& prep, Handoff& ho,
                         const int8_t* couplings = nullptr, const unsigned char* given = nullptr);

// Main-run forms by lattice storage: 0 spins in shared memory, 1 spins in a
// register, 2 register spins + neighbour table (X, Y >= 3), 3 as 0 with
// FP64 log g in global memory (teams whose state exceeds shared memory).
// (Spins of 65-256-site lattices in 2-4 register words with a neighbour
// table were built and measured: 3-7 % slower than form 0, whose loads are
// broadcasts or conflict-free columns.)
constexpr int kSmemBytes = 227 * 1024;

inline int main_form(const MainDesc& d) { return d.N > 64 ? 0 : (d.X >= 3 && d.Y >= 3 ? 2 : 1); }

// Shared-memory bytes of a team running d in form `form`.
inline int team_bytes(const MainDesc& d, int form, int team)
{
  const bool reg = form == 1 || form == 2;
  return align16(team_layout(team, d.L, d.nwL, d.nwM, d.I, reg ? 2 : d.nwL, form == 2 ? d.N : 0, form != 3).bytes +
                 16);
}

// The form d runs in: main_form, or FP64 log g in global memory when the
// shared-memory lattice form's state does not fit.
inline int fit_form(const MainDesc& d, int team)
{
  const int form = main_form(d);
  return form == 0 && team_bytes(d, 0, team) > kSmemBytes ? 3 : form;
}

// The kernel of a main-run launch: its form (fit_form, 0-3) plus
// kKernelRows when its problems keep lattices one row per word
// (lattice_rows; forms 0 and 3 only).  Problems of one launch share both.
inline int kernel_variant(const MainDesc& d, int team) { return fit_form(d, team) | (d.rows != 0 ? kKernelRows : 0); }

}  // namespace wlg
