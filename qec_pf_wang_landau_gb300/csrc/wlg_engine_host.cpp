// Host side of the batched engine (C++20): the pre-run -> main-run hand-off
// of the reference (file_io.cpp:558-659, mainrun.cu:79-113) for many
// heterogeneous problems, grouping into persistent launches, result
// stitching (result_handling.cpp:26-431) and the C ABI of wlg.h, part 2.

#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <map>
#include <memory>
#include <numbers>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

#include "../../include/wlg.h"
#include "wlg_batch.h"
#include "wlg_engine.h"
#include "wlg_internal.h"
#include "wlg_keys.h"
#include "wlg_pool.h"

namespace wlg {

// ---------------------------------------------------------- energy windows --
// interval.cpp:5-41: window length from a float division truncated toward
// zero, step = trunc(overlap * length), the last window ends at e_max.
wlg_status make_windows(int e_min, int e_max, int n, float overlap, std::vector<int>& start, std::vector<int>& end)
{
  if (n <= 0) return WLG_ERR_INVALID;
  if (overlap > 1 || overlap < 0) return WLG_ERR_INVALID;
  const int range = e_max - e_min + 1;
  const int len =
    static_cast<int>(static_cast<float>(range) / (1.0F + overlap * static_cast<float>(static_cast<unsigned>(n) - 1)));
  const int step = static_cast<int>(overlap * static_cast<float>(len));
  start.assign(static_cast<size_t>(n), 0);
  end.assign(static_cast<size_t>(n), 0);
  int s = e_min;
  for (int b = 0; b < n; ++b) {
    start[b] = s;
    end[b] = (b + 1 < n) ? s + len - 1 : e_max;
    if (start[b] >= end[b]) return WLG_ERR_EMPTY_WINDOW;
    s += step;
  }
  return WLG_OK;
}

namespace {

int energy_host(const int8_t* s, const int8_t* J, int X, int Y, int boundary)
{
  const int N = X * Y;
  int acc = 0;
  for (int i = 0; i < X; ++i)
    for (int j = 0; j < Y; ++j) {
      const int im = (i - 1 >= 0) ? i - 1 : X - 1;
      const int jm = (j - 1 >= 0) ? j - 1 : Y - 1;
      int up = s[im * Y + j] * J[N + im * Y + j];
      int left = s[i * Y + jm] * J[i * Y + jm];
      if (boundary == 1) {
        if (i == 0) up = 0;
        if (j == 0) left = 0;
      }
      acc += s[i * Y + j] * (up + left);
    }
  return -acc;
}

// ----------------------------------------------------------------- stitching --

// Slope of a curve at key x->first towards its successor.  At the curve's
// last key there is none: the reference (result_handling.cpp:125-126) reads
// the successor of the map's last node anyway, which with libstdc++ is the
// map's header, whose key field holds the map's element count and whose
// value is the next 8 bytes in memory (zero or pointer-sized garbage, ~0 as
// a double).  Reference mode uses that phantom node (key = count, value 0);
// defined mode reports "no slope".
bool slope(const Curve& c, Curve::const_iterator x, int mode, double& out)
{
  const auto xn = std::next(x);
  if (xn != c.end()) {
    out = (xn->second - x->second) / (xn->first - x->first);
    return true;
  }
  if (mode != WLG_STITCH_REFERENCE) return false;
  out = (0.0 - x->second) / (static_cast<int>(c.size()) - x->first);
  return true;
}

std::tuple<int, double> best_shared_key(const Curve& a, const Curve& b, int mode)
{
  int key = std::numeric_limits<int>::max();
  double best = std::numeric_limits<double>::max();
  auto x = a.begin();
  auto y = b.begin();
  while (x != a.end() && y != b.end()) {
    if (x->first == y->first) {
      double dx = 0, dy = 0;
      if (slope(a, x, mode, dx) && slope(b, y, mode, dy)) {
        const double d = std::abs(dx - dy);
        if (d < best) {
          best = d;
          key = x->first;
        }
      }
      ++x;
      ++y;
    } else if (x->first < y->first) {
      ++x;
    } else {
      ++y;
    }
  }
  return {key, best};
}

Curve cut(const Curve& c, int e, bool below)
{
  Curve o;
  for (const auto& [k, v] : c)
    if ((below && k < e) || (!below && k >= e)) o.emplace(k, v);
  return o;
}

}  // namespace

// result_handling.cpp:368-431.  `windows[b]` holds walker 0's nonzero log g
// of window b.  Output: normalised (E, log g) pairs, logsumexp = X*Y*ln 2.
wlg_status stitch_windows(std::vector<Curve> windows, int X, int Y, std::vector<std::pair<int, double>>& out, int mode)
{
  const size_t I = windows.size();
  for (auto& c : windows) {
    double mn = std::numeric_limits<double>::max();
    for (const auto& kv : c) mn = std::min(mn, kv.second);
    if (mn == std::numeric_limits<double>::max()) mn = 0;
    for (auto& kv : c) kv.second -= mn;
  }
  std::vector<std::pair<int, int>> keys;  // (next window, stitch energy)
  for (size_t i = 0; i + 1 < I; ++i) {
    int best_key = std::numeric_limits<int>::max();
    double best = std::numeric_limits<double>::max();
    int best_win = -1;
    for (size_t j = i + 1; j < I; ++j) {
      const auto [key, d] = best_shared_key(windows[i], windows[j], mode);
      if (key == std::numeric_limits<int>::max()) break;
      if (d < best) {
        best = d;
        best_key = key;
        best_win = static_cast<int>(j);
      }
    }
    if (best_win >= 0) keys.emplace_back(best_win, best_key);
  }
  std::vector<std::pair<int, int>> kept;  // drop keys that a later key undercuts
  for (size_t i = 0; i < keys.size(); ++i) {
    bool keep = true;
    for (size_t j = i + 1; j < keys.size(); ++j)
      if (keys[j].second <= keys[i].second) keep = false;
    if (keep) kept.push_back(keys[i]);
  }
  if (kept.empty() && I > 1) return WLG_ERR_STITCH;
  std::vector<std::pair<int, int>> chain;  // smallest energy per next window
  for (const auto& kv : kept) {
    if (!chain.empty() && chain.back().first == kv.first) {
      chain.back().second = std::min(chain.back().second, kv.second);
    } else {
      chain.push_back(kv);
    }
  }
  for (size_t i = 0; i < chain.size(); ++i) {
    const int e = chain[i].second;
    const size_t nxt = static_cast<size_t>(chain[i].first);
    const size_t prev = (i == 0) ? 0 : static_cast<size_t>(chain[i - 1].first);
    const auto a = windows[prev].find(e);
    const auto b = windows[nxt].find(e);
    if (a == windows[prev].end() || b == windows[nxt].end()) return WLG_ERR_STITCH;
    const double shift = a->second - b->second;
    for (auto& kv : windows[nxt]) kv.second += shift;
  }
  std::vector<Curve> parts;
  if (chain.empty()) {
    parts.push_back(windows[0]);
  } else {
    auto first = cut(windows[0], chain[0].second, true);
    if (!first.empty()) parts.push_back(std::move(first));
    for (size_t i = 1; i < chain.size(); ++i) {
      auto m = cut(cut(windows[static_cast<size_t>(chain[i - 1].first)], chain[i].second, true),
                   chain[i - 1].second, false);
      if (!m.empty()) parts.push_back(std::move(m));
    }
    auto last = cut(windows[static_cast<size_t>(chain.back().first)], chain.back().second, false);
    if (!last.empty()) parts.push_back(std::move(last));
  }
  double mx = -std::numeric_limits<double>::infinity();
  for (const auto& c : parts)
    for (const auto& kv : c) mx = std::max(mx, kv.second);
  double se = 0.0;
  for (const auto& c : parts)
    for (const auto& kv : c) se += std::exp(kv.second - mx);
  const double shift = mx + std::log(se);
  const double l2 = std::log(2) * static_cast<double>(X) * static_cast<double>(Y);
  out.clear();
  for (const auto& c : parts)
    for (const auto& kv : c) out.emplace_back(kv.first, kv.second + l2 - shift);
  return WLG_OK;
}

// result_handling.cpp:368-431 applied to the compact walker-0 output of one
// problem: each window's reachable energies with nonzero log g.
wlg_status stitched_curve(const MainDesc& d, const double* out, const int* win,
                          std::vector<std::pair<int, double>>& res, int mode)
{
  const int g = 1 << d.lg;
  std::vector<Curve> curves(static_cast<size_t>(d.I));
  for (int b = 0; b < d.I; ++b) {
    const int base = win[2 * d.I + b], len = win[3 * d.I + b];
    for (int c = 0; c < len; ++c) {
      const double v = out[static_cast<long long>(b) * d.L + c];
      if (v != 0) curves[b].emplace(base + c * g, v);
    }
  }
  return stitch_windows(std::move(curves), d.X, d.Y, res, mode);
}

}  // namespace wlg

using namespace wlg;

// ------------------------------------------------------------------ context --

struct DevBuf {
  void* p = nullptr;
  size_t cap = 0;
};


struct wlg_context {
  int device = 0;
  cudaStream_t stream = nullptr;      // where solves run
  cudaStream_t own_stream = nullptr;  // the context's own stream
  size_t budget = 0;
  size_t used = 0;
  DevBuf buf[kSlots];
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  static constexpr int kAux = 4;
  cudaStream_t aux[kAux] = {};          // main-run groups side by side
  cudaEvent_t aux_ev[kAux + 1] = {};    // fork, then one join per aux stream
  void release_aux()
  {
    for (auto& a : aux) {
      if (a != nullptr) {
        cudaStreamSynchronize(a);
        cudaStreamDestroy(a);
      }
      a = nullptr;
    }
    for (auto& e : aux_ev) {
      if (e != nullptr) cudaEventDestroy(e);
      e = nullptr;
    }
  }
  float t_pre = 0, t_main = 0;
  double t_handoff = 0, t_stitch = 0;
  long long h2d = 0, d2h = 0;
  int launches = 0;
  int main_forms = 0;
  std::vector<double> p_start_ms, p_end_ms;  // of the last solve, per problem
  std::map<std::pair<int, int>, int> tuned;  // teams per CTA by (form, team size), from wlg_context_autotune
  int stitching = WLG_STITCH_REFERENCE;
  std::string err;
  std::unique_ptr<wlg::WorkerPool> pool;  // host threads of the per-problem phases, started on first use
  wlg::WorkerPool& workers()
  {
    if (!pool) pool = std::make_unique<wlg::WorkerPool>(
      static_cast<int>(std::min(16u, std::max(1u, std::thread::hardware_concurrency()))));
    return *pool;
  }
};

namespace {

wlg_status grow(wlg_context* ctx, DevBuf& b, size_t bytes, std::string& err)
{
  if (bytes <= b.cap) return WLG_OK;
  bytes = std::max<size_t>(bytes, 256);
  if (b.p != nullptr) {
    cudaFree(b.p);
    ctx->used -= b.cap;
    b.p = nullptr;
    b.cap = 0;
  }
  if (ctx->budget != 0 && ctx->used + bytes > ctx->budget) {
    err = "device memory budget";
    return WLG_ERR_OOM;
  }
  const cudaError_t e = cudaMalloc(&b.p, bytes);
  if (e != cudaSuccess) {
    err = cudaGetErrorString(e);
    return wlg::cuda_status(e);
  }
  b.cap = bytes;
  ctx->used += bytes;
  return WLG_OK;
}

// The context's buffers grow on demand and are kept between batches.
struct ContextExec final : Exec {
  wlg_context* ctx;
  explicit ContextExec(wlg_context* c) : ctx(c)
  {
    device = c->device;
    stream = c->stream;
    ev = c->ev;
    per_cta = &c->tuned;
    pool = &c->workers();
    if (c->aux[0] != nullptr) {
      aux = c->aux;
      aux_ev = c->aux_ev;
      n_aux = wlg_context::kAux;
    }
  }
  wlg_status buffer(Slot slot, size_t bytes, void** out) override
  {
    const wlg_status st = grow(ctx, ctx->buf[slot], bytes, err);
    *out = ctx->buf[slot].p;
    return st;
  }
};

}  // namespace

namespace wlg {

wlg_status check_problem(const wlg_problem& q)
{
  if (q.X < 2 || q.Y < 2 || q.X * q.Y > 4096 || (q.boundary != 0 && q.boundary != 1)) return WLG_ERR_INVALID;
  if (q.pre_walkers <= 0 || q.pre_walkers > 1024 || q.pre_intervals <= 0 || q.pre_iterations < 0)
    return WLG_ERR_INVALID;
  if (q.intervals <= 0 || q.walkers_per_interval <= 0 || q.intervals * q.walkers_per_interval > 1024)
    return WLG_ERR_INVALID;
  if (q.overlap < 0 || q.overlap > 1 || q.iterations <= 0 || q.exchange_every <= 0 || q.max_outer < 0)
    return WLG_ERR_INVALID;
  if (q.exchange_mode != 0 && q.exchange_mode != 1) return WLG_ERR_INVALID;
  if (q.Y > 1024) return WLG_ERR_INVALID;
  return WLG_OK;
}

// Validation, the pre-run of every problem (one launch) and the hand-off to
// the main run on the host.
wlg_status prerun_descs(const wlg_problem* probs, int n, wlg_result* results, PreOut& po, int& threads, int& smem,
                        std::string& err)
{
  std::vector<PreDesc>& pd = po.pd;
  pd.assign(static_cast<size_t>(n), PreDesc{});
  long long oJ = 0, oS = 0, oF = 0, oG = 0;
  threads = 32;
  smem = 0;
  for (int p = 0; p < n; ++p) {
    if (check_problem(probs[p]) != WLG_OK) {
      err = "invalid problem " + std::to_string(p);
      return WLG_ERR_INVALID;
    }
    std::memset(&results[p], 0, sizeof(wlg_result));
  }
  for (int p = 0; p < n; ++p) {
    const wlg_problem& q = probs[p];
    PreDesc& d = pd[p];
    d.X = q.X;
    d.Y = q.Y;
    d.N = q.X * q.Y;
    d.boundary = q.boundary;
    d.prob = q.prob;
    d.error_class = q.error_class == 'I' ? 'i' : q.error_class;
    d.seed = q.seed;
    d.sample = q.sample;
    d.walkers = q.pre_walkers;
    d.n_int = q.pre_intervals;
    std::vector<int> s, e;
    // prerun.cu:23-25: coarse bins of [-2N, 2N] with overlap 1
    if (wlg::make_windows(-2 * d.N, 2 * d.N, q.pre_intervals, 1.0F, s, e) != WLG_OK) {
      err = "pre-run intervals produce empty bins";
      return WLG_ERR_INVALID;
    }
    d.len_int = e[0] - s[0] + 1;
    d.n_iter = q.pre_iterations;
    d.site_magic = static_cast<uint32_t>(((1u << 20) + q.Y - 1) / q.Y);
    for (int site = 0; site < d.N && d.site_magic != 0; ++site)
      if (static_cast<int>((static_cast<uint32_t>(site) * d.site_magic) >> 20) != site / q.Y) d.site_magic = 0;
    d.off_J = oJ;
    d.off_seen = oS;
    d.off_found = oF;
    d.off_fflag = oG;
    oJ += 2 * d.N;
    oS += 4 * d.N + 1;
    oF += static_cast<long long>(d.n_int) * d.N;
    oG += 2 * d.n_int;
    d.smem = wlg::align16(8 * (4 * d.N + 1) + 8 * d.n_int + 16 + 2 * d.N + d.walkers * d.N);
    smem = std::max(smem, d.smem);
    threads = std::max(threads, round32(d.walkers));
    results[p].pre_flips = static_cast<long long>(q.pre_walkers) * q.pre_iterations;
  }
  po.J8.assign(static_cast<size_t>(oJ), 0);
  po.seen.assign(static_cast<size_t>(oS), 0);
  po.found.assign(static_cast<size_t>(oF), 0);
  po.fflag.assign(static_cast<size_t>(oG), 0);
  if (smem > 227 * 1024) {
    err = "pre-run walkers x lattice too large for shared memory";
    return WLG_ERR_INVALID;
  }
  return WLG_OK;
}

wlg_status run_prerun(Exec& ex, const wlg_problem* probs, int n, wlg_result* results, PreOut& po,
                      const int8_t* couplings, const unsigned char* given)
{
  ex.h2d = ex.d2h = 0;
  ex.launches = 0;
  ex.main_forms = 0;
  ex.t_pre = ex.t_main = 0;
  ex.t_handoff = 0;
  int threads = 32, smem = 0;
  std::string err;
  wlg_status st = prerun_descs(probs, n, results, po, threads, smem, err);
  if (st != WLG_OK) return fail(ex, st, err);
  std::vector<PreDesc>& pd = po.pd;
  bool any_given = false;
  if (couplings != nullptr)
    for (int p = 0; p < n; ++p) {
      if (given != nullptr && given[p] == 0) continue;
      PreDesc& d = pd[p];
      for (int q = 0; q < 2 * d.N; ++q) {
        const int8_t v = couplings[d.off_J + q];
        if (v != 1 && v != -1) return fail(ex, WLG_ERR_INVALID, "couplings of problem " + std::to_string(p) + " not +-1");
        po.J8[d.off_J + q] = v;
      }
      d.given_J = 1;
      any_given = true;
    }
  const long long oJ = static_cast<long long>(po.J8.size()), oS = static_cast<long long>(po.seen.size());
  const long long oF = static_cast<long long>(po.found.size()), oG = static_cast<long long>(po.fflag.size());
  void *d_pd = nullptr, *d_J8 = nullptr, *d_seen = nullptr, *d_found = nullptr, *d_fflag = nullptr;
  if ((st = upload(ex, kPreDesc, pd, &d_pd)) != WLG_OK) return st;
  if ((st = ex.buffer(kJ8, static_cast<size_t>(oJ), &d_J8)) != WLG_OK) return st;
  if ((st = ex.buffer(kSeen, static_cast<size_t>(oS), &d_seen)) != WLG_OK) return st;
  if ((st = ex.buffer(kFound, static_cast<size_t>(oF), &d_found)) != WLG_OK) return st;
  if ((st = ex.buffer(kFflag, static_cast<size_t>(oG) * sizeof(int), &d_fflag)) != WLG_OK) return st;
  cudaMemsetAsync(d_found, 0, static_cast<size_t>(oF), ex.stream);
  if (any_given) {
    if (cudaMemcpyAsync(d_J8, po.J8.data(), static_cast<size_t>(oJ), cudaMemcpyHostToDevice, ex.stream) != cudaSuccess)
      return fail(ex, WLG_ERR_CUDA, "couplings upload failed");
    ex.h2d += oJ;
  }
  if (ex.ev != nullptr) cudaEventRecord(ex.ev[0], ex.stream);
  st = wlg::launch_pre_batch(static_cast<const PreDesc*>(d_pd), n, threads, smem, static_cast<int8_t*>(d_J8),
                             static_cast<uint8_t*>(d_seen), static_cast<int8_t*>(d_found), static_cast<int*>(d_fflag),
                             ex.stream);
  if (st != WLG_OK) return fail(ex, st, "pre-run launch failed");
  ++ex.launches;
  if (ex.ev != nullptr) cudaEventRecord(ex.ev[1], ex.stream);
  download(ex, d_J8, po.J8);
  download(ex, d_seen, po.seen);
  download(ex, d_found, po.found);
  download(ex, d_fflag, po.fflag);
  if (cudaStreamSynchronize(ex.stream) != cudaSuccess) return fail(ex, WLG_ERR_CUDA, "pre-run failed");
  if (ex.ev != nullptr) cudaEventElapsedTime(&ex.t_pre, ex.ev[0], ex.ev[1]);
  return WLG_OK;
}

// The hand-off to the main run (file_io.cpp:558-659, mainrun.cu:79-113)
// from pre-run outputs.
namespace {

// One problem's share of the hand-off, computed independently of the others.
struct HandoffPart {
  wlg_status status = WLG_OK;  // the problem's own failure (no lattice, windows)
  wlg_status fatal = WLG_OK;   // a failure of the whole batch
  const char* why = "";
  bool windows = false;  // ws/we were made
  bool main = false;     // the problem reaches the main run
  MainDesc d{};
  int lg = 0;
  std::vector<int> ws, we, win;
  std::vector<uint32_t> Jw, latw, maskw;
};

void handoff_one(const wlg_problem& q, const PreDesc& a, const PreOut& po, HandoffPart& out)
{
  const std::vector<int8_t>& J8 = po.J8;
  const std::vector<int8_t>& found = po.found;
  const std::vector<int>& fflag = po.fflag;
  const int N = a.N;
  const uint8_t* h = po.seen.data() + a.off_seen;
  int first = -1, last = -1;
  for (int i = 0; i <= 4 * N; ++i)
    if (h[i] == 1) {
      if (first < 0) first = i;
      last = i;
    }
  if (first < 0) {
    out.status = WLG_ERR_NO_LATTICE;
    return;
  }
  const int e_lo = -2 * N + first, e_hi = -2 * N + last;
  std::vector<int>& ws = out.ws;
  std::vector<int>& we = out.we;
  const wlg_status wst = wlg::make_windows(e_lo, e_hi, q.intervals, q.overlap, ws, we);
  if (wst != WLG_OK) {
    out.status = wst;
    return;
  }
  out.windows = true;
  // energy step of the lattice: 4 when every site has an even number of
  // bonds (periodic, or open 2x2), else 2; checked against the spectrum
  int g = (q.boundary == 0 || (q.X == 2 && q.Y == 2)) ? 4 : 2;
  for (int i = first; i <= last; ++i)
    if (h[i] == 1 && (i - first) % g != 0) g = ((i - first) % 2 == 0) ? 2 : 1;
  const int lg = g == 4 ? 2 : (g == 2 ? 1 : 0);
  // start lattices: lowest-energy stored lattice inside each window
  std::map<int, int> by_energy;
  for (int k = 0; k < a.n_int; ++k)
    if (fflag[a.off_fflag + k] != 0) by_energy.emplace(fflag[a.off_fflag + a.n_int + k], k);
  const int nwL = wlg::lattice_words(q.X, q.Y);
  std::vector<int> pick(static_cast<size_t>(q.intervals), -1), E0(static_cast<size_t>(q.intervals));
  bool ok = true;
  for (int b = 0; b < q.intervals && ok; ++b) {
    for (const auto& [en, k] : by_energy)
      if (en >= ws[b] && en <= we[b]) {
        pick[b] = k;
        E0[b] = en;
        break;
      }
    ok = pick[b] >= 0;
  }
  if (!ok) {
    out.status = WLG_ERR_NO_LATTICE;
    return;
  }
  MainDesc& d = out.d;
  d.X = q.X;
  d.Y = q.Y;
  d.N = N;
  d.boundary = q.boundary;
  d.I = q.intervals;
  d.W = q.walkers_per_interval;
  d.nwalk = d.I * d.W;
  d.team = round32(d.nwalk);
  d.e_min = e_lo;
  d.e_max = e_hi;
  d.lg = lg;
  d.n_iter = q.iterations;
  d.exch_every = q.exchange_every;
  d.exch_mode = q.exchange_mode;
  d.parity_base = q.global_parity ? static_cast<int>((static_cast<long long>(q.sample) * q.intervals) & 1) : 0;
  d.alpha = q.alpha;
  d.beta = q.beta;
  d.loop_lim = std::exp(q.beta);
  d.key_wl = static_cast<uint32_t>(wlg::key_u32(q.seed, static_cast<uint64_t>(q.sample)));
  d.key_ex = wlg::key_i32(q.seed, static_cast<uint64_t>(q.sample));
  d.site_magic = static_cast<uint32_t>(((1u << 20) + q.Y - 1) / q.Y);
  for (int site = 0; site < N; ++site)
    if (static_cast<int>((static_cast<uint32_t>(site) * d.site_magic) >> 20) != site / q.Y) ok = false;
  if (!ok) {
    out.fatal = WLG_ERR_INVALID;
    out.why = "lattice too large for the site division";
    return;
  }
  d.site_scale = (N - 1 + 0.999999);
  d.site_thr = static_cast<uint32_t>(N) * 2048u + 16384u;
  d.max_outer = q.max_outer;
  d.nwL = nwL;
  d.rows = wlg::lattice_rows(q.X, q.Y) ? 1 : 0;
  const int nbins = (e_hi - e_lo) / g + 1;
  d.nwM = (nbins + 31) / 32;
  // windows: start, end, compact base (first energy >= start on the lattice
  // of reachable energies), compact length, start energy
  int L = 1;
  std::vector<int> base(static_cast<size_t>(d.I)), len(static_cast<size_t>(d.I));
  for (int b = 0; b < d.I; ++b) {
    const int r = ((e_lo - ws[b]) % g + g) % g;
    base[b] = ws[b] + r;
    len[b] = base[b] <= we[b] ? (we[b] - base[b]) / g + 1 : 0;
    L = std::max(L, len[b]);
  }
  d.L = L;
  // bit-packed couplings (right bonds, then down bonds) and lattices in the
  // layout of lattice_bit
  auto pack = [&](const int8_t* v, std::vector<uint32_t>& dst) {
    const size_t at = dst.size();
    dst.resize(at + static_cast<size_t>(nwL), 0u);
    for (int s = 0; s < N; ++s) {
      int wd = 0, bit = 0;
      wlg::lattice_bit(q.X, q.Y, s, wd, bit);
      if (v[s] == -1) dst[at + static_cast<size_t>(wd)] |= 1u << bit;
    }
  };
  pack(J8.data() + a.off_J, out.Jw);
  pack(J8.data() + a.off_J + N, out.Jw);
  for (int b = 0; b < d.I; ++b) {
    const int8_t* src = found.data() + a.off_found + static_cast<long long>(pick[b]) * N;
    if (wlg::energy_host(src, J8.data() + a.off_J, q.X, q.Y, q.boundary) != E0[b]) {
      out.fatal = WLG_ERR_ENERGY_RANGE;
      out.why = "stored lattice energy mismatch";
      return;
    }
    pack(src, out.latw);
  }
  std::vector<int>& win = out.win;
  win.insert(win.end(), ws.begin(), ws.end());
  win.insert(win.end(), we.begin(), we.end());
  win.insert(win.end(), base.begin(), base.end());
  win.insert(win.end(), len.begin(), len.end());
  win.insert(win.end(), E0.begin(), E0.end());
  for (int wd = 0; wd < d.nwM; ++wd) {
    uint32_t v = 0;
    for (int bit = 0; bit < 32; ++bit) {
      const int c = wd * 32 + bit;
      if (c < nbins && h[first + c * g] == 1) v |= 1u << bit;
    }
    out.maskw.push_back(v);
  }
  d.off_state = -1;
  d.epoch_outer = 0;
  out.lg = lg;
  out.main = true;
}

}  // namespace

wlg_status handoff(Exec& ex, const wlg_problem* probs, int n, wlg_result* results, const PreOut& po, Prepared& prep,
                   Handoff& ho)
{
  using clock = std::chrono::steady_clock;
  const auto t0 = clock::now();
  // problems are independent: the host workers take them in chunks, then
  // the parts are packed in problem order
  std::vector<HandoffPart> parts(static_cast<size_t>(n));
  const auto one = [&](int p) { handoff_one(probs[p], po.pd[p], po, parts[p]); };
  if (ex.pool != nullptr) {
    ex.pool->run(n, 8, one);
  } else {
    for (int p = 0; p < n; ++p) one(p);
  }
  for (const HandoffPart& part : parts)
    if (part.fatal != WLG_OK) return fail(ex, part.fatal, part.why);
  std::vector<uint32_t>& Jw = ho.Jw;
  std::vector<uint32_t>& latw = ho.latw;
  std::vector<uint32_t>& maskw = ho.maskw;
  std::vector<int>& win = ho.win;
  Jw.clear();
  latw.clear();
  maskw.clear();
  win.clear();
  long long o_out = 0;
  prep.starts.assign(static_cast<size_t>(n), {});
  prep.ends.assign(static_cast<size_t>(n), {});
  for (int p = 0; p < n; ++p) {
    HandoffPart& part = parts[p];
    if (part.windows) {
      prep.starts[p] = std::move(part.ws);
      prep.ends[p] = std::move(part.we);
    }
    if (part.status != WLG_OK) {
      results[p].status = part.status;
      continue;
    }
    if (!part.main) continue;
    MainDesc d = part.d;
    d.off_J = static_cast<long long>(Jw.size());
    Jw.insert(Jw.end(), part.Jw.begin(), part.Jw.end());
    d.off_lat = static_cast<long long>(latw.size());
    latw.insert(latw.end(), part.latw.begin(), part.latw.end());
    d.off_win = static_cast<long long>(win.size());
    win.insert(win.end(), part.win.begin(), part.win.end());
    d.off_mask = static_cast<long long>(maskw.size());
    maskw.insert(maskw.end(), part.maskw.begin(), part.maskw.end());
    d.off_out = o_out;
    o_out += static_cast<long long>(d.I) * d.L;
    prep.main.push_back(d);
    prep.main_problem.push_back(p);
    prep.lg.push_back(part.lg);
  }
  ex.t_handoff = std::chrono::duration<double, std::milli>(clock::now() - t0).count();
  ho.n_out = o_out;
  return WLG_OK;
}

wlg_status prepare_batch(Exec& ex, const wlg_problem* probs, int n, wlg_result* results, Prepared& prep, Handoff& ho,
                         const int8_t* couplings, const unsigned char* given)
{
  PreOut po;
  const wlg_status st = run_prerun(ex, probs, n, results, po, couplings, given);
  if (st != WLG_OK) return st;
  return handoff(ex, probs, n, results, po, prep, ho);
}

}  // namespace wlg

namespace {

constexpr int kTimedEpoch = 4;  // outer iterations per launch under a time limit

// The main run of a prepared batch: one persistent launch per (form, team
// size).  time_limit_s > 0: resumable launches of kTimedEpoch outer
// iterations each, repeated until every problem finished or the limit
// passed (the reference checks its time limit after each outer iteration,
// mainrun.cu:376-383); unfinished problems end with WLG_ERR_TIMEOUT.
wlg_status run_main(Exec& ex, wlg_result* results, Prepared& prep, const Handoff& ho, std::vector<MainResult>& mres,
                    std::vector<double>& out_host, std::vector<int>& win_host, double time_limit_s)
{
  wlg_status st = WLG_OK;
  const std::vector<uint32_t>& Jw = ho.Jw;
  const std::vector<uint32_t>& latw = ho.latw;
  const std::vector<uint32_t>& maskw = ho.maskw;
  const std::vector<int>& win = ho.win;
  const long long o_out = ho.n_out;

  // ---------------- main run: one persistent launch per (lattice storage, team size)
  const int m = static_cast<int>(prep.main.size());
  mres.assign(static_cast<size_t>(m), MainResult{});
  // per problem of the batch (a sub-batch, as the autotuner runs, lists only
  // its main-run problems)
  size_t n_prob = prep.starts.size();
  for (const int p : prep.main_problem) n_prob = std::max(n_prob, static_cast<size_t>(p) + 1);
  ex.p_start_ms.assign(n_prob, -1.0);
  ex.p_end_ms.assign(n_prob, -1.0);
  out_host.assign(static_cast<size_t>(o_out), 0.0);
  win_host = win;
  if (m == 0) return WLG_OK;
  int sms = 1;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ex.device);
  // one launch per (form, team size); the form by lattice storage (fit_form)
  std::map<std::pair<int, int>, std::vector<int>> groups;
  for (int i = 0; i < m; ++i) groups[{wlg::kernel_variant(prep.main[i], prep.main[i].team), prep.main[i].team}].push_back(i);
  // Longest problems first (larger lattices take more outer iterations of
  // longer steps): the groups' launches are issued, and each group's queue
  // is ordered, by decreasing lattice size, so the batch's longest serial
  // chains start at once instead of waiting for SMs held by shorter ones.
  // Results do not depend on the order (every problem's trajectory is its own).
  std::vector<std::pair<std::pair<int, int>, std::vector<int>>> ordered(groups.begin(), groups.end());
  for (auto& [key, idx] : ordered)
    std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return prep.main[a].N > prep.main[b].N; });
  std::stable_sort(ordered.begin(), ordered.end(), [&](const auto& a, const auto& b) {
    return prep.main[a.second.front()].N > prep.main[b.second.front()].N;
  });
  std::vector<int> order;
  // variant, team, bytes, per_cta, first, count, L (max compact bins)
  std::vector<std::tuple<int, int, int, int, int, int, int>> launches;
  for (const auto& [key, idx] : ordered) {
    const int variant = key.first;
    const int team = key.second;
    int bytes = 0;
    int Lmax = 1;
    for (int i : idx) {
      bytes = std::max(bytes, wlg::team_bytes(prep.main[i], variant & 3, team));
      Lmax = std::max(Lmax, prep.main[i].L);
    }
    if (bytes > wlg::kSmemBytes) return fail(ex, WLG_ERR_INVALID, "problem state exceeds shared memory");
    int per_cta = team <= 256 ? 256 / team : 1;
    per_cta = std::min(per_cta, (227 * 1024) / bytes);
    if (team > 32) per_cta = std::min(per_cta, 15);
    // small batches: spread the teams over all SMs (>= 2 CTAs per SM) rather
    // than packing them into few CTAs
    per_cta = std::min(per_cta, static_cast<int>(idx.size()) / (2 * sms));
    per_cta = std::max(per_cta, 1);
    if (ex.per_cta != nullptr) {
      auto it = ex.per_cta->find({variant, team});
      if (it != ex.per_cta->end()) {
        per_cta = std::max(1, std::min(it->second, team <= 256 ? 256 / team : 1));
        per_cta = std::max(1, std::min(per_cta, (227 * 1024) / bytes));
      }
    }
    launches.emplace_back(variant, team, bytes, per_cta, static_cast<int>(order.size()), static_cast<int>(idx.size()),
                          Lmax);
    order.insert(order.end(), idx.begin(), idx.end());
  }
  const bool timed = time_limit_s > 0;
  void* d_state = nullptr;
  if (timed) {  // resumable runs: one state block per problem
    long long off = 0;
    for (MainDesc& d : prep.main) {
      d.off_state = off;
      d.epoch_outer = kTimedEpoch;
      off += wlg::align8(wlg::state_layout(d.team, d.I, d.nwL, d.L).bytes);
    }
    if ((st = ex.buffer(kState, static_cast<size_t>(off), &d_state)) != WLG_OK) return st;
    cudaMemsetAsync(d_state, 0, static_cast<size_t>(off), ex.stream);
  }
  void *d_md = nullptr, *d_order = nullptr, *d_Jw = nullptr, *d_latw = nullptr, *d_win = nullptr, *d_mask = nullptr;
  void *d_out = nullptr, *d_res = nullptr, *d_next = nullptr;
  if ((st = upload(ex, kMainDesc, prep.main, &d_md)) != WLG_OK) return st;
  if ((st = upload(ex, kOrder, order, &d_order)) != WLG_OK) return st;
  if ((st = upload(ex, kJw, Jw, &d_Jw)) != WLG_OK) return st;
  if ((st = upload(ex, kLatw, latw, &d_latw)) != WLG_OK) return st;
  if ((st = upload(ex, kWin, win, &d_win)) != WLG_OK) return st;
  if ((st = upload(ex, kMask, maskw, &d_mask)) != WLG_OK) return st;
  if ((st = ex.buffer(kOut, static_cast<size_t>(o_out) * sizeof(double), &d_out)) != WLG_OK) return st;
  if ((st = ex.buffer(kRes, static_cast<size_t>(m) * sizeof(MainResult), &d_res)) != WLG_OK) return st;
  if ((st = ex.buffer(kNext, launches.size() * sizeof(int), &d_next)) != WLG_OK) return st;
  if (timed) cudaMemsetAsync(d_res, 0, static_cast<size_t>(m) * sizeof(MainResult), ex.stream);
  // grids, and the global log g pool of the variant-3 launches (one slice per
  // resident team, launches side by side)
  std::vector<int> grids(launches.size());
  std::vector<long long> gpool_off(launches.size(), 0);
  long long gpool_doubles = 0;
  for (size_t g = 0; g < launches.size(); ++g) {
    const auto [variant, team, bytes, per_cta, first, count, Lmax] = launches[g];
    const int cap = wlg::main_batch_capacity(variant, team * per_cta, bytes * per_cta);
    if (cap <= 0) return fail(ex, WLG_ERR_CUDA, "main-run configuration does not fit an SM");
    grids[g] = std::min(cap, (count + per_cta - 1) / per_cta);
    if ((variant & 3) == 3) {
      gpool_off[g] = gpool_doubles;
      gpool_doubles += static_cast<long long>(grids[g]) * per_cta * Lmax * team;
    }
  }
  void* d_gpool = nullptr;
  if (gpool_doubles > 0 &&
      (st = ex.buffer(kGpool, static_cast<size_t>(gpool_doubles) * sizeof(double), &d_gpool)) != WLG_OK)
    return st;
  auto launch_all = [&]() -> wlg_status {
    cudaMemsetAsync(d_next, 0, launches.size() * sizeof(int), ex.stream);
    // groups side by side: a persistent launch's CTAs exit as its queue
    // drains, and the next group's CTAs take the freed SMs during its tail
    const int n_fork = ex.n_aux > 0 && launches.size() > 1 ? std::min<int>(ex.n_aux, static_cast<int>(launches.size())) : 0;
    if (n_fork > 0) {
      cudaEventRecord(ex.aux_ev[0], ex.stream);
      for (int a = 0; a < n_fork; ++a) cudaStreamWaitEvent(ex.aux[a], ex.aux_ev[0], 0);
    }
    wlg_status s2 = WLG_OK;
    for (size_t g = 0; g < launches.size() && s2 == WLG_OK; ++g) {
      const auto [variant, team, bytes, per_cta, first, count, Lmax] = launches[g];
      const int grid = grids[g];
      double* gp = (variant & 3) == 3 ? static_cast<double*>(d_gpool) + gpool_off[g] : nullptr;
      s2 = wlg::launch_main_batch(
        variant, static_cast<const MainDesc*>(d_md), static_cast<const int*>(d_order) + first, count, team, bytes,
        per_cta, grid, static_cast<int*>(d_next) + g, gp, static_cast<long long>(Lmax) * team,
        static_cast<const uint32_t*>(d_Jw), static_cast<const uint32_t*>(d_latw), static_cast<const int*>(d_win),
        static_cast<const uint32_t*>(d_mask), static_cast<double*>(d_out), static_cast<MainResult*>(d_res),
        static_cast<unsigned char*>(d_state), n_fork > 0 ? ex.aux[g % n_fork] : ex.stream);
      if (s2 == WLG_OK) {
        ++ex.launches;
        ex.main_forms |= 1 << (variant & 3);
      }
    }
    for (int a = 0; a < n_fork; ++a) {  // join (also after a failed launch)
      cudaEventRecord(ex.aux_ev[1 + a], ex.aux[a]);
      cudaStreamWaitEvent(ex.stream, ex.aux_ev[1 + a], 0);
    }
    if (s2 != WLG_OK) return fail(ex, s2, "main-run launch failed");
    return WLG_OK;
  };
  if (ex.ev != nullptr) cudaEventRecord(ex.ev[2], ex.stream);
  const auto t0 = std::chrono::steady_clock::now();
  for (;;) {
    if ((st = launch_all()) != WLG_OK) return st;
    if (!timed) break;
    download(ex, d_res, mres);
    if (cudaStreamSynchronize(ex.stream) != cudaSuccess) return fail(ex, WLG_ERR_CUDA, "main run failed");
    bool all = true;
    for (const MainResult& r : mres) all = all && r.done != 0;
    if (all) break;
    if (std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count() >= time_limit_s) {
      for (MainResult& r : mres)
        if (r.done == 0) r.status = WLG_ERR_TIMEOUT;
      break;
    }
  }
  if (ex.ev != nullptr) cudaEventRecord(ex.ev[3], ex.stream);
  std::vector<MainResult> last = mres;
  download(ex, d_res, mres);
  download(ex, d_out, out_host);
  if (cudaStreamSynchronize(ex.stream) != cudaSuccess) return fail(ex, WLG_ERR_CUDA, "main run failed");
  if (timed)
    for (int i = 0; i < m; ++i)
      if (last[i].status == WLG_ERR_TIMEOUT && last[i].done == 0) mres[i].status = WLG_ERR_TIMEOUT;
  if (ex.ev != nullptr) cudaEventElapsedTime(&ex.t_main, ex.ev[2], ex.ev[3]);
  long long t_first = 0;
  for (int i = 0; i < m; ++i) t_first = i == 0 ? mres[i].t_start : std::min(t_first, mres[i].t_start);
  for (int i = 0; i < m; ++i) {
    ex.p_start_ms[prep.main_problem[i]] = 1e-6 * static_cast<double>(mres[i].t_start - t_first);
    ex.p_end_ms[prep.main_problem[i]] = 1e-6 * static_cast<double>(mres[i].t_end - t_first);
  }
  for (int i = 0; i < m; ++i) {
    wlg_result& r = results[prep.main_problem[i]];
    r.status = mres[i].status;
    r.new_energy = mres[i].new_energy;
    r.outer_iterations = mres[i].outer;
    r.flips = mres[i].flips;
  }
  return WLG_OK;
}

// The whole batch up to the main-run results.
wlg_status run_batch(Exec& ex, const wlg_problem* probs, int n, wlg_result* results,
                     std::vector<MainResult>& mres, Prepared& prep, std::vector<double>& out_host,
                     std::vector<int>& win_host, const int8_t* couplings = nullptr)
{
  Handoff ho;
  const wlg_status st = wlg::prepare_batch(ex, probs, n, results, prep, ho, couplings);
  if (st != WLG_OK) return st;
  return run_main(ex, results, prep, ho, mres, out_host, win_host, 0.0);
}

void keep_stats(wlg_context* ctx, const Exec& ex)
{
  ctx->t_pre = ex.t_pre;
  ctx->t_main = ex.t_main;
  ctx->t_handoff = ex.t_handoff;
  ctx->t_stitch = 0;
  ctx->h2d = ex.h2d;
  ctx->d2h = ex.d2h;
  ctx->launches = ex.launches;
  ctx->main_forms = ex.main_forms;
  ctx->p_start_ms = ex.p_start_ms;
  ctx->p_end_ms = ex.p_end_ms;
  if (!ex.err.empty()) ctx->err = ex.err;
}

wlg_status raw_windows(Exec& ex, const wlg_problem* problems, int n, const Prepared& prep,
                       const std::vector<double>& out, const std::vector<int>& win, int* win_start, int* win_end,
                       double* raw_log_g, long long raw_capacity, long long* raw_offset);

// Pre-run outputs given by the caller (the layout wlg_prerun writes) as the
// hand-off's input; WLG_ERR_INVALID when couplings or stored lattices are
// not +-1.
wlg_status given_prerun(const wlg_problem* problems, int n, wlg_result* results, const unsigned char* seen,
                        const signed char* couplings, const int* found, const int* found_energy,
                        const signed char* lattices, PreOut& po, std::string& err)
{
  int threads = 0, smem = 0;
  wlg_status st = prerun_descs(problems, n, results, po, threads, smem, err);
  if (st != WLG_OK) return st;
  long long ob = 0;
  auto pm1 = [](const signed char* v, long long m) {
    for (long long i = 0; i < m; ++i)
      if (v[i] != 1 && v[i] != -1) return false;
    return true;
  };
  for (int p = 0; p < n; ++p) {
    const PreDesc& d = po.pd[p];
    bool valid = pm1(couplings + d.off_J, 2LL * d.N);
    for (int b = 0; b < d.n_int && valid; ++b)
      valid = found[ob + b] == 0 || pm1(lattices + d.off_found + static_cast<long long>(b) * d.N, d.N);
    if (!valid) {
      err = "couplings or stored lattice of problem " + std::to_string(p) + " not +-1";
      return WLG_ERR_INVALID;
    }
    std::memcpy(po.seen.data() + d.off_seen, seen + d.off_seen, static_cast<size_t>(4 * d.N + 1));
    std::memcpy(po.J8.data() + d.off_J, couplings + d.off_J, static_cast<size_t>(2 * d.N));
    std::memcpy(po.found.data() + d.off_found, lattices + d.off_found, static_cast<size_t>(d.n_int) * d.N);
    for (int b = 0; b < d.n_int; ++b) {
      po.fflag[d.off_fflag + b] = found[ob + b];
      po.fflag[d.off_fflag + d.n_int + b] = found_energy[ob + b];
    }
    ob += d.n_int;
  }
  return WLG_OK;
}

// An Exec for host-only phases: it hands out no device buffers.
struct HostExec final : Exec {
  wlg_status buffer(Slot, size_t, void**) override { return WLG_ERR_INVALID; }
};

// Dense walker-0 log g of window b (zeros where the lattice cannot reach).
void dense_window(const MainDesc& d, const std::vector<double>& out, const std::vector<int>& win, int b,
                  std::vector<double>& dense)
{
  const int s = win[d.off_win + b], e = win[d.off_win + d.I + b];
  const int base = win[d.off_win + 2 * d.I + b], len = win[d.off_win + 3 * d.I + b];
  dense.assign(static_cast<size_t>(e - s + 1), 0.0);
  for (int c = 0; c < len; ++c) dense[base + (c << d.lg) - s] = out[d.off_out + static_cast<long long>(b) * d.L + c];
}

}  // namespace

extern "C" {

wlg_status wlg_context_create(int device, size_t mem_budget_bytes, wlg_context** out)
{
  return wlg::guarded([&]() -> wlg_status {
    if (out == nullptr) return WLG_ERR_INVALID;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n) return WLG_ERR_INVALID;
    if (cudaSetDevice(device) != cudaSuccess) return WLG_ERR_CUDA;
    auto* ctx = new wlg_context();
    ctx->device = device;
    ctx->budget = mem_budget_bytes;
    if (cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking) != cudaSuccess) {
      delete ctx;
      return WLG_ERR_CUDA;
    }
    ctx->stream = ctx->own_stream;
    for (auto& e : ctx->ev) cudaEventCreate(&e);
    bool aux_ok = true;
    for (auto& a : ctx->aux) aux_ok = aux_ok && cudaStreamCreateWithFlags(&a, cudaStreamNonBlocking) == cudaSuccess;
    for (auto& e : ctx->aux_ev) aux_ok = aux_ok && cudaEventCreateWithFlags(&e, cudaEventDisableTiming) == cudaSuccess;
    if (!aux_ok) ctx->release_aux();  // launches then run one after another on the context's stream
    *out = ctx;
    return WLG_OK;
  });
}

wlg_status wlg_context_destroy(wlg_context* ctx)
{
  if (ctx == nullptr) return WLG_ERR_INVALID;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  for (DevBuf& b : ctx->buf)
    if (b.p != nullptr) cudaFree(b.p);
  for (auto& e : ctx->ev) cudaEventDestroy(e);
  ctx->release_aux();
  cudaStreamDestroy(ctx->own_stream);
  delete ctx;
  return WLG_OK;
}

wlg_status wlg_context_set_stream(wlg_context* ctx, wlg_stream stream)
{
  if (ctx == nullptr) return WLG_ERR_INVALID;
  cudaSetDevice(ctx->device);
  if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) return WLG_ERR_CUDA;
  ctx->stream = stream != nullptr ? static_cast<cudaStream_t>(stream) : ctx->own_stream;
  return WLG_OK;
}

wlg_status wlg_context_set_stitching(wlg_context* ctx, int mode)
{
  if (ctx == nullptr || (mode != WLG_STITCH_REFERENCE && mode != WLG_STITCH_DEFINED)) return WLG_ERR_INVALID;
  ctx->stitching = mode;
  return WLG_OK;
}

const char* wlg_context_last_error(const wlg_context* ctx) { return ctx == nullptr ? "" : ctx->err.c_str(); }

wlg_status wlg_solve_raw(wlg_context* ctx, const wlg_problem* problems, int n, wlg_result* results, int* win_start,
                         int* win_end, double* raw_log_g, long long raw_capacity, long long* raw_offset)
{
  return wlg::guarded([&]() -> wlg_status {
    if (ctx == nullptr || (n > 0 && (problems == nullptr || results == nullptr))) return WLG_ERR_INVALID;
    cudaSetDevice(ctx->device);
    std::vector<MainResult> mres;
    Prepared prep;
    std::vector<double> out;
    std::vector<int> win;
    ContextExec ex(ctx);
    wlg_status st = run_batch(ex, problems, n, results, mres, prep, out, win);
    keep_stats(ctx, ex);
    if (st != WLG_OK) return st;
    return raw_windows(ex, problems, n, prep, out, win, win_start, win_end, raw_log_g, raw_capacity, raw_offset);
  });
}

}  // extern "C"

namespace {

// Stitched, normalised log g of every problem that finished the main run
// into caller arrays (wlg_solve layout).
wlg_status stitch_all(wlg_context* ctx, const Prepared& prep, const std::vector<double>& out,
                      const std::vector<int>& win, wlg_result* results, int* energies, double* log_g,
                      long long capacity)
{
  const auto t0 = std::chrono::steady_clock::now();
  const size_t m = prep.main.size();
  // problems are independent: stitch them on the host's cores, then pack in
  // problem order
  std::vector<std::vector<std::pair<int, double>>> curves(m);
  std::vector<wlg_status> sst(m, WLG_OK);
  ctx->workers().run(static_cast<int>(m), 8, [&](int i) {
    if (results[prep.main_problem[i]].status != WLG_OK) return;
    const MainDesc& d = prep.main[i];
    sst[i] = wlg::stitched_curve(d, out.data() + d.off_out, win.data() + d.off_win, curves[i], ctx->stitching);
  });
  long long pos = 0;
  for (size_t i = 0; i < m; ++i) {
    wlg_result& r = results[prep.main_problem[i]];
    r.offset = pos;
    r.n_energies = 0;
    if (r.status != WLG_OK) continue;
    if (sst[i] != WLG_OK) {
      r.status = sst[i];
      continue;
    }
    const auto& res = curves[i];
    if (pos + static_cast<long long>(res.size()) > capacity) {
      ctx->err = "result arrays";
      return WLG_ERR_CAPACITY;
    }
    for (size_t k = 0; k < res.size(); ++k) {
      energies[pos + static_cast<long long>(k)] = res[k].first;
      log_g[pos + static_cast<long long>(k)] = res[k].second;
    }
    r.n_energies = static_cast<int>(res.size());
    pos += static_cast<long long>(res.size());
  }
  ctx->t_stitch = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return WLG_OK;
}

// The walker-0 log g of every window on the reference's dense layout.
wlg_status raw_windows(Exec& ex, const wlg_problem* problems, int n, const Prepared& prep,
                       const std::vector<double>& out, const std::vector<int>& win, int* win_start, int* win_end,
                       double* raw_log_g, long long raw_capacity, long long* raw_offset)
{
  long long pos = 0;
  std::vector<int> slot(static_cast<size_t>(n), -1);
  for (size_t i = 0; i < prep.main.size(); ++i) slot[prep.main_problem[i]] = static_cast<int>(i);
  long long wpos = 0;
  for (int p = 0; p < n; ++p) {
    if (raw_offset != nullptr) raw_offset[p] = pos;
    const int I = problems[p].intervals;
    for (int b = 0; b < I; ++b) {
      const bool have = !prep.starts[p].empty();
      if (win_start != nullptr) win_start[wpos + b] = have ? prep.starts[p][b] : 0;
      if (win_end != nullptr) win_end[wpos + b] = have ? prep.ends[p][b] : -1;
    }
    wpos += I;
    if (slot[p] < 0) continue;
    const MainDesc& d = prep.main[slot[p]];
    std::vector<double> dense;
    for (int b = 0; b < d.I; ++b) {
      dense_window(d, out, win, b, dense);
      if (pos + static_cast<long long>(dense.size()) > raw_capacity) return fail(ex, WLG_ERR_CAPACITY, "raw output");
      if (raw_log_g != nullptr) std::memcpy(raw_log_g + pos, dense.data(), dense.size() * sizeof(double));
      pos += static_cast<long long>(dense.size());
    }
  }
  return WLG_OK;
}

}  // namespace

extern "C" {

wlg_status wlg_solve(wlg_context* ctx, const wlg_problem* problems, int n, wlg_result* results, int* energies,
                     double* log_g, long long capacity)
{
  return wlg_solve_couplings(ctx, problems, n, nullptr, results, energies, log_g, capacity);
}

wlg_status wlg_solve_couplings(wlg_context* ctx, const wlg_problem* problems, int n, const signed char* couplings,
                               wlg_result* results, int* energies, double* log_g, long long capacity)
{
  return wlg::guarded([&]() -> wlg_status {
    if (ctx == nullptr || (n > 0 && (problems == nullptr || results == nullptr))) return WLG_ERR_INVALID;
    cudaSetDevice(ctx->device);
    std::vector<MainResult> mres;
    Prepared prep;
    std::vector<double> out;
    std::vector<int> win;
    ContextExec ex(ctx);
    wlg_status st = run_batch(ex, problems, n, results, mres, prep, out, win, reinterpret_cast<const int8_t*>(couplings));
    keep_stats(ctx, ex);
    if (st != WLG_OK) return st;
    return stitch_all(ctx, prep, out, win, results, energies, log_g, capacity);
  });
}

wlg_status wlg_prerun(wlg_context* ctx, const wlg_problem* problems, int n, unsigned char* seen,
                      signed char* couplings, int* found, int* found_energy, signed char* lattices)
{
  return wlg::guarded([&]() -> wlg_status {
    if (ctx == nullptr || n < 0 || (n > 0 && problems == nullptr)) return WLG_ERR_INVALID;
    cudaSetDevice(ctx->device);
    std::vector<wlg_result> res(static_cast<size_t>(n));
    PreOut po;
    ContextExec ex(ctx);
    const wlg_status st = run_prerun(ex, problems, n, res.data(), po);
    keep_stats(ctx, ex);
    if (st != WLG_OK) return st;
    long long ob = 0;  // bins so far
    for (int p = 0; p < n; ++p) {
      const PreDesc& d = po.pd[p];
      if (seen != nullptr) std::memcpy(seen + d.off_seen, po.seen.data() + d.off_seen, static_cast<size_t>(4 * d.N + 1));
      if (couplings != nullptr)
        std::memcpy(couplings + d.off_J, po.J8.data() + d.off_J, static_cast<size_t>(2 * d.N));
      if (lattices != nullptr)
        std::memcpy(lattices + d.off_found, po.found.data() + d.off_found, static_cast<size_t>(d.n_int) * d.N);
      for (int b = 0; b < d.n_int; ++b) {
        if (found != nullptr) found[ob + b] = po.fflag[d.off_fflag + b];
        if (found_energy != nullptr) found_energy[ob + b] = po.fflag[d.off_fflag + d.n_int + b];
      }
      ob += d.n_int;
    }
    return WLG_OK;
  });
}

wlg_status wlg_mainrun(wlg_context* ctx, const wlg_problem* problems, int n, const unsigned char* seen,
                       const signed char* couplings, const int* found, const int* found_energy,
                       const signed char* lattices, double time_limit_s, wlg_result* results, int* energies,
                       double* log_g, long long capacity)
{
  return wlg::guarded([&]() -> wlg_status {
    if (ctx == nullptr || n < 0 ||
        (n > 0 && (problems == nullptr || results == nullptr || seen == nullptr || couplings == nullptr ||
                   found == nullptr || found_energy == nullptr || lattices == nullptr)))
      return WLG_ERR_INVALID;
    cudaSetDevice(ctx->device);
    ContextExec ex(ctx);
    ex.h2d = ex.d2h = 0;
    ex.launches = 0;
    ex.main_forms = 0;
    ex.t_pre = ex.t_main = 0;
    ex.t_handoff = 0;
    PreOut po;
    std::string err;
    wlg_status st = given_prerun(problems, n, results, seen, couplings, found, found_energy, lattices, po, err);
    if (st != WLG_OK) {
      ctx->err = err;
      return st;
    }
    Prepared prep;
    Handoff ho;
    std::vector<MainResult> mres;
    std::vector<double> out;
    std::vector<int> win;
    st = handoff(ex, problems, n, results, po, prep, ho);
    if (st == WLG_OK) st = run_main(ex, results, prep, ho, mres, out, win, time_limit_s);
    keep_stats(ctx, ex);
    if (st != WLG_OK) return st;
    return stitch_all(ctx, prep, out, win, results, energies, log_g, capacity);
  });
}

wlg_status wlg_handoff(const wlg_problem* problems, int n, const unsigned char* seen, const signed char* couplings,
                       const int* found, const int* found_energy, const signed char* lattices, int* status,
                       int* e_min, int* e_max, unsigned char* spectrum, int* win_start, int* win_end,
                       signed char* start_lattices)
{
  return wlg::guarded([&]() -> wlg_status {
    if (n < 0 || (n > 0 && (problems == nullptr || seen == nullptr || couplings == nullptr || found == nullptr ||
                            found_energy == nullptr || lattices == nullptr || status == nullptr || e_min == nullptr ||
                            e_max == nullptr || spectrum == nullptr || win_start == nullptr || win_end == nullptr ||
                            start_lattices == nullptr)))
      return WLG_ERR_INVALID;
    std::vector<wlg_result> res(static_cast<size_t>(n));
    PreOut po;
    std::string err;
    wlg_status st = given_prerun(problems, n, res.data(), seen, couplings, found, found_energy, lattices, po, err);
    if (st != WLG_OK) return st;
    HostExec ex;
    Prepared prep;
    Handoff ho;
    if ((st = handoff(ex, problems, n, res.data(), po, prep, ho)) != WLG_OK) return st;
    std::vector<int> main_of(static_cast<size_t>(n), -1);
    for (size_t i = 0; i < prep.main.size(); ++i) main_of[prep.main_problem[i]] = static_cast<int>(i);
    long long ow = 0, ol = 0, os = 0;
    for (int p = 0; p < n; ++p) {
      const wlg_problem& q = problems[p];
      const int N = q.X * q.Y, I = q.intervals;
      std::fill(spectrum + os, spectrum + os + 4 * N + 1, 0);
      std::fill(win_start + ow, win_start + ow + I, 0);
      std::fill(win_end + ow, win_end + ow + I, 0);
      std::fill(start_lattices + ol, start_lattices + ol + static_cast<long long>(I) * N, 0);
      e_min[p] = e_max[p] = 0;
      if (main_of[p] < 0) {
        status[p] = res[p].status != WLG_OK ? res[p].status : WLG_ERR_NO_LATTICE;
      } else {
        const MainDesc& d = prep.main[main_of[p]];
        status[p] = WLG_OK;
        e_min[p] = d.e_min;
        e_max[p] = d.e_max;
        const int g = 1 << d.lg;
        for (int c = 0; c * g <= d.e_max - d.e_min; ++c)
          if ((ho.maskw[d.off_mask + (c >> 5)] >> (c & 31)) & 1u) spectrum[os + d.e_min + c * g + 2 * N] = 1;
        for (int b = 0; b < I; ++b) {
          win_start[ow + b] = ho.win[d.off_win + b];
          win_end[ow + b] = ho.win[d.off_win + I + b];
          const uint32_t* w = ho.latw.data() + d.off_lat + static_cast<long long>(b) * d.nwL;
          for (int s = 0; s < N; ++s) {
            int wd = 0, bit = 0;
            wlg::lattice_bit(q.X, q.Y, s, wd, bit);
            start_lattices[ol + static_cast<long long>(b) * N + s] = ((w[wd] >> bit) & 1u) ? -1 : 1;
          }
        }
      }
      ow += I;
      ol += static_cast<long long>(I) * N;
      os += 4 * N + 1;
    }
    return WLG_OK;
  });
}

wlg_status wlg_context_autotune(wlg_context* ctx, const wlg_problem* problems, int n, int max_outer,
                                wlg_tuning* out, int cap, int* n_out)
{
  return wlg::guarded([&]() -> wlg_status {
    if (ctx == nullptr || n <= 0 || problems == nullptr || max_outer <= 0 || (cap > 0 && out == nullptr))
      return WLG_ERR_INVALID;
    cudaSetDevice(ctx->device);
    std::vector<wlg_problem> probs(problems, problems + n);
    for (wlg_problem& q : probs) q.max_outer = max_outer;
    std::vector<wlg_result> res(static_cast<size_t>(n));
    ContextExec ex(ctx);
    Prepared prep;
    Handoff ho;
    wlg_status st = wlg::prepare_batch(ex, probs.data(), n, res.data(), prep, ho);
    if (st != WLG_OK) {
      ctx->err = ex.err;
      return st;
    }
    // problems by (form, team size), as run_main groups them
    std::map<std::pair<int, int>, std::vector<int>> groups;
    for (size_t i = 0; i < prep.main.size(); ++i) {
      const MainDesc& d = prep.main[i];
      groups[{kernel_variant(d, d.team), d.team}].push_back(static_cast<int>(i));
    }
    std::map<std::pair<int, int>, int> best;
    std::vector<wlg_tuning> found;
    for (const auto& [key, idx] : groups) {
      Prepared sub;
      for (int i : idx) {
        sub.main.push_back(prep.main[i]);
        sub.main_problem.push_back(prep.main_problem[i]);
      }
      const int limit = key.second <= 256 ? 256 / key.second : 1;
      wlg_tuning t{key.first & 3, key.second, 1, 0.0f, 0};
      float best_ms = 0.0f;
      for (int c = 1; c <= limit; c *= 2) {
        const std::map<std::pair<int, int>, int> force{{key, c}};
        ex.per_cta = &force;
        std::vector<MainResult> mres;
        std::vector<double> out_host;
        std::vector<int> win_host;
        Prepared run = sub;
        st = run_main(ex, res.data(), run, ho, mres, out_host, win_host, 0.0);
        if (st != WLG_OK) {
          ctx->err = ex.err;
          return st;
        }
        if (c == 1 || ex.t_main < best_ms) {
          best_ms = ex.t_main;
          t.per_cta = c;
        }
        ++t.candidates;
      }
      t.main_ms = best_ms;
      best[key] = t.per_cta;
      found.push_back(t);
    }
    for (const auto& [k, v] : best) ctx->tuned[k] = v;
    const int k = std::min(cap, static_cast<int>(found.size()));
    for (int i = 0; i < k; ++i) out[i] = found[i];
    if (n_out != nullptr) *n_out = static_cast<int>(found.size());
    return WLG_OK;
  });
}

wlg_status wlg_last_stats(const wlg_context* ctx, wlg_stats* out)
{
  if (ctx == nullptr || out == nullptr) return WLG_ERR_INVALID;
  out->pre_ms = ctx->t_pre;
  out->handoff_ms = ctx->t_handoff;
  out->main_ms = ctx->t_main;
  out->stitch_ms = ctx->t_stitch;
  out->h2d_bytes = ctx->h2d;
  out->d2h_bytes = ctx->d2h;
  out->kernel_launches = ctx->launches;
  out->main_forms = ctx->main_forms;
  return WLG_OK;
}

wlg_status wlg_last_main_times(const wlg_context* ctx, double* start_ms, double* end_ms, int cap, int* n_out)
{
  if (ctx == nullptr || n_out == nullptr || cap < 0) return WLG_ERR_INVALID;
  const int n = static_cast<int>(ctx->p_start_ms.size());
  *n_out = n;
  if (cap < n) return WLG_ERR_CAPACITY;
  for (int i = 0; i < n; ++i) {
    if (start_ms != nullptr) start_ms[i] = ctx->p_start_ms[i];
    if (end_ms != nullptr) end_ms[i] = ctx->p_end_ms[i];
  }
  return WLG_OK;
}

wlg_status wlg_class_log_probs(const int* energies, const double* log_g, const long long* offset, const int* count,
                               int n_classes, double prob, double* log_z, double* log_probs)
{
  return wlg::guarded([&]() -> wlg_status {
    if (n_classes <= 0 || prob <= 0 || prob >= 1 || energies == nullptr || log_g == nullptr) return WLG_ERR_INVALID;
    const double beta_n = 0.5 * std::log((1.0 - prob) / prob);
    std::vector<double> lz(static_cast<size_t>(n_classes));
    for (int c = 0; c < n_classes; ++c) {
      if (count[c] <= 0) return WLG_ERR_INVALID;
      double mx = -std::numeric_limits<double>::infinity();
      for (int i = 0; i < count[c]; ++i) {
        const long long k = offset[c] + i;
        mx = std::max(mx, log_g[k] - beta_n * energies[k]);
      }
      double s = 0;
      for (int i = 0; i < count[c]; ++i) {
        const long long k = offset[c] + i;
        s += std::exp(log_g[k] - beta_n * energies[k] - mx);
      }
      lz[c] = mx + std::log(s);
    }
    double mx = *std::max_element(lz.begin(), lz.end());
    double s = 0;
    for (double v : lz) s += std::exp(v - mx);
    const double lse = mx + std::log(s);
    for (int c = 0; c < n_classes; ++c) {
      if (log_z) log_z[c] = lz[c];
      if (log_probs) log_probs[c] = lz[c] - lse;
    }
    return WLG_OK;
  });
}

}  // extern "C"

// ----------------------------------------------- solve without allocating --

namespace wlg {
wlg_status noalloc_arena(void** out, size_t* bytes);
}

namespace {

// Device buffers carved in order out of the fixed arena of wlg_noalloc.cu.
struct ArenaExec final : Exec {
  unsigned char* base = nullptr;
  size_t cap = 0, used = 0;
  void* slot_ptr[kSlots] = {};
  size_t slot_cap[kSlots] = {};
  wlg_status buffer(Slot slot, size_t bytes, void** out) override
  {
    if (slot_ptr[slot] != nullptr && slot_cap[slot] >= bytes) {
      *out = slot_ptr[slot];
      return WLG_OK;
    }
    const size_t off = (used + 255) & ~size_t{255};
    if (off + bytes > cap) {
      err = "batch does not fit the " + std::to_string(cap >> 20) + " MiB no-allocation arena";
      return WLG_ERR_CAPACITY;
    }
    slot_ptr[slot] = base + off;
    slot_cap[slot] = bytes;
    used = off + bytes;
    *out = slot_ptr[slot];
    return WLG_OK;
  }
};

// Upper bound of the arena bytes a batch needs, from the problem parameters
// alone (windows of the full range [-2N, 2N], energy step 2), so oversized
// batches are rejected before anything runs.  This includes the global log g
// pool of the form-3 launches (run_main): one slice of L x team doubles per
// resident team, at most (problems + teams per CTA - 1) slices per launch (one
// launch per team size and lattice layout), counted for every problem whose
// full-range state would not fit shared memory (its real windows are never
// wider, so no form-3 problem is missed).
size_t noalloc_bound(const wlg_problem* probs, int n)
{
  auto pad = [](size_t x) { return (x + 255) & ~size_t{255}; };
  size_t pre_desc = 0, j8 = 0, seen = 0, found = 0, fflag = 0;
  size_t md = 0, order = 0, jw = 0, latw = 0, win = 0, mask = 0, out = 0, res = 0;
  // (team size, row layout) -> (form-3 problems, largest L): run_main's form-3 launches
  std::map<std::pair<int, bool>, std::pair<size_t, size_t>> pool;
  for (int p = 0; p < n; ++p) {
    const wlg_problem& q = probs[p];
    const size_t N = static_cast<size_t>(q.X) * q.Y, I = static_cast<size_t>(q.intervals);
    const size_t nwL = static_cast<size_t>(wlg::lattice_words(q.X, q.Y)), nbins = 2 * N + 1;
    MainDesc d{};
    d.X = q.X;
    d.Y = q.Y;
    d.N = static_cast<int>(N);
    d.I = q.intervals;
    d.L = static_cast<int>(nbins);
    d.nwL = static_cast<int>(nwL);
    d.nwM = static_cast<int>((nbins + 31) / 32);
    const int team = wlg::round32(q.intervals * q.walkers_per_interval);
    if (wlg::fit_form(d, team) == 3) {
      auto& e = pool[{team, wlg::lattice_rows(q.X, q.Y)}];
      e.first += 1;
      e.second = std::max(e.second, nbins);
    }
    pre_desc += sizeof(PreDesc);
    j8 += 2 * N;
    seen += 4 * N + 1;
    found += static_cast<size_t>(q.pre_intervals) * N;
    fflag += 2 * static_cast<size_t>(q.pre_intervals) * sizeof(int);
    md += sizeof(MainDesc);
    order += sizeof(int);
    jw += 2 * nwL * 4;
    latw += I * nwL * 4;
    win += 5 * I * sizeof(int);
    mask += (nbins + 31) / 32 * 4;
    out += I * nbins * sizeof(double);
    res += sizeof(MainResult);
  }
  size_t gpool = 0;
  for (const auto& [key, e] : pool) {
    const int team = key.first;
    const size_t per_cta_max = team <= 256 ? static_cast<size_t>(256 / team) : 1;
    gpool += (e.first + per_cta_max - 1) * e.second * static_cast<size_t>(team) * sizeof(double);
  }
  return pad(pre_desc) + pad(j8) + pad(seen) + pad(found) + pad(fflag) + pad(md) + pad(order) + pad(jw) + pad(latw) +
         pad(win) + pad(mask) + pad(out) + pad(res) + pad(64 * sizeof(int)) + pad(gpool);
}

}  // namespace

extern "C" {

wlg_status wlg_solve_raw_noalloc(const wlg_problem* problems, int n, wlg_result* results, int* win_start,
                                 int* win_end, double* raw_log_g, long long raw_capacity, long long* raw_offset,
                                 wlg_stream stream)
{
  return wlg::guarded([&]() -> wlg_status {
    if (n < 0 || (n > 0 && (problems == nullptr || results == nullptr))) return WLG_ERR_INVALID;
    ArenaExec ex;
    void* base = nullptr;
    wlg_status st = wlg::noalloc_arena(&base, &ex.cap);
    if (st != WLG_OK) return st;
    ex.base = static_cast<unsigned char*>(base);
    if (noalloc_bound(problems, n) > ex.cap) return WLG_ERR_CAPACITY;
    cudaGetDevice(&ex.device);
    ex.stream = wlg::as_stream(stream);
    std::vector<MainResult> mres;
    Prepared prep;
    std::vector<double> out;
    std::vector<int> win;
    st = run_batch(ex, problems, n, results, mres, prep, out, win);
    if (st != WLG_OK) return st;
    return raw_windows(ex, problems, n, prep, out, win, win_start, win_end, raw_log_g, raw_capacity, raw_offset);
  });
}

}  // extern "C"
