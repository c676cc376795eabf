// Serving loop (C++20): continuous batching of decoding requests over the
// batch engine's kernels.
//
// A request is one disorder sample; the server runs its four error classes
// (i, v, h, c) as four problems and retires the request with the classes'
// log-probabilities at the Nishimori temperature.  The loop runs in its own
// host thread:
//
//   admit   - pending requests whose worst-case device memory fits the
//             budget get arena blocks; an admission thread runs their
//             pre-run (one launch on its own stream) and the host hand-off
//             (prepare_batch, the batch engine's own code) while the loop
//             keeps launching epochs; then the loop gives them table slots
//             and uploads their main-run inputs;
//   launch  - every resident problem advances in "epochs": main-run launches
//             of at most `epoch_outer` outer iterations that suspend each
//             unfinished problem's state (walkers, histograms, log g, RNG
//             positions, window flags) in its arena block and resume it at the
//             next launch.  Problems are grouped by main-run form and team
//             size, one CUDA stream per group, two epochs in flight per group
//             so the device never waits for the host;
//   retire  - when an epoch's event completes, its snapshot of the result
//             table says which problems finished; their walker-0 log g is
//             copied back and stitched, and a request whose four classes are
//             done gets its class log-probabilities; a class whose pre-run
//             missed part of the spectrum goes back to admit at once, alone,
//             with a longer pre-run;
//   reclaim - a finished problem's block and slot are reused once no
//             in-flight epoch lists it any more.
//
// Requests that arrive while others run join the next epoch of their group,
// so their work overlaps on the device with everything resident.  A problem's
// trajectory depends only on its own streams and state, never on epoch
// boundaries or neighbours, so every result equals the batch engine's.  The
// kernels never wait on the host: all synchronisation is by stream order and
// events, and every launch ends after a bounded number of iterations.

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <bit>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <utility>
#include <vector>

#include "../../include/wlg.h"
#include "wlg_internal.h"
#include "wlg_batch.h"
#include "wlg_engine.h"

namespace {

using namespace wlg;
using Clock = std::chrono::steady_clock;

constexpr int kClasses = 4;
constexpr char kClassName[kClasses] = {'i', 'v', 'h', 'c'};
constexpr int kRing = 3;        // per-group launch buffers: two epochs in flight + one being built
constexpr int kMaxInFlight = 2;
constexpr int kSmemLimit = 227 * 1024;

// First-fit allocator over a device arena, 256-byte granules.
class Arena {
 public:
  void reset(size_t size)
  {
    free_.clear();
    free_[0] = size;
    used_ = 0;
  }
  bool alloc(size_t bytes, size_t* off)
  {
    bytes = round(bytes);
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second < bytes) continue;
      *off = it->first;
      const size_t rest = it->second - bytes, start = it->first + bytes;
      free_.erase(it);
      if (rest > 0) free_[start] = rest;
      used_ += bytes;
      return true;
    }
    return false;
  }
  void release(size_t off, size_t bytes)
  {
    bytes = round(bytes);
    used_ -= bytes;
    auto it = free_.emplace(off, bytes).first;
    auto nx = std::next(it);
    if (nx != free_.end() && it->first + it->second == nx->first) {
      it->second += nx->second;
      free_.erase(nx);
    }
    if (it != free_.begin()) {
      auto pv = std::prev(it);
      if (pv->first + pv->second == it->first) {
        pv->second += it->second;
        free_.erase(it);
      }
    }
  }
  size_t used() const { return used_; }

 private:
  static size_t round(size_t b) { return (b + 255) & ~size_t{255}; }
  std::map<size_t, size_t> free_;
  size_t used_ = 0;
};

// Pre-run buffers that grow on demand and are kept.
struct GrowExec final : Exec {
  void* p[kSlots] = {};
  size_t cap[kSlots] = {};
  ~GrowExec() override
  {
    for (void* q : p)
      if (q != nullptr) cudaFree(q);
  }
  wlg_status buffer(Slot slot, size_t bytes, void** out) override
  {
    if (bytes > cap[slot]) {
      if (p[slot] != nullptr) cudaFree(p[slot]);
      p[slot] = nullptr;
      cap[slot] = 0;
      const size_t want = std::max<size_t>(bytes + bytes / 4, 4096);
      const cudaError_t e = cudaMalloc(&p[slot], want);
      if (e != cudaSuccess) return fail(*this, WLG_ERR_OOM, cudaGetErrorString(e));
      cap[slot] = want;
    }
    *out = p[slot];
    return WLG_OK;
  }
};

// Arena block of one problem: saved state, walker-0 output, then the
// main-run inputs (couplings, start lattices, spectrum mask, windows).
struct BlockLayout {
  size_t state, out, J, lat, mask, win, bytes;
};

BlockLayout block_layout(int team, int I, int L, int nwL, int nwM)
{
  auto a8 = [](size_t x) { return (x + 7) & ~size_t{7}; };
  BlockLayout b{};
  size_t o = 0;
  b.state = o;
  o = a8(o + static_cast<size_t>(state_layout(team, I, nwL, L).bytes));
  b.out = o;
  o = a8(o + 8 * static_cast<size_t>(I) * L);
  b.J = o;
  o = a8(o + 4 * 2 * static_cast<size_t>(nwL));
  b.lat = o;
  o = a8(o + 4 * static_cast<size_t>(I) * nwL);
  b.mask = o;
  o = a8(o + 4 * static_cast<size_t>(nwM));
  b.win = o;
  o = a8(o + 4 * 5 * static_cast<size_t>(I));
  b.bytes = o;
  return b;
}

// Worst-case block of a request's problem from its parameters alone: windows
// of the full range [-2N, 2N] with energy step 2 bound L and the mask.
BlockLayout block_bound(const wlg_problem& q)
{
  const int N = q.X * q.Y;
  std::vector<int> s, e;
  int L = 2 * N + 1;
  if (make_windows(-2 * N, 2 * N, q.intervals, q.overlap, s, e) == WLG_OK) {
    L = 1;
    for (int b = 0; b < q.intervals; ++b) L = std::max(L, (e[b] - s[b]) / 2 + 1);
  }
  const int nbins = 2 * N + 1;
  return block_layout(round32(q.intervals * q.walkers_per_interval), q.intervals, L, lattice_words(q.X, q.Y),
                      (nbins + 31) / 32);
}

struct Problem {
  bool used = false;
  unsigned long long req = 0;
  int cls = 0;
  MainDesc d{};              // offsets absolute within the arena
  std::vector<int> win;      // windows (5 I) for stitching
  size_t off = 0, bytes = 0;  // arena block
  std::pair<int, int> group{-1, -1};  // (main-run form, team size)
  int ready_ev = -1;          // admission event the group streams wait for
  long long last_epoch = -1;  // last epoch of its group that lists it
  bool done = false;
};

struct Request {
  wlg_problem q{};
  std::vector<int8_t> J;  // given class-'i' couplings (2N), empty: drawn
  wlg_decoded out{};
  int remaining = kClasses;              // classes not yet done
  unsigned todo = (1u << kClasses) - 1;  // classes of the next admission
  bool part = false;                     // a pending re-admission of one class of an active request
  int pre_iterations[kClasses] = {};     // per class; 0: q.pre_iterations
  int attempts[kClasses] = {};           // re-admissions so far, per class
  int status[kClasses] = {};
  std::vector<std::pair<int, double>> curve[kClasses];
  int pre_iter(int c) const { return pre_iterations[c] > 0 ? pre_iterations[c] : q.pre_iterations; }
};

struct Epoch {
  long long id = 0;
  cudaEvent_t ev = nullptr;
  std::vector<int> slots;
  int buf = 0;
};

struct Group {
  int form = 0, team = 32;
  cudaStream_t stream = nullptr;
  std::vector<int> members;  // resident, unfinished slots
  std::deque<Epoch> inflight;
  long long next_id = 0, completed = -1;
  std::vector<char> waited;  // per admission event: already waited on
  int* d_order[kRing] = {};
  int* d_next[kRing] = {};
  int* h_order[kRing] = {};
  MainResult* h_snap[kRing] = {};
  cudaEvent_t ev[kRing] = {};
};

// One admission: requests with reserved arena blocks, prepared (pre-run +
// hand-off) by the admission thread while the loop keeps launching epochs.
struct AdmitJob {
  std::vector<std::pair<unsigned long long, Request>> batch;
  std::vector<std::pair<int, int>> who;  // per problem: (index in batch, class)
  std::vector<size_t> block_off;
  std::vector<BlockLayout> bound;
  std::vector<wlg_problem> qs;
  std::vector<int8_t> J;             // given couplings in problem order (empty: all drawn)
  std::vector<unsigned char> given;  // per problem
  std::vector<wlg_result> res;
  Prepared prep;
  Handoff ho;
  wlg_status st = WLG_OK;
  std::string err;
  bool done = false;  // under wlg_server::amu
};

}  // namespace

struct wlg_server {
  int device = 0;
  wlg_server_config cfg{};
  Clock::time_point t0;
  std::thread th;
  std::atomic<bool> stop{false};

  // shared with callers (under mu)
  mutable std::mutex mu;
  std::condition_variable cv_in, cv_out;
  std::deque<std::pair<unsigned long long, Request>> incoming;
  std::deque<wlg_decoded> finished;
  unsigned long long next_id = 1;
  wlg_server_stats stats{};
  std::string err;

  // owned by the loop thread
  bool fatal = false;
  cudaStream_t s_pre = nullptr, s_copy = nullptr;
  unsigned char* arena_dev = nullptr;
  Arena arena;
  MainDesc* d_desc = nullptr;
  MainResult* d_res = nullptr;
  std::vector<Problem> probs;
  std::vector<int> free_slots;
  int max_slot = 0;  // 1 + the highest slot in use
  std::map<std::pair<int, int>, Group> groups;
  std::map<unsigned long long, Request> active;
  std::deque<std::pair<unsigned long long, Request>> pending;
  std::vector<cudaEvent_t> admit_ev;
  std::vector<int> reclaim;  // finished slots waiting for their epochs
  std::unique_ptr<GrowExec> pre;  // used by the admission thread only
  std::unique_ptr<WorkerPool> apool;  // host workers of the admission's hand-off
  int sms = 1;

  // admission thread: pre-run + hand-off of one job at a time
  std::thread admitter;
  std::mutex amu;
  std::condition_variable acv;
  AdmitJob* a_todo = nullptr;
  bool a_stop = false;
  std::unique_ptr<AdmitJob> job;  // the loop's job in flight, if any

  double now_ms() const { return std::chrono::duration<double, std::milli>(Clock::now() - t0).count(); }
  void loop();
  bool admit();
  void finish_admission(AdmitJob& j);
  void admit_worker();
  bool launch();
  bool retire();
  bool do_reclaim();
  void complete(unsigned long long id, Request& r);
  void class_done(unsigned long long id, int cls, int status, long long outer,
                  std::vector<std::pair<int, double>>&& curve);
  void fail_all(const std::string& why);
  wlg_status setup();
  void teardown();
};

namespace {

bool cuda_ok(cudaError_t e) { return e == cudaSuccess; }

}  // namespace

wlg_status wlg_server::setup()
{
  if (!cuda_ok(cudaSetDevice(device))) return WLG_ERR_CUDA;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  if (!cuda_ok(cudaStreamCreateWithFlags(&s_pre, cudaStreamNonBlocking))) return WLG_ERR_CUDA;
  if (!cuda_ok(cudaStreamCreateWithFlags(&s_copy, cudaStreamNonBlocking))) return WLG_ERR_CUDA;
  if (!cuda_ok(cudaMalloc(&arena_dev, cfg.mem_budget_bytes))) return WLG_ERR_OOM;
  arena.reset(cfg.mem_budget_bytes);
  const size_t n = static_cast<size_t>(cfg.max_resident);
  if (!cuda_ok(cudaMalloc(&d_desc, n * sizeof(MainDesc)))) return WLG_ERR_OOM;
  if (!cuda_ok(cudaMalloc(&d_res, n * sizeof(MainResult)))) return WLG_ERR_OOM;
  probs.assign(n, Problem{});
  free_slots.clear();
  for (int s = cfg.max_resident - 1; s >= 0; --s) free_slots.push_back(s);
  pre = std::make_unique<GrowExec>();
  pre->device = device;
  pre->stream = s_pre;
  apool = std::make_unique<WorkerPool>(static_cast<int>(std::min(8u, std::max(1u, std::thread::hardware_concurrency()))));
  pre->pool = apool.get();
  stats.bytes_budget = static_cast<long long>(cfg.mem_budget_bytes);
  return WLG_OK;
}

void wlg_server::teardown()
{
  cudaSetDevice(device);
  for (auto& [k, g] : groups) {
    if (g.stream != nullptr) cudaStreamSynchronize(g.stream);
    for (int b = 0; b < kRing; ++b) {
      cudaFree(g.d_order[b]);
      cudaFree(g.d_next[b]);
      cudaFreeHost(g.h_order[b]);
      cudaFreeHost(g.h_snap[b]);
      if (g.ev[b] != nullptr) cudaEventDestroy(g.ev[b]);
    }
    if (g.stream != nullptr) cudaStreamDestroy(g.stream);
  }
  groups.clear();
  if (s_pre != nullptr) cudaStreamSynchronize(s_pre);
  if (s_copy != nullptr) cudaStreamSynchronize(s_copy);
  for (cudaEvent_t e : admit_ev) cudaEventDestroy(e);
  admit_ev.clear();
  pre.reset();
  apool.reset();
  cudaFree(d_desc);
  cudaFree(d_res);
  cudaFree(arena_dev);
  d_desc = nullptr;
  d_res = nullptr;
  arena_dev = nullptr;
  if (s_pre != nullptr) cudaStreamDestroy(s_pre);
  if (s_copy != nullptr) cudaStreamDestroy(s_copy);
  s_pre = s_copy = nullptr;
}

void wlg_server::fail_all(const std::string& why)
{
  fatal = true;
  {
    std::lock_guard<std::mutex> lk(mu);
    err = why;
  }
  auto retire_failed = [&](Request& r) {
    r.out.status = WLG_ERR_CUDA;
    r.out.done_ms = now_ms();
    std::lock_guard<std::mutex> lk(mu);
    finished.push_back(r.out);
    ++stats.completed;
  };
  // a re-admitted class's entry (part) belongs to a request in `active`,
  // which retires once
  for (auto& [id, r] : active) retire_failed(r);
  active.clear();
  for (auto& [id, r] : pending)
    if (!r.part) retire_failed(r);
  pending.clear();
  if (job) {  // an admission in flight: its thread reads only the job's copies of the parameters
    for (auto& [id, r] : job->batch)
      if (!r.part) retire_failed(r);
    job->batch.clear();
  }
  cv_out.notify_all();
}

void wlg_server::complete(unsigned long long id, Request& r)
{
  r.out.status = WLG_OK;
  for (int c = 0; c < kClasses; ++c)
    if (r.status[c] != WLG_OK) {
      r.out.status = r.status[c];
      break;
    }
  for (int c = 0; c < kClasses; ++c) r.out.log_z[c] = r.out.log_probs[c] = std::nan("");
  if (r.out.status == WLG_OK) {
    std::vector<int> E;
    std::vector<double> G;
    long long off[kClasses];
    int cnt[kClasses];
    for (int c = 0; c < kClasses; ++c) {
      off[c] = static_cast<long long>(E.size());
      cnt[c] = static_cast<int>(r.curve[c].size());
      for (const auto& [e, g] : r.curve[c]) {
        E.push_back(e);
        G.push_back(g);
      }
    }
    const wlg_status st =
      wlg_class_log_probs(E.data(), G.data(), off, cnt, kClasses, r.q.prob, r.out.log_z, r.out.log_probs);
    if (st != WLG_OK) r.out.status = st;
  }
  r.out.id = id;
  r.out.done_ms = now_ms();
  {
    std::lock_guard<std::mutex> lk(mu);
    finished.push_back(r.out);
    ++stats.completed;
  }
  cv_out.notify_all();
}

void wlg_server::class_done(unsigned long long id, int cls, int status, long long outer,
                            std::vector<std::pair<int, double>>&& curve)
{
  auto it = active.find(id);
  if (it == active.end()) return;
  Request& r = it->second;
  r.status[cls] = status;
  r.out.outer_iterations[cls] = outer;
  r.curve[cls] = std::move(curve);
  // A class whose pre-run missed part of the spectrum (a walker later found a
  // new energy, or a window got no start lattice) is re-admitted at once, on
  // its own, with twice the pre-run iterations, while the request's other
  // classes keep running: a deterministic function of the request, so the
  // result equals the batch engine's for that larger pre-run.  (The
  // reference aborts the whole run instead.)
  if ((status == WLG_ERR_NEW_ENERGY || status == WLG_ERR_NO_LATTICE) && r.attempts[cls] < cfg.max_readmit) {
    r.pre_iterations[cls] = static_cast<int>(std::min(2 * static_cast<long long>(r.pre_iter(cls)), 1ll << 30));
    r.attempts[cls] += 1;
    r.status[cls] = WLG_OK;
    r.curve[cls].clear();
    r.out.readmissions = std::max(r.out.readmissions, r.attempts[cls]);
    {
      std::lock_guard<std::mutex> lk(mu);
      ++stats.readmitted;
    }
    Request c;  // what the admission reads: parameters, couplings, this class's pre-run length
    c.q = r.q;
    c.J = r.J;
    c.todo = 1u << cls;
    c.part = true;
    std::copy(r.pre_iterations, r.pre_iterations + kClasses, c.pre_iterations);
    pending.emplace_front(id, std::move(c));
    return;  // the class stays outstanding in r.remaining
  }
  if (--r.remaining > 0) return;
  complete(id, r);
  active.erase(it);
}

// Pending requests -> reserved arena blocks -> the admission thread; a
// prepared job -> uploads -> groups.
bool wlg_server::admit()
{
  bool any = false;
  if (job) {
    bool ready;
    {
      std::lock_guard<std::mutex> lk(amu);
      ready = job->done;
    }
    if (!ready) return false;
    std::unique_ptr<AdmitJob> j = std::move(job);
    finish_admission(*j);
    any = true;
    if (fatal) return true;
  }
  if (pending.empty()) return any;
  auto nj = std::make_unique<AdmitJob>();
  std::vector<std::pair<unsigned long long, Request>>& batch = nj->batch;
  std::vector<size_t>& block_off = nj->block_off;
  std::vector<BlockLayout>& bound = nj->bound;
  while (!pending.empty() && static_cast<int>(batch.size()) < cfg.max_prerun_batch &&
         static_cast<int>(free_slots.size()) >= kClasses * static_cast<int>(batch.size() + 1)) {
    const Request& front = pending.front().second;
    const BlockLayout bl = block_bound(front.q);
    const int nc = std::popcount(front.todo);
    size_t offs[kClasses];
    int got = 0;
    for (; got < nc; ++got)
      if (!arena.alloc(bl.bytes, &offs[got])) break;
    if (got < nc) {
      for (int c = 0; c < got; ++c) arena.release(offs[c], bl.bytes);
      if (active.empty() && batch.empty() && reclaim.empty()) {  // can never fit
        auto [id, r] = std::move(pending.front());
        pending.pop_front();
        r.out.id = id;
        r.out.status = WLG_ERR_OOM;
        r.out.done_ms = now_ms();
        std::lock_guard<std::mutex> lk(mu);
        finished.push_back(r.out);
        ++stats.completed;
        cv_out.notify_all();
        continue;
      }
      break;
    }
    for (int c = 0, j = 0; c < kClasses; ++c)
      if ((front.todo >> c) & 1u) {
        block_off.push_back(offs[j++]);
        bound.push_back(bl);
        nj->who.emplace_back(static_cast<int>(batch.size()), c);
      }
    batch.push_back(std::move(pending.front()));
    pending.pop_front();
  }
  if (batch.empty()) return any;
  const int n = static_cast<int>(nj->who.size());
  nj->qs.resize(static_cast<size_t>(n));
  for (int k = 0; k < n; ++k) {
    const auto [i, c] = nj->who[k];
    const Request& r = batch[i].second;
    nj->qs[k] = r.q;
    nj->qs[k].error_class = kClassName[c];
    nj->qs[k].pre_iterations = r.pre_iter(c);
  }
  bool any_given = false;
  for (const auto& [id, r] : batch) any_given |= !r.J.empty();
  if (any_given)
    for (int k = 0; k < n; ++k) {
      const Request& r = batch[nj->who[k].first].second;
      const size_t twoN = 2 * static_cast<size_t>(r.q.X) * r.q.Y;
      if (r.J.empty())
        nj->J.insert(nj->J.end(), twoN, 1);
      else
        nj->J.insert(nj->J.end(), r.J.begin(), r.J.end());
      nj->given.push_back(r.J.empty() ? 0 : 1);
    }
  nj->res.resize(static_cast<size_t>(n));
  job = std::move(nj);
  {
    std::lock_guard<std::mutex> lk(amu);
    a_todo = job.get();
  }
  acv.notify_all();
  return true;
}

void wlg_server::admit_worker()
{
  cudaSetDevice(device);
  for (;;) {
    AdmitJob* j = nullptr;
    {
      std::unique_lock<std::mutex> lk(amu);
      acv.wait(lk, [&] { return a_stop || a_todo != nullptr; });
      if (a_todo == nullptr) return;  // stopping with nothing to do
      j = a_todo;
      a_todo = nullptr;
    }
    j->st = prepare_batch(*pre, j->qs.data(), static_cast<int>(j->qs.size()), j->res.data(), j->prep, j->ho,
                          j->J.empty() ? nullptr : j->J.data(), j->given.empty() ? nullptr : j->given.data());
    j->err = pre->err;
    std::lock_guard<std::mutex> lk(amu);
    j->done = true;
  }
}

// A prepared job: blocks, uploads, group membership, immediate results.
void wlg_server::finish_admission(AdmitJob& aj)
{
  std::vector<std::pair<unsigned long long, Request>>& batch = aj.batch;
  const std::vector<size_t>& block_off = aj.block_off;
  const std::vector<BlockLayout>& bound = aj.bound;
  const int n = static_cast<int>(aj.qs.size());
  std::vector<wlg_result>& res = aj.res;
  Prepared& prep = aj.prep;
  Handoff& ho = aj.ho;
  const wlg_status st = aj.st;
  if (batch.empty()) return;
  {
    std::lock_guard<std::mutex> lk(mu);
    ++stats.prerun_launches;
  }
  if (st != WLG_OK) {
    for (size_t k = 0; k < block_off.size(); ++k) arena.release(block_off[k], bound[k].bytes);
    for (auto& [id, r] : batch)
      if (!r.part) active.emplace(id, std::move(r));
    fail_all("pre-run: " + aj.err);
    return;
  }
  for (auto& [id, r] : batch)
    if (!r.part) active.emplace(id, std::move(r));
  // which batch problems reach the main run
  std::vector<int> main_of(static_cast<size_t>(n), -1);
  for (size_t i = 0; i < prep.main.size(); ++i) main_of[prep.main_problem[i]] = static_cast<int>(i);
  cudaEvent_t ev = nullptr;
  if (!cuda_ok(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming))) {
    fail_all("event");
    return;
  }
  const int ev_index = static_cast<int>(admit_ev.size());
  admit_ev.push_back(ev);
  std::vector<unsigned char> host;
  for (int k = 0; k < n; ++k) {
    const unsigned long long id = batch[aj.who[k].first].first;
    const int cls = aj.who[k].second;
    const size_t boff = block_off[k];
    const BlockLayout& bb = bound[k];
    if (main_of[k] < 0) {  // no main run (no lattice for a window, empty window, ...)
      arena.release(boff, bb.bytes);
      class_done(id, cls, res[k].status != WLG_OK ? res[k].status : WLG_ERR_NO_LATTICE, 0, {});
      continue;
    }
    MainDesc d = prep.main[main_of[k]];
    const BlockLayout bl = block_layout(d.team, d.I, d.L, d.nwL, d.nwM);
    const int form = kernel_variant(d, d.team);  // form | kKernelRows
    if (team_bytes(d, form & 3, d.team) > kSmemLimit || bl.bytes > bb.bytes) {
      arena.release(boff, bb.bytes);
      class_done(id, cls, WLG_ERR_INVALID, 0, {});
      continue;
    }
    // inputs: J, lattices, mask, windows, in the block's layout
    host.assign(bl.bytes - bl.J, 0);
    std::memcpy(host.data() + (bl.J - bl.J), ho.Jw.data() + d.off_J, 4 * 2 * static_cast<size_t>(d.nwL));
    std::memcpy(host.data() + (bl.lat - bl.J), ho.latw.data() + d.off_lat, 4 * static_cast<size_t>(d.I) * d.nwL);
    std::memcpy(host.data() + (bl.mask - bl.J), ho.maskw.data() + d.off_mask, 4 * static_cast<size_t>(d.nwM));
    std::memcpy(host.data() + (bl.win - bl.J), ho.win.data() + d.off_win, 4 * 5 * static_cast<size_t>(d.I));
    const int slot = free_slots.back();
    free_slots.pop_back();
    max_slot = std::max(max_slot, slot + 1);
    Problem& pr = probs[slot];
    pr = Problem{};
    pr.used = true;
    pr.req = id;
    pr.cls = cls;
    pr.win.assign(ho.win.begin() + d.off_win, ho.win.begin() + d.off_win + 5 * d.I);
    pr.off = boff;
    pr.bytes = bb.bytes;
    pr.ready_ev = ev_index;
    d.off_J = static_cast<long long>((boff + bl.J) / 4);
    d.off_lat = static_cast<long long>((boff + bl.lat) / 4);
    d.off_mask = static_cast<long long>((boff + bl.mask) / 4);
    d.off_win = static_cast<long long>((boff + bl.win) / 4);
    d.off_out = static_cast<long long>((boff + bl.out) / 8);
    d.off_state = static_cast<long long>(boff + bl.state);
    d.epoch_outer = cfg.epoch_outer;
    pr.d = d;
    bool ok = cuda_ok(cudaMemcpyAsync(arena_dev + boff + bl.J, host.data(), host.size(), cudaMemcpyHostToDevice, s_pre));
    ok = ok && cuda_ok(cudaMemsetAsync(arena_dev + boff + bl.state, 0, 32, s_pre));  // state header: fresh
    ok = ok && cuda_ok(cudaMemcpyAsync(d_desc + slot, &pr.d, sizeof(MainDesc), cudaMemcpyHostToDevice, s_pre));
    ok = ok && cuda_ok(cudaMemsetAsync(d_res + slot, 0, sizeof(MainResult), s_pre));
    if (!ok) {
      fail_all("upload");
      return;
    }
    auto key = std::make_pair(form, d.team);
    Group& g = groups[key];
    if (g.stream == nullptr) {
      g.form = form;
      g.team = d.team;
      ok = cuda_ok(cudaStreamCreateWithFlags(&g.stream, cudaStreamNonBlocking));
      for (int b = 0; b < kRing && ok; ++b) {
        ok = cuda_ok(cudaMalloc(&g.d_order[b], sizeof(int) * static_cast<size_t>(cfg.max_resident))) &&
             cuda_ok(cudaMalloc(&g.d_next[b], sizeof(int))) &&
             cuda_ok(cudaMallocHost(&g.h_order[b], sizeof(int) * static_cast<size_t>(cfg.max_resident))) &&
             cuda_ok(cudaMallocHost(&g.h_snap[b], sizeof(MainResult) * static_cast<size_t>(cfg.max_resident))) &&
             cuda_ok(cudaEventCreateWithFlags(&g.ev[b], cudaEventDisableTiming));
      }
      if (!ok) {
        fail_all("group setup");
        return;
      }
    }
    pr.group = key;
    g.members.push_back(slot);
  }
  // everything above was enqueued on s_pre (the copies from pageable host
  // memory have left `host` when they return)
  if (!cuda_ok(cudaEventRecord(ev, s_pre))) {
    fail_all("event record");
    return;
  }
  std::lock_guard<std::mutex> lk(mu);
  stats.bytes_in_use = static_cast<long long>(arena.used());
}

// One epoch per group with resident problems and fewer than two in flight.
bool wlg_server::launch()
{
  bool any = false;
  if (cfg.fail_after_epochs > 0 && stats.epochs >= cfg.fail_after_epochs) {  // injected (testing)
    fail_all("injected failure after " + std::to_string(cfg.fail_after_epochs) + " epochs");
    return true;
  }
  for (auto& [key, g] : groups) {
    if (g.members.empty() || static_cast<int>(g.inflight.size()) >= kMaxInFlight) continue;
    const int n = static_cast<int>(g.members.size());
    const int buf = static_cast<int>(g.next_id % kRing);
    int bytes = 0;
    if (static_cast<int>(g.waited.size()) < static_cast<int>(admit_ev.size())) g.waited.resize(admit_ev.size(), 0);
    for (int s : g.members) {
      const Problem& pr = probs[s];
      bytes = std::max(bytes, team_bytes(pr.d, g.form & 3, g.team));
      if (!g.waited[pr.ready_ev]) {
        if (!cuda_ok(cudaStreamWaitEvent(g.stream, admit_ev[pr.ready_ev], 0))) {
          fail_all("stream wait");
          return true;
        }
        g.waited[pr.ready_ev] = 1;
      }
    }
    int per_cta = g.team <= 256 ? 256 / g.team : 1;
    per_cta = std::min(per_cta, kSmemLimit / bytes);
    per_cta = std::min(per_cta, n / (2 * sms));
    per_cta = std::max(per_cta, 1);
    const int cap = main_batch_capacity(g.form, g.team * per_cta, bytes * per_cta);
    if (cap <= 0) {
      fail_all("main-run configuration does not fit an SM");
      return true;
    }
    const int grid = std::min(cap, (n + per_cta - 1) / per_cta);
    std::copy(g.members.begin(), g.members.end(), g.h_order[buf]);
    bool ok = cuda_ok(cudaMemcpyAsync(g.d_order[buf], g.h_order[buf], sizeof(int) * static_cast<size_t>(n),
                                      cudaMemcpyHostToDevice, g.stream));
    ok = ok && cuda_ok(cudaMemsetAsync(g.d_next[buf], 0, sizeof(int), g.stream));
    ok = ok && launch_main_batch(g.form, d_desc, g.d_order[buf], n, g.team, bytes, per_cta, grid, g.d_next[buf],
                                 nullptr, 0, reinterpret_cast<const uint32_t*>(arena_dev),
                                 reinterpret_cast<const uint32_t*>(arena_dev), reinterpret_cast<const int*>(arena_dev),
                                 reinterpret_cast<const uint32_t*>(arena_dev), reinterpret_cast<double*>(arena_dev),
                                 d_res, arena_dev, g.stream) == WLG_OK;
    ok = ok && cuda_ok(cudaMemcpyAsync(g.h_snap[buf], d_res, sizeof(MainResult) * static_cast<size_t>(max_slot),
                                       cudaMemcpyDeviceToHost, g.stream));
    ok = ok && cuda_ok(cudaEventRecord(g.ev[buf], g.stream));
    if (!ok) {
      fail_all("epoch launch");
      return true;
    }
    Epoch e;
    e.id = g.next_id++;
    e.ev = g.ev[buf];
    e.buf = buf;
    e.slots = g.members;
    for (int s : g.members) probs[s].last_epoch = e.id;
    g.inflight.push_back(std::move(e));
    any = true;
    std::lock_guard<std::mutex> lk(mu);
    ++stats.epochs;
    ++stats.main_launches;
  }
  return any;
}

// Completed epochs: finished problems -> outputs -> stitched curves.
bool wlg_server::retire()
{
  bool any = false;
  for (auto& [key, g] : groups) {
    while (!g.inflight.empty()) {
      Epoch& e = g.inflight.front();
      const cudaError_t q = cudaEventQuery(e.ev);
      if (q == cudaErrorNotReady) break;
      if (q != cudaSuccess) {
        fail_all(std::string("main run: ") + cudaGetErrorString(q));
        return true;
      }
      any = true;
      const MainResult* snap = g.h_snap[e.buf];
      std::vector<int> fin;
      for (int s : e.slots)
        if (!probs[s].done && snap[s].done != 0) fin.push_back(s);
      std::vector<std::vector<double>> outs(fin.size());
      for (size_t i = 0; i < fin.size(); ++i) {
        Problem& pr = probs[fin[i]];
        outs[i].assign(static_cast<size_t>(pr.d.I) * pr.d.L, 0.0);
        if (!cuda_ok(cudaMemcpyAsync(outs[i].data(), arena_dev + 8 * static_cast<size_t>(pr.d.off_out),
                                     outs[i].size() * sizeof(double), cudaMemcpyDeviceToHost, s_copy))) {
          fail_all("output copy");
          return true;
        }
      }
      if (!fin.empty() && !cuda_ok(cudaStreamSynchronize(s_copy))) {
        fail_all("output copy");
        return true;
      }
      for (size_t i = 0; i < fin.size(); ++i) {
        const int s = fin[i];
        Problem& pr = probs[s];
        pr.done = true;
        const MainResult r = snap[s];
        std::vector<std::pair<int, double>> curve;
        int status = r.status;
        if (status == WLG_OK) {
          status = stitched_curve(pr.d, outs[i].data(), pr.win.data(), curve, cfg.stitching);
        }
        class_done(pr.req, pr.cls, status, r.outer, std::move(curve));
        reclaim.push_back(s);
      }
      if (!fin.empty()) {
        auto& m = g.members;
        m.erase(std::remove_if(m.begin(), m.end(), [&](int s) { return probs[s].done; }), m.end());
      }
      g.completed = e.id;
      g.inflight.pop_front();
    }
  }
  return any;
}

// Finished problems whose last listing epoch completed give back their
// block and slot.
bool wlg_server::do_reclaim()
{
  if (reclaim.empty()) return false;
  bool any = false;
  std::vector<int> keep;
  for (int s : reclaim) {
    Problem& pr = probs[s];
    if (groups.at(pr.group).completed >= pr.last_epoch) {
      arena.release(pr.off, pr.bytes);
      pr = Problem{};
      free_slots.push_back(s);
      any = true;
    } else {
      keep.push_back(s);
    }
  }
  reclaim.swap(keep);
  while (max_slot > 0 && !probs[max_slot - 1].used) --max_slot;
  std::lock_guard<std::mutex> lk(mu);
  stats.bytes_in_use = static_cast<long long>(arena.used());
  return any;
}

void wlg_server::loop()
{
  if (!cuda_ok(cudaSetDevice(device))) {
    fail_all("cudaSetDevice");
    return;
  }
  while (!stop.load()) {
    {
      std::unique_lock<std::mutex> lk(mu);
      const bool idle = incoming.empty() && pending.empty() && active.empty() && reclaim.empty() && !job;
      if (idle) cv_in.wait_for(lk, std::chrono::milliseconds(2), [&] { return stop.load() || !incoming.empty(); });
      while (!incoming.empty()) {
        pending.push_back(std::move(incoming.front()));
        incoming.pop_front();
      }
    }
    if (stop.load()) break;
    if (fatal) {
      if (!pending.empty()) fail_all(err);
      std::this_thread::sleep_for(std::chrono::milliseconds(1));
      continue;
    }
    bool busy = false;
    try {
      busy |= retire();
      busy |= do_reclaim();
      busy |= admit();
      busy |= launch();
    } catch (const std::exception& ex) {
      fail_all(std::string("serving loop: ") + ex.what());
      continue;
    }
    long long resident = 0;
    for (const auto& [k, g] : groups) resident += static_cast<long long>(g.members.size());
    {
      std::lock_guard<std::mutex> lk(mu);
      stats.resident_problems = resident;
    }
    if (!busy) std::this_thread::sleep_for(std::chrono::microseconds(50));
  }
}

extern "C" {

wlg_status wlg_server_create(int device, const wlg_server_config* config, wlg_server** out)
{
  return wlg::guarded([&]() -> wlg_status {
    if (out == nullptr) return WLG_ERR_INVALID;
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count) return WLG_ERR_CUDA;
    auto s = std::make_unique<wlg_server>();
    s->device = device;
    if (config != nullptr) s->cfg = *config;
    if (s->cfg.mem_budget_bytes == 0) s->cfg.mem_budget_bytes = size_t{1} << 30;
    if (s->cfg.epoch_outer <= 0) s->cfg.epoch_outer = 4;
    if (s->cfg.max_prerun_batch <= 0) s->cfg.max_prerun_batch = 256;
    if (s->cfg.max_readmit == 0) s->cfg.max_readmit = 4;
    if (s->cfg.max_readmit < 0) s->cfg.max_readmit = 0;
    if (s->cfg.max_resident <= 0) s->cfg.max_resident = 8192;
    if (s->cfg.max_resident < kClasses) return WLG_ERR_INVALID;
    if (s->cfg.stitching != WLG_STITCH_REFERENCE && s->cfg.stitching != WLG_STITCH_DEFINED) return WLG_ERR_INVALID;
    s->t0 = Clock::now();
    const wlg_status st = s->setup();
    if (st != WLG_OK) {
      s->teardown();
      return st;
    }
    wlg_server* raw = s.release();
    raw->admitter = std::thread([raw] { raw->admit_worker(); });
    raw->th = std::thread([raw] { raw->loop(); });
    *out = raw;
    return WLG_OK;
  });
}

wlg_status wlg_server_submit(wlg_server* server, const wlg_problem* requests, int n, unsigned long long* ids)
{
  return wlg_server_submit_couplings(server, requests, n, nullptr, ids);
}

wlg_status wlg_server_submit_couplings(wlg_server* server, const wlg_problem* requests, int n,
                                       const signed char* couplings, unsigned long long* ids)
{
  return wlg::guarded([&]() -> wlg_status {
    if (server == nullptr || n < 0 || (n > 0 && (requests == nullptr || ids == nullptr))) return WLG_ERR_INVALID;
    std::vector<size_t> off_J(static_cast<size_t>(n) + 1, 0);
    for (int i = 0; i < n; ++i) {
      wlg_problem q = requests[i];
      q.error_class = 'i';
      if (check_problem(q) != WLG_OK || q.prob <= 0.0f || q.prob >= 1.0f) return WLG_ERR_INVALID;
      off_J[i + 1] = off_J[i] + 2 * static_cast<size_t>(q.X) * q.Y;
    }
    if (couplings != nullptr)
      for (size_t k = 0; k < off_J[n]; ++k)
        if (couplings[k] != 1 && couplings[k] != -1) return WLG_ERR_INVALID;
    std::lock_guard<std::mutex> lk(server->mu);
    const double t = server->now_ms();
    for (int i = 0; i < n; ++i) {
      Request r;
      r.q = requests[i];
      if (couplings != nullptr) r.J.assign(couplings + off_J[i], couplings + off_J[i + 1]);
      r.out.submit_ms = t;
      ids[i] = server->next_id++;
      r.out.id = ids[i];
      server->incoming.emplace_back(ids[i], std::move(r));
      ++server->stats.submitted;
    }
    server->cv_in.notify_all();
    return WLG_OK;
  });
}

wlg_status wlg_server_poll(wlg_server* server, wlg_decoded* out, int cap, int* n_out, int timeout_ms)
{
  return wlg::guarded([&]() -> wlg_status {
    if (server == nullptr || n_out == nullptr || cap < 0 || (cap > 0 && out == nullptr)) return WLG_ERR_INVALID;
    std::unique_lock<std::mutex> lk(server->mu);
    if (server->finished.empty() && timeout_ms > 0)
      server->cv_out.wait_for(lk, std::chrono::milliseconds(timeout_ms), [&] { return !server->finished.empty(); });
    int k = 0;
    while (k < cap && !server->finished.empty()) {
      out[k++] = server->finished.front();
      server->finished.pop_front();
    }
    *n_out = k;
    return WLG_OK;
  });
}

wlg_status wlg_server_stats_get(const wlg_server* server, wlg_server_stats* out)
{
  if (server == nullptr || out == nullptr) return WLG_ERR_INVALID;
  std::lock_guard<std::mutex> lk(server->mu);
  *out = server->stats;
  return WLG_OK;
}

const char* wlg_server_last_error(const wlg_server* server)
{
  if (server == nullptr) return "";
  std::lock_guard<std::mutex> lk(server->mu);
  return server->err.c_str();
}

wlg_status wlg_server_destroy(wlg_server* server)
{
  if (server == nullptr) return WLG_ERR_INVALID;
  server->stop.store(true);
  server->cv_in.notify_all();
  if (server->th.joinable()) server->th.join();
  {
    std::lock_guard<std::mutex> lk(server->amu);
    server->a_stop = true;
  }
  server->acv.notify_all();
  if (server->admitter.joinable()) server->admitter.join();
  server->teardown();
  delete server;
  return WLG_OK;
}

}  // extern "C"
