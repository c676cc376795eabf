/*
 * wlg.h — C ABI of the GB300 replica-exchange Wang-Landau engine.
 *
 * Two layers, both plain C (pointers, sizes, status codes; nothing throws):
 *
 *  1. Operators.  One entry point per device operation of the reference's
 *     kernel library (src/wl.cuh:24-514 of dfki-ric-quantum/qec_pf_wang_landau),
 *     on the reference's own data layout and argument meaning: int8 spins
 *     and couplings, per-walker offsets into dense uint64 histograms and
 *     double log g slices, caller-owned device buffers.  A maintainer swaps
 *     `wl::kernel<<<grid, block>>>(args...)` for `wlg_kernel(args..., stream)`;
 *     the engine picks the launch geometry.  Each comment names the reference
 *     interface the entry point replaces.
 *
 *  2. Engine.  Whole pre-run and main-run pipelines, the batched persistent
 *     form over many heterogeneous problems, and the serving queue.  All
 *     device memory is owned by the context.
 *
 * Device pointers are CUDA device addresses; `stream` is a cudaStream_t
 * (NULL = the legacy default stream).  Every call returns WLG_OK or an
 * error code; wlg_status_string() names it.
 */
#ifndef WLG_H_
#define WLG_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int wlg_status;
enum {
  WLG_OK = 0,
  WLG_ERR_INVALID = 1,      /* bad argument (sizes, boundary, overlap, ...) */
  WLG_ERR_CUDA = 2,         /* a CUDA runtime call or launch failed */
  WLG_ERR_NEW_ENERGY = 3,   /* a walker proposed an energy outside the pre-run spectrum */
  WLG_ERR_ENERGY_RANGE = 4, /* a start lattice's energy lies outside its window */
  WLG_ERR_NO_LATTICE = 5,   /* no pre-run lattice falls inside a window */
  WLG_ERR_OOM = 6,          /* device memory exhausted or over the configured budget */
  WLG_ERR_TIMEOUT = 7,      /* an iteration or time limit ended the run */
  WLG_ERR_STITCH = 8,       /* windows could not be stitched (no shared energies) */
  WLG_ERR_CAPACITY = 9,     /* an output buffer is too small */
  WLG_ERR_EMPTY_WINDOW = 10 /* window construction produced an empty window */
};

typedef void* wlg_stream;

const char* wlg_status_string(wlg_status s);
const char* wlg_version(void);

/* ===================================================================== *
 *  1. Operators (reference layout)                                       *
 * ===================================================================== */

/* Replaces wl::init_interactions (wl.cuh:95-100, wl.cu:364-386).
 * d_J: int8 [num_samples][2*lattice_size]; right bonds then down bonds. */
wlg_status wlg_init_interactions(int8_t* d_J, size_t lattice_size, int num_samples, int seed, float prob,
                                 wlg_stream stream);

/* Replaces wl::apply_x_horizontal_error / wl::apply_x_vertical_error
 * (wl.cuh:113-134, wl.cu:388-428) and the class switch of prerun.cu:56-75:
 * error_class 'h', 'v', 'c' (both) or anything else (no chain). */
wlg_status wlg_apply_error_class(int8_t* d_J, int X, int Y, int num_samples, char error_class, wlg_stream stream);

/* Replaces wl::init_lattice (wl.cuh:150-156, wl.cu:430-457).  The reference
 * installs each lattice's flip probability by an unordered float CAS; this
 * entry point fixes the winner to the lattice's first site, so the
 * probability is draw 0 of stream (seed+sample, 1) and spin s is -1 iff
 * draw s+1 of that stream lies below it. */
wlg_status wlg_init_lattice(int8_t* d_lattice, int X, int Y, size_t num_lattices, int seed, int walker_per_sample,
                            wlg_stream stream);

/* Replaces wl::calc_energy (wl.cuh:70-80, wl.cu:342-362); boundary 0 periodic, 1 open. */
wlg_status wlg_calc_energy(int boundary, int* d_energy, const int8_t* d_lattice, const int8_t* d_J,
                           const int* d_offset_lattice, int X, int Y, size_t num_lattices, int walker_per_sample,
                           wlg_stream stream);

/* Replaces wl::wang_landau_pre_run (wl.cuh:201-219, wl.cu:473-560).  Walkers
 * of a sample share its histogram; they advance round-synchronously (every
 * walker decides against the histogram of the previous round, then the
 * round's increments land, then each still-empty coarse bin stores the
 * lattice of the lowest-index walker that entered it).  A walker whose
 * proposal leaves [E_min, E_max] (the reference asserts) stops and keeps the
 * offending energy in d_energy.  At most 1024 walkers per sample. */
wlg_status wlg_wang_landau_pre_run(int* d_energy, int* d_flag_found_interval, int8_t* d_lattice,
                                   int8_t* d_found_interval_lattice, unsigned long long* d_histogram,
                                   uint64_t* d_seed_offset, const int8_t* d_J, const int* d_offset_lattice, int E_min,
                                   int E_max, int num_iterations, int X, int Y, int seed, unsigned num_intervals,
                                   int len_interval, size_t num_total_walker, int walker_per_sample, int boundary,
                                   wlg_stream stream);

/* Replaces wl::wang_landau (wl.cuh:473-497, wl.cu:1033-1175).  Walkers of
 * windows with cond == 1 walk inside their window with frozen histogram and
 * log g.  A walker that proposes an energy outside the pre-run spectrum
 * stops with d_found[t] = t + 1 and d_new_energy[t] = that energy, as in the
 * reference; otherwise d_found[t] = 0. */
wlg_status wlg_wang_landau(int8_t* d_lattice, const int8_t* d_J, unsigned long long* d_H, double* d_logG,
                           const double* d_factor, int* d_energy, int* d_new_energy, uint64_t* d_offset_iter,
                           int* d_found, const int* d_start, const int* d_end, const int* d_offset_histogram,
                           const int* d_offset_lattice, const int8_t* d_cond, const int8_t* d_spectrum,
                           const int* d_offset_spectrum, const int* d_cond_sample, int X, int Y, int num_iterations,
                           int num_lattices, int num_intervals, int walker_per_sample, int seed, int boundary,
                           wlg_stream stream);

/* Replaces wl::check_histogram (wl.cuh:393-405, wl.cu:892-967). */
wlg_status wlg_check_histogram(unsigned long long* d_H, double* d_factor, int8_t* d_cond,
                               const int* d_offset_histogram, const int* d_end, const int* d_start,
                               const int8_t* d_spectrum, const int* d_offset_spectrum, const int* d_cond_sample,
                               double alpha, int num_walker_total, int walker_per_sample, int num_intervals,
                               wlg_stream stream);

/* Replaces wl::calc_average_log_g followed by wl::redistribute_g_values
 * (wl.cuh:307-321 and :426-438, wl.cu:710-783 and :969-1031), fused: for
 * every flat window the walkers' log g becomes their mean, summed in walker
 * order (the reference's FP64 atomics have no fixed order).  The reference's
 * d_shared_logG scratch buffer is not needed. */
wlg_status wlg_average_log_g(double* d_logG, const int* d_start, const int* d_end, const int8_t* d_spectrum,
                             const int* d_offset_spectrum, const int8_t* d_cond, const int* d_offset_histogram,
                             const int* d_cond_sample, int num_samples, int walker_per_interval, int num_intervals,
                             wlg_stream stream);

/* Replaces wl::reset_d_cond (wl.cuh:261-265, wl.cu:596-613). */
wlg_status wlg_reset_cond(int8_t* d_cond, const double* d_factor, int total_intervals, double beta,
                          int walker_per_interval, wlg_stream stream);

/* Replaces wl::check_interactions_finished (wl.cuh:333-338, wl.cu:662-708):
 * d_cond_sample[k] = number of flat windows of sample k, or -1 when all are.
 * One kernel, no CUB scratch and no device synchronisation. */
wlg_status wlg_check_finished(int* d_cond_sample, const int8_t* d_cond, int num_intervals, int num_samples,
                              wlg_stream stream);

/* Replaces wl::replica_exchange (wl.cuh:360-372 and :510-514, wl.cu:785-890) with its
 * Fisher-Yates shuffle.  global_parity = 1 keeps the reference's parity on
 * the global window index (wl.cu:830); 0 uses the window index inside its
 * sample (identical when num_intervals is even). */
wlg_status wlg_replica_exchange(int* d_offset_lattice, int* d_energy, int* d_replica_indices,
                                uint64_t* d_offset_iter, const int* d_start, const int* d_end,
                                const int* d_offset_histogram, const int* d_cond_sample, const double* d_logG,
                                int even, int seed, int num_intervals, int walker_per_sample, int total_intervals,
                                int global_parity, wlg_stream stream);

/* Replace thrust::max_element at mainrun.cu:221-224, :273-276 and :342-344:
 * the maximum lands in the caller's device word d_out (no scratch). */
wlg_status wlg_max_int(const int* d_in, size_t n, int* d_out, wlg_stream stream);
wlg_status wlg_max_f64_nonneg(const double* d_in, size_t n, double* d_out, wlg_stream stream);

/* Diagnostic (no reference counterpart): n uniforms of the engine's stream
 * (key, subsequence, offset), the draws curand_init(key, subsequence, offset)
 * followed by curand_uniform would give. */
wlg_status wlg_uniforms(uint64_t key, uint64_t subseq, uint64_t offset, int n, float* d_out, wlg_stream stream);

/* ===================================================================== *
 *  2. Engine (context-owned device memory)                               *
 * ===================================================================== */

/* One Wang-Landau problem: disorder sample `sample` of a run seeded `seed`,
 * one error class.  The reference's `prerun -x X -y Y -p prob -n
 * pre_iterations -w pre_walkers -i pre_intervals -e class -r R -s seed`
 * followed by `mainrun -n iterations -a alpha -b beta -i intervals -w
 * walkers_per_interval -o overlap -c exchange_every ...` computes problems
 * sample = 0..R-1 (prerun.cu, mainrun.cu); every problem here reproduces the
 * reference's Philox streams for its (seed, sample). */
typedef struct {
  int X, Y;
  int boundary;           /* 0 periodic, 1 open */
  float prob;             /* bond flip probability (-p) */
  char error_class;       /* 'i' (or 'I'), 'h', 'v', 'c' (-e) */
  int seed;               /* run seed (-s); pre-run and main run use the same one */
  int sample;             /* disorder sample index within the run */
  int pre_walkers;        /* prerun -w, <= 1024 */
  int pre_intervals;      /* prerun -i */
  int pre_iterations;     /* prerun -n */
  int intervals;          /* mainrun -i */
  int walkers_per_interval; /* mainrun -w */
  float overlap;          /* mainrun -o */
  double alpha;           /* mainrun -a, flatness */
  double beta;            /* mainrun -b, final ln f */
  int iterations;         /* mainrun -n, WL steps per walker between flatness checks */
  int exchange_every;     /* mainrun -c */
  int exchange_mode;      /* 0: as the reference (its counter never advances, so exchange runs
                             only when exchange_every == 1); 1: every exchange_every iterations */
  int global_parity;      /* 1: exchange parity on the run-global window index (sample*intervals + b),
                             as the reference; 0: on the window index inside the problem */
  long long max_outer;    /* cap on outer iterations, 0 = none (the reference's --time_limit analogue) */
} wlg_problem;

typedef struct {
  int status;             /* WLG_OK, WLG_ERR_NEW_ENERGY, WLG_ERR_TIMEOUT, WLG_ERR_NO_LATTICE, ... */
  int new_energy;         /* the offending energy when status == WLG_ERR_NEW_ENERGY */
  long long outer_iterations;
  long long flips;        /* WL move attempts of the main run */
  long long pre_flips;    /* move attempts of the pre-run */
  int n_energies;         /* (E, log g) pairs of the stitched, normalised result */
  long long offset;       /* where they start in the caller's arrays */
} wlg_result;

typedef struct wlg_context wlg_context;

/* A context owns a CUDA stream and the device buffers of the engine on
 * `device`, four auxiliary streams on which a batch's launch groups (by
 * kernel form and team size) run side by side, joined back to the solve's
 * stream by events, and host worker threads for the per-problem host phases
 * (started on first use).  mem_budget_bytes = 0 means no limit beyond the
 * device's.  A context serves one host thread at a time (calls on it must
 * not overlap); use one context per thread for concurrent solves. */
wlg_status wlg_context_create(int device, size_t mem_budget_bytes, wlg_context** out);
wlg_status wlg_context_destroy(wlg_context* ctx);
/* Text of the last failure on ctx; valid until the next call on ctx. */
const char* wlg_context_last_error(const wlg_context* ctx);
/* Later solves on ctx run on `stream` (NULL: the context's own stream);
 * work already queued on the previous stream is finished first.  Solves
 * still return after their stream has reached the results. */
wlg_status wlg_context_set_stream(wlg_context* ctx, wlg_stream stream);

/* How stitching picks the energy where window i hands over to a later window
 * (result_handling.cpp:115-143): the shared energy whose slopes towards the
 * next energy agree best.  At a window's last energy there is no next one;
 * the reference reads past the end of its std::map there (:125-126), which
 * with libstdc++ yields a phantom successor whose energy is the window's
 * number of entries and whose value is ~0.  WLG_STITCH_REFERENCE (the
 * default) uses that phantom and so writes the reference's output bins;
 * WLG_STITCH_DEFINED skips energies without a successor. */
enum { WLG_STITCH_REFERENCE = 0, WLG_STITCH_DEFINED = 1 };
/* Stitching mode of later solves on ctx (wlg_solve, wlg_solve_couplings,
 * wlg_mainrun). */
wlg_status wlg_context_set_stitching(wlg_context* ctx, int mode);

/* Runs pre-run and main run of n problems as one batch on the GPU and
 * returns each problem's stitched, normalised log g (result_handling.cpp,
 * logsumexp = X*Y*ln 2): pairs (energies[i], log_g[i]) for i in
 * [offset, offset + n_energies).  capacity bounds the pair arrays
 * (4*X*Y + 1 per problem always suffices).  Per-problem failures are in
 * results[].status; the call itself fails only on invalid input or a
 * device error. */
wlg_status wlg_solve(wlg_context* ctx, const wlg_problem* problems, int n, wlg_result* results, int* energies,
                     double* log_g, long long capacity);

/* wlg_solve on given disorder (no counterpart in the reference, which
 * always draws it, wl.cu:364-386): couplings holds each problem's class-'i'
 * bond pattern, +-1, 2*X*Y entries per problem, problems concatenated, in
 * the reference's layout (right bonds [i*Y + j] then down bonds
 * [N + i*Y + j], wl.cu:77-87; the wrap-around bonds are unused with open
 * boundaries).  The problem's error_class still applies its logical chain
 * on top (prerun.cu:56-75); prob is not used for the bonds.  Every random
 * stream except the disorder is the one wlg_solve uses, so couplings equal
 * to the drawn ones give wlg_solve's results bit for bit.  NULL couplings:
 * wlg_solve. */
wlg_status wlg_solve_couplings(wlg_context* ctx, const wlg_problem* problems, int n, const signed char* couplings,
                               wlg_result* results, int* energies, double* log_g, long long capacity);

/* Syndromes of bond patterns (the decoding front-end; no counterpart in
 * the reference).  Plaquette (i, j) has corners (i, j), (i, j+1), (i+1, j),
 * (i+1, j+1) and is frustrated when
 * J_right(i, j) J_right(i+1, j) J_down(i, j) J_down(i, j+1) = -1; periodic
 * lattices have X*Y plaquettes (indices mod X, Y), open ones (X-1)*(Y-1),
 * row-major.  wlg_frustration writes syndrome[plaquette] = 1 for frustrated
 * plaquettes, else 0.  wlg_couplings_from_syndrome writes a +-1 pattern with
 * exactly the given frustrated plaquettes: every defect is moved along its
 * row to column 0 and then (periodic) along column 0 to plaquette (0, 0),
 * where defects cancel in pairs, or (open) out across the left edge; the
 * bonds crossed are -1.  A periodic syndrome with an odd number of defects
 * has no pattern (WLG_ERR_INVALID).  Decoding a syndrome: its pattern's
 * four error classes (wlg_server_submit_couplings) give the log-probability
 * of each logical class relative to the pattern. */
wlg_status wlg_frustration(int X, int Y, int boundary, const signed char* couplings, unsigned char* syndrome);
wlg_status wlg_couplings_from_syndrome(int X, int Y, int boundary, const unsigned char* syndrome,
                                       signed char* couplings);

/* Like wlg_solve, without stitching: the walker-0 log g of every window on
 * the reference's dense per-window layout (window b covers energies
 * win_start..win_end, zeros at unreachable energies), problem after
 * problem, window after window.  win_start/win_end receive intervals
 * entries per problem; raw_offset[p] gives problem p's first value. */
wlg_status wlg_solve_raw(wlg_context* ctx, const wlg_problem* problems, int n, wlg_result* results, int* win_start,
                         int* win_end, double* raw_log_g, long long raw_capacity, long long* raw_offset);

/* No counterpart in the reference.  wlg_solve_raw without a context and
 * without allocating any device memory, for callers that cannot call
 * cudaMalloc: a framework that owns the device's whole memory pool, a
 * latency-critical loop that cannot take an allocation's implicit
 * synchronisation, a deployment that forbids allocating after start-up.
 * Every device buffer it needs comes from one fixed 8 MiB arena compiled
 * into the library, which each GPU that loads the library holds until the
 * process exits.  A batch whose worst-case footprint (every window as wide
 * as the full energy range, including the global log g pool of problems too
 * large for shared memory) exceeds the arena is rejected with
 * WLG_ERR_CAPACITY before anything runs, leaving results and outputs as the
 * caller left them (400 problems of 6x6 lattices fit).  Runs on the current
 * device and `stream`; the call synchronises `stream` itself (after the
 * pre-run and at the end) and returns once the stream has finished the
 * batch.  The first call on a device also looks up the arena's device
 * address.  All calls share the
 * arena, which keeps the last call's contents: calls that overlap on the
 * GPU race, so serialise them. */
wlg_status wlg_solve_raw_noalloc(const wlg_problem* problems, int n, wlg_result* results, int* win_start,
                                 int* win_end, double* raw_log_g, long long raw_capacity, long long* raw_offset,
                                 wlg_stream stream);

/* The pre-run alone (prerun.cu:36-154) for a batch of problems (their
 * main-run fields are ignored): what the reference writes to
 * prerun_results.h5 (file_io.cpp:23-192).  Outputs are concatenated in
 * problem order; for problem p with N = X*Y and B = pre_intervals:
 *   seen[4N+1]          1 where the pre-run visited energy -2N + i, else 0
 *                       (the /Histogram/<k> dataset);
 *   couplings[2N]       +-1 after the error class (/Interaction/<k>);
 *   found[B], found_energy[B], lattices[B][N]: per coarse bin whether a
 *                       lattice was stored, its energy and spins +-1
 *                       (/Lattice/<k>/<E>).
 * Any output pointer may be NULL. */
wlg_status wlg_prerun(wlg_context* ctx, const wlg_problem* problems, int n, unsigned char* seen,
                      signed char* couplings, int* found, int* found_energy, signed char* lattices);

/* The main run and stitching (mainrun.cu:36-421) from pre-run outputs in
 * the layout wlg_prerun writes (the reference's mainrun reading
 * prerun_results.h5).  time_limit_s > 0 stops unfinished problems with
 * WLG_ERR_TIMEOUT once it passes (checked every 4 outer iterations; the
 * reference checks after each, mainrun.cu:376-383).  Results as wlg_solve. */
wlg_status wlg_mainrun(wlg_context* ctx, const wlg_problem* problems, int n, const unsigned char* seen,
                       const signed char* couplings, const int* found, const int* found_energy,
                       const signed char* lattices, double time_limit_s, wlg_result* results, int* energies,
                       double* log_g, long long capacity);

/* The hand-off from pre-run to main run alone (file_io.cpp:558-659 with
 * interval.cpp:5-41, as mainrun.cu:60-172 chains them), on the host: no
 * device, no context.  Inputs as wlg_mainrun.  Per problem p, in problem
 * order: status[p] (WLG_OK, or why its main run cannot start, e.g.
 * WLG_ERR_NO_LATTICE); e_min[p], e_max[p], the visited energy range;
 * spectrum[4N+1], 1 at every energy -2N + i the main run treats as
 * reachable; win_start/win_end[intervals], the windows; start_lattices
 * [intervals][N], each window's start lattice (spins +-1; every walker of
 * the window starts from it).  Arrays are concatenated over problems. */
wlg_status wlg_handoff(const wlg_problem* problems, int n, const unsigned char* seen, const signed char* couplings,
                       const int* found, const int* found_energy, const signed char* lattices, int* status,
                       int* e_min, int* e_max, unsigned char* spectrum, int* win_start, int* win_end,
                       signed char* start_lattices);

/* Plain form: the same problems computed with the reference's own structure
 * (prerun.cu:36-154, mainrun.cu:115-421) on the operators above — one
 * launch per operation, one thread per walker, state in global memory,
 * outer loop on the host with a device->host check per iteration.
 * Problems sharing all parameters but `sample` run as one R-sample run and
 * must hold samples 0..R-1.  Same outputs as wlg_solve; caller-allocated
 * nothing on the device (buffers are allocated and freed per call). */
wlg_status wlg_solve_plain(const wlg_problem* problems, int n, wlg_result* results, int* energies, double* log_g,
                           long long capacity, wlg_stream stream, long long* kernel_launches);

/* Autotuner: teams (problems) per CTA of the main-run launches, i.e. walkers
 * and windows per block.  The batch is prepared once and its main run timed
 * (CUDA events) with every power-of-two teams-per-CTA up to 256 threads per
 * CTA, each problem capped at max_outer outer iterations; the fastest choice
 * per (main-run form, team size) is kept by the context and used by every
 * later solve on it.  Results never depend on the choice (each problem's
 * trajectory is its own).  out[i] (up to cap) describes group i; *n_out =
 * number of groups. */
typedef struct {
  int form;        /* main-run form: 0 shared-memory lattice, 1 register lattice, 2 register + table */
  int team;        /* threads per team (walkers, rounded up to a warp) */
  int per_cta;     /* chosen teams per CTA */
  float main_ms;   /* its main-run time on the capped batch */
  int candidates;  /* choices timed */
} wlg_tuning;

wlg_status wlg_context_autotune(wlg_context* ctx, const wlg_problem* problems, int n, int max_outer,
                                wlg_tuning* out, int cap, int* n_out);

/* What the last wlg_solve / wlg_solve_raw did: time by phase in
 * milliseconds (device phases by CUDA events on the context's stream, host
 * phases by the host clock), bytes copied host->device and device->host,
 * the number of engine kernels launched, and which main-run kernel forms
 * ran (bit v for form v: 0 lattice and log g in shared memory, 1 lattice in
 * registers, 2 lattice in registers with a neighbour table, 3 lattice in
 * shared memory and FP64 log g in a global pool). */
typedef struct {
  double pre_ms, handoff_ms, main_ms, stitch_ms;
  long long h2d_bytes, d2h_bytes;
  int kernel_launches;
  int main_forms;
} wlg_stats;

wlg_status wlg_last_stats(const wlg_context* ctx, wlg_stats* out);

/* When the main run of each problem of the last wlg_solve / wlg_solve_raw
 * on ctx started and finished, in milliseconds from the first problem's
 * start, by the device clock (no counterpart in the reference, which runs
 * every sample for the whole loop).  Problem order; -1 for problems that did
 * not reach the main run.  *n_out = number of problems; WLG_ERR_CAPACITY
 * when cap is smaller.  A batch's main-run time is at least its longest
 * problem's end - start. */
wlg_status wlg_last_main_times(const wlg_context* ctx, double* start_ms, double* end_ms, int cap, int* n_out);

/* Secondary ceilings of the WL step on a device, measured by
 * microbenchmarks that fill every SM (no counterpart in the reference;
 * the rates its step depends on): shared-memory load bandwidth (128-bit,
 * conflict-free), Philox4x32-10 draws (the reference's cuRAND generator,
 * wl.cu:1074/:1114/:1167) and FP64 exp and log evaluations (its acceptance
 * exp, wl.cu:1113-1116, and factor log, wl.cu:1124), each the fastest of
 * three launches.  Takes a few tens of milliseconds; the calling thread's
 * current device is restored. */
typedef struct {
  int sm_count;
  double smem_gbs;           /* GB/s over the whole device */
  double philox_draws_per_s; /* 32-bit draws per second (four per Philox block) */
  double exp_f64_per_s;
  double log_f64_per_s;
} wlg_peaks;

wlg_status wlg_measure_peaks(int device, wlg_peaks* out);

/* Logical-class log-probabilities at the Nishimori temperature
 * beta_N = ln((1-p)/p) / 2 (no counterpart in the reference): for each of
 * n_classes normalised log g curves (energies[i], log_g[i]) with
 * i in [offset[c], offset[c] + count[c]), log Z_c = logsumexp(log g - beta_N E)
 * and log_probs[c] = log Z_c - logsumexp_c log Z_c. */
wlg_status wlg_class_log_probs(const int* energies, const double* log_g, const long long* offset, const int* count,
                               int n_classes, double prob, double* log_z, double* log_probs);

/* ---- Serving: continuous batching of decoding requests (no counterpart
 * in the reference, which runs one fixed batch per process).
 *
 * A request is one disorder sample, given as a wlg_problem whose
 * error_class is ignored: the server runs its four error classes i, v, h, c
 * and retires the request with the classes' log-probabilities at the
 * Nishimori temperature (wlg_class_log_probs).  Requests are admitted while
 * their device memory fits the budget; admitted problems keep their walker
 * state resident in device memory and advance in short main-run launches
 * ("epochs") shared with every other resident problem, so requests that
 * arrive while others run join the next epoch and finished ones leave it.
 * Each result equals the batch engine's for the same problems.  A server
 * owns a host thread and CUDA streams on `device`; submit and poll may be
 * called from any thread. */
typedef struct wlg_server wlg_server;

typedef struct {
  size_t mem_budget_bytes; /* device memory for resident problems; 0: 1 GiB */
  int epoch_outer;         /* outer WL iterations per main-run launch; 0: 4 */
  int max_prerun_batch;    /* requests per pre-run launch; 0: 256 */
  int max_resident;        /* resident problems (4 per request); 0: 8192 */
  int fail_after_epochs;   /* testing: a host-side failure is injected after this many epochs; 0: never */
  int stitching;           /* WLG_STITCH_REFERENCE (0) or WLG_STITCH_DEFINED */
  int max_readmit;         /* re-admissions of a class whose pre-run missed part of the spectrum
                              (WLG_ERR_NEW_ENERGY or WLG_ERR_NO_LATTICE), each with twice the
                              previous pre-run iterations; 0: 4; negative: none (the class retires
                              with that status, as the reference aborts its run) */
} wlg_server_config;

typedef struct {
  unsigned long long id;       /* as returned by wlg_server_submit */
  int status;                  /* WLG_OK, or the first failing class's status */
  int readmissions;            /* the most re-admissions of any one of its classes (max_readmit) */
  long long outer_iterations[4]; /* main-run outer iterations per class i, v, h, c */
  double log_z[4];             /* log Z_c at beta_N = ln((1-p)/p) / 2 */
  double log_probs[4];         /* log Z_c - logsumexp_c log Z_c */
  double submit_ms, done_ms;   /* host clock, milliseconds since the server started */
} wlg_decoded;

typedef struct {
  long long submitted, completed, resident_problems, epochs, main_launches, prerun_launches;
  long long bytes_in_use, bytes_budget;
  long long readmitted;        /* class re-admissions */
} wlg_server_stats;

wlg_status wlg_server_create(int device, const wlg_server_config* config, wlg_server** out);
/* Queues n requests; ids[i] receives request i's id.  Invalid requests are
 * rejected whole (WLG_ERR_INVALID, nothing queued). */
wlg_status wlg_server_submit(wlg_server* server, const wlg_problem* requests, int n, unsigned long long* ids);
/* wlg_server_submit on given disorder: couplings as wlg_solve_couplings
 * (the class-'i' pattern of each request, 2*X*Y entries, concatenated);
 * the four classes apply their chains on top.  NULL: wlg_server_submit. */
wlg_status wlg_server_submit_couplings(wlg_server* server, const wlg_problem* requests, int n,
                                       const signed char* couplings, unsigned long long* ids);
/* Up to `cap` finished requests in completion order; waits up to timeout_ms
 * (0: no wait) for at least one.  *n_out = 0 when none finished in time. */
wlg_status wlg_server_poll(wlg_server* server, wlg_decoded* out, int cap, int* n_out, int timeout_ms);
wlg_status wlg_server_stats_get(const wlg_server* server, wlg_server_stats* out);
/* Stops the loop (unfinished requests are dropped) and frees everything. */
wlg_status wlg_server_destroy(wlg_server* server);
/* Text of the failure that stopped the server ("" while it runs). */
const char* wlg_server_last_error(const wlg_server* server);

/* ---- HDF5 result files without libhdf5 (the prerun/mainrun programs write
 * the reference's layouts, file_io.cpp:23-192 and utils.cpp:137-236, in
 * HDF5 superblock-2 files; these read them back).  Paths are '/'-separated
 * below the root.  Types: 0 uint8, 1 int8, 2 int32, 3 uint64, 4 float64,
 * 5 compound {Key int32, Value float64} (16 bytes per element). */
unsigned int wlg_h5_lookup3(const void* data, size_t n, unsigned int init); /* the format's checksum */
/* Children of a group, one per line, groups with a trailing '/'. */
wlg_status wlg_h5_list(const char* file, const char* group, char* names, size_t cap);
/* A dataset's type, element count and (buf != NULL) little-endian bytes. */
wlg_status wlg_h5_read(const char* file, const char* dataset, int* type, unsigned long long* count, void* buf,
                       unsigned long long cap_bytes);
/* A fixed-length string attribute of a dataset (e.g. CodeVersion). */
wlg_status wlg_h5_attribute(const char* file, const char* dataset, const char* name, char* out, size_t cap);

#ifdef __cplusplus
}
#endif

#endif /* WLG_H_ */
