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

#ifdef __cplusplus
}
#endif

#endif /* WLG_H_ */
