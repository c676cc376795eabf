// Secondary ceilings of the WL step, measured on the device by
// microbenchmarks (wlg_measure_peaks): shared-memory load bandwidth (the
// level that holds the walker state of shared-memory teams), Philox4x32-10
// throughput (the draws of every step, wl.cu:1074/:1114/:1167 draw them
// with cuRAND) and FP64 exp / log throughput (the reference evaluates one
// exp of a log g difference per step, wl.cu:1113-1116, and a log of the
// modification factor per update, wl.cu:1124).
//
// Each kernel runs a fixed amount of independent work per thread on every
// SM at the occupancy the runtime reports for it; the rate is the work of
// the fastest of three event-timed launches after one warm-up launch, on a
// stream of this call's own.  Results go to a small device buffer so that
// no work is dead code.

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "../../include/wlg.h"
#include "wlg_internal.h"
#include "wlg_rng.cuh"

namespace {

constexpr int kThreads = 1024;
constexpr int kSmemVecs = 2048;  // 32 KB of 16-byte words per CTA (power of two)
constexpr int kSmemIters = 8192;
constexpr int kPhiloxIters = 4096;
constexpr int kF64Iters = 64;    // four evaluations per iteration

// Every thread loads four 16-byte words per iteration; the 32 lanes of a
// warp read 32 consecutive words (four conflict-free wavefronts).  The
// index stays in [0, kSmemVecs) by the mask.
__global__ void __launch_bounds__(kThreads) k_peak_smem(int iters, uint4* out)
{
  __shared__ uint4 buf[kSmemVecs];
  for (int i = threadIdx.x; i < kSmemVecs; i += blockDim.x)
    buf[i] = make_uint4(i, 3u * i, 5u * i, 7u * i);
  __syncthreads();
  const uint32_t base = static_cast<uint32_t>(__cvta_generic_to_shared(buf));
  uint4 acc = make_uint4(0u, 0u, 0u, 0u);
  int idx = threadIdx.x;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const uint32_t k = static_cast<uint32_t>(idx + u * (kSmemVecs / 4)) & (kSmemVecs - 1);
      uint32_t a, b, c, d;
      asm volatile("ld.shared.v4.u32 {%0, %1, %2, %3}, [%4];"
                   : "=r"(a), "=r"(b), "=r"(c), "=r"(d)
                   : "r"(base + 16u * k));
      acc.x ^= a;
      acc.y ^= b;
      acc.z ^= c;
      acc.w ^= d;
    }
    idx = (idx + 32) & (kSmemVecs - 1);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = acc;
}

// One Philox4x32-10 block (four 32-bit draws) per iteration, counters
// (iteration, thread), independent across iterations.
__global__ void __launch_bounds__(kThreads) k_peak_philox(int iters, uint4* out)
{
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  uint4 acc = make_uint4(0u, 0u, 0u, 0u);
#pragma unroll 4
  for (int i = 0; i < iters; ++i) {
    const uint4 r = wlg::philox10(static_cast<uint32_t>(i), t, 0x2545F491u, 0u, 0x9E3779B9u, 0x7F4A7C15u);
    acc.x ^= r.x;
    acc.y ^= r.y;
    acc.z ^= r.z;
    acc.w ^= r.w;
  }
  out[t] = acc;
}

// Four independent FP64 exp (kLog false) or log (kLog true) evaluations per
// iteration, arguments in the range the WL acceptance and factor use.
template <bool kLog>
__global__ void __launch_bounds__(kThreads) k_peak_f64(int iters, uint4* out)
{
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  const double x0 = kLog ? 1.0 + 1e-4 * (t & 1023) : -1e-3 * (t & 1023);
  double acc = 0.0;
  for (int i = 0; i < iters; ++i) {
    const double d = 1e-7 * i;
    if constexpr (kLog)
      acc += (log(x0 + d) + log(x0 + 0.25 + d)) + (log(x0 + 0.5 + d) + log(x0 + 0.75 + d));
    else
      acc += (exp(x0 - d) + exp(x0 - 0.25 - d)) + (exp(x0 - 0.5 - d) + exp(x0 - 0.75 - d));
  }
  const unsigned long long bits = static_cast<unsigned long long>(__double_as_longlong(acc));
  out[t] = make_uint4(static_cast<uint32_t>(bits), static_cast<uint32_t>(bits >> 32), 0u, 0u);
}

// Grid of `kernel` filling every SM at its reported occupancy.
template <typename K>
int full_grid(K kernel, int sms)
{
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kThreads, 0) != cudaSuccess || per_sm < 1)
    per_sm = 1;
  return sms * per_sm;
}

// Fastest of three launches after a warm-up, in seconds; negative on error.
template <typename K>
double time_kernel(K kernel, int grid, int iters, uint4* out, cudaStream_t s, cudaEvent_t e0, cudaEvent_t e1)
{
  kernel<<<grid, kThreads, 0, s>>>(iters, out);
  if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(s) != cudaSuccess) return -1.0;
  float best = 0.0f;
  for (int r = 0; r < 3; ++r) {
    cudaEventRecord(e0, s);
    kernel<<<grid, kThreads, 0, s>>>(iters, out);
    cudaEventRecord(e1, s);
    float ms = 0.0f;
    if (cudaGetLastError() != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
        cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess)
      return -1.0;
    best = r == 0 ? ms : std::min(best, ms);
  }
  return best > 0.0f ? best * 1e-3 : -1.0;
}

}  // namespace

extern "C" wlg_status wlg_measure_peaks(int device, wlg_peaks* out)
{
  return wlg::guarded([&]() -> wlg_status {
    if (out == nullptr) return WLG_ERR_INVALID;
    int prev = 0, sms = 0;
    if (cudaGetDevice(&prev) != cudaSuccess || cudaSetDevice(device) != cudaSuccess) return WLG_ERR_CUDA;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess || sms < 1) {
      cudaSetDevice(prev);
      return WLG_ERR_CUDA;
    }
    const int g_smem = full_grid(k_peak_smem, sms), g_philox = full_grid(k_peak_philox, sms);
    const int g_exp = full_grid(k_peak_f64<false>, sms), g_log = full_grid(k_peak_f64<true>, sms);
    const int g_max = std::max(std::max(g_smem, g_philox), std::max(g_exp, g_log));
    uint4* buf = nullptr;
    cudaStream_t s = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    wlg_status st = WLG_OK;
    if (cudaMalloc(&buf, static_cast<size_t>(g_max) * kThreads * sizeof(uint4)) != cudaSuccess ||
        cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess || cudaEventCreate(&e0) != cudaSuccess ||
        cudaEventCreate(&e1) != cudaSuccess) {
      st = WLG_ERR_CUDA;
    } else {
      const double t_smem = time_kernel(k_peak_smem, g_smem, kSmemIters, buf, s, e0, e1);
      const double t_philox = time_kernel(k_peak_philox, g_philox, kPhiloxIters, buf, s, e0, e1);
      const double t_exp = time_kernel(k_peak_f64<false>, g_exp, kF64Iters, buf, s, e0, e1);
      const double t_log = time_kernel(k_peak_f64<true>, g_log, kF64Iters, buf, s, e0, e1);
      if (t_smem <= 0.0 || t_philox <= 0.0 || t_exp <= 0.0 || t_log <= 0.0) {
        st = WLG_ERR_CUDA;
      } else {
        *out = wlg_peaks{};
        out->sm_count = sms;
        out->smem_gbs = static_cast<double>(g_smem) * kThreads * kSmemIters * 4.0 * 16.0 / t_smem * 1e-9;
        out->philox_draws_per_s = static_cast<double>(g_philox) * kThreads * kPhiloxIters * 4.0 / t_philox;
        out->exp_f64_per_s = static_cast<double>(g_exp) * kThreads * kF64Iters * 4.0 / t_exp;
        out->log_f64_per_s = static_cast<double>(g_log) * kThreads * kF64Iters * 4.0 / t_log;
      }
    }
    if (e1) cudaEventDestroy(e1);
    if (e0) cudaEventDestroy(e0);
    if (s) cudaStreamDestroy(s);
    if (buf) cudaFree(buf);
    cudaSetDevice(prev);
    return st;
  });
}
