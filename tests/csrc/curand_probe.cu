// Test-only probe: draws from cuRAND's Philox4_32_10 device API and CUDA's
// double exp/log, so the tests can pin the engine's own Philox streams and
// the oracle's host arithmetic against what the reference's kernels compute.
#include <cstdint>
#include <curand_kernel.h>

#include "../../qec_pf_wang_landau_gb300/csrc/wlg_accept.cuh"
#include "../../qec_pf_wang_landau_gb300/csrc/wlg_shadow.cuh"

namespace {

__global__ void k_curand(const unsigned long long* seeds, const unsigned long long* subseqs,
                         const unsigned long long* offsets, int n_triples, int n_draws, float* out)
{
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n_triples) return;
  curandStatePhilox4_32_10_t st;
  curand_init(seeds[q], subseqs[q], offsets[q], &st);
  for (int d = 0; d < n_draws; ++d) out[static_cast<size_t>(q) * n_draws + d] = curand_uniform(&st);
}

__global__ void k_exp_log(const double* x, double* e, double* l, int n)
{
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  e[q] = exp(x[q]);
  l[q] = log(x[q]);
}

__global__ void k_sqrt_chain(double x0, int n, double* f, double* lf)
{
  double x = x0;
  for (int q = 0; q < n; ++q) {
    f[q] = x;
    lf[q] = log(x);
    x = sqrt(x);
  }
}

__global__ void k_fast_exp(const float* x, float* y, int n)
{
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q < n) y[q] = __expf(x[q]);
}

__global__ void k_shadow(const double* g, const double* base, float* out, int n)
{
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q < n) out[q] = wlg::shadow_split(g[q], wlg::split_float(base[q]));
}

// max |__logf(x) - log(x)| over the floats with bit patterns [lo, hi]
__global__ void k_logf_maxerr(unsigned lo, unsigned hi, unsigned* max_bits)
{
  float worst = 0.0f;
  for (unsigned long long b = lo + blockIdx.x * static_cast<unsigned long long>(blockDim.x) + threadIdx.x; b <= hi;
       b += static_cast<unsigned long long>(gridDim.x) * blockDim.x) {
    const float x = __uint_as_float(static_cast<unsigned>(b));
    const double err = fabs(static_cast<double>(__logf(x)) - log(static_cast<double>(x)));
    worst = fmaxf(worst, __double2float_ru(err));
  }
  atomicMax(max_bits, __float_as_uint(worst));
}

// decide() against the exact rule u < min(1, exp(d)) for n draws with
// estimates df = d + noise, |noise| <= eps
__global__ void k_decide(const unsigned* x, const double* d, const float* df, const float* eps, int n, int* out)
{
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const wlg::Decision r = wlg::decide(x[q], wlg::log_uniform(x[q]), df[q], eps[q], false);
  const bool exact = static_cast<double>(wlg::unit_float(x[q])) < fmin(1.0, exp(d[q]));
  out[q] = r.known ? (r.acc == exact ? 1 : -1) : 0;
}

}  // namespace

extern "C" {

float probe_log_bound() { return wlg::kLogAbsErr; }

int probe_logf_maxerr(unsigned lo, unsigned hi, unsigned* d_max_bits)
{
  k_logf_maxerr<<<152 * 8, 256>>>(lo, hi, d_max_bits);
  return cudaDeviceSynchronize() == cudaSuccess ? 0 : 1;
}

int probe_decide(const unsigned* d_x, const double* d_d, const float* d_df, const float* d_eps, int n, int* d_out)
{
  k_decide<<<(n + 127) / 128, 128>>>(d_x, d_d, d_df, d_eps, n, d_out);
  return cudaDeviceSynchronize() == cudaSuccess ? 0 : 1;
}

// The engine's integer-formed log g shadows (wlg_shadow.cuh) for n pairs.
int probe_shadow(const double* d_g, const double* d_base, float* d_out, int n)
{
  k_shadow<<<(n + 127) / 128, 128>>>(d_g, d_base, d_out, n);
  return cudaDeviceSynchronize() == cudaSuccess ? 0 : 1;
}

int probe_fast_exp(const float* d_x, float* d_y, int n)
{
  k_fast_exp<<<(n + 127) / 128, 128>>>(d_x, d_y, n);
  return cudaDeviceSynchronize() == cudaSuccess ? 0 : 1;
}


int probe_curand_uniform(const unsigned long long* d_seeds, const unsigned long long* d_subseqs,
                         const unsigned long long* d_offsets, int n_triples, int n_draws, float* d_out)
{
  k_curand<<<(n_triples + 127) / 128, 128>>>(d_seeds, d_subseqs, d_offsets, n_triples, n_draws, d_out);
  return cudaDeviceSynchronize() == cudaSuccess ? 0 : 1;
}

int probe_exp_log(const double* d_x, double* d_exp, double* d_log, int n)
{
  k_exp_log<<<(n + 127) / 128, 128>>>(d_x, d_exp, d_log, n);
  return cudaDeviceSynchronize() == cudaSuccess ? 0 : 1;
}

int probe_sqrt_chain(double x0, int n, double* d_f, double* d_logf)
{
  k_sqrt_chain<<<1, 1>>>(x0, n, d_f, d_logf);
  return cudaDeviceSynchronize() == cudaSuccess ? 0 : 1;
}

}  // extern "C"
