// Arithmetic-rate probes used by the benchmark to measure this GPU's FP64
// roofline (no FP64 peak is published for the part): independent dependency
// chains per thread, results stored so nothing is optimised away; and the
// kernels' zero-dividend division (gbf::div0) beside the IEEE division, for
// the test that compares them bit for bit.  Built as its own library
// (libgbfprobe.so), apart from the product library; only the benchmark and
// the tests load it.
#include <cuda_runtime.h>

#include <algorithm>

#include "gbf_physics.cuh"

// modes of gbf_probe_arith
#define GBF_PROBE_DFMA 0
#define GBF_PROBE_DDIV 1
#define GBF_PROBE_DSQRT 2
#define GBF_PROBE_FFMA 3
#define GBF_PROBE_DDIV_ZERO 4  // divisions whose dividend is zero

namespace {

constexpr int kChains = 8;

template <int MODE>
__global__ void probe_kernel(double* out, int iters, double seed, double num) {
  double a[kChains];
#pragma unroll
  for (int k = 0; k < kChains; ++k) a[k] = seed + 1e-3 * (threadIdx.x + k);
  const double m = 0.999999999;
  const double c = 1e-9;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < kChains; ++k) {
      if (MODE == GBF_PROBE_DFMA) a[k] = fma(a[k], m, c);
      // num is a run-time value (1.25, or 0 for the zero dividend), so the
      // compiler cannot turn the division into a reciprocal
      if (MODE == GBF_PROBE_DDIV) a[k] = c + num / a[k];
      if (MODE == GBF_PROBE_DDIV_ZERO) a[k] = 1.5 + (num * a[k]) / a[k];
      if (MODE == GBF_PROBE_DSQRT) a[k] = sqrt(a[k]) + 0.5;
      if (MODE == GBF_PROBE_FFMA) a[k] = (double)fmaf((float)a[k], 0.9999f, 1e-7f);
    }
  }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < kChains; ++k) s += a[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// FP32 rate: keep the chain in float registers
__global__ void probe_ffma_kernel(double* out, int iters, double seed) {
  float a[kChains];
#pragma unroll
  for (int k = 0; k < kChains; ++k) a[k] = (float)seed + 1e-3f * (threadIdx.x + k);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < kChains; ++k) a[k] = fmaf(a[k], 0.9999f, 1e-7f);
  }
  float s = 0.f;
#pragma unroll
  for (int k = 0; k < kChains; ++k) s += a[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void div0_kernel(const double* a, const double* b, double* q_div0, double* q_ieee, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    q_div0[i] = gbf::div0(a[i], b[i]);
    q_ieee[i] = __ddiv_rn(a[i], b[i]);
  }
}

}  // namespace

// q_div0[i] = gbf::div0(a[i], b[i]) and q_ieee[i] = a[i] / b[i] (IEEE, round
// to nearest) for i < n.  Returns 0, or -1 for invalid arguments, -3 for a
// launch error.
extern "C" int gbf_probe_div0(const double* a, const double* b, double* q_div0, double* q_ieee, long long n,
                              void* stream) {
  if (!a || !b || !q_div0 || !q_ieee || n <= 0) return -1;
  const long long blocks = std::min<long long>((n + 255) / 256, 152LL * 8);
  div0_kernel<<<(int)blocks, 256, 0, (cudaStream_t)stream>>>(a, b, q_div0, q_ieee, n);
  return cudaGetLastError() == cudaSuccess ? 0 : -3;
}

// Runs `iters` iterations of 8 independent dependency chains of one operation
// per thread (blocks x threads threads) and stores one value per thread in
// out.  Returns 0, or -1 for invalid arguments, -3 for a launch error.
extern "C" int gbf_probe_arith(int mode, double* out, int blocks, int threads, int iters, void* stream) {
  if (!out || blocks <= 0 || threads <= 0 || threads > 1024 || iters <= 0) return -1;
  cudaStream_t s = (cudaStream_t)stream;
  switch (mode) {
    case GBF_PROBE_DFMA: probe_kernel<GBF_PROBE_DFMA><<<blocks, threads, 0, s>>>(out, iters, 1.0, 0.0); break;
    case GBF_PROBE_DDIV: probe_kernel<GBF_PROBE_DDIV><<<blocks, threads, 0, s>>>(out, iters, 1.5, 1.25); break;
    case GBF_PROBE_DSQRT: probe_kernel<GBF_PROBE_DSQRT><<<blocks, threads, 0, s>>>(out, iters, 2.0, 0.0); break;
    case GBF_PROBE_DDIV_ZERO:
      probe_kernel<GBF_PROBE_DDIV_ZERO><<<blocks, threads, 0, s>>>(out, iters, 1.5, 0.0);
      break;
    case GBF_PROBE_FFMA: probe_ffma_kernel<<<blocks, threads, 0, s>>>(out, iters, 1.0); break;
    default: return -1;
  }
  return cudaGetLastError() == cudaSuccess ? 0 : -3;
}
