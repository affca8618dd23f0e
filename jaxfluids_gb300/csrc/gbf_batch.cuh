// Batched sweep kernel shared by the batch translation units
// (gbf_batch.cu: the WENO5-Z / MUSCL / CHAR-ROE schemes with HLLC or Rusanov;
// gbf_batch_schemes.cu: the other inviscid schemes).
#pragma once

#include "gbf_kernels.cuh"

namespace gbf {

constexpr int kBatchMaxCellsPerThread = 4;

struct BatchParams {
  SweepParams base;            // scheme and tile shape (sizes are per case)
  const gbf_batch_case* cases;
  const int32_t* worklist;
  int ntiles;
  int stage;
  const double* cons;          // stage input (packed)
  const double* cons0;         // step state U^n (packed)
  double* out;                 // stage output (packed)
  double* dt_states;           // 4 per case
  int reduce_dt;
};

__device__ __forceinline__ void batch_case_params(const BatchParams& bp, int c, SweepParams& p) {
  p = bp.base;
  const gbf_batch_case& cs = bp.cases[c];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    p.n[a] = cs.n[a];
    p.tiles[a] = cs.tiles[a];
    p.one_dx[a] = 1.0 / cs.dx[a];
  }
  p.cons = bp.cons + cs.offset;
  p.cons0 = bp.cons0 + cs.offset;
  p.out = bp.out + cs.offset;
  p.dt_state = bp.dt_states + 4 * c;
  p.stage = bp.stage;
  p.reduce_dt = bp.reduce_dt;
}

template <int RECON, int RIEMANN>
__global__ void __launch_bounds__(256) batch_sweep_kernel(const BatchParams bp) {
  extern __shared__ double smem[];
  for (int item = blockIdx.x; item < bp.ntiles; item += gridDim.x) {
    const int c = bp.worklist[2 * item];
    const int tile = bp.worklist[2 * item + 1];
    SweepParams p;
    batch_case_params(bp, c, p);
    sweep_tile<RECON, RIEMANN, MODE_STAGE, kBatchMaxCellsPerThread, 0>(p, tile, smem);
  }
}

template <int RECON, int RIEMANN>
int launch_batch_one(const BatchParams& bp, int grid, int threads, size_t smem, cudaStream_t s) {
  auto k = batch_sweep_kernel<RECON, RIEMANN>;
  if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return GBF_ERR_CUDA;
  k<<<grid, threads, smem, s>>>(bp);
  return cudaGetLastError() == cudaSuccess ? GBF_OK : GBF_ERR_CUDA;
}

// The schemes of gbf_batch_schemes.cu: WENO5-JS, TENO5, WENO3-JS, WENO3-Z with
// HLLC, HLL or Rusanov, and HLL with WENO5-Z, MUSCL and CHAR-PRIMITIVE.
int launch_batch_sweep_schemes(const gbf_case* c, const BatchParams& bp, int grid, int threads, size_t smem,
                               cudaStream_t s);

}  // namespace gbf
