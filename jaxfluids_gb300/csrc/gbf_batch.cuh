// Batched fused TVD-RK3 stage kernels shared by the batch translation units
// (gbf_batch.cu: the WENO5-Z / MUSCL / CHAR-ROE schemes with HLLC or Rusanov
// and the host side; gbf_batch_schemes.cu, gbf_batch_schemes5.cu: the other
// inviscid schemes).
//
// A stage of the batch is the single-case fused stage (gbf_faces.cuh) over a
// work list of (case, tile) pairs: one launch of the face kernel walks the
// list once per active axis, each item computing every face of its cell tile
// along that axis (the last tile along the axis also the closing face of a
// non-periodic line) into the case's face buffer; then one epilogue launch
// walks the list again, each item forming its cells' divergence, RK
// combination, primitives of the new state and time-step reductions.  Every
// face is computed once, the primitives come from the stage's primitive
// buffer, and the arithmetic is the single-case path's, so a batched case
// advances bitwise like the same case alone.
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
  const double* prims;         // primitives of the stage input (packed)
  double* prims_out;           // primitives of the stage output (packed), or null
  double* faces[3];            // face fluxes of axis a: case c from faces[a] + 2 offset_c
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
  p.prims = bp.prims + cs.offset;
  p.dt_state = bp.dt_states + 4 * c;
  p.stage = bp.stage;
  p.reduce_dt = bp.reduce_dt;
}

// Faces per line along axis a of a case: N on a PERIODIC axis (face N - 1/2
// is face -1/2), N + 1 otherwise.
__device__ __forceinline__ int batch_faces_per_line(const SweepParams& p, int a) {
  return (p.bc[2 * a] == GBF_BC_PERIODIC) ? p.n[a] : p.n[a] + 1;
}

// The cell tile `tile` of a case: its origin and cell extents.
__device__ __forceinline__ void batch_tile(const SweepParams& p, const gbf_batch_case& cs, int tile, int b[3],
                                           int o[3], int e[3]) {
  b[2] = tile % cs.tiles[2];
  b[1] = (tile / cs.tiles[2]) % cs.tiles[1];
  b[0] = tile / (cs.tiles[2] * cs.tiles[1]);
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    o[a] = b[a] * p.t[a];
    e[a] = min(p.t[a], p.n[a] - o[a]);
  }
}

// The faces of axis AX of one work item (its cell tile; the last tile of a
// line also the closing face) into the case's face buffer.
template <int AX, int RECON, int RIEMANN>
__device__ __forceinline__ void batch_face_item(const BatchParams& bp, const SweepParams& p, const gbf_batch_case& cs,
                                                int tile, double* smem) {
  int b[3], o[3], fe[3];
  batch_tile(p, cs, tile, b, o, fe);
  const int nf = batch_faces_per_line(p, AX);
  if (b[AX] == cs.tiles[AX] - 1) fe[AX] = nf - o[AX];  // the line's last faces
  face_tile_body<AX, RECON, RIEMANN, 0>(p, o, fe, nf, bp.faces[AX] + 2 * cs.offset, smem);
}

// The faces of every active axis of every work item in one launch: the CTAs
// loop over (axis, item) pairs, the items of the first active axis first, so
// one tail per stage remains.  The item's case parameters live in shared
// memory, written once per item by one thread (a per-thread copy would cost
// every thread the whole struct in local memory).
template <int RECON, int RIEMANN>
__global__ void __launch_bounds__(256, 2) batch_face_kernel(const BatchParams bp) {
  extern __shared__ double smem[];
  __shared__ SweepParams sp;
  int axes[3], na = 0;
#pragma unroll
  for (int a = 0; a < 3; ++a)
    if ((bp.base.active_mask >> a) & 1) axes[na++] = a;
  const long long pairs = (long long)na * bp.ntiles;
  for (long long v = blockIdx.x; v < pairs; v += gridDim.x) {
    const int ax = axes[v / bp.ntiles];
    const int item = (int)(v % bp.ntiles);
    const int c = bp.worklist[2 * item];
    const int tile = bp.worklist[2 * item + 1];
    if (threadIdx.x == 0) batch_case_params(bp, c, sp);
    __syncthreads();
    const gbf_batch_case& cs = bp.cases[c];
    if (ax == 0)
      batch_face_item<0, RECON, RIEMANN>(bp, sp, cs, tile, smem);
    else if (ax == 1)
      batch_face_item<1, RECON, RIEMANN>(bp, sp, cs, tile, smem);
    else
      batch_face_item<2, RECON, RIEMANN>(bp, sp, cs, tile, smem);
    __syncthreads();  // the next pair rewrites the parameters and restages the pencil
  }
}

template <int RECON, int RIEMANN>
int launch_batch_faces_one(const BatchParams& bp, int grid, int threads, size_t smem, cudaStream_t s) {
  auto kern = batch_face_kernel<RECON, RIEMANN>;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return GBF_ERR_CUDA;
  kern<<<grid, threads, smem, s>>>(bp);
  return cudaGetLastError() == cudaSuccess ? GBF_OK : GBF_ERR_CUDA;
}

// The schemes of gbf_batch_schemes.cu: WENO5-JS, TENO5, WENO3-JS, WENO3-Z with
// HLLC, HLL or Rusanov, and HLL with WENO5-Z, MUSCL and CHAR-PRIMITIVE.
int launch_batch_faces_schemes(const gbf_case* c, const BatchParams& bp, int grid, int threads, size_t smem,
                               cudaStream_t s);

}  // namespace gbf
