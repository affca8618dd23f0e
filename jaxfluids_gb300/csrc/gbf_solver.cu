// Opaque solver handle: the fused TVD-RK3 path with its workspace and device
// time-step state owned by the library, for C callers that do not manage
// device memory themselves (the role SimulationManager plays in the reference,
// simulation_manager.py:94-138 construction, :296-401 time loop).
#include <cuda_runtime.h>

#include <new>

#include "gbf_kernels.cuh"

struct gbf_solver {
  gbf_case c;
  gbf_tile tile;
  bool has_tile;
  int device;
  void* workspace;
  double* dt_state;  // {dt, t, reduction slots}
};

using namespace gbf;

namespace {

int solver_create(const gbf_case* c, const gbf_tile* tile, gbf_solver** out) {
  if (!c || !out) return GBF_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  int st = gbf_case_check(c);
  if (st != GBF_OK) return st;
  const size_t ws = gbf_rk3_workspace_bytes(c);
  if (ws == 0) return GBF_ERR_INVALID_ARGUMENT;
  gbf_solver* s = new (std::nothrow) gbf_solver();
  if (!s) return GBF_ERR_INVALID_ARGUMENT;
  s->c = *c;
  s->has_tile = tile != nullptr;
  if (tile) s->tile = *tile;
  if (cudaGetDevice(&s->device) != cudaSuccess || cudaMalloc(&s->workspace, ws) != cudaSuccess) {
    delete s;
    return GBF_ERR_CUDA;
  }
  if (cudaMalloc((void**)&s->dt_state, 4 * sizeof(double)) != cudaSuccess) {
    cudaFree(s->workspace);
    delete s;
    return GBF_ERR_CUDA;
  }
  *out = s;
  return GBF_OK;
}

int solver_destroy(gbf_solver* s) {
  if (!s) return GBF_OK;
  int prev = -1;
  cudaGetDevice(&prev);
  cudaSetDevice(s->device);
  const bool ok = cudaFree(s->workspace) == cudaSuccess && cudaFree(s->dt_state) == cudaSuccess;
  if (prev >= 0) cudaSetDevice(prev);
  delete s;
  return ok ? GBF_OK : GBF_ERR_CUDA;
}

int solver_init(gbf_solver* s, const double* cons, double t0, void* stream) {
  if (!s) return GBF_ERR_INVALID_ARGUMENT;
  return gbf_rk3_init(&s->c, cons, nullptr, s->dt_state, t0, stream);
}

int solver_advance(gbf_solver* s, double* cons, int steps, void* stream) {
  if (!s) return GBF_ERR_INVALID_ARGUMENT;
  return gbf_rk3_advance(&s->c, cons, nullptr, s->dt_state, s->workspace, steps, s->has_tile ? &s->tile : nullptr,
                         stream);
}

int solver_time(gbf_solver* s, double* dt_t, void* stream) {
  if (!s || !dt_t) return GBF_ERR_INVALID_ARGUMENT;
  cudaStream_t st = (cudaStream_t)stream;
  if (cudaMemcpyAsync(dt_t, s->dt_state, 2 * sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess)
    return GBF_ERR_CUDA;
  return cudaStreamSynchronize(st) == cudaSuccess ? GBF_OK : GBF_ERR_CUDA;
}

}  // namespace

extern "C" int gbf_create(const gbf_case* c, const gbf_tile* tile, gbf_solver** out) {
  return record_status(solver_create(c, tile, out));
}

extern "C" int gbf_destroy(gbf_solver* s) { return record_status(solver_destroy(s)); }

extern "C" int gbf_solver_init(gbf_solver* s, const double* cons, double t0, void* stream) {
  return record_status(solver_init(s, cons, t0, stream));
}

extern "C" int gbf_solver_advance(gbf_solver* s, double* cons, int steps, void* stream) {
  return record_status(solver_advance(s, cons, steps, stream));
}

extern "C" int gbf_solver_time(gbf_solver* s, double* dt_t, void* stream) {
  return record_status(solver_time(s, dt_t, stream));
}
