// Allocation-free variant of gbf_rk3_advance.
//
// Some callers cannot hand this library any scratch memory and must not have
// it call cudaMalloc either:
//   * an XLA custom call (the way JAX-Fluids would bind this path) gets its
//     device memory only from XLA's allocator, which by default reserves most
//     of the GPU's memory up front, so a cudaMalloc from inside the handler
//     competes with it and can fail mid-run;
//   * host code with a fixed device-memory budget (a solver embedded in a
//     larger application) that forbids allocations it does not account for;
//   * host loops that must not stall: cudaFree synchronises the whole device.
// For them, the RK3 workspace (stage states, stage primitives, face fluxes)
// lives in a fixed device array compiled into this library.  The array is
// modest (GBF_NOALLOC_SCRATCH_BYTES, 32 MiB) and every GPU that loads the
// library holds it until the process exits.
#include <mutex>

#include "gbf_kernels.cuh"

namespace {

constexpr size_t kScratchDoubles = (size_t)GBF_NOALLOC_SCRATCH_BYTES / sizeof(double);

// The workspace of gbf_rk3_advance for cases whose gbf_rk3_workspace_bytes
// fits in GBF_NOALLOC_SCRATCH_BYTES.
static __device__ __align__(256) double g_rk3_stage_scratch[kScratchDoubles];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mutex;
double* g_scratch_ptr[kMaxDevices] = {};

// Device address of the scratch array on the current device.  In host code the
// array's name is only a host-side stand-in, so the address is looked up once
// per device, with that device current, and cached.
int scratch_on_current_device(double** out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess) return GBF_ERR_CUDA;
  if (dev < 0 || dev >= kMaxDevices) return GBF_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_rk3_stage_scratch) != cudaSuccess || !p) return GBF_ERR_CUDA;
    g_scratch_ptr[dev] = static_cast<double*>(p);
  }
  *out = g_scratch_ptr[dev];
  return GBF_OK;
}

}  // namespace

using namespace gbf;

static int gbf_rk3_advance_noalloc_impl(const gbf_case* c, double* cons, double* dt_state, int steps,
                                       const gbf_tile* tile, void* stream) {
  int st = gbf_case_check(c);
  if (st != GBF_OK) return st;
  // beyond the built-in scratch: refused before any CUDA call
  if (gbf_rk3_workspace_bytes(c) > (size_t)GBF_NOALLOC_SCRATCH_BYTES) return GBF_ERR_SIZE;
  if (!cons || !dt_state || steps < 0) return GBF_ERR_INVALID_ARGUMENT;
  if (((uintptr_t)cons & 7u) || ((uintptr_t)dt_state & 7u)) return GBF_ERR_ALIGNMENT;
  double* scratch = nullptr;
  if ((st = scratch_on_current_device(&scratch)) != GBF_OK) return st;
  // The workspace is packed at the start of the array for this case's size.
  // Every buffer in it is written before it is read within a call (the stage
  // primitives are derived from cons first, each stage writes its whole state,
  // primitives and face fluxes, the Lax-Friedrichs slots are cleared per
  // stage), so nothing left over from an earlier call is ever read.
  return rk3_advance_on(c, cons, nullptr, dt_state, scratch, steps, tile, (cudaStream_t)stream);
}

extern "C" int gbf_rk3_advance_noalloc(const gbf_case* c, double* cons, double* dt_state, int steps,
                                       const gbf_tile* tile, void* stream) {
  return record_status(gbf_rk3_advance_noalloc_impl(c, cons, dt_state, steps, tile, stream));
}
