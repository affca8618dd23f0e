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
// For them, the two RK3 stage buffers live in a fixed device array compiled
// into this library.  The array is modest (GBF_NOALLOC_MAX_CELLS cells, 32 MiB)
// and every GPU that loads the library holds it until the process exits.
#include <mutex>

#include "gbf_kernels.cuh"

namespace {

constexpr size_t kStateDoubles = (size_t)5 * GBF_NOALLOC_MAX_CELLS;

// Two stage buffers of up to GBF_NOALLOC_MAX_CELLS cells (5 doubles each).
static __device__ __align__(256) double g_rk3_stage_scratch[2 * kStateDoubles];

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
  CaseInfo ci;
  if ((st = make_case_info(c, &ci)) != GBF_OK) return st;
  if (ci.cells > (long long)GBF_NOALLOC_MAX_CELLS) return GBF_ERR_SIZE;  // beyond the built-in scratch
  if (!cons || !dt_state || steps < 0) return GBF_ERR_INVALID_ARGUMENT;
  if (((uintptr_t)cons & 7u) || ((uintptr_t)dt_state & 7u)) return GBF_ERR_ALIGNMENT;
  SweepParams p;
  int threads;
  size_t smem;
  if ((st = make_sweep_params(c, ci, tile, &p, &threads, &smem)) != GBF_OK) return st;
  double* scratch = nullptr;
  if ((st = scratch_on_current_device(&scratch)) != GBF_OK) return st;
  cudaStream_t s = (cudaStream_t)stream;
  // Stage buffers packed at the start of the array for this case's size.  Each
  // stage writes its whole buffer before the next stage reads it, so nothing
  // left over from an earlier call is ever read and nothing needs clearing.
  double* A = scratch;
  double* B = scratch + 5 * ci.cells;
  unsigned long long* red = (unsigned long long*)(dt_state + 2);
  p.dt_state = dt_state;
  for (int step = 0; step < steps; ++step) {
    p.stage = 0; p.cons = cons; p.cons0 = cons; p.out = A; p.reduce_dt = 0;
    if ((st = launch_sweep(c, p, threads, smem, s, MODE_STAGE)) != GBF_OK) return st;
    p.stage = 1; p.cons = A; p.cons0 = cons; p.out = B;
    if ((st = launch_sweep(c, p, threads, smem, s, MODE_STAGE)) != GBF_OK) return st;
    p.stage = 2; p.cons = B; p.cons0 = cons; p.out = cons; p.reduce_dt = 1;
    if ((st = launch_sweep(c, p, threads, smem, s, MODE_STAGE)) != GBF_OK) return st;
    if ((st = launch_dt_finalize(c, ci, red, dt_state, dt_state + 1, 1, s)) != GBF_OK) return st;
  }
  return GBF_OK;
}

extern "C" int gbf_rk3_advance_noalloc(const gbf_case* c, double* cons, double* dt_state, int steps,
                                       const gbf_tile* tile, void* stream) {
  return record_status(gbf_rk3_advance_noalloc_impl(c, cons, dt_state, steps, tile, stream));
}
