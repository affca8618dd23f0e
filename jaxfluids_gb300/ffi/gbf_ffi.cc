// XLA FFI custom-call handlers over the C ABI of libgbfluids.so: the binding
// through which JAX-Fluids (a JAX program, whose compiled step functions are
// XLA computations) reaches the GB300 kernels.  Each handler unpacks the case
// descriptor (the int64 attribute "desc", gbf_ffi_desc.h), calls one entry
// point of include/gbfluids.h on XLA's stream and maps a failing status to an
// FFI error; nothing here synchronises or allocates (workspaces are declared
// as extra results, so XLA's allocator owns them).
//
// Built by jaxfluids_gb300.build.build_ffi() against jax.ffi.include_dir()
// into libgbfluids_ffi.so, only where jaxlib is installed.  Registered and
// called from jaxfluids_gb300/jax_binding.py:
//   gbf_rhs_ffi             <- SpaceSolver.compute_rhs (solvers/space_solver.py:151-453)
//   gbf_rk3_init_ffi        <- the initial time step (time_integration/time_step_size.py:15-157)
//   gbf_rk3_advance_ffi     <- SimulationManager.do_runge_kutta_stages + next dt
//                              (simulation_manager.py:536-1077), fused
//   gbf_rhs_vjp_ffi         <- jax.grad of compute_rhs
//   gbf_rk3_step_vjp_ffi    <- jax.grad of one step of _feed_forward (simulation_manager.py:1296-1412)
#include <cuda_runtime.h>

#include <cstdint>

#include "gbf_ffi_desc.h"
#include "gbfluids.h"
#include "xla/ffi/api/ffi.h"

namespace ffi = xla::ffi;

namespace {

ffi::Error status_error(int st) {
  if (st == GBF_OK) return ffi::Error::Success();
  const ffi::ErrorCode code = (st == GBF_ERR_CUDA) ? ffi::ErrorCode::kInternal
                              : (st == GBF_ERR_UNSUPPORTED) ? ffi::ErrorCode::kUnimplemented
                                                            : ffi::ErrorCode::kInvalidArgument;
  return ffi::Error(code, gbf_status_string(st));
}

int unpack(ffi::Span<const int64_t> desc, gbf_case* c) {
  return gbf_case_from_words(desc.begin(), desc.size(), c);
}

// Copy `in` to `out` when XLA did not alias them (input_output_aliases is a
// request, not a guarantee).
int copy_if_distinct(const void* in, void* out, size_t bytes, cudaStream_t s) {
  if (in == out) return GBF_OK;
  return cudaMemcpyAsync(out, in, bytes, cudaMemcpyDeviceToDevice, s) == cudaSuccess ? GBF_OK : GBF_ERR_CUDA;
}

// compute_rhs: halo buffers of the primitives and conservatives in, interior
// right-hand side out (and a workspace of gbf_rhs_workspace_bytes(c) bytes,
// at least one); the volume force (gravity) added when the case has it.
ffi::Error RhsImpl(cudaStream_t stream, ffi::Buffer<ffi::F64> prims, ffi::Buffer<ffi::F64> cons,
                   ffi::ResultBuffer<ffi::F64> rhs, ffi::ResultBuffer<ffi::U8> workspace,
                   ffi::Span<const int64_t> desc) {
  gbf_case c;
  int st = unpack(desc, &c);
  if (st == GBF_OK && workspace->size_bytes() < gbf_rhs_workspace_bytes(&c)) st = GBF_ERR_SIZE;
  if (st == GBF_OK)
    st = gbf_rhs_ws(&c, prims.typed_data(), cons.typed_data(), rhs->typed_data(), nullptr,
                    workspace->untyped_data(), stream);
  if (st == GBF_OK && (c.flags & GBF_FLAG_GRAVITY))
    st = gbf_volume_force(&c, cons.typed_data(), rhs->typed_data(), stream);
  return status_error(st);
}

// The initial {dt, t, slots} of the interior conservatives (and, with
// with_prims, of the primitives they were built from).
ffi::Error Rk3InitImpl(cudaStream_t stream, ffi::Buffer<ffi::F64> cons, ffi::Buffer<ffi::F64> prims,
                       ffi::ResultBuffer<ffi::F64> dt_state, ffi::Span<const int64_t> desc, int64_t with_prims,
                       double t0) {
  gbf_case c;
  int st = unpack(desc, &c);
  if (st == GBF_OK)
    st = gbf_rk3_init(&c, cons.typed_data(), with_prims ? prims.typed_data() : nullptr, dt_state->typed_data(), t0,
                      stream);
  return status_error(st);
}

// `steps` fused TVD-RK3 steps of the interior conservatives; the workspace is
// a result of gbf_rk3_workspace_bytes(c) bytes.
ffi::Error Rk3AdvanceImpl(cudaStream_t stream, ffi::Buffer<ffi::F64> cons_in, ffi::Buffer<ffi::F64> prims,
                          ffi::Buffer<ffi::F64> dt_in, ffi::ResultBuffer<ffi::F64> cons_out,
                          ffi::ResultBuffer<ffi::F64> dt_out, ffi::ResultBuffer<ffi::U8> workspace,
                          ffi::Span<const int64_t> desc, int64_t steps, int64_t with_prims) {
  gbf_case c;
  int st = unpack(desc, &c);
  if (st == GBF_OK && workspace->size_bytes() < gbf_rk3_workspace_bytes(&c)) st = GBF_ERR_SIZE;
  if (st == GBF_OK) st = copy_if_distinct(cons_in.typed_data(), cons_out->typed_data(), cons_in.size_bytes(), stream);
  if (st == GBF_OK) st = copy_if_distinct(dt_in.typed_data(), dt_out->typed_data(), dt_in.size_bytes(), stream);
  if (st == GBF_OK)
    st = gbf_rk3_advance(&c, cons_out->typed_data(), with_prims ? prims.typed_data() : nullptr, dt_out->typed_data(),
                         workspace->untyped_data(), (int)steps, nullptr, stream);
  return status_error(st);
}

// VJP of compute_rhs at the interior conservatives: out = J^T w.
ffi::Error RhsVjpImpl(cudaStream_t stream, ffi::Buffer<ffi::F64> cons, ffi::Buffer<ffi::F64> w,
                      ffi::ResultBuffer<ffi::F64> out, ffi::ResultBuffer<ffi::U8> workspace,
                      ffi::Span<const int64_t> desc) {
  gbf_case c;
  int st = unpack(desc, &c);
  if (st == GBF_OK && workspace->size_bytes() < gbf_vjp_workspace_bytes(&c)) st = GBF_ERR_SIZE;
  if (st == GBF_OK)
    st = gbf_rhs_vjp(&c, cons.typed_data(), w.typed_data(), out->typed_data(), workspace->untyped_data(), nullptr,
                     stream);
  return status_error(st);
}

// VJP of one fixed-dt RK3 step (dt a device scalar): lam_out = (dU^{n+1}/dU^n)^T lam.
ffi::Error Rk3StepVjpImpl(cudaStream_t stream, ffi::Buffer<ffi::F64> cons, ffi::Buffer<ffi::F64> dt,
                          ffi::Buffer<ffi::F64> lam, ffi::ResultBuffer<ffi::F64> lam_out,
                          ffi::ResultBuffer<ffi::U8> workspace, ffi::Span<const int64_t> desc) {
  gbf_case c;
  int st = unpack(desc, &c);
  if (st == GBF_OK && workspace->size_bytes() < gbf_vjp_workspace_bytes(&c)) st = GBF_ERR_SIZE;
  if (st == GBF_OK)
    st = gbf_rk3_step_vjp(&c, cons.typed_data(), dt.typed_data(), lam.typed_data(), lam_out->typed_data(),
                          workspace->untyped_data(), nullptr, stream);
  return status_error(st);
}

}  // namespace

XLA_FFI_DEFINE_HANDLER_SYMBOL(gbf_rhs_ffi, RhsImpl,
                              ffi::Ffi::Bind()
                                  .Ctx<ffi::PlatformStream<cudaStream_t>>()
                                  .Arg<ffi::Buffer<ffi::F64>>()   // primitives, halo buffer
                                  .Arg<ffi::Buffer<ffi::F64>>()   // conservatives, halo buffer
                                  .Ret<ffi::Buffer<ffi::F64>>()   // rhs, interior
                                  .Ret<ffi::Buffer<ffi::U8>>()    // workspace
                                  .Attr<ffi::Span<const int64_t>>("desc"));

XLA_FFI_DEFINE_HANDLER_SYMBOL(gbf_rk3_init_ffi, Rk3InitImpl,
                              ffi::Ffi::Bind()
                                  .Ctx<ffi::PlatformStream<cudaStream_t>>()
                                  .Arg<ffi::Buffer<ffi::F64>>()   // conservatives, interior
                                  .Arg<ffi::Buffer<ffi::F64>>()   // primitives, interior (read with with_prims)
                                  .Ret<ffi::Buffer<ffi::F64>>()   // dt_state[4]
                                  .Attr<ffi::Span<const int64_t>>("desc")
                                  .Attr<int64_t>("with_prims")
                                  .Attr<double>("t0"));

XLA_FFI_DEFINE_HANDLER_SYMBOL(gbf_rk3_advance_ffi, Rk3AdvanceImpl,
                              ffi::Ffi::Bind()
                                  .Ctx<ffi::PlatformStream<cudaStream_t>>()
                                  .Arg<ffi::Buffer<ffi::F64>>()   // conservatives, interior
                                  .Arg<ffi::Buffer<ffi::F64>>()   // primitives of the first stage (with_prims)
                                  .Arg<ffi::Buffer<ffi::F64>>()   // dt_state[4]
                                  .Ret<ffi::Buffer<ffi::F64>>()   // conservatives after the steps
                                  .Ret<ffi::Buffer<ffi::F64>>()   // dt_state after the steps
                                  .Ret<ffi::Buffer<ffi::U8>>()    // workspace
                                  .Attr<ffi::Span<const int64_t>>("desc")
                                  .Attr<int64_t>("steps")
                                  .Attr<int64_t>("with_prims"));

XLA_FFI_DEFINE_HANDLER_SYMBOL(gbf_rhs_vjp_ffi, RhsVjpImpl,
                              ffi::Ffi::Bind()
                                  .Ctx<ffi::PlatformStream<cudaStream_t>>()
                                  .Arg<ffi::Buffer<ffi::F64>>()   // conservatives, interior
                                  .Arg<ffi::Buffer<ffi::F64>>()   // cotangent of the rhs
                                  .Ret<ffi::Buffer<ffi::F64>>()   // cotangent of the conservatives
                                  .Ret<ffi::Buffer<ffi::U8>>()    // workspace
                                  .Attr<ffi::Span<const int64_t>>("desc"));

XLA_FFI_DEFINE_HANDLER_SYMBOL(gbf_rk3_step_vjp_ffi, Rk3StepVjpImpl,
                              ffi::Ffi::Bind()
                                  .Ctx<ffi::PlatformStream<cudaStream_t>>()
                                  .Arg<ffi::Buffer<ffi::F64>>()   // U^n, interior
                                  .Arg<ffi::Buffer<ffi::F64>>()   // dt, a scalar
                                  .Arg<ffi::Buffer<ffi::F64>>()   // cotangent of U^{n+1}
                                  .Ret<ffi::Buffer<ffi::F64>>()   // cotangent of U^n
                                  .Ret<ffi::Buffer<ffi::U8>>()    // workspace
                                  .Attr<ffi::Span<const int64_t>>("desc"));
