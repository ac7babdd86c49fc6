// XLA FFI handlers over the C ABI (include/jdem_gb300.h): the custom calls a
// JaxDEM build with jaxlib registers for the fused step and for the collider's
// compute_force.
//
//   JdemStep   System.step(state, system, n)       jaxdem/system.py:701-748
//   JdemForce  DynamicCellList.compute_force       jaxdem/colliders/cell_list.py:434-464
//
// XLA owns the buffers and orders the custom call on its compute stream; each
// handler points the engine handle at that stream (jdem_set_stream), reads the
// inputs from XLA's device buffers and writes the results into XLA's result
// buffers with stream-ordered copies, so producers and consumers on the stream
// need no host synchronisation.  The handle (a JdemHandle* created through the
// C ABI for the system's shape and parameters) is passed as an int64 attribute.
//
// Compiled only where jaxlib's FFI headers are found (jax.ffi.include_dir()):
// jaxdem_gb300/build.py builds it into _lib/libjdem_xla_ffi.so when
// JDEM_JAX_INCLUDE names that directory or jax is importable.  Without them
// this translation unit is empty.
#if __has_include("xla/ffi/api/ffi.h")

#include <cuda_runtime.h>

#include <cstdint>

#include "jdem_gb300.h"
#include "xla/ffi/api/ffi.h"

namespace ffi = xla::ffi;

namespace {

ffi::Error engine_error(JdemHandle* h, int rc) {
  return ffi::Error(rc == JDEM_ERR_BAD_ARG ? ffi::ErrorCode::kInvalidArgument
                    : rc == JDEM_ERR_OOM  ? ffi::ErrorCode::kResourceExhausted
                    : rc == JDEM_ERR_UNSUPPORTED ? ffi::ErrorCode::kUnimplemented
                                                 : ffi::ErrorCode::kInternal,
                    jdem_last_error(h));
}

// (N, dim) positions, velocities, forces and (N) radii, masses: the element
// counts must agree with the handle's particle count.
bool shapes_ok(const JdemHandle* h, int64_t n_pos, int64_t n_rad) {
  int64_t n = 0;
  int32_t dim = 0;
  if (jdem_shape(h, &n, &dim) != JDEM_OK) return false;
  return n_rad == n && n_pos == n * dim;
}

ffi::Error StepImpl(cudaStream_t stream, int64_t handle, int64_t n, ffi::Buffer<ffi::F32> pos,
                    ffi::Buffer<ffi::F32> vel, ffi::Buffer<ffi::F32> force, ffi::Buffer<ffi::F32> rad,
                    ffi::Buffer<ffi::F32> mass, ffi::ResultBuffer<ffi::F32> pos_out,
                    ffi::ResultBuffer<ffi::F32> vel_out, ffi::ResultBuffer<ffi::F32> force_out) {
  auto* h = reinterpret_cast<JdemHandle*>(handle);
  if (!h) return ffi::Error(ffi::ErrorCode::kInvalidArgument, "jdem_step: null handle");
  if (!shapes_ok(h, (int64_t)pos.element_count(), (int64_t)rad.element_count()) ||
      vel.element_count() != pos.element_count() || force.element_count() != pos.element_count() ||
      mass.element_count() != rad.element_count())
    return ffi::Error(ffi::ErrorCode::kInvalidArgument, "jdem_step: buffer shapes do not match the handle");
  int rc = jdem_set_stream(h, (void*)stream);
  if (rc) return engine_error(h, rc);
  JdemHostState in{};
  in.pos_c = pos.typed_data();
  in.vel = vel.typed_data();
  in.force = force.typed_data();
  in.rad = rad.typed_data();
  in.mass = mass.typed_data();
  if ((rc = jdem_upload_device(h, &in))) return engine_error(h, rc);
  if ((rc = jdem_step_async(h, n))) return engine_error(h, rc);
  JdemHostState out{};
  out.pos_c = pos_out->typed_data();
  out.vel = vel_out->typed_data();
  out.force = force_out->typed_data();
  if ((rc = jdem_download_device_async(h, &out))) return engine_error(h, rc);
  return ffi::Error::Success();
}

ffi::Error ForceImpl(cudaStream_t stream, int64_t handle, ffi::Buffer<ffi::F32> pos, ffi::Buffer<ffi::F32> rad,
                     ffi::Buffer<ffi::F32> mass, ffi::ResultBuffer<ffi::F32> force_out) {
  auto* h = reinterpret_cast<JdemHandle*>(handle);
  if (!h) return ffi::Error(ffi::ErrorCode::kInvalidArgument, "jdem_force: null handle");
  if (!shapes_ok(h, (int64_t)pos.element_count(), (int64_t)rad.element_count()) ||
      mass.element_count() != rad.element_count())
    return ffi::Error(ffi::ErrorCode::kInvalidArgument, "jdem_force: buffer shapes do not match the handle");
  int rc = jdem_set_stream(h, (void*)stream);
  if (rc) return engine_error(h, rc);
  JdemHostState in{};
  in.pos_c = pos.typed_data();
  in.rad = rad.typed_data();
  in.mass = mass.typed_data();
  if ((rc = jdem_upload_device(h, &in))) return engine_error(h, rc);
  if ((rc = jdem_compute_force(h))) return engine_error(h, rc);
  JdemHostState out{};
  out.force = force_out->typed_data();
  if ((rc = jdem_download_device_async(h, &out))) return engine_error(h, rc);
  return ffi::Error::Success();
}

}  // namespace

XLA_FFI_DEFINE_HANDLER_SYMBOL(JdemStep, StepImpl,
                              ffi::Ffi::Bind()
                                  .Ctx<ffi::PlatformStream<cudaStream_t>>()
                                  .Attr<int64_t>("handle")
                                  .Attr<int64_t>("n")
                                  .Arg<ffi::Buffer<ffi::F32>>()  // pos_c (N, dim)
                                  .Arg<ffi::Buffer<ffi::F32>>()  // vel (N, dim)
                                  .Arg<ffi::Buffer<ffi::F32>>()  // force (N, dim)
                                  .Arg<ffi::Buffer<ffi::F32>>()  // rad (N)
                                  .Arg<ffi::Buffer<ffi::F32>>()  // mass (N)
                                  .Ret<ffi::Buffer<ffi::F32>>()  // pos_c
                                  .Ret<ffi::Buffer<ffi::F32>>()  // vel
                                  .Ret<ffi::Buffer<ffi::F32>>()  // force
);

XLA_FFI_DEFINE_HANDLER_SYMBOL(JdemForce, ForceImpl,
                              ffi::Ffi::Bind()
                                  .Ctx<ffi::PlatformStream<cudaStream_t>>()
                                  .Attr<int64_t>("handle")
                                  .Arg<ffi::Buffer<ffi::F32>>()  // pos_c (N, dim)
                                  .Arg<ffi::Buffer<ffi::F32>>()  // rad (N)
                                  .Arg<ffi::Buffer<ffi::F32>>()  // mass (N)
                                  .Ret<ffi::Buffer<ffi::F32>>()  // force (N, dim)
);

#endif  // __has_include("xla/ffi/api/ffi.h")
