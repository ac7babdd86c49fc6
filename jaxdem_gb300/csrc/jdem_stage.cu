// Integrator stages on caller device buffers (jdem_integrate): the split
// factory types' step_before_force / step_after_force
// (integrators/__init__.py:51-91) for callers that run the reference's own
// stage order and need one stage at a time.  One thread per particle, the
// arithmetic of the fused step kernels in the same operation order:
//   VelocityVerlet    velocity_verlet.py:29-61 (before), 66-95 (after)
//   DirectEuler       direct_euler.py:30-66 (after; before is the base no-op)
//   VelocityVerletSpiral, Spiral: rot_before / rot_after of jdem_rot.cuh
#include <cstdint>

#include "../../include/jdem_gb300.h"
#include "jdem_device.cuh"
#include "jdem_rot.cuh"

namespace jdem {
namespace {

template <int DIM>
__global__ void k_stage(long long n, int linear, int rotation, int stage, float dt, float* __restrict__ pos,
                        float* __restrict__ vel, const float* __restrict__ force, const float* __restrict__ mass,
                        const uint8_t* __restrict__ fixed, float4* __restrict__ q, float* __restrict__ angv,
                        const float* __restrict__ torque, const float* __restrict__ inertia) {
  constexpr int AD = DIM == 3 ? 3 : 1;
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float fr = (fixed && fixed[i]) ? 0.0f : 1.0f;
  // linear: v += F (dt * 0.5 / m) free, then pos_c += dt v (VV before); v += F (dt / m) free,
  // pos_c += dt v (Euler after); v += F (dt * 0.5 / m) free (VV after)
  const bool vv = linear == LIN_VERLET, eu = linear == LIN_EULER;
  if ((vv && (stage == 0 || stage == 1)) || (eu && stage == 1)) {
    const float m = mass[i];
    const float sc = vv ? dt * 0.5f / m : dt / m;
    const bool drift = (vv && stage == 0) || eu;
#pragma unroll
    for (int a = 0; a < DIM; ++a) {
      const float v = vel[i * DIM + a] + force[i * DIM + a] * sc * fr;
      vel[i * DIM + a] = v;
      if (drift) pos[i * DIM + a] = pos[i * DIM + a] + dt * v;
    }
  }
  const bool rot_now = (rotation == ROT_VVSPIRAL) || (rotation == ROT_SPIRAL && stage == 1);
  if (rot_now) {
    float4 qq = q[i];
    float w[3] = {0, 0, 0}, tq[3] = {0, 0, 0}, I[3] = {1, 1, 1}, invI[3] = {1, 1, 1};
#pragma unroll
    for (int a = 0; a < AD; ++a) {
      w[a] = angv[i * AD + a];
      tq[a] = torque[i * AD + a];
      I[a] = inertia[i * AD + a];
      invI[a] = 1.0f / I[a];
    }
    if (stage == 0) rot_before<DIM>(rotation, dt, qq, w, tq, I, invI, fr);
    else rot_after<DIM>(rotation, dt, qq, w, tq, I, invI, fr);
    q[i] = qq;
#pragma unroll
    for (int a = 0; a < AD; ++a) angv[i * AD + a] = w[a];
  }
}

}  // namespace
}  // namespace jdem

extern "C" int jdem_integrate(int32_t dim, int64_t n, int32_t linear, int32_t rotation, int32_t stage, float dt,
                              float* pos_c, float* vel, const float* force, const float* mass, const uint8_t* fixed,
                              float* q, float* ang_vel, const float* torque, const float* inertia, void* stream) {
  using namespace jdem;
  if ((dim != 2 && dim != 3) || n < 0 || (stage != 0 && stage != 1)) return JDEM_ERR_BAD_ARG;
  if (linear < JDEM_LIN_NONE || linear > JDEM_LIN_EULER || rotation < JDEM_ROT_NONE || rotation > JDEM_ROT_SPIRAL)
    return JDEM_ERR_BAD_ARG;
  if (n == 0) return JDEM_OK;
  if (linear != JDEM_LIN_NONE && (!pos_c || !vel || !force || !mass)) return JDEM_ERR_BAD_ARG;
  if (rotation != JDEM_ROT_NONE && (!q || !ang_vel || !torque || !inertia)) return JDEM_ERR_BAD_ARG;
  if (!(dt == dt)) return JDEM_ERR_BAD_ARG;
  if ((reinterpret_cast<uintptr_t>(q) & 15u) != 0u) return JDEM_ERR_BAD_ARG;  // q is read as float4
  const cudaStream_t st = static_cast<cudaStream_t>(stream);
  const unsigned int grid = (unsigned int)((n + 255) / 256);
  if (dim == 3)
    k_stage<3><<<grid, 256, 0, st>>>(n, linear, rotation, stage, dt, pos_c, vel, force, mass, fixed,
                                     reinterpret_cast<float4*>(q), ang_vel, torque, inertia);
  else
    k_stage<2><<<grid, 256, 0, st>>>(n, linear, rotation, stage, dt, pos_c, vel, force, mass, fixed,
                                     reinterpret_cast<float4*>(q), ang_vel, torque, inertia);
  return cudaGetLastError() == cudaSuccess ? JDEM_OK : JDEM_ERR_CUDA;
}
