// The stages of System.step (system.py:60-82) one at a time on caller device
// buffers, for the split factory types (callers that run the reference's own
// stage order): Domain.apply (jdem_domain_apply), the integrators'
// step_before_force / step_after_force (jdem_integrate) and ForceManager.apply
// (jdem_force_manager_apply), for spheres; the collider's stage is
// jdem_compute_force.  One thread per particle, the arithmetic of the fused
// step kernels in the same operation order:
//   VelocityVerlet    velocity_verlet.py:29-61 (before), 66-95 (after)
//   DirectEuler       direct_euler.py:30-66 (after; before is the base no-op)
//   VelocityVerletSpiral, Spiral: rot_before / rot_after of jdem_rot.cuh
//   ReflectDomain     reflect_sphere of jdem_device.cuh; FreeDomain free.py:40-63
#include <cstdint>
#include <cstring>

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

// ReflectDomain.apply for spheres (reflect.py:99-299 with clump_id == iota,
// pos_p == 0: reflect_sphere), with the orientation renormalisation of
// reflect.py:291-294 when q is given.
template <int DIM>
__global__ void k_stage_reflect(long long n, SysParams sp, float* __restrict__ pos, float* __restrict__ vel,
                                const float* __restrict__ force, const float* __restrict__ rad,
                                const float* __restrict__ mass, const uint8_t* __restrict__ fixed,
                                float4* __restrict__ q) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  float p[DIM], v[DIM], F[DIM];
#pragma unroll
  for (int a = 0; a < DIM; ++a) {
    p[a] = pos[i * DIM + a];
    v[a] = vel[i * DIM + a];
    F[a] = force[i * DIM + a];
  }
  reflect_sphere<DIM>(sp, p, v, F, rad[i], mass[i], fixed && fixed[i]);
#pragma unroll
  for (int a = 0; a < DIM; ++a) {
    pos[i * DIM + a] = p[a];
    vel[i * DIM + a] = v[a];
  }
  if (q) q[i] = reflect_q(q[i]);
}

// FreeDomain.apply (free.py:59-63): min and max of pos_c -+ (|pos_p| + rad)
// per axis, as order-preserving uints (bb[0..DIM) min, bb[3..3 + DIM) max).
template <int DIM>
__global__ void k_stage_bbox(long long n, const float* __restrict__ pos, const float* __restrict__ rad,
                             const float* __restrict__ pos_p, unsigned int* __restrict__ bb) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  float lo[DIM], hi[DIM];
#pragma unroll
  for (int a = 0; a < DIM; ++a) {
    lo[a] = INFINITY;
    hi[a] = -INFINITY;
  }
  if (i < n) {
    float nrm = 0.0f;
    if (pos_p) {
      float s2 = pos_p[i * DIM] * pos_p[i * DIM];
#pragma unroll
      for (int a = 1; a < DIM; ++a) s2 = s2 + pos_p[i * DIM + a] * pos_p[i * DIM + a];
      nrm = sqrtf(s2);
    }
    const float br = nrm + rad[i];
#pragma unroll
    for (int a = 0; a < DIM; ++a) {
      lo[a] = pos[i * DIM + a] - br;
      hi[a] = pos[i * DIM + a] + br;
    }
  }
#pragma unroll
  for (int a = 0; a < DIM; ++a) {
    float l = lo[a], h = hi[a];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      l = fminf(l, __shfl_xor_sync(0xffffffffu, l, o));
      h = fmaxf(h, __shfl_xor_sync(0xffffffffu, h, o));
    }
    if ((threadIdx.x & 31) == 0) {
      atomicMin(&bb[a], f2ord(l));
      atomicMax(&bb[3 + a], f2ord(h));
    }
  }
}

__global__ void k_stage_bbox_init(unsigned int* bb) {
  if (threadIdx.x < 6) bb[threadIdx.x] = threadIdx.x < 3 ? 0xFFFFFFFFu : 0u;
}

// ForceManager.apply for spheres (force_manager.py:338-425 with
// clump_id == iota: count 1, zero lever arms, identity segment sums):
// F = (F_contact + F_ext) + (F_com + g (m / 1)), T = T_contact + (T_ext + 0).
template <int DIM>
__global__ void k_stage_fm(long long n, float g0, float g1, float g2, float* __restrict__ force,
                           float* __restrict__ torque, const float* __restrict__ ext_f,
                           const float* __restrict__ ext_fc, const float* __restrict__ ext_t,
                           const float* __restrict__ mass) {
  constexpr int AD = DIM == 3 ? 3 : 1;
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float g[3] = {g0, g1, g2};
  const float m = mass[i];
#pragma unroll
  for (int a = 0; a < DIM; ++a) {
    const float fp = ext_f ? ext_f[i * DIM + a] : 0.0f;
    const float fc = (ext_fc ? ext_fc[i * DIM + a] : 0.0f) + g[a] * (m / 1.0f);
    force[i * DIM + a] = (force[i * DIM + a] + fp) + fc;
  }
  if (torque) {
#pragma unroll
    for (int a = 0; a < AD; ++a) torque[i * AD + a] = torque[i * AD + a] + ((ext_t ? ext_t[i * AD + a] : 0.0f) + 0.0f);
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

extern "C" int jdem_domain_apply(int32_t dim, int64_t n, int32_t domain, float dt, float restitution,
                                 const float* box_size, const float* anchor, float* pos_c, float* vel,
                                 const float* force, const float* rad, const float* mass, const uint8_t* fixed,
                                 const float* pos_p, float* q, float* box_out, float* anchor_out, void* stream) {
  using namespace jdem;
  if ((dim != 2 && dim != 3) || n < 0 || domain < JDEM_DOMAIN_FREE || domain > JDEM_DOMAIN_REFLECT)
    return JDEM_ERR_BAD_ARG;
  if (domain == JDEM_DOMAIN_PERIODIC || n == 0) return JDEM_OK;  // Domain.apply: nothing to do
  const cudaStream_t st = static_cast<cudaStream_t>(stream);
  const unsigned int grid = (unsigned int)((n + 255) / 256);
  if (domain == JDEM_DOMAIN_REFLECT) {
    if (!box_size || !anchor || !pos_c || !vel || !force || !rad || !mass) return JDEM_ERR_BAD_ARG;
    if ((reinterpret_cast<uintptr_t>(q) & 15u) != 0u) return JDEM_ERR_BAD_ARG;
    SysParams sp{};
    for (int a = 0; a < dim; ++a) {
      sp.box[a] = box_size[a];
      sp.anchor[a] = anchor[a];
    }
    sp.dt = dt;
    sp.restitution = restitution;
    sp.domain = DOM_REFLECT;
    if (dim == 3)
      k_stage_reflect<3><<<grid, 256, 0, st>>>(n, sp, pos_c, vel, force, rad, mass, fixed, reinterpret_cast<float4*>(q));
    else
      k_stage_reflect<2><<<grid, 256, 0, st>>>(n, sp, pos_c, vel, force, rad, mass, fixed, reinterpret_cast<float4*>(q));
    return cudaGetLastError() == cudaSuccess ? JDEM_OK : JDEM_ERR_CUDA;
  }
  // free: the bounding box, read back to the host
  if (!pos_c || !rad || !box_out || !anchor_out) return JDEM_ERR_BAD_ARG;
  unsigned int* bb = nullptr;
  if (cudaMallocAsync((void**)&bb, 6 * sizeof(unsigned int), st) != cudaSuccess) {
    cudaGetLastError();
    return JDEM_ERR_OOM;
  }
  unsigned int h[6] = {0, 0, 0, 0, 0, 0};
  k_stage_bbox_init<<<1, 32, 0, st>>>(bb);
  if (dim == 3) k_stage_bbox<3><<<grid, 256, 0, st>>>(n, pos_c, rad, pos_p, bb);
  else k_stage_bbox<2><<<grid, 256, 0, st>>>(n, pos_c, rad, pos_p, bb);
  cudaError_t e = cudaMemcpyAsync(h, bb, sizeof(h), cudaMemcpyDeviceToHost, st);
  const cudaError_t e2 = cudaFreeAsync(bb, st);
  if (e == cudaSuccess) e = e2;
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return JDEM_ERR_CUDA;
  }
  auto dec = [](unsigned int u) {  // inverse of the device's order-preserving encoding (f2ord)
    const unsigned int v = (u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u;
    float f;
    std::memcpy(&f, &v, sizeof(f));
    return f;
  };
  for (int a = 0; a < dim; ++a) {
    const float lo = dec(h[a]), hi = dec(h[3 + a]);
    box_out[a] = hi - lo;
    anchor_out[a] = lo;
  }
  return JDEM_OK;
}

extern "C" int jdem_force_manager_apply(int32_t dim, int64_t n, const float* gravity, float* force, float* torque,
                                        const float* external_force, const float* external_force_com,
                                        const float* external_torque, const float* mass, void* stream) {
  using namespace jdem;
  if ((dim != 2 && dim != 3) || n < 0) return JDEM_ERR_BAD_ARG;
  if (n == 0) return JDEM_OK;
  if (!gravity || !force || !mass) return JDEM_ERR_BAD_ARG;
  const cudaStream_t st = static_cast<cudaStream_t>(stream);
  const unsigned int grid = (unsigned int)((n + 255) / 256);
  const float g2 = dim == 3 ? gravity[2] : 0.0f;
  if (dim == 3)
    k_stage_fm<3><<<grid, 256, 0, st>>>(n, gravity[0], gravity[1], g2, force, torque, external_force,
                                        external_force_com, external_torque, mass);
  else
    k_stage_fm<2><<<grid, 256, 0, st>>>(n, gravity[0], gravity[1], g2, force, torque, external_force,
                                        external_force_com, external_torque, mass);
  return cudaGetLastError() == cudaSuccess ? JDEM_OK : JDEM_ERR_CUDA;
}
