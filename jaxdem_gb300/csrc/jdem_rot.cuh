// Rotational integrators of a sphere, one phase at a time, shared by k_rot
// (torque-free spheres, n steps in registers) and the Cundall-Strack step
// kernels (torque from the contacts every step).
//   VelocityVerletSpiral: velocity_verlet_spiral.py:83-116 (before), 156-180 (after)
//   Spiral:               spiral.py:56-144 (after)
//   omega_dot:            spiral.py:22-40
// Angular velocity and torque are lab-frame vectors (3D) or the z component
// (2D); the integrators advance the body-frame angular velocity.
#pragma once
#include "jdem_device.cuh"

namespace jdem {

template <int DIM>
__device__ __forceinline__ void omega_dot3(const float* w, const float* tq, const float* I,
                                           const float* invI, float* out) {
  if (DIM == 3) {
    float cx = w[1] * (I[2] * w[2]) - w[2] * (I[1] * w[1]);
    float cy = w[2] * (I[0] * w[0]) - w[0] * (I[2] * w[2]);
    float cz = w[0] * (I[1] * w[1]) - w[1] * (I[0] * w[0]);
    out[0] = (tq[0] - cx) * invI[0];
    out[1] = (tq[1] - cy) * invI[1];
    out[2] = (tq[2] - cz) * invI[2];
  } else {
    out[0] = tq[0] * invI[0];
  }
}

template <int DIM>
__device__ void ssprk3(float h, const float* w, const float* tq, const float* I, const float* invI,
                       float fr, float* wout) {
  constexpr int AD = DIM == 3 ? 3 : 1;
  float k1[3], k2[3], k3[3], tmp[3];
  omega_dot3<DIM>(w, tq, I, invI, k1);
  for (int a = 0; a < AD; ++a) {
    k1[a] = h * k1[a];
    tmp[a] = w[a] + k1[a];
  }
  omega_dot3<DIM>(tmp, tq, I, invI, k2);
  for (int a = 0; a < AD; ++a) {
    k2[a] = h * k2[a];
    tmp[a] = w[a] + 0.25f * (k1[a] + k2[a]);
  }
  omega_dot3<DIM>(tmp, tq, I, invI, k3);
  for (int a = 0; a < AD; ++a) {
    k3[a] = h * k3[a];
    wout[a] = w[a] + fr * (k1[a] + k2[a] + 4.0f * k3[a]) / 6.0f;
  }
}

// ReflectDomain.apply's orientation update of a sphere: q <- unit(dq q) with
// dq = from_small_rotvec(0) (reflect.py:291-294).
__device__ __forceinline__ float4 reflect_q(float4 qq) {
  return q_unit(q_mul(make_float4(1.0f - 0.0f / 8.0f, 0.0f, 0.0f, 0.0f), qq));
}

// step_before_force: the half step of the body-frame angular velocity under
// the torque tq, then q <- unit(q dq(dt w)) and w back in the lab frame.
// Only VelocityVerletSpiral has a before-force phase.
template <int DIM>
__device__ __forceinline__ void rot_before(int rot, float dt, float4& qq, float* w, const float* tq, const float* I,
                                           const float* invI, float fr) {
  if (rot != ROT_VVSPIRAL) return;
  float dt_2 = dt / 2.0f;
  float wb[3], tb[3], wn[3];
  if (DIM == 3) {
    q_rotate3(qq, -1.0f, w, wb);
    q_rotate3(qq, -1.0f, tq, tb);
  } else {
    wb[0] = w[0];
    tb[0] = tq[0];
  }
  ssprk3<DIM>(dt_2, wb, tb, I, invI, fr, wn);
  float rv[3];
  if (DIM == 3) {
    for (int a = 0; a < 3; ++a) rv[a] = 2.0f * dt_2 * wn[a];
  } else {
    float r = 2.0f * dt_2 * wn[0];
    rv[0] = 0.0f * r;
    rv[1] = 0.0f * r;
    rv[2] = 1.0f * r;
  }
  float4 dq = q_small_rotvec(rv[0], rv[1], rv[2]);
  qq = q_unit(q_mul(qq, dq));
  if (DIM == 3) q_rotate3(qq, 1.0f, wn, w);
  else w[0] = wn[0];
}

// step_after_force under the torque tq (nullptr: zero torque, the body-frame
// torque is then exactly 0).
template <int DIM>
__device__ __forceinline__ void rot_after(int rot, float dt, float4& qq, float* w, const float* tq, const float* I,
                                          const float* invI, float fr) {
  constexpr int AD = DIM == 3 ? 3 : 1;
  if (rot == ROT_VVSPIRAL) {
    float dt_2 = dt / 2.0f;
    float wb[3], tb[3] = {0, 0, 0}, wn[3];
    if (DIM == 3) {
      q_rotate3(qq, -1.0f, w, wb);
      if (tq) q_rotate3(qq, -1.0f, tq, tb);
    } else {
      wb[0] = w[0];
      if (tq) tb[0] = tq[0];
    }
    ssprk3<DIM>(dt_2, wb, tb, I, invI, fr, wn);
    if (DIM == 3) q_rotate3(qq, 1.0f, wn, w);
    else w[0] = wn[0];
  } else if (rot == ROT_SPIRAL) {
    float dt_2 = dt / 2.0f;
    float wb[3], tb[3] = {0, 0, 0}, wd[3], tmp[3], k1[3], k2[3], k3[3];
    if (DIM == 3) {
      q_rotate3(qq, -1.0f, w, wb);
      if (tq) q_rotate3(qq, -1.0f, tq, tb);
    } else {
      wb[0] = w[0];
      if (tq) tb[0] = tq[0];
    }
    omega_dot3<DIM>(wb, tb, I, invI, wd);
    float rv1[3], rv2[3];
    if (DIM == 3) {
      for (int a = 0; a < 3; ++a) {
        rv1[a] = 2.0f * dt_2 * wb[a];
        rv2[a] = 2.0f * dt_2 * dt_2 * wd[a];
      }
    } else {
      float r1 = 2.0f * dt_2 * wb[0], r2 = 2.0f * dt_2 * dt_2 * wd[0];
      rv1[0] = 0.0f * r1; rv1[1] = 0.0f * r1; rv1[2] = 1.0f * r1;
      rv2[0] = 0.0f * r2; rv2[1] = 0.0f * r2; rv2[2] = 1.0f * r2;
    }
    float4 dq = q_mul(q_small_rotvec(rv1[0], rv1[1], rv1[2]), q_small_rotvec(rv2[0], rv2[1], rv2[2]));
    qq = q_unit(q_mul(qq, dq));
    for (int a = 0; a < AD; ++a) {
      k1[a] = dt * wd[a];
      tmp[a] = wb[a] + k1[a];
    }
    omega_dot3<DIM>(tmp, tb, I, invI, k2);
    for (int a = 0; a < AD; ++a) {
      k2[a] = dt * k2[a];
      tmp[a] = wb[a] + 0.25f * (k1[a] + k2[a]);
    }
    omega_dot3<DIM>(tmp, tb, I, invI, k3);
    float wn[3];
    for (int a = 0; a < AD; ++a) {
      k3[a] = dt * k3[a];
      wn[a] = wb[a] + fr * (k1[a] + k2[a] + 4.0f * k3[a]) / 6.0f;
    }
    if (DIM == 3) q_rotate3(qq, 1.0f, wn, w);
    else w[0] = wn[0];
  }
}

}  // namespace jdem
