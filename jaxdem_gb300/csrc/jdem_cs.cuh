// Cundall-Strack pair law (CundallStrackForce.force, jaxdem/forces/cundall_strack.py:100-196),
// shared by the sphere kernels (jdem_cs.cu) and the rigid-clump kernels (jdem_rigid.cu).
#pragma once

#include "jdem_device.cuh"

namespace jdem {

// utils/linalg.py:164-181 (unit_and_norm): rsqrt of max(n2, 1e-16), 0 for a
// zero vector.
__device__ __forceinline__ float cs_inv_norm(float n2) { return n2 == 0.0f ? 0.0f : 1.0f / sqrtf(fmaxf(n2, 1e-16f)); }

// Force on i due to j and torque on i (cundall_strack.py:100-196), both spheres'
// states given; d = minimum-image r_i - r_j.  Adds into the two-sum
// accumulators F (+ eF) and T (+ eT).
template <int DIM>
__device__ __forceinline__ void cs_pair(const Bufs& b, int mi, int mj, float Ri, float Rj, float mi_, float mj_,
                                        const float* vi, const float* vj, const float* wi, const float* wj,
                                        const float* d, float* F, float* eF, float* T, float* eT) {
  constexpr int AD = DIM == 3 ? 3 : 1;
  const float4 pi_ = reinterpret_cast<const float4*>(b.mprop)[mi];
  const float4 pj_ = reinterpret_cast<const float4*>(b.mprop)[mj];
  const float Ei = pi_.x, Ej = pj_.x, Gi = pi_.y, Gj = pj_.y;
  // effective properties
  const float kn = (2.0f * Ei * Ri * Ej * Rj) / (Ei * Ri + Ej * Rj);
  const float kt = (2.0f * Gi * Ri * Gj * Rj) / (Gi * Ri + Gj * Rj);
  const float m_eff = (mi_ * mj_) / (mi_ + mj_);
  const float mu_eff = fminf(pi_.z, pj_.z);
  const float beta = b.young[mi * b.n_mat + mj];
  const float gamma_n = 2.0f * beta * sqrtf(kn * m_eff);
  const float gamma_t = 2.0f * beta * sqrtf(kt * m_eff);
  // geometry: (n, r) = unit_and_norm(r_ij)
  float n2 = d[0] * d[0] + d[1] * d[1];
  if (DIM == 3) n2 = n2 + d[2] * d[2];
  const float inv = cs_inv_norm(n2);
  const float r = n2 * inv;
  float n[3] = {d[0] * inv, d[1] * inv, DIM == 3 ? d[2] * inv : 0.0f};
  float delta = Ri + Rj - r;
  const float contact = delta > 0.0f ? 1.0f : 0.0f;
  delta = delta * contact;
  // contact-point arms and velocities (cross_3X3D_1X2D)
  float rci[3], rcj[3], vci[3], vcj[3];
  for (int a = 0; a < DIM; ++a) {
    rci[a] = -Ri * n[a];
    rcj[a] = Rj * n[a];
  }
  if (DIM == 3) {
    vci[0] = vi[0] + (wi[1] * rci[2] - wi[2] * rci[1]);
    vci[1] = vi[1] + (wi[2] * rci[0] - wi[0] * rci[2]);
    vci[2] = vi[2] + (wi[0] * rci[1] - wi[1] * rci[0]);
    vcj[0] = vj[0] + (wj[1] * rcj[2] - wj[2] * rcj[1]);
    vcj[1] = vj[1] + (wj[2] * rcj[0] - wj[0] * rcj[2]);
    vcj[2] = vj[2] + (wj[0] * rcj[1] - wj[1] * rcj[0]);
  } else {
    vci[0] = vi[0] + -wi[0] * rci[1];
    vci[1] = vi[1] + wi[0] * rci[0];
    vcj[0] = vj[0] + -wj[0] * rcj[1];
    vcj[1] = vj[1] + wj[0] * rcj[0];
  }
  float vrel[3], vt_vec[3];
  for (int a = 0; a < DIM; ++a) vrel[a] = vci[a] - vcj[a];
  float vn = vrel[0] * n[0] + vrel[1] * n[1];
  if (DIM == 3) vn = vn + vrel[2] * n[2];
  for (int a = 0; a < DIM; ++a) vt_vec[a] = vrel[a] - vn * n[a];
  float t2 = vt_vec[0] * vt_vec[0] + vt_vec[1] * vt_vec[1];
  if (DIM == 3) t2 = t2 + vt_vec[2] * vt_vec[2];
  const float tinv = cs_inv_norm(t2);
  const float vt = t2 * tinv;
  // normal force (strictly repulsive), tangential dashpot capped by Coulomb
  const float Fn = fmaxf(0.0f, kn * delta - gamma_n * vn) * contact;
  const float Ft = fminf(gamma_t * vt, mu_eff * Fn) * contact;
  float f[3], tq[3];
  for (int a = 0; a < DIM; ++a) f[a] = Fn * n[a] - Ft * (vt_vec[a] * tinv);
  // torque = cross(r_ci, F) - mu_r R_eff Fn unit(w_i - w_j)
  if (DIM == 3) {
    tq[0] = rci[1] * f[2] - rci[2] * f[1];
    tq[1] = rci[2] * f[0] - rci[0] * f[2];
    tq[2] = rci[0] * f[1] - rci[1] * f[0];
  } else {
    tq[0] = rci[0] * f[1] - rci[1] * f[0];
  }
  const float mu_r = fminf(pi_.w, pj_.w);
  const float R_eff = (Ri * Rj) / (Ri + Rj);
  float wr[3], w2 = 0.0f;
  for (int a = 0; a < AD; ++a) {
    wr[a] = wi[a] - wj[a];
    w2 = a == 0 ? wr[a] * wr[a] : w2 + wr[a] * wr[a];
  }
  // unit(): rsqrt of n2, with 1 in place of a zero n2 (utils/linalg.py:136-161)
  const float winv = 1.0f / sqrtf(w2 == 0.0f ? 1.0f : w2);
  const float roll = mu_r * R_eff * Fn;
  for (int a = 0; a < AD; ++a) tq[a] = tq[a] - roll * (wr[a] * winv);
  for (int a = 0; a < DIM; ++a) two_sum_acc(F[a], eF[a], f[a]);
  for (int a = 0; a < AD; ++a) two_sum_acc(T[a], eT[a], tq[a]);
}

}  // namespace jdem
