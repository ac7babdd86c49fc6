// Cundall-Strack contacts (CundallStrackForce, jaxdem/forces/cundall_strack.py:22-242).
//
// The law depends on the velocities and angular velocities of both spheres
// and exerts torques, so the rotational integrator runs every step and a
// sphere's neighbours must not change while its force is summed.  A step is
// therefore two kernels instead of the fused one:
//   k_cs_force  contact force and torque of every slot from its Verlet-list
//               row (or the stencil cells), reading positions, velocities and
//               angular velocities that nothing writes during the kernel;
//   k_cs_step   ForceManager, step_after_force of both integrators, then (in
//               MODE_STEP) the next step's domain.apply, step_before_force and
//               drift, exactly as the fused kernel orders them.
// k_cs_rot_pre is the rotational half of the first step of a call (k_pre
// does the translational half).  The model is stateless (no tangential
// history): the tangential force is the viscous dashpot capped by Coulomb
// friction, plus a rolling-friction torque.
#include "jdem_device.cuh"
#include "jdem_kernels.h"
#include "jdem_cs.cuh"
#include "jdem_pair.cuh"
#include "jdem_rot.cuh"

namespace jdem {

namespace {

unsigned int nblk_cs(long long n, int t) { return (unsigned int)((n + t - 1) / t); }

}  // namespace

// Contact force and torque of every slot.  Writes frc[sel] (contact force
// only; k_cs_step adds gravity) and the caller-order torque.
template <int DIM>
__global__ void k_cs_force(Bufs b) {
  constexpr int AD = DIM == 3 ? 3 : 1;
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= b.P) return;
  const unsigned int sel = ld_nc_u32(&b.ctl->sel), ps = ld_nc_u32(&b.ctl->pos_sel);
  const bool use_list = b.nl_cap > 0 && (ld_nc_u32(&b.ctl->status) & ST_NL_OVERFLOW) == 0u;
  const float4* __restrict__ P = b.pos[ps];
  const float4 pi = P[t];
  const float4 vi4 = b.vel[sel][t];
  const uint32_t tg = b.tag[sel][t];
  const SysParams& sp = b.sys[tg & TAG_SYS_MASK];
  const bool per = sp.domain == DOM_PERIODIC;
  const int mi = (tg >> TAG_MAT_SHIFT) & TAG_MAT_MASK;
  const int oi = b.orig[sel][t];
  if (!idx_ok(b.ctl, oi, b.P)) return;
  const float vi[3] = {vi4.x, vi4.y, vi4.z};
  float wi[3] = {0.0f, 0.0f, 0.0f};
  for (int a = 0; a < AD; ++a) wi[a] = b.rw[(long long)oi * AD + a];
  float F[3] = {0, 0, 0}, eF[3] = {0, 0, 0}, T[3] = {0, 0, 0}, eT[3] = {0, 0, 0};
  auto visit = [&](int j, bool may_wrap) {
    if (!idx_ok(b.ctl, j, b.P)) return;
    const float4 pj = P[j];
    float d[3];
    const float dsq = pair_disp<DIM>(sp, per && may_wrap, pi, pj, d[0], d[1], d[2]);
    const float R = pi.w + pj.w;
    if (!(dsq < R * R * 1.000001f)) return;
    const int oj = b.orig[sel][j];
    if (b.bond_w > 0 && !b.interact_same_bond) {
      bool bonded = false;
      for (int w = 0; w < b.bond_w; ++w) bonded |= (b.bond[(long long)oi * b.bond_w + w] == oj);
      if (bonded) return;
    }
    const float4 vj4 = b.vel[sel][j];
    const int mj = (b.tag[sel][j] >> TAG_MAT_SHIFT) & TAG_MAT_MASK;
    const float vj[3] = {vj4.x, vj4.y, vj4.z};
    float wj[3] = {0.0f, 0.0f, 0.0f};
    for (int a = 0; a < AD; ++a) wj[a] = b.rw[(long long)oj * AD + a];
    cs_pair<DIM>(b, mi, mj, pi.w, pj.w, vi4.w, vj4.w, vi, vj, wi, wj, d, F, eF, T, eT);
  };
  if (use_list) {
    int n = b.ncnt[t];
    if (!idx_ok(b.ctl, n, (long long)b.nl_cap + 1)) n = 0;
    const int32_t* nb = b.nbr + ((t >> 5) * b.nl_cap) * 32 + (t & 31);
    prefetch_list_block(b, t, n);
    for (int k = 0; k < n; ++k) {
      const uint32_t e = (uint32_t)nb[k * 32];
      visit((int)(e & kEntrySlot), (e & kEntryImage) != 0u);
    }
  } else {
    const long long local = b.key[sel][t] - sp.c0;
    if (idx_ok(b.ctl, local, (long long)sp.g[0] * sp.g[1] * (DIM == 3 ? sp.g[2] : 1)))
      for_each_candidate<DIM>(b.cell_start, sp, local, [&](int j) {
        if (j != (int)t) visit(j, true);
      });
  }
  b.frc[sel][t] = make_float4(F[0] + eF[0], F[1] + eF[1], DIM == 3 ? F[2] + eF[2] : 0.0f, 0.0f);
  // compute_force's epilogue adds cross(pos_p, F) = 0 for spheres (cell_list.py:452-464)
  for (int a = 0; a < AD; ++a) b.rtq[(long long)oi * AD + a] = T[a] + eT[a];
}

// ForceManager + step_after_force of both integrators; in MODE_STEP also the
// next step's apply / step_before_force / drift (integrate_particle), with the
// rotational before-force phase under the same torque.
template <int DIM>
__global__ void k_cs_step(Bufs b, int mode) {
  constexpr int AD = DIM == 3 ? 3 : 1;
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  float d2max = 0.0f;
  if (t < b.P) {
    const unsigned int sel = ld_nc_u32(&b.ctl->sel), ps = ld_nc_u32(&b.ctl->pos_sel);
    const float4 pi = b.pos[ps][t];
    const uint32_t tg = b.tag[sel][t];
    const SysParams& sp = b.sys[tg & TAG_SYS_MASK];
    const float4 v4 = b.vel[sel][t];
    const float4 f4 = b.frc[sel][t];
    float F[3] = {f4.x, f4.y, f4.z};
    d2max = integrate_particle<DIM>(b, mode, t, sel, ps, sp, pi, tg, v4, F);
    // rotation: ForceManager adds cross(r, F_part) = 0 to the torque
    const long long i = b.orig[sel][t];
    float4 qq = b.rq[i];
    float w[3] = {0, 0, 0}, tq[3] = {0, 0, 0}, I[3] = {1, 1, 1}, invI[3] = {1, 1, 1};
    for (int a = 0; a < AD; ++a) {
      w[a] = b.rw[i * AD + a];
      tq[a] = b.rtq[i * AD + a];
      I[a] = b.rinertia[i * AD + a];
      invI[a] = 1.0f / I[a];
    }
    const float fr = (tg & TAG_FIXED) ? 0.0f : 1.0f;
    rot_after<DIM>(sp.rot, sp.dt, qq, w, tq, I, invI, fr);
    if ((mode & 7) == MODE_STEP) {
      if (sp.domain == DOM_REFLECT) qq = reflect_q(qq);
      rot_before<DIM>(sp.rot, sp.dt, qq, w, tq, I, invI, fr);
    }
    b.rq[i] = qq;
    for (int a = 0; a < AD; ++a) b.rw[i * AD + a] = w[a];
  }
  warp_disp(b.ctl, d2max);
}

// First step of a call, rotational half: domain.apply's orientation update
// and step_before_force (caller order).
template <int DIM>
__global__ void k_cs_rot_pre(Bufs b) {
  constexpr int AD = DIM == 3 ? 3 : 1;
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= b.P) return;
  const SysParams& sp = b.sys[b.sys_of[i]];
  float4 qq = b.rq[i];
  float w[3] = {0, 0, 0}, tq[3] = {0, 0, 0}, I[3] = {1, 1, 1}, invI[3] = {1, 1, 1};
  for (int a = 0; a < AD; ++a) {
    w[a] = b.rw[i * AD + a];
    tq[a] = b.rtq[i * AD + a];
    I[a] = b.rinertia[i * AD + a];
    invI[a] = 1.0f / I[a];
  }
  const float fr = b.fixed_c[i] ? 0.0f : 1.0f;
  if (sp.domain == DOM_REFLECT) qq = reflect_q(qq);
  rot_before<DIM>(sp.rot, sp.dt, qq, w, tq, I, invI, fr);
  b.rq[i] = qq;
  for (int a = 0; a < AD; ++a) b.rw[i * AD + a] = w[a];
}

void launch_cs(int dim, const Bufs& b, int mode, cudaStream_t st) {
  if (b.P == 0) return;
  const unsigned int g = nblk_cs(b.P, 128);
  if (dim == 3) k_cs_force<3><<<g, 128, 0, st>>>(b);
  else k_cs_force<2><<<g, 128, 0, st>>>(b);
  if ((mode & 7) == MODE_FORCE_ONLY) return;
  if (dim == 3) k_cs_step<3><<<g, 128, 0, st>>>(b, mode);
  else k_cs_step<2><<<g, 128, 0, st>>>(b, mode);
}

void launch_cs_rot_pre(int dim, const Bufs& b, cudaStream_t st) {
  if (b.P == 0) return;
  if (dim == 3) k_cs_rot_pre<3><<<nblk_cs(b.P, 256), 256, 0, st>>>(b);
  else k_cs_rot_pre<2><<<nblk_cs(b.P, 256), 256, 0, st>>>(b);
}

}  // namespace jdem
