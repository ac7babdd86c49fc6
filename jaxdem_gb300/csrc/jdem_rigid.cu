// Rigid clumps: bodies made of several spheres (State.add_clump,
// jaxdem/state.py:1230-1420) whose members share the body's centre pos_c,
// velocity, orientation, angular velocity, mass and inertia and differ in
// their body-frame offsets pos_p and radii.
//
// The engine holds each clump's state once (cpos, cvel, cq, cw, ...) and the
// slots hold the members' world positions pos_c + R(q) pos_p, so binning,
// the Verlet list and the contact kernels work on spheres as before.  A step:
//   k_rb_force   per sphere: contact force from the list (spheres of one clump
//                excluded, colliders/__init__.py:225-243) and its torque about
//                the clump centre, cross(R(q) pos_p, F) (cell_list.py:452-464);
//                k_rb_cs_force for Cundall-Strack contacts, whose pair torques
//                are added to that;
//   k_rb_clump   per clump: ForceManager.apply -- F_contact + gravity * (M /
//                count) summed over the members, torques summed
//                (force_manager.py:338-425) -- then the integrators'
//                after-force phase and, in MODE_STEP, the next step's apply (free-domain
//                box or reflect impulses), before-force phase and drift;
//   k_rb_place   per slot: the member's new world position.
// Members are summed in caller order.  Periodic, free and reflect domains
// (the reflect domain's clump impulses: clump_reflect).
#include "jdem_device.cuh"
#include "jdem_cs.cuh"
#include "jdem_kernels.h"
#include "jdem_pair.cuh"
#include "jdem_rot.cuh"

namespace jdem {

namespace {

unsigned int nblk_rb(long long n, int t) { return (unsigned int)((n + t - 1) / t); }

// R(q) pos_p of caller index i (state._pos_p_rot, state.py:230-273)
template <int DIM>
__device__ __forceinline__ void lever(const Bufs& b, float4 q, long long i, float* r) {
  float pp[3] = {b.spp[i * DIM], b.spp[i * DIM + 1], DIM == 3 ? b.spp[i * DIM + 2] : 0.0f};
  if (DIM == 3) q_rotate3(q, 1.0f, pp, r);
  else q_rotate2(q, pp, r);
}

}  // namespace

// Contact force of every sphere and its torque about the clump centre.
template <int DIM, int LAW>
__global__ void k_rb_force(Bufs b) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= b.P) return;
  const unsigned int sel = ld_nc_u32(&b.ctl->sel), ps = ld_nc_u32(&b.ctl->pos_sel);
  const bool use_list = b.nl_cap > 0 && (ld_nc_u32(&b.ctl->status) & ST_NL_OVERFLOW) == 0u;
  const float4* __restrict__ P = b.pos[ps];
  const float4 pi = P[t];
  const uint32_t tg = b.tag[sel][t];
  const SysParams& sp = b.sys[tg & TAG_SYS_MASK];
  ContactSum<DIM, true, LAW> acc(b, sp, pi, tg, sel, t);
  if (use_list) {
    int n = b.ncnt[t];
    if (!idx_ok(b.ctl, n, (long long)b.nl_cap + 1)) n = 0;
    const int32_t* nb = b.nbr + ((t >> 5) * b.nl_cap) * 32 + (t & 31);
    prefetch_list_block(b, t, n);
    for (int k = 0; k < n; ++k) {
      const uint32_t e = (uint32_t)nb[k * 32];
      if (idx_ok(b.ctl, e & kEntrySlot, b.P)) acc.add(b, sel, (int)(e & kEntrySlot), P[e & kEntrySlot], true);
    }
  } else {
    const long long local = b.key[sel][t] - sp.c0;
    if (idx_ok(b.ctl, local, (long long)sp.g[0] * sp.g[1] * (DIM == 3 ? sp.g[2] : 1)))
      for_each_candidate<DIM>(b.cell_start, sp, local, [&](int j) {
        if (j != (int)t) acc.add(b, sel, j, P[j]);
      });
  }
  const float F[3] = {acc.fx + acc.ex, acc.fy + acc.ey, DIM == 3 ? acc.fz + acc.ez : 0.0f};
  const long long i = b.orig[sel][t];
  if (!idx_ok(b.ctl, i, b.P) || !idx_ok(b.ctl, b.sclump[i], b.NC)) return;
  float r[3] = {0.0f, 0.0f, 0.0f};
  lever<DIM>(b, b.cq[b.sclump[i]], i, r);
  // torque = sum of pair torques (0 for these laws) + cross(R(q) pos_p, F)
  float4 T = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  if (DIM == 3) {
    T.x = 0.0f + (r[1] * F[2] - r[2] * F[1]);
    T.y = 0.0f + (r[2] * F[0] - r[0] * F[2]);
    T.z = 0.0f + (r[0] * F[1] - r[1] * F[0]);
  } else {
    T.x = 0.0f + (r[0] * F[1] - r[1] * F[0]);
  }
  b.sf[i] = make_float4(F[0], F[1], F[2], 0.0f);
  b.stq[i] = T;
}

// Cundall-Strack contacts of every sphere (cundall_strack.py:100-196).  A
// member's velocity, angular velocity and mass are its clump's (every member
// stores the clump's values), and the contact arm runs from the sphere's own
// centre; the sphere's torque about the clump centre is the sum of the pair
// torques plus cross(R(q) pos_p, F) (cell_list.py:452-464).
template <int DIM>
__global__ void k_rb_cs_force(Bufs b) {
  constexpr int AD = DIM == 3 ? 3 : 1;
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= b.P) return;
  const unsigned int sel = ld_nc_u32(&b.ctl->sel), ps = ld_nc_u32(&b.ctl->pos_sel);
  const bool use_list = b.nl_cap > 0 && (ld_nc_u32(&b.ctl->status) & ST_NL_OVERFLOW) == 0u;
  const float4* __restrict__ P = b.pos[ps];
  const float4 pi = P[t];
  const uint32_t tg = b.tag[sel][t];
  const SysParams& sp = b.sys[tg & TAG_SYS_MASK];
  const bool per = sp.domain == DOM_PERIODIC;
  const int mi = (tg >> TAG_MAT_SHIFT) & TAG_MAT_MASK;
  const long long oi = b.orig[sel][t];
  if (!idx_ok(b.ctl, oi, b.P) || !idx_ok(b.ctl, b.sclump[oi], b.NC)) return;
  const int ci = b.sclump[oi];
  const float4 vi4 = b.cvel[ci], wi4 = b.cw[ci];
  const float Mi = b.cpos[ci].w;
  const float vi[3] = {vi4.x, vi4.y, vi4.z}, wi[3] = {wi4.x, wi4.y, wi4.z};
  float F[3] = {0, 0, 0}, eF[3] = {0, 0, 0}, T[3] = {0, 0, 0}, eT[3] = {0, 0, 0};
  auto visit = [&](int j, bool may_wrap) {
    if (!idx_ok(b.ctl, j, b.P)) return;
    const float4 pj = P[j];
    float d[3];
    const float dsq = pair_disp<DIM>(sp, per && may_wrap, pi, pj, d[0], d[1], d[2]);
    const float R = pi.w + pj.w;
    if (!(dsq < R * R * 1.000001f)) return;
    const int oj = b.orig[sel][j];
    if (!idx_ok(b.ctl, oj, b.P) || !idx_ok(b.ctl, b.sclump[oj], b.NC)) return;
    const int cj = b.sclump[oj];
    if (cj == ci) return;  // one body (valid_interaction_mask)
    if (b.bond_w > 0 && !b.interact_same_bond) {
      bool bonded = false;
      for (int w = 0; w < b.bond_w; ++w) bonded |= (b.bond[oi * b.bond_w + w] == oj);
      if (bonded) return;
    }
    const int mj = (b.tag[sel][j] >> TAG_MAT_SHIFT) & TAG_MAT_MASK;
    const float4 vj4 = b.cvel[cj], wj4 = b.cw[cj];
    const float vj[3] = {vj4.x, vj4.y, vj4.z}, wj[3] = {wj4.x, wj4.y, wj4.z};
    cs_pair<DIM>(b, mi, mj, pi.w, pj.w, Mi, b.cpos[cj].w, vi, vj, wi, wj, d, F, eF, T, eT);
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
  const float f[3] = {F[0] + eF[0], F[1] + eF[1], DIM == 3 ? F[2] + eF[2] : 0.0f};
  float r[3] = {0.0f, 0.0f, 0.0f};
  lever<DIM>(b, b.cq[ci], oi, r);
  float tq[3] = {0.0f, 0.0f, 0.0f};
  for (int a = 0; a < AD; ++a) tq[a] = T[a] + eT[a];
  if (DIM == 3) {
    tq[0] = tq[0] + (r[1] * f[2] - r[2] * f[1]);
    tq[1] = tq[1] + (r[2] * f[0] - r[0] * f[2]);
    tq[2] = tq[2] + (r[0] * f[1] - r[1] * f[0]);
  } else {
    tq[0] = tq[0] + (r[0] * f[1] - r[1] * f[0]);
  }
  b.sf[oi] = make_float4(f[0], f[1], f[2], 0.0f);
  b.stq[oi] = make_float4(tq[0], tq[1], tq[2], 0.0f);
}

// Linear and rotational state of clump c as registers.
struct ClumpState {
  float p[3], v[3], F[3], T[3], w[3], I[3], invI[3];
  float M, fr;
  float4 q;
};

template <int DIM>
__device__ __forceinline__ void load_clump(const Bufs& b, long long c, ClumpState& s) {
  constexpr int AD = DIM == 3 ? 3 : 1;
  const float4 p4 = b.cpos[c], v4 = b.cvel[c], f4 = b.cfrc[c], t4 = b.ctq[c], w4 = b.cw[c], I4 = b.cI[c];
  s.p[0] = p4.x; s.p[1] = p4.y; s.p[2] = p4.z;
  s.v[0] = v4.x; s.v[1] = v4.y; s.v[2] = v4.z;
  s.F[0] = f4.x; s.F[1] = f4.y; s.F[2] = f4.z;
  s.T[0] = t4.x; s.T[1] = t4.y; s.T[2] = t4.z;
  s.w[0] = w4.x; s.w[1] = w4.y; s.w[2] = w4.z;
  s.I[0] = I4.x; s.I[1] = I4.y; s.I[2] = I4.z;
  for (int a = 0; a < 3; ++a) s.invI[a] = a < AD ? 1.0f / s.I[a] : 1.0f;
  s.M = p4.w;
  s.fr = b.cfixed[c] ? 0.0f : 1.0f;
  s.q = b.cq[c];
}

// ReflectDomain.apply for one rigid clump (domains/reflect.py:165-297): every
// member's overshoot past the walls, the clump's deepest overshoot per axis;
// the members holding it are active, each with the Verlet time-of-collision
// fraction of its contact point (_toc.py:11-94), and the clump takes the
// smallest; impulses -(1 + e) v_n / (1/m + (r x n) . I^-1 (r x n)), shared
// among the active members of an axis, change the velocity and the angular
// velocity (sums over the members in caller order), and the remaining part of
// the step moves pos_c and q with the change.
template <int DIM>
__device__ void clump_reflect(const Bufs& b, const SysParams& sp, long long c, ClumpState& s) {
  constexpr int AD = DIM == 3 ? 3 : 1;
  const int m0 = b.cstart[c], m1 = b.cstart[c + 1];
  const float dt = sp.dt, e = sp.restitution;
  const float inv_mass = 1.0f / s.M;
  // segment_max of the members' overshoots (all >= 0)
  float max_lo[3] = {0, 0, 0}, max_hi[3] = {0, 0, 0};
  for (int m = m0; m < m1; ++m) {
    const long long i = b.cmember[m];
    float r[3] = {0, 0, 0};
    lever<DIM>(b, s.q, i, r);
    const float rad = b.rad_c[i];
    for (int a = 0; a < DIM; ++a) {
      const float pos = s.p[a] + r[a];
      const float lo = sp.anchor[a] + rad, hi = sp.anchor[a] + sp.box[a] - rad;
      max_lo[a] = fmaxf(max_lo[a], fmaxf(0.0f, lo - pos));
      max_hi[a] = fmaxf(max_hi[a], fmaxf(0.0f, pos - hi));
    }
  }
  // angular acceleration of the clump: R (tau_b - w_b x (I w_b)) / I
  float alpha_rot[3] = {0, 0, 0};
  if (DIM == 3) {
    float tb[3], wb[3], ab[3];
    q_rotate3(s.q, -1.0f, s.T, tb);
    q_rotate3(s.q, -1.0f, s.w, wb);
    omega_dot3<3>(wb, tb, s.I, s.invI, ab);
    q_rotate3(s.q, 1.0f, ab, alpha_rot);
  } else {
    alpha_rot[0] = s.T[0] * s.invI[0];
  }
  // body-frame wall normals n'_a = R^T e_a
  float np_[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  const float4 qc = make_float4(s.q.x, -s.q.y, -s.q.z, -s.q.w);
  for (int a = 0; a < DIM; ++a) {
    float ea[3] = {0, 0, 0};
    ea[a] = 1.0f;
    if (DIM == 3) q_rotate3(s.q, -1.0f, ea, np_[a]);
    else q_rotate2(qc, ea, np_[a]);
  }
  const float acc_c[3] = {s.F[0] * inv_mass, s.F[1] * inv_mass, DIM == 3 ? s.F[2] * inv_mass : 0.0f};
  // pass 2: the clump's collision fraction and the active members per axis
  float alpha_clump = 1.0f, count_active[3] = {0, 0, 0};
  for (int m = m0; m < m1; ++m) {
    const long long i = b.cmember[m];
    float r[3] = {0, 0, 0};
    lever<DIM>(b, s.q, i, r);
    const float rad = b.rad_c[i];
    float vcs[3], accc[3];
    if (DIM == 3) {
      vcs[0] = s.v[0] + (s.w[1] * r[2] - s.w[2] * r[1]);
      vcs[1] = s.v[1] + (s.w[2] * r[0] - s.w[0] * r[2]);
      vcs[2] = s.v[2] + (s.w[0] * r[1] - s.w[1] * r[0]);
      accc[0] = acc_c[0] + (alpha_rot[1] * r[2] - alpha_rot[2] * r[1]);
      accc[1] = acc_c[1] + (alpha_rot[2] * r[0] - alpha_rot[0] * r[2]);
      accc[2] = acc_c[2] + (alpha_rot[0] * r[1] - alpha_rot[1] * r[0]);
    } else {
      vcs[0] = s.v[0] + -s.w[0] * r[1];
      vcs[1] = s.v[1] + s.w[0] * r[0];
      accc[0] = acc_c[0] + -alpha_rot[0] * r[1];
      accc[1] = acc_c[1] + alpha_rot[0] * r[0];
    }
    float amin = 1.0f;
    for (int a = 0; a < DIM; ++a) {
      const float pos = s.p[a] + r[a];
      const float lo = sp.anchor[a] + rad, hi = sp.anchor[a] + sp.box[a] - rad;
      const float olo = fmaxf(0.0f, lo - pos), ohi = fmaxf(0.0f, pos - hi);
      const float ws = ((olo > 0.0f && olo == max_lo[a]) ? 1.0f : 0.0f) - ((ohi > 0.0f && ohi == max_hi[a]) ? 1.0f : 0.0f);
      const float act = fabsf(ws);
      const float delta = fmaxf(max_lo[a], max_hi[a]);
      const float al = toc_alpha(vcs[a], accc[a], delta, ws, dt);
      amin = fminf(amin, act > 0.0f ? al : 1.0f);
      count_active[a] = count_active[a] + act;
    }
    alpha_clump = fminf(alpha_clump, amin);
  }
  // pass 3: impulses
  const float dt_factor = (alpha_clump - 1.0f) * dt;
  float dv[3] = {0, 0, 0}, dw[3] = {0, 0, 0};
  for (int m = m0; m < m1; ++m) {
    const long long i = b.cmember[m];
    float r[3] = {0, 0, 0};
    lever<DIM>(b, s.q, i, r);
    const float pp[3] = {b.spp[i * DIM], b.spp[i * DIM + 1], DIM == 3 ? b.spp[i * DIM + 2] : 0.0f};
    const float rad = b.rad_c[i];
    float vcs[3], accc[3];
    if (DIM == 3) {
      vcs[0] = s.v[0] + (s.w[1] * r[2] - s.w[2] * r[1]);
      vcs[1] = s.v[1] + (s.w[2] * r[0] - s.w[0] * r[2]);
      vcs[2] = s.v[2] + (s.w[0] * r[1] - s.w[1] * r[0]);
      accc[0] = acc_c[0] + (alpha_rot[1] * r[2] - alpha_rot[2] * r[1]);
      accc[1] = acc_c[1] + (alpha_rot[2] * r[0] - alpha_rot[0] * r[2]);
      accc[2] = acc_c[2] + (alpha_rot[0] * r[1] - alpha_rot[1] * r[0]);
    } else {
      vcs[0] = s.v[0] + -s.w[0] * r[1];
      vcs[1] = s.v[1] + s.w[0] * r[0];
      accc[0] = acc_c[0] + -alpha_rot[0] * r[1];
      accc[1] = acc_c[1] + alpha_rot[0] * r[0];
    }
    float J[3] = {0, 0, 0};
    for (int a = 0; a < DIM; ++a) {
      const float pos = s.p[a] + r[a];
      const float lo = sp.anchor[a] + rad, hi = sp.anchor[a] + sp.box[a] - rad;
      const float olo = fmaxf(0.0f, lo - pos), ohi = fmaxf(0.0f, pos - hi);
      const float ws = ((olo > 0.0f && olo == max_lo[a]) ? 1.0f : 0.0f) - ((ohi > 0.0f && ohi == max_hi[a]) ? 1.0f : 0.0f);
      const float act = fabsf(ws);
      // denominator 1/m + sum_k invI_k (pos_p x n'_a)_k^2
      float denom_rot;
      if (DIM == 3) {
        const float* n = np_[a];
        const float cx = pp[1] * n[2] - pp[2] * n[1], cy = pp[2] * n[0] - pp[0] * n[2], cz = pp[0] * n[1] - pp[1] * n[0];
        denom_rot = s.invI[0] * (cx * cx) + s.invI[1] * (cy * cy) + s.invI[2] * (cz * cz);
      } else {
        const float cz = pp[0] * np_[a][1] - pp[1] * np_[a][0];
        denom_rot = s.invI[0] * (cz * cz);
      }
      float denom = inv_mass + denom_rot;
      denom = denom == 0.0f ? 1.0f : denom;
      const float vc = vcs[a] + dt_factor * accc[a];
      float j = -(1.0f + e) * vc / denom;
      const float closing = (vc * ws) < 0.0f ? 1.0f : 0.0f;
      const float weight = act / fmaxf(count_active[a], 1.0f);
      j = j * (weight * closing);
      J[a] = j;
      dv[a] = dv[a] + j * inv_mass;
    }
    // angular: moment of the impulse about the centre in the body frame
    if (DIM == 3) {
      float jb[3], mb[3], dl[3];
      q_rotate3(s.q, -1.0f, J, jb);
      mb[0] = (pp[1] * jb[2] - pp[2] * jb[1]) * s.invI[0];
      mb[1] = (pp[2] * jb[0] - pp[0] * jb[2]) * s.invI[1];
      mb[2] = (pp[0] * jb[1] - pp[1] * jb[0]) * s.invI[2];
      q_rotate3(s.q, 1.0f, mb, dl);
      for (int a = 0; a < 3; ++a) dw[a] = dw[a] + dl[a];
    } else {
      float jb[2];
      q_rotate2(qc, J, jb);
      dw[0] = dw[0] + (pp[0] * jb[1] - pp[1] * jb[0]) * s.invI[0];
    }
  }
  const bool fixed = s.fr == 0.0f;
  const float dt_rem = (1.0f - alpha_clump) * dt;
  for (int a = 0; a < DIM; ++a) {
    const float d = fixed ? 0.0f : dv[a];
    s.v[a] = s.v[a] + d;
    dv[a] = d;
  }
  for (int a = 0; a < AD; ++a) {
    dw[a] = fixed ? 0.0f : dw[a];
    s.w[a] = s.w[a] + dw[a];
  }
  float th[3];
  if (DIM == 3) {
    for (int a = 0; a < 3; ++a) th[a] = dw[a] * dt_rem;
  } else {
    th[0] = 0.0f;
    th[1] = 0.0f;
    th[2] = dw[0] * dt_rem;
  }
  s.q = q_unit(q_mul(q_small_rotvec(th[0], th[1], th[2]), s.q));
  for (int a = 0; a < DIM; ++a) s.p[a] = s.p[a] + dv[a] * dt_rem;
}

// The next step's apply (free domain: the box of pos_c -+ (|pos_p| + rad),
// free.py:59-63; reflect: clump_reflect), then step_before_force of both
// integrators and the drift.
template <int DIM>
__device__ __forceinline__ void clump_before(const Bufs& b, const SysParams& sp, long long c, int mode, ClumpState& s) {
  if (sp.domain == DOM_REFLECT) clump_reflect<DIM>(b, sp, c, s);
  if ((mode & MODE_BBOX) && sp.domain == DOM_FREE) {
    const int sys = b.csys[c];
    const float br = b.cbrad[c];
#pragma unroll
    for (int a = 0; a < DIM; ++a) {
      atomicMin((unsigned int*)&b.bbox[sys * 6 + a], f2ord(s.p[a] - br));
      atomicMax((unsigned int*)&b.bbox[sys * 6 + 3 + a], f2ord(s.p[a] + br));
    }
  }
  if (sp.lin == LIN_VERLET) {
    const float sc = sp.dt * 0.5f / s.M;
#pragma unroll
    for (int a = 0; a < DIM; ++a) {
      s.v[a] = s.v[a] + s.F[a] * sc * s.fr;
      s.p[a] = s.p[a] + sp.dt * s.v[a];
    }
  }
  rot_before<DIM>(sp.rot, sp.dt, s.q, s.w, s.T, s.I, s.invI, s.fr);
}

template <int DIM>
__device__ __forceinline__ void store_clump(const Bufs& b, long long c, const ClumpState& s, bool forces) {
  b.cpos[c] = make_float4(s.p[0], s.p[1], DIM == 3 ? s.p[2] : 0.0f, s.M);
  b.cvel[c] = make_float4(s.v[0], s.v[1], DIM == 3 ? s.v[2] : 0.0f, 0.0f);
  b.cq[c] = s.q;
  b.cw[c] = make_float4(s.w[0], DIM == 3 ? s.w[1] : 0.0f, DIM == 3 ? s.w[2] : 0.0f, 0.0f);
  if (forces) {
    b.cfrc[c] = make_float4(s.F[0], s.F[1], DIM == 3 ? s.F[2] : 0.0f, 0.0f);
    b.ctq[c] = make_float4(s.T[0], DIM == 3 ? s.T[1] : 0.0f, DIM == 3 ? s.T[2] : 0.0f, 0.0f);
  }
}

// ForceManager, step_after_force, and in MODE_STEP the next step's first half.
template <int DIM>
__global__ void k_rb_clump(Bufs b, int mode) {
  constexpr int AD = DIM == 3 ? 3 : 1;
  const long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (c >= b.NC) return;
  const SysParams& sp = b.sys[b.csys[c]];
  ClumpState s;
  load_clump<DIM>(b, c, s);
  const int m0 = b.cstart[c], m1 = b.cstart[c + 1];
  const float count = (float)(m1 - m0);
  float F[3] = {0.0f, 0.0f, 0.0f}, T[3] = {0.0f, 0.0f, 0.0f};
  for (int m = m0; m < m1; ++m) {
    const long long i = b.cmember[m];
    const float4 f = b.sf[i], t = b.stq[i];
    const float fi[3] = {f.x, f.y, f.z}, ti[3] = {t.x, t.y, t.z};
    // F_contact + F_part (0) + gravity * (mass / count); T_contact + T_part (0)
#pragma unroll
    for (int a = 0; a < DIM; ++a) F[a] = F[a] + ((fi[a] + 0.0f) + sp.gravity[a] * (s.M / count));
#pragma unroll
    for (int a = 0; a < AD; ++a) T[a] = T[a] + (ti[a] + 0.0f);
  }
  for (int a = 0; a < 3; ++a) {
    s.F[a] = a < DIM ? F[a] : 0.0f;
    s.T[a] = a < AD ? T[a] : 0.0f;
  }
  if (sp.lin == LIN_VERLET) {
    const float sc = sp.dt * 0.5f / s.M;
#pragma unroll
    for (int a = 0; a < DIM; ++a) s.v[a] = s.v[a] + s.F[a] * sc * s.fr;
  } else if (sp.lin == LIN_EULER) {
    const float sc = sp.dt / s.M;
#pragma unroll
    for (int a = 0; a < DIM; ++a) {
      s.v[a] = s.v[a] + s.F[a] * sc * s.fr;
      s.p[a] = s.p[a] + sp.dt * s.v[a];
    }
  }
  rot_after<DIM>(sp.rot, sp.dt, s.q, s.w, s.T, s.I, s.invI, s.fr);
  if ((mode & 7) == MODE_STEP) clump_before<DIM>(b, sp, c, mode, s);
  store_clump<DIM>(b, c, s, true);
}

// First step of a call: apply, step_before_force and drift of every clump.
template <int DIM>
__global__ void k_rb_pre(Bufs b, int mode) {
  const long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (c >= b.NC) return;
  const SysParams& sp = b.sys[b.csys[c]];
  ClumpState s;
  load_clump<DIM>(b, c, s);
  clump_before<DIM>(b, sp, c, mode, s);
  store_clump<DIM>(b, c, s, false);
}

// World position of every member slot from its clump's state; writes the
// current buffer (in_place) or the next one, and folds the displacement into
// the re-sort bound.
template <int DIM>
__global__ void k_rb_place(Bufs b, int in_place) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  float d2 = 0.0f;
  if (t < b.P) {
    const unsigned int sel = ld_nc_u32(&b.ctl->sel), ps = ld_nc_u32(&b.ctl->pos_sel);
    const float4 old = b.pos[ps][t];
    const long long i = b.orig[sel][t];
    const int c = b.sclump[i];
    const float4 pc = b.cpos[c];
    float r[3] = {0.0f, 0.0f, 0.0f};
    lever<DIM>(b, b.cq[c], i, r);
    const float w[3] = {pc.x + r[0], pc.y + r[1], DIM == 3 ? pc.z + r[2] : 0.0f};
    const float o[3] = {old.x, old.y, old.z};
#pragma unroll
    for (int a = 0; a < DIM; ++a) {
      const float d = w[a] - o[a];
      d2 = d2 + d * d;
    }
    b.pos[in_place ? ps : ps ^ 1u][t] = make_float4(w[0], w[1], w[2], old.w);
    if (!(d2 == d2) || d2 > 3.0e38f) {
      atomicOr(&b.ctl->status, ST_NONFINITE);
      d2 = 0.0f;
    }
  }
  warp_disp(b.ctl, d2);
}

// Upload: each clump's state from its first member (every member stores the
// clump's values) and its bounding radius max(norm(pos_p) + rad) (free.py:59).
template <int DIM>
__global__ void k_rb_init(Bufs b, const float* __restrict__ pos, const float* __restrict__ vel,
                          const float* __restrict__ frc, const float* __restrict__ rad, const float* __restrict__ mass,
                          const float4* __restrict__ q, const float* __restrict__ angv, const float* __restrict__ torque,
                          const float* __restrict__ inertia, const uint8_t* __restrict__ fixed,
                          const int32_t* __restrict__ sys_of) {
  constexpr int AD = DIM == 3 ? 3 : 1;
  const long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (c >= b.NC) return;
  const int m0 = b.cstart[c], m1 = b.cstart[c + 1];
  const long long i0 = b.cmember[m0];
  float p[3] = {0, 0, 0}, v[3] = {0, 0, 0}, f[3] = {0, 0, 0}, w[3] = {0, 0, 0}, t[3] = {0, 0, 0}, I[3] = {1, 1, 1};
  for (int a = 0; a < DIM; ++a) {
    p[a] = pos[i0 * DIM + a];
    v[a] = vel[i0 * DIM + a];
    f[a] = frc[i0 * DIM + a];
  }
  for (int a = 0; a < AD; ++a) {
    w[a] = angv[i0 * AD + a];
    t[a] = torque[i0 * AD + a];
    I[a] = inertia[i0 * AD + a];
  }
  b.cpos[c] = make_float4(p[0], p[1], p[2], mass[i0]);
  b.cvel[c] = make_float4(v[0], v[1], v[2], 0.0f);
  b.cfrc[c] = make_float4(f[0], f[1], f[2], 0.0f);
  b.cq[c] = q[i0];
  b.cw[c] = make_float4(w[0], w[1], w[2], 0.0f);
  b.ctq[c] = make_float4(t[0], t[1], t[2], 0.0f);
  b.cI[c] = make_float4(I[0], I[1], I[2], 0.0f);
  b.cfixed[c] = fixed[i0];
  b.csys[c] = sys_of[i0];
  float br = 0.0f;
  for (int m = m0; m < m1; ++m) {
    const long long i = b.cmember[m];
    float n2 = 0.0f;
    for (int a = 0; a < DIM; ++a) n2 = a == 0 ? b.spp[i * DIM] * b.spp[i * DIM] : n2 + b.spp[i * DIM + a] * b.spp[i * DIM + a];
    const float nrm = n2 == 0.0f ? 0.0f : sqrtf(fmaxf(n2, 1e-16f));
    br = fmaxf(br, nrm + rad[i]);
  }
  b.cbrad[c] = br;
}

// Caller-order world positions of the members (upload, neighbour-list API).
template <int DIM>
__global__ void k_rb_world(Bufs b, float* __restrict__ pos) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= b.P) return;
  const int c = b.sclump[i];
  const float4 pc = b.cpos[c];
  float r[3] = {0.0f, 0.0f, 0.0f};
  lever<DIM>(b, b.cq[c], i, r);
  const float w[3] = {pc.x + r[0], pc.y + r[1], pc.z + r[2]};
  for (int a = 0; a < DIM; ++a) pos[i * DIM + a] = w[a];
}

// Download: every member stores its clump's state (caller order).  per_sphere:
// force and torque are each sphere's own contact terms (compute_force).
// Null destinations are skipped.
template <int DIM>
__global__ void k_rb_unpack(Bufs b, float* __restrict__ pos, float* __restrict__ vel, float* __restrict__ frc,
                            float4* __restrict__ q, float* __restrict__ angv, float* __restrict__ torque,
                            int per_sphere) {
  constexpr int AD = DIM == 3 ? 3 : 1;
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= b.P) return;
  const int c = b.sclump[i];
  const float4 p = b.cpos[c], v = b.cvel[c], w = b.cw[c];
  const float4 f = per_sphere ? b.sf[i] : b.cfrc[c];
  const float4 t = per_sphere ? b.stq[i] : b.ctq[c];
  const float pa[3] = {p.x, p.y, p.z}, va[3] = {v.x, v.y, v.z}, fa[3] = {f.x, f.y, f.z};
  const float wa[3] = {w.x, w.y, w.z}, ta[3] = {t.x, t.y, t.z};
  // a null destination skips that field (trajectory frames select fields)
  for (int a = 0; a < DIM; ++a) {
    if (pos) pos[i * DIM + a] = pa[a];
    if (vel) vel[i * DIM + a] = va[a];
    if (frc) frc[i * DIM + a] = fa[a];
  }
  if (q) q[i] = b.cq[c];
  for (int a = 0; a < AD; ++a) {
    if (angv) angv[i * AD + a] = wa[a];
    if (torque) torque[i * AD + a] = ta[a];
  }
}

// Energies of clumps (thermal.py:24-80, force_manager.py:427-459): members
// carry the clump's mass and inertia, and each member's share is 1 / count,
// so the clump's terms are entered once, at its first member.
template <int DIM>
__global__ void k_rb_energy(Bufs b, double* __restrict__ out) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= b.P) return;
  const int c = b.sclump[i];
  double eg = 0.0, ek = 0.0, er = 0.0;
  if (b.cmember[b.cstart[c]] == i) {
    const SysParams& sp = b.sys[b.csys[c]];
    const float4 p = b.cpos[c], v = b.cvel[c], w4 = b.cw[c], I4 = b.cI[c];
    const float pa[3] = {p.x, p.y, p.z}, va[3] = {v.x, v.y, v.z};
    for (int a = 0; a < DIM; ++a) {
      eg -= (double)sp.gravity[a] * (double)pa[a] * (double)p.w;
      ek += 0.5 * (double)p.w * (double)va[a] * (double)va[a];
    }
    float wb[3] = {w4.x, 0.0f, 0.0f};
    const float I[3] = {I4.x, I4.y, I4.z};
    if (DIM == 3) {
      const float wl[3] = {w4.x, w4.y, w4.z};
      q_rotate3(b.cq[c], -1.0f, wl, wb);
      for (int a = 0; a < 3; ++a) er += 0.5 * (double)wb[a] * (double)(I[a] * wb[a]);
    } else {
      er = 0.5 * (double)wb[0] * (double)(I[0] * wb[0]);
    }
  }
  out[i * 3 + 1] = eg;
  out[i * 3 + 2] = ek;
  out[3 * b.P + i] = er;
}

void launch_rb(int dim, const Bufs& b, int mode, cudaStream_t st) {
  if (b.P == 0) return;
  const unsigned int g = nblk_rb(b.P, 128), gc = nblk_rb(b.NC, 128);
  if (dim == 3) {
    if (b.law == LAW_CS) k_rb_cs_force<3><<<g, 128, 0, st>>>(b);
    else if (b.law == LAW_HERTZ) k_rb_force<3, LAW_HERTZ><<<g, 128, 0, st>>>(b);
    else k_rb_force<3, LAW_SPRING><<<g, 128, 0, st>>>(b);
  } else {
    if (b.law == LAW_CS) k_rb_cs_force<2><<<g, 128, 0, st>>>(b);
    else if (b.law == LAW_HERTZ) k_rb_force<2, LAW_HERTZ><<<g, 128, 0, st>>>(b);
    else k_rb_force<2, LAW_SPRING><<<g, 128, 0, st>>>(b);
  }
  if ((mode & 7) == MODE_FORCE_ONLY) return;
  if (dim == 3) {
    k_rb_clump<3><<<gc, 128, 0, st>>>(b, mode);
    k_rb_place<3><<<g, 128, 0, st>>>(b, 0);
  } else {
    k_rb_clump<2><<<gc, 128, 0, st>>>(b, mode);
    k_rb_place<2><<<g, 128, 0, st>>>(b, 0);
  }
}

void launch_rb_pre(int dim, const Bufs& b, int mode, cudaStream_t st) {
  if (b.P == 0) return;
  const unsigned int g = nblk_rb(b.P, 128), gc = nblk_rb(b.NC, 128);
  if (dim == 3) {
    k_rb_pre<3><<<gc, 128, 0, st>>>(b, mode);
    k_rb_place<3><<<g, 128, 0, st>>>(b, 1);
  } else {
    k_rb_pre<2><<<gc, 128, 0, st>>>(b, mode);
    k_rb_place<2><<<g, 128, 0, st>>>(b, 1);
  }
  launch_fin(b, false, false, 0, st);
}

void launch_rb_init(int dim, const Bufs& b, const float* pos, const float* vel, const float* frc, const float* rad,
                    const float* mass, const float4* q, const float* angv, const float* torque, const float* inertia,
                    const uint8_t* fixed, const int32_t* sys_of, float* world, cudaStream_t st) {
  if (b.NC == 0) return;
  const unsigned int gc = nblk_rb(b.NC, 128), g = nblk_rb(b.P, 256);
  if (dim == 3) {
    k_rb_init<3><<<gc, 128, 0, st>>>(b, pos, vel, frc, rad, mass, q, angv, torque, inertia, fixed, sys_of);
    k_rb_world<3><<<g, 256, 0, st>>>(b, world);
  } else {
    k_rb_init<2><<<gc, 128, 0, st>>>(b, pos, vel, frc, rad, mass, q, angv, torque, inertia, fixed, sys_of);
    k_rb_world<2><<<g, 256, 0, st>>>(b, world);
  }
}

void launch_rb_unpack(int dim, const Bufs& b, float* pos, float* vel, float* frc, float4* q, float* angv,
                      float* torque, bool per_sphere, cudaStream_t st) {
  if (b.P == 0) return;
  const unsigned int g = nblk_rb(b.P, 256);
  if (dim == 3) k_rb_unpack<3><<<g, 256, 0, st>>>(b, pos, vel, frc, q, angv, torque, per_sphere ? 1 : 0);
  else k_rb_unpack<2><<<g, 256, 0, st>>>(b, pos, vel, frc, q, angv, torque, per_sphere ? 1 : 0);
}

void launch_rb_world(int dim, const Bufs& b, float* pos, cudaStream_t st) {
  if (b.P == 0 || b.NC == 0) return;
  if (dim == 3) k_rb_world<3><<<nblk_rb(b.P, 256), 256, 0, st>>>(b, pos);
  else k_rb_world<2><<<nblk_rb(b.P, 256), 256, 0, st>>>(b, pos);
}

void launch_rb_energy(int dim, const Bufs& b, double* out, cudaStream_t st) {
  if (b.P == 0) return;
  if (dim == 3) k_rb_energy<3><<<nblk_rb(b.P, 256), 256, 0, st>>>(b, out);
  else k_rb_energy<2><<<nblk_rb(b.P, 256), 256, 0, st>>>(b, out);
}

}  // namespace jdem

// ---------------------------------------------------------------- host side

#include <cstring>
#include <string>
#include <unordered_map>
#include <vector>

#include "jdem_internal.h"

using namespace jdem;

// Groups the spheres of an upload into rigid clumps: (system, clump_id)
// pairs, numbered in order of first appearance, members in caller order.
// Leaves b.NC = 0 when every sphere is its own body at its centre.
int JdemHandle::setup_clumps(const JdemHostState* s, bool device_ptrs) {
  b.NC = 0;
  b.sclump = nullptr;
  if (!s->clump_id && !s->pos_p) return JDEM_OK;
  const size_t N = (size_t)P;
  if (N == 0) return JDEM_OK;
  std::vector<int32_t> cid(N);
  std::vector<float> pp(N * dim, 0.0f);
  auto fetch = [&](void* dst, const void* src, size_t bytes) -> bool {
    if (!device_ptrs) {
      std::memcpy(dst, src, bytes);
      return true;
    }
    // on the active stream: ordered after the caller's work that produced src
    return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, stream) == cudaSuccess &&
           cudaStreamSynchronize(stream) == cudaSuccess;
  };
  if (s->clump_id) {
    if (!fetch(cid.data(), s->clump_id, N * 4)) return fail(JDEM_ERR_CUDA, "upload: reading clump_id");
  } else {
    for (size_t i = 0; i < N; ++i) cid[i] = (int32_t)i;
  }
  if (s->pos_p && !fetch(pp.data(), s->pos_p, N * dim * 4)) return fail(JDEM_ERR_CUDA, "upload: reading pos_p");
  bool offset = false;
  for (float v : pp) offset |= v != 0.0f;
  // system of each caller index
  std::vector<int32_t> sys_of(N);
  {
    size_t off = 0;
    for (int s2 = 0; s2 < S; ++s2)
      for (long long k = 0; k < desc[s2].n; ++k) sys_of[off++] = s2;
  }
  std::unordered_map<long long, int32_t> index;
  index.reserve(N * 2);
  std::vector<int32_t> clump_of(N), count;
  for (size_t i = 0; i < N; ++i) {
    if (cid[i] < 0) return fail(JDEM_ERR_BAD_ARG, "upload: clump_id must be >= 0");
    const long long key = (long long)sys_of[i] * (1LL << 32) + cid[i];
    auto it = index.find(key);
    int32_t c;
    if (it == index.end()) {
      c = (int32_t)count.size();
      index.emplace(key, c);
      count.push_back(0);
    } else {
      c = it->second;
    }
    clump_of[i] = c;
    ++count[(size_t)c];
  }
  const long long NC = (long long)count.size();
  if (NC == (long long)N && !offset) return JDEM_OK;  // spheres
  std::vector<int32_t> start((size_t)NC + 1, 0), member(N);
  for (long long c = 0; c < NC; ++c) start[(size_t)c + 1] = start[(size_t)c] + count[(size_t)c];
  {
    std::vector<int32_t> fill(start.begin(), start.end() - 1);
    for (size_t i = 0; i < N; ++i) member[(size_t)fill[(size_t)clump_of[i]]++] = (int32_t)i;
  }
  int rc;
  if (NC > rb_cap_c) {
    void** arrays[] = {(void**)&b.cpos, (void**)&b.cvel, (void**)&b.cq, (void**)&b.cw, (void**)&b.ctq,
                       (void**)&b.cfrc, (void**)&b.cI, (void**)&b.cbrad, (void**)&b.cstart, (void**)&b.csys,
                       (void**)&b.cfixed};
    for (void** a : arrays) {
      dfree(*a);
      *a = nullptr;
    }
    rb_cap_c = 0;
    const size_t c4 = sizeof(float4) * (size_t)NC;
    if ((rc = dalloc((void**)&b.cpos, c4)) || (rc = dalloc((void**)&b.cvel, c4)) || (rc = dalloc((void**)&b.cq, c4)) ||
        (rc = dalloc((void**)&b.cw, c4)) || (rc = dalloc((void**)&b.ctq, c4)) || (rc = dalloc((void**)&b.cfrc, c4)) ||
        (rc = dalloc((void**)&b.cI, c4)) || (rc = dalloc((void**)&b.cbrad, sizeof(float) * (size_t)NC)) ||
        (rc = dalloc((void**)&b.cstart, sizeof(int32_t) * ((size_t)NC + 1))) ||
        (rc = dalloc((void**)&b.csys, sizeof(int32_t) * (size_t)NC)) || (rc = dalloc((void**)&b.cfixed, (size_t)NC)))
      return rc;
    rb_cap_c = NC;
  }
  if ((long long)N > rb_cap_p) {
    void** arrays[] = {(void**)&b.cmember, (void**)&b.spp, (void**)&b.sf, (void**)&b.stq, (void**)&rb_sclump};
    for (void** a : arrays) {
      dfree(*a);
      *a = nullptr;
    }
    rb_cap_p = 0;
    if ((rc = dalloc((void**)&b.cmember, sizeof(int32_t) * N)) || (rc = dalloc((void**)&b.spp, sizeof(float) * N * 3)) ||
        (rc = dalloc((void**)&b.sf, sizeof(float4) * N)) || (rc = dalloc((void**)&b.stq, sizeof(float4) * N)) ||
        (rc = dalloc((void**)&rb_sclump, sizeof(int32_t) * N)))
      return rc;
    rb_cap_p = (long long)N;
  }
  JDEM_CUDA_TRY(this, cudaMemcpyAsync(b.cstart, start.data(), start.size() * 4, cudaMemcpyHostToDevice, stream));
  JDEM_CUDA_TRY(this, cudaMemcpyAsync(b.cmember, member.data(), N * 4, cudaMemcpyHostToDevice, stream));
  JDEM_CUDA_TRY(this, cudaMemcpyAsync(rb_sclump, clump_of.data(), N * 4, cudaMemcpyHostToDevice, stream));
  JDEM_CUDA_TRY(this, cudaMemcpyAsync(b.spp, pp.data(), N * dim * 4, cudaMemcpyHostToDevice, stream));
  // the host vectors go out of scope: finish the copies first
  JDEM_CUDA_TRY(this, cudaStreamSynchronize(stream));
  b.NC = NC;
  b.sclump = rb_sclump;
  return JDEM_OK;
}
