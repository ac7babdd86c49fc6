// Pair arithmetic, stencil traversal and the fused per-particle step shared by
// the slot-order kernels (jdem_kernels.cu) and the tile kernels (jdem_tiles.cu).
#pragma once
#include "jdem_device.cuh"

namespace jdem {

template <typename T>
__device__ __forceinline__ T warp_max(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    T w = __shfl_xor_sync(0xffffffffu, v, o);
    v = v > w ? v : w;
  }
  return v;
}

// Warp max of the squared displacement; lane 0 raises the kernel-wide
// maximum only when it exceeds the value already recorded, so the atomic is
// rare.  No thread waits on another; k_fin folds the maximum in afterwards.
// Every lane of the warp must call it.
__device__ __forceinline__ void warp_disp(Ctl* ctl, float d2) {
  d2 = warp_max(d2);
  if ((threadIdx.x & 31) == 0 && d2 > 0.0f && d2 > __uint_as_float(__ldcg(&ctl->maxdisp2)))
    atomicMax(&ctl->maxdisp2, __float_as_uint(d2));
}

// Block max of the squared displacement (NT threads a block): one L2 read of the
// kernel-wide maximum, and rarely one atomic, per block instead of per warp --
// every warp of a large launch would otherwise poll the same L2 line.  Every
// thread of the block must call it.
template <int NT>
__device__ __forceinline__ void block_disp(Ctl* ctl, float d2) {
  __shared__ float s_w[NT / 32];
  d2 = warp_max(d2);
  if ((threadIdx.x & 31) == 0) s_w[threadIdx.x >> 5] = d2;
  __syncthreads();
  if (threadIdx.x == 0) {
    float m = s_w[0];
#pragma unroll
    for (int w = 1; w < NT / 32; ++w) m = s_w[w] > m ? s_w[w] : m;
    if (m > 0.0f && m > __uint_as_float(__ldcg(&ctl->maxdisp2))) atomicMax(&ctl->maxdisp2, __float_as_uint(m));
  }
}

// Minimum-image displacement and squared distance, in the reference's order
// (periodic.py:74-79: d - box * round(d / box)).  When every |d / box| <= 0.5
// the rounded multiple is +-0 and d - box * (+-0) == d, so the correction is
// only evaluated for pairs that straddle half a box length on some axis.
template <int DIM>
__device__ __forceinline__ float pair_disp(const SysParams& sp, bool per, float4 pi, float4 pj, float& dx,
                                           float& dy, float& dz) {
  dx = pi.x - pj.x;
  dy = pi.y - pj.y;
  dz = DIM == 3 ? pi.z - pj.z : 0.0f;
  if (per) {
    const float tx = dx * sp.inv_box[0], ty = dy * sp.inv_box[1];
    const float tz = DIM == 3 ? dz * sp.inv_box[2] : 0.0f;
    if (fabsf(tx) > 0.5f || fabsf(ty) > 0.5f || (DIM == 3 && fabsf(tz) > 0.5f)) {
      dx = dx - sp.box[0] * rintf(tx);
      dy = dy - sp.box[1] * rintf(ty);
      if (DIM == 3) dz = dz - sp.box[2] * rintf(tz);
    }
  }
  float dsq = dx * dx + dy * dy;
  if (DIM == 3) dsq = dsq + dz * dz;
  return dsq;
}

// Visit every slot binned in the unique stencil cells of a slot's cell
// (cell_list.py:66-96 stencil, deduplicated for small periodic grids).  The
// three cells of a stencil row along x form at most two contiguous slot ranges.
template <int DIM, typename F>
__device__ __forceinline__ void for_each_candidate(const int32_t* __restrict__ cs, const SysParams& sp,
                                                   long long local, F&& f) {
  const bool per = sp.domain == DOM_PERIODIC;
  const int gx = sp.g[0], gy = sp.g[1];
  int cx = (int)(local % gx);
  long long rem = local / gx;
  int cy = (int)(rem % gy);
  int cz = DIM == 3 ? (int)(rem / gy) : 0;
  int ys[3], zs[3];
  int ny = axis_set(cy, gy, per, ys);
  int nz = DIM == 3 ? axis_set(cz, sp.g[2], per, zs) : 1;
  if (DIM == 2) zs[0] = 0;
  int xa0, xb0, xa1, xb1;
  x_ranges(cx, gx, per, xa0, xb0, xa1, xb1);
  for (int iz = 0; iz < nz; ++iz) {
    for (int iy = 0; iy < ny; ++iy) {
      long long row = sp.c0 + ((long long)zs[iz] * gy + ys[iy]) * gx;
      int ja = cs[row + xa0], jb = cs[row + xb0];
      for (int j = ja; j < jb; ++j) f(j);
      if (xa1 < xb1) {
        ja = cs[row + xa1];
        jb = cs[row + xb1];
        for (int j = ja; j < jb; ++j) f(j);
      }
    }
  }
}

// Compensated contact-force accumulator of one particle: the spring law
// (spring.py:97-108) or the Hertz law (hertz.py:99-117).
template <int DIM, bool GENERAL, int LAW>
struct ContactSum {
  float fx = 0.f, fy = 0.f, fz = 0.f, ex = 0.f, ey = 0.f, ez = 0.f;
  float4 pi;
  float k0;
  int mat_i, oi, ci;
  bool per;
  const SysParams* sp;

  __device__ __forceinline__ ContactSum(const Bufs& b, const SysParams& s, float4 p, uint32_t tg, unsigned int sel,
                                        long long t)
      : pi(p), sp(&s) {
    per = s.domain == DOM_PERIODIC;
    mat_i = (tg >> TAG_MAT_SHIFT) & TAG_MAT_MASK;
    k0 = b.young[mat_i * b.n_mat + mat_i];
    oi = (GENERAL && ((b.bond_w > 0 && !b.interact_same_bond) || b.sclump)) ? b.orig[sel][t] : 0;
    ci = (GENERAL && b.sclump) ? b.sclump[oi] : 0;
  }

  // Adds the force on i due to j (position pj).  The slot j is read only for
  // the material and bond lookups of GENERAL; self pairs are never passed.
  // may_wrap == false asserts d - box * round(d / box) == d on every axis (a
  // list entry of the same periodic image), so the minimum image is skipped.
  // Returns the squared distance (the pruning test of k_force reads it).
  __device__ __forceinline__ float add(const Bufs& b, unsigned int sel, int j, const float4& pj,
                                       bool may_wrap = true) {
    float dx, dy, dz;
    const float dsq = pair_disp<DIM>(*sp, per && may_wrap, pi, pj, dx, dy, dz);
    const float R = pi.w + pj.w;
    if (dsq < R * R * 1.000001f) {
      float k = k0;
      // GENERAL: several materials or bond exclusions (valid_interaction_mask,
      // colliders/__init__.py:225-243); otherwise both checks compile away
      if (GENERAL && b.n_mat > 1) {
        int mat_j = (b.tag[sel][j] >> TAG_MAT_SHIFT) & TAG_MAT_MASK;
        k = b.young[mat_i * b.n_mat + mat_j];
      }
      if (GENERAL && b.bond_w > 0 && !b.interact_same_bond) {
        int oj = b.orig[sel][j];
        bool bonded = false;
        for (int w = 0; w < b.bond_w; ++w) bonded |= (b.bond[(long long)oi * b.bond_w + w] == oj);
        if (bonded) return dsq;
      }
      // spheres of one rigid clump do not interact (clump_i != clump_j)
      if (GENERAL && b.sclump && b.sclump[b.orig[sel][j]] == ci) return dsq;
      contact(k, dsq, R, pj.w, dx, dy, dz);
    }
    return dsq;
  }

  // add() for a list entry of a kernel without the GENERAL lookups (one pair
  // constant, no bond or clump exclusions), without branches: the contact
  // arithmetic runs for every entry and its magnitude is zeroed off contact (a
  // zero term leaves the two-sum accumulator unchanged bit for bit), so the
  // four entries of a batch interleave instead of taking a divergent branch
  // each; a padding entry (valid false: past the row's end, loaded with the
  // slot's own position) is evaluated the same way and discarded.  Returns the
  // squared distance, like add().  (1M spheres: 74.8 -> 72.4 us a force launch.)
  // The arithmetic is contact()'s, written out here with the mask (as a shared
  // helper the compiler allocated registers worse: 74.6 against 72.5 us).
  __device__ __forceinline__ float add_plain(const float4& pj, bool may_wrap, bool valid) {
    float dx, dy, dz;
    const float dsq = pair_disp<DIM>(*sp, per && may_wrap, pi, pj, dx, dy, dz);
    const float R = pi.w + pj.w;
    const bool hit = valid && dsq < R * R * 1.000001f;
    float inv = inv_norm(dsq);
    float rr = dsq * inv;
    float delta = R - rr;
    delta = delta > 0.0f ? delta : 0.0f;
    if (LAW == LAW_HERTZ) {
      const float rs = (pi.w * pj.w) / (pi.w + pj.w);
      float mag = (k0 * sqrtf(rs)) * (delta * sqrtf(delta));
      mag = hit ? mag : 0.0f;
      two_sum_acc(fx, ex, mag * (dx * inv));
      two_sum_acc(fy, ey, mag * (dy * inv));
      if (DIM == 3) two_sum_acc(fz, ez, mag * (dz * inv));
    } else {
      float mag = k0 * delta * inv;
      mag = hit ? mag : 0.0f;
      two_sum_acc(fx, ex, mag * dx);
      two_sum_acc(fy, ey, mag * dy);
      if (DIM == 3) two_sum_acc(fz, ez, mag * dz);
    }
    return dsq;
  }

  // Contact force of one candidate, summed with the two-sum accumulator.
  __device__ __forceinline__ void contact(float k, float dsq, float R, float rj, float dx, float dy, float dz) {
    float inv = inv_norm(dsq);
    float rr = dsq * inv;
    float delta = R - rr;
    delta = delta > 0.0f ? delta : 0.0f;
    if (LAW == LAW_HERTZ) {
      // k = (4/3) E* sqrt(R*), R* = Ri Rj / (Ri + Rj); F = k delta^(3/2) n,
      // n = r_ij / r (unit_and_norm); delta^(3/2) = delta * sqrt(delta)
      const float rs = (pi.w * rj) / (pi.w + rj);
      const float mag = (k * sqrtf(rs)) * (delta * sqrtf(delta));
      two_sum_acc(fx, ex, mag * (dx * inv));
      two_sum_acc(fy, ey, mag * (dy * inv));
      if (DIM == 3) two_sum_acc(fz, ez, mag * (dz * inv));
    } else {
      float mag = k * delta * inv;
      two_sum_acc(fx, ex, mag * dx);
      two_sum_acc(fy, ey, mag * dy);
      if (DIM == 3) two_sum_acc(fz, ez, mag * dz);
    }
  }
};

// After the contact force of slot t: ForceManager gravity
// (force_manager.py:393-405), step_after_force, and, in MODE_STEP, the next
// step's ReflectDomain.apply, step_before_force and drift.  Returns the
// squared displacement of the drift.
// v4 is the slot's velocity record (vx, vy, vz, mass), loaded by the caller.
template <int DIM>
__device__ __forceinline__ float integrate_particle(const Bufs& b, int mode, long long t, unsigned int sel,
                                                    unsigned int ps, const SysParams& sp, float4 pi, uint32_t tg,
                                                    float4 v4, float* F, float4* p_out = nullptr,
                                                    float4* v_out = nullptr) {
  const int base_mode = mode & 7;
  if (base_mode == MODE_FORCE_ONLY) {
    b.frc[sel][t] = make_float4(F[0], F[1], F[2], 0.0f);
    return 0.0f;
  }
  const int s = tg & TAG_SYS_MASK;
  float m = v4.w;
  bool fixed = (tg & TAG_FIXED) != 0u;
  float fr = fixed ? 0.0f : 1.0f;
  float p[3] = {pi.x, pi.y, pi.z}, v[3] = {v4.x, v4.y, v4.z};
  // the system's fields in registers: the stores below could alias the table for
  // the compiler, which would otherwise load them again
  const int lin = sp.lin, domain = sp.domain;
  const float dt = sp.dt;
  // the Verlet half kick dt * 0.5 / m (velocity_verlet.py:58-60, 92-94) is the same
  // before and after the force: one division
  const float sc_half = dt * 0.5f / m;
  // ForceManager.apply: F_contact + F_part(0) + gravity * (mass / count)
#pragma unroll
  for (int a = 0; a < DIM; ++a) F[a] = (F[a] + 0.0f) + sp.gravity[a] * (m / 1.0f);
  if (lin == LIN_VERLET) {
#pragma unroll
    for (int a = 0; a < DIM; ++a) v[a] = v[a] + F[a] * sc_half * fr;
  } else if (lin == LIN_EULER) {
    float sc = dt / m;
#pragma unroll
    for (int a = 0; a < DIM; ++a) {
      v[a] = v[a] + F[a] * sc * fr;
      p[a] = p[a] + dt * v[a];
    }
  }
  // nothing on the step path reads the force back: a streaming store
  __stcs(&b.frc[sel][t], make_float4(F[0], F[1], F[2], 0.0f));
  if (base_mode == MODE_STEP) {
    if ((mode & MODE_BBOX) && domain == DOM_FREE) {
#pragma unroll
      for (int a = 0; a < DIM; ++a) {
        atomicMin((unsigned int*)&b.bbox[s * 6 + a], f2ord(p[a] - pi.w));
        atomicMax((unsigned int*)&b.bbox[s * 6 + 3 + a], f2ord(p[a] + pi.w));
      }
    }
    if (domain == DOM_REFLECT) reflect_sphere<DIM>(sp, p, v, F, pi.w, m, fixed);
    if (lin == LIN_VERLET) {
#pragma unroll
      for (int a = 0; a < DIM; ++a) {
        v[a] = v[a] + F[a] * sc_half * fr;
        p[a] = p[a] + dt * v[a];
      }
    }
  }
  float d2max = 0.0f;
  float pa[3] = {pi.x, pi.y, pi.z};
#pragma unroll
  for (int a = 0; a < DIM; ++a) {
    float d = p[a] - pa[a];
    d2max = d2max + d * d;
  }
  b.pos[ps ^ 1u][t] = make_float4(p[0], p[1], p[2], pi.w);
  b.vel[sel][t] = make_float4(v[0], v[1], v[2], m);
  if (p_out) *p_out = make_float4(p[0], p[1], p[2], pi.w);  // the values just stored
  if (v_out) *v_out = make_float4(v[0], v[1], v[2], m);
  if (!(d2max == d2max) || d2max > 3.0e38f) {
    atomicOr(&b.ctl->status, ST_NONFINITE);
    d2max = 0.0f;
  }
  return d2max;
}

// One particle (slot t) of the fused step: contact force from the Verlet list
// `nb` (n slot indices, `stride` ints apart) when use_list is set, else from
// the stencil cells (periodic minimum image of periodic.py:74-79), then
// integrate_particle.  With `prune_out` set (a prune pass of the dynamic
// pruning) the entries within r_i + r_j + b.prune_skin are also copied, in
// list order, to the inner row prune_out (same stride) and their count to
// *prune_cnt.
template <int DIM, bool GENERAL, int LAW>
__device__ __forceinline__ float particle_step(const Bufs& b, int mode, long long t, unsigned int sel,
                                               unsigned int ps, bool use_list, const int32_t* __restrict__ nb,
                                               int n, int stride, int32_t* __restrict__ prune_out = nullptr,
                                               int32_t* __restrict__ prune_cnt = nullptr) {
  const float4* __restrict__ P = b.pos[ps];
  const float4 pi = P[t];
  const uint32_t tg = b.tag[sel][t];
  const SysParams& sp = b.sys[tg & TAG_SYS_MASK];
  ContactSum<DIM, GENERAL, LAW> acc(b, sp, pi, tg, sel, t);
  if (use_list && !idx_ok(b.ctl, n, (long long)b.nl_cap + 1)) n = 0;
  // Rows without GENERAL lookups load four words and four positions per batch
  // without per-entry branches: list rows hold a multiple of four entries, so
  // the last batch's words stay inside the row, and its padding entries load
  // the slot's own position and are discarded.
  if (!GENERAL && use_list && prune_out) {
    int m = 0;
    for (int k = 0; k < n; k += 4) {
      uint32_t e[4];
      float4 q[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) e[u] = (uint32_t)__ldcs(&nb[(k + u) * stride]);
#pragma unroll
      for (int u = 0; u < 4; ++u)
        q[u] = P[k + u < n && idx_ok(b.ctl, e[u] & kEntrySlot, b.P) ? (long long)(e[u] & kEntrySlot) : t];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const bool valid = k + u < n;
        const float dsq = acc.add_plain(q[u], (e[u] & kEntryImage) != 0u, valid);
        const float rc = (pi.w + q[u].w + b.prune_skin) * 1.0001f;
        if (valid && dsq < rc * rc && idx_ok(b.ctl, m, b.nl_cap)) prune_out[(m++) * stride] = (int32_t)e[u];
      }
    }
    *prune_cnt = m;
  } else if (!GENERAL && use_list) {
    for (int k = 0; k < n; k += 4) {
      uint32_t e[4];
      float4 q[4];
      // list words are read once per step: streaming loads, so they do not
      // displace the neighbours' positions from L1
#pragma unroll
      for (int u = 0; u < 4; ++u) e[u] = (uint32_t)__ldcs(&nb[(k + u) * stride]);
#pragma unroll
      for (int u = 0; u < 4; ++u)
        q[u] = P[k + u < n && idx_ok(b.ctl, e[u] & kEntrySlot, b.P) ? (long long)(e[u] & kEntrySlot) : t];
#pragma unroll
      for (int u = 0; u < 4; ++u) acc.add_plain(q[u], (e[u] & kEntryImage) != 0u, k + u < n);
    }
  } else if (use_list && prune_out) {
    // prune pass: the full row, keeping the entries the next passes need
    int m = 0;
    for (int k = 0; k < n; k += 4) {
      uint32_t e[4];
      float4 q[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) e[u] = k + u < n ? (uint32_t)__ldcs(&nb[(k + u) * stride]) : 0u;
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        if (k + u < n && !idx_ok(b.ctl, e[u] & kEntrySlot, b.P)) e[u] = (uint32_t)t;
        q[u] = k + u < n ? P[e[u] & kEntrySlot] : pi;
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        if (k + u < n) {
          const float dsq = acc.add(b, sel, (int)(e[u] & kEntrySlot), q[u], GENERAL || (e[u] & kEntryImage) != 0u);
          const float rc = (pi.w + q[u].w + b.prune_skin) * 1.0001f;
          if (dsq < rc * rc && idx_ok(b.ctl, m, b.nl_cap)) prune_out[(m++) * stride] = (int32_t)e[u];
        }
      }
    }
    *prune_cnt = m;
  } else if (use_list) {
    for (int k = 0; k < n; k += 4) {
      uint32_t e[4];
      float4 q[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) e[u] = k + u < n ? (uint32_t)__ldcs(&nb[(k + u) * stride]) : 0u;
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        if (k + u < n && !idx_ok(b.ctl, e[u] & kEntrySlot, b.P)) e[u] = (uint32_t)t;
        q[u] = k + u < n ? P[e[u] & kEntrySlot] : pi;
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        if (k + u < n) acc.add(b, sel, (int)(e[u] & kEntrySlot), q[u], GENERAL || (e[u] & kEntryImage) != 0u);
      }
    }
  } else {
    const long long local = b.key[sel][t] - sp.c0;
    if (idx_ok(b.ctl, local, (long long)sp.g[0] * sp.g[1] * (DIM == 3 ? sp.g[2] : 1)))
      for_each_candidate<DIM>(b.cell_start, sp, local, [&](int j) {
        if (j != (int)t) acc.add(b, sel, j, P[j]);
      });
  }
  float F[3] = {acc.fx + acc.ex, acc.fy + acc.ey, DIM == 3 ? acc.fz + acc.ez : 0.0f};
  // loaded after the contact loop: holding it through the loop costs registers
  const float4 v4 = (mode & 7) == MODE_FORCE_ONLY ? make_float4(0.f, 0.f, 0.f, 0.f) : b.vel[sel][t];
  return integrate_particle<DIM>(b, mode, t, sel, ps, sp, pi, tg, v4, F);
}

}  // namespace jdem
