// Fused force kernels of the GB300 DEM step engine, instantiated per
// dimension in jdem_force2.cu and jdem_force3.cu (the two compile in
// parallel): k_force, one thread per slot, for handles above kSmallForceSlots
// slots, and k_force_small, G lanes per slot, below.  Each comes in every shape
// the autotuner may pick (JdemConfig.force_block, JdemConfig.small_lanes).
#pragma once
#include "jdem_device.cuh"
#include "jdem_kernels.h"
#include "jdem_pair.cuh"

namespace jdem {

// The fused step, one thread per slot: particle_step of jdem_pair.cuh, from
// the slot's Verlet-list row when NL is set and no row overflowed, else from
// the stencil cells.  NT threads a block with 1280 / NT blocks resident per SM
// (48 registers): occupancy hides the dependent list-word -> position gather
// chain better than the spills cost (84.5 us against 90 us at 64 registers on
// 1M spheres).  A thread's arithmetic does not depend on NT, so every block
// shape gives the same trajectory bit for bit.
template <int DIM, bool NL, bool GENERAL, int LAW, int NT>
__global__ void __launch_bounds__(NT, 1280 / NT) k_force(Bufs b, int mode) {
  long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  // control fields earlier kernels set and this one only reads (of status only the
  // list-overflow bit, which the list build sets): read-only path
  unsigned int sel = ld_nc_u32(&b.ctl->sel), ps = ld_nc_u32(&b.ctl->pos_sel);
  const bool use_list = NL && (ld_nc_u32(&b.ctl->status) & ST_NL_OVERFLOW) == 0u;
  // dynamic pruning (uniform over the launch): a prune pass walks the full
  // list and writes the inner one; the other passes walk the inner list
  const bool pruning = use_list && b.nbr2 != nullptr;
  const bool prune = pruning && (ld_nc_u32(&b.ctl->prune) | ld_nc_u32(&b.ctl->nl_dirty)) != 0u;
  float d2max = 0.0f;
  if (t < b.P) {
    const long long row = ((t >> 5) * b.nl_cap) * 32 + (t & 31);
    const bool inner = pruning && !prune;
    const int n = use_list ? (inner ? b.ncnt2[t] : b.ncnt[t]) : 0;
    const int32_t* nb = use_list ? (inner ? b.nbr2 : b.nbr) + row : nullptr;
    if (use_list) {
      prefetch_list_block(b, t, n, inner);
      // the velocity record, read after the contact loop
      asm volatile("prefetch.global.L2 [%0];" ::"l"(&b.vel[sel][t]));
    }
    d2max = particle_step<DIM, GENERAL, LAW>(b, mode, t, sel, ps, use_list, nb, n, 32,
                                             prune ? b.nbr2 + row : nullptr, prune ? b.ncnt2 + t : nullptr);
  }
  if ((mode & 7) != MODE_FORCE_ONLY) block_disp<NT>(b.ctl, d2max);
}

// Small systems: with too few slots to fill the GPU the duration of k_force is
// one thread's chain of dependent list-entry -> position loads.  G lanes share
// a slot: lane g sums the row entries g, g + G, ... (compensated), the group's
// partial sums are combined in lane order, and its first lane integrates.
template <int DIM, bool GENERAL, int LAW, int G>
__global__ void __launch_bounds__(128) k_force_small(Bufs b, int mode) {
  const long long t = (blockIdx.x * 128LL + threadIdx.x) / G;
  const int lane = threadIdx.x & 31, g = lane % G, base = lane - g;
  const unsigned int sel = ld_nc_u32(&b.ctl->sel), ps = ld_nc_u32(&b.ctl->pos_sel);
  const bool use_list = b.nl_cap > 0 && (ld_nc_u32(&b.ctl->status) & ST_NL_OVERFLOW) == 0u;
  float fx = 0.f, fy = 0.f, fz = 0.f, ex = 0.f, ey = 0.f, ez = 0.f;
  float4 pi = make_float4(0.f, 0.f, 0.f, 0.f);
  uint32_t tg = 0u;
  if (t < b.P) {
    const float4* __restrict__ P = b.pos[ps];
    pi = P[t];
    tg = b.tag[sel][t];
    const SysParams& sp = b.sys[tg & TAG_SYS_MASK];
    ContactSum<DIM, GENERAL, LAW> acc(b, sp, pi, tg, sel, t);
    if (use_list) {
      int n = b.ncnt[t];
      if (!idx_ok(b.ctl, n, (long long)b.nl_cap + 1)) n = 0;
      const int32_t* nb = b.nbr + ((t >> 5) * b.nl_cap) * 32 + (t & 31);
      if (GENERAL) {
        for (int k = g; k < n; k += G) {
          uint32_t e = (uint32_t)nb[k * 32];
          if (!idx_ok(b.ctl, e & kEntrySlot, b.P)) e = (uint32_t)t;
          acc.add(b, sel, (int)(e & kEntrySlot), P[e & kEntrySlot], GENERAL || (e & kEntryImage) != 0u);
        }
      } else {
        // the lane's entries g, g + G, ... four at a time, without branches (padding
        // entries take the slot's own position and add nothing): the same terms in
        // the same order as one entry at a time
        for (int k0 = g; k0 < n; k0 += 4 * G) {
          uint32_t e[4];
          float4 q[4];
#pragma unroll
          for (int u = 0; u < 4; ++u) e[u] = k0 + u * G < n ? (uint32_t)nb[(k0 + u * G) * 32] : 0u;
#pragma unroll
          for (int u = 0; u < 4; ++u)
            q[u] = P[k0 + u * G < n && idx_ok(b.ctl, e[u] & kEntrySlot, b.P) ? (long long)(e[u] & kEntrySlot) : t];
#pragma unroll
          for (int u = 0; u < 4; ++u) acc.add_plain(q[u], (e[u] & kEntryImage) != 0u, k0 + u * G < n);
        }
      }
    } else {
      int c = 0;
      for_each_candidate<DIM>(b.cell_start, sp, b.key[sel][t] - sp.c0, [&](int j) {
        if (j == (int)t) return;
        if (c % G == g) acc.add(b, sel, j, P[j]);
        ++c;
      });
    }
    fx = acc.fx; fy = acc.fy; fz = acc.fz;
    ex = acc.ex; ey = acc.ey; ez = acc.ez;
  }
  // the group's partial sums, in lane order, into its first lane
#pragma unroll
  for (int s = 1; s < G; ++s) {
    const float ofx = __shfl_sync(0xffffffffu, fx, base + s), oex = __shfl_sync(0xffffffffu, ex, base + s);
    const float ofy = __shfl_sync(0xffffffffu, fy, base + s), oey = __shfl_sync(0xffffffffu, ey, base + s);
    const float ofz = __shfl_sync(0xffffffffu, fz, base + s), oez = __shfl_sync(0xffffffffu, ez, base + s);
    if (g == 0) {
      two_sum_acc(fx, ex, ofx);
      ex = ex + oex;
      two_sum_acc(fy, ey, ofy);
      ey = ey + oey;
      if (DIM == 3) {
        two_sum_acc(fz, ez, ofz);
        ez = ez + oez;
      }
    }
  }
  float d2max = 0.0f;
  if (t < b.P && g == 0) {
    const SysParams& sp = b.sys[tg & TAG_SYS_MASK];
    float F[3] = {fx + ex, fy + ey, DIM == 3 ? fz + ez : 0.0f};
    const float4 v4 = (mode & 7) == MODE_FORCE_ONLY ? make_float4(0.f, 0.f, 0.f, 0.f) : b.vel[sel][t];
    d2max = integrate_particle<DIM>(b, mode, t, sel, ps, sp, pi, tg, v4, F);
  }
  if ((mode & 7) != MODE_FORCE_ONLY) warp_disp(b.ctl, d2max);
}

template <int DIM, bool GENERAL, int LAW>
void launch_force_small_g(const Bufs& b, int mode, cudaStream_t st) {
  const int G = b.small_lanes;
  const unsigned int gs = (unsigned int)((b.P * G + 127) / 128);
  if (G == 4) k_force_small<DIM, GENERAL, LAW, 4><<<gs, 128, 0, st>>>(b, mode);
  else if (G == 16) k_force_small<DIM, GENERAL, LAW, 16><<<gs, 128, 0, st>>>(b, mode);
  else k_force_small<DIM, GENERAL, LAW, 8><<<gs, 128, 0, st>>>(b, mode);
}

template <int DIM, bool NL, bool GENERAL, int LAW>
void launch_force_nt(const Bufs& b, int mode, cudaStream_t st) {
  // the block shapes are instantiated for the list path; the cell traversal
  // (no list, or a step whose row overflowed) always takes 128 threads
  const int NT = NL ? b.force_block : 128;
  const unsigned int g = (unsigned int)((b.P + NT - 1) / NT);
  if (NL && NT == 64) k_force<DIM, NL, GENERAL, LAW, 64><<<g, 64, 0, st>>>(b, mode);
  else if (NL && NT == 256) k_force<DIM, NL, GENERAL, LAW, 256><<<g, 256, 0, st>>>(b, mode);
  else k_force<DIM, NL, GENERAL, LAW, 128><<<g, 128, 0, st>>>(b, mode);
}

template <int DIM>
void launch_force_dim(const Bufs& b, int mode, cudaStream_t st) {
  const bool gen = b.n_mat > 1 || (b.bond_w > 0 && !b.interact_same_bond);
  const bool hertz = b.law == LAW_HERTZ;
  if (b.P <= kSmallForceSlots) {
    if (gen) hertz ? launch_force_small_g<DIM, true, LAW_HERTZ>(b, mode, st) : launch_force_small_g<DIM, true, LAW_SPRING>(b, mode, st);
    else hertz ? launch_force_small_g<DIM, false, LAW_HERTZ>(b, mode, st) : launch_force_small_g<DIM, false, LAW_SPRING>(b, mode, st);
    return;
  }
  if (b.nl_cap > 0) {
    if (gen) hertz ? launch_force_nt<DIM, true, true, LAW_HERTZ>(b, mode, st) : launch_force_nt<DIM, true, true, LAW_SPRING>(b, mode, st);
    else hertz ? launch_force_nt<DIM, true, false, LAW_HERTZ>(b, mode, st) : launch_force_nt<DIM, true, false, LAW_SPRING>(b, mode, st);
  } else {
    if (gen) hertz ? launch_force_nt<DIM, false, true, LAW_HERTZ>(b, mode, st) : launch_force_nt<DIM, false, true, LAW_SPRING>(b, mode, st);
    else hertz ? launch_force_nt<DIM, false, false, LAW_HERTZ>(b, mode, st) : launch_force_nt<DIM, false, false, LAW_SPRING>(b, mode, st);
  }
}

}  // namespace jdem
