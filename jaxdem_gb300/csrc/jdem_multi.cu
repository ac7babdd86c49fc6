// Small systems: many steps per launch.
//
// A system of a few thousand spheres fills a fraction of the GPU, and a
// step's force kernel is one chain of dependent loads; launching it (and the
// 1-thread k_fin) once per step costs more than the step itself.  k_multi is
// a cooperative launch (every block resident) that runs the steps of a chunk
// back to back with one grid barrier per step, and ends when the chunk is
// done or when the displacement bound calls for a re-sort.  The captured
// chunk is a while node whose body is the re-sort kernels (each returns at
// once when nothing is due), the list build and k_multi, which sets the
// while condition.
//
// Each step is k_force_small's (Bufs.small_lanes lanes a slot, the same
// operations in the same order) followed by k_fin's bound update, which every block evaluates
// from the same inputs, so the trajectory is bit-identical to the launch per
// step.  Positions written by other blocks in the previous step are read
// with L2-coherent loads (never the read-only path).
#include "jdem_device.cuh"
#include "jdem_kernels.h"
#include "jdem_pair.cuh"

namespace jdem {

namespace {

constexpr int kMultiT = 128;        // threads per block
constexpr int kMultiE = 6;          // list entries a lane keeps in registers (row entries g, g + G, ...; rows up to 6 G)
constexpr int kMultiMaxSys = 8;     // systems of a handle that takes the many-step path
constexpr unsigned int kBarrierSpins = 1u << 21;  // polls of the arrival count (about a second) before a barrier gives up

__device__ __forceinline__ unsigned int ld_relaxed_u32(const unsigned int* p) {
  unsigned int v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ unsigned int ld_acquire_u32(const unsigned int* p) {
  unsigned int v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void red_release_add(unsigned int* p, unsigned int v) {
  asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ void fence_acquire() { asm volatile("fence.acq_rel.gpu;" ::: "memory"); }

__device__ __forceinline__ float4 ldc4(const float4* p) { return __ldcg(p); }

// Grid barrier of a cooperative launch that also reduces step s's largest
// squared drift.  Thread 0 of each block folds its warps' maxima (s_wmax)
// into ctl->mx[s % 3] and arrives with one release add on the never-reset
// arrival count; every block then polls the count with acquire loads until
// it reaches its target (the launch's base plus gridDim.x per barrier) and
// reads the slot.  Bounded: a block that polls max_spins times
// records ST_BARRIER_TIMEOUT and returns false.  `extra` arrivals beyond the
// grid's are awaited too; they never come, so extra > 0 makes every block
// give up (the timeout path, exercised by a test through jdem_set_barrier_limit).
__device__ __forceinline__ bool grid_barrier_max(Ctl* ctl, unsigned int& target, unsigned int s,
                                                 const float* s_wmax, float& m2, unsigned int max_spins,
                                                 unsigned int extra) {
  __shared__ int s_ok;
  __shared__ unsigned int s_m2;
  __syncthreads();
  if (threadIdx.x == 0) {
    float bmax = 0.0f;
#pragma unroll
    for (int w = 0; w < kMultiT / 32; ++w) bmax = fmaxf(bmax, s_wmax[w]);
    unsigned int* slot = &ctl->mx[s % 3u];
    if (bmax > 0.0f) atomicMax(slot, __float_as_uint(bmax));
    red_release_add(&ctl->bar_count, 1u);
    target += gridDim.x;
    int ok = 1;
    unsigned int spins = 0;
    // acquire polls: the one that sees every arrival orders this block's later
    // reads after the other blocks' released writes (a separate fence after a
    // relaxed poll cost 0.25-0.3 us a step at 4096 spheres)
    while ((int)(ld_acquire_u32(&ctl->bar_count) - (target + extra)) < 0) {
      if (++spins > max_spins) {
        atomicOr(&ctl->status, ST_BARRIER_TIMEOUT);
        ok = 0;
        break;
      }
    }
    if (!ok) fence_acquire();
    s_ok = ok;
    s_m2 = ld_relaxed_u32(slot);
  }
  __syncthreads();
  m2 = __uint_as_float(s_m2);
  return s_ok != 0;
}

// ctl->steps_left = n: the steps of the captured chunk.
__global__ void k_multi_init(Ctl* ctl, unsigned int n) { ctl->steps_left = n; }

// Steps of one chunk until it ends or a re-sort is due.  A group of G lanes
// (4, 8 or 16, as k_force_small's) owns slot t: the row entries, tag and system of the slot are loaded
// once per launch (they change only at a re-sort), and the group's position
// and the first lane's velocity stay in registers from step to step (the
// group is their only writer), so a step's only dependent global loads are
// the neighbours' positions, written by other blocks in the previous step and
// read through L2.  The operations and their order are k_force_small's and
// k_fin's.
template <int DIM, bool GENERAL, int LAW, int G>
__global__ void __launch_bounds__(kMultiT) k_multi(Bufs b, cudaGraphConditionalHandle hw) {
  Ctl* ctl = b.ctl;
  const bool lead = blockIdx.x == 0 && threadIdx.x == 0;
  unsigned int left = ld_cg_u32(&ctl->steps_left);
  if (left == 0u) {  // the chunk is done (the same value in every block)
    if (lead) cudaGraphSetConditional(hw, 0u);
    return;
  }
  __shared__ float s_wmax[kMultiT / 32];
  // arrivals counted when the previous launch ended (every block of it had arrived)
  unsigned int target = ld_cg_u32(&ctl->bar_base);
  unsigned int s = ld_cg_u32(&ctl->mstep);
  const unsigned int sel = ld_cg_u32(&ctl->sel);
  unsigned int ps = ld_cg_u32(&ctl->pos_sel);
  const bool use_list = b.nl_cap > 0 && (ld_cg_u32(&ctl->status) & ST_NL_OVERFLOW) == 0u;
  float bound = __ldcg(&ctl->bound);
  const float skin_half = __ldcg(&ctl->skin_half);

  // The system table in shared memory: the acquire fence of every barrier
  // drops L1, and the integrator reads the system's fields every step.
  __shared__ SysParams s_sys[kMultiMaxSys];
  for (int i = threadIdx.x; i < b.S; i += kMultiT) s_sys[i] = b.sys[i];
  __syncthreads();

  const long long t = (blockIdx.x * (long long)kMultiT + threadIdx.x) / G;
  const int lane = threadIdx.x & 31, g = lane % G, base = lane - g;
  const bool live = t < b.P;
  uint32_t tg = 0u;
  int n = 0;
  const SysParams* spp = &s_sys[0];
  float4 pi = make_float4(0.f, 0.f, 0.f, 0.f), v4 = pi;
  const int32_t* nb = nullptr;
  uint32_t ent[kMultiE];
#pragma unroll
  for (int i = 0; i < kMultiE; ++i) ent[i] = 0u;
  if (live) {
    tg = b.tag[sel][t];
    spp = &s_sys[tg & TAG_SYS_MASK];
    pi = ldc4(&b.pos[ps][t]);
    if (g == 0) v4 = ldc4(&b.vel[sel][t]);
    if (use_list) {
      n = b.ncnt[t];
      if (!idx_ok(b.ctl, n, (long long)b.nl_cap + 1)) n = 0;
      nb = b.nbr + ((t >> 5) * b.nl_cap) * 32 + (t & 31);
#pragma unroll
      for (int i = 0; i < kMultiE; ++i) {
        const int k = g + i * G;
        ent[i] = k < n ? (uint32_t)nb[k * 32] : 0u;
        if (k < n && !idx_ok(b.ctl, ent[i] & kEntrySlot, b.P)) ent[i] = (uint32_t)t;
      }
    }
  }

  // per-slot material constants, read once
  ContactSum<DIM, GENERAL, LAW> acc(b, *spp, pi, tg, sel, live ? t : 0);

  bool ok = true;
  for (;;) {
    float fx = 0.f, fy = 0.f, fz = 0.f, ex = 0.f, ey = 0.f, ez = 0.f;
    if (live) {
      const float4* P = b.pos[ps];
      acc.fx = acc.fy = acc.fz = acc.ex = acc.ey = acc.ez = 0.0f;
      acc.pi = pi;
      if (use_list) {
        float4 q[kMultiE];
#pragma unroll
        for (int i = 0; i < kMultiE; ++i) q[i] = g + i * G < n ? ldc4(&P[ent[i] & kEntrySlot]) : pi;
#pragma unroll
        for (int i = 0; i < kMultiE; ++i) {
          if (GENERAL) {
            if (g + i * G < n)
              acc.add(b, sel, (int)(ent[i] & kEntrySlot), q[i], GENERAL || (ent[i] & kEntryImage) != 0u);
          } else {
            // branch-free (the padding entries hold the slot's own position): the
            // entries' arithmetic interleaves, and the sums equal k_force_small's
            acc.add_plain(q[i], (ent[i] & kEntryImage) != 0u, g + i * G < n);
          }
        }
        for (int k = g + kMultiE * G; k < n; k += G) {
          uint32_t e = (uint32_t)nb[k * 32];
          if (!idx_ok(b.ctl, e & kEntrySlot, b.P)) e = (uint32_t)t;
          acc.add(b, sel, (int)(e & kEntrySlot), ldc4(&P[e & kEntrySlot]), GENERAL || (e & kEntryImage) != 0u);
        }
      } else {
        int c = 0;
        for_each_candidate<DIM>(b.cell_start, *spp, b.key[sel][t] - spp->c0, [&](int j) {
          if (j == (int)t) return;
          if (c % G == g) acc.add(b, sel, j, ldc4(&P[j]));
          ++c;
        });
      }
      fx = acc.fx; fy = acc.fy; fz = acc.fz;
      ex = acc.ex; ey = acc.ey; ez = acc.ez;
    }
    // the group's partial sums, in lane order, into its first lane
#pragma unroll
    for (int k = 1; k < G; ++k) {
      const float ofx = __shfl_sync(0xffffffffu, fx, base + k), oex = __shfl_sync(0xffffffffu, ex, base + k);
      const float ofy = __shfl_sync(0xffffffffu, fy, base + k), oey = __shfl_sync(0xffffffffu, ey, base + k);
      const float ofz = __shfl_sync(0xffffffffu, fz, base + k), oez = __shfl_sync(0xffffffffu, ez, base + k);
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
    float d2 = 0.0f;
    if (live && g == 0) {
      float F[3] = {fx + ex, fy + ey, DIM == 3 ? fz + ez : 0.0f};
      float4 pn, vn;
      d2 = integrate_particle<DIM>(b, MODE_STEP, t, sel, ps, *spp, pi, tg, v4, F, &pn, &vn);
      pi = pn;
      v4 = vn;
    }
    // the new position to every lane of the group
    pi.x = __shfl_sync(0xffffffffu, pi.x, base);
    pi.y = __shfl_sync(0xffffffffu, pi.y, base);
    pi.z = __shfl_sync(0xffffffffu, pi.z, base);
    pi.w = __shfl_sync(0xffffffffu, pi.w, base);
    d2 = warp_max(d2);
    if (lane == 0) s_wmax[threadIdx.x >> 5] = d2;
    float m2;
    ok = grid_barrier_max(ctl, target, s, s_wmax, m2, b.bar_spins ? b.bar_spins : kBarrierSpins, b.bar_extra);
    if (!ok) break;
    // k_fin: bound += sqrt(max squared drift); positions flip
    bound = bound + sqrtf(m2);
    ps ^= 1u;
    --left;
    // the slot of step s + 2 was last read, by every block, before this barrier
    if (lead) ctl->mx[(s + 2u) % 3u] = 0u;
    ++s;
    if (bound > skin_half || left == 0u) break;
  }
  if (lead) {
    ctl->bar_base = target;
    ctl->mstep = s;
    ctl->bound = bound;
    ctl->pos_sel = ps;
    ctl->nl_dirty = 0u;
    if (bound > skin_half) ctl->need_rebuild = 1u;
    if (!ok) left = 0u;  // barrier failure: stop the chunk, the host reports the status
    ctl->steps_left = left;
    cudaGraphSetConditional(hw, left > 0u ? 1u : 0u);
  }
}

template <int DIM, bool GENERAL, int LAW, int G>
int multi_blocks_per_sm() {
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_multi<DIM, GENERAL, LAW, G>, kMultiT, 0) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return nb;
}

template <int DIM, bool GENERAL, int LAW, int G>
int launch_multi_t(const Bufs& b, cudaGraphConditionalHandle hw, unsigned int grid, cudaStream_t st) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(kMultiT);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k_multi<DIM, GENERAL, LAW, G>, b, hw) == cudaSuccess ? 0 : 1;
}

unsigned int multi_grid(const Bufs& b) { return (unsigned int)((b.P * b.small_lanes + kMultiT - 1) / kMultiT); }

// occupancy and launch of the instance for the handle's lane count
template <int DIM, bool GENERAL, int LAW>
int multi_blocks_per_sm_g(const Bufs& b) {
  if (b.small_lanes == 4) return multi_blocks_per_sm<DIM, GENERAL, LAW, 4>();
  if (b.small_lanes == 16) return multi_blocks_per_sm<DIM, GENERAL, LAW, 16>();
  return multi_blocks_per_sm<DIM, GENERAL, LAW, 8>();
}

template <int DIM, bool GENERAL, int LAW>
int launch_multi_g(const Bufs& b, cudaGraphConditionalHandle hw, unsigned int grid, cudaStream_t st) {
  if (b.small_lanes == 4) return launch_multi_t<DIM, GENERAL, LAW, 4>(b, hw, grid, st);
  if (b.small_lanes == 16) return launch_multi_t<DIM, GENERAL, LAW, 16>(b, hw, grid, st);
  return launch_multi_t<DIM, GENERAL, LAW, 8>(b, hw, grid, st);
}

bool multi_general(const Bufs& b) { return b.n_mat > 1 || (b.bond_w > 0 && !b.interact_same_bond); }

}  // namespace

bool multi_eligible(int dim, const Bufs& b, int device) {
  if (b.P <= 0 || b.P > kSmallForceSlots || b.NC || b.law == LAW_CS || b.S > kMultiMaxSys) return false;
  int sms = 0, coop = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
      cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, device) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (!coop) return false;
  const bool gen = multi_general(b), hertz = b.law == LAW_HERTZ;
  int per_sm;
  if (dim == 3) {
    per_sm = gen ? (hertz ? multi_blocks_per_sm_g<3, true, LAW_HERTZ>(b) : multi_blocks_per_sm_g<3, true, LAW_SPRING>(b))
                 : (hertz ? multi_blocks_per_sm_g<3, false, LAW_HERTZ>(b) : multi_blocks_per_sm_g<3, false, LAW_SPRING>(b));
  } else {
    per_sm = gen ? (hertz ? multi_blocks_per_sm_g<2, true, LAW_HERTZ>(b) : multi_blocks_per_sm_g<2, true, LAW_SPRING>(b))
                 : (hertz ? multi_blocks_per_sm_g<2, false, LAW_HERTZ>(b) : multi_blocks_per_sm_g<2, false, LAW_SPRING>(b));
  }
  return (long long)per_sm * sms >= (long long)multi_grid(b);
}

void launch_multi_init(const Bufs& b, unsigned int n, cudaStream_t st) { k_multi_init<<<1, 1, 0, st>>>(b.ctl, n); }

int launch_multi(int dim, const Bufs& b, cudaGraphConditionalHandle hw, cudaStream_t st) {
  const unsigned int grid = multi_grid(b);
  const bool gen = multi_general(b), hertz = b.law == LAW_HERTZ;
  if (dim == 3) {
    if (gen) return hertz ? launch_multi_g<3, true, LAW_HERTZ>(b, hw, grid, st) : launch_multi_g<3, true, LAW_SPRING>(b, hw, grid, st);
    return hertz ? launch_multi_g<3, false, LAW_HERTZ>(b, hw, grid, st) : launch_multi_g<3, false, LAW_SPRING>(b, hw, grid, st);
  }
  if (gen) return hertz ? launch_multi_g<2, true, LAW_HERTZ>(b, hw, grid, st) : launch_multi_g<2, true, LAW_SPRING>(b, hw, grid, st);
  return hertz ? launch_multi_g<2, false, LAW_HERTZ>(b, hw, grid, st) : launch_multi_g<2, false, LAW_SPRING>(b, hw, grid, st);
}

}  // namespace jdem
