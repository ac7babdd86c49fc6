// Kernels of the GB300 DEM step engine.
//
// Per step, in steady state, one kernel runs: k_force<DIM> evaluates the
// spring contact force of every particle against the particles binned in its
// 3^DIM stencil, adds gravity, applies the after-force half kick and, in the
// same pass, the next step's wall reflection, before-force half kick and drift
// (system.py:60-82 order).  Re-binning (counting sort by cell) runs only when
// the accumulated displacement bound exceeds half the skin; the rebuild
// kernels read a device flag and return at once otherwise.
//
// No atomics touch forces: every pair is evaluated from both sides, as the
// reference does (cell_list.py:222-260), and each thread sums its own row with
// a compensated (two-sum) accumulator, so results are deterministic.
#include "jdem_device.cuh"
#include "jdem_kernels.h"
#include "jdem_pair.cuh"
#include "jdem_rot.cuh"

namespace jdem {

// ---------------------------------------------------------------- utilities

// After a kernel that moved particles: bound += max displacement, raise
// need_rebuild past skin / 2; after a force kernel also flip the position
// buffer and retire the list-build request.  Inside a captured step it sets
// the condition of the next step's re-sort body.
enum : int { FIN_AFTER_FORCE = 1, FIN_SET_COND = 2 };

__global__ void k_fin(Ctl* ctl, int flags, cudaGraphConditionalHandle h) {
  float m2 = __uint_as_float(atomicExch(&ctl->maxdisp2, 0u));
  const float d = sqrtf(m2);
  float bd = ctl->bound + d;
  ctl->bound = bd;
  unsigned int nr = ctl->need_rebuild;
  if (bd > ctl->skin_half) nr = 1u;
  ctl->need_rebuild = nr;
  unsigned int nd = ctl->nl_dirty;
  // dynamic pruning: a force pass that rebuilt the inner list (prune or a
  // fresh outer list) restarts the drift count from its positions; the next
  // force pass prunes once the drift exceeds half the prune skin
  const bool pruned = (flags & FIN_AFTER_FORCE) && (ctl->prune | nd);
  if (pruned && ctl->pskin_half > 0.0f) ctl->prunes += 1u;
  const float pb = pruned ? d : ctl->pbound + d;
  ctl->pbound = pb;
  ctl->prune = pb > ctl->pskin_half ? 1u : 0u;
  if (flags & FIN_AFTER_FORCE) {
    ctl->pos_sel ^= 1u;
    nd = 0u;
    ctl->nl_dirty = 0u;
  }
  if (flags & FIN_SET_COND) cudaGraphSetConditional(h, (nr | nd) ? 1u : 0u);
}

// ------------------------------------------------------------ pack / unpack

// Caller-order staging arrays -> slot arrays (identity order); a re-sort
// follows before the first force evaluation.
template <int DIM>
__global__ void k_pack(Bufs b, const float* __restrict__ pos, const float* __restrict__ vel,
                       const float* __restrict__ frc, const float* __restrict__ rad,
                       const float* __restrict__ mass, const int32_t* __restrict__ mat,
                       const uint8_t* __restrict__ fixed, const int32_t* __restrict__ sys_of) {
  long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= b.P) return;
  float p[3] = {0, 0, 0}, v[3] = {0, 0, 0}, f[3] = {0, 0, 0};
#pragma unroll
  for (int a = 0; a < DIM; ++a) {
    p[a] = pos[i * DIM + a];
    v[a] = vel[i * DIM + a];
    f[a] = frc[i * DIM + a];
  }
  b.pos[0][i] = make_float4(p[0], p[1], p[2], rad[i]);
  b.pos[1][i] = b.pos[0][i];
  b.vel[0][i] = make_float4(v[0], v[1], v[2], mass[i]);
  b.frc[0][i] = make_float4(f[0], f[1], f[2], 0.0f);
  uint32_t tg = (uint32_t)sys_of[i] | (((uint32_t)mat[i] & TAG_MAT_MASK) << TAG_MAT_SHIFT) |
                (fixed[i] ? TAG_FIXED : 0u);
  b.tag[0][i] = tg;
  b.orig[0][i] = (int32_t)i;
  b.key[0][i] = 0;
}

// Slot arrays -> caller order (reference (N, dim) layout).
template <int DIM>
__global__ void k_unpack(Bufs b, float* __restrict__ pos, float* __restrict__ vel,
                         float* __restrict__ frc) {
  long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= b.P) return;
  unsigned int sel = ld_nc_u32(&b.ctl->sel), ps = ld_nc_u32(&b.ctl->pos_sel);
  long long i = b.orig[sel][t];
  // a null destination skips that field (trajectory frames select fields)
  if (pos) {
    float4 p = b.pos[ps][t];
    pos[i * DIM + 0] = p.x;
    pos[i * DIM + 1] = p.y;
    if (DIM == 3) pos[i * DIM + 2] = p.z;
  }
  if (vel) {
    float4 v = b.vel[sel][t];
    vel[i * DIM + 0] = v.x;
    vel[i * DIM + 1] = v.y;
    if (DIM == 3) vel[i * DIM + 2] = v.z;
  }
  if (frc) {
    float4 f = b.frc[sel][t];
    frc[i * DIM + 0] = f.x;
    frc[i * DIM + 1] = f.y;
    if (DIM == 3) frc[i * DIM + 2] = f.z;
  }
}

// Free-domain bounding box accumulators: ordered-int +inf in the min words,
// -inf in the max words of every system.
__global__ void k_bbox_reset(unsigned int* __restrict__ bb, int S) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < S * 6) bb[k] = (k % 6) < 3 ? 0xFFFFFFFFu : 0u;
}

// --------------------------------------------------------------- re-binning

// Free domain: binning frame = bounding box of the spheres (domains/free.py:59-63),
// one block per free system; grid capped at the system's cell capacity.
template <int DIM>
__global__ void k_grid_free(Bufs b) {
  if (ld_nc_u32(&b.ctl->need_rebuild) == 0u) return;
  int s = blockIdx.x;
  SysParams& sp = b.sys[s];
  if (sp.domain != DOM_FREE) return;
  unsigned int ps = ld_nc_u32(&b.ctl->pos_sel);
  float lo[3] = {3.4e38f, 3.4e38f, 3.4e38f}, hi[3] = {-3.4e38f, -3.4e38f, -3.4e38f};
  for (long long t = sp.p0 + threadIdx.x; t < sp.p0 + sp.np; t += blockDim.x) {
    float4 p = b.pos[ps][t];
    float pa[3] = {p.x, p.y, p.z};
#pragma unroll
    for (int a = 0; a < DIM; ++a) {
      lo[a] = fminf(lo[a], pa[a] - p.w);
      hi[a] = fmaxf(hi[a], pa[a] + p.w);
    }
  }
  __shared__ float slo[3][256], shi[3][256];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    slo[a][threadIdx.x] = lo[a];
    shi[a][threadIdx.x] = hi[a];
  }
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w)
      for (int a = 0; a < 3; ++a) {
        slo[a][threadIdx.x] = fminf(slo[a][threadIdx.x], slo[a][threadIdx.x + w]);
        shi[a][threadIdx.x] = fmaxf(shi[a][threadIdx.x], shi[a][threadIdx.x + w]);
      }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    double cell = sp.cell_bin;
    long long g[3] = {1, 1, 1};
    for (int it = 0; it < 64; ++it) {
      long long tot = 1;
      for (int a = 0; a < DIM; ++a) {
        double ext = (double)shi[a][0] - (double)slo[a][0];
        double q = ext / cell;
        g[a] = (q >= 1.0 && q < 1.0e9) ? (long long)ceil(q) : 1;
        if (g[a] > sp.ncap) g[a] = sp.ncap;
        tot *= g[a];
      }
      if (tot <= sp.ncap) break;
      cell *= 1.26;
    }
    long long tot = 1;
    for (int a = 0; a < DIM; ++a) tot *= g[a];
    if (tot > sp.ncap)
      for (int a = 0; a < DIM; ++a) g[a] = 1;  // non-finite extent: one cell, still correct
    for (int a = 0; a < DIM; ++a) {
      sp.glo[a] = isfinite(slo[a][0]) ? slo[a][0] : 0.0f;
      sp.gcell[a] = (float)cell;
      sp.g[a] = (int)g[a];
    }
    if (DIM == 2) sp.g[2] = 1;
  }
}

// Cell key of every slot + per-cell occupancy (the rank inside the cell comes
// from the atomic and is made deterministic by k_cellsort).
template <int DIM>
__global__ void k_bin(Bufs b) {
  if (ld_nc_u32(&b.ctl->need_rebuild) == 0u) return;
  long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= b.P) return;
  unsigned int sel = ld_nc_u32(&b.ctl->sel), ps = ld_nc_u32(&b.ctl->pos_sel);
  float4 p = b.pos[ps][t];
  uint32_t tg = b.tag[sel][t];
  const SysParams& sp = b.sys[tg & TAG_SYS_MASK];
  int cx = cell_coord(sp, 0, p.x);
  int cy = cell_coord(sp, 1, p.y);
  long long local = (long long)cy * sp.g[0] + cx;
  if (DIM == 3) {
    int cz = cell_coord(sp, 2, p.z);
    local += (long long)cz * sp.g[0] * sp.g[1];
  }
  int key = (int)(sp.c0 + local);
  if (!idx_ok(b.ctl, key, b.C)) key = 0;
  b.key_tmp[t] = key;
  // one atomic per distinct cell of the warp: slots are ordered by cell since
  // the last re-sort, so neighbouring lanes mostly share a cell
  const unsigned int active = __activemask();
  const unsigned int peers = __match_any_sync(active, key);
  const int leader = __ffs(peers) - 1;
  const int lane = threadIdx.x & 31;
  int base = 0;
  if (lane == leader) base = atomicAdd(&b.cnt[key], __popc(peers));
  base = __shfl_sync(peers, base, leader);
  b.slot_tmp[t] = base + __popc(peers & ((1u << lane) - 1u));
}

constexpr int SCAN_T = 256, SCAN_V = 8, SCAN_TILE = SCAN_T * SCAN_V;

// exclusive scan of cnt[0..C) -> cell_start[0..C], cell_start[C] = P.
__device__ __forceinline__ int block_excl_scan(int v, int* sh, int& total) {
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sh[wid] = x;
  __syncthreads();
  if (wid == 0) {
    int nw = blockDim.x >> 5;
    int w = lane < nw ? sh[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < nw) sh[lane] = w;
  }
  __syncthreads();
  int warp_off = wid > 0 ? sh[wid - 1] : 0;
  total = sh[(blockDim.x >> 5) - 1];
  __syncthreads();
  return warp_off + x - v;
}

__global__ void k_scan_reduce(Bufs b) {
  if (ld_nc_u32(&b.ctl->need_rebuild) == 0u) return;
  __shared__ int sh[32];
  long long base = (long long)blockIdx.x * SCAN_TILE;
  int s = 0;
#pragma unroll
  for (int k = 0; k < SCAN_V; ++k) {
    long long c = base + (long long)threadIdx.x * SCAN_V + k;
    if (c < b.C) s += b.cnt[c];
  }
  int total;
  block_excl_scan(s, sh, total);
  if (threadIdx.x == 0) b.scan_blk[blockIdx.x] = total;
}

__global__ void k_scan_top(Bufs b, int nblk) {
  if (ld_nc_u32(&b.ctl->need_rebuild) == 0u) return;
  __shared__ int sh[32];
  // one block of 1024 threads, each owning a run of ceil(nblk/1024) entries
  int per = (nblk + blockDim.x - 1) / blockDim.x;
  int lo = threadIdx.x * per, hi = min(nblk, lo + per);
  int s = 0;
  for (int i = lo; i < hi; ++i) s += b.scan_blk[i];
  int total;
  int off = block_excl_scan(s, sh, total);
  for (int i = lo; i < hi; ++i) {
    int v = b.scan_blk[i];
    b.scan_blk[i] = off;
    off += v;
  }
}

__global__ void k_scan_down(Bufs b) {
  if (ld_nc_u32(&b.ctl->need_rebuild) == 0u) return;
  __shared__ int sh[32];
  long long base = (long long)blockIdx.x * SCAN_TILE;
  int v[SCAN_V];
  int s = 0;
#pragma unroll
  for (int k = 0; k < SCAN_V; ++k) {
    long long c = base + (long long)threadIdx.x * SCAN_V + k;
    v[k] = c < b.C ? b.cnt[c] : 0;
    s += v[k];
  }
  int total;
  int off = block_excl_scan(s, sh, total) + b.scan_blk[blockIdx.x];
#pragma unroll
  for (int k = 0; k < SCAN_V; ++k) {
    long long c = base + (long long)threadIdx.x * SCAN_V + k;
    if (c < b.C) b.cell_start[c] = off;
    off += v[k];
  }
  if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) b.cell_start[b.C] = (int)b.P;
}

// The whole exclusive scan in one block of 1024 threads for small cell counts
// (C <= kScanSmallC): each thread sums a contiguous run of counts, the block
// scans the run sums, and each thread writes its run's offsets.  Integer sums,
// so the result equals the three-kernel scan's; one launch instead of three,
// which matters when a re-sort costs launch latency rather than bandwidth.
constexpr long long kScanSmallC = 65536;

__global__ void __launch_bounds__(1024) k_scan_small(Bufs b) {
  if (ld_nc_u32(&b.ctl->need_rebuild) == 0u) return;
  __shared__ int sh[32];
  const int C = (int)b.C;
  const int per = (C + (int)blockDim.x - 1) / (int)blockDim.x;
  const int lo = min(C, (int)threadIdx.x * per), hi = min(C, lo + per);
  int s = 0;
  for (int c = lo; c < hi; ++c) s += b.cnt[c];
  int total;
  int off = block_excl_scan(s, sh, total);
  for (int c = lo; c < hi; ++c) {
    const int v = b.cnt[c];
    b.cell_start[c] = off;
    off += v;
  }
  if (threadIdx.x == 0) b.cell_start[C] = (int)b.P;
}

// Slot t to its sorted position: the start of its cell plus its rank there.
__device__ __forceinline__ void scatter_slot(const Bufs& b, long long t) {
  const int key = b.key_tmp[t];
  if (!idx_ok(b.ctl, key, b.C)) return;
  const long long dst = (long long)b.cell_start[key] + b.slot_tmp[t];
  if (idx_ok(b.ctl, dst, b.P)) b.perm_tmp[dst] = (int)t;
}

__global__ void k_scatter(Bufs b) {
  if (ld_nc_u32(&b.ctl->need_rebuild) == 0u) return;
  long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= b.P) return;
  scatter_slot(b, t);
}

// Per cell: order the cell's slots by original index (the stable order of
// lax.sort([hash, iota]), cell_list.py:64) and clear the occupancy counter.
__device__ __forceinline__ void cell_order(const Bufs& b, unsigned int sel, long long c) {
  int a = b.cell_start[c], e = b.cell_start[c + 1];
  b.cnt[c] = 0;
  const int32_t* orig = b.orig[sel];
  if (!idx_ok(b.ctl, a, b.P + 1) || !idx_ok(b.ctl, e, b.P + 1)) return;
  for (int i = a; i < e; ++i)
    if (!idx_ok(b.ctl, b.perm_tmp[i], b.P)) return;
  for (int i = a + 1; i < e; ++i) {
    int x = b.perm_tmp[i];
    int ox = orig[x];
    int j = i - 1;
    while (j >= a && orig[b.perm_tmp[j]] > ox) {
      b.perm_tmp[j + 1] = b.perm_tmp[j];
      --j;
    }
    b.perm_tmp[j + 1] = x;
  }
}

__global__ void k_cellsort(Bufs b) {
  if (ld_nc_u32(&b.ctl->need_rebuild) == 0u) return;
  long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (c >= b.C) return;
  cell_order(b, ld_nc_u32(&b.ctl->sel), c);
}

// Small handles (at most kScanSmallC cells and kSortSmallP slots): the cell
// scan, the scatter and the per-cell ordering of a re-sort as three phases of
// one block of 1024 threads, two launches fewer per re-sort.  Each phase is
// k_scan_small's, k_scatter's and k_cellsort's, so the sorted order is the
// same; the block barriers between them make each phase's global writes
// visible to the next.
constexpr long long kSortSmallP = 32768;

__global__ void __launch_bounds__(1024) k_sort_small(Bufs b) {
  if (ld_nc_u32(&b.ctl->need_rebuild) == 0u) return;
  __shared__ int sh[32];
  const int C = (int)b.C;
  const int per = (C + (int)blockDim.x - 1) / (int)blockDim.x;
  const int lo = min(C, (int)threadIdx.x * per), hi = min(C, lo + per);
  int s = 0;
  for (int c = lo; c < hi; ++c) s += b.cnt[c];
  int total;
  int off = block_excl_scan(s, sh, total);
  for (int c = lo; c < hi; ++c) {
    const int v = b.cnt[c];
    b.cell_start[c] = off;
    off += v;
  }
  if (threadIdx.x == 0) b.cell_start[C] = (int)b.P;
  __syncthreads();
  for (long long t = threadIdx.x; t < b.P; t += blockDim.x) scatter_slot(b, t);
  __syncthreads();
  const unsigned int sel = ld_nc_u32(&b.ctl->sel);
  for (long long c = threadIdx.x; c < C; c += blockDim.x) cell_order(b, sel, c);
}

// After the gather: the sorted copies become current and the list is due.
__device__ __forceinline__ void sort_fin(Ctl* ctl) {
  ctl->sel ^= 1u;
  ctl->pos_sel ^= 1u;
  ctl->need_rebuild = 0u;
  ctl->nl_dirty = 1u;
  ctl->bound = 0.0f;
  ctl->rebuilds += 1u;
}

__global__ void k_sort_fin(Ctl* ctl) {
  if (ctl->need_rebuild == 0u) return;
  sort_fin(ctl);
}

// Gather every slot array into the spare copy in sorted order (k_sort_fin
// then flips the copies).
// FLIP (small handles, a few blocks): the last block to finish flips the
// copies itself, one launch fewer per re-sort.
template <bool FLIP>
__global__ void k_gather(Bufs b) {
  if (ld_nc_u32(&b.ctl->need_rebuild) == 0u) return;
  long long u = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  unsigned int sel = ld_nc_u32(&b.ctl->sel), ps = ld_nc_u32(&b.ctl->pos_sel);
  if (u < b.P) {
    int t = __ldcs(&b.perm_tmp[u]);  // old-order records are read once: streaming loads
    if (!idx_ok(b.ctl, t, b.P)) t = (int)u;
    const float4 p = __ldcs(&b.pos[ps][t]);
    b.pos[ps ^ 1u][u] = p;
    if (b.posw) {
      // positions wrapped into the primary box and the image they came from,
      // for the list build only
      const SysParams& sp = b.sys[b.tag[sel][t] & TAG_SYS_MASK];
      float4 w = p;
      int32_t im = 0;
      if (sp.domain == DOM_PERIODIC) {
        const float kx = floorf((p.x - sp.anchor[0]) / sp.box[0]);
        const float ky = floorf((p.y - sp.anchor[1]) / sp.box[1]);
        const float kz = floorf((p.z - sp.anchor[2]) / sp.box[2]);
        w.x = p.x - sp.box[0] * kx;
        w.y = p.y - sp.box[1] * ky;
        w.z = p.z - sp.box[2] * kz;
        if (fabsf(kx) < 500.0f && fabsf(ky) < 500.0f && fabsf(kz) < 500.0f) {
          im = ((int)kx + 512) | (((int)ky + 512) << 10) | (((int)kz + 512) << 20);
        } else {
          im = (1 << 30) | (int)(u & 0x3FFFFFFF);  // far image: unique, never equal to another's
        }
      }
      b.posw[u] = w;
      if (b.img) b.img[u] = im;
    }
    b.vel[sel ^ 1u][u] = __ldcs(&b.vel[sel][t]);
    // forces are not moved: every re-sort is followed by a force kernel that
    // rewrites frc for all slots before anything reads it
    b.tag[sel ^ 1u][u] = b.tag[sel][t];
    b.orig[sel ^ 1u][u] = __ldcs(&b.orig[sel][t]);
    b.key[sel ^ 1u][u] = __ldcs(&b.key_tmp[t]);
  }
  if (FLIP) {
    __syncthreads();
    if (threadIdx.x == 0) {
      __threadfence();
      if (atomicAdd(&b.ctl->gather_done, 1u) == gridDim.x - 1u) {
        __threadfence();
        b.ctl->gather_done = 0u;
        sort_fin(b.ctl);
      }
    }
  }
}


// ------------------------------------------------------------ first drift

// Step 1 of a call: domain.apply (reflect), step_before_force (VV), drift.
template <int DIM>
__global__ void k_pre(Bufs b, int mode) {
  long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  unsigned int sel = ld_nc_u32(&b.ctl->sel), ps = ld_nc_u32(&b.ctl->pos_sel);
  float d2 = 0.0f;
  if (t < b.P) {
    float4 p4 = b.pos[ps][t];
    float4 v4 = b.vel[sel][t];
    float4 f4 = b.frc[sel][t];
    uint32_t tg = b.tag[sel][t];
    const SysParams& sp = b.sys[tg & TAG_SYS_MASK];
    bool fixed = (tg & TAG_FIXED) != 0u;
    float p[3] = {p4.x, p4.y, p4.z}, v[3] = {v4.x, v4.y, v4.z}, F[3] = {f4.x, f4.y, f4.z};
    float p0[3] = {p[0], p[1], p[2]};
    float m = v4.w;
    if ((mode & MODE_BBOX) && sp.domain == DOM_FREE) {
      int s = tg & TAG_SYS_MASK;
#pragma unroll
      for (int a = 0; a < DIM; ++a) {
        atomicMin((unsigned int*)&b.bbox[s * 6 + a], f2ord(p[a] - p4.w));
        atomicMax((unsigned int*)&b.bbox[s * 6 + 3 + a], f2ord(p[a] + p4.w));
      }
    }
    if (sp.domain == DOM_REFLECT) reflect_sphere<DIM>(sp, p, v, F, p4.w, m, fixed);
    if (sp.lin == LIN_VERLET) {
      float sc = sp.dt * 0.5f / m;
      float fr = fixed ? 0.0f : 1.0f;
#pragma unroll
      for (int a = 0; a < DIM; ++a) {
        v[a] = v[a] + F[a] * sc * fr;
        p[a] = p[a] + sp.dt * v[a];
      }
    }
#pragma unroll
    for (int a = 0; a < DIM; ++a) {
      float d = p[a] - p0[a];
      d2 = d2 + d * d;
    }
    b.pos[ps][t] = make_float4(p[0], p[1], p[2], p4.w);
    b.vel[sel][t] = make_float4(v[0], v[1], v[2], m);
    if (!(d2 == d2) || d2 > 3.0e38f) {
      atomicOr(&b.ctl->status, ST_NONFINITE);
      d2 = 0.0f;
    }
  }
  warp_disp(b.ctl, d2);
}

// ---------------------------------------------------------- fused step

// Verlet list of every slot, built right after a re-sort: all j with
// |r_ij| < r_i + r_j + skin.  While the displacement bound stays below
// skin / 2 every contact of the following steps is in the list.  One thread
// per slot walks its stencil ranges four candidates at a time (independent
// loads); entries go to the sliced layout nbr[((t / 32) * cap + k) * 32 +
// t % 32], so a warp writes, and the force kernel reads, one coalesced row
// per k.  Entries are in ascending slot order within each stencil row.
template <int DIM>
__global__ void __launch_bounds__(256) k_nlbuild(Bufs b) {
  if (ld_nc_u32(&b.ctl->nl_dirty) == 0u) return;
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= b.P) return;
  const unsigned int sel = ld_nc_u32(&b.ctl->sel);
  const SysParams& sp = b.sys[b.tag[sel][t] & TAG_SYS_MASK];
  const bool per = sp.domain == DOM_PERIODIC;
  // Wrapped positions with one image shift per stencil row (every grid axis
  // >= 3 cells makes that shift unique); otherwise the minimum image.  The
  // test only selects list members, so it may round differently from the
  // force: the cutoff is widened by 1e-4 relative to stay a superset.
  const bool shifted = per && b.posw && sp.g[0] >= 3 && sp.g[1] >= 3 && (DIM == 2 || sp.g[2] >= 3);
  const float4* __restrict__ P = shifted ? b.posw : b.pos[ld_nc_u32(&b.ctl->pos_sel)];
  const float4 pi = P[t];
  const float skin = b.nl_skin;
  const int cap = b.nl_cap;
  int32_t* __restrict__ out = b.nbr + ((t >> 5) * cap) * 32 + (t & 31);
  // every periodic entry keeps the minimum image in the force kernel
  const uint32_t mark = per ? kEntryImage : 0u;
  int n = 0;
  auto range = [&](int ja, int jb, float sx, float sy, float sz) {
    if (!idx_ok(b.ctl, ja, b.P + 1) || !idx_ok(b.ctl, jb, b.P + 1)) return;
    for (int j = ja; j < jb; j += 4) {
      float4 q[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) q[u] = j + u < jb ? P[j + u] : pi;
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int jj = j + u;
        if (jj < jb && jj != (int)t) {
          float dsq;
          if (shifted) {
            float dx = (pi.x - q[u].x) + sx, dy = (pi.y - q[u].y) + sy;
            dsq = __fmaf_rn(dy, dy, dx * dx);
            if (DIM == 3) {
              float dz = (pi.z - q[u].z) + sz;
              dsq = __fmaf_rn(dz, dz, dsq);
            }
          } else {
            float dx, dy, dz;
            dsq = pair_disp<DIM>(sp, per, pi, q[u], dx, dy, dz);
          }
          float rc = (pi.w + q[u].w + skin) * 1.0001f;
          if (dsq < rc * rc) {
            if (n < cap) out[n * 32] = (int32_t)((uint32_t)jj | mark);
            ++n;
          }
        }
      }
    }
  };
  {
    const int32_t* __restrict__ cs = b.cell_start;
    const long long local = b.key[sel][t] - sp.c0;
    const int gx = sp.g[0], gy = sp.g[1], gz = sp.g[2];
    int cx = (int)(local % gx);
    long long rem = local / gx;
    int cy = (int)(rem % gy);
    int cz = DIM == 3 ? (int)(rem / gy) : 0;
    int ys[3], zs[3];
    int ny = axis_set(cy, gy, per, ys);
    int nz = DIM == 3 ? axis_set(cz, gz, per, zs) : 1;
    if (DIM == 2) zs[0] = 0;
    if (!idx_ok(b.ctl, local, (long long)gx * gy * (DIM == 3 ? gz : 1))) nz = 0;
    int xa0, xb0, xa1, xb1;
    x_ranges(cx, gx, per, xa0, xb0, xa1, xb1);
    // image shifts (only used when `shifted`)
    const float sxw = cx == 0 ? sp.box[0] : -sp.box[0];
    for (int iz = 0; iz < nz; ++iz) {
      const float sz = (DIM == 3 && shifted) ? (zs[iz] == gz - 1 && cz == 0 ? sp.box[2] : (zs[iz] == 0 && cz == gz - 1 ? -sp.box[2] : 0.0f)) : 0.0f;
      for (int iy = 0; iy < ny; ++iy) {
        const float sy = shifted ? (ys[iy] == gy - 1 && cy == 0 ? sp.box[1] : (ys[iy] == 0 && cy == gy - 1 ? -sp.box[1] : 0.0f)) : 0.0f;
        long long row = sp.c0 + ((long long)zs[iz] * gy + ys[iy]) * gx;
        range(cs[row + xa0], cs[row + xb0], 0.0f, sy, sz);
        if (xa1 < xb1) range(cs[row + xa1], cs[row + xb1], shifted ? sxw : 0.0f, sy, sz);
      }
    }
  }
  if (n > cap) {
    atomicOr(&b.ctl->status, ST_NL_OVERFLOW);
    n = cap;
  }
  b.ncnt[t] = n;
}

// Sets the condition of the re-sort body of a captured step.
__global__ void k_cond(const Ctl* ctl, cudaGraphConditionalHandle h) {
  unsigned int v = __ldcg(&ctl->need_rebuild) | __ldcg(&ctl->nl_dirty);
  cudaGraphSetConditional(h, v ? 1u : 0u);
}

// -------------------------------------------------------------- rotation

// Rotational degrees of freedom of smooth spheres, n steps in registers.
// Spring contacts exert no torque and gravity acts at the centre, so after
// the first step's before-force update torque is 0; the reflect domain only
// renormalises q (reflect.py:291-294 with a zero rotation vector).
// VelocityVerletSpiral: velocity_verlet_spiral.py:83-116, 156-180.
// Spiral: spiral.py (step_after_force).  omega_dot: spiral.py:22-40.
template <int DIM>
__global__ void k_rot(Bufs b, const int32_t* __restrict__ sys_of, float4* __restrict__ q,
                      float* __restrict__ angv, float* __restrict__ torque,
                      const float* __restrict__ inertia, const uint8_t* __restrict__ fixed,
                      long long nsteps) {
  constexpr int AD = DIM == 3 ? 3 : 1;
  long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= b.P) return;
  const SysParams& sp = b.sys[sys_of[i]];
  const int rot = sp.rot, domain = sp.domain;
  const float dt = sp.dt;
  float4 qq = q[i];
  float w[3] = {0, 0, 0}, tq[3] = {0, 0, 0}, I[3] = {1, 1, 1}, invI[3] = {1, 1, 1};
  for (int a = 0; a < AD; ++a) {
    w[a] = angv[i * AD + a];
    tq[a] = torque[i * AD + a];
    I[a] = inertia[i * AD + a];
    invI[a] = 1.0f / I[a];
  }
  float fr = fixed[i] ? 0.0f : 1.0f;
  for (long long s = 0; s < nsteps; ++s) {
    if (domain == DOM_REFLECT) qq = reflect_q(qq);
    rot_before<DIM>(rot, dt, qq, w, tq, I, invI, fr);
    // compute_force + ForceManager: torque = 0 + cross(0, F) + 0
    for (int a = 0; a < AD; ++a) tq[a] = 0.0f;
    rot_after<DIM>(rot, dt, qq, w, nullptr, I, invI, fr);
  }
  q[i] = qq;
  for (int a = 0; a < AD; ++a) {
    angv[i * AD + a] = w[a];
    torque[i * AD + a] = tq[a];
  }
}

// ----------------------------------------------------------- diagnostics

// Per-particle energies in caller order: 0.5 * sum_j of the pair energy
// (spring 0.5 k delta^2, spring.py:110-147; Hertz 0.4 k delta^(5/2),
// hertz.py:119-160; the 0.5 of _partition.py:39-51), gravity -m g.x
// (force_manager.py:450-459) and translational kinetic energy
// (thermal.py:24-47), as doubles; the host sums them in index order.
template <int DIM>
__global__ void k_energy(Bufs b, double* __restrict__ out) {
  long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= b.P) return;
  unsigned int sel = ld_nc_u32(&b.ctl->sel), ps = ld_nc_u32(&b.ctl->pos_sel);
  double e_pair = 0.0, e_grav = 0.0, e_kin = 0.0;
  const float4* __restrict__ P = b.pos[ps];
  float4 pi = P[t];
  uint32_t tg = b.tag[sel][t];
  const SysParams& sp = b.sys[tg & TAG_SYS_MASK];
  const bool per = sp.domain == DOM_PERIODIC;
  const int gx = sp.g[0], gy = sp.g[1];
  long long local = b.key[sel][t] - sp.c0;
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
  const int mat_i = (tg >> TAG_MAT_SHIFT) & TAG_MAT_MASK;
  const int oi = b.orig[sel][t];
  if (!idx_ok(b.ctl, oi, b.P)) return;
  if (!idx_ok(b.ctl, local, (long long)gx * gy * (DIM == 3 ? sp.g[2] : 1))) nz = 0;
  for (int iz = 0; iz < nz; ++iz)
    for (int iy = 0; iy < ny; ++iy) {
      long long row = sp.c0 + ((long long)zs[iz] * gy + ys[iy]) * gx;
      for (int r = 0; r < 2; ++r) {
        int ca = r == 0 ? xa0 : xa1, cb = r == 0 ? xb0 : xb1;
        if (ca >= cb) continue;
        for (int j = b.cell_start[row + ca]; j < b.cell_start[row + cb]; ++j) {
          if (j == (int)t) continue;
          float4 pj = P[j];
          float d[3] = {pi.x - pj.x, pi.y - pj.y, pi.z - pj.z};
          if (per)
            for (int a = 0; a < DIM; ++a) d[a] = d[a] - sp.box[a] * rintf(d[a] * sp.inv_box[a]);
          float dsq = d[0] * d[0] + d[1] * d[1];
          if (DIM == 3) dsq = dsq + d[2] * d[2];
          float R = pi.w + pj.w;
          if (!(dsq < R * R * 1.000001f)) continue;
          if (b.bond_w > 0 && !b.interact_same_bond) {
            int oj = b.orig[sel][j];
            bool bonded = false;
            for (int w = 0; w < b.bond_w; ++w) bonded |= (b.bond[(long long)oi * b.bond_w + w] == oj);
            if (bonded) continue;
          }
          if (b.sclump && b.sclump[oi] == b.sclump[b.orig[sel][j]]) continue;
          int mat_j = (b.tag[sel][j] >> TAG_MAT_SHIFT) & TAG_MAT_MASK;
          float k = b.young[mat_i * b.n_mat + mat_j];
          float e;
          if (b.law == LAW_CS) {
            // CundallStrackForce.energy (cundall_strack.py:197-236): 0.5 kn delta^2,
            // kn = 2 Ei Ri Ej Rj / (Ei Ri + Ej Rj), r = norm(r_ij)
            const float Ei = b.mprop[mat_i * 4], Ej = b.mprop[mat_j * 4];
            const float kn = (2.0f * Ei * pi.w * Ej * pj.w) / (Ei * pi.w + Ej * pj.w);
            float r = dsq == 0.0f ? 0.0f : sqrtf(fmaxf(dsq, 1e-16f));
            float s = R - r;
            s = s > 0.0f ? s : 0.0f;
            e = 0.5f * kn * (s * s);
          } else if (b.law == LAW_HERTZ) {
            // HertzianForce.energy (hertz.py:149-160): r = norm(r_ij),
            // E = 0.4 k delta^(5/2), k = (4/3) E* sqrt(R*)
            float r = dsq == 0.0f ? 0.0f : sqrtf(fmaxf(dsq, 1e-16f));
            float s = R - r;
            s = s > 0.0f ? s : 0.0f;
            float kk = k * sqrtf((pi.w * pj.w) / (pi.w + pj.w));
            e = 0.4f * kk * ((s * s) * sqrtf(s));
          } else {
            float inv = dsq == 0.0f ? 0.0f : 1.0f / sqrtf(fmaxf(dsq, 1e-16f));
            float rr = dsq * inv;
            float s = R - rr;
            s = s > 0.0f ? s : 0.0f;
            e = 0.5f * k * (s * s);
          }
          e_pair += (double)(0.5f * e);
        }
      }
    }
  float4 v4 = b.vel[sel][t];
  float p[3] = {pi.x, pi.y, pi.z}, v[3] = {v4.x, v4.y, v4.z};
  for (int a = 0; a < DIM; ++a) {
    e_grav -= (double)sp.gravity[a] * (double)p[a] * (double)v4.w;
    e_kin += 0.5 * (double)v4.w * (double)v[a] * (double)v[a];
  }
  out[(long long)oi * 3 + 0] = e_pair;
  out[(long long)oi * 3 + 1] = e_grav;
  out[(long long)oi * 3 + 2] = e_kin;
}

// Rotational kinetic energy 0.5 w_b . (I w_b), w_b in the body frame
// (thermal.py:50-80), caller order.
template <int DIM>
__global__ void k_ke_rot(long long N, const float4* __restrict__ q, const float* __restrict__ angv,
                         const float* __restrict__ inertia, double* __restrict__ out) {
  constexpr int AD = DIM == 3 ? 3 : 1;
  long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= N) return;
  float w[3] = {0, 0, 0}, wb[3] = {0, 0, 0};
  for (int a = 0; a < AD; ++a) w[a] = angv[i * AD + a];
  if (DIM == 3) q_rotate3(q[i], -1.0f, w, wb);
  else wb[0] = w[0];
  double e = 0.0;
  for (int a = 0; a < AD; ++a) e += (double)wb[a] * (double)inertia[i * AD + a] * (double)wb[a];
  out[i] = 0.5 * e;
}

// Canonical contacts: pairs with orig_i < orig_j and dsq < (ri + rj)^2 (of
// different clumps), evaluated with the same IEEE operations as the oracle.  Pass 0 counts per
// slot, pass 1 writes (orig_i, orig_j) at the scanned offsets.
template <int DIM>
__global__ void k_contacts(Bufs b, int pass, int32_t* __restrict__ counts,
                           const long long* __restrict__ offs, int32_t* __restrict__ pairs,
                           long long cap) {
  long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= b.P) return;
  unsigned int sel = ld_nc_u32(&b.ctl->sel), ps = ld_nc_u32(&b.ctl->pos_sel);
  const float4* __restrict__ P = b.pos[ps];
  float4 pi = P[t];
  uint32_t tg = b.tag[sel][t];
  const SysParams& sp = b.sys[tg & TAG_SYS_MASK];
  const bool per = sp.domain == DOM_PERIODIC;
  const int gx = sp.g[0], gy = sp.g[1];
  long long local = b.key[sel][t] - sp.c0;
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
  int oi = b.orig[sel][t];
  long long o = pass == 1 ? offs[t] : 0;
  int c = 0;
  if (!idx_ok(b.ctl, local, (long long)gx * gy * (DIM == 3 ? sp.g[2] : 1))) nz = 0;
  for (int iz = 0; iz < nz; ++iz)
    for (int iy = 0; iy < ny; ++iy) {
      long long row = sp.c0 + ((long long)zs[iz] * gy + ys[iy]) * gx;
      for (int r = 0; r < 2; ++r) {
        int ca = r == 0 ? xa0 : xa1, cb = r == 0 ? xb0 : xb1;
        if (ca >= cb) continue;
        for (int j = b.cell_start[row + ca]; j < b.cell_start[row + cb]; ++j) {
          int oj = b.orig[sel][j];
          if (oj <= oi) continue;
          // spheres of one rigid clump never interact
          if (b.sclump && b.sclump[oi] == b.sclump[oj]) continue;
          float4 pj = P[j];
          float d[3] = {pi.x - pj.x, pi.y - pj.y, pi.z - pj.z};
          if (per)
            for (int a = 0; a < DIM; ++a) d[a] = d[a] - sp.box[a] * rintf(d[a] * sp.inv_box[a]);
          float dsq = d[0] * d[0] + d[1] * d[1];
          if (DIM == 3) dsq = dsq + d[2] * d[2];
          float R = pi.w + pj.w;
          if (dsq < R * R) {
            if (pass == 1 && o + c < cap) {
              pairs[2 * (o + c)] = oi;
              pairs[2 * (o + c) + 1] = oj;
            }
            ++c;
          }
        }
      }
    }
  if (pass == 0) counts[t] = c;
}

// ------------------------------------------------------------- launchers

static inline unsigned int nblk(long long n, int t) { return (unsigned int)((n + t - 1) / t); }

void launch_pack(int dim, const Bufs& b, const float* pos, const float* vel, const float* frc,
                 const float* rad, const float* mass, const int32_t* mat, const uint8_t* fixed,
                 const int32_t* sys_of, cudaStream_t st) {
  if (b.P == 0) return;
  if (dim == 3) k_pack<3><<<nblk(b.P, 256), 256, 0, st>>>(b, pos, vel, frc, rad, mass, mat, fixed, sys_of);
  else k_pack<2><<<nblk(b.P, 256), 256, 0, st>>>(b, pos, vel, frc, rad, mass, mat, fixed, sys_of);
}

// Per-system summary of uploaded particle arrays for grid planning, so the
// host reads a few words per system instead of scanning every particle:
// out[8 s] = max radius, out[8 s + 1..3] = min (x - r), out[8 s + 4..6] =
// max (x + r) (order-preserving uints), out[8 s + 7] = flags (1: radius not
// finite or negative, 2: non-finite position, 4: material id out of range).
// A warp whose particles share one system reduces with shuffles first.
template <int DIM>
__global__ void __launch_bounds__(256) k_scan_input(long long N, const float* __restrict__ pos,
                                                    const float* __restrict__ rad, const int32_t* __restrict__ mat,
                                                    int n_mat, const int32_t* __restrict__ sys_of,
                                                    unsigned int* __restrict__ out) {
  __shared__ int w_sys[8];
  __shared__ float w_val[8][7];
  __shared__ unsigned int w_flag[8];
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const bool valid = i < N;
  const int s = valid ? sys_of[i] : -1;
  float r = 0.0f, lo[3] = {3.4e38f, 3.4e38f, 3.4e38f}, hi[3] = {-3.4e38f, -3.4e38f, -3.4e38f};
  unsigned int flags = 0u;
  if (valid) {
    r = rad[i];
    if (!(r >= 0.0f) || !isfinite(r)) flags |= 1u;
#pragma unroll
    for (int a = 0; a < DIM; ++a) {
      const float x = pos[i * DIM + a];
      if (!isfinite(x)) flags |= 2u;
      lo[a] = x - r;
      hi[a] = x + r;
    }
    if (mat && (mat[i] < 0 || mat[i] >= n_mat)) flags |= 4u;
    if (!(r >= 0.0f)) r = 0.0f;
  }
  // one system per warp: shuffle reduction, then one record per warp in
  // shared memory; mixed warps (a system boundary) use per-lane atomics
  const int s0 = __shfl_sync(0xffffffffu, s, 0);
  const bool uniform = __all_sync(0xffffffffu, s == s0 || s < 0) && s0 >= 0;
  if (uniform) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      r = fmaxf(r, __shfl_xor_sync(0xffffffffu, r, o));
      flags |= __shfl_xor_sync(0xffffffffu, flags, o);
#pragma unroll
      for (int a = 0; a < DIM; ++a) {
        lo[a] = fminf(lo[a], __shfl_xor_sync(0xffffffffu, lo[a], o));
        hi[a] = fmaxf(hi[a], __shfl_xor_sync(0xffffffffu, hi[a], o));
      }
    }
  } else if (valid) {
    unsigned int* o8 = out + 8 * (long long)s;
    atomicMax(&o8[0], f2ord(r));
#pragma unroll
    for (int a = 0; a < DIM; ++a) {
      atomicMin(&o8[1 + a], f2ord(lo[a]));
      atomicMax(&o8[4 + a], f2ord(hi[a]));
    }
    if (flags) atomicOr(&o8[7], flags);
  }
  if (lane == 0) {
    w_sys[wid] = uniform ? s0 : -1;
    w_val[wid][0] = r;
    for (int a = 0; a < 3; ++a) {
      w_val[wid][1 + a] = lo[a];
      w_val[wid][4 + a] = hi[a];
    }
    w_flag[wid] = flags;
  }
  __syncthreads();
  if (threadIdx.x != 0) return;
  // merge consecutive warps of one system; one set of atomics per run
  const int nw = blockDim.x >> 5;
  for (int w = 0; w < nw;) {
    const int sw = w_sys[w];
    if (sw < 0) {
      ++w;
      continue;
    }
    float v[7];
    for (int k = 0; k < 7; ++k) v[k] = w_val[w][k];
    unsigned int f = w_flag[w];
    int e = w + 1;
    for (; e < nw && w_sys[e] == sw; ++e) {
      v[0] = fmaxf(v[0], w_val[e][0]);
      for (int a = 0; a < 3; ++a) {
        v[1 + a] = fminf(v[1 + a], w_val[e][1 + a]);
        v[4 + a] = fmaxf(v[4 + a], w_val[e][4 + a]);
      }
      f |= w_flag[e];
    }
    unsigned int* o8 = out + 8 * (long long)sw;
    atomicMax(&o8[0], f2ord(v[0]));
    for (int a = 0; a < DIM; ++a) {
      atomicMin(&o8[1 + a], f2ord(v[1 + a]));
      atomicMax(&o8[4 + a], f2ord(v[4 + a]));
    }
    if (f) atomicOr(&o8[7], f);
    w = e;
  }
}

// State.create's default moment of inertia, 0.4 m r^2 (3D) / 0.5 m r^2 (2D)
// (state.py:817-823), per particle in caller order.
__global__ void k_default_inertia(long long N, int ad, float coeff, const float* __restrict__ mass,
                                  const float* __restrict__ rad, float* __restrict__ inertia) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= N) return;
  const float v = coeff * mass[i] * rad[i] * rad[i];
  for (int a = 0; a < ad; ++a) inertia[i * ad + a] = v;
}

void launch_scan_input(int dim, long long N, const float* pos, const float* rad, const int32_t* mat, int n_mat,
                       const int32_t* sys_of, unsigned int* out, cudaStream_t st) {
  if (N <= 0) return;
  if (dim == 3) k_scan_input<3><<<nblk(N, 256), 256, 0, st>>>(N, pos, rad, mat, n_mat, sys_of, out);
  else k_scan_input<2><<<nblk(N, 256), 256, 0, st>>>(N, pos, rad, mat, n_mat, sys_of, out);
}

void launch_default_inertia(int dim, long long N, const float* mass, const float* rad, float* inertia,
                            cudaStream_t st) {
  if (N <= 0) return;
  k_default_inertia<<<nblk(N, 256), 256, 0, st>>>(N, dim == 3 ? 3 : 1, dim == 2 ? 0.5f : 0.4f, mass, rad, inertia);
}

__global__ void k_identity_q(float4* q, long long n) {
  long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < n) q[i] = make_float4(1.0f, 0.0f, 0.0f, 0.0f);
}

void launch_identity_q(float4* q, long long n, cudaStream_t st) {
  if (n > 0) k_identity_q<<<nblk(n, 256), 256, 0, st>>>(q, n);
}

// Copy particle segments [src, src + n) -> [dst, dst + n) of `width` floats per
// particle for several arrays at once (serving: repack resident requests).
// seg[3k] = source particle offset, seg[3k + 1] = destination offset, seg[3k + 2] = count.
__global__ void k_segcopy(const long long* __restrict__ seg, int nseg, int narr, const float* const* __restrict__ src,
                          float* const* __restrict__ dst, const int* __restrict__ width) {
  int k = blockIdx.y;
  if (k >= nseg) return;
  long long so = seg[3 * k], dof = seg[3 * k + 1], n = seg[3 * k + 2];
  for (int a = 0; a < narr; ++a) {
    int w = width[a];
    long long tot = n * w;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < tot; i += (long long)gridDim.x * blockDim.x)
      dst[a][dof * w + i] = src[a][so * w + i];
  }
}

void launch_segcopy(const long long* seg, int nseg, int narr, const float* const* src, float* const* dst,
                    const int* width, cudaStream_t st) {
  if (nseg <= 0) return;
  dim3 g(64, (unsigned int)nseg);
  k_segcopy<<<g, 256, 0, st>>>(seg, nseg, narr, src, dst, width);
}

void launch_unpack(int dim, const Bufs& b, float* pos, float* vel, float* frc, cudaStream_t st) {
  if (b.P == 0) return;
  if (dim == 3) k_unpack<3><<<nblk(b.P, 256), 256, 0, st>>>(b, pos, vel, frc);
  else k_unpack<2><<<nblk(b.P, 256), 256, 0, st>>>(b, pos, vel, frc);
}

void launch_bbox_reset(const Bufs& b, cudaStream_t st) {
  if (b.S == 0) return;
  k_bbox_reset<<<(unsigned)((b.S * 6 + 255) / 256), 256, 0, st>>>((unsigned int*)b.bbox, b.S);
}

void launch_scan(const Bufs& b, cudaStream_t st) {
  if (b.C <= kScanSmallC) {
    k_scan_small<<<1, 1024, 0, st>>>(b);
    return;
  }
  unsigned int nb = nblk(b.C, SCAN_TILE);
  k_scan_reduce<<<nb, SCAN_T, 0, st>>>(b);
  k_scan_top<<<1, 1024, 0, st>>>(b, (int)nb);
  k_scan_down<<<nb, SCAN_T, 0, st>>>(b);
}

void launch_rebuild(int dim, const Bufs& b, bool any_free, cudaStream_t st) {
  if (b.P == 0) return;
  if (any_free) {
    if (dim == 3) k_grid_free<3><<<b.S, 256, 0, st>>>(b);
    else k_grid_free<2><<<b.S, 256, 0, st>>>(b);
  }
  if (dim == 3) k_bin<3><<<nblk(b.P, 256), 256, 0, st>>>(b);
  else k_bin<2><<<nblk(b.P, 256), 256, 0, st>>>(b);
  if (b.C <= kScanSmallC && b.P <= kSortSmallP) {
    k_sort_small<<<1, 1024, 0, st>>>(b);
  } else {
    launch_scan(b, st);
    k_scatter<<<nblk(b.P, 256), 256, 0, st>>>(b);
    k_cellsort<<<nblk(b.C, 256), 256, 0, st>>>(b);
  }
  if (b.P <= kSortSmallP) {
    k_gather<true><<<nblk(b.P, 256), 256, 0, st>>>(b);
  } else {
    k_gather<false><<<nblk(b.P, 256), 256, 0, st>>>(b);
    k_sort_fin<<<1, 1, 0, st>>>(b.ctl);
  }
}

void launch_pre(int dim, const Bufs& b, int mode, cudaStream_t st) {
  if (b.P == 0) return;
  if (dim == 3) k_pre<3><<<nblk(b.P, 256), 256, 0, st>>>(b, mode);
  else k_pre<2><<<nblk(b.P, 256), 256, 0, st>>>(b, mode);
  launch_fin(b, false, false, 0, st);
}

void launch_nlbuild(int dim, const Bufs& b, cudaStream_t st) {
  if (b.P == 0 || b.nl_cap <= 0) return;
  if (b.n_tiles > 0) {
    launch_tbuild(dim, b, st);
    return;
  }
  if (dim == 3) k_nlbuild<3><<<nblk(b.P, 256), 256, 0, st>>>(b);
  else k_nlbuild<2><<<nblk(b.P, 256), 256, 0, st>>>(b);
}

void launch_fin(const Bufs& b, bool after_force, bool set_cond, cudaGraphConditionalHandle h, cudaStream_t st) {
  k_fin<<<1, 1, 0, st>>>(b.ctl, (after_force ? FIN_AFTER_FORCE : 0) | (set_cond ? FIN_SET_COND : 0), h);
}

void launch_cond(const Bufs& b, cudaGraphConditionalHandle h, cudaStream_t st) { k_cond<<<1, 1, 0, st>>>(b.ctl, h); }

void launch_force(int dim, const Bufs& b, int mode, cudaStream_t st) {
  if (b.P == 0) return;
  if (b.NC) {
    launch_rb(dim, b, mode, st);
    return;
  }
  if (b.law == LAW_CS) {
    launch_cs(dim, b, mode, st);
    return;
  }
  if (dim == 3) launch_force_dim<3>(b, mode, st);
  else launch_force_dim<2>(b, mode, st);
}

void launch_rot(int dim, const Bufs& b, const int32_t* sys_of, float4* q, float* angv, float* torque,
                const float* inertia, const uint8_t* fixed, long long nsteps, cudaStream_t st) {
  if (b.P == 0 || nsteps == 0) return;
  if (dim == 3) k_rot<3><<<nblk(b.P, 256), 256, 0, st>>>(b, sys_of, q, angv, torque, inertia, fixed, nsteps);
  else k_rot<2><<<nblk(b.P, 256), 256, 0, st>>>(b, sys_of, q, angv, torque, inertia, fixed, nsteps);
}

void launch_ke_rot(int dim, long long N, const float4* q, const float* angv, const float* inertia,
                   double* out, cudaStream_t st) {
  if (N == 0) return;
  if (dim == 3) k_ke_rot<3><<<nblk(N, 256), 256, 0, st>>>(N, q, angv, inertia, out);
  else k_ke_rot<2><<<nblk(N, 256), 256, 0, st>>>(N, q, angv, inertia, out);
}

void launch_energy(int dim, const Bufs& b, double* out, cudaStream_t st) {
  if (b.P == 0) return;
  if (dim == 3) k_energy<3><<<nblk(b.P, 256), 256, 0, st>>>(b, out);
  else k_energy<2><<<nblk(b.P, 256), 256, 0, st>>>(b, out);
}


void launch_contacts(int dim, const Bufs& b, int pass, int32_t* counts, const long long* offs,
                     int32_t* pairs, long long cap, cudaStream_t st) {
  if (b.P == 0) return;
  if (dim == 3) k_contacts<3><<<nblk(b.P, 256), 256, 0, st>>>(b, pass, counts, offs, pairs, cap);
  else k_contacts<2><<<nblk(b.P, 256), 256, 0, st>>>(b, pass, counts, offs, pairs, cap);
}

}  // namespace jdem
