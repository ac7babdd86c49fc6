// Verlet-list build over bricks of cells held in shared memory (k_tbuild).
//
// A tile is a brick of home cells [x0, x1) x [y0, y1) x [z0, z1) of one
// system.  Its stencil region -- the brick grown by one cell on every axis,
// in "virtual" cell coordinates that may step one cell past a periodic face --
// is staged into shared memory: virtual rows (z, then y), and along each row
// the virtual cells in x order.  A virtual row is at most three contiguous
// slot ranges (image cell left of x = 0, cells inside the grid, image cell
// right of x = g - 1), so staging is coalesced and every load independent.
// Staged positions are the positions wrapped into the box at the re-sort plus
// the image shift of their virtual cell, so candidates are tested with plain
// differences; each home particle's list is the staged candidates of its
// 3^DIM virtual stencil cells (three consecutive virtual cells of a row are
// one contiguous range) within r_i + r_j + skin, in stencil order.
//
// The list is written in the slot-sliced layout the force kernel reads
// (nbr[((t / 32) * cap + k) * 32 + t % 32], slot indices).  Bit 31 of an
// entry marks a pair that may need the periodic minimum image: a neighbour in
// a shifted virtual cell, or one whose unwrapped position lies in another
// periodic image than the home particle's.  Unmarked pairs stay within
// r_i + r_j + 2 skin < box / 2 while the list lives, where the reference's
// d - box * round(d / box) equals d, so the force kernel skips that
// arithmetic for them.
//
// Tiles of systems with a periodic axis shorter than three cells (where the
// stencil wraps onto itself and the reference de-duplicates cells), and tiles
// whose stencil region exceeds the shared-memory capacity, build from global
// memory with the minimum image ("direct" tiles), every periodic entry marked.
#include "jdem_device.cuh"
#include "jdem_kernels.h"
#include "jdem_pair.cuh"

namespace jdem {

constexpr int TB = 256;            // threads per tile block
constexpr int kMaxHomeRows = 256;  // (y1 - y0) * (z1 - z0) of a tile

// Exclusive scan over the block (blockDim.x threads, a multiple of 32);
// returns this thread's offset.
__device__ __forceinline__ int tile_scan(int v, int* sh, int& total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sh[wid] = x;
  __syncthreads();
  if (wid == 0) {
    int w = lane < nw ? sh[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < nw) sh[lane] = w;
  }
  __syncthreads();
  const int off = wid > 0 ? sh[wid - 1] : 0;
  total = sh[nw - 1];
  __syncthreads();
  return off + x - v;
}

// Exclusive scan of a[0..n) in place by the block; returns the total.
__device__ __forceinline__ int tile_scan_inplace(int* a, int n, int* sh) {
  const int per = (n + blockDim.x - 1) / blockDim.x;
  const int lo = min(n, (int)threadIdx.x * per), hi = min(n, lo + per);
  int s = 0;
  for (int i = lo; i < hi; ++i) s += a[i];
  int total;
  int off = tile_scan(s, sh, total);
  for (int i = lo; i < hi; ++i) {
    const int v = a[i];
    a[i] = off;
    off += v;
  }
  __syncthreads();
  return total;
}

// Shape of a tile's staged region.
struct Brick {
  int W, H, D;     // home cells per axis
  int VX, VY, VZ;  // virtual cells per axis (home + 1 on each side)
  __device__ __forceinline__ Brick(const TileDesc& td, int dim) {
    W = td.x1 - td.x0;
    H = td.y1 - td.y0;
    D = dim == 3 ? td.z1 - td.z0 : 1;
    VX = W + 2;
    VY = H + 2;
    VZ = dim == 3 ? D + 2 : 1;
  }
};

// Real cell of a virtual cell (each coordinate at most one cell outside the
// grid) and the image shift that places it next to the tile; false when it
// lies outside a non-periodic grid.
template <int DIM>
__device__ __forceinline__ bool virt_cell(const SysParams& sp, bool per, int vx, int vy, int vz, long long& rc,
                                          float* sh) {
  const int v[3] = {vx, vy, vz};
  int r[3] = {0, 0, 0};
  sh[0] = sh[1] = sh[2] = 0.0f;
#pragma unroll
  for (int a = 0; a < DIM; ++a) {
    const int g = sp.g[a];
    if (v[a] < 0) {
      if (!per) return false;
      r[a] = v[a] + g;
      sh[a] = -sp.box[a];
    } else if (v[a] >= g) {
      if (!per) return false;
      r[a] = v[a] - g;
      sh[a] = sp.box[a];
    } else {
      r[a] = v[a];
    }
  }
  rc = sp.c0 + ((long long)r[2] * sp.g[1] + r[1]) * sp.g[0] + r[0];
  return true;
}

// The three contiguous slot ranges of virtual row (vy, vz), in staged order:
// the image cell left of x = 0, the cells inside the grid, the image cell
// right of x = g - 1.  Absent ranges (no wrap, or outside a non-periodic
// grid) have length 0.  plan = {ja0, ja1, ja2, len0, len1, len2}.
template <int DIM>
__device__ __forceinline__ int row_plan(const Bufs& b, const SysParams& sp, bool per, const TileDesc& td, int vy,
                                        int vz, int* plan) {
  const int gx = sp.g[0];
  const int pa[3] = {td.x0 - 1, max(td.x0 - 1, 0), td.x1 == gx ? gx : td.x1 + 1};
  const int pb[3] = {td.x0 == 0 ? td.x0 : td.x0 - 1, min(td.x1 + 1, gx), td.x1 == gx ? gx + 1 : td.x1 + 1};
  int total = 0;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    long long ra, rl;
    float s3[3];
    int ja = 0, len = 0;
    if (pa[k] < pb[k] && virt_cell<DIM>(sp, per, pa[k], vy, vz, ra, s3)) {
      virt_cell<DIM>(sp, per, pb[k] - 1, vy, vz, rl, s3);
      ja = b.cell_start[ra];
      len = b.cell_start[rl + 1] - ja;
    }
    plan[k] = ja;
    plan[3 + k] = len;
    total += len;
  }
  return total;
}

// Image shift of virtual row (vy, vz) and of the x pieces (see row_plan).
template <int DIM>
__device__ __forceinline__ void row_shift(const SysParams& sp, bool per, int vy, int vz, float* sh_yz,
                                          float* sh_x) {
  sh_yz[0] = per ? (vy < 0 ? -sp.box[1] : (vy >= sp.g[1] ? sp.box[1] : 0.0f)) : 0.0f;
  sh_yz[1] = (per && DIM == 3) ? (vz < 0 ? -sp.box[2] : (vz >= sp.g[2] ? sp.box[2] : 0.0f)) : 0.0f;
  sh_x[0] = per ? -sp.box[0] : 0.0f;
  sh_x[1] = 0.0f;
  sh_x[2] = per ? sp.box[0] : 0.0f;
}

// Largest index i in [lo, hi) with a[i] <= v (a non-decreasing, a[lo] <= v).
__device__ __forceinline__ int last_le(const int* a, int lo, int hi, int v) {
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (a[mid] <= v) lo = mid;
    else hi = mid;
  }
  return lo;
}

template <int DIM>
__global__ void __launch_bounds__(TB) k_tbuild(Bufs b) {
  if (ld_nc_u32(&b.ctl->nl_dirty) == 0u) return;
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ int s_hrow[kMaxHomeRows + 1];
  __shared__ int s_scan[32];
  const int NST = b.tb_nst, NVC = b.tb_nv, NR = b.tb_nrows, cap = b.nl_cap;
  float4* spos = (float4*)smem;             // staged wrapped positions + image shift
  int32_t* sslot = (int32_t*)(spos + NST);  // slot of each staged candidate
  int32_t* simg = sslot + NST;              // image code (bit 31: shifted virtual cell)
  int32_t* vstart = simg + NST;             // [NVC + 1] staged range of each virtual cell
  int32_t* splan = vstart + NVC + 1;        // [NR][6] row plans (row_plan)

  const TileDesc td = b.tiles[blockIdx.x];
  const SysParams& sp = b.sys[td.sys];
  const bool per = sp.domain == DOM_PERIODIC;
  const Brick bk(td, DIM);
  const int NV = bk.VX * bk.VY * bk.VZ, HD = bk.H * bk.D, nrows = bk.VY * bk.VZ;
  const float skin = b.nl_skin, eps = sp.nl_eps;
  const int32_t* __restrict__ cs = b.cell_start;
  const unsigned int sel = ld_nc_u32(&b.ctl->sel);
  bool direct = (td.flags & TILE_DIRECT) != 0 || NV > NVC || nrows > NR;
  if (!idx_ok(b.ctl, HD, kMaxHomeRows + 1)) return;  // block-uniform

  if (!direct) {
    // occupancy of every virtual cell -> staged offsets
    for (int v = threadIdx.x; v < NV; v += TB) {
      const int vx = td.x0 - 1 + v % bk.VX, vy = td.y0 - 1 + (v / bk.VX) % bk.VY;
      const int vz = DIM == 3 ? td.z0 - 1 + v / (bk.VX * bk.VY) : 0;
      long long rc;
      float sh[3];
      vstart[v] = virt_cell<DIM>(sp, per, vx, vy, vz, rc, sh) ? cs[rc + 1] - cs[rc] : 0;
    }
    __syncthreads();
    const int total = tile_scan_inplace(vstart, NV, s_scan);
    if (threadIdx.x == 0) vstart[NV] = total;
    direct = total > NST;  // block-uniform
  }

  if (direct) {
    // home particles row by row; candidates from global memory, minimum image
    for (int r = threadIdx.x; r < HD; r += TB) {
      const int y = td.y0 + r % bk.H, z = DIM == 3 ? td.z0 + r / bk.H : 0;
      const long long row = sp.c0 + ((long long)z * sp.g[1] + y) * sp.g[0];
      s_hrow[r] = cs[row + td.x1] - cs[row + td.x0];
    }
    __syncthreads();
    const int cnt = tile_scan_inplace(s_hrow, HD, s_scan);
    const float4* __restrict__ Pc = b.pos[ld_nc_u32(&b.ctl->pos_sel)];
    const uint32_t mark = per ? 0x80000000u : 0u;
    for (int h = threadIdx.x; h < cnt; h += TB) {
      const int r = last_le(s_hrow, 0, HD, h);
      const int y = td.y0 + r % bk.H, z = DIM == 3 ? td.z0 + r / bk.H : 0;
      const long long row = sp.c0 + ((long long)z * sp.g[1] + y) * sp.g[0];
      const long long slot = cs[row + td.x0] + (h - s_hrow[r]);
      if (!idx_ok(b.ctl, slot, b.P)) continue;
      const float4 pi = Pc[slot];
      int32_t* out = b.nbr + ((slot >> 5) * cap) * 32 + (slot & 31);
      int n = 0;
      for_each_candidate<DIM>(cs, sp, b.key[sel][slot] - sp.c0, [&](int j) {
        if (j == (int)slot) return;
        const float4 q = Pc[j];
        float dx, dy, dz;
        const float dsq = pair_disp<DIM>(sp, per, pi, q, dx, dy, dz);
        const float rc = (pi.w + q.w + skin) * 1.0001f + eps;
        if (dsq < rc * rc) {
          if (n < cap) out[n * 32] = (int32_t)((uint32_t)j | mark);
          ++n;
        }
      });
      if (n > cap) atomicOr(&b.ctl->status, ST_NL_OVERFLOW);
      b.ncnt[slot] = min(n, cap);
    }
    return;
  }

  // stage: row plans, then one warp per virtual row
  for (int r = threadIdx.x; r < nrows; r += TB)
    row_plan<DIM>(b, sp, per, td, td.y0 - 1 + r % bk.VY, DIM == 3 ? td.z0 - 1 + r / bk.VY : 0, splan + 6 * r);
  __syncthreads();
  {
    const int lane = threadIdx.x & 31;
    for (int r = threadIdx.x >> 5; r < nrows; r += TB / 32) {
      const int vy = td.y0 - 1 + r % bk.VY, vz = DIM == 3 ? td.z0 - 1 + r / bk.VY : 0;
      float syz[2], sx[3];
      row_shift<DIM>(sp, per, vy, vz, syz, sx);
      const bool row_shifted = syz[0] != 0.0f || syz[1] != 0.0f;
      int o = vstart[r * bk.VX];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const int ja = splan[6 * r + k], len = splan[6 * r + 3 + k];
        const int32_t shifted = (row_shifted || k != 1) ? (int32_t)0x80000000 : 0;
        for (int i = lane; i < len; i += 32) {
          if (!idx_ok(b.ctl, o + i, NST) || !idx_ok(b.ctl, ja + i, b.P)) continue;
          float4 w = b.posw[ja + i];
          w.x = w.x + sx[k];
          w.y = w.y + syz[0];
          if (DIM == 3) w.z = w.z + syz[1];
          w.w = w.w * 1.0001f;  // radius with the list cutoff's relative widening
          spos[o + i] = w;
          sslot[o + i] = ja + i;
          simg[o + i] = b.img[ja + i] | shifted;
        }
        o += len;
      }
    }
  }
  // home rows: staged ranges of the home cells of each (y, z) row
  for (int r = threadIdx.x; r < HD; r += TB) {
    const int iy = r % bk.H + 1, iz = DIM == 3 ? r / bk.H + 1 : 0;
    const int rb = (iz * bk.VY + iy) * bk.VX;
    s_hrow[r] = vstart[rb + bk.W + 1] - vstart[rb + 1];
  }
  __syncthreads();
  const int cnt = tile_scan_inplace(s_hrow, HD, s_scan);

  for (int h = threadIdx.x; h < cnt; h += TB) {
    const int r = last_le(s_hrow, 0, HD, h);
    const int iy = r % bk.H + 1, iz = DIM == 3 ? r / bk.H + 1 : 0;
    const int rb = (iz * bk.VY + iy) * bk.VX;
    const int oh = vstart[rb + 1] + (h - s_hrow[r]);
    const int ix = last_le(vstart, rb + 1, rb + bk.W + 1, oh) - rb;  // virtual x of the home cell
    if (!idx_ok(b.ctl, oh, vstart[NV])) continue;
    const long long slot = sslot[oh];
    const float4 pi = spos[oh];
    // (r_i + r_j + skin) * 1.0001 + eps with the staged radii already widened
    const float base_r = pi.w + skin * 1.0001f + eps;
    // entries of another image (shifted cell or different image counts) keep
    // the minimum image; the home particle is never shifted
    const int32_t img_h = (td.flags & TILE_ALLIMAGE) ? (int32_t)0x7FFFFFFF : simg[oh];
    int32_t* out = b.nbr + ((slot >> 5) * cap) * 32 + (slot & 31);
    int n = 0;
#pragma unroll 1
    for (int dz = (DIM == 3 ? -1 : 0); dz <= (DIM == 3 ? 1 : 0); ++dz) {
#pragma unroll 1
      for (int dy = -1; dy <= 1; ++dy) {
        const int vb = ((iz + dz) * bk.VY + (iy + dy)) * bk.VX + ix - 1;
        if (!idx_ok(b.ctl, vb, NV - 2)) continue;
        const int oa = vstart[vb], ob = vstart[vb + 3];
        auto test = [&](int oj, const float4& q) {
          const float ddx = pi.x - q.x, ddy = pi.y - q.y;
          float dsq = __fmaf_rn(ddy, ddy, ddx * ddx);
          if (DIM == 3) {
            const float ddz = pi.z - q.z;
            dsq = __fmaf_rn(ddz, ddz, dsq);
          }
          const float rc = base_r + q.w;
          if (dsq < rc * rc && oj != oh) {
            if (n < cap) out[n * 32] = (int32_t)((uint32_t)sslot[oj] | (simg[oj] != img_h ? 0x80000000u : 0u));
            ++n;
          }
        };
        int o = oa;
        for (; o + 4 <= ob; o += 4) {
          float4 q[4];
#pragma unroll
          for (int u = 0; u < 4; ++u) q[u] = spos[o + u];
#pragma unroll
          for (int u = 0; u < 4; ++u) test(o + u, q[u]);
        }
        for (; o < ob; ++o) test(o, spos[o]);
      }
    }
    if (n > cap) atomicOr(&b.ctl->status, ST_NL_OVERFLOW);
    b.ncnt[slot] = min(n, cap);
  }
}

size_t tbuild_smem(int nst, int nv, int nrows) {
  return (size_t)nst * (sizeof(float4) + 2 * sizeof(int32_t)) + (size_t)(nv + 1) * sizeof(int32_t) +
         (size_t)nrows * 6 * sizeof(int32_t);
}

// The dynamic shared-memory limit is a property of the kernel, shared by every
// handle in the process, so it is raised once to the largest request any
// handle can make (staged capacity 4096, 2048 virtual cells, 512 virtual rows).
int prepare_tbuild(size_t bytes) {
  static const size_t kMaxB = tbuild_smem(4096, 2048, 512);
  if (bytes > kMaxB) return 1;
  bool ok = cudaFuncSetAttribute(k_tbuild<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxB) == cudaSuccess;
  ok = ok && cudaFuncSetAttribute(k_tbuild<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxB) == cudaSuccess;
  return ok ? 0 : 1;
}

void launch_tbuild(int dim, const Bufs& b, cudaStream_t st) {
  if (b.P == 0 || b.n_tiles <= 0 || b.nl_cap <= 0) return;
  const size_t sm = tbuild_smem(b.tb_nst, b.tb_nv, b.tb_nrows);
  if (dim == 3) k_tbuild<3><<<b.n_tiles, TB, sm, st>>>(b);
  else k_tbuild<2><<<b.n_tiles, TB, sm, st>>>(b);
}

}  // namespace jdem
