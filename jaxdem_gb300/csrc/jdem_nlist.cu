// DynamicCellList.create_neighbor_list (colliders/cell_list.py:498-595) on the
// device, in the reference's visiting order: for each particle, the stencil
// cells of neighbor_mask (meshgrid "ij", last axis fastest), deduplicated
// under periodic wrap (cell_list.py:90-96), each scanned in ascending
// original index (the stable order of lax.sort, cell_list.py:64).  The grid
// is the reference's: cell = max(cell_size, cutoff / search_range)
// (cell_list.py:537-538) through _grid_params (_partition.py:54-99).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "jdem_device.cuh"
#include "jdem_internal.h"
#include "jdem_kernels.h"

using namespace jdem;

namespace {

struct NlGrid {
  float box[3];
  float anchor[3];
  float cell;
  int g[3];
  int domain;
  int sr;
  int dedup;
  long long c0;
};

__device__ __forceinline__ int nl_coord(const NlGrid& G, int a, float x) {
  float v;
  if (G.domain == DOM_PERIODIC) {
    float frac = floor_mod1((x - G.anchor[a]) / G.box[a]);
    v = floorf(frac * (float)G.g[a]);
  } else {
    v = floorf((x - G.anchor[a]) / G.cell);
  }
  return (v != v) ? 0 : (v < 0.0f ? 0 : (v > (float)(G.g[a] - 1) ? G.g[a] - 1 : (int)v));
}

template <int DIM>
__global__ void k_nl_key(long long P, const float* __restrict__ pos, const int32_t* __restrict__ sys_of,
                         const NlGrid* __restrict__ grids, int32_t* __restrict__ key,
                         int32_t* __restrict__ slot, int32_t* __restrict__ cnt) {
  long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= P) return;
  const NlGrid& G = grids[sys_of[i]];
  long long h = 0, stride = 1;
  for (int a = 0; a < DIM; ++a) {
    h += (long long)nl_coord(G, a, pos[i * DIM + a]) * stride;
    stride *= G.g[a];
  }
  int k = (int)(G.c0 + h);
  key[i] = k;
  slot[i] = atomicAdd(&cnt[k], 1);
}

__global__ void k_nl_scatter(long long P, const int32_t* __restrict__ key, const int32_t* __restrict__ slot,
                             const int32_t* __restrict__ start, int32_t* __restrict__ perm) {
  long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= P) return;
  perm[start[key[i]] + slot[i]] = (int)i;
}

__global__ void k_nl_cellsort(long long C, const int32_t* __restrict__ start, int32_t* __restrict__ perm) {
  long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (c >= C) return;
  int a = start[c], e = start[c + 1];
  for (int i = a + 1; i < e; ++i) {
    int x = perm[i];
    int j = i - 1;
    while (j >= a && perm[j] > x) {
      perm[j + 1] = perm[j];
      --j;
    }
    perm[j + 1] = x;
  }
}

template <int DIM>
__device__ __forceinline__ long long nl_stencil_hash(const NlGrid& G, const int* c, int m, int side) {
  int off[3] = {0, 0, 0};
  int rem = m;
  for (int a = DIM - 1; a >= 0; --a) {
    off[a] = rem % side - G.sr;
    rem /= side;
  }
  long long h = 0, stride = 1;
  for (int a = 0; a < DIM; ++a) {
    int x = c[a] + off[a];
    if (G.domain == DOM_PERIODIC) {
      int g = G.g[a];
      x = ((x % g) + g) % g;
    } else if (x < 0 || x >= G.g[a]) {
      return -1;
    }
    h += (long long)x * stride;
    stride *= G.g[a];
  }
  return h;
}

template <int DIM>
__global__ void k_nl_build(long long P, const float* __restrict__ pos, const int32_t* __restrict__ sys_of,
                           const NlGrid* __restrict__ grids, const int32_t* __restrict__ start,
                           const int32_t* __restrict__ perm, const int32_t* __restrict__ bond, int bond_w,
                           int interact_same_bond, const int32_t* __restrict__ body, float cutoff_sq, int max_nb,
                           int32_t* __restrict__ out, unsigned int* __restrict__ overflow) {
  long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= P) return;
  const NlGrid& G = grids[sys_of[i]];
  float pi[3] = {0, 0, 0};
  int c[3] = {0, 0, 0};
  for (int a = 0; a < DIM; ++a) {
    pi[a] = pos[i * DIM + a];
    c[a] = nl_coord(G, a, pi[a]);
  }
  int side = 2 * G.sr + 1;
  int M = side * side;
  if (DIM == 3) M *= side;
  int cnt = 0;
  bool ovf = false;
  for (int m = 0; m < M; ++m) {
    long long h = nl_stencil_hash<DIM>(G, c, m, side);
    if (h < 0) continue;
    if (G.dedup) {
      bool dup = false;
      for (int m2 = 0; m2 < m && !dup; ++m2) dup = nl_stencil_hash<DIM>(G, c, m2, side) == h;
      if (dup) continue;
    }
    long long cell = G.c0 + h;
    int local = 0;
    for (int k = start[cell]; k < start[cell + 1]; ++k) {
      int j = perm[k];
      // same body (valid_interaction_mask): a sphere, or a rigid clump's members
      if (body ? body[j] == body[i] : j == (int)i) continue;
      if (bond_w > 0 && !interact_same_bond) {
        bool bonded = false;
        for (int w = 0; w < bond_w; ++w) bonded |= bond[(long long)j * bond_w + w] == (int)i;
        if (bonded) continue;
      }
      float d2 = 0.0f;
      for (int a = 0; a < DIM; ++a) {
        float d = pi[a] - pos[(long long)j * DIM + a];
        // PeriodicDomain.displacement divides by the box (periodic.py:70-71)
        if (G.domain == DOM_PERIODIC) d = d - G.box[a] * rintf(d / G.box[a]);
        d2 = a == 0 ? d * d : d2 + d * d;
      }
      if (d2 <= cutoff_sq) {
        if (local < max_nb) {
          if (cnt < max_nb) out[i * max_nb + cnt] = j;
        } else {
          ovf = true;
        }
        ++local;
        ++cnt;
      }
    }
  }
  if (cnt > max_nb) ovf = true;
  if (ovf) atomicOr(overflow, 1u);
}

}  // namespace

int JdemHandle::neighbor_list(float cutoff, int max_nb, int32_t* out, int32_t* overflow) {
  if (!uploaded) return fail(JDEM_ERR_NOT_READY, "neighbor_list before upload");
  if (max_nb < 0 || !(cutoff >= 0.0f)) return fail(JDEM_ERR_BAD_ARG, "neighbor_list: bad cutoff or max_neighbors");
  if (overflow) *overflow = 0;
  if (P == 0 || max_nb == 0) return JDEM_OK;
  if (!out) return fail(JDEM_ERR_BAD_ARG, "neighbor_list: null output");
  cudaSetDevice(dev);
  // Reference grid per system.
  std::vector<NlGrid> grids((size_t)S);
  long long c_total = 0;
  bool hash_ovf = false;
  for (int s = 0; s < S; ++s) {
    const JdemSystemDesc& d = desc[s];
    NlGrid& G = grids[(size_t)s];
    std::memset(&G, 0, sizeof(G));
    G.domain = d.domain;
    G.sr = std::max(1, d.search_range);
    for (int a = 0; a < 3; ++a) {
      G.box[a] = a < dim ? cur_box[(size_t)s * 3 + a] : 1.0f;
      G.anchor[a] = a < dim ? cur_anchor[(size_t)s * 3 + a] : 0.0f;
      G.g[a] = 1;
    }
    float cell = std::max(d.cell_size, cutoff / (float)G.sr);
    G.cell = cell;
    long long tot = 1;
    double totf = 1.0;
    for (int a = 0; a < dim; ++a) {
      long long g = d.domain == DOM_PERIODIC ? (long long)std::floor(G.box[a] / cell)
                                             : (long long)std::ceil(G.box[a] / cell);
      if (g < 1) g = 1;
      totf *= (double)g;
      G.g[a] = (int)std::min<long long>(g, 1 << 30);
      tot *= g;
    }
    if (totf > 2147483647.0) hash_ovf = true;  // _partition.py:95-97
    if (totf > 268435456.0)
      return fail(JDEM_ERR_CAPACITY_OVERFLOW, "neighbor_list: reference grid exceeds 2^28 cells");
    int side = 2 * G.sr + 1;
    G.dedup = 0;
    if (d.domain == DOM_PERIODIC)
      for (int a = 0; a < dim; ++a)
        if (G.g[a] < side) G.dedup = 1;
    G.c0 = c_total;
    c_total += tot;
  }
  int rc;
  NlGrid* d_grids = nullptr;
  int32_t *d_key = nullptr, *d_slot = nullptr, *d_cnt = nullptr, *d_start = nullptr, *d_perm = nullptr,
          *d_out = nullptr, *d_blk = nullptr;
  unsigned int* d_ovf = nullptr;
  Ctl* d_ctl = nullptr;
  auto cleanup = [&]() {
    dfree(d_grids); dfree(d_key); dfree(d_slot); dfree(d_cnt); dfree(d_start);
    dfree(d_perm); dfree(d_out); dfree(d_blk); dfree(d_ovf); dfree(d_ctl);
  };
  long long nb = (c_total + 2047) / 2048 + 1;
  if ((rc = dalloc((void**)&d_grids, sizeof(NlGrid) * S)) || (rc = dalloc((void**)&d_key, 4 * (size_t)P)) ||
      (rc = dalloc((void**)&d_slot, 4 * (size_t)P)) || (rc = dalloc((void**)&d_cnt, 4 * (size_t)c_total)) ||
      (rc = dalloc((void**)&d_start, 4 * (size_t)(c_total + 1))) || (rc = dalloc((void**)&d_perm, 4 * (size_t)P)) ||
      (rc = dalloc((void**)&d_out, 4 * (size_t)P * max_nb)) || (rc = dalloc((void**)&d_blk, 4 * (size_t)nb)) ||
      (rc = dalloc((void**)&d_ovf, 4)) || (rc = dalloc((void**)&d_ctl, sizeof(Ctl)))) {
    cleanup();
    return rc;
  }
  // positions in caller order: state.pos, the members' world positions for clumps
  if (b.NC) launch_rb_world(dim, b, st_pos, stream);
  else launch_unpack(dim, b, st_pos, st_vel, st_frc, stream);
  cudaMemcpyAsync(d_grids, grids.data(), sizeof(NlGrid) * S, cudaMemcpyHostToDevice, stream);
  cudaMemsetAsync(d_cnt, 0, 4 * (size_t)c_total, stream);
  cudaMemsetAsync(d_out, 0xFF, 4 * (size_t)P * max_nb, stream);
  cudaMemsetAsync(d_ovf, 0, 4, stream);
  Ctl c;
  std::memset(&c, 0, sizeof(c));
  c.need_rebuild = 1u;
  cudaMemcpyAsync(d_ctl, &c, sizeof(Ctl), cudaMemcpyHostToDevice, stream);
  unsigned int pb = (unsigned int)((P + 255) / 256);
  if (dim == 3) k_nl_key<3><<<pb, 256, 0, stream>>>(P, st_pos, st_sys, d_grids, d_key, d_slot, d_cnt);
  else k_nl_key<2><<<pb, 256, 0, stream>>>(P, st_pos, st_sys, d_grids, d_key, d_slot, d_cnt);
  // scan through the engine's scan kernels on a scratch view
  Bufs v = b;
  v.cnt = d_cnt;
  v.cell_start = d_start;
  v.scan_blk = d_blk;
  v.C = c_total;
  v.ctl = d_ctl;
  launch_scan(v, stream);
  k_nl_scatter<<<pb, 256, 0, stream>>>(P, d_key, d_slot, d_start, d_perm);
  k_nl_cellsort<<<(unsigned int)((c_total + 255) / 256), 256, 0, stream>>>(c_total, d_start, d_perm);
  float cutoff_sq = cutoff * cutoff;
  if (dim == 3)
    k_nl_build<3><<<pb, 256, 0, stream>>>(P, st_pos, st_sys, d_grids, d_start, d_perm, d_bond, bond_w,
                                          interact_same_bond, b.NC ? b.sclump : nullptr, cutoff_sq, max_nb, d_out,
                                          d_ovf);
  else
    k_nl_build<2><<<pb, 256, 0, stream>>>(P, st_pos, st_sys, d_grids, d_start, d_perm, d_bond, bond_w,
                                          interact_same_bond, b.NC ? b.sclump : nullptr, cutoff_sq, max_nb, d_out,
                                          d_ovf);
  cudaError_t e = cudaGetLastError();
  unsigned int h_ovf = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, d_out, 4 * (size_t)P * max_nb, cudaMemcpyDeviceToHost, stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&h_ovf, d_ovf, 4, cudaMemcpyDeviceToHost, stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
  cleanup();
  if (e != cudaSuccess) return fail(JDEM_ERR_CUDA, std::string("neighbor_list: ") + cudaGetErrorString(e));
  if (overflow) *overflow = (h_ovf || hash_ovf) ? 1 : 0;
  return sync_status();
}

int JdemHandle::domain_state(float* box, float* anchor) {
  if (!uploaded) return fail(JDEM_ERR_NOT_READY, "domain_state before upload");
  int rc = sync_status();
  if (rc && rc != JDEM_ERR_NONFINITE) return rc;
  for (size_t k = 0; k < cur_box.size(); ++k) {
    if (box) box[k] = cur_box[k];
    if (anchor) anchor[k] = cur_anchor[k];
  }
  return JDEM_OK;
}
