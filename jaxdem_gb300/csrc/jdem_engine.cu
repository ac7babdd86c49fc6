// Host side of the GB300 DEM step engine: device memory, CUDA-graph chunks
// and the C ABI declared in include/jdem_gb300.h.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <new>
#include <string>
#include <vector>

#include "../../include/jdem_gb300.h"
#include "jdem_device.cuh"
#include "jdem_kernels.h"
#include "jdem_internal.h"

using namespace jdem;

namespace {

// largest Verlet-list row
constexpr int kMaxListCap = 384;

const char* kStatusNames[] = {"ok",          "bad argument", "capacity overflow", "hash overflow",
                              "non-finite state", "out of device memory", "timeout",
                              "unsupported configuration", "CUDA error", "not ready"};

}  // namespace

// ------------------------------------------------------------------ helpers

int JdemHandle::fail(int code, const std::string& msg) {
  err = msg;
  return code;
}

void JdemHandle::free_all() {
  free_frames();
  for (auto& kv : graphs) cudaGraphExecDestroy(kv.second);
  graphs.clear();
  for (void* p : allocs) cudaFree(p);
  allocs.clear();
  alloc_bytes.clear();
  device_bytes = 0;
  if (h_status) cudaFreeHost(h_status);
  h_status = nullptr;
  if (own) cudaStreamDestroy(own);
  if (side) cudaStreamDestroy(side);
  own = nullptr;
  stream = nullptr;
  side = nullptr;
  for (auto& e : ev_pool) cudaEventDestroy(e);
  ev_pool.clear();
}

int JdemHandle::dalloc(void** p, size_t bytes) {
  if (bytes == 0) bytes = 16;
  cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(JDEM_ERR_OOM, std::string("cudaMalloc(") + std::to_string(bytes) + "): " +
                                  cudaGetErrorString(e));
  }
  allocs.push_back(*p);
  alloc_bytes[*p] = bytes;
  device_bytes += (long long)bytes;
  return JDEM_OK;
}

void JdemHandle::dfree(void* p) {
  if (!p) return;
  auto it = std::find(allocs.begin(), allocs.end(), p);
  if (it != allocs.end()) allocs.erase(it);
  auto jt = alloc_bytes.find(p);
  if (jt != alloc_bytes.end()) {
    device_bytes -= (long long)jt->second;
    alloc_bytes.erase(jt);
  }
  cudaFree(p);
}

void JdemHandle::drop_graphs() {
  for (auto& kv : graphs) cudaGraphExecDestroy(kv.second);
  graphs.clear();
  multi_used = false;
}

// Host restatement of the grid choice: binning cell = 2 r_max + skin, grown
// until the system's cell count fits the budget (any cell at least as large
// as the contact range gives the same contact set).
static void choose_grid(SysParams& sp, int dim, float rmax, float skin, long long np,
                        const float* lo_bb, const float* hi_bb) {
  float cell = 2.0f * rmax + skin;
  if (!(cell > 0.0f)) cell = 1.0f;
  long long budget = std::max(4096LL, 4 * np);
  for (int it = 0; it < 200; ++it) {
    long long tot = 1;
    for (int a = 0; a < dim; ++a) {
      long long g;
      if (sp.domain == DOM_PERIODIC) {
        g = (long long)std::floor(sp.box[a] / cell);
        if (g < 1) g = 1;
      } else if (sp.domain == DOM_REFLECT) {
        g = (long long)std::ceil(sp.box[a] / cell);
        if (g < 1) g = 1;
      } else {
        double ext = (double)hi_bb[a] - (double)lo_bb[a];
        g = (long long)std::ceil(ext / cell);
        if (g < 1) g = 1;
        g += 2;  // headroom: the bounding box grows as particles move
      }
      sp.g[a] = (int)std::min<long long>(g, 1 << 30);
      tot *= g;
    }
    if (tot <= budget) break;
    cell *= 1.1f;
  }
  if (dim == 2) sp.g[2] = 1;
  sp.cell_bin = cell;
  for (int a = 0; a < 3; ++a) {
    sp.glo[a] = sp.domain == DOM_FREE ? lo_bb[a] : sp.anchor[a];
    sp.gcell[a] = cell;
  }
  long long ncell = 1;
  for (int a = 0; a < dim; ++a) ncell *= sp.g[a];
  sp.ncap = sp.domain == DOM_FREE ? ncell * 2 : ncell;
}

int JdemHandle::setup(const JdemConfig* cfg) {
  if (!cfg || (cfg->dim != 2 && cfg->dim != 3) || cfg->n_systems < 1 || !cfg->systems)
    return fail(JDEM_ERR_BAD_ARG, "config: dim must be 2 or 3 and n_systems >= 1");
  if ((uint32_t)cfg->n_systems > TAG_SYS_MASK) return fail(JDEM_ERR_CAPACITY_OVERFLOW, "too many systems");
  if (cfg->n_materials < 1 || (uint32_t)cfg->n_materials > TAG_MAT_MASK || !cfg->young_eff)
    return fail(JDEM_ERR_BAD_ARG, "config: n_materials in [1, 2047] and young_eff required");
  if (cfg->bond_width < 0) return fail(JDEM_ERR_BAD_ARG, "config: bond_width < 0");
  if (!(cfg->skin >= 0.0f)) return fail(JDEM_ERR_BAD_ARG, "config: skin must be >= 0");
  dev = cfg->device;
  JDEM_CUDA_TRY(this, cudaSetDevice(dev));
  dim = cfg->dim;
  S = cfg->n_systems;
  skin = cfg->skin;
  chunk = cfg->chunk_steps > 0 ? cfg->chunk_steps : 50;
  n_mat = cfg->n_materials;
  bond_w = cfg->bond_width;
  interact_same_bond = cfg->interact_same_bond_id;
  use_nl = cfg->neighbor_list >= 0;
  if (cfg->graph_mode < 0 || cfg->graph_mode > 2) return fail(JDEM_ERR_BAD_ARG, "config: graph_mode in 0..2");
  if (cfg->force_law != JDEM_FORCE_SPRING && cfg->force_law != JDEM_FORCE_HERTZ &&
      cfg->force_law != JDEM_FORCE_CUNDALL_STRACK)
    return fail(JDEM_ERR_UNSUPPORTED, "config: unknown force_law");
  if (cfg->force_law == JDEM_FORCE_CUNDALL_STRACK && !cfg->material_props)
    return fail(JDEM_ERR_BAD_ARG, "config: Cundall-Strack needs material_props");
  graph_mode = cfg->graph_mode;
  use_conditional = graph_mode == 0;
  nl_request = cfg->neighbor_list;
  if (!std::isfinite(cfg->prune_skin)) return fail(JDEM_ERR_BAD_ARG, "config: prune_skin must be finite");
  prune_req = cfg->prune_skin;
  brick_tt = cfg->brick_particles > 0 ? (double)cfg->brick_particles : 0.0;  // 0: by handle size (plan_tiles)
  if (cfg->force_block != 0 && cfg->force_block != 64 && cfg->force_block != 128 && cfg->force_block != 256)
    return fail(JDEM_ERR_BAD_ARG, "config: force_block must be 0, 64, 128 or 256");
  if (cfg->small_lanes != 0 && cfg->small_lanes != 4 && cfg->small_lanes != 8 && cfg->small_lanes != 16)
    return fail(JDEM_ERR_BAD_ARG, "config: small_lanes must be 0, 4, 8 or 16");
  b.force_block = cfg->force_block ? cfg->force_block : 128;
  b.small_lanes = cfg->small_lanes ? cfg->small_lanes : 8;
  int rc0 = set_systems(cfg->systems, S);
  if (rc0) return rc0;
  JDEM_CUDA_TRY(this, cudaStreamCreateWithFlags(&own, cudaStreamNonBlocking));
  JDEM_CUDA_TRY(this, cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking));
  stream = own;
  JDEM_CUDA_TRY(this, cudaMallocHost((void**)&h_status, sizeof(Ctl)));
  int rc;
  if ((rc = dalloc((void**)&b.ctl, sizeof(Ctl)))) return rc;
  if ((rc = dalloc((void**)&d_young, sizeof(float) * n_mat * n_mat))) return rc;
  JDEM_CUDA_TRY(this, cudaMemcpyAsync(d_young, cfg->young_eff, sizeof(float) * n_mat * n_mat,
                                      cudaMemcpyHostToDevice, stream));
  if ((rc = ensure_capacity(P, S))) return rc;
  b.young = d_young;
  b.n_mat = n_mat;
  b.law = cfg->force_law == JDEM_FORCE_HERTZ ? LAW_HERTZ
          : cfg->force_law == JDEM_FORCE_CUNDALL_STRACK ? LAW_CS : LAW_SPRING;
  if (b.law == LAW_CS) {
    float* d_mprop = nullptr;
    if ((rc = dalloc((void**)&d_mprop, sizeof(float) * 4 * n_mat))) return rc;
    JDEM_CUDA_TRY(this, cudaMemcpyAsync(d_mprop, cfg->material_props, sizeof(float) * 4 * n_mat,
                                        cudaMemcpyHostToDevice, stream));
    b.mprop = d_mprop;
  }
  b.bond_w = bond_w;
  b.interact_same_bond = interact_same_bond;
  if ((rc = bind_systems())) return rc;
  JDEM_CUDA_TRY(this, cudaStreamSynchronize(stream));
  return JDEM_OK;
}

// Validate and adopt a system list (sets desc, S, P).
int JdemHandle::set_systems(const JdemSystemDesc* systems, int n_systems) {
  if (!systems || n_systems < 1) return fail(JDEM_ERR_BAD_ARG, "at least one system is required");
  if ((uint32_t)n_systems > TAG_SYS_MASK) return fail(JDEM_ERR_CAPACITY_OVERFLOW, "too many systems");
  long long p = 0;
  for (int s = 0; s < n_systems; ++s) {
    const JdemSystemDesc& d = systems[s];
    if (d.n < 0) return fail(JDEM_ERR_BAD_ARG, "system n < 0");
    if (d.domain < 0 || d.domain > 2) return fail(JDEM_ERR_BAD_ARG, "unknown domain");
    if (d.linear_integrator < 0 || d.linear_integrator > 2) return fail(JDEM_ERR_BAD_ARG, "unknown linear integrator");
    if (d.rotation_integrator < 0 || d.rotation_integrator > 2)
      return fail(JDEM_ERR_BAD_ARG, "unknown rotation integrator");
    if (!std::isfinite(d.dt)) return fail(JDEM_ERR_BAD_ARG, "dt must be finite");
    for (int a = 0; a < dim; ++a)
      if (d.domain != DOM_FREE && !(d.box_size[a] > 0.0f)) return fail(JDEM_ERR_BAD_ARG, "box_size must be positive");
    if (d.domain == DOM_REFLECT && !(d.restitution > 0.0f && d.restitution <= 1.0f))
      return fail(JDEM_ERR_BAD_ARG, "restitution_coefficient must be in (0, 1]");
    p += d.n;
  }
  if (p >= (1LL << 31) - 1) return fail(JDEM_ERR_CAPACITY_OVERFLOW, "more than 2^31-2 particles");
  desc.assign(systems, systems + n_systems);
  S = n_systems;
  P = p;
  return JDEM_OK;
}

// Grow every particle- and system-sized array to hold p_need particles and
// s_need systems (growth by 1.5x; shrinking keeps the allocation).
int JdemHandle::ensure_capacity(long long p_need, int s_need) {
  int rc;
  if (p_need > p_cap || p_cap == 0) {
    long long cap = std::max(std::max(p_need, 1LL), p_cap + p_cap / 2);
    drop_graphs();
    void** arrays[] = {(void**)&b.pos[0], (void**)&b.pos[1], (void**)&b.vel[0], (void**)&b.vel[1],
                       (void**)&b.frc[0], (void**)&b.frc[1], (void**)&b.tag[0], (void**)&b.tag[1],
                       (void**)&b.orig[0], (void**)&b.orig[1], (void**)&b.key[0], (void**)&b.key[1],
                       (void**)&b.key_tmp, (void**)&b.slot_tmp, (void**)&b.perm_tmp, (void**)&st_pos,
                       (void**)&st_vel, (void**)&st_frc, (void**)&st_rad, (void**)&st_mass, (void**)&st_mat,
                       (void**)&st_fixed, (void**)&st_sys, (void**)&d_q, (void**)&d_w, (void**)&d_tq,
                       (void**)&d_inertia, (void**)&d_bond, (void**)&b.nbr, (void**)&b.ncnt, (void**)&b.posw,
                       (void**)&b.img};
    for (void** a : arrays) {
      dfree(*a);
      *a = nullptr;
    }
    b.nl_cap = 0;
    nl_alloc_p = 0;
    nl_alloc_ints = 0;
    size_t p4 = sizeof(float4) * (size_t)cap, p1 = sizeof(int32_t) * (size_t)cap;
    size_t pd = sizeof(float) * (size_t)cap * dim;
    size_t pa = sizeof(float) * (size_t)cap * (dim == 3 ? 3 : 1);
    for (int k = 0; k < 2; ++k) {
      if ((rc = dalloc((void**)&b.pos[k], p4))) return rc;
      if ((rc = dalloc((void**)&b.vel[k], p4))) return rc;
      if ((rc = dalloc((void**)&b.frc[k], p4))) return rc;
      if ((rc = dalloc((void**)&b.tag[k], p1))) return rc;
      if ((rc = dalloc((void**)&b.orig[k], p1))) return rc;
      if ((rc = dalloc((void**)&b.key[k], p1))) return rc;
    }
    if ((rc = dalloc((void**)&b.key_tmp, p1)) || (rc = dalloc((void**)&b.slot_tmp, p1)) ||
        (rc = dalloc((void**)&b.perm_tmp, p1)) || (rc = dalloc((void**)&st_pos, pd)) ||
        (rc = dalloc((void**)&st_vel, pd)) || (rc = dalloc((void**)&st_frc, pd)) ||
        (rc = dalloc((void**)&st_rad, p1)) || (rc = dalloc((void**)&st_mass, p1)) ||
        (rc = dalloc((void**)&st_mat, p1)) || (rc = dalloc((void**)&st_fixed, (size_t)cap)) ||
        (rc = dalloc((void**)&st_sys, p1)) || (rc = dalloc((void**)&d_q, p4)) || (rc = dalloc((void**)&d_w, pa)) ||
        (rc = dalloc((void**)&d_tq, pa)) || (rc = dalloc((void**)&d_inertia, pa)))
      return rc;
    if (bond_w > 0 && (rc = dalloc((void**)&d_bond, sizeof(int32_t) * (size_t)cap * bond_w))) return rc;
    p_cap = cap;
  }
  if (s_need > s_cap) {
    int cap = std::max(s_need, s_cap + s_cap / 2);
    drop_graphs();
    dfree(b.sys);
    dfree(b.bbox);
    b.sys = nullptr;
    b.bbox = nullptr;
    if ((rc = dalloc((void**)&b.sys, sizeof(SysParams) * cap)) || (rc = dalloc((void**)&b.bbox, sizeof(float) * 6 * cap)))
      return rc;
    s_cap = cap;
  }
  b.bond = d_bond;
  b.rq = (float4*)d_q;
  b.rw = d_w;
  b.rtq = d_tq;
  b.rinertia = d_inertia;
  b.sys_of = st_sys;
  b.fixed_c = st_fixed;
  b.rad_c = st_rad;
  return JDEM_OK;
}

// Per-particle system index (caller order) for the current system list.
int JdemHandle::bind_systems() {
  b.P = P;
  b.S = S;
  std::vector<int32_t> sys_of((size_t)std::max(P, 1LL));
  long long off = 0;
  for (int s = 0; s < S; ++s)
    for (long long i = 0; i < desc[s].n; ++i) sys_of[(size_t)(off++)] = s;
  JDEM_CUDA_TRY(this, cudaMemcpyAsync(st_sys, sys_of.data(), sizeof(int32_t) * (size_t)std::max(P, 1LL),
                                      cudaMemcpyHostToDevice, stream));
  JDEM_CUDA_TRY(this, cudaStreamSynchronize(stream));
  return JDEM_OK;
}

// Replace the system list of a live handle (serving): capacity grows as
// needed, graphs are dropped when the shape changes, and the new state must
// be uploaded before stepping.
int JdemHandle::rebind(const JdemSystemDesc* systems, int n_systems) {
  JDEM_CUDA_TRY(this, cudaSetDevice(dev));
  int rc = set_systems(systems, n_systems);
  if (rc) return rc;
  if ((rc = ensure_capacity(P, S))) return rc;
  drop_graphs();
  uploaded = false;
  return bind_systems();
}

// Grid + cell arrays from the uploaded radii (host copy rad_h) and positions:
// per-system maximum radius and bounding box, then plan_grid.
// Per-system grids from the maximum radius and (free domain) bounding box,
// cell arrays sized to fit, then the Verlet-list capacity.
int JdemHandle::plan_grid(const float* rmax_s, const float* lo_s, const float* hi_s) {
  sys_h.assign((size_t)S, SysParams{});
  long long c_total = 0, off = 0;
  any_free = false;
  for (int s = 0; s < S; ++s) {
    const JdemSystemDesc& d = desc[s];
    SysParams& sp = sys_h[s];
    std::memset(&sp, 0, sizeof(sp));
    for (int a = 0; a < 3; ++a) {
      float bx = a < dim ? d.box_size[a] : 1.0f;
      sp.box[a] = bx;
      sp.inv_box[a] = 1.0f / bx;  // system.py:69-74
      sp.anchor[a] = a < dim ? d.anchor[a] : 0.0f;
      sp.gravity[a] = a < dim ? d.gravity[a] : 0.0f;
    }
    sp.domain = d.domain;
    sp.lin = d.linear_integrator;
    sp.rot = d.rotation_integrator;
    sp.dt = d.dt;
    sp.restitution = d.restitution;
    sp.p0 = off;
    sp.np = d.n;
    float lo[3] = {0, 0, 0}, hi[3] = {1, 1, 1};
    for (int a = 0; a < dim; ++a) {
      lo[a] = lo_s[(size_t)s * 3 + a];
      hi[a] = hi_s[(size_t)s * 3 + a];
    }
    if (d.domain == DOM_FREE) any_free = true;
    choose_grid(sp, dim, rmax_s[s], skin, d.n, lo, hi);
    // list cutoff widening: a few float32 ulps of the largest coordinate the
    // list build subtracts (wrapped positions plus a box-length image shift)
    float ext = 0.0f;
    for (int a = 0; a < dim; ++a) ext = std::max(ext, std::fabs(sp.anchor[a]) + 2.0f * sp.box[a]);
    sp.nl_eps = 8.0f * ext * 5.9604645e-8f;
    sp.c0 = c_total;
    c_total += sp.ncap;
    if (c_total >= (1LL << 31) - 2)
      return fail(JDEM_ERR_HASH_OVERFLOW, "total cell count exceeds the int32 hash range");
    off += d.n;
  }
  if (c_total > c_cap) {
    drop_graphs();
    dfree(b.cell_start);
    dfree(b.cnt);
    dfree(b.scan_blk);
    b.cell_start = b.cnt = b.scan_blk = nullptr;
    int rc;
    if ((rc = dalloc((void**)&b.cell_start, sizeof(int32_t) * (size_t)(c_total + 1)))) return rc;
    if ((rc = dalloc((void**)&b.cnt, sizeof(int32_t) * (size_t)c_total))) return rc;
    long long nb = (c_total + 2047) / 2048 + 1;
    if ((rc = dalloc((void**)&b.scan_blk, sizeof(int32_t) * (size_t)nb))) return rc;
    c_cap = c_total;
  }
  if (c_total != C) drop_graphs();
  C = c_total;
  b.C = C;
  JDEM_CUDA_TRY(this, cudaMemsetAsync(b.cnt, 0, sizeof(int32_t) * (size_t)C, stream));
  JDEM_CUDA_TRY(this, cudaMemcpyAsync(b.sys, sys_h.data(), sizeof(SysParams) * S, cudaMemcpyHostToDevice, stream));
  JDEM_CUDA_TRY(this, cudaStreamSynchronize(stream));
  if (!use_nl) return plan_list(0);
  int rc_t = plan_tiles();
  if (rc_t) return rc_t;
  // Verlet-list capacity: expected neighbours within 2 r_max + skin at the
  // densest system, plus six standard deviations of a Poisson count.  A row
  // that overflows switches the steps to the cell traversal (still exact)
  // until the host doubles the capacity.
  double mean_max = 0.0;
  for (int s = 0; s < S; ++s) {
    const SysParams& sp = sys_h[s];
    double vol = 1.0;
    double rl = 2.0 * rmax_s[s] + skin;
    for (int a = 0; a < dim; ++a)
      vol *= sp.domain == DOM_FREE ? std::max(1e-30, (double)sp.g[a] * (double)sp.gcell[a]) : (double)sp.box[a];
    double sphere = dim == 3 ? 4.18879 * rl * rl * rl : 3.14159 * rl * rl;
    double mean = desc[s].n / vol * sphere;
    mean_max = std::max(mean_max, mean);
  }
  int cap = (int)std::ceil(mean_max + 6.0 * std::sqrt(mean_max) + 8.0);
  cap = std::min(256, (cap + 7) / 8 * 8);
  if (nl_request > 0) cap = nl_request;
  return plan_list(cap);
}

// Tiles of the brick list build (jdem_tiles.cu) for every system: bricks of
// cells holding about brick_tt particles (unless configured, 240, and 60 for handles of at most
// kSmallForceSlots slots, whose few bricks would leave most SMs idle), near-cubic so the staged stencil region
// (the brick grown by one cell per side) is small against the brick; a system
// smaller than one brick is one tile.  Free domains re-grid on the device at
// every re-sort, so a handle with one keeps the per-slot list build (no tiles).
int JdemHandle::plan_tiles() {
  std::vector<TileDesc> t;
  int nst = 0, nv = 0, nrows = 0;
  if (!any_free && use_nl) {
    const double TT = brick_tt > 0.0 ? brick_tt : (P <= kSmallForceSlots ? 60.0 : 240.0);
    constexpr long long kMaxNV = 2048, kMaxHomeRows = 256, kMaxRows = 512;
    double stage_max = 0.0;
    long long nv_max = 0, rows_max = 0;
    for (int s = 0; s < S; ++s) {
      if (desc[s].n == 0) continue;
      const SysParams& sp = sys_h[s];
      const long long g[3] = {sp.g[0], sp.g[1], dim == 3 ? sp.g[2] : 1};
      const double cells = (double)g[0] * (double)g[1] * (double)g[2];
      const double occ = (double)desc[s].n / cells;
      const bool per = sp.domain == DOM_PERIODIC;
      int flags = (per && (g[0] < 3 || g[1] < 3 || (dim == 3 && g[2] < 3))) ? TILE_DIRECT : 0;
      // Unflagged list entries skip the minimum image: a pair in the same image
      // stays within r_i + r_j + 2 skin <= cell + skin while the list lives,
      // which must be below half the smallest box edge.
      float bmin = sp.box[0];
      for (int a = 1; a < dim; ++a) bmin = std::min(bmin, sp.box[a]);
      if (per && !(1.01f * (sp.cell_bin + skin) < 0.5f * bmin)) flags |= TILE_ALLIMAGE;
      // brick edge lengths in cells
      const double V = std::max(1.0, TT / std::max(occ, 1e-12));
      long long e[3];
      if (dim == 3) {
        const double side = std::cbrt(V);
        e[2] = std::min(g[2], std::max(1LL, (long long)std::llround(side)));
        e[1] = std::min(g[1], std::max(1LL, (long long)std::llround(side)));
        e[0] = std::min(g[0], std::max(1LL, (long long)std::llround(V / (double)(e[1] * e[2]))));
      } else {
        const double side = std::sqrt(V);
        e[2] = 1;
        e[1] = std::min(g[1], std::max(1LL, (long long)std::llround(side)));
        e[0] = std::min(g[0], std::max(1LL, (long long)std::llround(V / (double)e[1])));
      }
      while (e[1] * e[2] > kMaxHomeRows) {
        if (e[1] >= e[2]) e[1] = (e[1] + 1) / 2;
        else e[2] = (e[2] + 1) / 2;
      }
      long long nb[3];
      for (int a = 0; a < 3; ++a) nb[a] = (g[a] + e[a] - 1) / e[a];
      for (long long kz = 0; kz < nb[2]; ++kz)
        for (long long ky = 0; ky < nb[1]; ++ky)
          for (long long kx = 0; kx < nb[0]; ++kx) {
            TileDesc d{};
            d.sys = s;
            d.x0 = (int)(kx * g[0] / nb[0]);
            d.x1 = (int)((kx + 1) * g[0] / nb[0]);
            d.y0 = (int)(ky * g[1] / nb[1]);
            d.y1 = (int)((ky + 1) * g[1] / nb[1]);
            d.z0 = (int)(kz * g[2] / nb[2]);
            d.z1 = (int)((kz + 1) * g[2] / nb[2]);
            d.flags = flags;
            t.push_back(d);
            const long long v = (long long)(d.x1 - d.x0 + 2) * (d.y1 - d.y0 + 2) * (dim == 3 ? d.z1 - d.z0 + 2 : 1);
            const long long rows = (long long)(d.y1 - d.y0 + 2) * (dim == 3 ? d.z1 - d.z0 + 2 : 1);
            if (!flags && v <= kMaxNV && rows <= kMaxRows) {
              nv_max = std::max(nv_max, v);
              rows_max = std::max(rows_max, rows);
              stage_max = std::max(stage_max, (double)v * occ);
            }
          }
      if ((long long)t.size() > (1LL << 30)) return fail(JDEM_ERR_CAPACITY_OVERFLOW, "too many list tiles");
    }
    nv = (int)std::max(nv_max, 32LL);
    nrows = (int)std::max(rows_max, 9LL);
    nst = (int)std::min(4096.0, std::max(512.0, std::ceil((1.35 * stage_max + 64.0) / 256.0) * 256.0));
  }
  const bool same = t.size() == tiles_h.size() && nst == b.tb_nst && nv == b.tb_nv && nrows == b.tb_nrows &&
                    (t.empty() || std::memcmp(t.data(), tiles_h.data(), sizeof(TileDesc) * t.size()) == 0);
  if (!same) {
    drop_graphs();
    if ((long long)t.size() > tiles_alloc) {
      dfree(d_tiles);
      d_tiles = nullptr;
      tiles_alloc = 0;
      int rc = dalloc((void**)&d_tiles, sizeof(TileDesc) * t.size());
      if (rc) return rc;
      tiles_alloc = (long long)t.size();
    }
    if (!t.empty())
      JDEM_CUDA_TRY(this, cudaMemcpyAsync(d_tiles, t.data(), sizeof(TileDesc) * t.size(), cudaMemcpyHostToDevice,
                                          stream));
    JDEM_CUDA_TRY(this, cudaStreamSynchronize(stream));  // t is freed on return
    tiles_h.swap(t);
  }
  b.tiles = d_tiles;
  b.n_tiles = (int)tiles_h.size();
  b.tb_nst = nst;
  b.tb_nv = nv;
  b.tb_nrows = nrows;
  return JDEM_OK;
}

// (Re)allocate the Verlet list for cap entries per slot (0: no list), one
// cap x 32 block of entries per warp of slots.
int JdemHandle::plan_list(int cap) {
  // a multiple of four entries per row: the force kernels read rows in batches of four
  cap = std::min((cap + 3) / 4 * 4, kMaxListCap);
  const long long need = cap <= 0 ? 0 : ((P + 31) / 32) * 32LL * cap;
  if (cap > 0 && b.n_tiles > 0 && prepare_tbuild(tbuild_smem(b.tb_nst, b.tb_nv, b.tb_nrows)))
    return fail(JDEM_ERR_CUDA, "cannot raise shared memory for the list build");
  if (cap == b.nl_cap && (cap == 0 || (b.nbr && need <= nl_alloc_ints && P <= nl_alloc_p))) return JDEM_OK;
  drop_graphs();
  dfree(b.nbr);
  dfree(b.ncnt);
  dfree(b.nbr2);
  dfree(b.ncnt2);
  b.nbr = nullptr;
  b.ncnt = nullptr;
  b.nbr2 = nullptr;
  b.ncnt2 = nullptr;
  b.nl_cap = 0;
  nl_alloc_ints = 0;
  b.nl_skin = skin;
  if (cap <= 0 || P == 0) return JDEM_OK;
  int rc;
  if ((rc = dalloc((void**)&b.nbr, sizeof(int32_t) * (size_t)need))) return rc;
  if ((rc = dalloc((void**)&b.ncnt, sizeof(int32_t) * (size_t)P))) return rc;
  // dynamic pruning: the fused kernel of large sphere systems (k_force) only
  const float ps = prune_req == 0.0f ? skin / 3.0f : prune_req;
  b.prune_skin = 0.0f;
  if (ps > 0.0f && ps < skin && P > kSmallForceSlots && b.law != LAW_CS && b.NC == 0) {
    if ((rc = dalloc((void**)&b.nbr2, sizeof(int32_t) * (size_t)need))) return rc;
    if ((rc = dalloc((void**)&b.ncnt2, sizeof(int32_t) * (size_t)P))) return rc;
    b.prune_skin = ps;
  }
  // empty rows until the first build
  JDEM_CUDA_TRY(this, cudaMemsetAsync(b.ncnt, 0, sizeof(int32_t) * (size_t)P, stream));
  dfree(b.posw);
  dfree(b.img);
  b.posw = nullptr;
  b.img = nullptr;
  if ((rc = dalloc((void**)&b.posw, sizeof(float4) * (size_t)P))) return rc;
  if ((rc = dalloc((void**)&b.img, sizeof(int32_t) * (size_t)P))) return rc;
  b.nl_cap = cap;
  nl_alloc_p = P;
  nl_alloc_ints = need;
  return JDEM_OK;
}

int JdemHandle::reset_ctl() {
  Ctl c;
  std::memset(&c, 0, sizeof(c));
  c.need_rebuild = 1u;
  c.skin_half = 0.5f * skin;
  c.prune = 1u;
  c.pskin_half = b.nbr2 ? 0.5f * b.prune_skin : 0.0f;
  JDEM_CUDA_TRY(this, cudaMemcpyAsync(b.ctl, &c, sizeof(Ctl), cudaMemcpyHostToDevice, stream));
  return JDEM_OK;
}

int JdemHandle::upload(const JdemHostState* s, bool device_ptrs) {
  if (!s || !s->pos_c || !s->rad || !s->mass) return fail(JDEM_ERR_BAD_ARG, "upload: pos_c, rad and mass are required");
  JDEM_CUDA_TRY(this, cudaSetDevice(dev));
  // the arrays are copied before they are checked: until this upload
  // succeeds the handle holds no valid state
  uploaded = false;
  cudaMemcpyKind kind = device_ptrs ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  size_t N = (size_t)P;
  int ad = dim == 3 ? 3 : 1;
  int rc;
  if (N) {
    JDEM_CUDA_TRY(this, cudaMemcpyAsync(st_pos, s->pos_c, N * dim * 4, kind, stream));
    if (s->vel) JDEM_CUDA_TRY(this, cudaMemcpyAsync(st_vel, s->vel, N * dim * 4, kind, stream));
    else JDEM_CUDA_TRY(this, cudaMemsetAsync(st_vel, 0, N * dim * 4, stream));
    if (s->force) JDEM_CUDA_TRY(this, cudaMemcpyAsync(st_frc, s->force, N * dim * 4, kind, stream));
    else JDEM_CUDA_TRY(this, cudaMemsetAsync(st_frc, 0, N * dim * 4, stream));
    JDEM_CUDA_TRY(this, cudaMemcpyAsync(st_rad, s->rad, N * 4, kind, stream));
    JDEM_CUDA_TRY(this, cudaMemcpyAsync(st_mass, s->mass, N * 4, kind, stream));
    if (s->mat_id) JDEM_CUDA_TRY(this, cudaMemcpyAsync(st_mat, s->mat_id, N * 4, kind, stream));
    else JDEM_CUDA_TRY(this, cudaMemsetAsync(st_mat, 0, N * 4, stream));
    if (s->fixed) JDEM_CUDA_TRY(this, cudaMemcpyAsync(st_fixed, s->fixed, N, kind, stream));
    else JDEM_CUDA_TRY(this, cudaMemsetAsync(st_fixed, 0, N, stream));
    if (bond_w > 0) {
      if (!s->bond_id) return fail(JDEM_ERR_BAD_ARG, "upload: bond_id required when bond_width > 0");
      JDEM_CUDA_TRY(this, cudaMemcpyAsync(d_bond, s->bond_id, N * bond_w * 4, kind, stream));
    }
  }
  if (N) {
    // rotational state in caller order; defaults on the device
    if (s->q) JDEM_CUDA_TRY(this, cudaMemcpyAsync(d_q, s->q, N * 16, kind, stream));
    else launch_identity_q((float4*)d_q, (long long)N, stream);
    if (s->ang_vel) JDEM_CUDA_TRY(this, cudaMemcpyAsync(d_w, s->ang_vel, N * ad * 4, kind, stream));
    else JDEM_CUDA_TRY(this, cudaMemsetAsync(d_w, 0, N * ad * 4, stream));
    if (s->torque) JDEM_CUDA_TRY(this, cudaMemcpyAsync(d_tq, s->torque, N * ad * 4, kind, stream));
    else JDEM_CUDA_TRY(this, cudaMemsetAsync(d_tq, 0, N * ad * 4, stream));
    if (s->inertia) JDEM_CUDA_TRY(this, cudaMemcpyAsync(d_inertia, s->inertia, N * ad * 4, kind, stream));
    else launch_default_inertia(dim, (long long)N, st_mass, st_rad, d_inertia, stream);
    // rigid clumps: the clumps' state from their members, and the members'
    // world positions in place of pos_c for everything that follows
    if ((rc = setup_clumps(s, device_ptrs))) return rc;
    if (b.NC) {
      launch_rb_init(dim, b, st_pos, st_vel, st_frc, st_rad, st_mass, (const float4*)d_q, d_w, d_tq, d_inertia,
                     st_fixed, st_sys, st_pos, stream);
      JDEM_CUDA_TRY(this, cudaGetLastError());
    }
  }
  // per-system maximum radius, bounding box and input checks, reduced on the
  // device (k_scan_input): the host reads eight words per system
  std::vector<float> rmax((size_t)S, 0.0f), lo((size_t)S * 3, 0.0f), hi((size_t)S * 3, 1.0f);
  if (N) {
    if ((long long)S > scan_alloc) {
      dfree(d_scan);
      d_scan = nullptr;
      scan_alloc = 0;
      if ((rc = dalloc((void**)&d_scan, sizeof(unsigned int) * 8 * (size_t)S))) return rc;
      scan_alloc = S;
    }
    std::vector<unsigned int> init((size_t)S * 8, 0u);
    for (int s2 = 0; s2 < S; ++s2)
      for (int a = 1; a <= 3; ++a) init[(size_t)s2 * 8 + a] = 0xFFFFFFFFu;
    JDEM_CUDA_TRY(this, cudaMemcpyAsync(d_scan, init.data(), init.size() * 4, cudaMemcpyHostToDevice, stream));
    launch_scan_input(dim, P, st_pos, st_rad, s->mat_id ? st_mat : nullptr, n_mat, st_sys, d_scan, stream);
    JDEM_CUDA_TRY(this, cudaGetLastError());
    JDEM_CUDA_TRY(this, cudaMemcpyAsync(init.data(), d_scan, init.size() * 4, cudaMemcpyDeviceToHost, stream));
    JDEM_CUDA_TRY(this, cudaStreamSynchronize(stream));
    auto dec = [](unsigned int u) {
      unsigned int v = (u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u;
      float f;
      std::memcpy(&f, &v, 4);
      return f;
    };
    for (int s2 = 0; s2 < S; ++s2) {
      const unsigned int* o8 = init.data() + (size_t)s2 * 8;
      if (o8[7] & 1u) return fail(JDEM_ERR_BAD_ARG, "radius must be finite and >= 0");
      if (o8[7] & 2u) return fail(JDEM_ERR_NONFINITE, "non-finite position in upload");
      if (o8[7] & 4u) return fail(JDEM_ERR_BAD_ARG, "mat_id outside [0, n_materials)");
      if (desc[s2].n == 0) continue;
      rmax[(size_t)s2] = dec(o8[0]);
      for (int a = 0; a < dim; ++a) {
        lo[(size_t)s2 * 3 + a] = dec(o8[1 + a]);
        hi[(size_t)s2 * 3 + a] = dec(o8[4 + a]);
      }
    }
  }
  rc = plan_grid(rmax.data(), lo.data(), hi.data());
  if (rc) return rc;
  if (N) {
    // Is any rotational update non-trivial?  With omega = torque = 0 and
    // q = identity every rotation integrator and the reflect renormalisation
    // leave the state bit-identical, so the rotation kernel can be skipped.
    // Arrays the caller did not pass hold exactly those defaults.
    bool rot_nonzero = false;
    auto host_view = [&](const float* src, size_t count, std::vector<float>& tmp) -> const float* {
      if (!device_ptrs) return src;
      tmp.resize(count);
      // on the active stream: ordered after the caller's work that produced src
      if (cudaMemcpyAsync(tmp.data(), src, count * 4, cudaMemcpyDeviceToHost, stream) != cudaSuccess ||
          cudaStreamSynchronize(stream) != cudaSuccess)
        return nullptr;
      return tmp.data();
    };
    std::vector<float> tmp;
    if (s->q) {
      const float* q = host_view(s->q, N * 4, tmp);
      if (!q) return fail(JDEM_ERR_CUDA, "upload: reading q");
      for (size_t i = 0; i < N && !rot_nonzero; ++i)
        rot_nonzero = q[i * 4] != 1.0f || q[i * 4 + 1] != 0.0f || q[i * 4 + 2] != 0.0f || q[i * 4 + 3] != 0.0f;
    }
    for (const float* src : {s->ang_vel, s->torque}) {
      if (!src || rot_nonzero) continue;
      const float* v = host_view(src, N * ad, tmp);
      if (!v) return fail(JDEM_ERR_CUDA, "upload: reading rotational state");
      for (size_t i = 0; i < N * ad && !rot_nonzero; ++i) rot_nonzero = v[i] != 0.0f;
    }
    rot_active = rot_nonzero;
    launch_pack(dim, b, st_pos, st_vel, st_frc, st_rad, st_mass, st_mat, st_fixed, st_sys, stream);
    JDEM_CUDA_TRY(this, cudaGetLastError());
  }
  rc = reset_ctl();
  if (rc) return rc;
  cur_box.assign((size_t)S * 3, 0.0f);
  cur_anchor.assign((size_t)S * 3, 0.0f);
  for (int s2 = 0; s2 < S; ++s2)
    for (int a = 0; a < 3; ++a) {
      cur_box[(size_t)s2 * 3 + a] = a < dim ? desc[s2].box_size[a] : 0.0f;
      cur_anchor[(size_t)s2 * 3 + a] = a < dim ? desc[s2].anchor[a] : 0.0f;
    }
  bbox_pending = false;
  steps_done = 0;
  sticky_status = 0;
  uploaded = true;
  JDEM_CUDA_TRY(this, cudaStreamSynchronize(stream));
  return JDEM_OK;
}

// Upload from device arrays already in the reference layout, without any
// host read: per-system maximum radius and bounding box come from the caller.
// Spheres only, none fixed.  d_mat (material ids), d_q (orientation) and d_w
// (angular velocity) may be null: material 0, identity, zero spin; the
// inertia takes State.create's default from mass and radius.  rot: some
// system's rotation integrator has a non-trivial state to advance.
int JdemHandle::upload_resident(const float* d_pos, const float* d_vel, const float* d_frc, const float* d_rad,
                                const float* d_mass, const float* rmax_s, const float* lo_s, const float* hi_s,
                                const int32_t* d_mat, const float* d_q, const float* d_w, bool rot,
                                const float* d_torque) {
  JDEM_CUDA_TRY(this, cudaSetDevice(dev));
  int rc = plan_grid(rmax_s, lo_s, hi_s);
  if (rc) return rc;
  size_t N = (size_t)P;
  int ad = dim == 3 ? 3 : 1;
  if (N) {
    cudaMemcpyKind k = cudaMemcpyDeviceToDevice;
    JDEM_CUDA_TRY(this, cudaMemcpyAsync(st_pos, d_pos, N * dim * 4, k, stream));
    JDEM_CUDA_TRY(this, cudaMemcpyAsync(st_vel, d_vel, N * dim * 4, k, stream));
    if (d_frc) JDEM_CUDA_TRY(this, cudaMemcpyAsync(st_frc, d_frc, N * dim * 4, k, stream));
    else JDEM_CUDA_TRY(this, cudaMemsetAsync(st_frc, 0, N * dim * 4, stream));
    JDEM_CUDA_TRY(this, cudaMemcpyAsync(st_rad, d_rad, N * 4, k, stream));
    JDEM_CUDA_TRY(this, cudaMemcpyAsync(st_mass, d_mass, N * 4, k, stream));
    if (d_mat) JDEM_CUDA_TRY(this, cudaMemcpyAsync(st_mat, d_mat, N * 4, k, stream));
    else JDEM_CUDA_TRY(this, cudaMemsetAsync(st_mat, 0, N * 4, stream));
    JDEM_CUDA_TRY(this, cudaMemsetAsync(st_fixed, 0, N, stream));
    if (d_w) JDEM_CUDA_TRY(this, cudaMemcpyAsync(this->d_w, d_w, N * ad * 4, k, stream));
    else JDEM_CUDA_TRY(this, cudaMemsetAsync(this->d_w, 0, N * ad * 4, stream));
    // the torque of the last step: the next call's first rotational half-kick under
    // Cundall-Strack contacts (k_cs_rot_pre) reads it
    if (d_torque) JDEM_CUDA_TRY(this, cudaMemcpyAsync(d_tq, d_torque, N * ad * 4, k, stream));
    else JDEM_CUDA_TRY(this, cudaMemsetAsync(d_tq, 0, N * ad * 4, stream));
    launch_default_inertia(dim, (long long)N, st_mass, st_rad, d_inertia, stream);
    if (d_q) JDEM_CUDA_TRY(this, cudaMemcpyAsync(this->d_q, d_q, N * 16, k, stream));
    else launch_identity_q((float4*)this->d_q, (long long)N, stream);
    rot_active = rot;
    b.NC = 0;
    b.sclump = nullptr;
    launch_pack(dim, b, st_pos, st_vel, st_frc, st_rad, st_mass, st_mat, st_fixed, st_sys, stream);
    JDEM_CUDA_TRY(this, cudaGetLastError());
  }
  if ((rc = reset_ctl())) return rc;
  cur_box.assign((size_t)S * 3, 0.0f);
  cur_anchor.assign((size_t)S * 3, 0.0f);
  for (int s2 = 0; s2 < S; ++s2)
    for (int a = 0; a < 3; ++a) {
      cur_box[(size_t)s2 * 3 + a] = a < dim ? desc[s2].box_size[a] : 0.0f;
      cur_anchor[(size_t)s2 * 3 + a] = a < dim ? desc[s2].anchor[a] : 0.0f;
    }
  bbox_pending = false;
  steps_done = 0;
  sticky_status = 0;
  uploaded = true;
  return JDEM_OK;
}

// One step's device work after the first drift: re-sort if needed, then the
// fused force kernel.
void JdemHandle::enqueue_step(int mode) {
  launch_rebuild(dim, b, any_free, stream);
  launch_nlbuild(dim, b, stream);
  launch_force(dim, b, mode, stream);
  launch_fin(b, true, false, 0, stream);
}

// Conditional handle on the graph being captured on `stream`.
int JdemHandle::capture_handle(cudaGraphConditionalHandle* hc) {
  cudaStreamCaptureStatus cst;
  cudaGraph_t cg;
  JDEM_CUDA_TRY(this, cudaStreamGetCaptureInfo(stream, &cst, nullptr, &cg, nullptr, nullptr, nullptr));
  JDEM_CUDA_TRY(this, cudaGraphConditionalHandleCreate(hc, cg, 0, cudaGraphCondAssignDefault));
  return JDEM_OK;
}

// One step inside a stream capture: the re-sort and list-build kernels form
// the body of a conditional node whose condition the previous k_fin (or, for
// the first step, k_cond) sets from the device flags, so a step without a
// re-sort launches two kernels (k_force, k_fin).
int JdemHandle::capture_step_conditional(int mode, cudaGraphConditionalHandle hc,
                                         cudaGraphConditionalHandle* next) {
  cudaStreamCaptureStatus cst;
  cudaGraph_t cg;
  const cudaGraphNode_t* deps = nullptr;
  size_t nd = 0;
  JDEM_CUDA_TRY(this, cudaStreamGetCaptureInfo(stream, &cst, nullptr, &cg, &deps, nullptr, &nd));
  cudaGraphNodeParams prm = {cudaGraphNodeTypeConditional};
  prm.type = cudaGraphNodeTypeConditional;
  prm.conditional.handle = hc;
  prm.conditional.type = cudaGraphCondTypeIf;
  prm.conditional.size = 1;
  cudaGraphNode_t node;
  JDEM_CUDA_TRY(this, cudaGraphAddNode(&node, cg, deps, nullptr, nd, &prm));
  cudaGraph_t body = prm.conditional.phGraph_out[0];
  JDEM_CUDA_TRY(this, cudaStreamBeginCaptureToGraph(side, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
  launch_rebuild(dim, b, any_free, side);
  launch_nlbuild(dim, b, side);
  cudaGraph_t body_out;
  JDEM_CUDA_TRY(this, cudaStreamEndCapture(side, &body_out));
  JDEM_CUDA_TRY(this, cudaStreamUpdateCaptureDependencies(stream, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
  launch_force(dim, b, mode, stream);
  if (next) {
    int rc = capture_handle(next);
    if (rc) return rc;
    launch_fin(b, true, true, *next, stream);
  } else {
    launch_fin(b, true, false, 0, stream);
  }
  return JDEM_OK;
}

// A chunk of nsteps MODE_STEP steps of a small system as one while node:
// body = re-sort kernels (returning at once when nothing is due), list build,
// and the cooperative many-step kernel, which runs steps until the chunk ends
// or a re-sort is due and sets the while condition (jdem_multi.cu).
int JdemHandle::capture_multi(long long nsteps, cudaGraphExec_t* ge) {
  *ge = nullptr;
  JDEM_CUDA_TRY(this, cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaSuccess;
  bool ok = false;
  do {
    launch_multi_init(b, (unsigned int)nsteps, stream);
    cudaStreamCaptureStatus cst;
    cudaGraph_t cg;
    const cudaGraphNode_t* deps = nullptr;
    size_t nd = 0;
    if ((e = cudaStreamGetCaptureInfo(stream, &cst, nullptr, &cg, &deps, nullptr, &nd)) != cudaSuccess) break;
    cudaGraphConditionalHandle hw;
    if ((e = cudaGraphConditionalHandleCreate(&hw, cg, 1, cudaGraphCondAssignDefault)) != cudaSuccess) break;
    cudaGraphNodeParams prm = {cudaGraphNodeTypeConditional};
    prm.type = cudaGraphNodeTypeConditional;
    prm.conditional.handle = hw;
    prm.conditional.type = cudaGraphCondTypeWhile;
    prm.conditional.size = 1;
    cudaGraphNode_t node;
    if ((e = cudaGraphAddNode(&node, cg, deps, nullptr, nd, &prm)) != cudaSuccess) break;
    cudaGraph_t body = prm.conditional.phGraph_out[0];
    if ((e = cudaStreamBeginCaptureToGraph(side, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal)) !=
        cudaSuccess)
      break;
    launch_rebuild(dim, b, any_free, side);
    launch_nlbuild(dim, b, side);
    const int lrc = launch_multi(dim, b, hw, side);
    cudaGraph_t body_out;
    const cudaError_t e2 = cudaStreamEndCapture(side, &body_out);
    if (lrc || e2 != cudaSuccess) {
      e = e2 != cudaSuccess ? e2 : cudaErrorNotSupported;
      break;
    }
    if ((e = cudaStreamUpdateCaptureDependencies(stream, &node, nullptr, 1, cudaStreamSetCaptureDependencies)) !=
        cudaSuccess)
      break;
    ok = true;
  } while (false);
  const cudaError_t ee = cudaStreamEndCapture(stream, &g);
  if (ok && ee == cudaSuccess && g) ok = cudaGraphInstantiate(ge, g, 0) == cudaSuccess;
  if (g) cudaGraphDestroy(g);
  if (!ok) {
    *ge = nullptr;
    cudaGetLastError();
    return fail(JDEM_ERR_CUDA, std::string("many-step graph capture: ") + cudaGetErrorString(e));
  }
  return JDEM_OK;
}

int JdemHandle::run_graph(long long nsteps, int mode_last) {
  if (graph_mode == 2) {
    for (long long k = 0; k < nsteps; ++k) enqueue_step(k + 1 == nsteps ? mode_last : MODE_STEP);
    JDEM_CUDA_TRY(this, cudaGetLastError());
    return JDEM_OK;
  }
  // key: (nsteps, mode of the final step)
  long long key = nsteps * 64 + mode_last;
  auto it = graphs.find(key);
  if (it == graphs.end()) {
    // Graphs are captured on the handle's own stream, which has no pending
    // work of the caller's, and launched on the active stream (possibly the
    // caller's) below; the capture only records work, it runs nothing.
    struct Restore {
      cudaStream_t& ref;
      cudaStream_t saved;
      ~Restore() { ref = saved; }
    } restore{stream, stream};
    stream = own;
    cudaGraphExec_t ge = nullptr;
    if (use_conditional && use_multi && mode_last == MODE_STEP && !any_free && multi_eligible(dim, b, dev)) {
      if (capture_multi(nsteps, &ge) != JDEM_OK) {
        use_multi = false;  // the per-step graphs below
        err.clear();
      } else {
        multi_used = true;
      }
    }
    for (int attempt = 0; attempt < 2 && !ge; ++attempt) {
      bool cond = use_conditional && attempt == 0;
      cudaGraph_t g = nullptr;
      JDEM_CUDA_TRY(this, cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
      int rc = JDEM_OK;
      cudaGraphConditionalHandle hc = 0;
      if (cond) {
        rc = capture_handle(&hc);
        if (rc == JDEM_OK) launch_cond(b, hc, stream);
      }
      for (long long k = 0; k < nsteps && rc == JDEM_OK; ++k) {
        int m = k + 1 == nsteps ? mode_last : MODE_STEP;
        if (cond) {
          cudaGraphConditionalHandle nx = 0;
          rc = capture_step_conditional(m, hc, k + 1 < nsteps ? &nx : nullptr);
          hc = nx;
        } else {
          enqueue_step(m);
        }
      }
      cudaError_t e = cudaStreamEndCapture(stream, &g);
      if (rc == JDEM_OK && e == cudaSuccess) {
        e = cudaGraphInstantiate(&ge, g, 0);
        if (e != cudaSuccess) ge = nullptr;
      }
      if (g) cudaGraphDestroy(g);
      if (!ge) {
        cudaGetLastError();
        if (!cond) return fail(JDEM_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
        use_conditional = false;  // fall back to unconditional re-sort launches
      }
    }
    it = graphs.emplace(key, ge).first;
  }
  JDEM_CUDA_TRY(this, cudaGraphLaunch(it->second, stream));
  return JDEM_OK;
}

int JdemHandle::step_async(long long n) {
  if (!uploaded) return fail(JDEM_ERR_NOT_READY, "step before upload");
  if (n < 0) return fail(JDEM_ERR_BAD_ARG, "n < 0");
  if (n == 0 || P == 0) {
    steps_done += n;
    return JDEM_OK;
  }
  JDEM_CUDA_TRY(this, cudaSetDevice(dev));
  int bbox = any_free ? MODE_BBOX : 0;
  if (any_free) launch_bbox_reset(b, stream);  // stream-ordered: no host round trip
  rb_force_only = false;
  if (b.NC) {
    launch_rb_pre(dim, b, n == 1 ? bbox : 0, stream);
  } else {
    launch_pre(dim, b, n == 1 ? bbox : 0, stream);
    if (b.law == LAW_CS) launch_cs_rot_pre(dim, b, stream);
  }
  JDEM_CUDA_TRY(this, cudaGetLastError());
  // steps 1 .. n-1 run MODE_STEP (their epilogue starts the next step);
  // step n-1 also records the free-domain box; step n is MODE_STEP_LAST.
  long long mid = n - 1;
  long long plain = any_free && mid > 0 ? mid - 1 : mid;
  int rc;
  while (plain >= chunk) {
    if ((rc = run_graph(chunk, MODE_STEP))) return rc;
    plain -= chunk;
  }
  if (plain > 0)
    if ((rc = run_graph(plain, MODE_STEP))) return rc;
  if (any_free && mid > 0)
    if ((rc = run_graph(1, MODE_STEP | MODE_BBOX))) return rc;
  if ((rc = run_graph(1, MODE_STEP_LAST))) return rc;
  // Cundall-Strack and rigid clumps integrate the rotation every step
  if (rot_active && b.law != LAW_CS && !b.NC) {
    launch_rot(dim, b, st_sys, (float4*)d_q, d_w, d_tq, d_inertia, st_fixed, n, stream);
    JDEM_CUDA_TRY(this, cudaGetLastError());
  }
  if (any_free) bbox_pending = true;
  steps_done += n;
  return JDEM_OK;
}

int JdemHandle::sync_status() {
  JDEM_CUDA_TRY(this, cudaMemcpyAsync(h_status, b.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, stream));
  JDEM_CUDA_TRY(this, cudaStreamSynchronize(stream));
  const Ctl* c = (const Ctl*)h_status;
  sticky_status |= c->status & ~(unsigned int)ST_NL_OVERFLOW;
  rebuilds = c->rebuilds;
  prunes = c->prunes;
  if (c->status & ST_NL_OVERFLOW) {
    // a list row overflowed: those steps used the cell traversal (still
    // exact); double the capacity and rebuild the list before the next step
    int grown = std::min(kMaxListCap, std::max(16, 2 * b.nl_cap));
    int rc = grown > b.nl_cap ? plan_list(grown) : JDEM_OK;
    if (rc) return rc;
    // a full re-sort: it refreshes the wrapped positions the new list build reads
    unsigned int st = c->status & ~(unsigned int)ST_NL_OVERFLOW, one = 1u;
    JDEM_CUDA_TRY(this, cudaMemcpyAsync(&b.ctl->status, &st, 4, cudaMemcpyHostToDevice, stream));
    JDEM_CUDA_TRY(this, cudaMemcpyAsync(&b.ctl->need_rebuild, &one, 4, cudaMemcpyHostToDevice, stream));
    JDEM_CUDA_TRY(this, cudaMemcpyAsync(&b.ctl->nl_dirty, &one, 4, cudaMemcpyHostToDevice, stream));
    JDEM_CUDA_TRY(this, cudaStreamSynchronize(stream));
    nl_regrowths += 1;
  }
  if (bbox_pending) {
    // FreeDomain.apply of the last step: box = max - min, anchor = min (free.py:59-63)
    std::vector<unsigned int> bb((size_t)S * 6);
    JDEM_CUDA_TRY(this, cudaMemcpyAsync(bb.data(), b.bbox, sizeof(unsigned int) * S * 6, cudaMemcpyDeviceToHost,
                                        stream));
    JDEM_CUDA_TRY(this, cudaStreamSynchronize(stream));
    auto dec = [](unsigned int u) {
      unsigned int v = (u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u;
      float f;
      std::memcpy(&f, &v, 4);
      return f;
    };
    for (int s2 = 0; s2 < S; ++s2) {
      if (desc[s2].domain != DOM_FREE || desc[s2].n == 0) continue;
      for (int a = 0; a < dim; ++a) {
        float lo = dec(bb[(size_t)s2 * 6 + a]), hi = dec(bb[(size_t)s2 * 6 + 3 + a]);
        cur_box[(size_t)s2 * 3 + a] = hi - lo;
        cur_anchor[(size_t)s2 * 3 + a] = lo;
      }
    }
    bbox_pending = false;
  }
  if (c->status & ST_NONFINITE) return fail(JDEM_ERR_NONFINITE, "non-finite position or velocity");
  if (c->status & ST_BARRIER_TIMEOUT) {
    // the many-step kernel stopped early: leave it for the per-step graphs
    use_multi = false;
    drop_graphs();
    Ctl fresh = *c;  // barrier bookkeeping back to zero, the timeout bit cleared
    fresh.status &= ~(unsigned int)ST_BARRIER_TIMEOUT;
    fresh.bar_count = fresh.bar_base = fresh.mstep = 0u;
    fresh.mx[0] = fresh.mx[1] = fresh.mx[2] = 0u;
    std::memcpy(h_status, &fresh, sizeof(Ctl));
    JDEM_CUDA_TRY(this, cudaMemcpyAsync(b.ctl, h_status, sizeof(Ctl), cudaMemcpyHostToDevice, stream));
    JDEM_CUDA_TRY(this, cudaStreamSynchronize(stream));
    sticky_status &= ~(unsigned int)ST_BARRIER_TIMEOUT;
    return fail(JDEM_ERR_TIMEOUT,
                "many-step kernel: a grid barrier timed out; the steps of that chunk are incomplete "
                "(later steps run one launch per step)");
  }

  return JDEM_OK;
}

int JdemHandle::step_timed(long long n, double* total_ms, double* force_ms) {
  if (!uploaded) return fail(JDEM_ERR_NOT_READY, "step before upload");
  if (n <= 0) return fail(JDEM_ERR_BAD_ARG, "n must be positive");
  JDEM_CUDA_TRY(this, cudaSetDevice(dev));
  size_t need = (size_t)(2 * n + 2);
  while (ev_pool.size() < need) {
    cudaEvent_t e;
    JDEM_CUDA_TRY(this, cudaEventCreate(&e));
    ev_pool.push_back(e);
  }
  if (any_free) {
    int rc = step_async(n);  // free domain keeps the graph path (box bookkeeping)
    if (rc) return rc;
    return sync_status();
  }
  JDEM_CUDA_TRY(this, cudaEventRecord(ev_pool[0], stream));
  rb_force_only = false;
  if (b.NC) {
    launch_rb_pre(dim, b, 0, stream);
  } else {
    launch_pre(dim, b, 0, stream);
    if (b.law == LAW_CS) launch_cs_rot_pre(dim, b, stream);
  }
  for (long long k = 0; k < n; ++k) {
    launch_rebuild(dim, b, any_free, stream);
    launch_nlbuild(dim, b, stream);
    JDEM_CUDA_TRY(this, cudaEventRecord(ev_pool[2 + 2 * k], stream));
    launch_force(dim, b, k + 1 == n ? MODE_STEP_LAST : MODE_STEP, stream);
    JDEM_CUDA_TRY(this, cudaEventRecord(ev_pool[3 + 2 * k], stream));
    launch_fin(b, true, false, 0, stream);
  }
  if (rot_active && b.law != LAW_CS && !b.NC)
    launch_rot(dim, b, st_sys, (float4*)d_q, d_w, d_tq, d_inertia, st_fixed, n, stream);
  JDEM_CUDA_TRY(this, cudaEventRecord(ev_pool[1], stream));
  JDEM_CUDA_TRY(this, cudaGetLastError());
  JDEM_CUDA_TRY(this, cudaEventSynchronize(ev_pool[1]));
  float ms = 0.0f;
  JDEM_CUDA_TRY(this, cudaEventElapsedTime(&ms, ev_pool[0], ev_pool[1]));
  double fsum = 0.0;
  for (long long k = 0; k < n; ++k) {
    float f = 0.0f;
    JDEM_CUDA_TRY(this, cudaEventElapsedTime(&f, ev_pool[2 + 2 * k], ev_pool[3 + 2 * k]));
    fsum += f;
  }
  if (total_ms) *total_ms = ms;
  if (force_ms) *force_ms = fsum;
  steps_done += n;
  return sync_status();
}

int JdemHandle::download(JdemHostState* s, bool device_ptrs, bool wait) {
  if (!uploaded) return fail(JDEM_ERR_NOT_READY, "download before upload");
  if (!s) return fail(JDEM_ERR_BAD_ARG, "download: null state");
  JDEM_CUDA_TRY(this, cudaSetDevice(dev));
  cudaMemcpyKind kind = device_ptrs ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  size_t N = (size_t)P;
  int ad = dim == 3 ? 3 : 1;
  if (N) {
    if (b.NC) launch_rb_unpack(dim, b, st_pos, st_vel, st_frc, (float4*)d_q, d_w, d_tq, rb_force_only, stream);
    else launch_unpack(dim, b, st_pos, st_vel, st_frc, stream);
    JDEM_CUDA_TRY(this, cudaGetLastError());
    if (s->pos_c) JDEM_CUDA_TRY(this, cudaMemcpyAsync(s->pos_c, st_pos, N * dim * 4, kind, stream));
    if (s->vel) JDEM_CUDA_TRY(this, cudaMemcpyAsync(s->vel, st_vel, N * dim * 4, kind, stream));
    if (s->force) JDEM_CUDA_TRY(this, cudaMemcpyAsync(s->force, st_frc, N * dim * 4, kind, stream));
    if (s->q) JDEM_CUDA_TRY(this, cudaMemcpyAsync(s->q, d_q, N * 16, kind, stream));
    if (s->ang_vel) JDEM_CUDA_TRY(this, cudaMemcpyAsync(s->ang_vel, d_w, N * ad * 4, kind, stream));
    if (s->torque) JDEM_CUDA_TRY(this, cudaMemcpyAsync(s->torque, d_tq, N * ad * 4, kind, stream));
  }
  return wait ? sync_status() : JDEM_OK;
}

int JdemHandle::set_stream(void* s) {
  JDEM_CUDA_TRY(this, cudaSetDevice(dev));
  cudaStream_t next = s ? (cudaStream_t)s : own;
  if (next == stream) return JDEM_OK;
  // work queued on the previous stream comes before anything queued on the next one
  cudaEvent_t ev;
  JDEM_CUDA_TRY(this, cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  cudaError_t e = cudaEventRecord(ev, stream);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(next, ev, 0);
  cudaEventDestroy(ev);
  JDEM_CUDA_TRY(this, e);
  stream = next;
  return JDEM_OK;
}

int JdemHandle::compute_force() {
  if (!uploaded) return fail(JDEM_ERR_NOT_READY, "compute_force before upload");
  if (P == 0) return JDEM_OK;
  JDEM_CUDA_TRY(this, cudaSetDevice(dev));
  launch_rebuild(dim, b, any_free, stream);
  launch_nlbuild(dim, b, stream);
  launch_force(dim, b, MODE_FORCE_ONLY, stream);
  int ad = dim == 3 ? 3 : 1;
  // smooth-sphere laws exert no torque; Cundall-Strack wrote its own, and
  // rigid clumps keep each sphere's force and torque for the download
  rb_force_only = b.NC > 0;
  if (b.law != LAW_CS && !b.NC) JDEM_CUDA_TRY(this, cudaMemsetAsync(d_tq, 0, (size_t)P * ad * 4, stream));
  JDEM_CUDA_TRY(this, cudaGetLastError());
  return sync_status();
}

int JdemHandle::energy(double* out, bool per_system) {
  if (!uploaded) return fail(JDEM_ERR_NOT_READY, "energy before upload");
  JDEM_CUDA_TRY(this, cudaSetDevice(dev));
  int ns = per_system ? S : 1;
  std::vector<double> acc((size_t)ns * 4, 0.0);
  if (P > 0) {
    // the binning is kept valid for the current positions by the skin
    // criterion; the rebuild kernels return at once unless a re-sort is due
    launch_rebuild(dim, b, any_free, stream);
    double* d_out = nullptr;
    int rc;
    if ((rc = dalloc((void**)&d_out, sizeof(double) * 4 * (size_t)P))) return rc;
    launch_energy(dim, b, d_out, stream);
    launch_ke_rot(dim, (long long)P, (const float4*)d_q, d_w, d_inertia, d_out + 3 * (size_t)P, stream);
    if (b.NC) launch_rb_energy(dim, b, d_out, stream);  // the clumps' terms, once per clump
    JDEM_CUDA_TRY(this, cudaGetLastError());
    std::vector<double> h((size_t)P * 4);
    JDEM_CUDA_TRY(this, cudaMemcpyAsync(h.data(), d_out, sizeof(double) * 4 * (size_t)P, cudaMemcpyDeviceToHost, stream));
    JDEM_CUDA_TRY(this, cudaStreamSynchronize(stream));
    dfree(d_out);
    long long off = 0;
    for (int s = 0; s < S; ++s) {
      int o = per_system ? s : 0;
      for (long long i = off; i < off + desc[s].n; ++i) {
        for (int c = 0; c < 3; ++c) acc[(size_t)o * 4 + c] += h[(size_t)i * 3 + c];
        acc[(size_t)o * 4 + 3] += h[3 * (size_t)P + (size_t)i];
      }
      off += desc[s].n;
    }
  }
  for (size_t k = 0; k < acc.size(); ++k) out[k] = acc[k];
  return sync_status();
}

int JdemHandle::contacts(int32_t* pairs, long long cap, long long* count) {
  if (!uploaded) return fail(JDEM_ERR_NOT_READY, "contacts before upload");
  if (!count || (cap > 0 && !pairs)) return fail(JDEM_ERR_BAD_ARG, "contacts: null output");
  *count = 0;
  if (P == 0) return JDEM_OK;
  JDEM_CUDA_TRY(this, cudaSetDevice(dev));
  launch_rebuild(dim, b, any_free, stream);
  int32_t* d_cnt = nullptr;
  long long* d_off = nullptr;
  int rc;
  if ((rc = dalloc((void**)&d_cnt, sizeof(int32_t) * (size_t)P))) return rc;
  launch_contacts(dim, b, 0, d_cnt, nullptr, nullptr, 0, stream);
  std::vector<int32_t> cnt((size_t)P);
  JDEM_CUDA_TRY(this, cudaMemcpyAsync(cnt.data(), d_cnt, sizeof(int32_t) * (size_t)P, cudaMemcpyDeviceToHost, stream));
  JDEM_CUDA_TRY(this, cudaStreamSynchronize(stream));
  std::vector<long long> off((size_t)P);
  long long tot = 0;
  for (long long t = 0; t < P; ++t) {
    off[(size_t)t] = tot;
    tot += cnt[(size_t)t];
  }
  *count = tot;
  if (tot > 0) {
    int32_t* d_pairs = nullptr;
    if ((rc = dalloc((void**)&d_off, sizeof(long long) * (size_t)P))) return rc;
    if ((rc = dalloc((void**)&d_pairs, sizeof(int32_t) * 2 * (size_t)tot))) return rc;
    JDEM_CUDA_TRY(this, cudaMemcpyAsync(d_off, off.data(), sizeof(long long) * (size_t)P, cudaMemcpyHostToDevice, stream));
    launch_contacts(dim, b, 1, nullptr, d_off, d_pairs, tot, stream);
    std::vector<int32_t> hp((size_t)tot * 2);
    JDEM_CUDA_TRY(this, cudaMemcpyAsync(hp.data(), d_pairs, sizeof(int32_t) * 2 * (size_t)tot, cudaMemcpyDeviceToHost, stream));
    JDEM_CUDA_TRY(this, cudaStreamSynchronize(stream));
    dfree(d_pairs);
    dfree(d_off);
    std::vector<long long> keys((size_t)tot);
    for (long long k = 0; k < tot; ++k) keys[(size_t)k] = ((long long)hp[2 * k] << 32) | (uint32_t)hp[2 * k + 1];
    std::sort(keys.begin(), keys.end());
    long long w = std::min(cap, tot);
    for (long long k = 0; k < w; ++k) {
      pairs[2 * k] = (int32_t)(keys[(size_t)k] >> 32);
      pairs[2 * k + 1] = (int32_t)(keys[(size_t)k] & 0xFFFFFFFFLL);
    }
  }
  dfree(d_cnt);
  return sync_status();
}

// ------------------------------------------------------------------- C ABI

extern "C" {

int jdem_abi_version(void) { return JDEM_ABI_VERSION; }

const char* jdem_status_string(int code) {
  if (code < 0 || code > 9) return "unknown status";
  return kStatusNames[code];
}

int jdem_create(const JdemConfig* cfg, JdemHandle** out) {
  if (!out) return JDEM_ERR_BAD_ARG;
  *out = nullptr;
  JdemHandle* h = new (std::nothrow) JdemHandle();
  if (!h) return JDEM_ERR_OOM;
  int rc = jdem_guard(&h->err, [&] { return h->setup(cfg); });
  if (rc) {
    std::fprintf(stderr, "jdem_create: %s\n", h->err.c_str());
    h->free_all();
    delete h;
    return rc;
  }
  *out = h;
  return JDEM_OK;
}

int jdem_destroy(JdemHandle* h) {
  if (!h) return JDEM_ERR_BAD_ARG;
  cudaSetDevice(h->dev);
  if (h->stream) cudaStreamSynchronize(h->stream);
  if (h->own && h->own != h->stream) cudaStreamSynchronize(h->own);
  h->free_all();
  delete h;
  return JDEM_OK;
}

const char* jdem_last_error(const JdemHandle* h) { return h ? h->err.c_str() : "null handle"; }

int jdem_upload(JdemHandle* h, const JdemHostState* s) {
  return h ? jdem_guard(&h->err, [&] { return h->upload(s, false); }) : JDEM_ERR_BAD_ARG;
}
int jdem_upload_device(JdemHandle* h, const JdemHostState* s) {
  return h ? jdem_guard(&h->err, [&] { return h->upload(s, true); }) : JDEM_ERR_BAD_ARG;
}

int jdem_step(JdemHandle* h, int64_t n) {
  if (!h) return JDEM_ERR_BAD_ARG;
  return jdem_guard(&h->err, [&] {
    int rc = h->step_async(n);
    return rc ? rc : h->sync_status();
  });
}

int jdem_step_async(JdemHandle* h, int64_t n) {
  return h ? jdem_guard(&h->err, [&] { return h->step_async(n); }) : JDEM_ERR_BAD_ARG;
}
int jdem_sync(JdemHandle* h) { return h ? jdem_guard(&h->err, [&] { return h->sync_status(); }) : JDEM_ERR_BAD_ARG; }

int jdem_step_timed(JdemHandle* h, int64_t n, double* total_ms, double* force_ms) {
  return h ? jdem_guard(&h->err, [&] { return h->step_timed(n, total_ms, force_ms); }) : JDEM_ERR_BAD_ARG;
}

int jdem_download(JdemHandle* h, JdemHostState* s) {
  return h ? jdem_guard(&h->err, [&] { return h->download(s, false); }) : JDEM_ERR_BAD_ARG;
}
int jdem_download_device(JdemHandle* h, JdemHostState* s) {
  return h ? jdem_guard(&h->err, [&] { return h->download(s, true); }) : JDEM_ERR_BAD_ARG;
}
int jdem_download_device_async(JdemHandle* h, JdemHostState* s) {
  return h ? jdem_guard(&h->err, [&] { return h->download(s, true, false); }) : JDEM_ERR_BAD_ARG;
}
int jdem_set_stream(JdemHandle* h, void* stream) {
  return h ? jdem_guard(&h->err, [&] { return h->set_stream(stream); }) : JDEM_ERR_BAD_ARG;
}
int jdem_compute_force(JdemHandle* h) {
  return h ? jdem_guard(&h->err, [&] { return h->compute_force(); }) : JDEM_ERR_BAD_ARG;
}

int jdem_energy(JdemHandle* h, double out[4]) {
  if (!h || !out) return JDEM_ERR_BAD_ARG;
  return jdem_guard(&h->err, [&] { return h->energy(out, false); });
}

int jdem_energy_per_system(JdemHandle* h, double* out) {
  if (!h || !out) return JDEM_ERR_BAD_ARG;
  return jdem_guard(&h->err, [&] { return h->energy(out, true); });
}

int jdem_contacts(JdemHandle* h, int32_t* pairs, int64_t cap, int64_t* count) {
  if (!h) return JDEM_ERR_BAD_ARG;
  long long c = 0;
  int rc = jdem_guard(&h->err, [&] { return h->contacts(pairs, cap, &c); });
  if (count) *count = c;
  return rc;
}

int jdem_neighbor_list(JdemHandle* h, float cutoff, int32_t max_neighbors, int32_t* out, int32_t* overflow) {
  if (!h) return JDEM_ERR_BAD_ARG;
  return jdem_guard(&h->err, [&] { return h->neighbor_list(cutoff, max_neighbors, out, overflow); });
}

int jdem_domain_state(JdemHandle* h, float* box, float* anchor) {
  if (!h) return JDEM_ERR_BAD_ARG;
  return jdem_guard(&h->err, [&] { return h->domain_state(box, anchor); });
}

int jdem_stats(JdemHandle* h, JdemStats* out) {
  if (!h || !out) return JDEM_ERR_BAD_ARG;
  if (h->uploaded) {
    int rc = jdem_guard(&h->err, [&] { return h->sync_status(); });
    if (rc && rc != JDEM_ERR_NONFINITE) return rc;
  }
  out->n_particles = h->P;
  out->n_cells = h->C;
  out->n_systems = h->S;
  out->dim = h->dim;
  out->rebuilds = h->rebuilds;
  out->steps = h->steps_done;
  out->device_status = h->sticky_status;
  out->graphs = (int32_t)h->graphs.size();
  out->device_bytes = h->device_bytes;
  out->list_regrowths = h->nl_regrowths;
  out->list_capacity = h->b.nl_cap;
  out->list_tiles = h->b.n_tiles;
  out->many_step = h->multi_used ? 1 : 0;
  out->prunes = (int32_t)h->prunes;
  return JDEM_OK;
}

void* jdem_stream(JdemHandle* h) { return h ? (void*)h->stream : nullptr; }

int jdem_set_barrier_limit(JdemHandle* h, uint32_t spins, uint32_t extra_arrivals) {
  if (!h) return JDEM_ERR_BAD_ARG;
  h->b.bar_spins = spins;
  h->b.bar_extra = extra_arrivals;
  h->drop_graphs();  // captured kernel parameters hold the old values
  if (extra_arrivals == 0) h->use_multi = true;
  return JDEM_OK;
}

int jdem_shape(const JdemHandle* h, int64_t* n_particles, int32_t* dim) {
  if (!h || !n_particles || !dim) return JDEM_ERR_BAD_ARG;
  *n_particles = h->P;
  *dim = h->dim;
  return JDEM_OK;
}

int jdem_host_register(void* ptr, size_t bytes) {
  if (!ptr || bytes == 0) return JDEM_ERR_BAD_ARG;
  cudaError_t e = cudaHostRegister(ptr, bytes, cudaHostRegisterDefault);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return JDEM_ERR_CUDA;
  }
  return JDEM_OK;
}

int jdem_host_unregister(void* ptr) {
  if (!ptr) return JDEM_ERR_BAD_ARG;
  cudaError_t e = cudaHostUnregister(ptr);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return JDEM_ERR_CUDA;
  }
  return JDEM_OK;
}

}  // extern "C"
