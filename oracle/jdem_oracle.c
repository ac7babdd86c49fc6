/*
 * CPU restatement of JaxDEM's per-step hot path in C with OpenMP.
 *
 * TEST INFRASTRUCTURE ONLY: this is the oracle (checker) and the timed CPU
 * baseline.  Only tests/, __graft_entry__.smoke() and bench.py's
 * cpu_baseline / reference arm load it.  Parity is pinned against the
 * reference's own known-answer tests (see oracle/dem_ref.py); bit-level
 * parity with XLA's reduction order is unpinned.
 *
 * Semantics follow the JaxDEM sources (paths relative to the project):
 *   step order             jaxdem/system.py:60-82
 *   cell-list parameters   jaxdem/colliders/_partition.py:54-99
 *   partition + stencil    jaxdem/colliders/cell_list.py:35-96
 *   pair traversal         jaxdem/colliders/cell_list.py:187-261 (chunks of 4)
 *   spring force           jaxdem/forces/spring.py:69-108
 *   periodic displacement  jaxdem/domains/periodic.py:74-79 (rint = half-even)
 *   reflect walls + TOC    jaxdem/domains/reflect.py:99-299, _toc.py:11-94
 *   free bounding box      jaxdem/domains/free.py:40-63
 *   gravity                jaxdem/forces/force_manager.py:393-397
 *   velocity Verlet        jaxdem/integrators/velocity_verlet.py:29-95
 *   direct Euler           jaxdem/integrators/direct_euler.py:30-66
 * Spheres only (clump_id = iota, pos_p = 0, no bonds).  Cell coordinates are
 * clamped into the grid (see dem_ref.cell_coords).  Built with
 * -ffp-contract=off so every float operation rounds as written.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

enum { DOM_FREE = 0, DOM_PERIODIC = 1, DOM_REFLECT = 2 };
enum { LIN_NONE = 0, LIN_VERLET = 1, LIN_EULER = 2 };

typedef struct {
  int dim, domain;
  float box[3], anchor[3], inv_box[3];
  float cell_req; /* requested cell size (collider.cell_size) */
  int sr;         /* search range */
  int64_t g[3], stride[3];
  float cell[3];
  int64_t ncell;
  int n_mat;
  const float* young;
} Grid;

static void grid_setup(Grid* G) {
  for (int a = 0; a < G->dim; ++a) {
    if (G->domain == DOM_PERIODIC) {
      int64_t g = (int64_t)floorf(G->box[a] / G->cell_req);
      if (g < 1) g = 1;
      G->g[a] = g;
      G->cell[a] = G->box[a] / (float)g;
    } else {
      int64_t g = (int64_t)ceilf(G->box[a] / G->cell_req);
      if (g < 1) g = 1;
      G->g[a] = g;
      G->cell[a] = G->cell_req;
    }
  }
  G->stride[0] = 1;
  for (int a = 1; a < G->dim; ++a) G->stride[a] = G->stride[a - 1] * G->g[a - 1];
  G->ncell = G->stride[G->dim - 1] * G->g[G->dim - 1];
}

static inline float floor_mod1(float x) {
  float m = fmodf(x, 1.0f);
  if (m < 0.0f) m = m + 1.0f;
  return m;
}

static inline void coords_of(const Grid* G, const float* p, int64_t* c) {
  for (int a = 0; a < G->dim; ++a) {
    float v;
    if (G->domain == DOM_PERIODIC) {
      float frac = floor_mod1((p[a] - G->anchor[a]) / G->box[a]);
      v = floorf(frac * (float)G->g[a]);
    } else {
      v = floorf((p[a] - G->anchor[a]) / G->cell_req);
    }
    int64_t ci = (int64_t)v;
    if (ci < 0) ci = 0;
    if (ci > G->g[a] - 1) ci = G->g[a] - 1;
    c[a] = ci;
  }
}

/* Stable counting sort of particles by cell hash: perm lists particle
 * indices cell by cell, ascending index within a cell (lax.sort is stable). */
static void build_cells(const Grid* G, int64_t n, const float* pos, int64_t* hash, int64_t* start,
                        int64_t* perm) {
  int d = G->dim;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    int64_t c[3];
    coords_of(G, pos + i * d, c);
    int64_t h = 0;
    for (int a = 0; a < d; ++a) h += c[a] * G->stride[a];
    hash[i] = h;
  }
  memset(start, 0, sizeof(int64_t) * (size_t)(G->ncell + 1));
  for (int64_t i = 0; i < n; ++i) start[hash[i] + 1]++;
  for (int64_t c = 0; c < G->ncell; ++c) start[c + 1] += start[c];
  int64_t* fill = (int64_t*)malloc(sizeof(int64_t) * (size_t)G->ncell);
  memcpy(fill, start, sizeof(int64_t) * (size_t)G->ncell);
  for (int64_t i = 0; i < n; ++i) perm[fill[hash[i]]++] = i;
  free(fill);
}

/* Force on i due to j: spring.py:97-108 with periodic._displacement. */
static inline void spring_pair(const Grid* G, const float* pi, const float* pj, float ri, float rj,
                               float k, int same, float* f) {
  int d = G->dim;
  float rij[3];
  float R = ri + rj;
  for (int a = 0; a < d; ++a) {
    float x = pi[a] - pj[a];
    if (G->domain == DOM_PERIODIC) x = x - G->box[a] * rintf(x * G->inv_box[a]);
    rij[a] = x;
  }
  float d_sq = rij[0] * rij[0];
  for (int a = 1; a < d; ++a) d_sq = d_sq + rij[a] * rij[a];
  float inv = (d_sq == 0.0f) ? 0.0f : 1.0f / sqrtf(d_sq > 1e-16f ? d_sq : 1e-16f);
  float r = d_sq * inv;
  float delta = R - r;
  if (!(delta > 0.0f)) delta = 0.0f;
  delta = delta * (same ? 0.0f : 1.0f);
  float mag = k * delta * inv;
  for (int a = 0; a < d; ++a) f[a] = mag * rij[a];
}

/* compute_force via the cell list in the reference's visiting order. */
static void cell_list_force(const Grid* G, int64_t n, const float* pos, const float* rad,
                            const int32_t* mat, const int64_t* hash, const int64_t* start,
                            const int64_t* perm, float* force, int acc64) {
  int d = G->dim;
  int side = 2 * G->sr + 1;
  int M = d == 3 ? side * side * side : side * side;
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t i = 0; i < n; ++i) {
    int64_t c[3];
    coords_of(G, pos + i * d, c);
    int64_t nh[343];
    for (int m = 0; m < M; ++m) {
      int off[3];
      int rem = m;
      for (int a = d - 1; a >= 0; --a) {
        off[a] = rem % side - G->sr;
        rem /= side;
      }
      int64_t h = 0;
      int oob = 0;
      for (int a = 0; a < d; ++a) {
        int64_t x = c[a] + off[a];
        if (G->domain == DOM_PERIODIC) {
          int64_t g = G->g[a];
          x = ((x % g) + g) % g;
        } else if (x < 0 || x >= G->g[a]) {
          oob = 1;
        }
        h += x * G->stride[a];
      }
      nh[m] = oob ? -1 : h;
    }
    if (G->domain == DOM_PERIODIC) {
      /* _dedup_stencil_hashes: an entry equal to an earlier one becomes -1 */
      int64_t orig[343];
      memcpy(orig, nh, sizeof(int64_t) * (size_t)M);
      for (int b = 0; b < M; ++b)
        for (int a = 0; a < b; ++a)
          if (orig[a] == orig[b]) {
            nh[b] = -1;
            break;
          }
    }
    double tot64[3] = {0, 0, 0};
    float tot[3] = {0, 0, 0};
    for (int m = 0; m < M; ++m) {
      int64_t h = nh[m];
      if (h < 0) continue;
      float acc[3] = {0, 0, 0};
      double acc64v[3] = {0, 0, 0};
      int64_t k0 = start[h], k1 = start[h + 1];
      for (int64_t k = k0; k < k1; k += 4) {
        float chunk[3] = {0, 0, 0};
        for (int u = 0; u < 4 && k + u < k1; ++u) {
          int64_t j = perm[k + u];
          float f[3];
          float kk = G->young[mat[i] * G->n_mat + mat[j]];
          spring_pair(G, pos + i * d, pos + j * d, rad[i], rad[j], kk, i == j, f);
          for (int a = 0; a < d; ++a) {
            chunk[a] = chunk[a] + f[a];
            acc64v[a] += (double)f[a];
          }
        }
        for (int a = 0; a < d; ++a) acc[a] = acc[a] + chunk[a];
      }
      for (int a = 0; a < d; ++a) {
        tot[a] = tot[a] + acc[a];
        tot64[a] += acc64v[a];
      }
    }
    for (int a = 0; a < d; ++a) force[i * d + a] = acc64 ? (float)tot64[a] : tot[a];
  }
  (void)hash;
}

/* _toc.verlet_collision_fraction for one coordinate. */
static inline float toc_alpha(float v_end, float acc, float delta, float ws, float dt) {
  float v_0 = v_end - dt * acc;
  float v_mid = v_end - 0.5f * dt * acc;
  float v_0_n = v_0 * ws, v_mid_n = v_mid * ws, acc_n = acc * ws;
  float A = 0.5f * acc_n * dt * dt;
  float B = v_0_n * dt;
  float dw = delta + v_mid_n * dt;
  float disc = B * B + 4.0f * A * dw;
  if (!(disc > 0.0f)) disc = 0.0f;
  float sq = disc > 0.0f ? sqrtf(disc) : 0.0f;
  float alpha;
  if (B < 0.0f) {
    float den = (B - sq < -1e-10f) ? B - sq : -1.0f;
    alpha = 2.0f * dw / den;
  } else {
    float den = (fabsf(2.0f * A) > 1e-10f) ? 2.0f * A : 1.0f;
    alpha = (-B - sq) / den;
  }
  if (alpha < 0.0f) alpha = 0.0f;
  if (alpha > 1.0f) alpha = 1.0f;
  return alpha;
}

/* ReflectDomain.apply for one sphere (segment reductions are identities). */
static inline void reflect_one(int d, const float* box, const float* anchor, float e, float dt,
                               float* p, float* v, const float* F, float rad, float mass,
                               int fixed) {
  float inv_mass = 1.0f / mass;
  float denom = inv_mass + 0.0f;
  if (denom == 0.0f) denom = 1.0f;
  float delta[3], ws[3], act[3], acc[3], alpha[3];
  for (int a = 0; a < d; ++a) {
    float lo = anchor[a] + rad, hi = anchor[a] + box[a] - rad;
    float olo = lo - p[a];
    if (!(olo > 0.0f)) olo = 0.0f;
    float ohi = p[a] - hi;
    if (!(ohi > 0.0f)) ohi = 0.0f;
    delta[a] = olo > ohi ? olo : ohi;
    ws[a] = (olo > 0.0f ? 1.0f : 0.0f) - (ohi > 0.0f ? 1.0f : 0.0f);
    act[a] = fabsf(ws[a]);
    acc[a] = F[a] * inv_mass;
    alpha[a] = toc_alpha(v[a], acc[a], delta[a], ws[a], dt);
  }
  float amin = 1.0f;
  for (int a = 0; a < d; ++a) {
    float x = act[a] > 0.0f ? alpha[a] : 1.0f;
    if (x < amin) amin = x;
  }
  float dt_factor = (amin - 1.0f) * dt;
  float dt_rem = (1.0f - amin) * dt;
  for (int a = 0; a < d; ++a) {
    float vc = v[a] + dt_factor * acc[a];
    float j = -(1.0f + e) * vc / denom;
    float closing = (vc * ws[a]) < 0.0f ? 1.0f : 0.0f;
    float cs = act[a] > 1.0f ? act[a] : 1.0f;
    float w = act[a] / cs;
    j = j * (w * closing);
    float dv = j * inv_mass;
    if (fixed) dv = 0.0f;
    v[a] = v[a] + dv;
    p[a] = p[a] + dv * dt_rem;
  }
}

static int64_t max_i64(int64_t a, int64_t b) { return a > b ? a : b; }

/* n steps of _step_once for spheres.  Returns 0 on success. */
int oracle_step(int dim, int64_t n, int domain, const float* box_in, const float* anchor_in,
                float restitution, const float* gravity, float dt, float cell_size,
                int search_range, int n_mat, const float* young_eff, int linear, float* pos,
                float* vel, float* force, const float* rad, const float* mass,
                const int32_t* mat_id, const uint8_t* fixed, int64_t steps, int n_threads,
                int acc64, float* box_out, float* anchor_out) {
#ifdef _OPENMP
  if (n_threads > 0) omp_set_num_threads(n_threads);
#endif
  if (dim != 2 && dim != 3) return 1;
  Grid G;
  memset(&G, 0, sizeof(G));
  G.dim = dim;
  G.domain = domain;
  G.cell_req = cell_size;
  G.sr = search_range;
  G.n_mat = n_mat;
  G.young = young_eff;
  for (int a = 0; a < dim; ++a) {
    G.box[a] = box_in[a];
    G.anchor[a] = anchor_in[a];
  }
  int64_t* hash = (int64_t*)malloc(sizeof(int64_t) * (size_t)max_i64(n, 1));
  int64_t* perm = (int64_t*)malloc(sizeof(int64_t) * (size_t)max_i64(n, 1));
  int64_t* start = NULL;
  int64_t cap = 0;
  for (int64_t s = 0; s < steps; ++s) {
    /* 3. domain.apply */
    if (domain == DOM_REFLECT) {
#pragma omp parallel for schedule(static)
      for (int64_t i = 0; i < n; ++i)
        reflect_one(dim, G.box, G.anchor, restitution, dt, pos + i * dim, vel + i * dim,
                    force + i * dim, rad[i], mass[i], fixed[i]);
    } else if (domain == DOM_FREE && n > 0) {
      for (int a = 0; a < dim; ++a) {
        float lo = pos[a] - rad[0], hi = pos[a] + rad[0];
        for (int64_t i = 1; i < n; ++i) {
          float l = pos[i * dim + a] - rad[i], h = pos[i * dim + a] + rad[i];
          if (l < lo) lo = l;
          if (h > hi) hi = h;
        }
        G.box[a] = hi - lo;
        G.anchor[a] = lo;
      }
    }
    /* 4. inv_box refresh */
    for (int a = 0; a < dim; ++a) G.inv_box[a] = 1.0f / G.box[a];
    /* 5. linear before */
    if (linear == LIN_VERLET) {
#pragma omp parallel for schedule(static)
      for (int64_t i = 0; i < n; ++i) {
        float sc = dt * 0.5f / mass[i];
        float fr = fixed[i] ? 0.0f : 1.0f;
        for (int a = 0; a < dim; ++a) {
          vel[i * dim + a] = vel[i * dim + a] + force[i * dim + a] * sc * fr;
          pos[i * dim + a] = pos[i * dim + a] + dt * vel[i * dim + a];
        }
      }
    }
    /* 7. collider.compute_force */
    grid_setup(&G);
    if (G.ncell + 1 > cap) {
      free(start);
      cap = G.ncell + 1;
      start = (int64_t*)malloc(sizeof(int64_t) * (size_t)cap);
    }
    build_cells(&G, n, pos, hash, start, perm);
    cell_list_force(&G, n, pos, rad, mat_id, hash, start, perm, force, acc64);
    /* 8. force_manager.apply (gravity), 9. linear after */
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
      float fr = fixed[i] ? 0.0f : 1.0f;
      for (int a = 0; a < dim; ++a) {
        float fcom = gravity[a] * (mass[i] / 1.0f);
        float f = force[i * dim + a] + 0.0f + fcom;
        force[i * dim + a] = f;
        if (linear == LIN_VERLET) {
          float sc = dt * 0.5f / mass[i];
          vel[i * dim + a] = vel[i * dim + a] + f * sc * fr;
        } else if (linear == LIN_EULER) {
          float sc = dt / mass[i];
          vel[i * dim + a] = vel[i * dim + a] + f * sc * fr;
          pos[i * dim + a] = pos[i * dim + a] + dt * vel[i * dim + a];
        }
      }
    }
  }
  if (box_out)
    for (int a = 0; a < dim; ++a) box_out[a] = G.box[a];
  if (anchor_out)
    for (int a = 0; a < dim; ++a) anchor_out[a] = G.anchor[a];
  free(hash);
  free(perm);
  free(start);
  return 0;
}

/* collider.compute_force alone (no integration): forces at the given positions. */
int oracle_force(int dim, int64_t n, int domain, const float* box, const float* anchor,
                 float cell_size, int search_range, int n_mat, const float* young_eff,
                 const float* pos, const float* rad, const int32_t* mat_id, float* force,
                 int n_threads, int acc64) {
#ifdef _OPENMP
  if (n_threads > 0) omp_set_num_threads(n_threads);
#endif
  Grid G;
  memset(&G, 0, sizeof(G));
  G.dim = dim;
  G.domain = domain;
  G.cell_req = cell_size;
  G.sr = search_range;
  G.n_mat = n_mat;
  G.young = young_eff;
  for (int a = 0; a < dim; ++a) {
    G.box[a] = box[a];
    G.anchor[a] = anchor[a];
    G.inv_box[a] = 1.0f / box[a];
  }
  grid_setup(&G);
  int64_t* hash = (int64_t*)malloc(sizeof(int64_t) * (size_t)max_i64(n, 1));
  int64_t* perm = (int64_t*)malloc(sizeof(int64_t) * (size_t)max_i64(n, 1));
  int64_t* start = (int64_t*)malloc(sizeof(int64_t) * (size_t)(G.ncell + 1));
  build_cells(&G, n, pos, hash, start, perm);
  cell_list_force(&G, n, pos, rad, mat_id, hash, start, perm, force, acc64);
  free(hash);
  free(perm);
  free(start);
  return 0;
}

int oracle_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
