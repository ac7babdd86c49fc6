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
 *   Hertz force            jaxdem/forces/hertz.py:63-117 (young_eff holds (4/3) E*)
 *   periodic displacement  jaxdem/domains/periodic.py:74-79 (rint = half-even)
 *   reflect walls + TOC    jaxdem/domains/reflect.py:99-299, _toc.py:11-94
 *   free bounding box      jaxdem/domains/free.py:40-63
 *   gravity                jaxdem/forces/force_manager.py:393-397
 *   velocity Verlet        jaxdem/integrators/velocity_verlet.py:29-95
 *   direct Euler           jaxdem/integrators/direct_euler.py:30-66
 * Spheres only (clump_id = iota, pos_p = 0, no bonds).  Cell coordinates are
 * clamped into the grid (see dem_ref.cell_coords).  Built with
 * -ffp-contract=off so every floating-point operation rounds as written.
 */
#include <math.h>
#include <stdint.h>
/* One source, two builds: float (default, the engine's arithmetic) and, with
 * -DJDEM_ORACLE_F64, double (the reference's jax_enable_x64 tests). */
/* Round half to even (jnp.round) without a libm call: adding and subtracting
 * 1.5 * 2^(mantissa bits) rounds in the default mode; exact for |x| below
 * 2^(mantissa bits - 1), otherwise rint. */
static inline float rint_f(float x) {
  const float m = 12582912.0f; /* 1.5 * 2^23 */
  if (x < 4194304.0f && x > -4194304.0f) {
    volatile float t = x + m;
    return t - m;
  }
  return rintf(x);
}
static inline double rint_d(double x) {
  const double m = 6755399441055744.0; /* 1.5 * 2^52 */
  if (x < 2251799813685248.0 && x > -2251799813685248.0) {
    volatile double t = x + m;
    return t - m;
  }
  return rint(x);
}
#ifdef JDEM_ORACLE_F64
typedef double real;
#define FN(name) name##_f64
#define R_SQRT sqrt
#define R_FLOOR floor
#define R_CEIL ceil
#define R_RINT rint_d
#define R_FMOD fmod
#define R_FABS fabs
#define R_POW pow
#else
typedef float real;
#define FN(name) name
#define R_SQRT sqrtf
#define R_FLOOR floorf
#define R_CEIL ceilf
#define R_RINT rint_f
#define R_FMOD fmodf
#define R_FABS fabsf
#define R_POW powf
#endif
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

enum { DOM_FREE = 0, DOM_PERIODIC = 1, DOM_REFLECT = 2 };
enum { LIN_NONE = 0, LIN_VERLET = 1, LIN_EULER = 2 };

typedef struct {
  int dim, domain;
  real box[3], anchor[3], inv_box[3];
  real cell_req; /* requested cell size (collider.cell_size) */
  int sr;         /* search range */
  int64_t g[3], stride[3];
  real cell[3];
  int64_t ncell;
  int n_mat;
  const real* young; /* spring k, or (4/3) E* for the Hertz law */
  int law;           /* 0 spring, 1 Hertz */
} Grid;

static void grid_setup(Grid* G) {
  for (int a = 0; a < G->dim; ++a) {
    if (G->domain == DOM_PERIODIC) {
      int64_t g = (int64_t)R_FLOOR(G->box[a] / G->cell_req);
      if (g < 1) g = 1;
      G->g[a] = g;
      G->cell[a] = G->box[a] / (real)g;
    } else {
      int64_t g = (int64_t)R_CEIL(G->box[a] / G->cell_req);
      if (g < 1) g = 1;
      G->g[a] = g;
      G->cell[a] = G->cell_req;
    }
  }
  G->stride[0] = 1;
  for (int a = 1; a < G->dim; ++a) G->stride[a] = G->stride[a - 1] * G->g[a - 1];
  G->ncell = G->stride[G->dim - 1] * G->g[G->dim - 1];
}

static inline real floor_mod1(real x) {
  real m = R_FMOD(x, 1.0f);
  if (m < 0.0f) m = m + 1.0f;
  return m;
}

static inline void coords_of(const Grid* G, const real* p, int64_t* c) {
  for (int a = 0; a < G->dim; ++a) {
    real v;
    if (G->domain == DOM_PERIODIC) {
      real frac = floor_mod1((p[a] - G->anchor[a]) / G->box[a]);
      v = R_FLOOR(frac * (real)G->g[a]);
    } else {
      v = R_FLOOR((p[a] - G->anchor[a]) / G->cell_req);
    }
    int64_t ci = (int64_t)v;
    if (ci < 0) ci = 0;
    if (ci > G->g[a] - 1) ci = G->g[a] - 1;
    c[a] = ci;
  }
}

/* Stable counting sort of particles by cell hash: perm lists particle
 * indices cell by cell, ascending index within a cell (lax.sort is stable). */
static void build_cells(const Grid* G, int64_t n, const real* pos, int64_t* hash, int64_t* start,
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
static inline void spring_pair(const Grid* G, const real* pi, const real* pj, real ri, real rj,
                               real k, int same, real* f) {
  int d = G->dim;
  real rij[3];
  real R = ri + rj;
  for (int a = 0; a < d; ++a) {
    real x = pi[a] - pj[a];
    if (G->domain == DOM_PERIODIC) x = x - G->box[a] * R_RINT(x * G->inv_box[a]);
    rij[a] = x;
  }
  real d_sq = rij[0] * rij[0];
  for (int a = 1; a < d; ++a) d_sq = d_sq + rij[a] * rij[a];
  real inv = (d_sq == 0.0f) ? 0.0f : 1.0f / R_SQRT(d_sq > 1e-16f ? d_sq : 1e-16f);
  real r = d_sq * inv;
  real delta = R - r;
  if (!(delta > 0.0f)) delta = 0.0f;
  delta = delta * (same ? 0.0f : 1.0f);
  real mag = k * delta * inv;
  for (int a = 0; a < d; ++a) f[a] = mag * rij[a];
}

/* Force on i due to j: hertz.py:99-117.  k43 = (4/3) E*; k = k43 sqrt(R*),
 * (n, r) = unit_and_norm(r_ij) (utils/linalg.py:164-181), F = k pow(delta, 1.5) n. */
static inline void hertz_pair(const Grid* G, const real* pi, const real* pj, real ri, real rj,
                              real k43, int same, real* f) {
  int d = G->dim;
  real rij[3];
  real R_star = (ri * rj) / (ri + rj);
  real k = k43 * R_SQRT(R_star);
  for (int a = 0; a < d; ++a) {
    real x = pi[a] - pj[a];
    if (G->domain == DOM_PERIODIC) x = x - G->box[a] * R_RINT(x * G->inv_box[a]);
    rij[a] = x;
  }
  real n2 = rij[0] * rij[0];
  for (int a = 1; a < d; ++a) n2 = n2 + rij[a] * rij[a];
  real inv = (n2 == 0.0f) ? 0.0f : 1.0f / R_SQRT(n2 > 1e-16f ? n2 : 1e-16f);
  real r = n2 * inv;
  real delta = (ri + rj) - r;
  if (!(delta > 0.0f)) delta = 0.0f;
  delta = delta * (same ? 0.0f : 1.0f);
  real mag = k * R_POW(delta, (real)1.5);
  for (int a = 0; a < d; ++a) f[a] = mag * (rij[a] * inv);
}

/* Stencil cell hashes of position p (cell_list.py:66-96): periodic axes wrap
 * by floor-mod, other axes mark out-of-grid cells -1, and for periodic grids
 * with fewer than 2*sr+1 cells along some axis a repeated hash becomes -1
 * (_dedup_stencil_hashes, cell_list.py:90-96).  Returns the stencil size M. */
static int stencil_hashes(const Grid* G, const real* p, int64_t* nh) {
  int d = G->dim;
  int side = 2 * G->sr + 1;
  int M = d == 3 ? side * side * side : side * side;
  {
    int64_t c[3];
    coords_of(G, p, c);
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
    int small_grid = 0;
    for (int a = 0; a < d; ++a) small_grid |= G->g[a] < side;
    if (G->domain == DOM_PERIODIC && small_grid) {
      /* _dedup_stencil_hashes: an entry equal to an earlier one becomes -1
       * (duplicates exist only when some axis has fewer than 2*sr+1 cells) */
      int64_t orig[343];
      memcpy(orig, nh, sizeof(int64_t) * (size_t)M);
      for (int b = 0; b < M; ++b)
        for (int a = 0; a < b; ++a)
          if (orig[a] == orig[b]) {
            nh[b] = -1;
            break;
          }
    }
  }
  return M;
}

/* compute_force via the cell list in the reference's visiting order. */
static void cell_list_force(const Grid* G, int64_t n, const real* pos, const real* rad,
                            const int32_t* mat, const int64_t* hash, const int64_t* start,
                            const int64_t* perm, real* force, int acc64) {
  int d = G->dim;
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t i = 0; i < n; ++i) {
    int64_t nh[343];
    const int M = stencil_hashes(G, pos + i * d, nh);
    double tot64[3] = {0, 0, 0};
    real tot[3] = {0, 0, 0};
    for (int m = 0; m < M; ++m) {
      int64_t h = nh[m];
      if (h < 0) continue;
      real acc[3] = {0, 0, 0};
      double acc64v[3] = {0, 0, 0};
      int64_t k0 = start[h], k1 = start[h + 1];
      for (int64_t k = k0; k < k1; k += 4) {
        real chunk[3] = {0, 0, 0};
        for (int u = 0; u < 4 && k + u < k1; ++u) {
          int64_t j = perm[k + u];
          real f[3];
          real kk = G->young[mat[i] * G->n_mat + mat[j]];
          if (G->law == 1)
            hertz_pair(G, pos + i * d, pos + j * d, rad[i], rad[j], kk, i == j, f);
          else
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
    for (int a = 0; a < d; ++a) force[i * d + a] = acc64 ? (real)tot64[a] : tot[a];
  }
  (void)hash;
}

/* _toc.verlet_collision_fraction for one coordinate. */
static inline real toc_alpha(real v_end, real acc, real delta, real ws, real dt) {
  real v_0 = v_end - dt * acc;
  real v_mid = v_end - 0.5f * dt * acc;
  real v_0_n = v_0 * ws, v_mid_n = v_mid * ws, acc_n = acc * ws;
  real A = 0.5f * acc_n * dt * dt;
  real B = v_0_n * dt;
  real dw = delta + v_mid_n * dt;
  real disc = B * B + 4.0f * A * dw;
  if (!(disc > 0.0f)) disc = 0.0f;
  real sq = disc > 0.0f ? R_SQRT(disc) : 0.0f;
  real alpha;
  if (B < 0.0f) {
    real den = (B - sq < -1e-10f) ? B - sq : -1.0f;
    alpha = 2.0f * dw / den;
  } else {
    real den = (R_FABS(2.0f * A) > 1e-10f) ? 2.0f * A : 1.0f;
    alpha = (-B - sq) / den;
  }
  if (alpha < 0.0f) alpha = 0.0f;
  if (alpha > 1.0f) alpha = 1.0f;
  return alpha;
}

/* ReflectDomain.apply for one sphere (segment reductions are identities). */
static inline void reflect_one(int d, const real* box, const real* anchor, real e, real dt,
                               real* p, real* v, const real* F, real rad, real mass,
                               int fixed) {
  real inv_mass = 1.0f / mass;
  real denom = inv_mass + 0.0f;
  if (denom == 0.0f) denom = 1.0f;
  real delta[3], ws[3], act[3], acc[3], alpha[3];
  for (int a = 0; a < d; ++a) {
    real lo = anchor[a] + rad, hi = anchor[a] + box[a] - rad;
    real olo = lo - p[a];
    if (!(olo > 0.0f)) olo = 0.0f;
    real ohi = p[a] - hi;
    if (!(ohi > 0.0f)) ohi = 0.0f;
    delta[a] = olo > ohi ? olo : ohi;
    ws[a] = (olo > 0.0f ? 1.0f : 0.0f) - (ohi > 0.0f ? 1.0f : 0.0f);
    act[a] = R_FABS(ws[a]);
    acc[a] = F[a] * inv_mass;
    alpha[a] = toc_alpha(v[a], acc[a], delta[a], ws[a], dt);
  }
  real amin = 1.0f;
  for (int a = 0; a < d; ++a) {
    real x = act[a] > 0.0f ? alpha[a] : 1.0f;
    if (x < amin) amin = x;
  }
  real dt_factor = (amin - 1.0f) * dt;
  real dt_rem = (1.0f - amin) * dt;
  for (int a = 0; a < d; ++a) {
    real vc = v[a] + dt_factor * acc[a];
    real j = -(1.0f + e) * vc / denom;
    real closing = (vc * ws[a]) < 0.0f ? 1.0f : 0.0f;
    real cs = act[a] > 1.0f ? act[a] : 1.0f;
    real w = act[a] / cs;
    j = j * (w * closing);
    real dv = j * inv_mass;
    if (fixed) dv = 0.0f;
    v[a] = v[a] + dv;
    p[a] = p[a] + dv * dt_rem;
  }
}

static int64_t max_i64(int64_t a, int64_t b) { return a > b ? a : b; }

/* n steps of _step_once for spheres.  Returns 0 on success. */
int FN(oracle_step)(int dim, int64_t n, int domain, const real* box_in, const real* anchor_in,
                real restitution, const real* gravity, real dt, real cell_size,
                int search_range, int n_mat, const real* young_eff, int linear, real* pos,
                real* vel, real* force, const real* rad, const real* mass,
                const int32_t* mat_id, const uint8_t* fixed, int64_t steps, int n_threads,
                int acc64, real* box_out, real* anchor_out, int law) {
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
  G.law = law;
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
        real lo = pos[a] - rad[0], hi = pos[a] + rad[0];
        for (int64_t i = 1; i < n; ++i) {
          real l = pos[i * dim + a] - rad[i], h = pos[i * dim + a] + rad[i];
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
        real sc = dt * 0.5f / mass[i];
        real fr = fixed[i] ? 0.0f : 1.0f;
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
      real fr = fixed[i] ? 0.0f : 1.0f;
      for (int a = 0; a < dim; ++a) {
        real fcom = gravity[a] * (mass[i] / 1.0f);
        real f = force[i * dim + a] + 0.0f + fcom;
        force[i * dim + a] = f;
        if (linear == LIN_VERLET) {
          real sc = dt * 0.5f / mass[i];
          vel[i * dim + a] = vel[i * dim + a] + f * sc * fr;
        } else if (linear == LIN_EULER) {
          real sc = dt / mass[i];
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
int FN(oracle_force)(int dim, int64_t n, int domain, const real* box, const real* anchor,
                 real cell_size, int search_range, int n_mat, const real* young_eff,
                 const real* pos, const real* rad, const int32_t* mat_id, real* force,
                 int n_threads, int acc64, int law) {
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
  G.law = law;
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

/* Canonical contact set: pairs (i < j) with d_sq < (r_i + r_j)^2, d the
 * displacement of periodic.py:74-79 (d - box * round(d * inv_box)) summed
 * left to right, enumerated through the cell list (only pairs within one
 * stencil, as in the reference).  The reference has no contact-set API;
 * utils/contacts.py:21-86 keeps the candidates whose spring force is nonzero,
 * i.e. whose overlap is positive.  Called with pairs == NULL it returns the
 * count; otherwise it writes at most cap pairs, grouped by i in ascending
 * order (j in visiting order within a group), and returns the count.  A
 * negative return is an allocation failure. */
int64_t FN(oracle_contacts)(int dim, int64_t n, int domain, const real* box, const real* anchor,
                            real cell_size, const real* pos, const real* rad, int64_t* pairs,
                            int64_t cap, int n_threads) {
#ifdef _OPENMP
  if (n_threads > 0) omp_set_num_threads(n_threads);
#endif
  Grid G;
  memset(&G, 0, sizeof(G));
  G.dim = dim;
  G.domain = domain;
  G.cell_req = cell_size;
  G.sr = 1;
  for (int a = 0; a < dim; ++a) {
    G.box[a] = box[a];
    G.anchor[a] = anchor[a];
    G.inv_box[a] = 1.0f / box[a];
  }
  grid_setup(&G);
  int64_t* hash = (int64_t*)malloc(sizeof(int64_t) * (size_t)max_i64(n, 1));
  int64_t* perm = (int64_t*)malloc(sizeof(int64_t) * (size_t)max_i64(n, 1));
  int64_t* start = (int64_t*)malloc(sizeof(int64_t) * (size_t)(G.ncell + 1));
  int64_t* cnt = (int64_t*)malloc(sizeof(int64_t) * (size_t)(n + 1));
  if (!hash || !perm || !start || !cnt) {
    free(hash);
    free(perm);
    free(start);
    free(cnt);
    return -1;
  }
  build_cells(&G, n, pos, hash, start, perm);
  int64_t total = 0;
  for (int pass = 0; pass < (pairs ? 2 : 1); ++pass) {
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < n; ++i) {
      int64_t nh[27];
      const int M = stencil_hashes(&G, pos + i * dim, nh);
      int64_t c = 0, o = pass ? cnt[i] : 0;
      for (int m = 0; m < M; ++m) {
        int64_t h = nh[m];
        if (h < 0) continue;
        for (int64_t k = start[h]; k < start[h + 1]; ++k) {
          int64_t j = perm[k];
          if (j <= i) continue;
          real dsq = 0.0f;
          for (int a = 0; a < dim; ++a) {
            real x = pos[i * dim + a] - pos[j * dim + a];
            if (domain == DOM_PERIODIC) x = x - G.box[a] * R_RINT(x * G.inv_box[a]);
            dsq = a == 0 ? x * x : dsq + x * x;
          }
          real R = rad[i] + rad[j];
          if (dsq < R * R) {
            if (pass && o + c < cap) {
              pairs[2 * (o + c)] = i;
              pairs[2 * (o + c) + 1] = j;
            }
            ++c;
          }
        }
      }
      if (!pass) cnt[i] = c;
    }
    if (!pass) {
      /* exclusive prefix: cnt[i] becomes the first output row of i */
      for (int64_t i = 0; i < n; ++i) {
        int64_t c = cnt[i];
        cnt[i] = total;
        total += c;
      }
    }
  }
  free(hash);
  free(perm);
  free(start);
  free(cnt);
  return total;
}

int FN(oracle_max_threads)(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
