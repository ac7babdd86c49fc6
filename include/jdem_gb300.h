/*
 * jdem_gb300 -- C ABI of the GB300 DEM step engine.
 *
 * The engine replaces JaxDEM's per-step hot path (paths relative to the
 * JaxDEM project):
 *   System.step / _step_once           jaxdem/system.py:60-98, 701-748
 *   DynamicCellList.compute_force      jaxdem/colliders/cell_list.py:434-464
 *   DynamicCellList.compute_potential_energy  jaxdem/colliders/cell_list.py:466-496
 *   SpringForce.force / energy         jaxdem/forces/spring.py:69-147
 *   ForceManager.apply (gravity)       jaxdem/forces/force_manager.py:338-425
 *   VelocityVerlet before/after        jaxdem/integrators/velocity_verlet.py:29-95
 *   DirectEuler after                  jaxdem/integrators/direct_euler.py:30-66
 *   VelocityVerletSpiral / Spiral      jaxdem/integrators/velocity_verlet_spiral.py:36-180,
 *                                      jaxdem/integrators/spiral.py
 *   Periodic / Reflect / Free domains  jaxdem/domains/periodic.py:74-79,
 *                                      jaxdem/domains/reflect.py:99-299, _toc.py:11-94,
 *                                      jaxdem/domains/free.py:40-63
 * JaxDEM itself has no native FFI; these entry points are what a JAX FFI
 * custom call (or the ctypes binding shipped in jaxdem_gb300/_lib.py) binds.
 *
 * Conventions.  Every function returns an int status (JDEM_OK = 0).  No C++
 * exception crosses this boundary.  A handle owns its device memory, which
 * stays resident between calls; host buffers belong to the caller.  All work
 * is ordered on the handle's active stream: its own stream, or the caller's
 * after jdem_set_stream.  A handle is not internally locked: use one handle
 * per host thread.  Arrays use the reference's row-major layouts:
 * pos_c/vel/force (N, dim), q (N, 4) as (w, x, y, z), ang_vel/torque/inertia
 * (N, 1) in 2D or (N, 3) in 3D, bond_id (N, W) padded with -1.  With several
 * systems in one handle their particles are concatenated in system order.
 */
#ifndef JDEM_GB300_H
#define JDEM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define JDEM_ABI_VERSION 13

enum {
  JDEM_OK = 0,
  JDEM_ERR_BAD_ARG = 1,
  JDEM_ERR_CAPACITY_OVERFLOW = 2,
  JDEM_ERR_HASH_OVERFLOW = 3,
  JDEM_ERR_NONFINITE = 4,
  JDEM_ERR_OOM = 5,
  JDEM_ERR_TIMEOUT = 6,
  JDEM_ERR_UNSUPPORTED = 7,
  JDEM_ERR_CUDA = 8,
  JDEM_ERR_NOT_READY = 9
};

enum { JDEM_DOMAIN_FREE = 0, JDEM_DOMAIN_PERIODIC = 1, JDEM_DOMAIN_REFLECT = 2 };
enum { JDEM_LIN_NONE = 0, JDEM_LIN_VERLET = 1, JDEM_LIN_EULER = 2 };
enum { JDEM_ROT_NONE = 0, JDEM_ROT_VERLET_SPIRAL = 1, JDEM_ROT_SPIRAL = 2 };
/* System.force_model: SpringForce (forces/spring.py), HertzianForce (forces/hertz.py) or
 * CundallStrackForce (forces/cundall_strack.py) */
enum { JDEM_FORCE_SPRING = 0, JDEM_FORCE_HERTZ = 1, JDEM_FORCE_CUNDALL_STRACK = 2 };

typedef struct JdemHandle JdemHandle;

/* One independent system (a System pytree: domain, integrators, dt). */
typedef struct {
  int64_t n;                   /* particles */
  int32_t domain;              /* JDEM_DOMAIN_*   (System.domain type) */
  int32_t linear_integrator;   /* JDEM_LIN_*      (System.linear_integrator) */
  int32_t rotation_integrator; /* JDEM_ROT_*      (System.rotation_integrator) */
  float dt;                    /* System.dt */
  float box_size[3];           /* Domain.box_size */
  float anchor[3];             /* Domain.anchor */
  float restitution;           /* ReflectDomain.restitution_coefficient */
  float gravity[3];            /* ForceManager.gravity */
  float cell_size;             /* DynamicCellList.cell_size (used by the neighbour list) */
  int32_t search_range;        /* max(DynamicCellList.neighbor_mask) */
} JdemSystemDesc;

typedef struct {
  int32_t dim;                  /* 2 or 3, shared by all systems of a handle */
  int32_t n_systems;            /* >= 1 */
  const JdemSystemDesc* systems;
  float skin;                   /* binning margin; 0 re-sorts every step */
  int32_t n_materials;          /* MaterialTable size M */
  const float* young_eff;       /* M*M row-major pair constant of the force law: spring k =
                                   MaterialTable.young_eff; Hertz (4/3) E* with
                                   1/E* = (1 - nu_i^2)/E_i + (1 - nu_j^2)/E_j (hertz.py:99-105);
                                   Cundall-Strack the damping ratio beta of e = min(e_i, e_j)
                                   (cundall_strack.py:143-150) */
  int32_t bond_width;           /* W of State.bond_id, 0 when there are no bonds */
  int32_t interact_same_bond_id;/* System.interact_same_bond_id */
  int32_t chunk_steps;          /* steps per captured CUDA graph (<= 0: 50) */
  int32_t device;               /* CUDA device ordinal */
  int32_t neighbor_list;        /* Verlet list built at each re-sort: 0 = on (capacity from the
                                   density), > 0 = on with this initial capacity (rounded up
                                   to a multiple of 4), -1 = off */
  int32_t graph_mode;           /* 0: CUDA graphs whose re-sort kernels sit in conditional nodes;
                                   systems of at most 32768 slots whose cooperative launch fits
                                   run each chunk as one many-step kernel in a while node;
                                   1: plain graphs (re-sort kernels always launched, returning
                                   early when no re-sort is due; profilers can see every node);
                                   2: no graphs (direct launches) */
  int32_t force_law;            /* JDEM_FORCE_* */
  const float* material_props;  /* Cundall-Strack only: M*4 per material (young, shear modulus
                                   young / (2 (1 + poisson)), mu, mu_r) */
  float prune_skin;             /* dynamic pruning of the Verlet list (systems above 32768 slots,
                                   spring / Hertz spheres): on steps between re-sorts the force
                                   kernel walks an inner list of the pairs within
                                   r_i + r_j + prune_skin, rebuilt from the full list whenever
                                   the drift since its build exceeds prune_skin / 2.
                                   0: skin / 3; < 0: off (every step walks the full list) */
  int32_t brick_particles;      /* list build: particles per brick of cells staged in shared
                                   memory (<= 0: 240, or 60 for handles of at most 32768
                                   slots) */
  int32_t force_block;          /* threads per block of the fused force kernel of handles above
                                   32768 slots: 64, 128 or 256 (0: 128); results do not depend
                                   on it */
  int32_t small_lanes;          /* lanes sharing a slot in the force kernels of handles of at
                                   most 32768 slots (per-step and many-step): 4, 8 or 16
                                   (0: 8); the partial sums of a slot combine in lane order */
} JdemConfig;

/* Particle arrays in the reference layout.  Upload reads every field that is
 * not NULL (rad, mass are required; q/ang_vel/torque/inertia/mat_id/fixed/
 * bond_id default to identity/zero/State.create defaults when NULL).
 * Download writes pos_c, vel, force, q, ang_vel, torque when not NULL.
 * Rigid clumps (State.add_clump, state.py:1230-1420): pos_p (N, dim) holds each
 * sphere's body-frame offset and clump_id (N) the clump index within its
 * system; members store their clump's pos_c, vel, q, ang_vel, mass and
 * inertia.  NULL for both means every sphere is its own body.  Clumps take
 * every force law: a Cundall-Strack contact of a member uses its clump's
 * velocity, angular velocity and mass, with the contact arm from the sphere's
 * own centre (cundall_strack.py:126-176), and jdem_neighbor_list lists the
 * members' world positions without same-clump pairs. */
typedef struct {
  float* pos_c;
  float* vel;
  float* force;
  float* q;
  float* ang_vel;
  float* torque;
  float* rad;
  float* mass;
  float* inertia;
  int32_t* mat_id;
  uint8_t* fixed;
  int32_t* bond_id;
  float* pos_p;
  int32_t* clump_id;
} JdemHostState;

typedef struct {
  int64_t n_particles;
  int64_t n_cells;
  int32_t n_systems;
  int32_t dim;
  int64_t rebuilds;          /* re-sorts since the last upload */
  int64_t steps;             /* steps since the last upload */
  uint32_t device_status;    /* sticky device status bits: 1 non-finite state, 2 capacity,
                                4 neighbour overflow, 16 grid-barrier timeout, 32 an index
                                out of range (only the bounds-checked build sets it) */
  int32_t graphs;            /* instantiated CUDA graphs */
  int64_t device_bytes;      /* device memory held by the handle */
  int64_t list_regrowths;    /* Verlet-list capacity doublings after a row overflowed */
  int32_t list_capacity;     /* entries per Verlet-list row (0: no list) */
  int32_t list_tiles;        /* cell bricks of the shared-memory list path (0: slot-order path) */
  int32_t many_step;         /* 1: step chunks run as one cooperative launch of many steps (small systems) */
  int32_t prunes;            /* inner-list builds of the dynamic pruning since the last upload */
} JdemStats;

/* ABI version of the loaded library (JDEM_ABI_VERSION). */
int jdem_abi_version(void);
/* Human-readable name of a status code. */
const char* jdem_status_string(int code);

/* System.create: allocate a handle for cfg->n_systems systems.
 * Replaces the per-slot Create methods (cell_list.py:374-432,
 * domains/__init__.py:62-121, force_manager.py:80-190) on the device side. */
int jdem_create(const JdemConfig* cfg, JdemHandle** out);
int jdem_destroy(JdemHandle* h);
/* Message of the last failing call on this handle ("" if none). */
const char* jdem_last_error(const JdemHandle* h);

/* Copy a State (State.create layout, state.py:369-867) to the device.
 * host: host pointers.  jdem_upload_device takes device pointers. */
int jdem_upload(JdemHandle* h, const JdemHostState* host);
int jdem_upload_device(JdemHandle* h, const JdemHostState* dev);

/* System.step(state, system, n) (system.py:701-748): n applications of
 * _step_once (system.py:60-82), captured in CUDA graphs of chunk_steps
 * steps.  Blocks until done and reports device status. */
int jdem_step(JdemHandle* h, int64_t n);
/* Same, without waiting; jdem_sync() waits and reports status. */
int jdem_step_async(JdemHandle* h, int64_t n);
int jdem_sync(JdemHandle* h);
/* jdem_step with CUDA-event timing: *total_ms = whole call on the stream,
 * *force_ms = summed duration of the fused force/integrate kernel launches
 * (each bracketed by its own events; launched without graphs). */
int jdem_step_timed(JdemHandle* h, int64_t n, double* total_ms, double* force_ms);

/* Read the State back (reference layout). */
int jdem_download(JdemHandle* h, JdemHostState* host);
int jdem_download_device(JdemHandle* h, JdemHostState* dev);

/* Destinations of jdem_rollout, stacked along a leading frame axis T in the
 * reference's particle order; a NULL pointer skips that field.
 *   pos_c, vel, force  (T, N, dim)      q  (T, N, 4)
 *   ang_vel, torque    (T, N, 1|3)
 *   box, anchor        (T, n_systems, 3): Domain.box_size / anchor after the
 *                      frame's steps (unused axes 0), always host memory. */
typedef struct {
  float* pos_c;
  float* vel;
  float* force;
  float* q;
  float* ang_vel;
  float* torque;
  float* box;
  float* anchor;
  int32_t device_ptrs; /* 1: the particle fields are device memory (frames stay in HBM) */
  int32_t ring;        /* host particle fields: device frame slots in flight (0: 3) */
} JdemFrames;

/* System.trajectory_rollout (system.py:606-699; scan body _trajectory_rollout,
 * system.py:99-120) with the default save_fn: for t in [0, n_frames), run
 * strides[t] steps (System.step), then save frame t -- a stride of 0 saves the
 * current state again.  Host destinations are filled from a ring of device
 * frame slots by a second stream whose copies overlap the next frame's steps
 * (fully for page-locked destinations -- cudaHostAlloc / jdem_host_register;
 * a pageable destination makes each frame's copy return only once it has
 * landed).  Blocks until every frame has landed. */
int jdem_rollout(JdemHandle* h, const int64_t* strides, int64_t n_frames, const JdemFrames* out);

/* DynamicCellList.compute_force (cell_list.py:434-464): contact forces at the
 * current positions (no gravity, no integration); torque = 0 for spheres.
 * Results are read with jdem_download. */
int jdem_compute_force(JdemHandle* h);

/* thermal.compute_energy terms summed over all systems (thermal.py:153-177):
 * out[0] = collider PE (cell_list.py:466-496), out[1] = gravity PE
 * (force_manager.py:427-479), out[2] = translational KE, out[3] = rotational KE. */
int jdem_energy(JdemHandle* h, double out[4]);
/* Same terms per system: out has 4 * n_systems doubles. */
int jdem_energy_per_system(JdemHandle* h, double* out);

/* Contact pairs (i < j, global indices, sorted lexicographically) with
 * |r_ij|^2 < (R_i + R_j)^2 -- the pairs whose spring overlap is positive
 * (utils/contacts.py:21-86 keeps the slots with nonzero force).  Writes at
 * most cap pairs to pairs[2*cap]; *count receives the total. */
int jdem_contacts(JdemHandle* h, int32_t* pairs, int64_t cap, int64_t* count);

/* DynamicCellList.create_neighbor_list (cell_list.py:498-595): per particle,
 * the indices within cutoff in the reference's stencil order, -1 padded;
 * out is (N, max_neighbors) int32 in caller order (global indices), and
 * *overflow is set when a row needed more than max_neighbors slots. */
int jdem_neighbor_list(JdemHandle* h, float cutoff, int32_t max_neighbors, int32_t* out,
                       int32_t* overflow);

/* Current Domain.box_size / Domain.anchor per system (n_systems * 3 floats
 * each, unused axes 0).  For the free domain these are the bounding box of
 * the last step's FreeDomain.apply (domains/free.py:40-63). */
int jdem_domain_state(JdemHandle* h, float* box, float* anchor);

int jdem_stats(JdemHandle* h, JdemStats* out);
/* Particle count and dimension of the handle's system list, without touching
 * the device (jdem_stats first reads the device status, which waits for the
 * handle's stream). */
int jdem_shape(const JdemHandle* h, int64_t* n_particles, int32_t* dim);
/* cudaStream_t the handle launches on (as void*): its own stream, or the one
 * given to jdem_set_stream. */
void* jdem_stream(JdemHandle* h);

/* Stream-ordered use, as an XLA FFI handler needs it (the reference's System.step
 * and compute_force, system.py:701-748 and colliders/cell_list.py:434-464, are
 * functional and XLA orders them on its compute stream): queue every later call's
 * work on `stream` (a cudaStream_t of the handle's device, as void*; NULL returns
 * to the handle's own stream).  Work already queued on the previous stream is
 * ordered before the next stream's work by an event, without a host wait.  CUDA
 * graphs are still captured on the handle's own stream and launched on `stream`.
 * Afterwards jdem_upload_device reads the caller's arrays after everything the
 * caller queued on `stream` before the call; it waits on the host once, for the
 * eight-word per-system summary (maximum radius, bounding box, input checks) that
 * sizes the cell grid.  jdem_step_async and jdem_download_device_async queue
 * their work and return; the results are valid for later work on `stream`. */
int jdem_set_stream(JdemHandle* h, void* stream);
/* jdem_download_device without the host wait: the copies into the caller's
 * device arrays are queued on the active stream; device status bits are read
 * by the next jdem_sync / jdem_step / jdem_stats. */
int jdem_download_device_async(JdemHandle* h, JdemHostState* dev);

/* Fault-path control of the many-step kernel's grid barrier (graph_mode 0, small
 * systems): a barrier polls at most `spins` times (0: the default, about a second)
 * before it gives up, and with extra_arrivals > 0 it also waits for that many
 * arrivals that never come, so every barrier gives up.  A barrier that gave up makes
 * the next jdem_sync / jdem_step return JDEM_ERR_TIMEOUT; the steps of that chunk are
 * incomplete and the handle runs later steps one launch per step.  For tests of the
 * timeout path; normal use never calls it. */
int jdem_set_barrier_limit(JdemHandle* h, uint32_t spins, uint32_t extra_arrivals);

/* One integrator stage on caller-owned device buffers, for callers that run the
 * reference's stage order themselves through the split factory types
 * (Integrator.step_before_force / step_after_force, integrators/__init__.py:51-91):
 * stage 0 = step_before_force, 1 = step_after_force of the linear integrator
 * `linear` (JDEM_LIN_*: VelocityVerlet velocity_verlet.py:29-95, DirectEuler
 * direct_euler.py:30-66) and of the rotation integrator `rotation` (JDEM_ROT_*:
 * VelocityVerletSpiral velocity_verlet_spiral.py:36-180, Spiral spiral.py:56-144);
 * either may be NONE.  pos_c, vel, force: n*dim floats; mass: n; fixed: n bytes
 * or NULL (every particle free); q: n*4 floats (w, x, y, z), 16-byte aligned;
 * ang_vel, torque, inertia: n*(dim == 3 ? 3 : 1) floats (lab frame; rotation
 * only).  pos_c, vel, q and ang_vel are updated in place with the fused step's
 * arithmetic; work is queued on `stream` (NULL: the default stream), nothing is
 * allocated and nothing waits. */
int jdem_integrate(int32_t dim, int64_t n, int32_t linear, int32_t rotation, int32_t stage, float dt,
                   float* pos_c, float* vel, const float* force, const float* mass, const uint8_t* fixed,
                   float* q, float* ang_vel, const float* torque, const float* inertia, void* stream);

/* Domain.apply of one sphere system (system.py:60-82, first stage) on caller-owned
 * device buffers: JDEM_DOMAIN_PERIODIC has nothing to do (domains/__init__.py:123-189);
 * JDEM_DOMAIN_REFLECT reflects spheres off the walls with the Verlet time-of-collision
 * correction (reflect.py:99-299, _toc.py:11-94), using the previous step's force, and
 * renormalises q when given (reflect.py:291-294); JDEM_DOMAIN_FREE writes the bounding
 * box of pos_c -+ (|pos_p| + rad) to box_out / anchor_out (host arrays of dim floats,
 * free.py:40-63; pos_p may be NULL) and waits for it on the host.  box_size and anchor
 * are host arrays of dim floats; fixed may be NULL; q is 16-byte aligned or NULL.
 * Rigid clumps take System.step (jdem_step). */
int jdem_domain_apply(int32_t dim, int64_t n, int32_t domain, float dt, float restitution,
                      const float* box_size, const float* anchor, float* pos_c, float* vel, const float* force,
                      const float* rad, const float* mass, const uint8_t* fixed, const float* pos_p, float* q,
                      float* box_out, float* anchor_out, void* stream);

/* ForceManager.apply of one sphere system on caller-owned device buffers
 * (force_manager.py:338-425 with every sphere its own body): force += external_force,
 * then + external_force_com + gravity * mass; torque += external_torque.  gravity is a
 * host array of dim floats; the external arrays may be NULL (zero); torque may be NULL
 * (not updated).  Queued on `stream`, nothing waits. */
int jdem_force_manager_apply(int32_t dim, int64_t n, const float* gravity, float* force, float* torque,
                             const float* external_force, const float* external_force_com,
                             const float* external_torque, const float* mass, void* stream);

/* Contact forces of one sphere system from caller-owned device buffers, without
 * allocating device memory.  No counterpart in the reference: it exists for callers
 * that may not call cudaMalloc while they run, such as an XLA FFI handler (XLA owns
 * and preallocates the device memory pool) or code inside another framework's
 * memory budget.  Scratch lives in one fixed device array per GPU, held until exit;
 * n is limited to JDEM_NOALLOC_MAX_PARTICLES (larger n: JDEM_ERR_CAPACITY_OVERFLOW)
 * and the grid is coarsened to JDEM_NOALLOC_MAX_CELLS cells.  Calls that overlap on
 * the GPU race on that array.  The first call on a device resolves the array's
 * address and must come before any stream capture.  pos (n, dim), rad (n) and force
 * (n, dim) are device pointers; box_size/anchor are host arrays of dim floats;
 * young is the spring stiffness; work is queued on stream without waiting. */
#define JDEM_NOALLOC_MAX_PARTICLES 65536
#define JDEM_NOALLOC_MAX_CELLS 131072
int jdem_compute_force_noalloc(int32_t dim, int64_t n, int32_t domain, const float* box_size,
                               const float* anchor, float young, const float* pos, const float* rad,
                               float* force, void* stream);

/* ---- Serving: continuous batching of rollout requests on one GPU ----------
 * A request is one independent system (State + System) and a step count, the
 * unit of System.step(state, system, n) / trajectory_rollout.  Requests are
 * admitted in arrival order while the active set stays under max_active,
 * target_particles and hbm_budget_bytes; every epoch advances all active
 * requests together (one batched launch per kernel) by
 * min(chunk_steps, smallest remaining count).  Between epochs a request's
 * state stays on the device (repacked device-to-device when the active set
 * changes).  Spheres with the spring or Hertz law and the server's material
 * table; each request brings its own domain, integrators (rotation included),
 * dt, material ids and rotational state. */
typedef struct JdemServer JdemServer;

typedef struct {
  int32_t dim;               /* 2 or 3 (one server per dimension) */
  int32_t device;
  int32_t max_active;        /* concurrent requests (<= 0: 1024) */
  int32_t chunk_steps;       /* steps per epoch at most (<= 0: 50) */
  int64_t target_particles;  /* admit while the active particles stay below this (<= 0: 4 Mi) */
  double hbm_budget_bytes;   /* admission limit on the resident footprint (<= 0: 150e9) */
  float skin;                /* binning skin of the batch */
  float young;               /* spring stiffness when n_materials is 0 */
  int32_t force_law;         /* JDEM_FORCE_SPRING, _HERTZ or _CUNDALL_STRACK (System.force_model) */
  int32_t n_materials;       /* size M of young_eff (0: one material of stiffness `young`) */
  const float* young_eff;    /* M*M pair constants, as JdemConfig.young_eff (copied at create) */
  const float* material_props; /* Cundall-Strack only: M*4, as JdemConfig.material_props (copied) */
} JdemServeConfig;

typedef struct {
  JdemSystemDesc system;     /* n, domain, integrators, dt, box, gravity */
  int64_t steps;
  const float* pos;          /* (n, dim) host arrays, copied at submit */
  const float* vel;
  const float* rad;
  const float* mass;
  const int32_t* mat_id;     /* (n) material ids, NULL: material 0 */
  const float* q;            /* (n, 4) orientation (w, x, y, z), NULL: identity */
  const float* ang_vel;      /* (n, 1) in 2D or (n, 3) in 3D, NULL: zero */
} JdemRequest;

typedef struct {
  int32_t state;             /* 0 pending, 1 active, 2 done, 3 cancelled, 4 failed */
  int32_t status;            /* status code of a failed request */
  int64_t n;
  int64_t steps;             /* steps completed */
  double submit_s, admit_s, done_s;  /* steady-clock seconds */
} JdemRequestInfo;

typedef struct {
  int64_t submitted, completed, epochs, repacks, particle_steps, max_active, failures;
  int64_t pending, active, bytes_in_use;
} JdemServeStats;

int jdem_serve_create(const JdemServeConfig* cfg, JdemServer** out);
/* Thread-safe; validates and copies the request.  *id identifies it. */
int jdem_serve_submit(JdemServer* s, const JdemRequest* req, int64_t* id);
/* Cancel a pending or active request (takes effect at the next epoch). */
int jdem_serve_cancel(JdemServer* s, int64_t id);
/* Ids of requests that finished (done, cancelled or failed) since the last poll. */
int jdem_serve_poll(JdemServer* s, int64_t* ids, int32_t cap, int32_t* count);
/* Final pos_c, vel, force of a done request (any pointer may be NULL) and its timings. */
int jdem_serve_result(JdemServer* s, int64_t id, float* pos, float* vel, float* force, JdemRequestInfo* info);
/* Same, into host arrays of a JdemHostState: pos_c, vel, force, q, ang_vel and
 * torque are written where not NULL (the other fields are ignored). */
int jdem_serve_result_state(JdemServer* s, int64_t id, JdemHostState* out, JdemRequestInfo* info);
/* Free a finished request's buffers. */
int jdem_serve_release(JdemServer* s, int64_t id);
/* Wait until no request is pending or active (timeout_s <= 0: no limit). */
int jdem_serve_drain(JdemServer* s, double timeout_s);
int jdem_serve_stats(JdemServer* s, JdemServeStats* out);
const char* jdem_serve_last_error(JdemServer* s);
int jdem_serve_destroy(JdemServer* s);

/* Page-lock caller host memory for asynchronous copies (cudaHostRegister). */
int jdem_host_register(void* ptr, size_t bytes);
int jdem_host_unregister(void* ptr);

#ifdef __cplusplus
}
#endif
#endif /* JDEM_GB300_H */
