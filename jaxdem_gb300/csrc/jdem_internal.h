// Host-side handle of the GB300 DEM step engine (not part of the public ABI).
#pragma once
#include <map>
#include <new>
#include <string>
#include <vector>

#include "../../include/jdem_gb300.h"
#include "jdem_device.cuh"

// Run a CUDA call; on failure record the message on the handle and return
// JDEM_ERR_OOM / JDEM_ERR_CUDA from the enclosing member function.
#define JDEM_CUDA_TRY(h, expr)                                                          \
  do {                                                                                  \
    cudaError_t _e = (expr);                                                            \
    if (_e != cudaSuccess) {                                                            \
      return (h)->fail(_e == cudaErrorMemoryAllocation ? JDEM_ERR_OOM : JDEM_ERR_CUDA,   \
                       std::string(#expr) + ": " + cudaGetErrorString(_e));            \
    }                                                                                   \
  } while (0)

struct JdemHandle;

// Runs the body of an entry point: a C++ exception (a failed host allocation,
// thread creation) becomes an error status and never crosses the C boundary.
template <typename F>
int jdem_guard(std::string* err, F&& body) noexcept {
  const char* what = "internal error";
  int code = JDEM_ERR_CUDA;
  try {
    return body();
  } catch (const std::bad_alloc&) {
    what = "host allocation failed";
    code = JDEM_ERR_OOM;
  } catch (...) {
  }
  if (err) {
    try {
      *err = what;
    } catch (...) {
    }
  }
  return code;
}

struct JdemHandle {
  // configuration
  int dev = 0;
  int dim = 3;
  int S = 0;
  long long P = 0;
  long long C = 0;
  long long p_cap = 0;  // allocated particle capacity
  long long c_cap = 0;  // allocated cell capacity
  int s_cap = 0;        // allocated system capacity
  long long nl_alloc_p = 0;
  long long nl_alloc_ints = 0;  // allocated Verlet-list entries
  std::vector<jdem::TileDesc> tiles_h;
  jdem::TileDesc* d_tiles = nullptr;
  long long tiles_alloc = 0;
  unsigned int* d_scan = nullptr;  // per-system upload summary (k_scan_input)
  long long scan_alloc = 0;
  float skin = 0.0f;
  int chunk = 50;
  int n_mat = 1;
  int bond_w = 0;
  int interact_same_bond = 0;
  std::vector<JdemSystemDesc> desc;
  std::vector<jdem::SysParams> sys_h;
  bool any_free = false;
  bool use_nl = true;
  int nl_request = 0;
  float prune_req = 0.0f;  // JdemConfig.prune_skin (0: skin / 3, < 0: off)
  double brick_tt = 0.0;  // particles per list-build brick (JdemConfig.brick_particles; 0: by handle size)
  bool rot_active = false;
  bool uploaded = false;
  bool bbox_pending = false;
  // current domain frame per system (free domain: last apply's bounding box)
  std::vector<float> cur_box, cur_anchor;

  // device state
  jdem::Bufs b{};
  float* d_young = nullptr;
  int32_t* d_bond = nullptr;
  float *st_pos = nullptr, *st_vel = nullptr, *st_frc = nullptr, *st_rad = nullptr, *st_mass = nullptr;
  int32_t *st_mat = nullptr, *st_sys = nullptr;
  uint8_t* st_fixed = nullptr;
  float4* d_q4 = nullptr;
  float *d_q = nullptr, *d_w = nullptr, *d_tq = nullptr, *d_inertia = nullptr;

  // rigid clumps: device arrays sized for the clump / sphere counts of the
  // last upload (b.NC = 0 when every sphere is its own body)
  long long rb_cap_c = 0, rb_cap_p = 0;
  int32_t* rb_sclump = nullptr;  // owner of b.sclump (b.sclump is null for sphere uploads)
  bool rb_force_only = false;  // the last force evaluation was compute_force
  // trajectory frames (jdem_rollout): device slot ring and the copy stream
  // that drains it
  cudaStream_t copy_stream = nullptr;
  std::vector<cudaEvent_t> ev_frame;  // per slot: unpacked, copied
  char* d_frames = nullptr;
  size_t d_frames_bytes = 0;

  // runtime
  cudaStream_t stream = nullptr;  // active stream: own, or the caller's (jdem_set_stream)
  cudaStream_t side = nullptr;     // captures the conditional re-sort bodies
  bool use_conditional = true;
  bool use_multi = true;  // small systems: many steps per cooperative launch (jdem_multi.cu)
  bool multi_used = false;  // a cached graph runs its steps as one cooperative many-step launch
  int graph_mode = 0;
  cudaStream_t own = nullptr;  // created by the handle: graph captures, and the default active stream
  void* h_status = nullptr;
  std::map<long long, cudaGraphExec_t> graphs;
  std::vector<cudaEvent_t> ev_pool;
  std::vector<void*> allocs;
  std::map<void*, size_t> alloc_bytes;
  long long device_bytes = 0;
  long long steps_done = 0;
  long long rebuilds = 0;
  long long prunes = 0;  // inner-list builds (dynamic pruning) since the upload
  long long nl_regrowths = 0;
  unsigned int sticky_status = 0;
  std::string err;

  int fail(int code, const std::string& msg);
  void free_all();
  int dalloc(void** p, size_t bytes);
  void dfree(void* p);
  void drop_graphs();
  int setup(const JdemConfig* cfg);
  int set_systems(const JdemSystemDesc* systems, int n_systems);
  int ensure_capacity(long long p_need, int s_need);
  int bind_systems();
  int rebind(const JdemSystemDesc* systems, int n_systems);
  int plan_grid(const float* rmax_s, const float* lo_s, const float* hi_s);
  int upload_resident(const float* d_pos, const float* d_vel, const float* d_frc, const float* d_rad,
                      const float* d_mass, const float* rmax_s, const float* lo_s, const float* hi_s,
                      const int32_t* d_mat = nullptr, const float* d_q = nullptr, const float* d_w = nullptr,
                      bool rot = false, const float* d_torque = nullptr);
  int plan_tiles();
  int plan_list(int cap);
  int reset_ctl();
  int upload(const JdemHostState* s, bool device_ptrs);
  void enqueue_step(int mode);
  int capture_multi(long long nsteps, cudaGraphExec_t* ge);
  int capture_handle(cudaGraphConditionalHandle* hc);
  int capture_step_conditional(int mode, cudaGraphConditionalHandle hc, cudaGraphConditionalHandle* next);
  int run_graph(long long nsteps, int mode_last);
  int step_async(long long n);
  int sync_status();
  int step_timed(long long n, double* total_ms, double* force_ms);
  int download(JdemHostState* s, bool device_ptrs, bool wait = true);
  int set_stream(void* s);
  int compute_force();
  int energy(double* out, bool per_system);
  int contacts(int32_t* pairs, long long cap, long long* count);
  int neighbor_list(float cutoff, int max_neighbors, int32_t* out, int32_t* overflow);
  int domain_state(float* box, float* anchor);
  int rollout(const int64_t* strides, long long n_frames, const JdemFrames* out);
  int setup_clumps(const JdemHostState* s, bool device_ptrs);
  void free_frames();
};
