// Serving loop: continuous batching of rollout requests on one GPU.
//
// Requests (one independent system each, with a step count) are admitted in
// arrival order while the active set stays under the particle target, the
// slot limit and the HBM budget.  A worker thread advances every active
// request in one batched handle by K = min(chunk, smallest remaining step
// count) steps per epoch.  When the active set changes (a request finished,
// a request arrived, a request was cancelled) the continuing requests' state
// is repacked device-to-device into the new batch layout -- it never leaves
// the GPU between chunks -- and newcomers are copied in from pinned host
// memory.  Finished requests are copied out to pinned host buffers.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/jdem_gb300.h"
#include "jdem_device.cuh"
#include "jdem_internal.h"
#include "jdem_kernels.h"

using namespace jdem;

namespace {

enum ReqState { REQ_PENDING = 0, REQ_ACTIVE = 1, REQ_DONE = 2, REQ_CANCELLED = 3, REQ_FAILED = 4 };

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct Req {
  int64_t id = 0;
  JdemSystemDesc desc{};
  int64_t steps_total = 0, steps_done = 0;
  double t_submit = 0, t_admit = 0, t_done = 0;
  float rmax = 0, lo[3] = {0, 0, 0}, hi[3] = {1, 1, 1};
  float *h_pos = nullptr, *h_vel = nullptr, *h_rad = nullptr, *h_mass = nullptr;  // pinned inputs
  int32_t* h_mat = nullptr;                                                       // (n) material ids
  float *h_q = nullptr, *h_w = nullptr;                                           // rotational state
  float *o_pos = nullptr, *o_vel = nullptr, *o_frc = nullptr;                     // pinned outputs
  float *o_q = nullptr, *o_w = nullptr;
  bool rot = false;  // a rotation integrator with a non-trivial state (non-identity q or spin)
  char* block = nullptr;  // one page-locked allocation holding every array above
  int state = REQ_PENDING;
  int status = JDEM_OK;
  bool cancel = false;
  size_t bytes = 0;
};

void free_req(Req* r) {
  cudaFreeHost(r->block);
  delete r;
}

// Device staging arrays in the reference layout for one batch layout.
struct Staging {
  float *pos = nullptr, *vel = nullptr, *frc = nullptr, *rad = nullptr, *mass = nullptr;
  float *mat = nullptr;  // int32 material ids, moved as 4-byte words
  float *q = nullptr, *w = nullptr;
  float* tq = nullptr;  // torque of the last step (Cundall-Strack: the next half-kick reads it)
  long long cap = 0;
};

void free_staging(Staging& s) {
  for (float* p : {s.pos, s.vel, s.frc, s.rad, s.mass, s.mat, s.q, s.w, s.tq}) cudaFree(p);
  s = Staging{};
}

constexpr int kStagedArrays = 9;

}  // namespace

struct JdemServer {
  JdemServeConfig cfg{};
  JdemHandle* h = nullptr;
  std::mutex mtx;
  std::condition_variable cv;        // wakes the worker
  std::condition_variable done_cv;   // wakes drain()
  std::deque<Req*> pending;
  std::vector<Req*> active;
  std::unordered_map<int64_t, Req*> all;
  std::vector<int64_t> finished_unpolled;
  // released requests that may still sit in `active` until the next repack;
  // the worker frees them once they have left it (guarded by mtx)
  std::vector<Req*> graveyard;
  std::thread worker;
  bool stop = false;
  bool broken = false;  // the worker stopped on a host error: requests fail
  int64_t next_id = 1;
  Staging st[2];
  int cur = 0;            // staging holding the live batch layout
  bool cur_valid = false; // st[cur].pos/vel/frc hold the live batch's latest state
  long long* d_seg = nullptr;
  const float** d_src = nullptr;
  float** d_dst = nullptr;
  int* d_width = nullptr;
  size_t bytes_in_use = 0;
  int64_t unfinished = 0;  // submitted, not yet done / cancelled / failed (guarded by mtx)
  int64_t n_active = 0;    // admitted and not yet finished (guarded by mtx)
  JdemServeStats stats{};
  std::vector<float> young_eff;  // M * M pair constants of the force law
  std::vector<float> mat_props;  // Cundall-Strack: M * 4 per-material properties
  std::string err;

  int fail(int code, const std::string& m) {
    err = m;
    return code;
  }
  int ensure_staging(Staging& s, long long n);
  int repack(std::vector<Req*>& next);
  int finish(std::vector<Req*>& done);
  void loop();
  void run_epochs();
  void reap();
};

static int dmalloc(void** p, size_t bytes) {
  if (cudaMalloc(p, bytes ? bytes : 16) != cudaSuccess) {
    cudaGetLastError();
    return JDEM_ERR_OOM;
  }
  return JDEM_OK;
}

int JdemServer::ensure_staging(Staging& s, long long n) {
  if (n <= s.cap) return JDEM_OK;
  long long cap = std::max(n, s.cap + s.cap / 2);
  free_staging(s);
  int d = cfg.dim, ad = d == 3 ? 3 : 1;
  if (dmalloc((void**)&s.pos, 4 * cap * d) || dmalloc((void**)&s.vel, 4 * cap * d) ||
      dmalloc((void**)&s.frc, 4 * cap * d) || dmalloc((void**)&s.rad, 4 * cap) || dmalloc((void**)&s.mass, 4 * cap) ||
      dmalloc((void**)&s.mat, 4 * cap) || dmalloc((void**)&s.q, 16 * cap) || dmalloc((void**)&s.w, 4 * cap * ad) ||
      dmalloc((void**)&s.tq, 4 * cap * ad))
    return fail(JDEM_ERR_OOM, "serve: staging allocation failed");
  s.cap = cap;
  return JDEM_OK;
}

// Build the next batch layout in the spare staging buffers and rebind the
// handle: continuing requests are copied device-to-device from the live
// staging (refreshed from the handle first), newcomers from pinned host memory.
int JdemServer::repack(std::vector<Req*>& next) {
  cudaStream_t s = h->stream;
  long long P = 0;
  for (Req* r : next) P += r->desc.n;
  int nxt = cur ^ 1;
  int rc = ensure_staging(st[nxt], std::max(P, 1LL));
  if (rc) return rc;
  // offsets of continuing requests in the live layout
  std::unordered_map<int64_t, long long> old_off;
  {
    long long o = 0;
    for (Req* r : active) {
      old_off[r->id] = o;
      o += r->desc.n;
    }
  }
  bool any_cont = false;
  for (Req* r : next) any_cont |= old_off.count(r->id) > 0;
  if (any_cont && !cur_valid) {
    JdemHostState out{};
    out.pos_c = st[cur].pos;
    out.vel = st[cur].vel;
    out.force = st[cur].frc;
    out.q = st[cur].q;
    out.ang_vel = st[cur].w;
    out.torque = st[cur].tq;
    rc = h->download(&out, true);
    if (rc) return fail(rc, std::string("serve: download ") + h->err);
    cur_valid = true;
  }
  std::vector<long long> seg;
  std::vector<JdemSystemDesc> descs;
  std::vector<float> rmax, lo, hi;
  long long o = 0;
  const int d = cfg.dim, ad = d == 3 ? 3 : 1;
  bool rot = false;
  for (Req* r : next) {
    rot |= r->rot;
    auto it = old_off.find(r->id);
    if (it != old_off.end()) {
      seg.push_back(it->second);
      seg.push_back(o);
      seg.push_back(r->desc.n);
    } else {
      size_t n = (size_t)r->desc.n;
      if (n) {
        cudaMemcpyAsync(st[nxt].pos + o * d, r->h_pos, 4 * n * d, cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(st[nxt].vel + o * d, r->h_vel, 4 * n * d, cudaMemcpyHostToDevice, s);
        cudaMemsetAsync(st[nxt].frc + o * d, 0, 4 * n * d, s);
        cudaMemcpyAsync(st[nxt].rad + o, r->h_rad, 4 * n, cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(st[nxt].mass + o, r->h_mass, 4 * n, cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(st[nxt].mat + o, r->h_mat, 4 * n, cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(st[nxt].q + o * 4, r->h_q, 16 * n, cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(st[nxt].w + o * ad, r->h_w, 4 * n * ad, cudaMemcpyHostToDevice, s);
        cudaMemsetAsync(st[nxt].tq + o * ad, 0, 4 * n * ad, s);
      }
    }
    descs.push_back(r->desc);
    rmax.push_back(r->rmax);
    for (int a = 0; a < 3; ++a) {
      lo.push_back(r->lo[a]);
      hi.push_back(r->hi[a]);
    }
    o += r->desc.n;
  }
  int nseg = (int)(seg.size() / 3);
  if (nseg > 0) {
    // segment table and array pointers, copied with the stream (then synchronised)
    if (!d_seg) {
      if (dmalloc((void**)&d_src, sizeof(float*) * kStagedArrays) ||
          dmalloc((void**)&d_dst, sizeof(float*) * kStagedArrays) || dmalloc((void**)&d_width, sizeof(int) * kStagedArrays))
        return fail(JDEM_ERR_OOM, "serve: table allocation failed");
    }
    cudaFree(d_seg);
    d_seg = nullptr;
    if (dmalloc((void**)&d_seg, sizeof(long long) * seg.size())) return fail(JDEM_ERR_OOM, "serve: segment table");
    const float* src[kStagedArrays] = {st[cur].pos, st[cur].vel, st[cur].frc, st[cur].rad, st[cur].mass,
                                       st[cur].mat,  st[cur].q,   st[cur].w,   st[cur].tq};
    float* dst[kStagedArrays] = {st[nxt].pos, st[nxt].vel, st[nxt].frc, st[nxt].rad, st[nxt].mass,
                                 st[nxt].mat, st[nxt].q,   st[nxt].w,   st[nxt].tq};
    int width[kStagedArrays] = {d, d, d, 1, 1, 1, 4, ad, ad};
    cudaMemcpyAsync(d_seg, seg.data(), sizeof(long long) * seg.size(), cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(d_src, src, sizeof(src), cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(d_dst, dst, sizeof(dst), cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(d_width, width, sizeof(width), cudaMemcpyHostToDevice, s);
    launch_segcopy(d_seg, nseg, kStagedArrays, d_src, d_dst, d_width, s);
  }
  if (cudaStreamSynchronize(s) != cudaSuccess) return fail(JDEM_ERR_CUDA, "serve: repack copies failed");
  if (next.empty()) {
    active.clear();
    cur = nxt;
    cur_valid = false;
    return JDEM_OK;
  }
  rc = h->rebind(descs.data(), (int)descs.size());
  if (rc) return fail(rc, std::string("serve: rebind ") + h->err);
  rc = h->upload_resident(st[nxt].pos, st[nxt].vel, st[nxt].frc, st[nxt].rad, st[nxt].mass, rmax.data(), lo.data(),
                          hi.data(), (const int32_t*)st[nxt].mat, st[nxt].q, st[nxt].w, rot, st[nxt].tq);
  if (rc) return fail(rc, std::string("serve: upload ") + h->err);
  active = next;
  cur = nxt;
  cur_valid = true;  // st[cur] now equals the uploaded state
  stats.repacks += 1;
  return JDEM_OK;
}

// Copy the finished requests' state to their pinned host outputs.
int JdemServer::finish(std::vector<Req*>& done) {
  if (done.empty()) return JDEM_OK;
  cudaStream_t s = h->stream;
  JdemHostState out{};
  out.pos_c = st[cur].pos;
  out.vel = st[cur].vel;
  out.force = st[cur].frc;
  out.q = st[cur].q;
  out.ang_vel = st[cur].w;
  out.torque = st[cur].tq;
  int rc = h->download(&out, true);
  if (rc) return fail(rc, std::string("serve: download ") + h->err);
  cur_valid = true;
  long long o = 0;
  const int d = cfg.dim, ad = d == 3 ? 3 : 1;
  for (Req* r : active) {
    if (std::find(done.begin(), done.end(), r) != done.end() && r->desc.n) {
      size_t n = (size_t)r->desc.n;
      cudaMemcpyAsync(r->o_pos, st[cur].pos + o * d, 4 * n * d, cudaMemcpyDeviceToHost, s);
      cudaMemcpyAsync(r->o_vel, st[cur].vel + o * d, 4 * n * d, cudaMemcpyDeviceToHost, s);
      cudaMemcpyAsync(r->o_frc, st[cur].frc + o * d, 4 * n * d, cudaMemcpyDeviceToHost, s);
      cudaMemcpyAsync(r->o_q, st[cur].q + o * 4, 16 * n, cudaMemcpyDeviceToHost, s);
      cudaMemcpyAsync(r->o_w, st[cur].w + o * ad, 4 * n * ad, cudaMemcpyDeviceToHost, s);
    }
    o += r->desc.n;
  }
  if (cudaStreamSynchronize(s) != cudaSuccess) return fail(JDEM_ERR_CUDA, "serve: result copies failed");
  return JDEM_OK;
}

// Free released requests that are no longer part of the live layout (caller holds mtx).
void JdemServer::reap() {
  size_t k = 0;
  for (Req* r : graveyard) {
    if (std::find(active.begin(), active.end(), r) != active.end())
      graveyard[k++] = r;
    else
      free_req(r);
  }
  graveyard.resize(k);
}

// The worker thread.  A C++ exception (a failed host allocation) ends the
// loop: every pending and live request fails with JDEM_ERR_OOM, waiters are
// woken, and later submissions are refused.
void JdemServer::loop() {
  try {
    run_epochs();
  } catch (...) {
    std::lock_guard<std::mutex> lk(mtx);
    broken = true;
    err = "serve: host allocation failed in the worker";
    double t = now_s();
    for (auto& kv : all) {
      Req* r = kv.second;
      if (r->state != REQ_PENDING && r->state != REQ_ACTIVE) continue;
      if (r->state == REQ_ACTIVE) {
        bytes_in_use -= r->bytes;
        n_active -= 1;
      }
      r->state = REQ_FAILED;
      r->status = JDEM_ERR_OOM;
      r->t_done = t;
      unfinished -= 1;
      finished_unpolled.push_back(r->id);
    }
    pending.clear();
    active.clear();
    stats.failures += 1;
    done_cv.notify_all();
  }
}

void JdemServer::run_epochs() {
  cudaSetDevice(cfg.device);
  for (;;) {
    std::vector<Req*> next, done, dropped;
    bool changed = false;
    {
      std::unique_lock<std::mutex> lk(mtx);
      cv.wait_for(lk, std::chrono::milliseconds(1), [&] { return stop || !pending.empty() || !active.empty(); });
      if (stop) return;
      reap();
      // cancellations of active requests take effect at this epoch boundary
      // `active` is the live batch layout; requests that finished in the last
      // epoch are still in it and leave it with this repack
      for (Req* r : active) {
        if (r->state != REQ_ACTIVE) {
          changed = true;
        } else if (r->cancel) {
          dropped.push_back(r);
          changed = true;
        } else {
          next.push_back(r);
        }
      }
      long long parts = 0;
      for (Req* r : next) parts += r->desc.n;
      while (!pending.empty()) {
        Req* r = pending.front();
        if (r->cancel) {
          pending.pop_front();
          dropped.push_back(r);
          continue;
        }
        bool room = (int)next.size() < cfg.max_active &&
                    (next.empty() || parts + r->desc.n <= cfg.target_particles) &&
                    (double)(bytes_in_use + r->bytes) <= cfg.hbm_budget_bytes;
        if (!room) break;
        pending.pop_front();
        r->state = REQ_ACTIVE;
        r->t_admit = now_s();
        n_active += 1;
        bytes_in_use += r->bytes;
        parts += r->desc.n;
        next.push_back(r);
        changed = true;
      }
      for (Req* r : dropped) {
        if (r->state == REQ_ACTIVE) {
          bytes_in_use -= r->bytes;
          n_active -= 1;
        }
        unfinished -= 1;
        r->state = REQ_CANCELLED;
        r->t_done = now_s();
        finished_unpolled.push_back(r->id);
      }
      if (!dropped.empty()) done_cv.notify_all();
      if (next.empty() && !changed) continue;
      stats.max_active = std::max<int64_t>(stats.max_active, (int64_t)next.size());
    }
    int rc = JDEM_OK;
    if (changed || next.size() != active.size()) rc = repack(next);
    long long K = 0;
    if (rc == JDEM_OK && !active.empty()) {
      K = std::max<long long>(1, cfg.chunk_steps);
      for (Req* r : active) K = std::min<long long>(K, r->steps_total - r->steps_done);
      if (K > 0) {
        rc = h->step_async(K);
        if (rc == JDEM_OK) rc = h->sync_status();
        cur_valid = false;
      }
      if (rc == JDEM_OK) {
        long long parts = 0;
        for (Req* r : active) {
          r->steps_done += K;
          parts += r->desc.n;
          if (r->steps_done >= r->steps_total) done.push_back(r);
        }
        stats.epochs += 1;
        stats.particle_steps += parts * K;
        if (!done.empty()) rc = finish(done);
      }
    }
    std::lock_guard<std::mutex> lk(mtx);
    reap();
    if (rc != JDEM_OK) {
      // the whole batch failed (device status or CUDA error): fail its live requests,
      // both the current layout and the newcomers a failed repack did not place
      std::vector<Req*> live(active);
      for (Req* r : next)
        if (std::find(live.begin(), live.end(), r) == live.end()) live.push_back(r);
      for (Req* r : live) {
        if (r->state != REQ_ACTIVE) continue;
        r->state = REQ_FAILED;
        r->status = rc;
        r->t_done = now_s();
        bytes_in_use -= r->bytes;
        n_active -= 1;
        unfinished -= 1;
        finished_unpolled.push_back(r->id);
      }
      active.clear();
      cur_valid = false;
      stats.failures += 1;
      done_cv.notify_all();
      continue;
    }
    double t = now_s();
    for (Req* r : done) {
      r->state = REQ_DONE;
      r->t_done = t;
      bytes_in_use -= r->bytes;
      n_active -= 1;
      unfinished -= 1;
      finished_unpolled.push_back(r->id);
      stats.completed += 1;
    }
    if (!done.empty()) {
      done_cv.notify_all();
    }
  }
}

extern "C" {

int jdem_serve_create(const JdemServeConfig* cfg, JdemServer** out) {
  if (!cfg || !out || (cfg->dim != 2 && cfg->dim != 3)) return JDEM_ERR_BAD_ARG;
  *out = nullptr;
  JdemServer* s = new (std::nothrow) JdemServer();
  if (!s) return JDEM_ERR_OOM;
  s->cfg = *cfg;
  if (s->cfg.chunk_steps <= 0) s->cfg.chunk_steps = 50;
  if (s->cfg.max_active <= 0) s->cfg.max_active = 1024;
  if (s->cfg.target_particles <= 0) s->cfg.target_particles = 4 << 20;
  if (!(s->cfg.hbm_budget_bytes > 0)) s->cfg.hbm_budget_bytes = 150e9;
  // the batch handle starts with one placeholder system and is rebound per epoch
  JdemSystemDesc d{};
  d.n = 0;
  d.domain = JDEM_DOMAIN_PERIODIC;
  d.linear_integrator = JDEM_LIN_VERLET;
  d.dt = 1e-3f;
  for (int a = 0; a < 3; ++a) d.box_size[a] = 1.0f;
  const bool cs = cfg->force_law == JDEM_FORCE_CUNDALL_STRACK;
  if (cfg->force_law != JDEM_FORCE_SPRING && cfg->force_law != JDEM_FORCE_HERTZ && !cs) {
    delete s;
    return JDEM_ERR_UNSUPPORTED;
  }
  if (cfg->n_materials < 0 || (cfg->n_materials > 0 && !cfg->young_eff) ||
      (cs && (cfg->n_materials <= 0 || !cfg->material_props))) {
    delete s;
    return JDEM_ERR_BAD_ARG;  // Cundall-Strack takes its beta and per-material tables explicitly
  }
  float young = cfg->young > 0 ? cfg->young : 1e3f;
  const int M = cfg->n_materials > 0 ? cfg->n_materials : 1;
  try {
    if (cfg->n_materials > 0) s->young_eff.assign(cfg->young_eff, cfg->young_eff + (size_t)M * M);
    else s->young_eff.assign(1, young);
    if (cs) s->mat_props.assign(cfg->material_props, cfg->material_props + (size_t)M * 4);
  } catch (...) {
    delete s;
    return JDEM_ERR_OOM;
  }
  s->cfg.n_materials = M;
  s->cfg.young_eff = nullptr;  // the server keeps its own copies
  s->cfg.material_props = nullptr;
  JdemConfig ec{};
  ec.dim = cfg->dim;
  ec.n_systems = 1;
  ec.systems = &d;
  ec.skin = cfg->skin;
  ec.n_materials = M;
  ec.young_eff = s->young_eff.data();
  ec.force_law = cfg->force_law;
  ec.material_props = cs ? s->mat_props.data() : nullptr;
  ec.chunk_steps = s->cfg.chunk_steps;
  ec.device = cfg->device;
  ec.graph_mode = 2;  // the batch changes between epochs: direct launches
  int rc = jdem_create(&ec, &s->h);
  if (rc) {
    delete s;
    return rc;
  }
  try {
    s->worker = std::thread([s] { s->loop(); });
  } catch (...) {
    jdem_destroy(s->h);
    delete s;
    return JDEM_ERR_OOM;
  }
  *out = s;
  return JDEM_OK;
}

int jdem_serve_submit(JdemServer* s, const JdemRequest* req, int64_t* id) {
  if (!s || !req || !req->pos || !req->vel || !req->rad || !req->mass) return JDEM_ERR_BAD_ARG;
  if (req->system.n < 0 || req->steps < 0) return JDEM_ERR_BAD_ARG;
  const int d = s->cfg.dim;
  const size_t n = (size_t)req->system.n;
  Req* r = new (std::nothrow) Req();
  if (!r) return JDEM_ERR_OOM;
  r->desc = req->system;
  r->steps_total = req->steps;
  r->t_submit = now_s();
  // validate on the host (a request with bad input never joins a batch)
  for (int a = 0; a < 3; ++a) {
    r->lo[a] = 3.4e38f;
    r->hi[a] = -3.4e38f;
  }
  const int ad = d == 3 ? 3 : 1;
  for (size_t i = 0; i < n; ++i) {
    float rr = req->rad[i];
    if (!(rr >= 0.0f) || !std::isfinite(rr) || !(req->mass[i] > 0.0f) ||
        (req->mat_id && (req->mat_id[i] < 0 || req->mat_id[i] >= s->cfg.n_materials))) {
      delete r;
      return JDEM_ERR_BAD_ARG;
    }
    if (req->system.rotation_integrator != JDEM_ROT_NONE) {
      // a rotation integrator has work only for a non-identity orientation or a spin
      if (req->q)
        r->rot |= req->q[i * 4] != 1.0f || req->q[i * 4 + 1] != 0.0f || req->q[i * 4 + 2] != 0.0f ||
                  req->q[i * 4 + 3] != 0.0f;
      if (req->ang_vel)
        for (int a = 0; a < ad; ++a) r->rot |= req->ang_vel[i * ad + a] != 0.0f;
    }
    if (req->ang_vel)
      for (int a = 0; a < ad; ++a)
        if (!std::isfinite(req->ang_vel[i * ad + a])) {
          delete r;
          return JDEM_ERR_NONFINITE;
        }
    r->rmax = std::max(r->rmax, rr);
    for (int a = 0; a < d; ++a) {
      float x = req->pos[i * d + a];
      if (!std::isfinite(x) || !std::isfinite(req->vel[i * d + a])) {
        delete r;
        return JDEM_ERR_NONFINITE;
      }
      r->lo[a] = std::min(r->lo[a], x - rr);
      r->hi[a] = std::max(r->hi[a], x + rr);
    }
  }
  if (n == 0)
    for (int a = 0; a < 3; ++a) {
      r->lo[a] = 0.0f;
      r->hi[a] = 1.0f;
    }
  // pinned copies of the inputs and room for the outputs
  // page-locked copies of the inputs and room for the outputs, carved from one
  // allocation (page-locking is slow: one call per request, not one per array)
  auto up = [](size_t b) { return (b + 255) / 256 * 256; };
  size_t vec = up(4 * std::max<size_t>(n, 1) * d), sca = up(4 * std::max<size_t>(n, 1));
  size_t q4 = up(16 * std::max<size_t>(n, 1)), wv = up(4 * std::max<size_t>(n, 1) * ad);
  if (cudaMallocHost((void**)&r->block, 5 * vec + 3 * sca + 2 * q4 + 2 * wv) != cudaSuccess) {
    cudaGetLastError();
    r->block = nullptr;
    free_req(r);
    return JDEM_ERR_OOM;
  }
  {
    char* c = r->block;
    auto take = [&](size_t b) {
      char* q = c;
      c += b;
      return q;
    };
    r->h_pos = (float*)take(vec);
    r->h_vel = (float*)take(vec);
    r->o_pos = (float*)take(vec);
    r->o_vel = (float*)take(vec);
    r->o_frc = (float*)take(vec);
    r->h_rad = (float*)take(sca);
    r->h_mass = (float*)take(sca);
    r->h_mat = (int32_t*)take(sca);
    r->h_q = (float*)take(q4);
    r->o_q = (float*)take(q4);
    r->h_w = (float*)take(wv);
    r->o_w = (float*)take(wv);
  }
  std::memcpy(r->h_pos, req->pos, 4 * n * d);
  std::memcpy(r->h_vel, req->vel, 4 * n * d);
  std::memcpy(r->h_rad, req->rad, 4 * n);
  std::memcpy(r->h_mass, req->mass, 4 * n);
  if (req->mat_id) std::memcpy(r->h_mat, req->mat_id, 4 * n);
  else std::memset(r->h_mat, 0, 4 * n);
  if (req->q) {
    std::memcpy(r->h_q, req->q, 16 * n);
  } else {
    for (size_t i = 0; i < n; ++i) {
      r->h_q[i * 4] = 1.0f;
      r->h_q[i * 4 + 1] = r->h_q[i * 4 + 2] = r->h_q[i * 4 + 3] = 0.0f;
    }
  }
  if (req->ang_vel) std::memcpy(r->h_w, req->ang_vel, 4 * n * ad);
  else std::memset(r->h_w, 0, 4 * n * ad);
  // resident footprint: slot arrays (both copies), staging (both layouts, with the
  // material id, rotational state and torque), both Verlet lists
  r->bytes = n * (size_t)(2 * 96 + 2 * 4 * (3 * d + 3 + 4 + 2 * ad) + 8 * 64);
  if ((double)r->bytes > s->cfg.hbm_budget_bytes) {
    // could never be admitted: reject instead of blocking the queue
    free_req(r);
    return JDEM_ERR_CAPACITY_OVERFLOW;
  }
  {
    std::lock_guard<std::mutex> lk(s->mtx);
    if (s->broken) {
      free_req(r);
      return JDEM_ERR_CUDA;
    }
    r->id = s->next_id++;
    try {
      s->all[r->id] = r;
      s->pending.push_back(r);
    } catch (...) {
      s->all.erase(r->id);
      free_req(r);
      return JDEM_ERR_OOM;
    }
    s->unfinished += 1;
    s->stats.submitted += 1;
  }
  s->cv.notify_one();
  if (id) *id = r->id;
  return JDEM_OK;
}

int jdem_serve_cancel(JdemServer* s, int64_t id) {
  if (!s) return JDEM_ERR_BAD_ARG;
  std::lock_guard<std::mutex> lk(s->mtx);
  auto it = s->all.find(id);
  if (it == s->all.end()) return JDEM_ERR_BAD_ARG;
  if (it->second->state == REQ_PENDING || it->second->state == REQ_ACTIVE) it->second->cancel = true;
  s->cv.notify_one();
  return JDEM_OK;
}

int jdem_serve_poll(JdemServer* s, int64_t* ids, int32_t cap, int32_t* count) {
  if (!s || !count) return JDEM_ERR_BAD_ARG;
  std::lock_guard<std::mutex> lk(s->mtx);
  int32_t n = (int32_t)std::min<size_t>((size_t)std::max(cap, 0), s->finished_unpolled.size());
  for (int32_t k = 0; k < n; ++k) ids[k] = s->finished_unpolled[(size_t)k];
  s->finished_unpolled.erase(s->finished_unpolled.begin(), s->finished_unpolled.begin() + n);
  *count = n;
  return JDEM_OK;
}

int jdem_serve_result(JdemServer* s, int64_t id, float* pos, float* vel, float* force, JdemRequestInfo* info) {
  if (!s) return JDEM_ERR_BAD_ARG;
  std::lock_guard<std::mutex> lk(s->mtx);
  auto it = s->all.find(id);
  if (it == s->all.end()) return JDEM_ERR_BAD_ARG;
  Req* r = it->second;
  if (info) {
    info->state = r->state;
    info->status = r->status;
    info->n = r->desc.n;
    info->steps = r->steps_done;
    info->submit_s = r->t_submit;
    info->admit_s = r->t_admit;
    info->done_s = r->t_done;
  }
  if (r->state != REQ_DONE) return r->state == REQ_FAILED ? r->status : (pos || vel || force ? JDEM_ERR_NOT_READY : JDEM_OK);
  size_t vec = 4 * (size_t)r->desc.n * s->cfg.dim;
  if (pos) std::memcpy(pos, r->o_pos, vec);
  if (vel) std::memcpy(vel, r->o_vel, vec);
  if (force) std::memcpy(force, r->o_frc, vec);
  return JDEM_OK;
}

int jdem_serve_result_state(JdemServer* s, int64_t id, JdemHostState* out, JdemRequestInfo* info) {
  if (!s) return JDEM_ERR_BAD_ARG;
  const bool want = out && (out->pos_c || out->vel || out->force || out->q || out->ang_vel || out->torque);
  int rc = jdem_serve_result(s, id, want ? out->pos_c : nullptr, want ? out->vel : nullptr,
                             want ? out->force : nullptr, info);
  if (rc || !want) return rc;
  std::lock_guard<std::mutex> lk(s->mtx);
  auto it = s->all.find(id);
  if (it == s->all.end()) return JDEM_ERR_BAD_ARG;
  Req* r = it->second;
  const size_t n = (size_t)r->desc.n;
  const int ad = s->cfg.dim == 3 ? 3 : 1;
  if (out->q) std::memcpy(out->q, r->o_q, 16 * n);
  if (out->ang_vel) std::memcpy(out->ang_vel, r->o_w, 4 * n * ad);
  if (out->torque) std::memset(out->torque, 0, 4 * n * ad);  // smooth spheres: no contact torque
  return JDEM_OK;
}

int jdem_serve_release(JdemServer* s, int64_t id) {
  if (!s) return JDEM_ERR_BAD_ARG;
  std::lock_guard<std::mutex> lk(s->mtx);
  auto it = s->all.find(id);
  if (it == s->all.end()) return JDEM_ERR_BAD_ARG;
  Req* r = it->second;
  if (r->state == REQ_PENDING || r->state == REQ_ACTIVE) return JDEM_ERR_NOT_READY;
  try {
    s->graveyard.push_back(r);
  } catch (...) {
    return JDEM_ERR_OOM;  // still registered: release can be retried
  }
  s->all.erase(it);
  s->cv.notify_one();
  return JDEM_OK;
}

int jdem_serve_drain(JdemServer* s, double timeout_s) {
  if (!s) return JDEM_ERR_BAD_ARG;
  std::unique_lock<std::mutex> lk(s->mtx);
  // the worker moves a request from `pending` into its batch outside the lock, so
  // idleness is the count of unfinished requests, not the queues' contents
  auto idle = [&] { return s->unfinished == 0; };
  if (timeout_s > 0) {
    if (!s->done_cv.wait_for(lk, std::chrono::duration<double>(timeout_s), idle)) return JDEM_ERR_TIMEOUT;
  } else {
    s->done_cv.wait(lk, idle);
  }
  return JDEM_OK;
}

int jdem_serve_stats(JdemServer* s, JdemServeStats* out) {
  if (!s || !out) return JDEM_ERR_BAD_ARG;
  std::lock_guard<std::mutex> lk(s->mtx);
  *out = s->stats;
  out->pending = (int64_t)s->pending.size();
  out->active = s->n_active;
  out->bytes_in_use = (int64_t)s->bytes_in_use;
  return JDEM_OK;
}

const char* jdem_serve_last_error(JdemServer* s) { return s ? s->err.c_str() : "null server"; }

int jdem_serve_destroy(JdemServer* s) {
  if (!s) return JDEM_ERR_BAD_ARG;
  {
    std::lock_guard<std::mutex> lk(s->mtx);
    s->stop = true;
  }
  s->cv.notify_all();
  if (s->worker.joinable()) s->worker.join();
  for (auto& kv : s->all) free_req(kv.second);
  for (Req* r : s->graveyard) free_req(r);
  for (auto& st : s->st) free_staging(st);
  cudaFree(s->d_seg);
  cudaFree(s->d_src);
  cudaFree(s->d_dst);
  cudaFree(s->d_width);
  jdem_destroy(s->h);
  delete s;
  return JDEM_OK;
}

}  // extern "C"
