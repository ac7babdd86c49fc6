// Trajectory frames of System.trajectory_rollout (jaxdem/system.py:606-699,
// scan body system.py:99-120) with the default save_fn.
//
// The strides run on the handle's stream exactly as jdem_step_async runs
// them.  After each stride the selected fields are unpacked from slot order
// into the caller's particle order, into one slot of a small device ring; a
// second stream copies the slot to the host while the next stride's steps
// run.  The ring slot is reused only after its copy has finished (an event
// the compute stream waits on).
//
// Pageable destinations.  There is no page-locked staging: on a coherent host
// (Grace) the copy engine writes resident pageable memory at several times
// the rate of a host-side memcpy out of a staging buffer.  What is slow is a
// fresh allocation: the kernel zero-fills each page at its first touch, at
// one core's memset speed.  Worker threads therefore touch every frame's
// destination pages ahead of that frame's copy, in parallel with the steps.
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <cstring>
#include <memory>
#include <string>
#include <thread>
#include <vector>

#include "../../include/jdem_gb300.h"
#include "jdem_device.cuh"
#include "jdem_internal.h"
#include "jdem_kernels.h"

using namespace jdem;

namespace {

constexpr int kDefaultRing = 3;
constexpr int kMaxRing = 16;

size_t round_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

float ord_to_float(unsigned int u) {
  unsigned int v = (u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u;
  float f;
  std::memcpy(&f, &v, 4);
  return f;
}

// one saved field: caller destination (frame 0), bytes per frame, offset in a
// ring slot
struct FrameField {
  float* dst;
  size_t bytes;
  size_t off;
};

bool page_locked(const void* p) {
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeHost;
}

// Touches the pages of every pageable destination, frame by frame, on a few
// worker threads; wait(t) returns once frame t's pages are resident.
class Prefault {
 public:
  Prefault(const FrameField* f, int nf, long long T) : T_(T), done_(new std::atomic<int>[(size_t)T]) {
    for (int k = 0; k < nf; ++k)
      if (f[k].dst && f[k].bytes && !page_locked(f[k].dst)) regions_.push_back(f[k]);
    for (long long t = 0; t < T; ++t) done_[t].store(regions_.empty() ? 1 : 0, std::memory_order_relaxed);
    if (regions_.empty()) return;
    long ps = sysconf(_SC_PAGESIZE);
    page_ = ps > 0 ? (size_t)ps : 4096;
    unsigned hw = std::thread::hardware_concurrency();
    int n = (int)std::min<long long>(T, std::max(1u, std::min(8u, hw / 2)));
    try {
      for (int w = 0; w < n; ++w) workers_.emplace_back([this, w, n] { run(w, n); });
    } catch (...) {
      // no threads: stop the ones started and copy without the pre-touch
      stop_.store(true);
      for (auto& th : workers_) th.join();
      workers_.clear();
      for (long long t = 0; t < T; ++t) done_[t].store(1, std::memory_order_relaxed);
    }
  }
  ~Prefault() {
    stop_.store(true);
    for (auto& th : workers_) th.join();
  }
  void wait(long long t) const {
    while (!done_[t].load(std::memory_order_acquire)) std::this_thread::yield();
  }

 private:
  void run(int w, int n) {
    for (long long t = w; t < T_ && !stop_.load(std::memory_order_relaxed); t += n) {
      for (const FrameField& r : regions_) {
        volatile char* p = (volatile char*)r.dst + (size_t)t * r.bytes;
        for (size_t o = 0; o < r.bytes; o += page_) p[o] = 0;
        p[r.bytes - 1] = 0;
      }
      done_[t].store(1, std::memory_order_release);
    }
  }
  long long T_;
  size_t page_ = 4096;
  std::vector<FrameField> regions_;
  std::unique_ptr<std::atomic<int>[]> done_;
  std::vector<std::thread> workers_;
  std::atomic<bool> stop_{false};
};

}  // namespace

void JdemHandle::free_frames() {
  if (copy_stream) {
    cudaStreamSynchronize(copy_stream);
    cudaStreamDestroy(copy_stream);
  }
  copy_stream = nullptr;
  for (cudaEvent_t e : ev_frame) cudaEventDestroy(e);
  ev_frame.clear();
  if (d_frames) dfree(d_frames);
  d_frames = nullptr;
  d_frames_bytes = 0;
}

int JdemHandle::rollout(const int64_t* strides, long long T, const JdemFrames* out) {
  if (!uploaded) return fail(JDEM_ERR_NOT_READY, "rollout before upload");
  if (!out || T < 0 || (T > 0 && !strides)) return fail(JDEM_ERR_BAD_ARG, "rollout: bad arguments");
  for (long long t = 0; t < T; ++t)
    if (strides[t] < 0) return fail(JDEM_ERR_BAD_ARG, "rollout: negative stride");
  if (out->ring < 0) return fail(JDEM_ERR_BAD_ARG, "rollout: negative ring");
  if (T == 0) return JDEM_OK;
  JDEM_CUDA_TRY(this, cudaSetDevice(dev));
  int rc;
  // the frame boxes start from the current domain frame
  if (bbox_pending && (rc = sync_status()) && rc != JDEM_ERR_NONFINITE) return rc;

  const size_t N = (size_t)P;
  const int ad = dim == 3 ? 3 : 1;
  // fields in ring-slot order: pos_c, vel, force (unpacked), q, ang_vel, torque (copied)
  FrameField f[6] = {{out->pos_c, N * dim * 4, 0}, {out->vel, N * dim * 4, 0}, {out->force, N * dim * 4, 0},
                     {out->q, N * 16, 0},          {out->ang_vel, N * ad * 4, 0}, {out->torque, N * ad * 4, 0}};
  const float* rot_src[3] = {d_q, d_w, d_tq};
  size_t slot = 0;
  for (auto& x : f)
    if (x.dst) {
      x.off = slot;
      slot += round_up(x.bytes, 256);
    }
  const bool device_dst = out->device_ptrs != 0;
  const bool want_box = out->box || out->anchor;
  const bool rec_bbox = want_box && any_free && N > 0;

  // raw bounding-box words of every frame (free domains), read once at the end
  unsigned int* d_bbw = nullptr;
  if (rec_bbox && (rc = dalloc((void**)&d_bbw, sizeof(unsigned int) * 6 * (size_t)S * (size_t)T))) return rc;
  std::vector<char> fresh((size_t)T, 0);

  // host destinations: a ring of device slots drained by the copy stream
  int R = 0;
  if (!device_dst && slot > 0 && N > 0) {
    R = out->ring > 0 ? std::min(out->ring, kMaxRing) : kDefaultRing;
    R = (int)std::min<long long>(R, T);
    size_t need = slot * (size_t)R;
    if (need > d_frames_bytes) {
      if (d_frames) dfree(d_frames);
      d_frames = nullptr;
      d_frames_bytes = 0;
      if ((rc = dalloc((void**)&d_frames, need))) {
        dfree(d_bbw);
        return rc;
      }
      d_frames_bytes = need;
    }
    if (!copy_stream) JDEM_CUDA_TRY(this, cudaStreamCreateWithFlags(&copy_stream, cudaStreamNonBlocking));
    while ((int)ev_frame.size() < 2 * R) {
      cudaEvent_t e;
      JDEM_CUDA_TRY(this, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
      ev_frame.push_back(e);
    }
  }

  std::unique_ptr<Prefault> prefault;
  if (R > 0) prefault.reset(new Prefault(f, 6, T));

  // on an error, wait for every copy already queued before returning: the
  // copy engine must not write into caller memory after this call ends
  auto stop = [&](int code) {
    cudaStreamSynchronize(stream);
    if (copy_stream) cudaStreamSynchronize(copy_stream);
    if (d_bbw) dfree(d_bbw);
    return code;
  };
  for (long long t = 0; t < T; ++t) {
    if ((rc = step_async(strides[t]))) return stop(rc);
    if (rec_bbox && strides[t] > 0) {
      cudaError_t e = cudaMemcpyAsync(d_bbw + (size_t)t * 6 * S, b.bbox, sizeof(unsigned int) * 6 * (size_t)S,
                                      cudaMemcpyDeviceToDevice, stream);
      if (e != cudaSuccess) return stop(fail(JDEM_ERR_CUDA, std::string("rollout box: ") + cudaGetErrorString(e)));
      fresh[(size_t)t] = 1;
    }
    if (slot == 0 || N == 0) continue;
    if (device_dst) {
      // frames stay in HBM: unpack straight into frame t
      float* dp[6];
      for (int k = 0; k < 6; ++k) dp[k] = f[k].dst ? (float*)((char*)f[k].dst + (size_t)t * f[k].bytes) : nullptr;
      if (b.NC) {
        // rigid clumps: every field from the clumps' state
        launch_rb_unpack(dim, b, dp[0], dp[1], dp[2], (float4*)dp[3], dp[4], dp[5], false, stream);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return stop(fail(JDEM_ERR_CUDA, std::string("rollout unpack: ") + cudaGetErrorString(e)));
        continue;
      }
      if (dp[0] || dp[1] || dp[2]) launch_unpack(dim, b, dp[0], dp[1], dp[2], stream);
      for (int k = 3; k < 6; ++k)
        if (f[k].dst) {
          cudaError_t e = cudaMemcpyAsync((char*)f[k].dst + (size_t)t * f[k].bytes, rot_src[k - 3], f[k].bytes,
                                          cudaMemcpyDeviceToDevice, stream);
          if (e != cudaSuccess) return stop(fail(JDEM_ERR_CUDA, std::string("rollout: ") + cudaGetErrorString(e)));
        }
      cudaError_t e = cudaGetLastError();
      if (e != cudaSuccess) return stop(fail(JDEM_ERR_CUDA, std::string("rollout unpack: ") + cudaGetErrorString(e)));
      continue;
    }
    const int r = (int)(t % R);
    cudaEvent_t ev_unpacked = ev_frame[2 * r], ev_copied = ev_frame[2 * r + 1];
    if (t >= R) {
      // the slot's previous frame: its copy must end before the slot is rewritten
      cudaError_t e = cudaStreamWaitEvent(stream, ev_copied, 0);
      if (e != cudaSuccess) return stop(fail(JDEM_ERR_CUDA, std::string("rollout: ") + cudaGetErrorString(e)));
    }
    char* ds = d_frames + (size_t)r * slot;
    float* sp_[6];
    for (int k = 0; k < 6; ++k) sp_[k] = f[k].dst ? (float*)(ds + f[k].off) : nullptr;
    cudaError_t e;
    if (b.NC) {
      launch_rb_unpack(dim, b, sp_[0], sp_[1], sp_[2], (float4*)sp_[3], sp_[4], sp_[5], false, stream);
      e = cudaGetLastError();
    } else {
      launch_unpack(dim, b, sp_[0], sp_[1], sp_[2], stream);
      e = cudaGetLastError();
      for (int k = 3; k < 6 && e == cudaSuccess; ++k)
        if (f[k].dst) e = cudaMemcpyAsync(ds + f[k].off, rot_src[k - 3], f[k].bytes, cudaMemcpyDeviceToDevice, stream);
    }
    if (e == cudaSuccess) e = cudaEventRecord(ev_unpacked, stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(copy_stream, ev_unpacked, 0);
    // page-locked destinations are written by the copy engine while the host
    // goes on; for pageable ones the copy returns once the frame has landed
    prefault->wait(t);
    for (int k = 0; k < 6 && e == cudaSuccess; ++k)
      if (f[k].dst)
        e = cudaMemcpyAsync((char*)f[k].dst + (size_t)t * f[k].bytes, ds + f[k].off, f[k].bytes,
                            cudaMemcpyDeviceToHost, copy_stream);
    if (e == cudaSuccess) e = cudaEventRecord(ev_copied, copy_stream);
    if (e != cudaSuccess) return stop(fail(JDEM_ERR_CUDA, std::string("rollout frame: ") + cudaGetErrorString(e)));
  }

  // frame boxes: free systems from the recorded words, others constant
  std::vector<unsigned int> words;
  if (rec_bbox) {
    words.resize((size_t)T * 6 * S);
    cudaError_t e = cudaMemcpyAsync(words.data(), d_bbw, words.size() * 4, cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) return stop(fail(JDEM_ERR_CUDA, std::string("rollout box: ") + cudaGetErrorString(e)));
  }
  if (copy_stream) {
    cudaError_t e = cudaStreamSynchronize(copy_stream);
    if (e != cudaSuccess) return stop(fail(JDEM_ERR_CUDA, std::string("rollout copy: ") + cudaGetErrorString(e)));
  }
  if (d_bbw) dfree(d_bbw);
  if (want_box) {
    std::vector<float> box(cur_box), anc(cur_anchor);
    for (long long t = 0; t < T; ++t) {
      if (rec_bbox && fresh[(size_t)t])
        for (int s = 0; s < S; ++s) {
          if (desc[s].domain != DOM_FREE || desc[s].n == 0) continue;
          const unsigned int* w = &words[((size_t)t * S + s) * 6];
          for (int a = 0; a < dim; ++a) {
            float lo = ord_to_float(w[a]), hi = ord_to_float(w[3 + a]);
            box[(size_t)s * 3 + a] = hi - lo;
            anc[(size_t)s * 3 + a] = lo;
          }
        }
      if (out->box) std::memcpy(out->box + (size_t)t * 3 * S, box.data(), sizeof(float) * 3 * S);
      if (out->anchor) std::memcpy(out->anchor + (size_t)t * 3 * S, anc.data(), sizeof(float) * 3 * S);
    }
  }
  return sync_status();
}

extern "C" int jdem_rollout(JdemHandle* h, const int64_t* strides, int64_t n_frames, const JdemFrames* out) {
  if (!h) return JDEM_ERR_BAD_ARG;
  return jdem_guard(&h->err, [&] { return h->rollout(strides, (long long)n_frames, out); });
}
