// jdem_compute_force_noalloc: contact forces of one sphere system from
// caller-owned device buffers, with no device allocation at all.
//
// Who needs this: callers that are not allowed to call cudaMalloc while
// they run -- an XLA FFI custom-call handler (XLA owns the device memory
// pool and preallocates most of the GPU, so an allocation behind its back can
// fail or fragment the pool), code executing inside another framework's
// memory budget, or a caller that must not synchronise the device (cudaFree
// synchronises).  They pass inputs and outputs; the scratch this kernel
// needs (cell counts, cell starts, keys, ranks, the cell-ordered index list)
// lives in g_noalloc_scratch below, a fixed-size array that every GPU loading
// the library holds until the process exits.
//
// Limits: n <= JDEM_NOALLOC_MAX_PARTICLES; the binning grid is coarsened on
// the device until it fits JDEM_NOALLOC_MAX_CELLS cells (any cell at least as
// wide as the contact range finds the same contacts).  Larger inputs are
// rejected with JDEM_ERR_CAPACITY_OVERFLOW before any device work.
//
// Every call shares the one scratch array and leaves its contents behind;
// the counters that must start at zero are cleared by the call itself.  Calls
// whose device work overlaps (on different streams, or from different host
// threads) race on the scratch: serialise them on one stream.
//
// Set-up: the first call on each device, with that device current, looks up
// the array's device address with cudaGetSymbolAddress and caches it (the
// host-side symbol is only a stand-in and must never be passed to a kernel).
// Make that first call before any stream capture.  The cache is keyed on the
// device's current context: after cudaDeviceReset (a new primary context, the
// module loaded again, possibly elsewhere) the next call looks the address up
// again, and that call too must come before any stream capture.
//
// Order inside a cell is ascending particle index, so the forces are the same
// bit for bit from call to call: cells of at most kSmallCell particles are
// insertion-sorted by one thread; larger cells (the coarsened grids of dilute
// or clustered inputs) are ordered by a block that marks the members in a
// bitmap of all particle indices and writes the marked indices out in order,
// O(n / 32 + m) per cell instead of O(m^2).
#include <cuda.h>

#include <cstdio>
#include <mutex>

#include "../../include/jdem_gb300.h"
#include "jdem_device.cuh"

using namespace jdem;

namespace {

constexpr int kMaxP = JDEM_NOALLOC_MAX_PARTICLES;
constexpr int kMaxC = JDEM_NOALLOC_MAX_CELLS;
constexpr int kSmallCell = 32;                          // insertion sort up to this many members
constexpr int kMaxLarge = kMaxP / (kSmallCell + 1) + 1; // cells with more members, at most
constexpr int kBitWords = (kMaxP + 31) / 32;            // bitmap of every particle index
constexpr int kSortThreads = 1024;
static_assert(kBitWords % kSortThreads == 0, "bitmap words split evenly over the sort block");

struct NaParams {
  float box[3];
  float inv_box[3];
  float anchor[3];
  float origin[3];
  float cell;
  int g[3];
  int ncell;
  int dim;
  int domain;
  int n;
  float k;
};

struct NoAllocScratch {
  NaParams prm;
  int cnt[kMaxC];
  int start[kMaxC + 1];
  int key[kMaxP];
  int slot[kMaxP];
  int perm[kMaxP];
  int n_large;            // cells with more than kSmallCell members (zeroed by k_na_setup)
  int large[kMaxLarge];   // their indices
};

static __device__ __align__(256) NoAllocScratch g_noalloc_scratch;

// Radius maximum (and the free-domain bounding box) in one block, then the
// grid; every thread then clears the cell counters.
__global__ void k_na_setup(NoAllocScratch* S, int n, int dim, int domain, float bx, float by, float bz,
                           float ax, float ay, float az, float k, const float* __restrict__ pos,
                           const float* __restrict__ rad) {
  __shared__ float s_r[1024], s_lo[3][1024], s_hi[3][1024];
  float rmax = 0.0f, lo[3] = {3.4e38f, 3.4e38f, 3.4e38f}, hi[3] = {-3.4e38f, -3.4e38f, -3.4e38f};
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    float r = rad[i];
    rmax = fmaxf(rmax, r);
    for (int a = 0; a < dim; ++a) {
      float x = pos[(long long)i * dim + a];
      lo[a] = fminf(lo[a], x - r);
      hi[a] = fmaxf(hi[a], x + r);
    }
  }
  s_r[threadIdx.x] = rmax;
  for (int a = 0; a < 3; ++a) {
    s_lo[a][threadIdx.x] = lo[a];
    s_hi[a][threadIdx.x] = hi[a];
  }
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      s_r[threadIdx.x] = fmaxf(s_r[threadIdx.x], s_r[threadIdx.x + w]);
      for (int a = 0; a < 3; ++a) {
        s_lo[a][threadIdx.x] = fminf(s_lo[a][threadIdx.x], s_lo[a][threadIdx.x + w]);
        s_hi[a][threadIdx.x] = fmaxf(s_hi[a][threadIdx.x], s_hi[a][threadIdx.x + w]);
      }
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    NaParams& P = S->prm;
    float box[3] = {bx, by, bz}, anc[3] = {ax, ay, az};
    float cell = 2.0f * s_r[0];
    if (!(cell > 0.0f) || !isfinite(cell)) cell = 1.0f;
    int g[3] = {1, 1, 1};
    for (int it = 0; it < 400; ++it) {
      long long tot = 1;
      for (int a = 0; a < dim; ++a) {
        float ext = domain == DOM_FREE ? s_hi[a][0] - s_lo[a][0] : box[a];
        float q = domain == DOM_PERIODIC ? floorf(ext / cell) : ceilf(ext / cell);
        g[a] = (q >= 1.0f && q < 1.0e9f) ? (int)q : 1;
        tot *= g[a];
      }
      if (tot <= kMaxC) break;
      cell *= 1.1f;
    }
    long long tot = 1;
    for (int a = 0; a < dim; ++a) tot *= g[a];
    if (tot > kMaxC)
      for (int a = 0; a < 3; ++a) g[a] = 1;
    for (int a = 0; a < 3; ++a) {
      P.box[a] = a < dim ? box[a] : 1.0f;
      P.inv_box[a] = 1.0f / P.box[a];
      P.anchor[a] = a < dim ? anc[a] : 0.0f;
      float o = domain == DOM_FREE ? s_lo[a][0] : P.anchor[a];
      P.origin[a] = (a < dim && isfinite(o)) ? o : 0.0f;
      P.g[a] = a < dim ? g[a] : 1;
    }
    P.cell = cell;
    P.ncell = P.g[0] * P.g[1] * P.g[2];
    P.dim = dim;
    P.domain = domain;
    P.n = n;
    P.k = k;
    S->n_large = 0;
  }
  for (int c = threadIdx.x; c < kMaxC; c += blockDim.x) S->cnt[c] = 0;
}

__device__ __forceinline__ int na_coord(const NaParams& P, int a, float x) {
  float v;
  if (P.domain == DOM_PERIODIC) v = floorf(floor_mod1((x - P.anchor[a]) / P.box[a]) * (float)P.g[a]);
  else v = floorf((x - P.origin[a]) / P.cell);
  return (v != v) ? 0 : (v < 0.0f ? 0 : (v > (float)(P.g[a] - 1) ? P.g[a] - 1 : (int)v));
}

__global__ void k_na_bin(NoAllocScratch* S, const float* __restrict__ pos) {
  const NaParams& P = S->prm;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P.n) return;
  int h = 0, stride = 1;
  for (int a = 0; a < P.dim; ++a) {
    h += na_coord(P, a, pos[(long long)i * P.dim + a]) * stride;
    stride *= P.g[a];
  }
  S->key[i] = h;
  S->slot[i] = atomicAdd(&S->cnt[h], 1);
}

// Exclusive scan of the cell counters in one block.
__global__ void k_na_scan(NoAllocScratch* S) {
  __shared__ int part[1024];
  const int C = S->prm.ncell;
  int per = (C + blockDim.x - 1) / blockDim.x;
  int lo = threadIdx.x * per, hi = min(C, lo + per);
  int s = 0;
  for (int c = lo; c < hi; ++c) s += S->cnt[c];
  part[threadIdx.x] = s;
  __syncthreads();
  for (int o = 1; o < (int)blockDim.x; o <<= 1) {
    int v = threadIdx.x >= o ? part[threadIdx.x - o] : 0;
    __syncthreads();
    part[threadIdx.x] += v;
    __syncthreads();
  }
  int off = part[threadIdx.x] - s;
  for (int c = lo; c < hi; ++c) {
    S->start[c] = off;
    off += S->cnt[c];
  }
  if (threadIdx.x == blockDim.x - 1) S->start[C] = part[threadIdx.x];
}

__global__ void k_na_scatter(NoAllocScratch* S) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= S->prm.n) return;
  S->perm[S->start[S->key[i]] + S->slot[i]] = i;
}

// Ascending index inside each cell: a deterministic visiting order.  Small
// cells are insertion-sorted here; larger ones are listed for k_na_bigsort.
__global__ void k_na_cellsort(NoAllocScratch* S) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= S->prm.ncell) return;
  int a = S->start[c], e = S->start[c + 1];
  if (e - a > kSmallCell) {
    S->large[atomicAdd(&S->n_large, 1)] = c;  // at most n / (kSmallCell + 1) cells
    return;
  }
  for (int i = a + 1; i < e; ++i) {
    int x = S->perm[i];
    int j = i - 1;
    while (j >= a && S->perm[j] > x) {
      S->perm[j + 1] = S->perm[j];
      --j;
    }
    S->perm[j + 1] = x;
  }
}

// A cell of m > kSmallCell members in ascending index order: the members set
// their bits in a shared bitmap of all n indices, then a block scan of the
// words' bit counts gives each word its first output position, and each
// thread writes its words' set bits out in increasing order.
__global__ void __launch_bounds__(kSortThreads) k_na_bigsort(NoAllocScratch* S) {
  __shared__ unsigned int bm[kBitWords];
  __shared__ int part[kSortThreads];
  constexpr int kPer = kBitWords / kSortThreads;  // words per thread
  const int words = (S->prm.n + 31) / 32;
  const int n_large = S->n_large;
  for (int L = blockIdx.x; L < n_large; L += gridDim.x) {
    const int c = S->large[L];
    const int a = S->start[c], e = S->start[c + 1];
    for (int w = threadIdx.x; w < words; w += kSortThreads) bm[w] = 0u;
    __syncthreads();
    for (int k = a + threadIdx.x; k < e; k += kSortThreads) {
      const int i = S->perm[k];
      atomicOr(&bm[i >> 5], 1u << (i & 31));
    }
    __syncthreads();
    // thread t owns words [t * kPer, (t + 1) * kPer)
    const int w0 = threadIdx.x * kPer;
    int cnt = 0;
#pragma unroll
    for (int q = 0; q < kPer; ++q) cnt += w0 + q < words ? __popc(bm[w0 + q]) : 0;
    part[threadIdx.x] = cnt;
    __syncthreads();
    for (int o = 1; o < kSortThreads; o <<= 1) {
      const int v = (int)threadIdx.x >= o ? part[threadIdx.x - o] : 0;
      __syncthreads();
      part[threadIdx.x] += v;
      __syncthreads();
    }
    int out = a + part[threadIdx.x] - cnt;
#pragma unroll
    for (int q = 0; q < kPer; ++q) {
      if (w0 + q >= words) break;
      unsigned int bits = bm[w0 + q];
      while (bits) {
        const int b = __ffs(bits) - 1;
        S->perm[out++] = (w0 + q) * 32 + b;
        bits &= bits - 1u;
      }
    }
    __syncthreads();  // the bitmap and the scan are reused by the next cell
  }
}

// Spring contact force of particle i (forces/spring.py:97-108 with the
// periodic minimum image of domains/periodic.py:74-79), compensated sum.
template <int DIM>
__global__ void k_na_force(NoAllocScratch* S, const float* __restrict__ pos, const float* __restrict__ rad,
                           float* __restrict__ force) {
  const NaParams& P = S->prm;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P.n) return;
  const bool per = P.domain == DOM_PERIODIC;
  float pi[3] = {0, 0, 0};
  for (int a = 0; a < DIM; ++a) pi[a] = pos[(long long)i * DIM + a];
  const float ri = rad[i];
  int h = S->key[i];
  int cx = h % P.g[0];
  int rem = h / P.g[0];
  int cy = rem % P.g[1];
  int cz = DIM == 3 ? rem / P.g[1] : 0;
  int ys[3], zs[3] = {0, 0, 0};
  int ny = axis_set(cy, P.g[1], per, ys);
  int nz = DIM == 3 ? axis_set(cz, P.g[2], per, zs) : 1;
  int xa0, xb0, xa1, xb1;
  x_ranges(cx, P.g[0], per, xa0, xb0, xa1, xb1);
  float f[3] = {0, 0, 0}, e[3] = {0, 0, 0};
  for (int iz = 0; iz < nz; ++iz)
    for (int iy = 0; iy < ny; ++iy) {
      int row = (zs[iz] * P.g[1] + ys[iy]) * P.g[0];
      for (int r = 0; r < 2; ++r) {
        int ca = r == 0 ? xa0 : xa1, cb = r == 0 ? xb0 : xb1;
        if (ca >= cb) continue;
        for (int k = S->start[row + ca]; k < S->start[row + cb]; ++k) {
          int j = S->perm[k];
          if (j == i) continue;
          float d[3] = {0, 0, 0};
          for (int a = 0; a < DIM; ++a) {
            d[a] = pi[a] - pos[(long long)j * DIM + a];
            if (per) d[a] = d[a] - P.box[a] * rintf(d[a] * P.inv_box[a]);
          }
          float dsq = d[0] * d[0] + d[1] * d[1];
          if (DIM == 3) dsq = dsq + d[2] * d[2];
          float R = ri + rad[j];
          if (!(dsq < R * R * 1.000001f)) continue;
          float inv = dsq == 0.0f ? 0.0f : 1.0f / sqrtf(fmaxf(dsq, 1e-16f));
          float rr = dsq * inv;
          float delta = R - rr;
          delta = delta > 0.0f ? delta : 0.0f;
          float mag = P.k * delta * inv;
          for (int a = 0; a < DIM; ++a) two_sum_acc(f[a], e[a], mag * d[a]);
        }
      }
    }
  for (int a = 0; a < DIM; ++a) force[(long long)i * DIM + a] = f[a] + e[a];
}

std::mutex g_mtx;
// per device: the context the address was looked up in, and the address
struct DevScratch {
  unsigned long long ctx_id = 0;
  NoAllocScratch* ptr = nullptr;
};
DevScratch g_dev[256];

// Unique id of the calling thread's current context (never reused within the
// process, unlike a context's address), through the driver entry points the
// runtime exposes; 0 when unavailable.
unsigned long long current_context_id() {
  using GetCurrent = CUresult (*)(CUcontext*);
  using GetId = CUresult (*)(CUcontext, unsigned long long*);
  static GetCurrent get_current = nullptr;
  static GetId get_id = nullptr;
  static bool looked_up = false;
  if (!looked_up) {
    void* f1 = nullptr;
    void* f2 = nullptr;
    cudaDriverEntryPointQueryResult q1, q2;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) == cudaSuccess &&
        q1 == cudaDriverEntryPointSuccess &&
        cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) == cudaSuccess &&
        q2 == cudaDriverEntryPointSuccess) {
      get_current = (GetCurrent)f1;
      get_id = (GetId)f2;
    }
    cudaGetLastError();
    looked_up = true;
  }
  if (!get_current || !get_id) return 0;
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (get_current(&ctx) != CUDA_SUCCESS || !ctx || get_id(ctx, &id) != CUDA_SUCCESS) return 0;
  return id;
}

}  // namespace

extern "C" int jdem_compute_force_noalloc(int32_t dim, int64_t n, int32_t domain, const float* box_size,
                                          const float* anchor, float young, const float* pos, const float* rad,
                                          float* force, void* stream) {
  if (n < 0) {
    std::fprintf(stderr, "jdem_compute_force_noalloc: n = %lld is negative\n", (long long)n);
    return JDEM_ERR_BAD_ARG;
  }
  if (n > kMaxP) {
    std::fprintf(stderr,
                 "jdem_compute_force_noalloc: n = %lld exceeds the fixed scratch limit of %d particles "
                 "(JDEM_NOALLOC_MAX_PARTICLES); use jdem_create/jdem_compute_force for larger systems\n",
                 (long long)n, kMaxP);
    return JDEM_ERR_CAPACITY_OVERFLOW;
  }
  if ((dim != 2 && dim != 3) || domain < 0 || domain > 2) return JDEM_ERR_BAD_ARG;
  if (n == 0) return JDEM_OK;
  if (!pos || !rad || !force || !box_size || !anchor) return JDEM_ERR_BAD_ARG;
  for (int a = 0; a < dim; ++a)
    if (domain != DOM_FREE && !(box_size[a] > 0.0f)) return JDEM_ERR_BAD_ARG;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 256) return JDEM_ERR_CUDA;
  NoAllocScratch* S = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_mtx);
    // first call on this device, or a new context since (cudaDeviceReset):
    // look the array's address up in the current context
    const unsigned long long ctx = current_context_id();
    DevScratch& d = g_dev[dev];
    if (!d.ptr || ctx != d.ctx_id) {
      void* p = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess || !p) {
        cudaGetLastError();
        std::fprintf(stderr, "jdem_compute_force_noalloc: cudaGetSymbolAddress failed: %s\n",
                     cudaGetErrorString(e));
        return JDEM_ERR_CUDA;
      }
      d.ptr = (NoAllocScratch*)p;
      d.ctx_id = ctx;
    }
    S = d.ptr;
  }
  cudaStream_t st = (cudaStream_t)stream;
  float b[3] = {1, 1, 1}, an[3] = {0, 0, 0};
  for (int a = 0; a < dim; ++a) {
    b[a] = box_size[a];
    an[a] = anchor[a];
  }
  int ni = (int)n;
  unsigned int pb = (unsigned int)((ni + 255) / 256);
  k_na_setup<<<1, 1024, 0, st>>>(S, ni, dim, domain, b[0], b[1], b[2], an[0], an[1], an[2], young, pos, rad);
  k_na_bin<<<pb, 256, 0, st>>>(S, pos);
  k_na_scan<<<1, 1024, 0, st>>>(S);
  k_na_scatter<<<pb, 256, 0, st>>>(S);
  k_na_cellsort<<<(kMaxC + 255) / 256, 256, 0, st>>>(S);
  k_na_bigsort<<<64, kSortThreads, 0, st>>>(S);
  if (dim == 3) k_na_force<3><<<pb, 256, 0, st>>>(S, pos, rad, force);
  else k_na_force<2><<<pb, 256, 0, st>>>(S, pos, rad, force);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    std::fprintf(stderr, "jdem_compute_force_noalloc: launch failed: %s\n", cudaGetErrorString(e));
    return JDEM_ERR_CUDA;
  }
  return JDEM_OK;
}
