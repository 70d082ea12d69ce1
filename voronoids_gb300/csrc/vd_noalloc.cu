// Edge extraction that allocates no memory (vd_edges_from_simplices_noalloc).
//
// Who needs this: a caller that is not allowed to allocate GPU memory at
// the moment it wants an edge list -- for instance a host application whose
// memory manager owns the whole device and refuses further cudaMalloc calls,
// a latency-bound loop that cannot afford the device-wide synchronisation a
// cudaMalloc/cudaFree pair can cause, or a plugin running under a fixed
// memory budget that was reserved when the process started.  Such a caller
// passes its simplices and an output buffer it already owns; every scratch
// array this operation needs lives in one statically sized device array that
// is part of the library image.
//
// The work is the same as the tree's own edge extraction (vd_edges.cu):
// every edge of every simplex is bucketed by its smaller endpoint, each
// bucket is sorted and de-duplicated, and a scan places the unique edges.
// Limits: at most kNaMaxSimplices simplices and kNaMaxVertices vertex ids.
//
// Shared state: every call on a device uses the same scratch array, and it
// keeps whatever the previous call left there; the counters that must start
// at zero are cleared at the start of each call.  Two calls whose GPU work
// overlaps (different streams or threads without ordering between them)
// race on the array and produce garbage.  The first call on each device
// looks up the array's device address with cudaGetSymbolAddress while that
// device is current (again after the device's context has been recreated,
// e.g. by cudaDeviceReset); make that first call before starting any stream
// capture on the device.  Every call waits for its own work on its stream
// to finish before it returns.
#include <cuda.h>
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/voronoids_gpu.h"
#include "vd_common.cuh"

namespace {

constexpr long long kNaMaxSimplices = 131072;  // 2^17
constexpr int kNaMaxVertices = 65536;          // 2^16
constexpr long long kNaBuf = 6 * kNaMaxSimplices;
constexpr int kNaSeg = 1024;  // bucket length sorted in one warp's shared memory

// Scratch layout (ints): cnt, off, ucnt, uoff (kNaMaxVertices + 1 each),
// buckets (kNaBuf), padded sort area for long buckets (2 * kNaBuf), list of
// long buckets (kNaMaxVertices), control words (16).
constexpr long long kNaCnt = 0;
constexpr long long kNaOff = kNaCnt + kNaMaxVertices + 1;
constexpr long long kNaUcnt = kNaOff + kNaMaxVertices + 1;
constexpr long long kNaUoff = kNaUcnt + kNaMaxVertices + 1;
constexpr long long kNaBucket = kNaUoff + kNaMaxVertices + 1;
constexpr long long kNaPad = kNaBucket + kNaBuf;
constexpr long long kNaBig = kNaPad + 2 * kNaBuf;
constexpr long long kNaCtl = kNaBig + kNaMaxVertices;
constexpr long long kNaInts = kNaCtl + 16;

// The scratch array itself (about 10.5 MB), held by every device that loads
// the library until the process exits.
static __device__ __align__(256) int g_na_scratch[kNaInts];

constexpr unsigned FULL = 0xffffffffu;

// ctl[0] = number of long buckets, ctl[1] = error flag (bad vertex id)
__global__ void k_na_count(const int* simp, long long ns, int nv, int dim, int* S) {
  int* cnt = S + kNaCnt;
  int* ctl = S + kNaCtl;
  for (long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x; s < ns;
       s += (long long)gridDim.x * blockDim.x) {
    const int4 v = reinterpret_cast<const int4*>(simp)[s];
    const int a[4] = {v.x, v.y, v.z, v.w};
    for (int i = 0; i <= dim; ++i)
      for (int j = i + 1; j <= dim; ++j) {
        const int x = a[i], y = a[j];
        if (x < 0 || y < 0) continue;
        if (x >= nv || y >= nv) {
          atomicExch(ctl + 1, 1);
          continue;
        }
        if (x == y) continue;
        atomicAdd(cnt + min(x, y), 1);
      }
  }
}

// exclusive scan of in[0..n) into out[0..n], one block of 1024 threads
__global__ void __launch_bounds__(1024) k_na_scan(const int* in, int* out, int n) {
  __shared__ int wsum[32];
  const int per = (n + blockDim.x - 1) / blockDim.x;
  const int lo = threadIdx.x * per, hi = min(n, lo + per);
  int local = 0;
  for (int i = lo; i < hi; ++i) local += in[i];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int x = local;
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(FULL, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) wsum[w] = x;
  __syncthreads();
  if (w == 0) {
    int t = wsum[lane];
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(FULL, t, o);
      if (lane >= o) t += y;
    }
    wsum[lane] = t;
  }
  __syncthreads();
  int run = x - local + (w > 0 ? wsum[w - 1] : 0);
  for (int i = lo; i < hi; ++i) {
    out[i] = run;
    run += in[i];
  }
  if (threadIdx.x == blockDim.x - 1) out[n] = run;
}

__global__ void k_na_fill(const int* simp, long long ns, int nv, int dim, int* S) {
  int* cnt = S + kNaCnt;
  const int* off = S + kNaOff;
  int* buf = S + kNaBucket;
  for (long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x; s < ns;
       s += (long long)gridDim.x * blockDim.x) {
    const int4 v = reinterpret_cast<const int4*>(simp)[s];
    const int a[4] = {v.x, v.y, v.z, v.w};
    for (int i = 0; i <= dim; ++i)
      for (int j = i + 1; j <= dim; ++j) {
        const int x = a[i], y = a[j];
        if (x < 0 || y < 0 || x >= nv || y >= nv || x == y) continue;
        const int u = min(x, y);
        const int k = atomicSub(cnt + u, 1) - 1;  // counts return to zero
        if (k >= 0) buf[off[u] + k] = max(x, y);
      }
  }
}

__device__ void bitonic(int* a, int P, int lane, int nthreads, bool block) {
  for (int k = 2; k <= P; k <<= 1)
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = lane; i < P; i += nthreads) {
        const int l = i ^ j;
        if (l > i) {
          const int x = a[i], y = a[l];
          if ((x > y) == ((i & k) == 0)) {
            a[i] = y;
            a[l] = x;
          }
        }
      }
      if (block)
        __syncthreads();
      else
        __syncwarp();
    }
}

// one warp per vertex: sort + unique its bucket in shared memory
__global__ void __launch_bounds__(128) k_na_uniq(int nv, int* S) {
  __shared__ int sm[4][kNaSeg];
  const int* off = S + kNaOff;
  int* buf = S + kNaBucket;
  int* ucnt = S + kNaUcnt;
  int* big = S + kNaBig;
  int* ctl = S + kNaCtl;
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int* a = sm[w];
  for (int u = blockIdx.x * 4 + w; u < nv; u += gridDim.x * 4) {
    const int b = off[u], L = off[u + 1] - b;
    if (L > kNaSeg) {
      if (lane == 0) big[atomicAdd(ctl, 1)] = u;
      continue;
    }
    if (L <= 1) {
      if (lane == 0) ucnt[u] = L;
      continue;
    }
    int P = 2;
    while (P < L) P <<= 1;
    for (int i = lane; i < P; i += 32) a[i] = i < L ? buf[b + i] : 0x7fffffff;
    __syncwarp();
    bitonic(a, P, lane, 32, false);
    int outc = 0;
    for (int i0 = 0; i0 < L; i0 += 32) {
      const int i = i0 + lane;
      const bool keep = i < L && (i == 0 || a[i] != a[i - 1]);
      const unsigned m = __ballot_sync(FULL, keep);
      if (keep) buf[b + outc + __popc(m & ((1u << lane) - 1))] = a[i];
      outc += __popc(m);
    }
    if (lane == 0) ucnt[u] = outc;
    __syncwarp();
  }
}

// one block per long bucket, sorted in the padded area at 2 * off[u]
__global__ void __launch_bounds__(1024) k_na_uniq_big(int* S) {
  const int* off = S + kNaOff;
  int* buf = S + kNaBucket;
  int* ucnt = S + kNaUcnt;
  const int* big = S + kNaBig;
  const int nbig = S[kNaCtl];
  __shared__ int wsum[32];
  __shared__ int running;
  for (int t = blockIdx.x; t < nbig; t += gridDim.x) {
    const int u = big[t];
    const int b = off[u], L = off[u + 1] - b;
    int* a = S + kNaPad + 2LL * b;
    int P = 2;
    while (P < L) P <<= 1;
    for (int i = threadIdx.x; i < P; i += blockDim.x) a[i] = i < L ? buf[b + i] : 0x7fffffff;
    __syncthreads();
    bitonic(a, P, threadIdx.x, blockDim.x, true);
    if (threadIdx.x == 0) running = 0;
    __syncthreads();
    for (int i0 = 0; i0 < L; i0 += blockDim.x) {
      const int i = i0 + threadIdx.x;
      const bool keep = i < L && (i == 0 || a[i] != a[i - 1]);
      const unsigned m = __ballot_sync(FULL, keep);
      const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
      if (lane == 0) wsum[w] = __popc(m);
      __syncthreads();
      int before = 0, tot = 0;
      for (int k = 0; k < (int)(blockDim.x >> 5); ++k) {
        if (k < w) before += wsum[k];
        tot += wsum[k];
      }
      if (keep) buf[b + running + before + __popc(m & ((1u << lane) - 1))] = a[i];
      __syncthreads();
      if (threadIdx.x == 0) running += tot;
      __syncthreads();
    }
    if (threadIdx.x == 0) ucnt[u] = running;
    __syncthreads();
  }
}

__global__ void k_na_out(int nv, const int* S, uint2* out, long long cap) {
  const int* off = S + kNaOff;
  const int* buf = S + kNaBucket;
  const int* ucnt = S + kNaUcnt;
  const int* uoff = S + kNaUoff;
  const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  for (int u = w; u < nv; u += nw) {
    const int b = off[u], o = uoff[u], c = ucnt[u];
    for (int k = lane; k < c; k += 32)
      if (o + k < cap) out[o + k] = make_uint2((unsigned)u, (unsigned)buf[b + k]);
  }
}

// Device address of g_na_scratch per device, remembered together with the id
// of the CUDA context it was looked up in.  The address belongs to the
// module loaded in that context: after cudaDeviceReset (or any other end of
// the device's primary context) the module is loaded again and the array may
// sit elsewhere, so a new context id means a new lookup.  Context ids come
// from the driver API (cuCtxGetCurrent, cuCtxGetId), reached through the
// runtime's driver entry points so that the library needs no libcuda link.
constexpr int kNaMaxDevices = 64;
struct NaSlot {
  unsigned long long ctx_id;
  int* addr;
};
NaSlot g_na_slot[kNaMaxDevices] = {};
std::mutex g_na_mutex;

typedef CUresult (*CtxGetCurrentFn)(CUcontext*);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long*);

// Id of the calling thread's current context, 0 if none or unknown.
unsigned long long current_ctx_id() {
  static CtxGetCurrentFn get_current = nullptr;
  static CtxGetIdFn get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<CtxGetCurrentFn>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<CtxGetIdFn>(f);
  });
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (!get_current || !get_id || get_current(&ctx) != CUDA_SUCCESS || !ctx || get_id(ctx, &id) != CUDA_SUCCESS)
    return 0;
  return id;
}

int na_scratch(int** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kNaMaxDevices) return VD_ERR_CUDA;
  std::lock_guard<std::mutex> lock(g_na_mutex);
  NaSlot& slot = g_na_slot[dev];
  const unsigned long long id = current_ctx_id();
  if (id != 0 && slot.addr && slot.ctx_id == id) {
    *out = slot.addr;
    return VD_OK;
  }
  // first call on this device, or a new context: look the address up with
  // the device current (this may also make the primary context current)
  void* p = nullptr;
  if (cudaGetSymbolAddress(&p, g_na_scratch) != cudaSuccess || !p) return VD_ERR_CUDA;
  slot.addr = static_cast<int*>(p);
  slot.ctx_id = current_ctx_id();  // 0 (unknown): looked up again on the next call
  *out = slot.addr;
  return VD_OK;
}

}  // namespace

extern "C" int vd_edges_from_simplices_noalloc(int dim, const int32_t* d_simp, int64_t ns, int64_t nverts,
                                               uint32_t* d_uv, int64_t cap, int64_t* n_edges, void* stream) {
  if ((dim != 2 && dim != 3) || ns < 0 || nverts < 0 || cap < 0 || !n_edges) return VD_ERR_ARG;
  if (ns > kNaMaxSimplices || nverts > kNaMaxVertices) return VD_ERR_ARG;  // beyond the static scratch
  if ((ns > 0 && !d_simp) || (cap > 0 && !d_uv)) return VD_ERR_ARG;
  int* S = nullptr;
  int rc = na_scratch(&S);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  const int nv = (int)nverts;
  // zero what the call counts into: bucket counts and the control words
  if (cudaMemsetAsync(S + kNaCnt, 0, sizeof(int) * (nv + 1), st) != cudaSuccess ||
      cudaMemsetAsync(S + kNaCtl, 0, sizeof(int) * 16, st) != cudaSuccess)
    return VD_ERR_CUDA;
  const int blocks = 1024;
  k_na_count<<<blocks, 256, 0, st>>>(d_simp, ns, nv, dim, S);
  k_na_scan<<<1, 1024, 0, st>>>(S + kNaCnt, S + kNaOff, nv);
  k_na_fill<<<blocks, 256, 0, st>>>(d_simp, ns, nv, dim, S);
  k_na_uniq<<<blocks, 128, 0, st>>>(nv, S);
  k_na_uniq_big<<<64, 1024, 0, st>>>(S);
  k_na_scan<<<1, 1024, 0, st>>>(S + kNaUcnt, S + kNaUoff, nv);
  k_na_out<<<blocks, 256, 0, st>>>(nv, S, reinterpret_cast<uint2*>(d_uv), cap);
  vd::note_launches(7);
  // launch errors of this call, read without clearing an error the caller's
  // thread may hold from before
  if (cudaPeekAtLastError() != cudaSuccess) return VD_ERR_CUDA;
  int host[2] = {0, 0};
  if (cudaMemcpyAsync(&host[0], S + kNaUoff + nv, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaMemcpyAsync(&host[1], S + kNaCtl + 1, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess)
    return VD_ERR_CUDA;
  if (cudaStreamSynchronize(st) != cudaSuccess) return VD_ERR_CUDA;
  *n_edges = host[0];
  if (host[1]) return VD_ERR_ARG;  // a vertex id was >= nverts
  return host[0] > cap ? VD_ERR_ARG : VD_OK;
}
