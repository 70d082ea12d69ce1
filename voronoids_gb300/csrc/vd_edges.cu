// Sorted Delaunay edge list among input points (both endpoints non-super),
// as input-index pairs (u < v), sorted lexicographically.
//
// The reference exposes the graph only through its simplex map
// (PyDelauanyTree.simplices, src/lib.rs:87-100); the parity contract of this
// build is the sorted edge list derived from it.  Instead of a global sort of
// all (simplex, edge) instances, instances are bucketed by their smaller
// endpoint (counting pass + exclusive scan + scatter), each bucket is sorted
// and de-duplicated by one warp in shared memory, and a second scan places the
// unique edges.  Buckets longer than a warp's buffer are sorted by a block in
// global memory.  A simplex emits an edge only where the emission rule below
// picks it (about 2.6 instances per edge in 3D instead of ~5.2, one in 2D).
#include <cuda_runtime.h>

#include <vector>

#include "vd_common.cuh"

namespace vd {
namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr int kScanBlock = 512;
constexpr int kScanTile = kScanBlock * 4;
constexpr int kWarpSeg = 256;

// ---- exclusive scan (tile scan + recursive scan of tile sums) --------------
__global__ void k_scan_tile(const int* in, int* out, int* sums, long long n) {
  __shared__ int s[kScanBlock];
  const long long base = (long long)blockIdx.x * kScanTile;
  int v[4];
  int local = 0;
  for (int k = 0; k < 4; ++k) {
    long long i = base + threadIdx.x * 4 + k;
    v[k] = i < n ? in[i] : 0;
    local += v[k];
  }
  // block exclusive scan of `local`
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int x = local;
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(FULL, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) s[w] = x;
  __syncthreads();
  if (w == 0) {
    int t = lane < kScanBlock / 32 ? s[lane] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(FULL, t, o);
      if (lane >= o) t += y;
    }
    if (lane < kScanBlock / 32) s[lane] = t;
  }
  __syncthreads();
  int excl = x - local + (w > 0 ? s[w - 1] : 0);
  for (int k = 0; k < 4; ++k) {
    long long i = base + threadIdx.x * 4 + k;
    if (i < n) out[i] = excl;
    excl += v[k];
  }
  if (threadIdx.x == kScanBlock - 1) sums[blockIdx.x] = excl;
}

__global__ void k_scan_add(int* out, const int* sums, long long n) {
  const long long base = (long long)blockIdx.x * kScanTile;
  const int add = sums[blockIdx.x];
  for (int k = threadIdx.x; k < kScanTile; k += blockDim.x) {
    long long i = base + k;
    if (i < n) out[i] += add;
  }
}

// out[i] = sum(in[0..i)) for i < n, out[n] = total.  `tmp` holds
// scan_scratch_ints(n) ints.
void exclusive_scan(const int* in, int* out, long long n, int* tmp, cudaStream_t st) {
  if (n <= 0) {
    cudaMemsetAsync(out, 0, sizeof(int), st);
    return;
  }
  const long long tiles = (n + kScanTile - 1) / kScanTile;
  int* sums = tmp;
  k_scan_tile<<<(unsigned)tiles, kScanBlock, 0, st>>>(in, out, sums, n);
  note_launches(1);
  if (tiles == 1) {
    cudaMemcpyAsync(out + n, sums, sizeof(int), cudaMemcpyDeviceToDevice, st);
    return;
  }
  int* scanned = tmp + tiles;
  exclusive_scan(sums, scanned, tiles, scanned + tiles + 1, st);
  k_scan_add<<<(unsigned)tiles, 256, 0, st>>>(out, scanned, n);
  note_launches(1);
  cudaMemcpyAsync(out + n, scanned + tiles, sizeof(int), cudaMemcpyDeviceToDevice, st);
}

// ---- edge instances ---------------------------------------------------------
// Simplex s emits its edge (v[i], v[j]) only if s is below its neighbours
// across the faces that contain the edge (the faces opposite the other
// vertices; a hull face counts as no neighbour).  Around an edge the
// simplices form a ring (2D: a pair) in which each one's neighbours across
// those faces are its two ring neighbours, so the ring's lowest slot always
// emits: every edge still appears, about a third as often in 3D and exactly
// once in 2D, which shrinks the buckets to sort.
template <int NV>
__device__ __forceinline__ bool emits(int s, const int* nb, int i, int j) {
  for (int k = 0; k < NV; ++k) {
    if (k == i || k == j) continue;
    if (nb[k] >= 0 && (nb[k] >> 2) < s) return false;
  }
  return true;
}

template <int D>
__global__ void k_edge_count(DevTree T, int nsimp, int n_in, int* cnt) {
  constexpr int NV = D + 1;
  const int NS = T.nsuper;
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < nsimp; s += gridDim.x * blockDim.x) {
    const int4 v = reinterpret_cast<const int4*>(T.simp + s)[0];
    if (v.x < 0) continue;
    const int4 n = reinterpret_cast<const int4*>(T.simp + s)[1];
    const int a[4] = {v.x, v.y, v.z, v.w};
    const int nb[4] = {n.x, n.y, n.z, n.w};
    for (int i = 0; i < NV; ++i)
      for (int j = i + 1; j < NV; ++j) {
        int x = a[i], y = a[j];
        if (x < NS || y < NS || !emits<NV>(s, nb, i, j)) continue;
        if (max(x, y) - NS >= n_in) {
          set_error(T.ctr, E_INTERNAL);
          continue;
        }
        atomicAdd(cnt + (min(x, y) - NS), 1);
      }
  }
}

template <int D>
__global__ void k_edge_fill(DevTree T, int nsimp, int n_in, int* cnt, const int* off, int* buf) {
  constexpr int NV = D + 1;
  const int NS = T.nsuper;
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < nsimp; s += gridDim.x * blockDim.x) {
    const int4 v = reinterpret_cast<const int4*>(T.simp + s)[0];
    if (v.x < 0) continue;
    const int4 n = reinterpret_cast<const int4*>(T.simp + s)[1];
    const int a[4] = {v.x, v.y, v.z, v.w};
    const int nb[4] = {n.x, n.y, n.z, n.w};
    for (int i = 0; i < NV; ++i)
      for (int j = i + 1; j < NV; ++j) {
        int x = a[i], y = a[j];
        if (x < NS || y < NS || !emits<NV>(s, nb, i, j)) continue;
        int u = min(x, y) - NS, w = max(x, y) - NS;
        if (w >= n_in) continue;
        int k = atomicSub(cnt + u, 1) - 1;  // cnt returns to 0
        if (k >= 0) buf[off[u] + k] = w;
      }
  }
}

// one warp per vertex: sort + unique its bucket in shared memory
__global__ void __launch_bounds__(256) k_edge_uniq(int n_in, const int* off, int* buf, int* ucnt,
                                                   int* big, int* nbig) {
  __shared__ int sm[8][kWarpSeg];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int* a = sm[w];
  for (int u = blockIdx.x * 8 + w; u < n_in; u += gridDim.x * 8) {
    const int b = off[u], L = off[u + 1] - b;
    if (L > kWarpSeg) {
      if (lane == 0) big[atomicAdd(nbig, 1)] = u;
      continue;
    }
    if (L <= 1) {
      if (lane == 0) ucnt[u] = L;
      continue;
    }
    if (L <= 64) {
      // common case: two keys per lane (positions lane, lane + 32), bitonic
      // network on registers and shuffles, no shared memory
      int a = lane < L ? buf[b + lane] : 0x7fffffff;
      int c = lane + 32 < L ? buf[b + lane + 32] : 0x7fffffff;
      for (int k = 2; k <= 64; k <<= 1)
        for (int j = k >> 1; j > 0; j >>= 1) {
          if (j == 32) {  // k == 64: pairs (lane, lane + 32), ascending
            const int lo = min(a, c), hi = max(a, c);
            a = lo;
            c = hi;
            continue;
          }
          const bool lower = (lane & j) == 0;
          const int ya = __shfl_xor_sync(FULL, a, j), yc = __shfl_xor_sync(FULL, c, j);
          const bool upa = (lane & k) == 0, upc = ((lane + 32) & k) == 0;
          a = (lower == upa) ? min(a, ya) : max(a, ya);
          c = (lower == upc) ? min(c, yc) : max(c, yc);
        }
      // unique: keep the first of each run
      const int pa = __shfl_up_sync(FULL, a, 1), pc = __shfl_up_sync(FULL, c, 1);
      const int a31 = __shfl_sync(FULL, a, 31);
      const bool ka = lane < L && (lane == 0 || a != pa);
      const bool kc = lane + 32 < L && c != (lane == 0 ? a31 : pc);
      const unsigned ma = __ballot_sync(FULL, ka), mc = __ballot_sync(FULL, kc);
      const unsigned below = (1u << lane) - 1;
      if (ka) buf[b + __popc(ma & below)] = a;
      if (kc) buf[b + __popc(ma) + __popc(mc & below)] = c;
      if (lane == 0) ucnt[u] = __popc(ma) + __popc(mc);
      continue;
    }
    int P = 2;
    while (P < L) P <<= 1;
    for (int i = lane; i < P; i += 32) a[i] = i < L ? buf[b + i] : 0x7fffffff;
    __syncwarp();
    for (int k = 2; k <= P; k <<= 1)
      for (int j = k >> 1; j > 0; j >>= 1) {
        for (int i = lane; i < P; i += 32) {
          int l = i ^ j;
          if (l > i) {
            int x = a[i], y = a[l];
            bool up = (i & k) == 0;
            if ((x > y) == up) {
              a[i] = y;
              a[l] = x;
            }
          }
        }
        __syncwarp();
      }
    int outc = 0;
    for (int i0 = 0; i0 < L; i0 += 32) {
      int i = i0 + lane;
      bool keep = i < L && (i == 0 || a[i] != a[i - 1]);
      unsigned m = __ballot_sync(FULL, keep);
      if (keep) buf[b + outc + __popc(m & ((1u << lane) - 1))] = a[i];
      outc += __popc(m);
    }
    if (lane == 0) ucnt[u] = outc;
    __syncwarp();
  }
}

// one block per long bucket: bitonic sort in a padded global scratch area
__global__ void __launch_bounds__(1024) k_edge_uniq_big(const int* big, const int* off, int* buf,
                                                        int* ucnt, int* scratch,
                                                        const long long* soff) {
  const int u = big[blockIdx.x];
  const int b = off[u], L = off[u + 1] - b;
  int* a = scratch + soff[blockIdx.x];
  int P = 2;
  while (P < L) P <<= 1;
  for (int i = threadIdx.x; i < P; i += blockDim.x) a[i] = i < L ? buf[b + i] : 0x7fffffff;
  __syncthreads();
  for (int k = 2; k <= P; k <<= 1)
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = threadIdx.x; i < P; i += blockDim.x) {
        int l = i ^ j;
        if (l > i) {
          int x = a[i], y = a[l];
          bool up = (i & k) == 0;
          if ((x > y) == up) {
            a[i] = y;
            a[l] = x;
          }
        }
      }
      __syncthreads();
    }
  __shared__ int wsum[32];
  __shared__ int running;
  if (threadIdx.x == 0) running = 0;
  __syncthreads();
  for (int i0 = 0; i0 < L; i0 += blockDim.x) {
    int i = i0 + threadIdx.x;
    bool keep = i < L && (i == 0 || a[i] != a[i - 1]);
    unsigned m = __ballot_sync(FULL, keep);
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
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
}

__global__ void k_edge_out(int n_in, const int* off, const int* buf, const int* ucnt,
                           const int* uoff, uint2* out, long long cap) {
  const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  for (int u = w; u < n_in; u += nw) {
    const int b = off[u], o = uoff[u], c = ucnt[u];
    for (int k = lane; k < c; k += 32)
      if (o + k < cap) out[o + k] = make_uint2((unsigned)u, (unsigned)buf[b + k]);
  }
}

}  // namespace

int64_t scan_scratch_ints(int64_t n) {
  int64_t total = 64;
  int64_t t = (n + kScanTile - 1) / kScanTile;
  while (t > 1) {
    total += 2 * t + 2;
    t = (t + kScanTile - 1) / kScanTile;
  }
  return total + 4;
}

// Returns the number of unique edges written to d_out (or -1 on a CUDA error).
void scan_ints(const int* in, int* out, int64_t n, int* tmp, cudaStream_t st) { exclusive_scan(in, out, n, tmp, st); }

int64_t run_edges(const DevTree& T, const Launch& L, int dim, int nsimp, int n_in,
                  const EdgeScratch& S, uint2* d_out, int64_t cap_out, int* d_total_pair, int* h_total_pair) {
  cudaStream_t st = L.stream;
  note_launches(4);  // count, fill, unique, output (scans count themselves)
  cudaMemsetAsync(S.cnt, 0, sizeof(int) * (n_in + 1), st);
  cudaMemsetAsync(S.nbig, 0, sizeof(int), st);
  if (dim == 3) {
    k_edge_count<3><<<L.blocks, 256, 0, st>>>(T, nsimp, n_in, S.cnt);
  } else {
    k_edge_count<2><<<L.blocks, 256, 0, st>>>(T, nsimp, n_in, S.cnt);
  }
  exclusive_scan(S.cnt, S.off, n_in, S.scan_tmp, st);
  if (dim == 3) {
    k_edge_fill<3><<<L.blocks, 256, 0, st>>>(T, nsimp, n_in, S.cnt, S.off, S.buf);
  } else {
    k_edge_fill<2><<<L.blocks, 256, 0, st>>>(T, nsimp, n_in, S.cnt, S.off, S.buf);
  }
  k_edge_uniq<<<L.blocks, 256, 0, st>>>(n_in, S.off, S.buf, S.ucnt, S.big, S.nbig);
  exclusive_scan(S.ucnt, S.uoff, n_in, S.scan_tmp, st);
  k_edge_out<<<L.blocks, 256, 0, st>>>(n_in, S.off, S.buf, S.ucnt, S.uoff, d_out, cap_out);
  cudaMemcpyAsync(d_total_pair, S.uoff + n_in, sizeof(int), cudaMemcpyDeviceToDevice, st);
  cudaMemcpyAsync(d_total_pair + 1, S.nbig, sizeof(int), cudaMemcpyDeviceToDevice, st);
  cudaMemcpyAsync(h_total_pair, d_total_pair, 2 * sizeof(int), cudaMemcpyDeviceToHost, st);
  if (cudaStreamSynchronize(st) != cudaSuccess) return -1;
  if (h_total_pair[1] == 0) return h_total_pair[0];

  // long buckets: sort them in padded scratch, then redo the placement
  if (sort_big_buckets(L, n_in, S.off, S.buf, S.ucnt, S.big, h_total_pair[1]) != 0) return -1;
  note_launches(1);
  exclusive_scan(S.ucnt, S.uoff, n_in, S.scan_tmp, st);
  k_edge_out<<<L.blocks, 256, 0, st>>>(n_in, S.off, S.buf, S.ucnt, S.uoff, d_out, cap_out);
  cudaMemcpyAsync(h_total_pair, S.uoff + n_in, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (cudaStreamSynchronize(st) != cudaSuccess) return -1;
  return h_total_pair[0];
}

int sort_big_buckets(const Launch& L, int n, const int* off, int* buf, int* ucnt, const int* big, int nbig) {
  if (nbig <= 0) return 0;
  cudaStream_t st = L.stream;
  std::vector<int> hbig(nbig);
  std::vector<int> hoff(n + 1);
  cudaMemcpyAsync(hbig.data(), big, sizeof(int) * nbig, cudaMemcpyDeviceToHost, st);
  cudaMemcpyAsync(hoff.data(), off, sizeof(int) * (n + 1), cudaMemcpyDeviceToHost, st);
  if (cudaStreamSynchronize(st) != cudaSuccess) return -1;
  std::vector<long long> soff(nbig + 1, 0);
  for (int i = 0; i < nbig; ++i) {
    long long len = hoff[hbig[i] + 1] - hoff[hbig[i]], P = 2;
    while (P < len) P <<= 1;
    soff[i + 1] = soff[i] + P;
  }
  int* scratch = nullptr;
  long long* dsoff = nullptr;
  if (cudaMalloc(&scratch, sizeof(int) * soff[nbig]) != cudaSuccess) return -1;
  if (cudaMalloc(&dsoff, sizeof(long long) * (nbig + 1)) != cudaSuccess) {
    cudaFree(scratch);
    return -1;
  }
  cudaMemcpyAsync(dsoff, soff.data(), sizeof(long long) * (nbig + 1), cudaMemcpyHostToDevice, st);
  k_edge_uniq_big<<<nbig, 1024, 0, st>>>(big, off, buf, ucnt, scratch, dsoff);
  note_launches(1);
  const cudaError_t e = cudaStreamSynchronize(st);
  cudaFree(scratch);
  cudaFree(dsoff);
  return e == cudaSuccess ? 0 : -1;
}

int sort_buckets(const Launch& L, int n, const int* off, int* buf, int* ucnt, int* big, int* nbig, int* d_pair,
                 int* h_pair) {
  cudaStream_t st = L.stream;
  cudaMemsetAsync(nbig, 0, sizeof(int), st);
  note_launches(1);
  k_edge_uniq<<<L.blocks, 256, 0, st>>>(n, off, buf, ucnt, big, nbig);
  cudaMemcpyAsync(h_pair, nbig, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (cudaStreamSynchronize(st) != cudaSuccess) return -1;
  return sort_big_buckets(L, n, off, buf, ucnt, big, h_pair[0]);
}

}  // namespace vd
