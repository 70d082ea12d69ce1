// Super-simplex sizing from points already in device memory.
//
// The reference's bounding_sphere (src/geometry.rs:99-142) takes the
// bounding box, then walks the points in order and multiplies the radius by
// 1.5 whenever a point is not strictly inside.  Every point lies in the box,
// so its distance to the centre is at most the half diagonal up to rounding;
// once the radius has grown by 1.5 no later point can fail.  The loop is
// therefore equivalent to: r = r0 * 1.5 if any point fails `d^2 < r0^2`,
// else r0 -- an order-independent reduction, computed here with the same
// per-point rounding sequence (no fused operations) as the reference.
#include <cuda_runtime.h>

#include <algorithm>

#include "vd_common.cuh"

namespace vd {
namespace {

// Order-preserving map of a double to an unsigned key.
__device__ __forceinline__ unsigned long long dkey(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

template <int D>
__global__ void k_bbox(const double* xyz, long long n, unsigned long long* mm) {
  unsigned long long lo[3] = {~0ull, ~0ull, ~0ull}, hi[3] = {0, 0, 0};
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    for (int k = 0; k < D; ++k) {
      const unsigned long long key = dkey(xyz[i * D + k]);
      lo[k] = key < lo[k] ? key : lo[k];
      hi[k] = key > hi[k] ? key : hi[k];
    }
  }
  for (int k = 0; k < D; ++k) {
    for (int o = 16; o; o >>= 1) {
      const unsigned long long a = __shfl_down_sync(0xffffffffu, lo[k], o);
      const unsigned long long b = __shfl_down_sync(0xffffffffu, hi[k], o);
      lo[k] = a < lo[k] ? a : lo[k];
      hi[k] = b > hi[k] ? b : hi[k];
    }
    if ((threadIdx.x & 31) == 0) {
      atomicMin(mm + k, lo[k]);
      atomicMax(mm + 3 + k, hi[k]);
    }
  }
}

template <int D>
__global__ void k_outside(const double* xyz, long long n, double c0, double c1, double c2, double r0,
                          int* flag) {
  const double c[3] = {c0, c1, c2};
  const double rr = __dmul_rn(r0, r0);
  bool out = false;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    double d = 0.0;
    for (int k = 0; k < D; ++k) {
      const double t = __dsub_rn(c[k], xyz[i * D + k]);
      d = __dadd_rn(d, __dmul_rn(t, t));
    }
    out = out || !(d < rr);
  }
  if (__any_sync(0xffffffffu, out) && (threadIdx.x & 31) == 0) atomicOr(flag, 1);
}

// Slots left in the per-warp fresh-slot chunks of k_check are marked dead,
// so that every slot below nsimp is a simplex or a dead record.
__global__ void k_close_chunks(DevTree T) {
  for (int w = blockIdx.x * blockDim.x + threadIdx.x; w < T.cap_wchunk; w += gridDim.x * blockDim.x) {
    const int2 ch = T.wchunk[w];
    for (int k = 0; k < ch.y; ++k) {
      int4* p = reinterpret_cast<int4*>(T.simp + ch.x + k);
      p[0] = make_int4(-1, -1, -1, -1);
      p[1] = make_int4(-1, -1, -1, -1);
    }
    T.wchunk[w] = make_int2(0, 0);
  }
}

// ---- batched build ----------------------------------------------------------
// One block per set (grid-stride over sets); blockDim.x = 256.
template <int D>
__global__ void k_set_bbox(const double* xyz, const long long* off, int nsets, unsigned long long* mm) {
  __shared__ unsigned long long sh[8][6];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int s = blockIdx.x; s < nsets; s += gridDim.x) {
    unsigned long long lo[3] = {~0ull, ~0ull, ~0ull}, hi[3] = {0, 0, 0};
    for (long long i = off[s] + threadIdx.x; i < off[s + 1]; i += blockDim.x)
      for (int k = 0; k < D; ++k) {
        const unsigned long long key = dkey(xyz[i * D + k]);
        lo[k] = key < lo[k] ? key : lo[k];
        hi[k] = key > hi[k] ? key : hi[k];
      }
    for (int k = 0; k < D; ++k)
      for (int o = 16; o; o >>= 1) {
        const unsigned long long a = __shfl_down_sync(0xffffffffu, lo[k], o);
        const unsigned long long b = __shfl_down_sync(0xffffffffu, hi[k], o);
        lo[k] = a < lo[k] ? a : lo[k];
        hi[k] = b > hi[k] ? b : hi[k];
      }
    if (lane == 0)
      for (int k = 0; k < 3; ++k) {
        sh[warp][k] = lo[k];
        sh[warp][3 + k] = hi[k];
      }
    __syncthreads();
    if (threadIdx.x < 6) {
      const int k = threadIdx.x;
      unsigned long long r = sh[0][k];
      for (int w = 1; w < (int)(blockDim.x >> 5); ++w) r = k < 3 ? (sh[w][k] < r ? sh[w][k] : r) : (sh[w][k] > r ? sh[w][k] : r);
      mm[6LL * s + k] = r;
    }
    __syncthreads();
  }
}

template <int D>
__global__ void k_set_outside(const double* xyz, const long long* off, int nsets, const double* cr, int* flags) {
  for (int s = blockIdx.x; s < nsets; s += gridDim.x) {
    const double c[3] = {cr[4LL * s], cr[4LL * s + 1], cr[4LL * s + 2]};
    const double rr = __dmul_rn(cr[4LL * s + 3], cr[4LL * s + 3]);
    bool out = false;
    for (long long i = off[s] + threadIdx.x; i < off[s + 1]; i += blockDim.x) {
      double d = 0.0;
      for (int k = 0; k < D; ++k) {
        const double t = __dsub_rn(c[k], xyz[i * D + k]);
        d = __dadd_rn(d, __dmul_rn(t, t));
      }
      out = out || !(d < rr);
    }
    out = __syncthreads_or(out);
    if (threadIdx.x == 0) flags[s] = out ? 1 : 0;
  }
}

__global__ void k_set_fill(const long long* off, int nsets, int* set_of) {
  for (int s = blockIdx.x; s < nsets; s += gridDim.x)
    for (long long i = off[s] + threadIdx.x; i < off[s + 1]; i += blockDim.x) set_of[i] = s;
}

__global__ void k_localize(uint2* uv, long long m, const int* set_of, const long long* off) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < m; e += (long long)gridDim.x * blockDim.x) {
    uint2 p = uv[e];
    const unsigned base = (unsigned)off[set_of[p.x]];
    p.x -= base;
    p.y -= base;
    uv[e] = p;
  }
}

__global__ void k_set_edge_offsets(const int* uoff, const long long* off, int nsets, long long* eoff) {
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s <= nsets; s += gridDim.x * blockDim.x)
    eoff[s] = uoff[off[s]];
}

}  // namespace

void launch_set_bbox(const Launch& L, int dim, const double* d_xyz, const long long* off, int nsets,
                     unsigned long long* d_mm) {
  note_launches(1);
  const int g = std::min(nsets, L.blocks);
  if (dim == 3)
    k_set_bbox<3><<<g, 256, 0, L.stream>>>(d_xyz, off, nsets, d_mm);
  else
    k_set_bbox<2><<<g, 256, 0, L.stream>>>(d_xyz, off, nsets, d_mm);
}

void launch_set_outside(const Launch& L, int dim, const double* d_xyz, const long long* off, int nsets,
                        const double* cr, int* d_flags) {
  note_launches(1);
  const int g = std::min(nsets, L.blocks);
  if (dim == 3)
    k_set_outside<3><<<g, 256, 0, L.stream>>>(d_xyz, off, nsets, cr, d_flags);
  else
    k_set_outside<2><<<g, 256, 0, L.stream>>>(d_xyz, off, nsets, cr, d_flags);
}

void launch_set_fill(const Launch& L, const long long* off, int nsets, int* set_of) {
  note_launches(1);
  k_set_fill<<<std::min(nsets, L.blocks), 256, 0, L.stream>>>(off, nsets, set_of);
}

void launch_localize(const Launch& L, uint2* uv, int64_t m, const int* set_of, const long long* off) {
  if (m <= 0) return;
  note_launches(1);
  const int64_t b = std::min<int64_t>((m + 255) / 256, L.blocks);
  k_localize<<<(int)b, 256, 0, L.stream>>>(uv, m, set_of, off);
}

void launch_set_edge_offsets(const Launch& L, const int* uoff, const long long* off, int nsets,
                             long long* eoff) {
  note_launches(1);
  const int b = std::min((nsets + 256) / 256, L.blocks);
  k_set_edge_offsets<<<b, 256, 0, L.stream>>>(uoff, off, nsets, eoff);
}

void launch_bbox(const Launch& L, int dim, const double* d_xyz, int64_t n, unsigned long long* d_mm) {
  note_launches(1);
  if (dim == 3)
    k_bbox<3><<<L.blocks, 256, 0, L.stream>>>(d_xyz, n, d_mm);
  else
    k_bbox<2><<<L.blocks, 256, 0, L.stream>>>(d_xyz, n, d_mm);
}

void launch_outside(const Launch& L, int dim, const double* d_xyz, int64_t n, const double* c, double r0,
                    int* d_flag) {
  note_launches(1);
  if (dim == 3)
    k_outside<3><<<L.blocks, 256, 0, L.stream>>>(d_xyz, n, c[0], c[1], c[2], r0, d_flag);
  else
    k_outside<2><<<L.blocks, 256, 0, L.stream>>>(d_xyz, n, c[0], c[1], 0.0, r0, d_flag);
}

void launch_close_chunks(const DevTree& T, const Launch& L) {
  note_launches(1);
  k_close_chunks<<<(T.cap_wchunk + 255) / 256, 256, 0, L.stream>>>(T);
}

}  // namespace vd
