// Voronoi dual of a finished tree.
//
// The reference's purpose is the Voronoi tessellation (README.md:2-4,
// Cargo.toml:6), but it stores only the Voronoi vertices: the circumcentre
// and radius of every simplex (Simplex::center / radius,
// src/delaunay_tree.rs:10-17, computed by src/geometry.rs:2-56).  Here the
// rest of the dual comes from the final simplex pool:
//
//   Voronoi vertices  the circumcentres of the live simplices (vd_circum in
//                     vd_locate.cu), numbered as the simplices are exported;
//   Voronoi edges     one per interior facet: the two live simplices that
//                     share it, (i, j) with i < j, sorted (a face pointing at
//                     the super-simplex hull has no second simplex);
//   Voronoi cells     per input vertex, the sorted live simplices incident to
//                     it: the vertices of the vertex's cell.
//
// Edges: every live slot counts its faces whose neighbour has a larger slot,
// a scan over the live ranks places them, and each slot writes its (at most
// D + 1) pairs in order of the neighbour's rank; ranks grow with slots, so
// the list comes out sorted.  Cells: incidences are bucketed by vertex
// (count, scan, scatter) and every bucket is sorted with the edge
// extraction's bucket sort.
#include <cuda_runtime.h>

#include "vd_common.cuh"

namespace vd {
namespace {

template <int D>
__global__ void k_dual_count(DevTree T, int nsimp, const int* rank, int* cnt) {
  constexpr int NV = D + 1;
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < nsimp; s += gridDim.x * blockDim.x) {
    const int4 v = reinterpret_cast<const int4*>(T.simp + s)[0];
    if (v.x < 0) continue;
    const int4 n = reinterpret_cast<const int4*>(T.simp + s)[1];
    const int na[4] = {n.x, n.y, n.z, n.w};
    int c = 0;
    for (int f = 0; f < NV; ++f) {
      const int code = na[f];
      if (code < 0) continue;
      const int o = code >> 2;
      if (bad_simp(T, o) || o >= nsimp) {
        set_error(T.ctr, E_INTERNAL);
        continue;
      }
      c += o > s;
    }
    cnt[rank[s]] = c;
  }
}

template <int D>
__global__ void k_dual_fill(DevTree T, int nsimp, const int* rank, const int* off, int2* out) {
  constexpr int NV = D + 1;
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < nsimp; s += gridDim.x * blockDim.x) {
    const int4 v = reinterpret_cast<const int4*>(T.simp + s)[0];
    if (v.x < 0) continue;
    const int4 n = reinterpret_cast<const int4*>(T.simp + s)[1];
    const int na[4] = {n.x, n.y, n.z, n.w};
    int r[4], c = 0;
    for (int f = 0; f < NV; ++f) {
      const int code = na[f];
      if (code < 0) continue;
      const int o = code >> 2;
      if (bad_simp(T, o) || o >= nsimp || o <= s) continue;
      // insertion into the sorted list of this slot's partners
      int k = c++;
      const int ro = rank[o];
      while (k > 0 && r[k - 1] > ro) {
        r[k] = r[k - 1];
        --k;
      }
      r[k] = ro;
    }
    const int rs = rank[s], b = off[rs];
    for (int k = 0; k < c; ++k) out[b + k] = make_int2(rs, r[k]);
  }
}

template <int D>
__global__ void k_cell_count(DevTree T, int nsimp, int n_in, int* cnt) {
  constexpr int NV = D + 1;
  const int NS = T.nsuper;
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < nsimp; s += gridDim.x * blockDim.x) {
    const int4 v = reinterpret_cast<const int4*>(T.simp + s)[0];
    if (v.x < 0) continue;
    const int a[4] = {v.x, v.y, v.z, v.w};
    for (int j = 0; j < NV; ++j) {
      const int u = a[j] - NS;
      if (a[j] < NS) continue;
      if (u >= n_in) {
        set_error(T.ctr, E_INTERNAL);
        continue;
      }
      atomicAdd(cnt + u, 1);
    }
  }
}

template <int D>
__global__ void k_cell_fill(DevTree T, int nsimp, int n_in, const int* rank, int* cnt, const int* off, int* buf) {
  constexpr int NV = D + 1;
  const int NS = T.nsuper;
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < nsimp; s += gridDim.x * blockDim.x) {
    const int4 v = reinterpret_cast<const int4*>(T.simp + s)[0];
    if (v.x < 0) continue;
    const int a[4] = {v.x, v.y, v.z, v.w};
    const int rs = rank[s];
    for (int j = 0; j < NV; ++j) {
      const int u = a[j] - NS;
      if (a[j] < NS || u >= n_in) continue;
      const int k = atomicSub(cnt + u, 1) - 1;  // counts return to zero
      if (k >= 0) buf[off[u] + k] = rs;
    }
  }
}

}  // namespace

void launch_dual_edges(const DevTree& T, const Launch& L, int dim, int nsimp, const int* rank, int* cnt, int* off,
                       int* tmp, int nlive, int2* out, bool fill) {
  cudaStream_t st = L.stream;
  if (!fill) {
    note_launches(1);
    if (dim == 3)
      k_dual_count<3><<<L.blocks, 256, 0, st>>>(T, nsimp, rank, cnt);
    else
      k_dual_count<2><<<L.blocks, 256, 0, st>>>(T, nsimp, rank, cnt);
    scan_ints(cnt, off, nlive, tmp, st);
    return;
  }
  note_launches(1);
  if (dim == 3)
    k_dual_fill<3><<<L.blocks, 256, 0, st>>>(T, nsimp, rank, off, out);
  else
    k_dual_fill<2><<<L.blocks, 256, 0, st>>>(T, nsimp, rank, off, out);
}

void launch_cell_count(const DevTree& T, const Launch& L, int dim, int nsimp, int n_in, int* cnt, int* off,
                       int* tmp) {
  cudaStream_t st = L.stream;
  cudaMemsetAsync(cnt, 0, sizeof(int) * (n_in + 1), st);
  note_launches(1);
  if (dim == 3)
    k_cell_count<3><<<L.blocks, 256, 0, st>>>(T, nsimp, n_in, cnt);
  else
    k_cell_count<2><<<L.blocks, 256, 0, st>>>(T, nsimp, n_in, cnt);
  scan_ints(cnt, off, n_in, tmp, st);
}

void launch_cell_fill(const DevTree& T, const Launch& L, int dim, int nsimp, int n_in, const int* rank, int* cnt,
                      const int* off, int* buf) {
  note_launches(1);
  if (dim == 3)
    k_cell_fill<3><<<L.blocks, 256, 0, L.stream>>>(T, nsimp, n_in, rank, cnt, off, buf);
  else
    k_cell_fill<2><<<L.blocks, 256, 0, L.stream>>>(T, nsimp, n_in, rank, cnt, off, buf);
}

}  // namespace vd
