// Exact validator of a device tree: replaces `check_delaunay`
// (src/delaunay_tree.rs:512-541 3D, :642-671 2D), which compares every
// vertex against every simplex's floating circumsphere (O(S*V)) and only for
// simplices without super vertices.  Here every simplex and every facet is
// checked once, exactly:
//   - each simplex is positively oriented;
//   - adjacency is symmetric (n[f] of s points at (o, g) and n[g] of o back);
//   - local Delaunay: the vertex of o opposite the shared facet is not
//     strictly inside the circumsphere of s (unperturbed exact sign), and is
//     outside in the perturbed sense (the unique triangulation built here).
// Locally Delaunay everywhere implies globally Delaunay (Delaunay's lemma).
#include <cuda_runtime.h>

#include "../../include/voronoids_gpu.h"
#include "vd_common.cuh"

namespace vd {
namespace {

template <int D>
__global__ void k_check(DevTree T, int nsimp, unsigned long long* out) {
  constexpr int NV = D + 1;
  vdp::Tally tl = {0, 0, 0, 0};
  int perr = 0;
  unsigned long long nonpos = 0, asym = 0, notdel = 0, notpert = 0, hull = 0, facets = 0;
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < nsimp; s += gridDim.x * blockDim.x) {
    const int4 v = reinterpret_cast<const int4*>(T.simp + s)[0];
    const int4 n = reinterpret_cast<const int4*>(T.simp + s)[1];
    if (v.x < 0) continue;
    const int va[4] = {v.x, v.y, v.z, v.w};
    const int na[4] = {n.x, n.y, n.z, n.w};
    vdp::VPt p[NV];
    bool badv = false;
    for (int j = 0; j < NV; ++j) badv = badv || bad_vert(T, va[j]);
    if (badv) {
      ++asym;
      continue;
    }
    for (int j = 0; j < NV; ++j) {
      const double4_32a a = reinterpret_cast<const double4_32a*>(T.pts)[va[j]];
      p[j] = vdp::VPt{a.x, a.y, a.z, a.w};
    }
    // orientation of the simplex itself: o_D with p_D replaced by p_D
    if (vdp::exit_face<D, true>(p, p[D], 1u << D, tl, perr) >= 0) ++nonpos;
    for (int f = 0; f < NV; ++f) {
      const int code = na[f];
      if (code < 0) {
        ++hull;
        continue;
      }
      const int o = code >> 2, g = code & 3;
      if (bad_simp(T, o)) {
        ++asym;
        continue;
      }
      const int back = reinterpret_cast<const int*>(T.simp + o)[4 + g];
      const int opp = reinterpret_cast<const int*>(T.simp + o)[g];
      if (back != ((s << 2) | f) || opp < 0 || bad_vert(T, opp)) {
        ++asym;
        continue;
      }
      if (o < s) continue;
      ++facets;
      const double4_32a a = reinterpret_cast<const double4_32a*>(T.pts)[opp];
      const vdp::VPt q{a.x, a.y, a.z, a.w};
      if (vdp::insphere_sign<D>(p, q, tl, perr) > 0) ++notdel;
      if (vdp::in_conflict<D>(p, va, q, opp, tl, perr)) ++notpert;
    }
  }
  const unsigned FULL = 0xffffffffu;
  unsigned long long vals[6] = {nonpos, asym, notdel, notpert, hull, facets};
  for (int k = 0; k < 6; ++k) {
    unsigned long long x = vals[k];
    for (int o = 16; o; o >>= 1) x += __shfl_down_sync(FULL, x, o);
    if ((threadIdx.x & 31) == 0 && x) atomicAdd(out + k, x);
  }
  if (perr) set_error(T.ctr, E_PRECISION);
}

// Caller triangulation -> device records: vertex i of `xyz` (dim doubles) as
// a 32-byte (x, y, z | 0, 0) record.
template <int D>
__global__ void k_pack_points(const double* xyz, long long n, double4_32a* out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    out[i] = make_double4_32a(xyz[i * D], xyz[i * D + 1], D == 3 ? xyz[i * D + 2] : 0.0, 0.0);
}

// Plain neighbour ids -> face codes (o << 2 | g, g the face of o whose
// neighbour is s).  A structural fault is kept visible to k_check instead of
// being repaired: a vertex id outside [0, npts) becomes npts (k_check counts
// it as a structural violation), a neighbour id outside [0, ns) becomes the
// out-of-range code ns << 2, and a neighbour with no face pointing back gets
// a face whose link does not point back either (counted as asymmetric).
template <int D>
__global__ void k_face_codes(const int4* verts, const int4* nbrs, int ns, int npts, Simplex* out) {
  constexpr int NV = D + 1;
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < ns; s += gridDim.x * blockDim.x) {
    const int4 v = verts[s], n = nbrs[s];
    int va[4] = {v.x, v.y, v.z, v.w}, na[4] = {n.x, n.y, n.z, n.w}, code[4] = {-1, -1, -1, -1};
    for (int j = 0; j < NV; ++j)
      if (va[j] < 0 || va[j] >= npts) va[j] = npts;
    if (D == 2) va[3] = -1;
    for (int f = 0; f < NV; ++f) {
      const int o = na[f];
      if (o == -1) continue;
      if (o < 0 || o >= ns) {
        code[f] = ns << 2;
        continue;
      }
      const int4 b = nbrs[o];
      const int ba[4] = {b.x, b.y, b.z, b.w};
      int g = 0;
      while (g < NV && ba[g] != s) ++g;
      if (g == NV) g = 0;  // no face of o points back, so neither does face 0
      code[f] = (o << 2) | g;
    }
    Simplex r;
    for (int j = 0; j < 4; ++j) {
      r.v[j] = va[j];
      r.n[j] = code[j];
    }
    out[s] = r;
  }
}

}  // namespace

void launch_check(const DevTree& T, const Launch& L, int dim, int nsimp, unsigned long long* d_out) {
  note_launches(1);
  cudaMemsetAsync(d_out, 0, 6 * sizeof(unsigned long long), L.stream);
  if (dim == 3)
    k_check<3><<<L.blocks, 256, 0, L.stream>>>(T, nsimp, d_out);
  else
    k_check<2><<<L.blocks, 256, 0, L.stream>>>(T, nsimp, d_out);
}

}  // namespace vd

// ---------------------------------------------------------------------------
// check_delaunay on a caller's triangulation (see include/voronoids_gpu.h).
extern "C" int vd_check_triangulation(int dim, const double* pts, int64_t npts, const int32_t* verts,
                                      const int32_t* nbrs, int64_t ns, int* ok, int64_t* violations) {
  using namespace vd;
  if ((dim != 2 && dim != 3) || !ok || npts < 0 || ns < 0 || npts > 0x7ffffff0LL || ns >= (int64_t(1) << 29) ||
      (npts > 0 && !pts) || (ns > 0 && (!verts || !nbrs)))
    return VD_ERR_ARG;
  *ok = 0;
  int dev = 0, sms = 1;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return VD_ERR_CUDA;
  double* d_xyz = nullptr;
  double4_32a* d_pts = nullptr;
  int4 *d_v = nullptr, *d_n = nullptr;
  Simplex* d_simp = nullptr;
  Counters* d_ctr = nullptr;
  unsigned long long* d_out = nullptr;
  cudaStream_t st = nullptr;
  int rc = VD_OK;
  const size_t np = (size_t)std::max<int64_t>(npts, 1), nsz = (size_t)std::max<int64_t>(ns, 1);
  if (cudaMalloc((void**)&d_xyz, sizeof(double) * dim * np) != cudaSuccess ||
      cudaMalloc((void**)&d_pts, sizeof(double4_32a) * np) != cudaSuccess ||
      cudaMalloc((void**)&d_v, sizeof(int4) * nsz) != cudaSuccess ||
      cudaMalloc((void**)&d_n, sizeof(int4) * nsz) != cudaSuccess ||
      cudaMalloc((void**)&d_simp, sizeof(Simplex) * nsz) != cudaSuccess ||
      cudaMalloc((void**)&d_ctr, sizeof(Counters)) != cudaSuccess ||
      cudaMalloc((void**)&d_out, 6 * sizeof(unsigned long long)) != cudaSuccess)
    rc = VD_ERR_NOMEM;
  if (rc == VD_OK && cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) rc = VD_ERR_CUDA;
  unsigned long long h[6] = {0, 0, 0, 0, 0, 0};
  Counters hc;
  memset(&hc, 0, sizeof(hc));
  if (rc == VD_OK) {
    bool good = cudaMemsetAsync(d_ctr, 0, sizeof(Counters), st) == cudaSuccess;
    if (npts > 0)
      good = good && cudaMemcpyAsync(d_xyz, pts, sizeof(double) * dim * npts, cudaMemcpyHostToDevice, st) == cudaSuccess;
    if (ns > 0)
      good = good && cudaMemcpyAsync(d_v, verts, sizeof(int4) * ns, cudaMemcpyHostToDevice, st) == cudaSuccess &&
             cudaMemcpyAsync(d_n, nbrs, sizeof(int4) * ns, cudaMemcpyHostToDevice, st) == cudaSuccess;
    Launch L;
    L.blocks = sms * 8;
    L.warps = sms * 20;
    L.stream = st;
    if (good) {
      note_launches(2);
      if (dim == 3) {
        k_pack_points<3><<<L.blocks, 256, 0, st>>>(d_xyz, npts, d_pts);
        k_face_codes<3><<<L.blocks, 256, 0, st>>>(d_v, d_n, (int)ns, (int)npts, d_simp);
      } else {
        k_pack_points<2><<<L.blocks, 256, 0, st>>>(d_xyz, npts, d_pts);
        k_face_codes<2><<<L.blocks, 256, 0, st>>>(d_v, d_n, (int)ns, (int)npts, d_simp);
      }
      DevTree T;
      memset(&T, 0, sizeof(T));
      T.pts = reinterpret_cast<vdp::VPt*>(d_pts);
      T.simp = d_simp;
      T.ctr = d_ctr;
      T.nsets = 1;
      T.cap_simp = (int)ns;
      T.cap_verts = (int)npts;
      launch_check(T, L, dim, (int)ns, d_out);
      good = cudaGetLastError() == cudaSuccess &&
             cudaMemcpyAsync(h, d_out, sizeof(h), cudaMemcpyDeviceToHost, st) == cudaSuccess &&
             cudaMemcpyAsync(&hc, d_ctr, sizeof(hc), cudaMemcpyDeviceToHost, st) == cudaSuccess;
    }
    if (cudaStreamSynchronize(st) != cudaSuccess || !good) rc = VD_ERR_CUDA;
  }
  if (st) cudaStreamDestroy(st);
  cudaFree(d_xyz);
  cudaFree(d_pts);
  cudaFree(d_v);
  cudaFree(d_n);
  cudaFree(d_simp);
  cudaFree(d_ctr);
  cudaFree(d_out);
  if (rc != VD_OK) return rc;
  if (violations)
    for (int k = 0; k < 6; ++k) violations[k] = (int64_t)h[k];
  *ok = (h[0] == 0 && h[1] == 0 && h[2] == 0 && h[3] == 0) ? 1 : 0;
  return hc.err ? hc.err : VD_OK;
}
