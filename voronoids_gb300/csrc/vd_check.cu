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
