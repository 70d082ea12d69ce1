// Point location queries on a finished tree: the conflict region of a query
// point, i.e. the simplices whose circumsphere strictly contains it
// (`locate`, src/delaunay_tree.rs:33-58 with find_all_neighbors :60-75).
//
// One thread per query: a visibility walk from the finest location hint of
// the set to the simplex that contains the point, then a breadth-first
// search over face neighbours with the exact conflict test.  The query takes
// the role of the newest vertex (largest id), so a point exactly on a
// circumsphere is outside: the reference's strict `dist < r`.  The conflict
// region is connected, so the search finds all of it.
#include <cuda_runtime.h>

#include <algorithm>

#include "vd_common.cuh"

namespace vd {
namespace {

__device__ __forceinline__ int g4(const int4& v, int j) { return j == 0 ? v.x : j == 1 ? v.y : j == 2 ? v.z : v.w; }

__device__ __forceinline__ void load_simp(const DevTree& T, int s, int4& v, int4& n) {
  const int4* p = reinterpret_cast<const int4*>(T.simp + s);
  v = p[0];
  n = p[1];
}

template <int D>
__device__ __forceinline__ int hint_cell(const SetGeo& g, const vdp::VPt& p, int level) {
  const int side = 1 << level;
  const double c[3] = {p.x, p.y, p.z};
  int idx = 0;
  for (int k = D - 1; k >= 0; --k) {
    int i = (int)((c[k] - g.org[k]) * g.scale * side);
    i = i < 0 ? 0 : (i >= side ? side - 1 : i);
    idx = idx * side + i;
  }
  const int off = D == 3 ? ((1 << (3 * level)) - 1) / 7 : ((1 << (2 * level)) - 1) / 3;
  return g.hint_off + off + idx;
}

template <int D>
__global__ void k_locate(DevTree T, const double* q, int nq, int cap_per, const int* rank, int* out, int* counts) {
  constexpr int NV = D + 1;
  const int qkey = 0x7fffffff;  // newer than every vertex
  vdp::Tally tl = {0, 0, 0, 0};
  int perr = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nq; i += gridDim.x * blockDim.x) {
    const vdp::VPt p{q[(long long)i * D], q[(long long)i * D + 1], D == 3 ? q[(long long)i * D + 2] : 0.0, 0.0};
    const vdp::FPt fp = vdp::split_point(p.x, p.y, p.z);
    const SetGeo& g = T.sets[0];
    int cur = -1;
    for (int l = g.hint_levels; l >= 0 && cur < 0; --l) cur = T.hint[hint_cell<D>(g, p, l)];
    if (cur < 0 || bad_simp(T, cur)) cur = g.root;
    int4 v, nn;
    load_simp(T, cur, v, nn);
    for (int k = 0; k < 64 && v.x < 0 && nn.x >= 0; ++k) {  // dead slot: into its star
      cur = nn.x >> 2;
      if (bad_simp(T, cur)) break;
      load_simp(T, cur, v, nn);
    }
    int* o = out + (long long)i * cap_per;
    if (v.x < 0 || bad_simp(T, cur)) {
      set_error(T.ctr, E_INTERNAL);
      counts[i] = 0;
      continue;
    }
    // visibility walk
    bool outside = false;
    for (int step = 0; step < (1 << 16); ++step) {
      vdp::FPt fv[NV];
      for (int j = 0; j < NV; ++j) fv[j] = T.ptf[g4(v, j)];
      auto load64 = [&](vdp::VPt* v64, vdp::VPt& p64) {
        for (int j = 0; j < NV; ++j) v64[j] = T.pts[g4(v, j)];
        p64 = p;
      };
      const int f = vdp::exit_face_hl<D>(fv, fp, (1u << NV) - 1, tl, perr, load64);
      if (f < 0) break;
      const int code = g4(nn, f);
      if (code < 0 || bad_simp(T, code >> 2)) {
        outside = code < 0;
        break;
      }
      cur = code >> 2;
      load_simp(T, cur, v, nn);
    }
    if (outside) {
      counts[i] = -1;
      continue;
    }
    // breadth-first search of the conflict region (the containing simplex
    // is in it unless the point is one of its vertices)
    int cnt = 0;
    auto conflict = [&](int s, const int4& sv) {
      vdp::FPt fv[NV];
      int key[NV];
      for (int j = 0; j < NV; ++j) {
        key[j] = g4(sv, j);
        fv[j] = T.ptf[key[j]];
      }
      auto load64 = [&](vdp::VPt* v64, vdp::VPt& p64) {
        for (int j = 0; j < NV; ++j) v64[j] = T.pts[key[j]];
        p64 = p;
      };
      return vdp::in_conflict_hl<D>(fv, key, fp, qkey, tl, perr, load64);
    };
    if (conflict(cur, v)) {
      if (cap_per > 0) o[0] = cur;
      cnt = 1;
    }
    for (int h = 0; h < cnt && h < cap_per; ++h) {
      int4 cv, cn;
      load_simp(T, o[h], cv, cn);
      for (int f = 0; f < NV; ++f) {
        const int code = g4(cn, f);
        if (code < 0) continue;
        const int nb = code >> 2;
        if (bad_simp(T, nb)) continue;
        bool seen = false;
        for (int k = 0; k < cnt && k < cap_per && !seen; ++k) seen = o[k] == nb;
        if (seen) continue;
        int4 bv, bn;
        load_simp(T, nb, bv, bn);
        if (!conflict(nb, bv)) continue;
        if (cnt < cap_per) o[cnt] = nb;
        ++cnt;
      }
    }
    for (int k = 0; k < cnt && k < cap_per; ++k) o[k] = rank[o[k]];  // numbering of the simplex export
    counts[i] = cnt;
  }
  if (perr) set_error(T.ctr, E_PRECISION);
}

__global__ void k_live_flags(DevTree T, int nsimp, int* flags) {
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < nsimp; s += gridDim.x * blockDim.x)
    flags[s] = T.simp[s].v[0] >= 0 ? 1 : 0;
}

// Circumsphere of every live simplex, in the order of the simplex export
// (rank), for the dictionary view of the reference (PySimplex.center and
// .radius, src/lib.rs:32-59).  FP64 closed form relative to vertex 0:
// 3D c = p0 + (|a|^2 (b x c) + |b|^2 (c x a) + |c|^2 (a x b)) / (2 a.(b x c)),
// 2D the same in the plane.  These are floating-point values (the reference's
// own are too, src/geometry.rs:2-56); the triangulation never uses them.
template <int D>
__global__ void k_circum(DevTree T, int nsimp, const int* rank, double* centers, double* radii) {
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < nsimp; s += gridDim.x * blockDim.x) {
    const int4 v = reinterpret_cast<const int4*>(T.simp + s)[0];
    if (v.x < 0) continue;
    const int o = rank[s];
    const vdp::VPt p0 = T.pts[v.x], p1 = T.pts[v.y], p2 = T.pts[v.z];
    double cx, cy, cz = 0.0;
    if (D == 3) {
      const vdp::VPt p3 = T.pts[v.w];
      const double ax = p1.x - p0.x, ay = p1.y - p0.y, az = p1.z - p0.z;
      const double bx = p2.x - p0.x, by = p2.y - p0.y, bz = p2.z - p0.z;
      const double qx = p3.x - p0.x, qy = p3.y - p0.y, qz = p3.z - p0.z;
      const double a2 = ax * ax + ay * ay + az * az, b2 = bx * bx + by * by + bz * bz, q2 = qx * qx + qy * qy + qz * qz;
      const double bcx = by * qz - bz * qy, bcy = bz * qx - bx * qz, bcz = bx * qy - by * qx;
      const double cax = qy * az - qz * ay, cay = qz * ax - qx * az, caz = qx * ay - qy * ax;
      const double abx = ay * bz - az * by, aby = az * bx - ax * bz, abz = ax * by - ay * bx;
      const double den = 2.0 * (ax * bcx + ay * bcy + az * bcz);
      cx = (a2 * bcx + b2 * cax + q2 * abx) / den;
      cy = (a2 * bcy + b2 * cay + q2 * aby) / den;
      cz = (a2 * bcz + b2 * caz + q2 * abz) / den;
    } else {
      const double ax = p1.x - p0.x, ay = p1.y - p0.y, bx = p2.x - p0.x, by = p2.y - p0.y;
      const double a2 = ax * ax + ay * ay, b2 = bx * bx + by * by;
      const double den = 2.0 * (ax * by - ay * bx);
      cx = (by * a2 - ay * b2) / den;
      cy = (ax * b2 - bx * a2) / den;
    }
    centers[3LL * o] = p0.x + cx;
    centers[3LL * o + 1] = p0.y + cy;
    centers[3LL * o + 2] = D == 3 ? p0.z + cz : 0.0;
    radii[o] = sqrt(cx * cx + cy * cy + cz * cz);
  }
}

}  // namespace

void launch_circum(const DevTree& T, const Launch& L, int dim, int nsimp, const int* rank, double* centers,
                   double* radii) {
  note_launches(1);
  if (dim == 3)
    k_circum<3><<<L.blocks, 256, 0, L.stream>>>(T, nsimp, rank, centers, radii);
  else
    k_circum<2><<<L.blocks, 256, 0, L.stream>>>(T, nsimp, rank, centers, radii);
}

void launch_locate(const DevTree& T, const Launch& L, int dim, const double* d_q, int nq, int cap_per,
                   const int* rank, int* out, int* counts) {
  note_launches(1);
  const int blocks = std::max(1, std::min((nq + 127) / 128, L.blocks * 2));
  if (dim == 3)
    k_locate<3><<<blocks, 128, 0, L.stream>>>(T, d_q, nq, cap_per, rank, out, counts);
  else
    k_locate<2><<<blocks, 128, 0, L.stream>>>(T, d_q, nq, cap_per, rank, out, counts);
}

void launch_live_rank(const DevTree& T, const Launch& L, int nsimp, int* flags, int* rank, int* tmp) {
  note_launches(1);
  k_live_flags<<<L.blocks, 256, 0, L.stream>>>(T, nsimp, flags);
  scan_ints(flags, rank, nsimp, tmp, L.stream);
}

}  // namespace vd
