// Host build of the device predicate tiers, exported for CPU tests.
// The same header is compiled for sm_103a into the device library; here it
// is compiled by the host compiler with -ffp-contract=off.
#include <stdint.h>

#include "vd_predicates.cuh"

namespace {
vdp::VPt at(const double* p, int i) { return vdp::VPt{p[3 * i], p[3 * i + 1], p[3 * i + 2], 0.0}; }
}  // namespace

extern "C" {

// pts: dim+2 xyz triples (simplex, then query); keys: dim+2 ints.
// tier_out (may be NULL): 0 f32, 1 f64, 2 exact.  Returns +1 conflict, -1 not.
int vdh_in_conflict(int dim, const double* pts, const int* keys, int* tier_out, int* err_out) {
  vdp::VPt p[4];
  for (int i = 0; i <= dim; ++i) p[i] = at(pts, i);
  vdp::VPt q = at(pts, dim + 1);
  vdp::Tally t = {0, 0, 0, 0};
  int err = 0;
  bool c = dim == 3 ? vdp::in_conflict<3>(p, keys, q, keys[dim + 1], t, err)
                    : vdp::in_conflict<2>(p, keys, q, keys[dim + 1], t, err);
  if (tier_out) *tier_out = t.f32 ? 0 : (t.f64 ? 1 : 2);
  if (err_out) *err_out = err;
  return c ? 1 : -1;
}

// Exact tier only (perturbed when sos != 0): the integer evaluation first,
// then the expansions.
int vdh_insphere_exact(int dim, const double* pts, const int* keys, int sos, int* err_out) {
  vdp::VPt p[4];
  for (int i = 0; i <= dim; ++i) p[i] = at(pts, i);
  vdp::VPt q = at(pts, dim + 1);
  int err = 0;
  int s = dim == 3 ? vdp::exact_insphere_sos<3>(p, keys, q, keys[dim + 1], err, sos != 0)
                   : vdp::exact_insphere_sos<2>(p, keys, q, keys[dim + 1], err, sos != 0);
  if (err_out) *err_out = err;
  return s;
}

// The expansion form of the exact tier alone (the form of kernels that keep
// their register allocation small).
int vdh_insphere_exact_expansion(int dim, const double* pts, const int* keys, int sos, int* err_out) {
  vdp::VPt p[4];
  for (int i = 0; i <= dim; ++i) p[i] = at(pts, i);
  vdp::VPt q = at(pts, dim + 1);
  int err = 0;
  int s = dim == 3 ? vdp::exact_insphere_sos<3, 0>(p, keys, q, keys[dim + 1], err, sos != 0)
                   : vdp::exact_insphere_sos<2, 0>(p, keys, q, keys[dim + 1], err, sos != 0);
  if (err_out) *err_out = err;
  return s;
}

// Face of simplex v (dim+1 points) that p is strictly behind (first one), or -1.
int vdh_exit_face(int dim, const double* pts, unsigned mask, int strict, int* err_out) {
  vdp::VPt v[4];
  for (int i = 0; i <= dim; ++i) v[i] = at(pts, i);
  vdp::VPt p = at(pts, dim + 1);
  vdp::Tally t = {0, 0, 0, 0};
  int err = 0, f;
  if (dim == 3)
    f = strict ? vdp::exit_face<3, true>(v, p, mask, t, err) : vdp::exit_face<3>(v, p, mask, t, err);
  else
    f = strict ? vdp::exit_face<2, true>(v, p, mask, t, err) : vdp::exit_face<2>(v, p, mask, t, err);
  if (err_out) *err_out = err;
  return f;
}

// Exact orient sign of dim+1 points via the exact tier (det of rows a_k - last).
int vdh_orient_exact(int dim, const double* pts, int* err_out) {
  int err = 0, s;
  if (dim == 3)
    s = vdp::exact_orient3(at(pts, 0), at(pts, 1), at(pts, 2), at(pts, 3), err);
  else
    s = vdp::exact_orient2(at(pts, 0), at(pts, 1), at(pts, 2), err);
  if (err_out) *err_out = err;
  return s;
}

}  // extern "C"

extern "C" {

// Split-coordinate tier followed by the FP64/exact tiers, as the device uses it.
int vdh_in_conflict_hl(int dim, const double* pts, const int* keys, int* tier_out, int* err_out) {
  vdp::VPt p[4];
  vdp::FPt f[4];
  for (int i = 0; i <= dim; ++i) {
    p[i] = at(pts, i);
    f[i] = vdp::split_point(p[i].x, p[i].y, p[i].z);
  }
  vdp::VPt q = at(pts, dim + 1);
  vdp::FPt fq = vdp::split_point(q.x, q.y, q.z);
  vdp::Tally t = {0, 0, 0, 0};
  int err = 0;
  auto load = [&](vdp::VPt* v, vdp::VPt& qq) {
    for (int i = 0; i <= dim; ++i) v[i] = p[i];
    qq = q;
  };
  bool c = dim == 3 ? vdp::in_conflict_hl<3>(f, keys, fq, keys[dim + 1], t, err, load)
                    : vdp::in_conflict_hl<2>(f, keys, fq, keys[dim + 1], t, err, load);
  if (tier_out) *tier_out = t.f32 ? 0 : (t.f64 ? 1 : 2);
  if (err_out) *err_out = err;
  return c ? 1 : -1;
}

// Split-coordinate f32 tier alone: +1/-1 certified, 0 undecided.
int vdh_insphere_hl(int dim, const double* pts) {
  vdp::FPt f[4];
  for (int i = 0; i <= dim; ++i) f[i] = vdp::split_point(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]);
  const int k = dim + 1;
  vdp::FPt fq = vdp::split_point(pts[3 * k], pts[3 * k + 1], pts[3 * k + 2]);
  return dim == 3 ? vdp::insphere_hl<3>(f, fq) : vdp::insphere_hl<2>(f, fq);
}

int vdh_exit_face_hl(int dim, const double* pts, unsigned mask, int strict, int* err_out) {
  vdp::VPt v[4];
  vdp::FPt f[4];
  for (int i = 0; i <= dim; ++i) {
    v[i] = at(pts, i);
    f[i] = vdp::split_point(v[i].x, v[i].y, v[i].z);
  }
  vdp::VPt p = at(pts, dim + 1);
  vdp::FPt fp = vdp::split_point(p.x, p.y, p.z);
  vdp::Tally t = {0, 0, 0, 0};
  int err = 0, r;
  auto load = [&](vdp::VPt* vv, vdp::VPt& pp) {
    for (int i = 0; i <= dim; ++i) vv[i] = v[i];
    pp = p;
  };
  if (dim == 3)
    r = strict ? vdp::exit_face_hl<3, true>(f, fp, mask, t, err, load) : vdp::exit_face_hl<3>(f, fp, mask, t, err, load);
  else
    r = strict ? vdp::exit_face_hl<2, true>(f, fp, mask, t, err, load) : vdp::exit_face_hl<2>(f, fp, mask, t, err, load);
  if (err_out) *err_out = err;
  return r;
}

}  // extern "C"
