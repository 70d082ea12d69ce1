// CPU oracle for the GB300 Delaunay build -- TEST INFRASTRUCTURE ONLY.
//
// Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load
// this library.  It restates, sequentially and with exact arithmetic, the
// semantics of the reference crate kazewong/Voronoids:
//
//   bounding_sphere            src/geometry.rs:99-142     (bit-exact restatement)
//   DelaunayTree<3,4>::new     src/delaunay_tree.rs:389-510 (super vertices)
//   DelaunayTree<2,3>::new     src/delaunay_tree.rs:544-640
//   circumsphere_2d / _3d      src/geometry.rs:2-56       (float variant, diagnostics)
//   in_sphere (strict)         src/geometry.rs:91-97      (exact + strict)
//   locate / find_all_neighbors src/delaunay_tree.rs:33-75 (conflict region by BFS)
//   get_new_simplices          src/delaunay_tree.rs:77-123 (star from boundary facets)
//   pair_simplices             src/delaunay_tree.rs:674-695 (intra-star adjacency)
//   insert_point               src/delaunay_tree.rs:125-211 (apply one insertion)
//   check_delaunay             src/delaunay_tree.rs:512-541, 642-671 (validator)
//
// Differences from the reference, all deliberate:
//  * predicates are exact (f64 filter, then big-integer arithmetic) instead of
//    a floating circumcenter; a point exactly on a circumsphere is resolved by
//    the perturbation rule (larger vertex id = larger lift perturbation),
//    which equals the reference's strict `<` whenever the query is the newest
//    vertex, i.e. for its sequential input-order insertion;
//  * point location walks from the last created simplex instead of the kd-tree
//    nearest vertex (location picks the start of the BFS only; the conflict
//    region it finds is the same set);
//  * duplicate points are skipped (the reference panics, src/delaunay_tree.rs:53);
//    of a group of equal points the one with the smallest insertion priority
//    is kept;
//  * ghost simplices are represented as "no neighbour" (-1) across the
//    super-simplex hull; they never conflict in the reference either.
//
// The big-integer path is written independently of the device code's
// floating-point expansions so that the two exact methods check each other.
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <atomic>
#include <condition_variable>
#include <functional>
#include <mutex>
#include <map>
#include <thread>
#include <unordered_map>
#include <vector>

namespace {

// ---------------------------------------------------------------------------
// Big integers (sign + magnitude, base 2^32).
// ---------------------------------------------------------------------------
struct Big {
  int sign = 0;                 // -1, 0, +1
  std::vector<uint32_t> mag;    // little endian, no leading zero limbs
};

void trim(std::vector<uint32_t>& m) {
  while (!m.empty() && m.back() == 0) m.pop_back();
}

int cmp_mag(const std::vector<uint32_t>& a, const std::vector<uint32_t>& b) {
  if (a.size() != b.size()) return a.size() < b.size() ? -1 : 1;
  for (size_t i = a.size(); i-- > 0;)
    if (a[i] != b[i]) return a[i] < b[i] ? -1 : 1;
  return 0;
}

std::vector<uint32_t> add_mag(const std::vector<uint32_t>& a, const std::vector<uint32_t>& b) {
  std::vector<uint32_t> r(std::max(a.size(), b.size()) + 1, 0);
  uint64_t carry = 0;
  for (size_t i = 0; i < r.size(); ++i) {
    uint64_t s = carry;
    if (i < a.size()) s += a[i];
    if (i < b.size()) s += b[i];
    r[i] = (uint32_t)s;
    carry = s >> 32;
  }
  trim(r);
  return r;
}

// a - b with |a| >= |b|
std::vector<uint32_t> sub_mag(const std::vector<uint32_t>& a, const std::vector<uint32_t>& b) {
  std::vector<uint32_t> r(a.size(), 0);
  int64_t borrow = 0;
  for (size_t i = 0; i < a.size(); ++i) {
    int64_t s = (int64_t)a[i] - borrow - (i < b.size() ? (int64_t)b[i] : 0);
    borrow = 0;
    if (s < 0) {
      s += ((int64_t)1 << 32);
      borrow = 1;
    }
    r[i] = (uint32_t)s;
  }
  trim(r);
  return r;
}

Big badd(const Big& a, const Big& b) {
  if (a.sign == 0) return b;
  if (b.sign == 0) return a;
  Big r;
  if (a.sign == b.sign) {
    r.sign = a.sign;
    r.mag = add_mag(a.mag, b.mag);
    return r;
  }
  int c = cmp_mag(a.mag, b.mag);
  if (c == 0) return r;
  if (c > 0) {
    r.sign = a.sign;
    r.mag = sub_mag(a.mag, b.mag);
  } else {
    r.sign = b.sign;
    r.mag = sub_mag(b.mag, a.mag);
  }
  return r;
}

Big bneg(Big a) {
  a.sign = -a.sign;
  return a;
}
Big bsub(const Big& a, const Big& b) { return badd(a, bneg(b)); }

Big bmul(const Big& a, const Big& b) {
  Big r;
  if (a.sign == 0 || b.sign == 0) return r;
  std::vector<uint64_t> acc(a.mag.size() + b.mag.size() + 1, 0);
  std::vector<uint32_t> m(a.mag.size() + b.mag.size() + 1, 0);
  for (size_t i = 0; i < a.mag.size(); ++i) {
    uint64_t carry = 0;
    for (size_t j = 0; j < b.mag.size(); ++j) {
      uint64_t cur = (uint64_t)a.mag[i] * b.mag[j] + m[i + j] + carry;
      m[i + j] = (uint32_t)cur;
      carry = cur >> 32;
    }
    size_t k = i + b.mag.size();
    while (carry) {
      uint64_t cur = (uint64_t)m[k] + carry;
      m[k] = (uint32_t)cur;
      carry = cur >> 32;
      ++k;
    }
  }
  trim(m);
  r.mag = m;
  r.sign = a.sign * b.sign;
  return r;
}

// Exact value x * 2^-emin as a big integer (x = mant * 2^e, e >= emin).
Big from_double(double x, int emin) {
  Big r;
  if (x == 0.0) return r;
  int k;
  double f = std::frexp(std::fabs(x), &k);
  uint64_t m = (uint64_t)std::ldexp(f, 53);
  int e = k - 53;
  int sh = e - emin;
  // m << sh
  std::vector<uint32_t> mag;
  int limbs = sh / 32, bits = sh % 32;
  mag.assign(limbs, 0);
  unsigned __int128 v = (unsigned __int128)m << bits;
  while (v) {
    mag.push_back((uint32_t)v);
    v >>= 32;
  }
  trim(mag);
  r.mag = mag;
  r.sign = x > 0 ? 1 : -1;
  return r;
}

int low_exponent(double x) {
  int k;
  std::frexp(std::fabs(x), &k);
  return k - 53;
}

// ---------------------------------------------------------------------------
// Exact predicates.  Points are given as raw coordinates; differences are
// formed exactly in big integers after aligning all inputs to a common
// binary exponent.
// ---------------------------------------------------------------------------
struct P3 {
  double x, y, z;
};

int emin_of(const P3* p, int n) {
  int em = 1 << 30;
  for (int i = 0; i < n; ++i) {
    const double c[3] = {p[i].x, p[i].y, p[i].z};
    for (double v : c)
      if (v != 0.0) em = std::min(em, low_exponent(v));
  }
  return em == (1 << 30) ? 0 : em;
}

// det2 rows (a, b)
Big bdet2(const Big& ax, const Big& ay, const Big& bx, const Big& by) {
  return bsub(bmul(ax, by), bmul(ay, bx));
}

// det3 rows (a, b, c)
Big bdet3(const Big* x, const Big* y, const Big* z, int a, int b, int c) {
  Big t1 = bmul(z[a], bdet2(x[b], y[b], x[c], y[c]));
  Big t2 = bmul(z[b], bdet2(x[a], y[a], x[c], y[c]));
  Big t3 = bmul(z[c], bdet2(x[a], y[a], x[b], y[b]));
  return badd(bsub(t1, t2), t3);
}

// O_i = orient(T with p_i replaced by q) for the simplex p[0..dim], all
// exactly, plus the exact lifted determinant sum_i |p_i - q|^2 O_i.
void exact_lifted(int dim, const P3* p, const P3& q, int* osign, int* detsign) {
  P3 all[5];
  int nv = dim + 1;
  for (int i = 0; i < nv; ++i) all[i] = p[i];
  all[nv] = q;
  int em = emin_of(all, nv + 1);
  Big qx = from_double(q.x, em), qy = from_double(q.y, em), qz = from_double(q.z, em);
  Big x[4], y[4], z[4];
  for (int i = 0; i < nv; ++i) {
    x[i] = bsub(from_double(p[i].x, em), qx);
    y[i] = bsub(from_double(p[i].y, em), qy);
    z[i] = bsub(from_double(p[i].z, em), qz);
  }
  Big det;
  for (int i = 0; i < nv; ++i) {
    int o[3], t = 0;
    for (int k = 0; k < nv; ++k)
      if (k != i) o[t++] = k;
    Big Oi;
    if (dim == 3) {
      Oi = bdet3(x, y, z, o[0], o[1], o[2]);
      if (!(i & 1)) Oi = bneg(Oi);
    } else {
      Oi = bdet2(x[o[0]], y[o[0]], x[o[1]], y[o[1]]);
      if (i & 1) Oi = bneg(Oi);
    }
    osign[i] = Oi.sign;
    Big w = badd(bmul(x[i], x[i]), bmul(y[i], y[i]));
    if (dim == 3) w = badd(w, bmul(z[i], z[i]));
    det = badd(det, bmul(w, Oi));
  }
  *detsign = det.sign;
}

// orient of (p[0..dim]) in the repository's convention:
// 3D det[a-d; b-d; c-d], 2D det[a-c; b-c]
int exact_orient(int dim, const P3* p) {
  int nv = dim + 1;
  int em = emin_of(p, nv);
  const P3& o = p[dim];
  Big ox = from_double(o.x, em), oy = from_double(o.y, em), oz = from_double(o.z, em);
  Big x[3], y[3], z[3];
  for (int i = 0; i < dim; ++i) {
    x[i] = bsub(from_double(p[i].x, em), ox);
    y[i] = bsub(from_double(p[i].y, em), oy);
    z[i] = bsub(from_double(p[i].z, em), oz);
  }
  if (dim == 3) return bdet3(x, y, z, 0, 1, 2).sign;
  return bdet2(x[0], y[0], x[1], y[1]).sign;
}

// f64 filter for orient; returns 0 when undecided.
int filter_orient(int dim, const P3* p) {
  const P3& o = p[dim];
  double x[3], y[3], z[3];
  double mx = 0;
  for (int i = 0; i < dim; ++i) {
    x[i] = p[i].x - o.x;
    y[i] = p[i].y - o.y;
    z[i] = p[i].z - o.z;
    mx = std::max({mx, std::fabs(x[i]), std::fabs(y[i]), std::fabs(z[i])});
  }
  if (!(mx < 1e30)) return 0;
  double det, perm;
  if (dim == 3) {
    double m12 = x[1] * y[2] - y[1] * x[2], p12 = std::fabs(x[1] * y[2]) + std::fabs(y[1] * x[2]);
    double m02 = x[0] * y[2] - y[0] * x[2], p02 = std::fabs(x[0] * y[2]) + std::fabs(y[0] * x[2]);
    double m01 = x[0] * y[1] - y[0] * x[1], p01 = std::fabs(x[0] * y[1]) + std::fabs(y[0] * x[1]);
    det = z[0] * m12 - z[1] * m02 + z[2] * m01;
    perm = std::fabs(z[0]) * p12 + std::fabs(z[1]) * p02 + std::fabs(z[2]) * p01;
  } else {
    det = x[0] * y[1] - y[0] * x[1];
    perm = std::fabs(x[0] * y[1]) + std::fabs(y[0] * x[1]);
  }
  if (!(perm > 1e-150)) return 0;
  double bound = 32.0 * 1.1102230246251565e-16 * perm;
  if (det > bound) return 1;
  if (det < -bound) return -1;
  return 0;
}

int orient(int dim, const P3* p, long long* nexact) {
  int s = filter_orient(dim, p);
  if (s != 0) return s;
  if (nexact) ++*nexact;
  return exact_orient(dim, p);
}

// Sign of the unperturbed lifted determinant from an f64 evaluation with a
// permanent-based error bound; 0 when the bound cannot decide (the caller
// then evaluates it exactly).
int lifted_filter(int dim, const P3* p, const P3& q) {
  const int nv = dim + 1;
  double x[4], y[4], z[4], mx = 0;
  for (int i = 0; i < nv; ++i) {
    x[i] = p[i].x - q.x;
    y[i] = p[i].y - q.y;
    z[i] = p[i].z - q.z;
    mx = std::max({mx, std::fabs(x[i]), std::fabs(y[i]), std::fabs(z[i])});
  }
  if (!(mx < 1e30)) return 0;
  double det = 0, perm = 0;
  for (int i = 0; i < nv; ++i) {
    int o[3], t = 0;
    for (int k = 0; k < nv; ++k)
      if (k != i) o[t++] = k;
    double Oi, Pi;
    if (dim == 3) {
      auto m = [&](int a, int b) { return x[a] * y[b] - y[a] * x[b]; };
      auto pm = [&](int a, int b) { return std::fabs(x[a] * y[b]) + std::fabs(y[a] * x[b]); };
      Oi = z[o[0]] * m(o[1], o[2]) - z[o[1]] * m(o[0], o[2]) + z[o[2]] * m(o[0], o[1]);
      Pi = std::fabs(z[o[0]]) * pm(o[1], o[2]) + std::fabs(z[o[1]]) * pm(o[0], o[2]) +
           std::fabs(z[o[2]]) * pm(o[0], o[1]);
      if (!(i & 1)) Oi = -Oi;
    } else {
      Oi = x[o[0]] * y[o[1]] - y[o[0]] * x[o[1]];
      Pi = std::fabs(x[o[0]] * y[o[1]]) + std::fabs(y[o[0]] * x[o[1]]);
      if (i & 1) Oi = -Oi;
    }
    const double w = x[i] * x[i] + y[i] * y[i] + z[i] * z[i];
    det += w * Oi;
    perm += w * Pi;
  }
  if (!(perm > 1e-150)) return 0;
  const double bound = 64.0 * 1.1102230246251565e-16 * perm;
  return det > bound ? 1 : (det < -bound ? -1 : 0);
}

// Perturbed conflict test: +1 inside, -1 outside (never 0).
int insphere_sos(int dim, const P3* p, const int* key, const P3& q, int qkey, long long* nexact,
                 long long* nsos) {
  int nv = dim + 1;
  // f64 filter
  double x[4], y[4], z[4], mx = 0;
  for (int i = 0; i < nv; ++i) {
    x[i] = p[i].x - q.x;
    y[i] = p[i].y - q.y;
    z[i] = p[i].z - q.z;
    mx = std::max({mx, std::fabs(x[i]), std::fabs(y[i]), std::fabs(z[i])});
  }
  if (mx < 1e30) {
    double det = 0, perm = 0;
    for (int i = 0; i < nv; ++i) {
      int o[3], t = 0;
      for (int k = 0; k < nv; ++k)
        if (k != i) o[t++] = k;
      double Oi, Pi;
      if (dim == 3) {
        auto m = [&](int a, int b) { return x[a] * y[b] - y[a] * x[b]; };
        auto pm = [&](int a, int b) { return std::fabs(x[a] * y[b]) + std::fabs(y[a] * x[b]); };
        Oi = z[o[0]] * m(o[1], o[2]) - z[o[1]] * m(o[0], o[2]) + z[o[2]] * m(o[0], o[1]);
        Pi = std::fabs(z[o[0]]) * pm(o[1], o[2]) + std::fabs(z[o[1]]) * pm(o[0], o[2]) +
             std::fabs(z[o[2]]) * pm(o[0], o[1]);
        if (!(i & 1)) Oi = -Oi;
      } else {
        Oi = x[o[0]] * y[o[1]] - y[o[0]] * x[o[1]];
        Pi = std::fabs(x[o[0]] * y[o[1]]) + std::fabs(y[o[0]] * x[o[1]]);
        if (i & 1) Oi = -Oi;
      }
      double w = x[i] * x[i] + y[i] * y[i] + z[i] * z[i];
      det += w * Oi;
      perm += w * Pi;
    }
    if (perm > 1e-150) {
      double bound = 64.0 * 1.1102230246251565e-16 * perm;
      if (det > bound) return 1;
      if (det < -bound) return -1;
    }
  }
  if (nexact) ++*nexact;
  int os[4], ds;
  exact_lifted(dim, p, q, os, &ds);
  if (ds != 0) return ds;
  if (nsos) ++*nsos;
  // perturbation: walk the vertices from the largest key down
  int order[4];
  for (int i = 0; i < nv; ++i) order[i] = i;
  std::sort(order, order + nv, [&](int a, int b) { return key[a] > key[b]; });
  for (int t = 0; t < nv; ++t) {
    int i = order[t];
    if (key[i] < qkey) return -1;
    if (os[i] != 0) return os[i];
  }
  return -1;
}

// ---------------------------------------------------------------------------
// Reference super simplex (bit-exact restatement, host libm cos/sin).
// ---------------------------------------------------------------------------
bool rs_in_sphere(const double* v, const double* c, double r, int dim) {
  double d = 0.0;
  for (int i = 0; i < dim; ++i) d += (c[i] - v[i]) * (c[i] - v[i]);
  return d < r * r;
}

void bounding_sphere(int dim, const double* pts, int64_t n, double* center, double* radius) {
  double lo[3], hi[3];
  for (int i = 0; i < dim; ++i) {
    double l = INFINITY, h = -INFINITY;
    for (int64_t k = 0; k < n; ++k) {
      double v = pts[k * dim + i];
      l = std::fmin(l, v);
      h = std::fmax(h, v);
    }
    lo[i] = l;
    hi[i] = h;
    center[i] = (h + l) / 2.0;
  }
  double su = 0.0, sl = 0.0;
  for (int i = 0; i < dim; ++i) su += (hi[i] - center[i]) * (hi[i] - center[i]);
  for (int i = 0; i < dim; ++i) sl += (lo[i] - center[i]) * (lo[i] - center[i]);
  double ud = std::sqrt(su), ld = std::sqrt(sl);
  double r = ud > ld ? ud : ld;
  for (int64_t k = 0; k < n; ++k) {
    if (!rs_in_sphere(pts + k * dim, center, r, dim)) r = r * 1.5;
  }
  *radius = r;
}

// out: (dim+1) super vertices, each 3 doubles (z = 0 in 2D), in reference order.
void super_vertices(int dim, const double* pts, int64_t n, double* out, double* R) {
  double c[3] = {0, 0, 0}, r;
  bounding_sphere(dim, pts, n, c, &r);
  r *= 10.0;
  *R = r;
  const double pi = 3.141592653589793;
  double c1 = std::cos(2. * pi / 3.), s1 = std::sin(2. * pi / 3.);
  double c2 = std::cos(4. * pi / 3.), s2 = std::sin(4. * pi / 3.);
  if (dim == 3) {
    double v[4][3] = {{c[0], c[1], c[2] + r},
                      {c[0] + r, c[1], c[2] - r},
                      {c[0] + r * c1, c[1] + r * s1, c[2] - r},
                      {c[0] + r * c2, c[1] + r * s2, c[2] - r}};
    for (int i = 0; i < 4; ++i)
      for (int j = 0; j < 3; ++j) out[i * 3 + j] = v[i][j];
  } else {
    double v[3][2] = {{c[0] + r, c[1]}, {c[0] + r * c1, c[1] + r * s1}, {c[0] + r * c2, c[1] + r * s2}};
    for (int i = 0; i < 3; ++i) {
      out[i * 3 + 0] = v[i][0];
      out[i * 3 + 1] = v[i][1];
      out[i * 3 + 2] = 0.0;
    }
  }
}

// Float variant of the reference circumsphere (src/geometry.rs:2-56): the 2D
// slope formula; in 3D the system `direction * c = planes` solved as
// nalgebra 0.32.4's LU does it (restated from its published algorithm:
// partial pivoting on the first largest |a| of the column, multipliers scaled
// by the reciprocal of the pivot, unit lower triangular forward solve,
// column-oriented upper triangular back solve), then the radius to vertex 0.
void circumsphere_float(int dim, const double* v, double* center, double* radius) {
  if (dim == 2) {
    double x1 = v[0], y1 = v[1], x2 = v[2], y2 = v[3], x3 = v[4], y3 = v[5];
    double d0 = (x1 + x2) / 2.0, d1 = (y1 + y2) / 2.0;
    double e0 = (x2 + x3) / 2.0, e1 = (y2 + y3) / 2.0;
    double m_ab = (y2 - y1) / (x2 - x1);
    double m_bc = (y3 - y2) / (x3 - x2);
    double m_d = -1. / m_ab, m_e = -1. / m_bc;
    double x = (m_d * d0 - m_e * e0 + e1 - d1) / (m_d - m_e);
    double y = m_d * (x - d0) + d1;
    center[0] = x;
    center[1] = y;
    *radius = std::sqrt((x - x1) * (x - x1) + (y - y1) * (y - y1));
    return;
  }
  double A[3][3], b[3];
  for (int i = 0; i < 3; ++i) {
    double s = 0.0;
    for (int j = 0; j < 3; ++j) {
      A[i][j] = v[(i + 1) * 3 + j] - v[j];
      const double mid = (v[(i + 1) * 3 + j] + v[j]) / 2.0;
      const double t = A[i][j] * mid;
      s = j == 0 ? t : s + t;  // column_sum: ((m0 + m1) + m2)
    }
    b[i] = s;
  }
  for (int k = 0; k < 3; ++k) {
    int p = k;
    for (int i = k + 1; i < 3; ++i)
      if (std::fabs(A[i][k]) > std::fabs(A[p][k])) p = i;
    if (A[p][k] == 0.0) continue;
    if (p != k) {
      for (int j = 0; j < 3; ++j) std::swap(A[k][j], A[p][j]);
      std::swap(b[k], b[p]);
    }
    const double inv = 1.0 / A[k][k];
    for (int i = k + 1; i < 3; ++i) A[i][k] *= inv;
    for (int j = k + 1; j < 3; ++j)
      for (int i = k + 1; i < 3; ++i) A[i][j] = A[i][j] + (-A[k][j]) * A[i][k];
  }
  for (int i = 0; i < 3; ++i)
    for (int j = i + 1; j < 3; ++j) b[j] = b[j] + (-b[i]) * A[j][i];
  for (int i = 2; i >= 0; --i) {
    const double x = b[i] / A[i][i];
    b[i] = x;
    for (int k = 0; k < i; ++k) b[k] = b[k] + (-x) * A[k][i];
  }
  for (int j = 0; j < 3; ++j) center[j] = b[j];
  const double dx = v[0] - b[0], dy = v[1] - b[1], dz = v[2] - b[2];
  *radius = std::sqrt(dx * dx + dy * dy + dz * dz);
}

// Insertion priority: a bijective 32-bit mix of the vertex id and the seed.
uint32_t mix32(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7feb352dU;
  x ^= x >> 15;
  x *= 0x846ca68bU;
  x ^= x >> 16;
  return x;
}
uint32_t priority(uint32_t vid, uint64_t seed) {
  uint32_t x = vid ^ (uint32_t)seed;
  x = mix32(x);
  x ^= (uint32_t)(seed >> 32);
  return mix32(x);
}

// ---------------------------------------------------------------------------
// Sequential Bowyer-Watson.
// ---------------------------------------------------------------------------
struct Simplex {
  int v[4];
  int n[4];
  bool alive;
};

struct Tree {
  int dim = 3;
  int ns = 4;  // number of super vertices
  std::vector<P3> pts;       // vertex id -> coordinates
  std::vector<Simplex> s;
  std::vector<int> dup_of;   // input index -> kept input index, or -1
  int last = 0;
  int status = 0;
  long long nexact = 0, nsos = 0, nwalk = 0, maxcav = 0, maxfac = 0;
  std::vector<int> mark;     // BFS stamps
  int stamp = 0;
};

enum { OK = 0, ERR_ARG = 1, ERR_OUTSIDE = 6, ERR_WALK = 10, ERR_DEGENERATE = 12 };

void simplex_points(const Tree& t, int si, P3* out) {
  for (int i = 0; i <= t.dim; ++i) out[i] = t.pts[t.s[si].v[i]];
}

// visibility walk to a simplex whose closed hull contains p
int locate(Tree& t, const P3& p, int start) {
  int cur = start;
  long long cap = 64 + 4 * (long long)t.s.size();
  for (long long step = 0; step < cap; ++step) {
    const Simplex& S = t.s[cur];
    int nv = t.dim + 1, moved = -1;
    for (int j = 0; j < nv; ++j) {
      P3 q[4];
      simplex_points(t, cur, q);
      q[j] = p;
      if (orient(t.dim, q, &t.nexact) < 0) {
        moved = j;
        break;
      }
    }
    if (moved < 0) return cur;
    ++t.nwalk;
    int nb = S.n[moved];
    if (nb < 0) return -2;  // outside the super simplex
    cur = nb;
  }
  return -1;
}

int insert_vertex(Tree& t, int vid) {
  const P3 p = t.pts[vid];
  int nv = t.dim + 1;
  int start = t.last;
  if (!t.s[start].alive) start = 0;
  while (!t.s[start].alive) ++start;
  int c0 = locate(t, p, start);
  if (c0 == -2) return ERR_OUTSIDE;
  if (c0 < 0) return ERR_WALK;
  for (int i = 0; i < nv; ++i) {
    const P3& q = t.pts[t.s[c0].v[i]];
    if (q.x == p.x && q.y == p.y && q.z == p.z) return ERR_ARG;  // duplicate (pre-filtered)
  }
  // conflict region by BFS (locate + find_all_neighbors)
  if (t.mark.size() < t.s.size()) t.mark.resize(t.s.size() * 2 + 16, 0);
  ++t.stamp;
  std::vector<int> cav{c0};
  t.mark[c0] = t.stamp;
  struct Facet {
    int simp, face, outer;
  };
  std::vector<Facet> bnd;
  for (size_t h = 0; h < cav.size(); ++h) {
    int c = cav[h];
    for (int f = 0; f < nv; ++f) {
      int nb = t.s[c].n[f];
      if (nb < 0) {
        bnd.push_back({c, f, -1});
        continue;
      }
      if (t.mark[nb] == t.stamp) continue;
      P3 q[4];
      simplex_points(t, nb, q);
      int key[4];
      for (int i = 0; i < nv; ++i) key[i] = t.s[nb].v[i];
      if (insphere_sos(t.dim, q, key, p, vid, &t.nexact, &t.nsos) > 0) {
        t.mark[nb] = t.stamp;
        cav.push_back(nb);
      } else {
        bnd.push_back({c, f, nb});
      }
    }
  }
  t.maxcav = std::max<long long>(t.maxcav, (long long)cav.size());
  t.maxfac = std::max<long long>(t.maxfac, (long long)bnd.size());
  // star: one new simplex per boundary facet (get_new_simplices)
  int base = (int)t.s.size();
  t.s.resize(base + bnd.size());
  // ridge -> (new simplex, face) for intra-star adjacency (pair_simplices)
  std::map<std::array<int, 2>, std::pair<int, int>> open;
  for (size_t k = 0; k < bnd.size(); ++k) {
    const Facet& F = bnd[k];
    Simplex ns;
    ns.alive = true;
    for (int i = 0; i < 4; ++i) {
      ns.v[i] = (i < nv) ? t.s[F.simp].v[i] : -1;
      ns.n[i] = -1;
    }
    ns.v[F.face] = vid;
    ns.n[F.face] = F.outer;
    int id = base + (int)k;
    if (F.outer >= 0) {
      Simplex& O = t.s[F.outer];
      for (int j = 0; j < nv; ++j)
        if (O.n[j] == F.simp) O.n[j] = id;
    }
    for (int g = 0; g < nv; ++g) {
      if (g == F.face) continue;
      std::array<int, 2> ridge = {-1, -1};
      int r = 0;
      for (int i = 0; i < nv; ++i)
        if (i != g && i != F.face) ridge[r++] = ns.v[i];
      if (r == 2 && ridge[0] > ridge[1]) std::swap(ridge[0], ridge[1]);
      auto it = open.find(ridge);
      if (it == open.end()) {
        open[ridge] = {id, g};
      } else {
        ns.n[g] = it->second.first;
        t.s[it->second.first].n[it->second.second] = id;
        open.erase(it);
      }
    }
    t.s[id] = ns;
  }
  if (!open.empty()) return ERR_WALK;
  for (int c : cav) t.s[c].alive = false;
  t.last = base;
  return OK;
}

// Duplicate groups: of equal points the one with the smallest priority is
// kept; dup_of[k] = kept input index for the others.
void mark_duplicates(Tree& t, int64_t n, uint64_t seed) {
  // duplicate groups: keep the smallest priority
  t.dup_of.assign(n, -1);
  {
    struct K {
      double x, y, z;
      bool operator==(const K& o) const { return x == o.x && y == o.y && z == o.z; }
    };
    struct H {
      size_t operator()(const K& k) const {
        uint64_t a, b, c;
        memcpy(&a, &k.x, 8);
        memcpy(&b, &k.y, 8);
        memcpy(&c, &k.z, 8);
        return (size_t)(a * 0x9E3779B97F4A7C15ULL ^ (b + 0x632BE59BD9B4E019ULL) * 31 ^ c);
      }
    };
    std::unordered_map<K, int64_t, H> best;
    best.reserve(n * 2);
    for (int64_t k = 0; k < n; ++k) {
      const P3& p = t.pts[t.ns + k];
      K key{p.x == 0.0 ? 0.0 : p.x, p.y == 0.0 ? 0.0 : p.y, p.z == 0.0 ? 0.0 : p.z};
      auto it = best.find(key);
      if (it == best.end()) {
        best.emplace(key, k);
      } else {
        int64_t j = it->second;
        uint32_t pk = priority((uint32_t)(t.ns + k), seed), pj = priority((uint32_t)(t.ns + j), seed);
        if (pk < pj) {
          t.dup_of[j] = (int)k;
          it->second = k;
        } else {
          t.dup_of[k] = (int)j;
        }
      }
    }
    // resolve chains to the final kept index
    for (int64_t k = 0; k < n; ++k) {
      if (t.dup_of[k] < 0) continue;
      const P3& p = t.pts[t.ns + k];
      K key{p.x == 0.0 ? 0.0 : p.x, p.y == 0.0 ? 0.0 : p.y, p.z == 0.0 ? 0.0 : p.z};
      t.dup_of[k] = (int)best[key];
    }
  }
}

// ---------------------------------------------------------------------------
// Parallel path of the reference, restated with std::thread for the CPU
// baseline: src/lib.rs:104-125 (the first 1e5 points one at a time, the rest
// through add_points_to_tree), src/delaunay_tree.rs:336-386 (queue,
// placement, then per round TreeUpdate::new in parallel and one apply),
// src/scheduler.rs:6-28 (queue entry: located conflict region and its
// 2-ring of simplex ids) and :30-55 (greedy round = 1 + round of the
// previous point sharing a 2-ring simplex).  Apply checks that an update's
// conflict region and outer shell are unchanged since it was computed (the
// placement is made on the tree before the rounds); a stale update is
// recomputed on the spot, so the result is the exact triangulation.
// ---------------------------------------------------------------------------
struct Update {
  int vid = -1;
  std::vector<int> cav;
  struct Facet {
    int simp, face, outer;
  };
  std::vector<Facet> bnd;
  int status = OK;
};

// Persistent worker pool (the role rayon's global pool plays in the
// reference): run(n, fn) calls fn(i, tid) for i < n on all threads.
class Pool {
 public:
  explicit Pool(int threads) : threads_(std::max(1, threads)) {
    for (int k = 1; k < threads_; ++k) workers_.emplace_back([this, k] { loop(k); });
  }
  ~Pool() {
    {
      std::lock_guard<std::mutex> lk(mu_);
      quit_ = true;
      ++gen_;
    }
    cv_.notify_all();
    for (auto& w : workers_) w.join();
  }
  int threads() const { return threads_; }
  template <class F>
  void run(int64_t n, F&& fn) {
    if (n <= 0) return;
    std::function<void(int64_t, int)> job = fn;
    {
      std::lock_guard<std::mutex> lk(mu_);
      job_ = &job;
      n_ = n;
      next_.store(0);
      busy_ = threads_ - 1;
      ++gen_;
    }
    cv_.notify_all();
    work(0);
    std::unique_lock<std::mutex> lk(mu_);
    done_cv_.wait(lk, [&] { return busy_ == 0; });
    job_ = nullptr;
  }

 private:
  void work(int tid) {
    const int64_t grain = std::max<int64_t>(1, n_ / (16 * threads_));
    for (;;) {
      const int64_t b = next_.fetch_add(grain);
      if (b >= n_) break;
      const int64_t e = std::min<int64_t>(n_, b + grain);
      for (int64_t i = b; i < e; ++i) (*job_)(i, tid);
    }
  }
  void loop(int tid) {
    uint64_t seen = 0;
    for (;;) {
      {
        std::unique_lock<std::mutex> lk(mu_);
        cv_.wait(lk, [&] { return gen_ != seen; });
        seen = gen_;
        if (quit_) return;
      }
      work(tid);
      {
        std::lock_guard<std::mutex> lk(mu_);
        --busy_;
      }
      done_cv_.notify_all();
    }
  }
  int threads_;
  std::vector<std::thread> workers_;
  std::mutex mu_;
  std::condition_variable cv_, done_cv_;
  std::function<void(int64_t, int)>* job_ = nullptr;
  int64_t n_ = 0;
  std::atomic<int64_t> next_{0};
  int busy_ = 0;
  uint64_t gen_ = 0;
  bool quit_ = false;
};

// Read-only visibility walk (no counters touched).
int locate_ro(const Tree& t, const P3& p, int start, long long* nexact) {
  int cur = start;
  const long long cap = 64 + 4 * (long long)t.s.size();
  for (long long step = 0; step < cap; ++step) {
    int nv = t.dim + 1, moved = -1;
    for (int j = 0; j < nv; ++j) {
      P3 q[4];
      simplex_points(t, cur, q);
      q[j] = p;
      if (orient(t.dim, q, nexact) < 0) {
        moved = j;
        break;
      }
    }
    if (moved < 0) return cur;
    const int nb = t.s[cur].n[moved];
    if (nb < 0) return -2;
    cur = nb;
  }
  return -1;
}

// TreeUpdate::new (src/delaunay_tree.rs:709-740): conflict region and its
// boundary facets of vertex vid against the current tree, read-only.
void compute_update(const Tree& t, int vid, int start, Update& u, long long* nexact) {
  u.vid = vid;
  u.cav.clear();
  u.bnd.clear();
  u.status = OK;
  const P3 p = t.pts[vid];
  const int nv = t.dim + 1;
  long long nsos = 0;
  const int c0 = locate_ro(t, p, start, nexact);
  if (c0 < 0) {
    u.status = c0 == -2 ? ERR_OUTSIDE : ERR_WALK;
    return;
  }
  u.cav.push_back(c0);
  for (size_t h = 0; h < u.cav.size(); ++h) {
    const int c = u.cav[h];
    for (int f = 0; f < nv; ++f) {
      const int nb = t.s[c].n[f];
      if (nb < 0) {
        u.bnd.push_back({c, f, -1});
        continue;
      }
      if (std::find(u.cav.begin(), u.cav.end(), nb) != u.cav.end()) continue;
      P3 q[4];
      simplex_points(t, nb, q);
      int key[4];
      for (int i = 0; i < nv; ++i) key[i] = t.s[nb].v[i];
      if (insphere_sos(t.dim, q, key, p, vid, nexact, &nsos) > 0)
        u.cav.push_back(nb);
      else
        u.bnd.push_back({c, f, nb});
    }
  }
}

// insert_point (src/delaunay_tree.rs:125-211) of a computed update: star of
// new simplices, one per boundary facet, stitched by shared ridges.
void apply_update(Tree& t, const Update& u) {
  const int nv = t.dim + 1;
  const int base = (int)t.s.size();
  t.s.resize(base + u.bnd.size());
  std::map<std::array<int, 2>, std::pair<int, int>> open;
  for (size_t k = 0; k < u.bnd.size(); ++k) {
    const Update::Facet& F = u.bnd[k];
    Simplex ns;
    ns.alive = true;
    for (int i = 0; i < 4; ++i) {
      ns.v[i] = (i < nv) ? t.s[F.simp].v[i] : -1;
      ns.n[i] = -1;
    }
    ns.v[F.face] = u.vid;
    ns.n[F.face] = F.outer;
    const int id = base + (int)k;
    if (F.outer >= 0) {
      Simplex& O = t.s[F.outer];
      for (int j = 0; j < nv; ++j)
        if (O.n[j] == F.simp) O.n[j] = id;
    }
    for (int g = 0; g < nv; ++g) {
      if (g == F.face) continue;
      std::array<int, 2> ridge = {-1, -1};
      int r = 0;
      for (int i = 0; i < nv; ++i)
        if (i != g && i != F.face) ridge[r++] = ns.v[i];
      if (r == 2 && ridge[0] > ridge[1]) std::swap(ridge[0], ridge[1]);
      auto it = open.find(ridge);
      if (it == open.end()) {
        open[ridge] = {id, g};
      } else {
        ns.n[g] = it->second.first;
        t.s[it->second.first].n[it->second.second] = id;
        open.erase(it);
      }
    }
    t.s[id] = ns;
  }
  for (int c : u.cav) t.s[c].alive = false;
  t.last = base;
}

// Location hints: a coarse grid over the super simplex's bounding box, each
// cell holding a live simplex near it (the reference starts its search at
// the kd-tree nearest vertex, src/delaunay_tree.rs:35-40).
struct Grid {
  double lo[3], inv[3];
  int side = 1;
  std::vector<int> cell;
  int index(const P3& p, int dim) const {
    const double c[3] = {p.x, p.y, p.z};
    int idx = 0;
    for (int k = dim - 1; k >= 0; --k) {
      int i = (int)((c[k] - lo[k]) * inv[k] * side);
      i = std::min(std::max(i, 0), side - 1);
      idx = idx * side + i;
    }
    return idx;
  }
  void build(const Tree& t) {
    const int dim = t.dim;
    for (int k = 0; k < 3; ++k) {
      lo[k] = 1e300;
      double hi = -1e300;
      for (int i = 0; i < t.ns; ++i) {
        const double c = k == 0 ? t.pts[i].x : (k == 1 ? t.pts[i].y : t.pts[i].z);
        lo[k] = std::min(lo[k], c);
        hi = std::max(hi, c);
      }
      inv[k] = hi > lo[k] ? 1.0 / (hi - lo[k]) : 1.0;
    }
    side = dim == 3 ? 64 : 512;
    cell.assign(dim == 3 ? side * side * side : side * side, -1);
    for (size_t s = 0; s < t.s.size(); ++s) {
      if (!t.s[s].alive) continue;
      P3 c{0, 0, 0};
      for (int i = 0; i <= dim; ++i) {
        c.x += t.pts[t.s[s].v[i]].x / (dim + 1);
        c.y += t.pts[t.s[s].v[i]].y / (dim + 1);
        c.z += t.pts[t.s[s].v[i]].z / (dim + 1);
      }
      cell[index(c, dim)] = (int)s;
    }
  }
  int start(const Tree& t, const P3& p) const {
    int s = cell[index(p, t.dim)];
    if (s < 0 || !t.s[s].alive) {
      s = t.last;
      while (!t.s[s].alive) --s;
    }
    return s;
  }
};

int nrounds_last = 0;  // rounds of the last parallel build (diagnostics)

int build_parallel(Tree& t, int64_t n, int threads, int64_t prefix) {
  const int nv = t.dim + 1;
  std::vector<int> order;
  for (int64_t k = 0; k < n; ++k)
    if (t.dup_of[k] < 0) order.push_back((int)(t.ns + k));
  const int64_t seq = std::min<int64_t>(prefix, (int64_t)order.size());
  for (int64_t i = 0; i < seq; ++i) {
    const int rc = insert_vertex(t, order[i]);
    if (rc != OK) return rc;
  }
  const int64_t m = (int64_t)order.size() - seq;
  if (m <= 0) return OK;
  Grid grid;
  grid.build(t);
  Pool pool(threads);
  // make_queue: conflict region and 2-ring of every remaining point
  std::vector<std::vector<int>> ring(m);
  std::vector<long long> nex(threads, 0);
  std::vector<int> qstatus(m, OK);
  pool.run(m, [&](int64_t i, int tid) {
    Update u;
    compute_update(t, order[seq + i], grid.start(t, t.pts[order[seq + i]]), u, &nex[tid]);
    qstatus[i] = u.status;
    std::vector<int>& r = ring[i];
    for (int c : u.cav)
      for (int f = 0; f < nv; ++f) {
        const int a = t.s[c].n[f];
        if (a < 0) continue;
        for (int g = 0; g < nv; ++g)
          if (t.s[a].n[g] >= 0) r.push_back(t.s[a].n[g]);
      }
    std::sort(r.begin(), r.end());
    r.erase(std::unique(r.begin(), r.end()), r.end());
  });
  for (int64_t i = 0; i < m; ++i)
    if (qstatus[i] != OK) return qstatus[i];
  // find_placement: greedy rounds over shared 2-ring simplices
  std::vector<int> placement(m, 1);
  {
    std::unordered_map<int, int64_t> last;  // simplex -> last point that holds it in its 2-ring
    last.reserve(m * 8);
    int maxr = 1;
    for (int64_t i = 0; i < m; ++i) {
      int r = 1;
      for (int site : ring[i]) {
        auto it = last.find(site);
        if (it != last.end()) r = std::max(r, placement[it->second] + 1);
      }
      for (int site : ring[i]) last[site] = i;
      placement[i] = r;
      maxr = std::max(maxr, r);
    }
    t.maxcav = std::max<long long>(t.maxcav, 0);
    nrounds_last = maxr;
    std::vector<std::vector<int64_t>> rounds(maxr + 1);
    for (int64_t i = 0; i < m; ++i) rounds[placement[i]].push_back(i);
    ring.clear();
    ring.shrink_to_fit();
    std::vector<Update> ups;
    for (int r = 1; r <= maxr; ++r) {
      const auto& batch = rounds[r];
      if (batch.empty()) continue;
      ups.assign(batch.size(), Update());
      pool.run((int64_t)batch.size(), [&](int64_t i, int tid) {
        const int vid = order[seq + batch[i]];
        compute_update(t, vid, grid.start(t, t.pts[vid]), ups[i], &nex[tid]);
      });
      for (auto& u : ups) {
        bool fresh = u.status == OK;
        for (int c : u.cav) fresh = fresh && t.s[c].alive;
        for (const auto& F : u.bnd) fresh = fresh && (F.outer < 0 || t.s[F.outer].alive);
        if (!fresh) {  // the tree changed under this update: recompute it now
          int start = grid.start(t, t.pts[u.vid]);
          if (!u.cav.empty() && u.cav[0] < (int)t.s.size() && t.s[u.cav[0]].alive) start = u.cav[0];
          compute_update(t, u.vid, start, u, &t.nexact);
          if (u.status != OK) return u.status;
        }
        apply_update(t, u);
      }
    }
  }
  for (long long e : nex) t.nexact += e;
  return OK;
}

// ---------------------------------------------------------------------------
// The reference's own floating-point semantics (diagnostic, not the parity
// contract).  A sequential restatement of the reference's insertion path with
// its data model and its inexact conflict test, used to count how often that
// test decides differently from the exact one:
//   DelaunayTree::new super + ghost simplices  src/delaunay_tree.rs:389-510, :544-640
//   locate / find_all_neighbors                :33-75 (the nearest vertex's
//                                              simplices, then every conflicting
//                                              simplex reached from them)
//   get_new_simplices                          :77-123
//   insert_point                               :125-211
//   pair_simplices, TreeUpdate::new            :674-740
//   circumsphere_2d / _3d, in_sphere           src/geometry.rs:2-97
// The nearest vertex comes from a uniform grid instead of the kiddo 4.2.0
// kd-tree; equal distances go to the smallest vertex id (kiddo's own tie rule
// is not pinned).  A point whose located set is empty (the reference panics,
// :53) is counted and skipped.
// ---------------------------------------------------------------------------
struct RSimplex {
  int v[4];
  double c[3];
  double r;
  std::vector<int> nb;  // unordered neighbour ids, as the reference keeps them
  bool alive;
};

// Circumsphere of the reference (src/geometry.rs:2-56) over the dim
// coordinates of the vertices, in the order the simplex lists them.
void ref_circumsphere(int dim, const P3* q, double* c, double* r) {
  double v[12];
  for (int j = 0; j <= dim; ++j) {
    const double x[3] = {q[j].x, q[j].y, q[j].z};
    for (int k = 0; k < dim; ++k) v[j * dim + k] = x[k];
  }
  circumsphere_float(dim, v, c, r);
}

bool ref_conflict(int dim, const P3& p, const RSimplex& s) {
  const double v[3] = {p.x, p.y, p.z};
  return rs_in_sphere(v, s.c, s.r, dim);
}

// Nearest vertex by a uniform grid over the input box; vertices outside the
// box (super and ghost vertices) are checked one by one.
struct NNGrid {
  int dim = 3, side = 1;
  double lo[3] = {0, 0, 0}, w[3] = {1, 1, 1};
  std::vector<std::vector<int>> cell;
  std::vector<int> far;
  void init(int d, const std::vector<P3>& in, int64_t n) {
    dim = d;
    double hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    lo[0] = lo[1] = lo[2] = INFINITY;
    for (const P3& p : in) {
      const double c[3] = {p.x, p.y, p.z};
      for (int k = 0; k < dim; ++k) {
        lo[k] = std::min(lo[k], c[k]);
        hi[k] = std::max(hi[k], c[k]);
      }
    }
    side = std::max(1, (int)std::floor(std::pow(std::max<double>(1.0, (double)n / 2.0), 1.0 / dim)));
    side = std::min(side, dim == 3 ? 256 : 2048);
    for (int k = 0; k < 3; ++k) {
      if (k >= dim) {
        lo[k] = 0;
        w[k] = 1;
        continue;
      }
      w[k] = std::max((hi[k] - lo[k]) / side, 1e-300);
    }
    cell.assign((size_t)std::pow(side, dim), {});
  }
  bool cell_of(const P3& p, int* ic) const {
    const double c[3] = {p.x, p.y, p.z};
    bool inside = true;
    for (int k = 0; k < 3; ++k) {
      if (k >= dim) {
        ic[k] = 0;
        continue;
      }
      const double u = (c[k] - lo[k]) / w[k];
      if (!(u >= 0.0) || u > (double)side) inside = false;
      ic[k] = u < 0.0 ? 0 : (u >= side ? side - 1 : (int)u);
    }
    return inside;
  }
  size_t index(const int* ic) const {
    size_t i = 0;
    for (int k = dim - 1; k >= 0; --k) i = i * side + ic[k];
    return i;
  }
  void add(int id, const P3& p) {
    int ic[3];
    if (cell_of(p, ic))
      cell[index(ic)].push_back(id);
    else
      far.push_back(id);
  }
  int nearest(const P3& p, const std::vector<P3>& pts) const {
    double best = INFINITY;
    int bi = -1;
    auto test = [&](int id) {
      const P3& q = pts[id];
      double d = (p.x - q.x) * (p.x - q.x) + (p.y - q.y) * (p.y - q.y);
      if (dim == 3) d += (p.z - q.z) * (p.z - q.z);
      if (d < best || (d == best && id < bi)) {
        best = d;
        bi = id;
      }
    };
    for (int id : far) test(id);
    int ic[3];
    cell_of(p, ic);
    const double c[3] = {p.x, p.y, p.z};
    for (int r = 0; r <= side; ++r) {
      int a[3], b[3];
      for (int k = 0; k < 3; ++k) {
        a[k] = k < dim ? std::max(0, ic[k] - r) : 0;
        b[k] = k < dim ? std::min(side - 1, ic[k] + r) : 0;
      }
      for (int z = a[2]; z <= b[2]; ++z)
        for (int y = a[1]; y <= b[1]; ++y)
          for (int x = a[0]; x <= b[0]; ++x) {
            const int cc[3] = {x, y, z};
            int cheb = 0;
            for (int k = 0; k < dim; ++k) cheb = std::max(cheb, std::abs(cc[k] - ic[k]));
            if (cheb != r) continue;
            for (int id : cell[index(cc)]) test(id);
          }
      // any vertex in a later ring is at least this far from p
      double gap = INFINITY;
      for (int k = 0; k < dim; ++k) {
        gap = std::min(gap, c[k] - (lo[k] + (ic[k] - r) * w[k]));
        gap = std::min(gap, (lo[k] + (ic[k] + r + 1) * w[k]) - c[k]);
      }
      if (bi >= 0 && gap > 0 && best <= gap * gap) break;
    }
    return bi;
  }
};

struct RTree {
  int dim = 3, M = 4;
  std::vector<P3> pts;
  std::vector<std::vector<int>> vsimp;
  std::vector<RSimplex> s;
  int64_t max_id = 0;
  NNGrid grid;
  std::vector<int> mark;
  int stamp = 0;
  long long inserted = 0, empty = 0, malformed = 0, max_killed = 0;
};

// DelaunayTree::new (src/delaunay_tree.rs:389-510 3D, :544-640 2D): super
// vertices, ghost vertices, the super simplex with the bounding sphere
// (centre, 10 r) as its sphere, and radius-0 ghost simplices on its faces.
void ref_new(RTree& t, int dim, const double* in, int64_t n) {
  t.dim = dim;
  t.M = dim + 1;
  double cen[3] = {0, 0, 0}, r;
  bounding_sphere(dim, in, n, cen, &r);
  double sv[4][3] = {};
  double R;
  super_vertices(dim, in, n, &sv[0][0], &R);
  if (dim == 3) {
    for (int i = 0; i < 4; ++i) t.pts.push_back({sv[i][0], sv[i][1], sv[i][2]});
    const P3 top{cen[0], cen[1], R + cen[2]};
    t.pts.push_back(top);
    t.pts.push_back(top);
    t.pts.push_back(top);
    t.pts.push_back({cen[0] + R, cen[1], cen[2] - R});
    t.vsimp = {{0, 1, 2, 3}, {0, 1, 3, 4}, {0, 1, 2, 4}, {0, 2, 3, 4}, {1}, {2}, {3}, {4}};
    const int sv_ids[5][4] = {{0, 1, 2, 3}, {4, 0, 1, 2}, {5, 0, 2, 3}, {6, 0, 3, 1}, {7, 1, 2, 3}};
    for (int k = 0; k < 5; ++k) {
      RSimplex S{};
      for (int j = 0; j < 4; ++j) S.v[j] = sv_ids[k][j];
      S.alive = true;
      if (k == 0) {
        S.c[0] = cen[0];
        S.c[1] = cen[1];
        S.c[2] = cen[2];
        S.r = R;
        S.nb = {1, 2, 3, 4};
      } else {
        S.r = 0.0;
        S.nb = {0};
      }
      t.s.push_back(S);
    }
    t.max_id = 4;
  } else {
    for (int i = 0; i < 3; ++i) t.pts.push_back({sv[i][0], sv[i][1], 0.0});
    for (int i = 0; i < 3; ++i) t.pts.push_back({sv[i][0], sv[i][1], 0.0});
    t.vsimp = {{0, 1, 2}, {0, 1, 3}, {0, 2, 3}, {1}, {2}, {3}};
    const int sv_ids[4][3] = {{0, 1, 2}, {3, 0, 1}, {4, 0, 2}, {5, 1, 2}};
    for (int k = 0; k < 4; ++k) {
      RSimplex S{};
      for (int j = 0; j < 3; ++j) S.v[j] = sv_ids[k][j];
      S.v[3] = -1;
      S.alive = true;
      if (k == 0) {
        S.c[0] = cen[0];
        S.c[1] = cen[1];
        S.r = R;
        S.nb = {1, 2, 3};
      } else {
        S.r = 0.0;
        S.nb = {0};
      }
      t.s.push_back(S);
    }
    t.max_id = 3;
  }
  std::vector<P3> box;
  for (int64_t k = 0; k < n; ++k) box.push_back({in[k * dim], in[k * dim + 1], dim == 3 ? in[k * dim + 2] : 0.0});
  t.grid.init(dim, box, n);
  for (int id = 0; id < (int)t.pts.size(); ++id) t.grid.far.push_back(id);
}

// TreeUpdate::new + insert_point for vertex `vid` (already in t.pts).
void ref_insert(RTree& t, int vid) {
  const P3 p = t.pts[vid];
  const int M = t.M, N = t.dim;
  if (t.mark.size() < t.s.size() + 64) t.mark.resize(2 * t.s.size() + 64, 0);
  ++t.stamp;
  // locate: the nearest vertex's simplices, then find_all_neighbors from
  // each one in conflict
  const int nn = t.grid.nearest(p, t.pts);
  std::vector<int> out;
  std::vector<int> stack;
  for (int id : t.vsimp[nn]) {
    if (!ref_conflict(N, p, t.s[id])) continue;
    if (t.mark[id] != t.stamp) {
      t.mark[id] = t.stamp;
      out.push_back(id);
    }
    stack.push_back(id);
    while (!stack.empty()) {
      const int node = stack.back();
      stack.pop_back();
      for (int nb : t.s[node].nb) {
        if (t.mark[nb] == t.stamp || !ref_conflict(N, p, t.s[nb])) continue;
        t.mark[nb] = t.stamp;
        out.push_back(nb);
        stack.push_back(nb);
      }
    }
  }
  if (out.empty()) {  // the reference panics here (src/delaunay_tree.rs:53)
    ++t.empty;
    return;
  }
  std::sort(out.begin(), out.end());
  t.max_killed = std::max<long long>(t.max_killed, (long long)out.size());
  // get_new_simplices for every killed simplex
  struct New {
    int v[4];
    int outer, killed;
  };
  std::vector<New> nw;
  for (int k : out) {
    const RSimplex& K = t.s[k];
    for (int nb : K.nb) {
      const RSimplex& B = t.s[nb];
      if (ref_conflict(N, p, B)) continue;
      New x{{vid, 0, 0, 0}, nb, k};
      if (N == 2) x.v[3] = -1;
      int count = 1;
      for (int i = 0; i < M; ++i) {
        bool in_k = false;
        for (int j = 0; j < M; ++j) in_k = in_k || K.v[j] == B.v[i];
        if (in_k) {
          if (count < M) x.v[count] = B.v[i];
          ++count;
        }
      }
      if (count != M) ++t.malformed;
      nw.push_back(x);
    }
  }
  // pair_simplices: new simplices sharing N vertices are neighbours
  const int64_t base = t.max_id;
  t.s.resize(base + 1 + nw.size());
  for (size_t i = 0; i < nw.size(); ++i) {
    RSimplex& S = t.s[base + 1 + i];
    P3 q[4];
    for (int j = 0; j < M; ++j) {
      S.v[j] = nw[i].v[j];
      q[j] = t.pts[nw[i].v[j]];
    }
    S.v[3] = N == 2 ? -1 : S.v[3];
    ref_circumsphere(N, q, S.c, &S.r);
    S.nb = {nw[i].outer};
    S.alive = true;
  }
  for (size_t i = 0; i < nw.size(); ++i) {
    for (int& x : t.s[nw[i].outer].nb)
      if (x == nw[i].killed) x = (int)(base + 1 + i);
  }
  for (size_t i = 0; i < nw.size(); ++i)
    for (size_t j = i + 1; j < nw.size(); ++j) {
      int count = 0;
      for (int k = 0; k < M; ++k)
        for (int l = 0; l < M; ++l) count += nw[i].v[l] == nw[j].v[k];
      if (count == N) {
        t.s[base + 1 + i].nb.push_back((int)(base + 1 + j));
        t.s[base + 1 + j].nb.push_back((int)(base + 1 + i));
      }
    }
  if ((int)t.vsimp.size() <= vid) t.vsimp.resize(vid + 1);
  for (size_t i = 0; i < nw.size(); ++i)
    for (int j = 0; j < M; ++j) t.vsimp[nw[i].v[j]].push_back((int)(base + 1 + i));
  for (int k : out)
    for (int i = 0; i < M; ++i) {
      auto& l = t.vsimp[t.s[k].v[i]];
      l.erase(std::remove(l.begin(), l.end(), k), l.end());
    }
  for (int k : out) t.s[k].alive = false;
  t.max_id += (int64_t)nw.size();
  t.grid.add(vid, p);
  ++t.inserted;
}

}  // namespace

extern "C" {

// ---- reference arithmetic restatements -----------------------------------
void vdo_bounding_sphere(int dim, const double* pts, int64_t n, double* center, double* radius) {
  bounding_sphere(dim, pts, n, center, radius);
}
void vdo_super_vertices(int dim, const double* pts, int64_t n, double* out, double* R) {
  super_vertices(dim, pts, n, out, R);
}
void vdo_circumsphere_float(int dim, const double* v, double* center, double* radius) {
  circumsphere_float(dim, v, center, radius);
}
uint32_t vdo_priority(uint32_t vid, uint64_t seed) { return priority(vid, seed); }

// ---- exact predicates (pts are (dim+1) or (dim+2) xyz triples) -----------
int vdo_orient(int dim, const double* pts) {
  P3 p[4];
  for (int i = 0; i <= dim; ++i) p[i] = {pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]};
  return exact_orient(dim, p);
}
int vdo_insphere_sos(int dim, const double* pts, const int* keys) {
  P3 p[4], q;
  for (int i = 0; i <= dim; ++i) p[i] = {pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]};
  int k = dim + 1;
  q = {pts[3 * k], pts[3 * k + 1], pts[3 * k + 2]};
  return insphere_sos(dim, p, keys, q, keys[k], nullptr, nullptr);
}
// exact unperturbed lifted determinant sign
int vdo_insphere_exact(int dim, const double* pts) {
  P3 p[4], q;
  for (int i = 0; i <= dim; ++i) p[i] = {pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]};
  int k = dim + 1;
  q = {pts[3 * k], pts[3 * k + 1], pts[3 * k + 2]};
  int os[4], ds;
  exact_lifted(dim, p, q, os, &ds);
  return ds;
}

// ---- sequential triangulation ---------------------------------------------
// pts: n points of `dim` doubles.  The super simplex is sized from the same
// points (src/lib.rs:104-125).  Returns an opaque handle; *status is 0 or an
// error code.  Duplicates are skipped (kept: smallest priority).
void* vdo_build(int dim, const double* pts, int64_t n, uint64_t seed, int* status) {
  Tree* t = new Tree();
  t->dim = dim;
  t->ns = dim + 1;
  *status = OK;
  if ((dim != 2 && dim != 3) || n < 1) {
    *status = ERR_ARG;
    return t;
  }
  double sv[12], R;
  super_vertices(dim, pts, n, sv, &R);
  for (int i = 0; i <= dim; ++i) t->pts.push_back({sv[3 * i], sv[3 * i + 1], sv[3 * i + 2]});
  for (int64_t k = 0; k < n; ++k)
    t->pts.push_back({pts[k * dim], pts[k * dim + 1], dim == 3 ? pts[k * dim + 2] : 0.0});
  Simplex s0;
  s0.alive = true;
  for (int i = 0; i < 4; ++i) {
    s0.v[i] = i <= dim ? i : -1;
    s0.n[i] = -1;
  }
  {  // positive orientation
    P3 q[4];
    for (int i = 0; i <= dim; ++i) q[i] = t->pts[i];
    int o = exact_orient(dim, q);
    if (o == 0) {
      *status = ERR_DEGENERATE;
      return t;
    }
    if (o < 0) std::swap(s0.v[0], s0.v[1]);
  }
  t->s.push_back(s0);
  mark_duplicates(*t, n, seed);
  for (int64_t k = 0; k < n; ++k) {
    if (t->dup_of[k] >= 0) continue;
    int rc = insert_vertex(*t, (int)(t->ns + k));
    if (rc != OK) {
      *status = rc;
      return t;
    }
  }
  return t;
}

// The reference's parallel path (see build_parallel) on `threads` host
// threads; `prefix` points are inserted one at a time first (1e5 in
// src/lib.rs:108).  Same result as vdo_build.
void* vdo_build_parallel(int dim, const double* pts, int64_t n, uint64_t seed, int threads, int64_t prefix,
                         int* status) {
  Tree* t = new Tree();
  t->dim = dim;
  t->ns = dim + 1;
  *status = OK;
  if ((dim != 2 && dim != 3) || n < 1 || threads < 1) {
    *status = ERR_ARG;
    return t;
  }
  double sv[12], R;
  super_vertices(dim, pts, n, sv, &R);
  for (int i = 0; i <= dim; ++i) t->pts.push_back({sv[3 * i], sv[3 * i + 1], sv[3 * i + 2]});
  for (int64_t k = 0; k < n; ++k)
    t->pts.push_back({pts[k * dim], pts[k * dim + 1], dim == 3 ? pts[k * dim + 2] : 0.0});
  Simplex s0;
  s0.alive = true;
  for (int i = 0; i < 4; ++i) {
    s0.v[i] = i <= dim ? i : -1;
    s0.n[i] = -1;
  }
  P3 q[4];
  for (int i = 0; i <= dim; ++i) q[i] = t->pts[i];
  const int o = exact_orient(dim, q);
  if (o == 0) {
    *status = ERR_DEGENERATE;
    return t;
  }
  if (o < 0) std::swap(s0.v[0], s0.v[1]);
  t->s.push_back(s0);
  mark_duplicates(*t, n, seed);
  *status = build_parallel(*t, n, threads, prefix);
  return t;
}

// Diagnostics: winners of one resolution pass for the next `nact` points (by
// priority) against the tree built from the first `n_built` points, under
// the strict rule (cavities disjoint from other cavities and their outer
// shells) and under the relaxed rule (cavities disjoint; a cavity next to a
// lower-priority cavity wins only if the shared facets stay locally Delaunay).
// out: strict winners, relaxed winners, adjacent pairs, failed facet tests.
void vdo_round_sim(int dim, const double* pts, int64_t n_built, int64_t nact, uint64_t seed, int64_t* out) {
  Tree t;
  t.dim = dim;
  t.ns = dim + 1;
  const int64_t n = n_built + nact;
  double sv[12], R;
  super_vertices(dim, pts, n, sv, &R);
  for (int i = 0; i <= dim; ++i) t.pts.push_back({sv[3 * i], sv[3 * i + 1], sv[3 * i + 2]});
  for (int64_t k = 0; k < n; ++k) t.pts.push_back({pts[k * dim], pts[k * dim + 1], dim == 3 ? pts[k * dim + 2] : 0.0});
  Simplex s0;
  s0.alive = true;
  for (int i = 0; i < 4; ++i) {
    s0.v[i] = i <= dim ? i : -1;
    s0.n[i] = -1;
  }
  P3 q[4];
  for (int i = 0; i <= dim; ++i) q[i] = t.pts[i];
  if (exact_orient(dim, q) < 0) std::swap(s0.v[0], s0.v[1]);
  t.s.push_back(s0);
  for (int64_t k = 0; k < n_built; ++k) insert_vertex(t, (int)(t.ns + k));
  const int nv = dim + 1;
  std::vector<Update> up(nact);
  std::vector<uint32_t> key(nact);
  for (int64_t i = 0; i < nact; ++i) {
    const int vid = (int)(t.ns + n_built + i);
    int start = t.last;
    while (!t.s[start].alive) --start;
    compute_update(t, vid, start, up[i], &t.nexact);
    key[i] = priority((uint32_t)vid, seed);
  }
  const uint32_t NONE = 0xffffffffu;
  std::vector<uint32_t> cc(t.s.size(), NONE), cn(t.s.size(), NONE);
  std::vector<int64_t> owner(t.s.size(), -1);
  for (int64_t i = 0; i < nact; ++i) {
    for (int c : up[i].cav)
      if (key[i] < cc[c]) {
        cc[c] = key[i];
        owner[c] = i;
      }
    for (const auto& F : up[i].bnd)
      if (F.outer >= 0) cn[F.outer] = std::min(cn[F.outer], key[i]);
  }
  int64_t strict = 0, relaxed = 0, adjacent = 0, failed = 0;
  long long nsos = 0;
  for (int64_t i = 0; i < nact; ++i) {
    bool own = true;
    for (int c : up[i].cav) own = own && cc[c] == key[i];
    bool s_ok = own;
    for (int c : up[i].cav) s_ok = s_ok && cn[c] > key[i];
    for (const auto& F : up[i].bnd)
      if (F.outer >= 0) s_ok = s_ok && cc[F.outer] > key[i];
    strict += s_ok;
    bool r_ok = own;
    for (const auto& F : up[i].bnd) {
      if (!r_ok) break;
      if (F.outer < 0 || cc[F.outer] >= key[i]) continue;
      ++adjacent;
      // new simplex of i on this facet; the lower candidate's point must not conflict
      P3 p[4];
      int kk[4];
      for (int j = 0; j < nv; ++j) {
        kk[j] = t.s[F.simp].v[j];
        p[j] = t.pts[kk[j]];
      }
      kk[F.face] = up[i].vid;
      p[F.face] = t.pts[up[i].vid];
      const int x = up[owner[F.outer]].vid;
      if (insphere_sos(dim, p, kk, t.pts[x], x, &t.nexact, &nsos) > 0) {
        ++failed;
        r_ok = false;
      }
    }
    relaxed += r_ok;
  }
  out[0] = strict;
  out[1] = relaxed;
  out[2] = adjacent;
  out[3] = failed;
}

void vdo_free(void* h) { delete (Tree*)h; }
int vdo_parallel_rounds(void) { return nrounds_last; }

int64_t vdo_num_duplicates(void* h) {
  Tree* t = (Tree*)h;
  int64_t c = 0;
  for (int d : t->dup_of) c += d >= 0;
  return c;
}

void vdo_stats(void* h, long long* out) {
  Tree* t = (Tree*)h;
  long long alive = 0;
  for (auto& s : t->s) alive += s.alive;
  out[0] = alive;
  out[1] = (long long)t->s.size();
  out[2] = t->nexact;
  out[3] = t->nsos;
  out[4] = t->nwalk;
  out[5] = t->maxcav;
  out[6] = t->maxfac;
}

// Sorted unique edge list among input points (input indices, u < v).
int64_t vdo_edges(void* h, int64_t* uv, int64_t cap) {
  Tree* t = (Tree*)h;
  std::vector<uint64_t> e;
  int nv = t->dim + 1;
  for (auto& s : t->s) {
    if (!s.alive) continue;
    for (int i = 0; i < nv; ++i)
      for (int j = i + 1; j < nv; ++j) {
        int a = s.v[i], b = s.v[j];
        if (a < t->ns || b < t->ns) continue;
        a -= t->ns;
        b -= t->ns;
        if (a > b) std::swap(a, b);
        e.push_back(((uint64_t)a << 32) | (uint32_t)b);
      }
  }
  std::sort(e.begin(), e.end());
  e.erase(std::unique(e.begin(), e.end()), e.end());
  if (uv) {
    int64_t m = std::min<int64_t>(cap, (int64_t)e.size());
    for (int64_t i = 0; i < m; ++i) {
      uv[2 * i] = (int64_t)(e[i] >> 32);
      uv[2 * i + 1] = (int64_t)(e[i] & 0xffffffffu);
    }
  }
  return (int64_t)e.size();
}

// Vertex coordinates (super first) and alive simplices in the handle's own
// numbering, for the validator.
int64_t vdo_num_vertices(void* h) { return (int64_t)((Tree*)h)->pts.size(); }
void vdo_vertices(void* h, double* xyz) {
  Tree* t = (Tree*)h;
  for (size_t i = 0; i < t->pts.size(); ++i) {
    xyz[3 * i] = t->pts[i].x;
    xyz[3 * i + 1] = t->pts[i].y;
    xyz[3 * i + 2] = t->pts[i].z;
  }
}

// ---- validator for any triangulation -------------------------------------
// verts: nvert xyz triples (vertex id = index, super vertices first).
// simp: ns rows of 4 vertex ids (2D: 3 used), nbr: ns rows of 4 neighbour
// simplex indices (row-local, -1 = hull).  out[0..7]:
//  0 non-positive simplices, 1 asymmetric adjacencies, 2 facets whose
//  opposite vertex is strictly inside (exact, unperturbed), 3 facets failing
//  the perturbed test, 4 hull facets, 5 facets checked, 6 vertices missing
//  from every simplex (among `expect_vertices` first ids), 7 exact calls
void vdo_validate(int dim, const double* verts, int64_t nvert, const int32_t* simp,
                  const int32_t* nbr, int64_t ns, int64_t expect_vertices, long long* out) {
  for (int i = 0; i < 8; ++i) out[i] = 0;
  const int nv = dim + 1;
  auto P = [&](int v) { return P3{verts[3 * v], verts[3 * v + 1], verts[3 * v + 2]}; };
  // the simplices are split over host threads, each with its own counts
  const int nth = (int)std::max<unsigned>(1, std::min<unsigned>(64, std::thread::hardware_concurrency()));
  std::vector<std::array<long long, 8>> part(nth);
  auto work = [&](int tid) {
    std::array<long long, 8> c{};
    const int64_t lo = ns * tid / nth, hi = ns * (tid + 1) / nth;
    for (int64_t s = lo; s < hi; ++s) {
      const int32_t* v = simp + 4 * s;
      P3 q[4];
      for (int i = 0; i < nv; ++i) q[i] = P(v[i]);
      if (orient(dim, q, &c[7]) <= 0) c[0]++;
      for (int f = 0; f < nv; ++f) {
        int o = nbr[4 * s + f];
        if (o < 0) {
          c[4]++;
          continue;
        }
        // neighbour must point back and share the facet
        const int32_t* w = simp + 4 * o;
        int back = -1;
        for (int g = 0; g < nv; ++g)
          if (nbr[4 * o + g] == s) back = g;
        bool ok = back >= 0;
        if (ok) {
          for (int i = 0; i < nv; ++i) {
            if (i == f) continue;
            bool found = false;
            for (int g = 0; g < nv; ++g)
              if (g != back && w[g] == v[i]) found = true;
            ok = ok && found;
          }
        }
        if (!ok) {
          c[1]++;
          continue;
        }
        if (o < s) continue;  // each interior facet once
        c[5]++;
        int opp = w[back];
        P3 e = P(opp);
        // unperturbed sign: f64 filter, big integers when it cannot decide
        int ds = lifted_filter(dim, q, e);
        if (ds == 0) {
          int os[4];
          exact_lifted(dim, q, e, os, &ds);
          ++c[7];
        }
        if (ds > 0) c[2]++;
        int key[4];
        for (int i = 0; i < nv; ++i) key[i] = v[i];
        if (insphere_sos(dim, q, key, e, opp, &c[7], nullptr) > 0) c[3]++;
      }
    }
    part[tid] = c;
  };
  std::vector<std::thread> th;
  for (int t = 1; t < nth; ++t) th.emplace_back(work, t);
  work(0);
  for (auto& x : th) x.join();
  for (const auto& c : part)
    for (int i = 0; i < 8; ++i) out[i] += c[i];
  std::vector<char> seen(nvert, 0);
  for (int64_t s = 0; s < ns; ++s)
    for (int i = 0; i < nv; ++i) seen[simp[4 * s + i]] = 1;
  for (int64_t i = 0; i < expect_vertices && i < nvert; ++i)
    if (!seen[i]) out[6]++;
}

// Export alive simplices of an oracle handle (same layout as vdo_validate).
int64_t vdo_simplices(void* h, int32_t* simp, int32_t* nbr) {
  Tree* t = (Tree*)h;
  std::vector<int> remap(t->s.size(), -1);
  int64_t k = 0;
  for (size_t i = 0; i < t->s.size(); ++i)
    if (t->s[i].alive) remap[i] = (int)k++;
  if (simp) {
    int64_t r = 0;
    for (size_t i = 0; i < t->s.size(); ++i) {
      if (!t->s[i].alive) continue;
      for (int j = 0; j < 4; ++j) {
        simp[4 * r + j] = t->s[i].v[j];
        int nb = t->s[i].n[j];
        nbr[4 * r + j] = (j <= t->dim && nb >= 0) ? remap[nb] : -1;
      }
      ++r;
    }
  }
  return k;
}

int vdo_status(void* h) { return ((Tree*)h)->status; }


// ---- the reference's float semantics (diagnostic) --------------------------
// Sequential insertion of all n points in input order with the reference's
// inexact conflict test.  stats (NULL or 8): inserted, empty located sets
// (skipped; the reference panics), new simplices whose outer neighbour did not
// share a facet with the removed one, largest removed set, live simplices
// (ghosts excluded), vertex count, 0, 0.
void* vdo_build_float(int dim, const double* pts, int64_t n, long long* stats) {
  if ((dim != 2 && dim != 3) || n < 1) return nullptr;
  RTree* t = new RTree();
  ref_new(*t, dim, pts, n);
  const int first = (int)t->pts.size();
  for (int64_t k = 0; k < n; ++k)
    t->pts.push_back({pts[k * dim], pts[k * dim + 1], dim == 3 ? pts[k * dim + 2] : 0.0});
  t->vsimp.resize(t->pts.size());
  for (int64_t k = 0; k < n; ++k) ref_insert(*t, first + (int)k);
  if (stats) {
    long long live = 0;
    for (const RSimplex& S : t->s) {
      if (!S.alive) continue;
      bool ghost = false;
      for (int j = 0; j < t->M; ++j) ghost = ghost || (S.v[j] >= t->M && S.v[j] < 2 * t->M);
      live += !ghost;
    }
    const long long v[8] = {t->inserted, t->empty, t->malformed, t->max_killed, live, (long long)t->pts.size(), 0, 0};
    for (int i = 0; i < 8; ++i) stats[i] = v[i];
  }
  return t;
}

// Sorted unique edges (u < v, input numbering) of the live simplices.
int64_t vdo_float_edges(void* h, int64_t* out, int64_t cap) {
  RTree* t = (RTree*)h;
  const int first = 2 * t->M;
  std::vector<std::pair<int, int>> e;
  for (const RSimplex& S : t->s) {
    if (!S.alive) continue;
    for (int i = 0; i < t->M; ++i)
      for (int j = i + 1; j < t->M; ++j) {
        const int a = S.v[i], b = S.v[j];
        if (a < first || b < first || a == b) continue;
        e.push_back({std::min(a, b) - first, std::max(a, b) - first});
      }
  }
  std::sort(e.begin(), e.end());
  e.erase(std::unique(e.begin(), e.end()), e.end());
  if (out)
    for (int64_t k = 0; k < (int64_t)e.size() && k < cap; ++k) {
      out[2 * k] = e[k].first;
      out[2 * k + 1] = e[k].second;
    }
  return (int64_t)e.size();
}

// The live non-ghost simplices in vdo_validate's layout: vertex ids super
// 0..dim then the inputs, each simplex turned to positive orientation by an
// exact orient (a degenerate one is left as it is), neighbours by face.
// *bad counts links that cannot be placed on a face (a neighbour that is
// dead, shares a number of vertices other than dim, or repeats a face).
int64_t vdo_float_export(void* h, double* verts, int32_t* simp, int32_t* nbr, long long* bad) {
  RTree* t = (RTree*)h;
  const int M = t->M, dim = t->dim;
  auto ghost_or_dead = [&](int id) {
    const RSimplex& S = t->s[id];
    if (!S.alive) return true;
    for (int j = 0; j < M; ++j)
      if (S.v[j] >= M && S.v[j] < 2 * M) return true;
    return false;
  };
  std::vector<int> idx(t->s.size(), -1);
  int64_t k = 0;
  for (size_t i = 0; i < t->s.size(); ++i)
    if (!ghost_or_dead((int)i)) idx[i] = (int)k++;
  const int64_t nverts = (int64_t)t->pts.size() - M;
  if (verts)
    for (int64_t v = 0; v < nverts; ++v) {
      const P3& q = t->pts[v < M ? v : v + M];
      verts[3 * v] = q.x;
      verts[3 * v + 1] = q.y;
      verts[3 * v + 2] = q.z;
    }
  if (!simp) return k;
  long long nbad = 0;
  auto map_vertex = [&](int v) { return v < M ? v : v - M; };
  for (size_t i = 0; i < t->s.size(); ++i) {
    if (idx[i] < 0) continue;
    const RSimplex& S = t->s[i];
    int v[4] = {-1, -1, -1, -1};
    for (int j = 0; j < M; ++j) v[j] = S.v[j];
    P3 q[4];
    for (int j = 0; j < M; ++j) q[j] = t->pts[v[j]];
    if (orient(dim, q, nullptr) < 0) std::swap(v[0], v[1]);
    int nb[4] = {-1, -1, -1, -1};
    for (int o : S.nb) {
      if (!t->s[o].alive) {
        ++nbad;
        continue;
      }
      if (idx[o] < 0) continue;  // a ghost: the hull
      int missing = -1, shared = 0;
      for (int j = 0; j < M; ++j) {
        bool in_o = false;
        for (int l = 0; l < M; ++l) in_o = in_o || t->s[o].v[l] == v[j];
        if (in_o)
          ++shared;
        else
          missing = j;
      }
      if (shared != dim || nb[missing] >= 0) {
        ++nbad;
        continue;
      }
      nb[missing] = idx[o];
    }
    const int64_t r = idx[i];
    for (int j = 0; j < 4; ++j) {
      simp[4 * r + j] = j < M ? map_vertex(v[j]) : -1;
      nbr[4 * r + j] = nb[j];
    }
  }
  if (bad) *bad = nbad;
  return k;
}

void vdo_float_free(void* h) { delete (RTree*)h; }

}  // extern "C"
