// Exact geometric predicates for the GB300 Delaunay build (2D and 3D).
//
// These replace the reference's floating-point conflict test
// (circumsphere + `dist^2 < r^2`, src/geometry.rs:2-97) with exact signs:
//
//   tier 1  FP32 semi-static filter: differences taken in f64, rounded to f32,
//           determinant and permanent evaluated in f32, certified when
//           |det| > c * 2^-24 * permanent (constants derived below);
//   tier 2  FP64 filter of the same shape with c * 2^-53;
//   tier 3  exact sign with floating-point expansion arithmetic
//           (Shewchuk 1997, "Adaptive Precision Floating-Point Arithmetic and
//           Fast Robust Geometric Predicates", DCG 18: Two-Sum, Two-Product,
//           Grow-Expansion, Scale-Expansion, Compress), restated here.
//
// Conflict (`in_sphere`, src/geometry.rs:91-97) is strict in the reference: a
// point on the circumsphere is not in conflict.  An exact zero is resolved by
// symbolic perturbation of the lifted coordinate, ordered by vertex key (the
// vertex id; larger id = larger perturbation).  When the query has the
// largest id, the perturbed answer is "outside", i.e. exactly the reference's
// strict rule for its sequential insertion order (src/lib.rs:104-125), so the
// perturbed triangulation is the unique one that strict sequential insertion
// in input order produces, and any parallel order reproduces it.
//
// Conventions (checked numerically in tests/test_predicates_host.py):
//   orient3d(a,b,c,d) = det[a-d; b-d; c-d]      (positive simplex: > 0)
//   orient2d(a,b,c)   = det[a-c; b-c]           (counter-clockwise: > 0)
//   insphere(T, q)    = det[p_i - q, |p_i - q|^2]_{i=0..3}   > 0 <=> q inside
//   incircle(T, q)    = det[p_i - q, |p_i - q|^2]_{i=0..2}   > 0 <=> q inside
// With d_i = p_i - q these expand along the lifted column as
//   insphere = sum_i |d_i|^2 * O_i,   O_i = orient(T with p_i replaced by q)
//   O_i = (-1)^(i+1) det3(d_k, k != i)  in 3D,   (-1)^i det2(d_k, k != i)  in 2D.
// The O_i are the barycentric numerators of q, which is also what the
// symbolic perturbation needs: raising the lift of p_i by eps moves the
// answer by eps * O_i, raising the lift of q moves it by -eps * orient(T).
//
// Error bounds (first order; u = unit roundoff of the tier, inputs carry a
// relative error u_in from the f64 difference and the f32 rounding):
//   orient2d : 2 roundings + degree 2  -> needs 4u,  uses 8u
//   incircle : 7 roundings + degree 4  -> needs 11u, uses 14u
//   orient3d : 5 roundings + degree 3  -> needs 8u,  uses 12u
//   insphere : 12 roundings + degree 5 -> needs 17u, uses 20u
// The slack (>= 2.5u * permanent) absorbs second-order terms and underflow:
// the filters only answer when every |difference| <= 2^12 (f32) / 2^100
// (f64) and the permanent is >= 2^-60 (f32) / 2^-500 (f64); an underflowed
// product then contributes at most ~2^-96 (f32) / ~2^-767 (f64) in absolute
// terms, far below the slack.  Otherwise the next tier runs.
//
// The exact tier is exact when every coordinate is 0 or has magnitude in
// [2^-150, 2^150] (checked when points are uploaded): every expansion
// component then stays in the normal range.  Expansions are capped at
// VDP_XCAP components; exceeding it sets an error flag (never a silent wrong
// answer).
#pragma once
#include <math.h>
#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define VDP_HD __host__ __device__ __forceinline__
#define VDP_NI static __host__ __device__ __noinline__
#else
#define VDP_HD inline
#define VDP_NI static __attribute__((noinline))
#endif

#ifndef VDP_XCAP
#define VDP_XCAP 40
#endif

namespace vdp {

// Vertex record: coordinates (z = 0 in 2D) and a pad word.
struct alignas(32) VPt {
  double x, y, z, w;
};

// Per-thread counters of which tier decided each predicate.
struct Tally {
  unsigned f32, f64, exact, sos;  // per thread and launch: 32 bits suffice and keep registers free
};

enum : int { PRED_ERR_XCAP = 1 };

// ---------------------------------------------------------------------------
// Rounded arithmetic that the compiler may neither contract nor reorder.
// Host translation units that include this header build with
// -ffp-contract=off.
// ---------------------------------------------------------------------------
VDP_HD double xmul(double a, double b) {
#if defined(__CUDA_ARCH__)
  return __dmul_rn(a, b);
#else
  return a * b;
#endif
}
VDP_HD double xadd(double a, double b) {
#if defined(__CUDA_ARCH__)
  return __dadd_rn(a, b);
#else
  return a + b;
#endif
}
VDP_HD double xsub(double a, double b) {
#if defined(__CUDA_ARCH__)
  return __dsub_rn(a, b);
#else
  return a - b;
#endif
}
VDP_HD double xfma(double a, double b, double c) {
#if defined(__CUDA_ARCH__)
  return __fma_rn(a, b, c);
#else
  return fma(a, b, c);
#endif
}
VDP_HD float ffma(float a, float b, float c) {
#if defined(__CUDA_ARCH__)
  return __fmaf_rn(a, b, c);
#else
  return fmaf(a, b, c);
#endif
}
VDP_HD float fmulr(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fmul_rn(a, b);
#else
  return a * b;
#endif
}
VDP_HD float to_f32(double a) {
#if defined(__CUDA_ARCH__)
  return __double2float_rn(a);
#else
  return (float)a;
#endif
}


// Overloads used by the templated filters (same code for f32 and f64).
VDP_HD float vfma(float a, float b, float c) { return ffma(a, b, c); }
VDP_HD double vfma(double a, double b, double c) { return xfma(a, b, c); }
VDP_HD float vabs(float a) { return fabsf(a); }
VDP_HD double vabs(double a) { return fabs(a); }
VDP_HD float vmax(float a, float b) { return fmaxf(a, b); }
VDP_HD double vmax(double a, double b) { return fmax(a, b); }

// Error-free transformations.
VDP_HD void two_sum(double a, double b, double& s, double& e) {
  s = xadd(a, b);
  double bv = xsub(s, a);
  double av = xsub(s, bv);
  e = xadd(xsub(a, av), xsub(b, bv));
}
VDP_HD void two_prod(double a, double b, double& p, double& e) {
  p = xmul(a, b);
  e = xfma(a, b, -p);
}

// ---------------------------------------------------------------------------
// Expansions: nonoverlapping components in increasing magnitude, zeros
// eliminated (zero itself is the single component 0.0).
// ---------------------------------------------------------------------------
struct Xp {
  int n;
  double c[VDP_XCAP];
};

VDP_HD void xp_zero(Xp& h) {
  h.n = 1;
  h.c[0] = 0.0;
}
VDP_HD int xp_sign(const Xp& h) {
  double t = h.c[h.n - 1];
  return (t > 0.0) - (t < 0.0);
}

// h += b (Grow-Expansion, in place; zero elimination).
VDP_HD void xp_grow(Xp& h, double b, int& err) {
  double q = b;
  int k = 0;
  for (int i = 0; i < h.n; ++i) {
    double s, e;
    two_sum(q, h.c[i], s, e);
    if (e != 0.0) h.c[k++] = e;
    q = s;
  }
  if (q != 0.0 || k == 0) {
    if (k >= VDP_XCAP) {
      err |= PRED_ERR_XCAP;
      return;
    }
    h.c[k++] = q;
  }
  h.n = k;
}

// Compress (two sweeps): same value, nonadjacent components, largest
// component carrying the sign.
VDP_HD void xp_compress(Xp& h) {
  int m = h.n;
  if (m <= 1) return;
  double g[VDP_XCAP];
  int bottom = m - 1;
  double q = h.c[m - 1];
  for (int i = m - 2; i >= 0; --i) {
    double s, r;
    two_sum(q, h.c[i], s, r);
    if (r != 0.0) {
      g[bottom--] = s;
      q = r;
    } else {
      q = s;
    }
  }
  g[bottom] = q;
  int top = 0;
  for (int i = bottom + 1; i < m; ++i) {
    double s, r;
    two_sum(g[i], q, s, r);
    if (r != 0.0) h.c[top++] = r;
    q = s;
  }
  h.c[top++] = q;
  h.n = top;
}

// acc += sgn * e * b  (Scale-Expansion accumulated term by term).
VDP_HD void xp_scale_add(Xp& acc, const double* e, int ne, double b, int& err) {
  for (int i = 0; i < ne; ++i) {
    double p, t;
    two_prod(e[i], b, p, t);
    if (t != 0.0) xp_grow(acc, t, err);
    if (p != 0.0) xp_grow(acc, p, err);
  }
  xp_compress(acc);
}

// acc += sgn * e * f   with sgn = +1 / -1.
VDP_HD void xp_mul_add(Xp& acc, const double* e, int ne, const double* f, int nf,
                       double sgn, int& err) {
  for (int j = 0; j < nf; ++j) {
    if (f[j] == 0.0) continue;
    xp_scale_add(acc, e, ne, sgn * f[j], err);
  }
}

// Exact difference a - b as a one- or two-component expansion.
struct X2 {
  int n;
  double c[2];
};
VDP_HD X2 x2_diff(double a, double b) {
  X2 r;
  double s, e;
  two_sum(a, -b, s, e);
  if (e != 0.0) {
    r.n = 2;
    r.c[0] = e;
    r.c[1] = s;
  } else {
    r.n = 1;
    r.c[0] = s;
  }
  return r;
}

// m = px*qy - py*qx
VDP_HD void xp_minor2(Xp& m, const X2& px, const X2& py, const X2& qx, const X2& qy,
                      int& err) {
  xp_zero(m);
  xp_mul_add(m, px.c, px.n, qy.c, qy.n, 1.0, err);
  xp_mul_add(m, py.c, py.n, qx.c, qx.n, -1.0, err);
}

// D = det3 rows (p, q, r) = pz*m(q,r) - qz*m(p,r) + rz*m(p,q); times sgn.
VDP_HD void xp_det3(Xp& D, Xp& tmp, const X2* x, const X2* y, const X2* z, int i0, int i1,
                    int i2, double sgn, int& err) {
  xp_zero(D);
  xp_minor2(tmp, x[i1], y[i1], x[i2], y[i2], err);
  xp_mul_add(D, z[i0].c, z[i0].n, tmp.c, tmp.n, sgn, err);
  xp_minor2(tmp, x[i0], y[i0], x[i2], y[i2], err);
  xp_mul_add(D, z[i1].c, z[i1].n, tmp.c, tmp.n, -sgn, err);
  xp_minor2(tmp, x[i0], y[i0], x[i1], y[i1], err);
  xp_mul_add(D, z[i2].c, z[i2].n, tmp.c, tmp.n, sgn, err);
}

// Exact sign of det3 of three difference rows given in plain f64 inputs:
// rows are (a_k - p) for the three points a_k.
VDP_NI int exact_orient3(const VPt& a0, const VPt& a1, const VPt& a2, const VPt& p, int& err) {
  X2 x[3], y[3], z[3];
  const VPt* a[3] = {&a0, &a1, &a2};
  for (int k = 0; k < 3; ++k) {
    x[k] = x2_diff(a[k]->x, p.x);
    y[k] = x2_diff(a[k]->y, p.y);
    z[k] = x2_diff(a[k]->z, p.z);
  }
  Xp D, tmp;
  xp_det3(D, tmp, x, y, z, 0, 1, 2, 1.0, err);
  return xp_sign(D);
}

// Exact sign of det2 rows (a0 - p, a1 - p).
VDP_NI int exact_orient2(const VPt& a0, const VPt& a1, const VPt& p, int& err) {
  X2 x0 = x2_diff(a0.x, p.x), y0 = x2_diff(a0.y, p.y);
  X2 x1 = x2_diff(a1.x, p.x), y1 = x2_diff(a1.y, p.y);
  Xp m;
  xp_minor2(m, x0, y0, x1, y1, err);
  return xp_sign(m);
}

// Symbolic-perturbation decision once the lifted determinant is exactly 0.
// s[i] = sign of O_i, key[i] = vertex key of p_i, qkey = key of q.
// Returns +1 (inside) or -1 (outside); never 0.
template <int NV>
VDP_HD int sos_decide(const int* s, const int* key, int qkey) {
  bool used[NV] = {};
  for (int step = 0; step < NV; ++step) {
    int best = -1;
    for (int i = 0; i < NV; ++i)
      if (!used[i] && (best < 0 || key[i] > key[best])) best = i;
    if (key[best] < qkey) return -1;  // q carries the largest remaining perturbation
    used[best] = true;
    if (s[best] != 0) return s[best];
  }
  return -1;
}

// ---------------------------------------------------------------------------
// Exact tier in integer arithmetic.  The FP64 pipe of this GPU is narrow
// (a few operations per clock per SM) while 32-bit integer multiply-adds run
// at full rate, so the lifted determinant is evaluated on integers: every
// coordinate of the D + 2 points is m * 2^e with a 53-bit integer m (read
// from its bit pattern); with e0 the lowest set bit among them, each one is
// an integer multiple of 2^e0.  When all of them are below 2^(e0 + 126),
// the rows d = p_i - q are 127-bit integers and the determinant is computed
// exactly with 32-bit limbs (sign-magnitude, schoolbook products).  Wider
// spreads of exponents are left to the expansion path.
// ---------------------------------------------------------------------------
template <int N>
struct SInt {
  uint32_t m[N];
  int neg;
};

template <int N>
VDP_HD bool sint_zero(const SInt<N>& a) {
  uint32_t o = 0;
  for (int i = 0; i < N; ++i) o |= a.m[i];
  return o == 0;
}
template <int N>
VDP_HD int sint_sign(const SInt<N>& a) { return sint_zero(a) ? 0 : (a.neg ? -1 : 1); }

// |a| vs |b|
template <int N>
VDP_HD int mag_cmp(const uint32_t* a, const uint32_t* b) {
  for (int i = N - 1; i >= 0; --i)
    if (a[i] != b[i]) return a[i] < b[i] ? -1 : 1;
  return 0;
}

// acc += x (signed), both N limbs; the caller sizes N so that no carry leaves
template <int N>
VDP_HD void sint_add(SInt<N>& acc, const SInt<N>& x) {
  if (sint_zero(x)) return;
  if (sint_zero(acc) || acc.neg == x.neg) {
    if (sint_zero(acc)) acc.neg = x.neg;
    unsigned long long c = 0;
    for (int i = 0; i < N; ++i) {
      c += (unsigned long long)acc.m[i] + x.m[i];
      acc.m[i] = (uint32_t)c;
      c >>= 32;
    }
    return;
  }
  // opposite signs: subtract the smaller magnitude from the larger
  const uint32_t* big = acc.m;
  const uint32_t* small = x.m;
  int sign = acc.neg;
  uint32_t tmp[N];
  if (mag_cmp<N>(acc.m, x.m) < 0) {
    for (int i = 0; i < N; ++i) tmp[i] = acc.m[i];
    big = x.m;
    small = tmp;
    sign = x.neg;
  }
  long long br = 0;
  uint32_t out[N];
  for (int i = 0; i < N; ++i) {
    long long d = (long long)big[i] - small[i] - br;
    br = d < 0 ? 1 : 0;
    out[i] = (uint32_t)(d + (br << 32));
  }
  for (int i = 0; i < N; ++i) acc.m[i] = out[i];
  acc.neg = sign;
}

// r = a * b (signed), NA + NB limbs
template <int NA, int NB>
VDP_HD void sint_mul(SInt<NA + NB>& r, const SInt<NA>& a, const SInt<NB>& b) {
  for (int i = 0; i < NA + NB; ++i) r.m[i] = 0;
  for (int i = 0; i < NA; ++i) {
    if (a.m[i] == 0) continue;
    unsigned long long c = 0;
    for (int j = 0; j < NB; ++j) {
      c += (unsigned long long)a.m[i] * b.m[j] + r.m[i + j];
      r.m[i + j] = (uint32_t)c;
      c >>= 32;
    }
    for (int k = i + NB; c && k < NA + NB; ++k) {
      c += r.m[k];
      r.m[k] = (uint32_t)c;
      c >>= 32;
    }
  }
  r.neg = a.neg ^ b.neg;
}

template <int NS, int ND>
VDP_HD void sint_widen(SInt<ND>& d, const SInt<NS>& s) {
  for (int i = 0; i < ND; ++i) d.m[i] = i < NS ? s.m[i] : 0;
  d.neg = s.neg;
}

VDP_HD unsigned long long dbits(double x) {
#if defined(__CUDA_ARCH__)
  return (unsigned long long)__double_as_longlong(x);
#else
  unsigned long long b;
  memcpy(&b, &x, 8);
  return b;
#endif
}

// x = m * 2^e with the 53-bit integer m; false for 0, subnormals, inf, NaN.
VDP_HD bool dsplit(double x, unsigned long long& m, int& e, int& neg) {
  const unsigned long long b = dbits(x);
  const int ef = (int)((b >> 52) & 0x7ff);
  if (ef == 0 || ef == 0x7ff) return false;
  m = (b & 0xfffffffffffffULL) | (1ULL << 52);
  e = ef - 1075;
  neg = (int)(b >> 63);
  return true;
}

VDP_HD int ctz64(unsigned long long v) {
#if defined(__CUDA_ARCH__)
  return __ffsll((long long)v) - 1;
#else
  return __builtin_ctzll(v);
#endif
}

// Integer exact lifted determinant.  Returns 2 when the exponents spread
// too far (undecided); otherwise the sign of the determinant, and the signs
// of the minors O_i in s[] (for the perturbation rule).
template <int D>
VDP_HD int insphere_int(const VPt* p, const VPt& q, int* s) {
  constexpr int NV = D + 1;
  constexpr int NP = NV + 1;
  double c[NP][3];
  for (int i = 0; i < NV; ++i) {
    c[i][0] = p[i].x;
    c[i][1] = p[i].y;
    c[i][2] = p[i].z;
  }
  c[NV][0] = q.x;
  c[NV][1] = q.y;
  c[NV][2] = q.z;
  int e0 = 1 << 30, top = -(1 << 30);
  for (int i = 0; i < NP; ++i)
    for (int k = 0; k < D; ++k) {
      if (c[i][k] == 0.0) continue;
      unsigned long long m;
      int e, ng;
      if (!dsplit(c[i][k], m, e, ng)) return 2;
      const int lo = e + ctz64(m);
      e0 = lo < e0 ? lo : e0;
      top = e + 53 > top ? e + 53 : top;
    }
  if (top == -(1 << 30)) return 0;  // all coordinates zero
  if (top - e0 > 126) return 2;
  // coordinates as 4-limb integers (value / 2^e0)
  SInt<4> v[NP][3];
  for (int i = 0; i < NP; ++i)
    for (int k = 0; k < 3; ++k) {
      SInt<4>& z = v[i][k];
      z.m[0] = z.m[1] = z.m[2] = z.m[3] = 0;
      z.neg = 0;
      if (k >= D || c[i][k] == 0.0) continue;
      unsigned long long m;
      int e, ng;
      dsplit(c[i][k], m, e, ng);
      const int tz = ctz64(m);  // drop the zero low bits: m * 2^e, m odd
      m >>= tz;
      e += tz;
      const int sh = e - e0;  // 0 <= sh (e0 is the lowest set bit), m << sh < 2^126
      const int w = sh >> 5, b = sh & 31;
      const unsigned long long lo = m << b;
      const unsigned long long hi = b ? (m >> (64 - b)) : 0ULL;
      const uint32_t part[4] = {(uint32_t)lo, (uint32_t)(lo >> 32), (uint32_t)hi, (uint32_t)(hi >> 32)};
      for (int t = 0; t < 4; ++t)
        if (w + t < 4) z.m[w + t] = part[t];
      z.neg = ng;
    }
  // rows d_i = p_i - q
  SInt<4> d[NV][3];
  for (int i = 0; i < NV; ++i)
    for (int k = 0; k < 3; ++k) {
      d[i][k] = v[i][k];
      SInt<4> nq = v[NV][k];
      nq.neg ^= 1;
      sint_add(d[i][k], nq);
    }
  SInt<D == 3 ? 21 : 17> det;
  for (int i = 0; i < (D == 3 ? 21 : 17); ++i) det.m[i] = 0;
  det.neg = 0;
  for (int i = 0; i < NV; ++i) {
    // w_i = |d_i|^2 (8 limbs)
    SInt<8> w, t8;
    for (int j = 0; j < 8; ++j) w.m[j] = 0;
    w.neg = 0;
    for (int k = 0; k < D; ++k) {
      sint_mul<4, 4>(t8, d[i][k], d[i][k]);
      sint_add(w, t8);
    }
    if constexpr (D == 3) {
      int o[3], t = 0;
      for (int k = 0; k < 4; ++k)
        if (k != i) o[t++] = k;
      // det3 rows (x, y, z) of o[0..2], expanded along z as the expansion path does
      SInt<12> O, t12;
      for (int j = 0; j < 12; ++j) O.m[j] = 0;
      O.neg = 0;
      const int pr[3][2] = {{1, 2}, {0, 2}, {0, 1}};
      for (int r = 0; r < 3; ++r) {
        const int a = o[pr[r][0]], b = o[pr[r][1]];
        SInt<8> mnr, t2;
        sint_mul<4, 4>(mnr, d[a][0], d[b][1]);
        sint_mul<4, 4>(t2, d[a][1], d[b][0]);
        t2.neg ^= 1;
        sint_add(mnr, t2);
        sint_mul<4, 8>(t12, d[o[r]][2], mnr);
        if (r == 1) t12.neg ^= 1;
        sint_add(O, t12);
      }
      if (!(i & 1)) O.neg ^= 1;  // O_i = (-1)^(i+1) det3
      s[i] = sint_sign(O);
      SInt<20> t20;
      SInt<21> t21;
      sint_mul<8, 12>(t20, w, O);
      sint_widen(t21, t20);
      sint_add(det, t21);
    } else {
      int o[2], t = 0;
      for (int k = 0; k < 3; ++k)
        if (k != i) o[t++] = k;
      SInt<8> O, t2;
      sint_mul<4, 4>(O, d[o[0]][0], d[o[1]][1]);
      sint_mul<4, 4>(t2, d[o[0]][1], d[o[1]][0]);
      t2.neg ^= 1;
      sint_add(O, t2);
      if (i & 1) O.neg ^= 1;  // O_i = (-1)^i minor
      s[i] = sint_sign(O);
      SInt<16> t16;
      SInt<17> t17;
      sint_mul<8, 8>(t16, w, O);
      sint_widen(t17, t16);
      sint_add(det, t17);
    }
  }
  return sint_sign(det);
}

// Exact, perturbed insphere (3D) / incircle (2D).  p[i] positively oriented.
// With sos = false the plain sign of the lifted determinant is returned
// (0 when q is exactly on the circumsphere).  `tie`, when given, is set to 1
// if the answer came from the symbolic perturbation (an exact tie).
//
// XT selects the integer tier in front of the expansions.  The integer code
// is wide (many live limbs); a kernel whose register allocation must stay
// small calls the XT = 0 form, which is the expansion path alone.
template <int D, int XT = 1>
VDP_NI int exact_insphere_sos(const VPt* p, const int* key, const VPt& q, int qkey, int& err,
                              bool sos = true, int* tie = nullptr) {
  constexpr int NV = D + 1;
  if constexpr (XT != 0) {
    int si[NV];
    const int r = insphere_int<D>(p, q, si);
    if (r != 2) {
      if (r != 0 || !sos) return r;
      if (tie) *tie = 1;
      return sos_decide<NV>(si, key, qkey);
    }
  }
  X2 x[NV], y[NV], z[NV];
  for (int k = 0; k < NV; ++k) {
    x[k] = x2_diff(p[k].x, q.x);
    y[k] = x2_diff(p[k].y, q.y);
    z[k] = x2_diff(p[k].z, q.z);
  }
  Xp det, O, tmp, w;
  xp_zero(det);
  int s[NV];
  for (int i = 0; i < NV; ++i) {
    if (D == 3) {
      int o[3], t = 0;
      for (int k = 0; k < 4; ++k)
        if (k != i) o[t++] = k;
      xp_det3(O, tmp, x, y, z, o[0], o[1], o[2], (i & 1) ? 1.0 : -1.0, err);
    } else {
      int o[2], t = 0;
      for (int k = 0; k < 3; ++k)
        if (k != i) o[t++] = k;
      xp_minor2(O, x[o[0]], y[o[0]], x[o[1]], y[o[1]], err);
      if (i & 1)
        for (int c = 0; c < O.n; ++c) O.c[c] = -O.c[c];
    }
    s[i] = xp_sign(O);
    xp_zero(w);
    xp_mul_add(w, x[i].c, x[i].n, x[i].c, x[i].n, 1.0, err);
    xp_mul_add(w, y[i].c, y[i].n, y[i].c, y[i].n, 1.0, err);
    if (D == 3) xp_mul_add(w, z[i].c, z[i].n, z[i].c, z[i].n, 1.0, err);
    xp_mul_add(det, w.c, w.n, O.c, O.n, 1.0, err);
  }
  int sg = xp_sign(det);
  if (sg != 0 || !sos) return sg;
  if (tie) *tie = 1;
  return sos_decide<NV>(s, key, qkey);
}

// ---------------------------------------------------------------------------
// Filters.  Each returns +1 / -1 when certified and 0 when undecided.
// ---------------------------------------------------------------------------
constexpr float kU32 = 5.9604644775390625e-8f;    // 2^-24
constexpr double kU64 = 1.1102230246251565e-16;   // 2^-53
constexpr float kMax32 = 4096.0f;                 // 2^12
constexpr float kMinPerm32 = 8.673617379884035e-19f;  // 2^-60
constexpr double kMax64 = 1.2676506002282294e30;      // 2^100
constexpr double kMinPerm64 = 3.054936363499605e-151; // 2^-500

template <typename T>
VDP_HD int sgn_bound(T det, T bound) {
  return det > bound ? 1 : (det < -bound ? -1 : 0);
}

// insphere (3D), rows d = p_i - q.
template <typename T>
VDP_HD int insphere3_filter(const T* x, const T* y, const T* z, T cbound, T maxabs, T minperm) {
  T mx = 0;
  for (int i = 0; i < 4; ++i) {
    mx = vmax(mx, vabs(x[i]));
    mx = vmax(mx, vabs(y[i]));
    mx = vmax(mx, vabs(z[i]));
  }
  if (!(mx <= maxabs)) return 0;
  // minors m(i,j) = x_i y_j - y_i x_j and their permanents
  T m01 = vfma(x[0], y[1], -(y[0] * x[1])), p01 = vabs(x[0] * y[1]) + vabs(y[0] * x[1]);
  T m02 = vfma(x[0], y[2], -(y[0] * x[2])), p02 = vabs(x[0] * y[2]) + vabs(y[0] * x[2]);
  T m03 = vfma(x[0], y[3], -(y[0] * x[3])), p03 = vabs(x[0] * y[3]) + vabs(y[0] * x[3]);
  T m12 = vfma(x[1], y[2], -(y[1] * x[2])), p12 = vabs(x[1] * y[2]) + vabs(y[1] * x[2]);
  T m13 = vfma(x[1], y[3], -(y[1] * x[3])), p13 = vabs(x[1] * y[3]) + vabs(y[1] * x[3]);
  T m23 = vfma(x[2], y[3], -(y[2] * x[3])), p23 = vabs(x[2] * y[3]) + vabs(y[2] * x[3]);
  // O_i = (-1)^(i+1) det3(rows k != i)
  T D123 = vfma(z[3], m12, vfma(z[1], m23, -(z[2] * m13)));
  T D023 = vfma(z[3], m02, vfma(z[0], m23, -(z[2] * m03)));
  T D013 = vfma(z[3], m01, vfma(z[0], m13, -(z[1] * m03)));
  T D012 = vfma(z[2], m01, vfma(z[0], m12, -(z[1] * m02)));
  T P123 = vabs(z[1]) * p23 + vabs(z[2]) * p13 + vabs(z[3]) * p12;
  T P023 = vabs(z[0]) * p23 + vabs(z[2]) * p03 + vabs(z[3]) * p02;
  T P013 = vabs(z[0]) * p13 + vabs(z[1]) * p03 + vabs(z[3]) * p01;
  T P012 = vabs(z[0]) * p12 + vabs(z[1]) * p02 + vabs(z[2]) * p01;
  T w0 = vfma(z[0], z[0], vfma(y[0], y[0], x[0] * x[0]));
  T w1 = vfma(z[1], z[1], vfma(y[1], y[1], x[1] * x[1]));
  T w2 = vfma(z[2], z[2], vfma(y[2], y[2], x[2] * x[2]));
  T w3 = vfma(z[3], z[3], vfma(y[3], y[3], x[3] * x[3]));
  T det = vfma(w3, D012, vfma(-w2, D013, vfma(w1, D023, -(w0 * D123))));
  T perm = w0 * P123 + w1 * P023 + w2 * P013 + w3 * P012;
  if (!(perm >= minperm)) return 0;
  return sgn_bound(det, cbound * perm);
}

// incircle (2D), rows d = p_i - q.
template <typename T>
VDP_HD int incircle_filter(const T* x, const T* y, T cbound, T maxabs, T minperm) {
  T mx = 0;
  for (int i = 0; i < 3; ++i) {
    mx = vmax(mx, vabs(x[i]));
    mx = vmax(mx, vabs(y[i]));
  }
  if (!(mx <= maxabs)) return 0;
  T m12 = vfma(x[1], y[2], -(y[1] * x[2])), p12 = vabs(x[1] * y[2]) + vabs(y[1] * x[2]);
  T m02 = vfma(x[0], y[2], -(y[0] * x[2])), p02 = vabs(x[0] * y[2]) + vabs(y[0] * x[2]);
  T m01 = vfma(x[0], y[1], -(y[0] * x[1])), p01 = vabs(x[0] * y[1]) + vabs(y[0] * x[1]);
  T w0 = vfma(y[0], y[0], x[0] * x[0]);
  T w1 = vfma(y[1], y[1], x[1] * x[1]);
  T w2 = vfma(y[2], y[2], x[2] * x[2]);
  T det = vfma(w2, m01, vfma(-w1, m02, w0 * m12));
  T perm = w0 * p12 + w1 * p02 + w2 * p01;
  if (!(perm >= minperm)) return 0;
  return sgn_bound(det, cbound * perm);
}

// Full tiered conflict test: is q strictly inside the circumsphere of the
// positively oriented simplex p[0..D] (with symbolic perturbation)?
template <int D>
VDP_HD bool in_conflict(const VPt* p, const int* key, const VPt& q, int qkey, Tally& t,
                        int& err) {
  constexpr int NV = D + 1;
  double dx[NV], dy[NV], dz[NV];
  for (int i = 0; i < NV; ++i) {
    dx[i] = xsub(p[i].x, q.x);
    dy[i] = xsub(p[i].y, q.y);
    dz[i] = xsub(p[i].z, q.z);
  }
  float fx[NV], fy[NV], fz[NV];
  for (int i = 0; i < NV; ++i) {
    fx[i] = to_f32(dx[i]);
    fy[i] = to_f32(dy[i]);
    fz[i] = to_f32(dz[i]);
  }
  int s;
  if (D == 3)
    s = insphere3_filter<float>(fx, fy, fz, 20.0f * kU32, kMax32, kMinPerm32);
  else
    s = incircle_filter<float>(fx, fy, 14.0f * kU32, kMax32, kMinPerm32);
  if (s != 0) {
    t.f32++;
    return s > 0;
  }
  if (D == 3)
    s = insphere3_filter<double>(dx, dy, dz, 20.0 * kU64, kMax64, kMinPerm64);
  else
    s = incircle_filter<double>(dx, dy, 14.0 * kU64, kMax64, kMinPerm64);
  if (s != 0) {
    t.f64++;
    return s > 0;
  }
  t.exact++;
  int tie = 0;
  s = exact_insphere_sos<D>(p, key, q, qkey, err, true, &tie);
  t.sos += tie;
  return s > 0;
}

// Unperturbed tiered sign of the lifted determinant (validator use).
template <int D>
VDP_HD int insphere_sign(const VPt* p, const VPt& q, Tally& t, int& err) {
  constexpr int NV = D + 1;
  double dx[NV], dy[NV], dz[NV];
  for (int i = 0; i < NV; ++i) {
    dx[i] = xsub(p[i].x, q.x);
    dy[i] = xsub(p[i].y, q.y);
    dz[i] = xsub(p[i].z, q.z);
  }
  int s;
  if (D == 3)
    s = insphere3_filter<double>(dx, dy, dz, 20.0 * kU64, kMax64, kMinPerm64);
  else
    s = incircle_filter<double>(dx, dy, 14.0 * kU64, kMax64, kMinPerm64);
  if (s != 0) {
    t.f64++;
    return s;
  }
  t.exact++;
  int key[NV] = {};
  return exact_insphere_sos<D>(p, key, q, 0, err, false);
}

// ---------------------------------------------------------------------------
// Orientation of the point p against the faces of a positively oriented
// simplex v[0..D]: o_j = orient(v with v_j replaced by p) for each face j
// whose bit is set in `mask`.  Returns the first face with o_j < 0 (with
// STRICT: o_j <= 0), or -1 when p is inside the closed (STRICT: open)
// simplex w.r.t. those faces.
// ---------------------------------------------------------------------------
template <typename T>
VDP_HD int det3_filter(T ax, T ay, T az, T bx, T by, T bz, T cx, T cy, T cz, T cbound,
                       T minperm) {
  T mbc = vfma(bx, cy, -(by * cx)), pbc = vabs(bx * cy) + vabs(by * cx);
  T mac = vfma(ax, cy, -(ay * cx)), pac = vabs(ax * cy) + vabs(ay * cx);
  T mab = vfma(ax, by, -(ay * bx)), pab = vabs(ax * by) + vabs(ay * bx);
  T det = vfma(cz, mab, vfma(az, mbc, -(bz * mac)));
  T perm = vabs(az) * pbc + vabs(bz) * pac + vabs(cz) * pab;
  if (!(perm >= minperm)) return 0;
  return sgn_bound(det, cbound * perm);
}

template <typename T>
VDP_HD int det2_filter(T ax, T ay, T bx, T by, T cbound, T minperm) {
  T det = vfma(ax, by, -(ay * bx));
  T perm = vabs(ax * by) + vabs(ay * bx);
  if (!(perm >= minperm)) return 0;
  return sgn_bound(det, cbound * perm);
}

template <int D, bool STRICT = false>
VDP_HD int exit_face(const VPt* v, const VPt& p, unsigned mask, Tally& t, int& err) {
  constexpr int NV = D + 1;
  double dx[NV], dy[NV], dz[NV];
  float fx[NV], fy[NV], fz[NV];
  float fmx = 0.0f;
  double dmx = 0.0;
  for (int i = 0; i < NV; ++i) {
    dx[i] = xsub(v[i].x, p.x);
    dy[i] = xsub(v[i].y, p.y);
    dz[i] = xsub(v[i].z, p.z);
    fx[i] = to_f32(dx[i]);
    fy[i] = to_f32(dy[i]);
    fz[i] = to_f32(dz[i]);
    fmx = vmax(fmx, vmax(vabs(fx[i]), vmax(vabs(fy[i]), vabs(fz[i]))));
    dmx = vmax(dmx, vmax(vabs(dx[i]), vmax(vabs(dy[i]), vabs(dz[i]))));
  }
  const bool ok32 = fmx <= kMax32;
  const bool ok64 = dmx <= kMax64;
  for (int j = 0; j < NV; ++j) {
    if (!((mask >> j) & 1u)) continue;
    int o[D], k = 0;
    for (int i = 0; i < NV; ++i)
      if (i != j) o[k++] = i;
    int s = 0;
    if (D == 3) {
      if (ok32)
        s = det3_filter<float>(fx[o[0]], fy[o[0]], fz[o[0]], fx[o[1]], fy[o[1]], fz[o[1]],
                               fx[o[2]], fy[o[2]], fz[o[2]], 12.0f * kU32, kMinPerm32);
      if (s != 0) {
        t.f32++;
      } else {
        if (ok64)
          s = det3_filter<double>(dx[o[0]], dy[o[0]], dz[o[0]], dx[o[1]], dy[o[1]], dz[o[1]],
                                  dx[o[2]], dy[o[2]], dz[o[2]], 12.0 * kU64, kMinPerm64);
        if (s != 0) {
          t.f64++;
        } else {
          t.exact++;
          s = exact_orient3(v[o[0]], v[o[1]], v[o[2]], p, err);
        }
      }
      if (!(j & 1)) s = -s;  // (-1)^(j+1)
    } else {
      if (ok32)
        s = det2_filter<float>(fx[o[0]], fy[o[0]], fx[o[1]], fy[o[1]], 8.0f * kU32, kMinPerm32);
      if (s != 0) {
        t.f32++;
      } else {
        if (ok64)
          s = det2_filter<double>(dx[o[0]], dy[o[0]], dx[o[1]], dy[o[1]], 8.0 * kU64, kMinPerm64);
        if (s != 0) {
          t.f64++;
        } else {
          t.exact++;
          s = exact_orient2(v[o[0]], v[o[1]], p, err);
        }
      }
      if (j & 1) s = -s;  // (-1)^j
    }
    if (s < 0 || (STRICT && s == 0)) return j;
  }
  return -1;
}

// ---------------------------------------------------------------------------
// FP32 tier on split coordinates.  Each coordinate is kept as a pair of
// floats, hi = fl32(x) and lo = fl32(x - hi), so a difference a - q is formed
// in f32 alone as (a_hi - q_hi) + (a_lo - q_lo) and the first tier never
// touches the FP64 pipe.  Error of one difference (u = 2^-24, M = largest
// |coordinate| involved):  |d~ - d| <= 2u|d| + 10u^2 M.  The relative part
// doubles the input error of the earlier analysis; the absolute part is
// propagated through the derivative of each determinant (sum over the inputs
// of |d det / d d_k| <= #monomials * degree * L^(degree-1), L = max |d~|):
//   orient2d : 6u   relative -> 10u * perm,  40 L   u^2 M -> 128 u^2 M L
//   incircle : 15u  relative -> 20u * perm,  480 L^3 u^2 M -> 1024 u^2 M L^3
//   orient3d : 11u  relative -> 16u * perm,  180 L^2 u^2 M -> 512 u^2 M L^2
//   insphere : 22u  relative -> 28u * perm,  3600 L^4 u^2 M -> 8192 u^2 M L^4
// A point whose split is not accurate (0 < |x| < 2^-60 or |x| > 2^60) carries
// a NaN in hw, which fails every comparison and sends the test to FP64.
// ---------------------------------------------------------------------------
struct alignas(32) FPt {
  float hx, hy, hz, hw;
  float lx, ly, lz, lw;
};

VDP_HD float fsub_rn(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fsub_rn(a, b);
#else
  return a - b;
#endif
}
VDP_HD float fadd_rn(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fadd_rn(a, b);
#else
  return a + b;
#endif
}

VDP_HD FPt split_point(double x, double y, double z) {
  FPt f;
  const double c[3] = {x, y, z};
  float h[3], l[3];
  bool ok = true;
  for (int k = 0; k < 3; ++k) {
    const double a = fabs(c[k]);
    if (a != 0.0 && (a < 8.673617379884035e-19 || a > 1.152921504606847e18)) ok = false;  // 2^-60, 2^60
    h[k] = to_f32(c[k]);
    l[k] = to_f32(xsub(c[k], (double)h[k]));
  }
  f.hx = h[0];
  f.hy = h[1];
  f.hz = h[2];
  f.lx = l[0];
  f.ly = l[1];
  f.lz = l[2];
  f.hw = ok ? 0.0f : __builtin_nanf("");
  f.lw = 0.0f;
  return f;
}

VDP_HD float hl_diff(float ah, float al, float qh, float ql) { return fadd_rn(fsub_rn(ah, qh), fsub_rn(al, ql)); }

// Differences of NV points to p and the magnitudes M (coordinates) and L
// (differences) of the tier's absolute error term.
template <int NV>
VDP_HD void hl_diffs(const FPt* v, const FPt& p, float* x, float* y, float* z, float& M, float& L) {
  M = fmaxf(fabsf(p.hx), fmaxf(fabsf(p.hy), fabsf(p.hz)));
  float flag = p.hw;  // NaN if any point cannot use this tier (fmaxf would drop it)
  L = 0.0f;
  for (int i = 0; i < NV; ++i) {
    x[i] = hl_diff(v[i].hx, v[i].lx, p.hx, p.lx);
    y[i] = hl_diff(v[i].hy, v[i].ly, p.hy, p.ly);
    z[i] = hl_diff(v[i].hz, v[i].lz, p.hz, p.lz);
    M = fmaxf(M, fmaxf(fabsf(v[i].hx), fmaxf(fabsf(v[i].hy), fabsf(v[i].hz))));
    flag += v[i].hw;
    L = fmaxf(L, fmaxf(fabsf(x[i]), fmaxf(fabsf(y[i]), fabsf(z[i]))));
  }
  M += flag;
  L += flag;
}

constexpr float kU32sq = 3.552713678800501e-15f;  // 2^-48

// insphere / incircle on split coordinates: +1 / -1 certified, 0 undecided.
//
// Two bounds, cheap first.  The tight one is the error bound above with the
// permanent perm (the determinant with every product replaced by its
// magnitude).  With L = max |difference|, every |w_i| <= 3 L^2 and every
// permanent minor <= 6 L^3 (3D; 2D: w <= 2 L^2, minor <= 2 L^2), so perm <=
// 72 L^5 (2D: 12 L^4) and the tight relative part 28u perm (2D: 20u perm) is
// below 2048u L^5 = 2^-13 L^5 (2D: 256u L^4 = 2^-16 L^4) with 1.5% to spare
// for the rounding of the bound itself.  A determinant above that needs no
// permanent at all; only the rest pays for it.  The cheap bound is used for
// L >= 2^-12 (2D: 2^-15), where L^5 (L^4) stays far from underflow.
template <int D>
VDP_HD int insphere_hl(const FPt* v, const FPt& q) {
  constexpr int NV = D + 1;
  float x[NV], y[NV], z[NV], M, L;
  hl_diffs<NV>(v, q, x, y, z, M, L);
  if (!(L <= kMax32) || !(M <= 1.152921504606847e18f)) return 0;
  if (D == 3) {
    const float abs_term = 8192.0f * kU32sq * M * (L * L) * (L * L);
    float m01 = ffma(x[0], y[1], -(y[0] * x[1]));
    float m02 = ffma(x[0], y[2], -(y[0] * x[2]));
    float m03 = ffma(x[0], y[3], -(y[0] * x[3]));
    float m12 = ffma(x[1], y[2], -(y[1] * x[2]));
    float m13 = ffma(x[1], y[3], -(y[1] * x[3]));
    float m23 = ffma(x[2], y[3], -(y[2] * x[3]));
    float D123 = ffma(z[3], m12, ffma(z[1], m23, -(z[2] * m13)));
    float D023 = ffma(z[3], m02, ffma(z[0], m23, -(z[2] * m03)));
    float D013 = ffma(z[3], m01, ffma(z[0], m13, -(z[1] * m03)));
    float D012 = ffma(z[2], m01, ffma(z[0], m12, -(z[1] * m02)));
    float w0 = ffma(z[0], z[0], ffma(y[0], y[0], x[0] * x[0]));
    float w1 = ffma(z[1], z[1], ffma(y[1], y[1], x[1] * x[1]));
    float w2 = ffma(z[2], z[2], ffma(y[2], y[2], x[2] * x[2]));
    float w3 = ffma(z[3], z[3], ffma(y[3], y[3], x[3] * x[3]));
    float det = ffma(w3, D012, ffma(-w2, D013, ffma(w1, D023, -(w0 * D123))));
    if (L >= 2.44140625e-4f) {  // 2^-12
      const float L2 = L * L;
      const float cheap = 1.220703125e-4f * (L2 * L2 * L) + 1.001f * abs_term;  // 2^-13 L^5
      if (det > cheap) return 1;
      if (det < -cheap) return -1;
    }
    float p01 = fabsf(x[0] * y[1]) + fabsf(y[0] * x[1]);
    float p02 = fabsf(x[0] * y[2]) + fabsf(y[0] * x[2]);
    float p03 = fabsf(x[0] * y[3]) + fabsf(y[0] * x[3]);
    float p12 = fabsf(x[1] * y[2]) + fabsf(y[1] * x[2]);
    float p13 = fabsf(x[1] * y[3]) + fabsf(y[1] * x[3]);
    float p23 = fabsf(x[2] * y[3]) + fabsf(y[2] * x[3]);
    float P123 = fabsf(z[1]) * p23 + fabsf(z[2]) * p13 + fabsf(z[3]) * p12;
    float P023 = fabsf(z[0]) * p23 + fabsf(z[2]) * p03 + fabsf(z[3]) * p02;
    float P013 = fabsf(z[0]) * p13 + fabsf(z[1]) * p03 + fabsf(z[3]) * p01;
    float P012 = fabsf(z[0]) * p12 + fabsf(z[1]) * p02 + fabsf(z[2]) * p01;
    float perm = w0 * P123 + w1 * P023 + w2 * P013 + w3 * P012;
    if (!(perm >= kMinPerm32)) return 0;
    return sgn_bound(det, 28.0f * kU32 * perm + abs_term);
  } else {
    const float abs_term = 1024.0f * kU32sq * M * (L * L) * L;
    float m12 = ffma(x[1], y[2], -(y[1] * x[2]));
    float m02 = ffma(x[0], y[2], -(y[0] * x[2]));
    float m01 = ffma(x[0], y[1], -(y[0] * x[1]));
    float w0 = ffma(y[0], y[0], x[0] * x[0]);
    float w1 = ffma(y[1], y[1], x[1] * x[1]);
    float w2 = ffma(y[2], y[2], x[2] * x[2]);
    float det = ffma(w2, m01, ffma(-w1, m02, w0 * m12));
    if (L >= 3.0517578125e-5f) {  // 2^-15
      const float L2 = L * L;
      const float cheap = 1.52587890625e-5f * (L2 * L2) + 1.001f * abs_term;  // 2^-16 L^4
      if (det > cheap) return 1;
      if (det < -cheap) return -1;
    }
    float p12 = fabsf(x[1] * y[2]) + fabsf(y[1] * x[2]);
    float p02 = fabsf(x[0] * y[2]) + fabsf(y[0] * x[2]);
    float p01 = fabsf(x[0] * y[1]) + fabsf(y[0] * x[1]);
    float perm = w0 * p12 + w1 * p02 + w2 * p01;
    if (!(perm >= kMinPerm32)) return 0;
    return sgn_bound(det, 20.0f * kU32 * perm + abs_term);
  }
}

// The FP64 and exact tiers of in_conflict (used when the split tier is undecided).
template <int D, int XT = 1>
VDP_HD bool in_conflict_64(const VPt* p, const int* key, const VPt& q, int qkey, Tally& t, int& err) {
  constexpr int NV = D + 1;
  double dx[NV], dy[NV], dz[NV];
  for (int i = 0; i < NV; ++i) {
    dx[i] = xsub(p[i].x, q.x);
    dy[i] = xsub(p[i].y, q.y);
    dz[i] = xsub(p[i].z, q.z);
  }
  int s;
  if (D == 3)
    s = insphere3_filter<double>(dx, dy, dz, 20.0 * kU64, kMax64, kMinPerm64);
  else
    s = incircle_filter<double>(dx, dy, 14.0 * kU64, kMax64, kMinPerm64);
  if (s != 0) {
    t.f64++;
    return s > 0;
  }
  t.exact++;
  int tie = 0;
  s = exact_insphere_sos<D, XT>(p, key, q, qkey, err, true, &tie);
  t.sos += tie;
  return s > 0;
}

// Tiered conflict test starting from split coordinates; load64(v, q) fills
// the f64 coordinates when the f32 tier cannot decide.
template <int D, int XT = 1, class Load64>
VDP_HD bool in_conflict_hl(const FPt* fv, const int* key, const FPt& fq, int qkey, Tally& t, int& err,
                           Load64 load64) {
  const int s = insphere_hl<D>(fv, fq);
  if (s != 0) {
    t.f32++;
    return s > 0;
  }
  VPt v[D + 1], q;
  load64(v, q);
  return in_conflict_64<D, XT>(v, key, q, qkey, t, err);
}

// exit_face on split coordinates (same contract as exit_face).
template <int D, bool STRICT = false, class Load64>
VDP_HD int exit_face_hl(const FPt* fv, const FPt& fp, unsigned mask, Tally& t, int& err, Load64 load64) {
  constexpr int NV = D + 1;
  float x[NV], y[NV], z[NV], M, L;
  hl_diffs<NV>(fv, fp, x, y, z, M, L);
  const bool ok32 = (L <= kMax32) && (M <= 1.152921504606847e18f);
  const float abs3 = 512.0f * kU32sq * M * L * L, abs2 = 128.0f * kU32sq * M * L;
  bool have64 = false;
  VPt v[NV], p;
  double dx[NV], dy[NV], dz[NV], dmx = 0.0;
  for (int j = 0; j < NV; ++j) {
    if (!((mask >> j) & 1u)) continue;
    int o[D], k = 0;
    for (int i = 0; i < NV; ++i)
      if (i != j) o[k++] = i;
    int s = 0;
    if (ok32) {
      if (D == 3) {
        float mbc = ffma(x[o[1]], y[o[2]], -(y[o[1]] * x[o[2]]));
        float pbc = fabsf(x[o[1]] * y[o[2]]) + fabsf(y[o[1]] * x[o[2]]);
        float mac = ffma(x[o[0]], y[o[2]], -(y[o[0]] * x[o[2]]));
        float pac = fabsf(x[o[0]] * y[o[2]]) + fabsf(y[o[0]] * x[o[2]]);
        float mab = ffma(x[o[0]], y[o[1]], -(y[o[0]] * x[o[1]]));
        float pab = fabsf(x[o[0]] * y[o[1]]) + fabsf(y[o[0]] * x[o[1]]);
        float det = ffma(z[o[2]], mab, ffma(z[o[0]], mbc, -(z[o[1]] * mac)));
        float perm = fabsf(z[o[0]]) * pbc + fabsf(z[o[1]]) * pac + fabsf(z[o[2]]) * pab;
        if (perm >= kMinPerm32) s = sgn_bound(det, 16.0f * kU32 * perm + abs3);
      } else {
        float det = ffma(x[o[0]], y[o[1]], -(y[o[0]] * x[o[1]]));
        float perm = fabsf(x[o[0]] * y[o[1]]) + fabsf(y[o[0]] * x[o[1]]);
        if (perm >= kMinPerm32) s = sgn_bound(det, 10.0f * kU32 * perm + abs2);
      }
    }
    if (s != 0) {
      t.f32++;
    } else {
      if (!have64) {
        load64(v, p);
        for (int i = 0; i < NV; ++i) {
          dx[i] = xsub(v[i].x, p.x);
          dy[i] = xsub(v[i].y, p.y);
          dz[i] = xsub(v[i].z, p.z);
          dmx = fmax(dmx, fmax(fabs(dx[i]), fmax(fabs(dy[i]), fabs(dz[i]))));
        }
        have64 = true;
      }
      if (dmx <= kMax64) {
        if (D == 3)
          s = det3_filter<double>(dx[o[0]], dy[o[0]], dz[o[0]], dx[o[1]], dy[o[1]], dz[o[1]], dx[o[2]],
                                  dy[o[2]], dz[o[2]], 12.0 * kU64, kMinPerm64);
        else
          s = det2_filter<double>(dx[o[0]], dy[o[0]], dx[o[1]], dy[o[1]], 8.0 * kU64, kMinPerm64);
      }
      if (s != 0) {
        t.f64++;
      } else {
        t.exact++;
        s = D == 3 ? exact_orient3(v[o[0]], v[o[1]], v[o[2]], p, err) : exact_orient2(v[o[0]], v[o[1]], p, err);
      }
    }
    if (D == 3) {
      if (!(j & 1)) s = -s;  // (-1)^(j+1)
    } else {
      if (j & 1) s = -s;  // (-1)^j
    }
    if (s < 0 || (STRICT && s == 0)) return j;
  }
  return -1;
}

// Exact coordinate equality (duplicate detection).
VDP_HD bool same_point(const VPt& a, const VPt& b) {
  return a.x == b.x && a.y == b.y && a.z == b.z;
}

}  // namespace vdp
