// Shared host/device building blocks of the collocation-BEM path: quad8 and
// line3 shape functions, Gauss-Legendre table access, Telles transformation,
// quasi-singular order estimation, nearest-element-point search and the
// decomposed exponential. Compiled both by nvcc (device kernels) and by the
// host C++ compiler (mesh preparation on the caller side of the C-ABI).
//
// The algorithms and constants follow MultiFEBE's lib/fbem (citations at each
// function). Where the reference computes in binary128 (the nearest-point
// Newton step, lib/fbem/src/geometry.f90:5107-5150) this code uses
// double-double arithmetic, which rounds to the same binary64 results.
#pragma once
#include <cmath>
#include <cstdint>

#ifdef __CUDACC__
#define MFB_HD __host__ __device__ __forceinline__
#define MFB_HDN __host__ __device__
#else
#define MFB_HD inline
#define MFB_HDN
#endif

namespace mfb {

constexpr double kPi = 3.14159265358979323846264338328;
constexpr double k2Pi = 6.28318530717958623199592693709;
constexpr double kPi2 = 1.57079632679489661923132169164;
constexpr double k1_4Pi = 0.07957747154594767280411105048;
constexpr double kXiTol = 0.5e-12;  // check_xi_tolerance, shape_functions.f90:280

// ----------------------------------------------------------------------------
// Gauss-Legendre tables: 32 rules on [-1,1] (gl11) and [0,1] (gl01), point k of
// rule n at [(n-1)*32 + k-1]. Device code reads them from __constant__ memory
// (defined in the kernel translation unit), host code from host_tables.cpp.
// ----------------------------------------------------------------------------
struct GLTables {
  double x11[1024], w11[1024], x01[1024], w01[1024];
};
#ifdef __CUDACC__
// defined here: all device code lives in one translation unit (mfbem_abi.cu)
__constant__ GLTables c_gl;
#endif
extern GLTables h_gl;

MFB_HD double gl11x(int k, int n) {
#ifdef __CUDA_ARCH__
  return c_gl.x11[(n - 1) * 32 + k - 1];
#else
  return h_gl.x11[(n - 1) * 32 + k - 1];
#endif
}
MFB_HD double gl11w(int k, int n) {
#ifdef __CUDA_ARCH__
  return c_gl.w11[(n - 1) * 32 + k - 1];
#else
  return h_gl.w11[(n - 1) * 32 + k - 1];
#endif
}
MFB_HD double gl01x(int k, int n) {
#ifdef __CUDA_ARCH__
  return c_gl.x01[(n - 1) * 32 + k - 1];
#else
  return h_gl.x01[(n - 1) * 32 + k - 1];
#endif
}
MFB_HD double gl01w(int k, int n) {
#ifdef __CUDA_ARCH__
  return c_gl.w01[(n - 1) * 32 + k - 1];
#else
  return h_gl.w01[(n - 1) * 32 + k - 1];
#endif
}

// ----------------------------------------------------------------------------
// Double-double arithmetic (Dekker / Knuth error-free transformations)
// ----------------------------------------------------------------------------
struct dd {
  double hi, lo;
  dd() = default;
  MFB_HD dd(double a) : hi(a), lo(0.0) {}
  MFB_HD dd(double a, double b) : hi(a), lo(b) {}
};
MFB_HD dd dd_from(double a) { return dd{a, 0.0}; }
MFB_HD dd two_sum(double a, double b) {
  double s = a + b;
  double bb = s - a;
  double e = (a - (s - bb)) + (b - bb);
  return dd{s, e};
}
MFB_HD dd quick_two_sum(double a, double b) {
  double s = a + b;
  return dd{s, b - (s - a)};
}
MFB_HD dd two_prod(double a, double b) {
  double p = a * b;
  return dd{p, fma(a, b, -p)};
}
MFB_HD dd operator+(dd a, dd b) {
  dd s = two_sum(a.hi, b.hi);
  dd t = two_sum(a.lo, b.lo);
  s.lo += t.hi;
  s = quick_two_sum(s.hi, s.lo);
  s.lo += t.lo;
  return quick_two_sum(s.hi, s.lo);
}
MFB_HD dd operator-(dd a) { return dd{-a.hi, -a.lo}; }
MFB_HD dd operator-(dd a, dd b) { return a + (-b); }
MFB_HD dd operator*(dd a, dd b) {
  dd p = two_prod(a.hi, b.hi);
  p.lo += a.hi * b.lo + a.lo * b.hi;
  return quick_two_sum(p.hi, p.lo);
}
MFB_HD dd operator/(dd a, dd b) {
  double q1 = a.hi / b.hi;
  dd r = a - b * dd_from(q1);
  double q2 = r.hi / b.hi;
  r = r - b * dd_from(q2);
  double q3 = r.hi / b.hi;
  dd q = quick_two_sum(q1, q2);
  return q + dd_from(q3);
}
MFB_HD double dd_round(dd a) { return a.hi + a.lo; }
MFB_HD bool dd_lt(dd a, dd b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
MFB_HD dd dd_sqrt(dd a) {
  if (a.hi <= 0.0) return dd{0.0, 0.0};
  double x = sqrt(a.hi);
  dd xx = two_prod(x, x);
  dd r = a - xx;
  double corr = r.hi / (2.0 * x);
  return quick_two_sum(x, corr);
}

// ----------------------------------------------------------------------------
// Shape functions (continuous, delta = 0): resources_shape_functions/
// phi_quad8.rc, dphidxi{1,2}_quad8.rc, phi_quad4.rc, phi_line3.rc,
// dphidxi_line3.rc. quad8 node order 1(-1,-1) 2(1,-1) 3(1,1) 4(-1,1) 5(0,-1)
// 6(1,0) 7(0,1) 8(-1,0).
// ----------------------------------------------------------------------------
MFB_HD double q8xi(int k, int c) {
  // reference coordinates of quad8 node k (0-based), xi_quad8.rc
  const int t = k * 2 + c;
  // packed table: (-1,-1) (1,-1) (1,1) (-1,1) (0,-1) (1,0) (0,1) (-1,0)
  const signed char v[16] = {-1, -1, 1, -1, 1, 1, -1, 1, 0, -1, 1, 0, 0, 1, -1, 0};
  return (double)v[t];
}
// quad8 edges (vertex, vertex, mid), shape_functions.f90:841-880
MFB_HD int q8edge(int e, int j) {
  const signed char v[12] = {0, 1, 4, 1, 2, 5, 2, 3, 6, 3, 0, 7};
  return v[e * 3 + j];
}

template <typename T>
MFB_HD void phi_q8(T x1, T x2, T phi[8]) {
  const T one = T(1.0), q = T(0.25), h = T(0.5), two = T(2.0);
  T a3 = q * (one + x1), a4 = q * (one - x1);
  T a5 = one + x2, a6 = one - x2;
  T a7 = one - x1 * x1, a8 = one - x2 * x2;
  phi[0] = a4 * a6 * (-x1 - a5);
  phi[1] = a3 * a6 * (x1 - a5);
  phi[2] = a3 * a5 * (x1 - a6);
  phi[3] = a4 * a5 * (-x1 - a6);
  phi[4] = h * a6 * a7;
  phi[5] = two * a3 * a8;
  phi[6] = h * a5 * a7;
  phi[7] = two * a4 * a8;
}
template <typename T>
MFB_HD void dphi_q8(T x1, T x2, T d1[8], T d2[8]) {
  const T one = T(1.0), q = T(0.25), h = T(0.5), two = T(2.0);
  {
    T a3 = x2 + one, a4 = x2 - one, a5 = x2 + two * x1, a6 = x2 - two * x1, a7 = -q, a8 = -x1;
    d1[0] = a7 * a4 * a5;
    d1[1] = -a7 * a4 * a6;
    d1[2] = -a7 * a3 * a5;
    d1[3] = a7 * a3 * a6;
    d1[4] = -a8 * a4;
    d1[5] = h * (-one) * a3 * a4;
    d1[6] = a8 * a3;
    d1[7] = -d1[5];
  }
  {
    T a3 = x1 + one, a4 = x1 - one, a5 = two * x2 + x1, a6 = two * x2 - x1, a7 = -q, a8 = -x2;
    d2[0] = a7 * a4 * a5;
    d2[1] = -a7 * a3 * a6;
    d2[2] = -a7 * a3 * a5;
    d2[3] = a7 * a4 * a6;
    d2[4] = -h * (-one) * a3 * a4;
    d2[5] = a8 * a3;
    d2[6] = -d2[4];
    d2[7] = -a8 * a4;
  }
}
MFB_HD void phi_q4(double x1, double x2, double p[4]) {
  double a3 = 0.25 * (1.0 + x1), a4 = 0.25 * (1.0 - x1), a5 = 1.0 + x2, a6 = 1.0 - x2;
  p[0] = a4 * a6;
  p[1] = a3 * a6;
  p[2] = a3 * a5;
  p[3] = a4 * a5;
}
MFB_HD void dphi_q4(double x1, double x2, double d1[4], double d2[4]) {
  d1[0] = -0.25 * (1.0 - x2);
  d1[1] = 0.25 * (1.0 - x2);
  d1[2] = 0.25 * (1.0 + x2);
  d1[3] = -0.25 * (1.0 + x2);
  d2[0] = -0.25 * (1.0 - x1);
  d2[1] = -0.25 * (1.0 + x1);
  d2[2] = 0.25 * (1.0 + x1);
  d2[3] = 0.25 * (1.0 - x1);
}
template <typename T>
MFB_HD void phi_l3(T xi, T p[3]) {
  const T h = T(0.5), one = T(1.0);
  T a2 = h * xi, a3 = xi - one, a4 = xi + one;
  p[0] = a2 * a3;
  p[1] = a2 * a4;
  p[2] = -a3 * a4;
}
template <typename T>
MFB_HD void dphi_l3(T xi, T d[3]) {
  const T h = T(0.5), two = T(2.0);
  d[0] = xi - h;
  d[1] = xi + h;
  d[2] = -two * xi;
}
// dd flavours (the reference evaluates these formulas in binary128)
MFB_HD dd ddmul(dd a, double b) { return a * dd_from(b); }

MFB_HD void geom_q8(const double* x /*8x3*/, double xi1, double xi2, double xp[3], double T1[3], double T2[3],
                    double phi[8]) {
  double d1[8], d2[8];
  phi_q8<double>(xi1, xi2, phi);
  dphi_q8<double>(xi1, xi2, d1, d2);
  xp[0] = xp[1] = xp[2] = 0.0;
  T1[0] = T1[1] = T1[2] = 0.0;
  T2[0] = T2[1] = T2[2] = 0.0;
  for (int k = 0; k < 8; ++k)
    for (int c = 0; c < 3; ++c) {
      xp[c] = xp[c] + phi[k] * x[3 * k + c];
      T1[c] = T1[c] + d1[k] * x[3 * k + c];
      T2[c] = T2[c] + d2[k] * x[3 * k + c];
    }
}
MFB_HD void cross3(const double a[3], const double b[3], double c[3]) {
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}
MFB_HD double norm3(const double a[3]) { return sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]); }

// ----------------------------------------------------------------------------
// Element lengths: fbem_jacobian3d_1d + fbem_length3d in tolerance mode
// (geometry.f90:1469-1504, 2794-2882) and fbem_characteristic_length
// (geometry.f90:3357-3389).
// ----------------------------------------------------------------------------
MFB_HD double jac_l3(const double* x /*3x3*/, double xi) {
  double d[3];
  dphi_l3<double>(xi, d);
  double t0 = 0, t1 = 0, t2 = 0;
  for (int i = 0; i < 3; ++i) {
    t0 = t0 + d[i] * x[3 * i + 0];
    t1 = t1 + d[i] * x[3 * i + 1];
    t2 = t2 + d[i] * x[3 * i + 2];
  }
  return sqrt(t0 * t0 + t1 * t1 + t2 * t2);
}
MFB_HD double length_l3(const double* x, double tol) {
  double ltol = (tol <= 0.0) ? 1e-6 : tol;
  double err = ltol + 1.0;
  double len = jac_l3(x, gl11x(1, 1)) * gl11w(1, 1);
  int j = 4;
  while (err >= ltol) {
    double old = len;
    len = 0.0;
    for (int i = 1; i <= j; ++i) len = len + jac_l3(x, gl11x(i, j)) * gl11w(i, j);
    err = fabs((old - len) / len);
    j += 3;
    if (j >= 32) {
      len = 0.0;
      for (int i = 1; i <= 31; ++i) len = len + jac_l3(x, gl11x(i, 31)) * gl11w(i, 31);
      len = 0.0;
      for (int i = 1; i <= 32; ++i) len = len + jac_l3(x, gl11x(i, 32)) * gl11w(i, 32);
      break;
    }
  }
  return len;
}
MFB_HD double clen_q8(const double* x, double tol) {
  double lmax = 0.0;
  for (int e = 0; e < 4; ++e) {
    double xe[9];
    for (int n = 0; n < 3; ++n)
      for (int c = 0; c < 3; ++c) xe[3 * n + c] = x[3 * q8edge(e, n) + c];
    double l = length_l3(xe, tol);
    if (e == 0 || l > lmax) lmax = l;
  }
  return lmax;
}

// ----------------------------------------------------------------------------
// Telles transformation, telles_transformation.f90:77-162,221-233
// ----------------------------------------------------------------------------
MFB_HD double telles_barr(double d) {
  double r = (d < 3.0) ? d / (0.89039 * d + 0.32883) : 1.0;
  return r > 1.0 ? 1.0 : r;
}
struct Telles {
  double a, b, c, d;
};
MFB_HD Telles telles11(double bx, double br) {
  double w = bx / (1.0 + 2.0 * br);
  double p = 1.0 / (3.0 * (1.0 + 2.0 * br)) * (3.0 - 2.0 * br - 3.0 * w * bx);
  double q = w / 2.0 * ((3.0 - 2.0 * br) / (1.0 + 2.0 * br) - 2.0 * (w * w) - 1.0);
  double R2 = sqrt(q * q + p * p * p);
  double R31 = -q + R2, R32 = -q - R2;
  const double d13 = 1.0 / 3.0;
  R31 = (R31 >= 0.0) ? pow(R31, d13) : -pow(fabs(R31), d13);
  R32 = (R32 >= 0.0) ? pow(R32, d13) : -pow(fabs(R32), d13);
  double bg = R31 + R32 + w;
  double Q = 1.0 + 3.0 * (bg * bg);
  Telles t;
  t.a = (1.0 - br) / Q;
  t.b = -3.0 * bg * t.a;
  t.c = (br + 3.0 * (bg * bg)) / Q;
  t.d = -t.b;
  return t;
}
MFB_HD void telles_map(const Telles& t, double g, double& xi, double& jac) {
  xi = t.a * (g * g * g) + t.b * (g * g) + t.c * g + t.d;
  jac = 3.0 * t.a * (g * g) + 2.0 * t.b * g + t.c;
}

// ----------------------------------------------------------------------------
// Quasi-singular order estimator (quasisingular_integration.f90:318-711). The
// per-relative-error curve parameters are computed once on the host
// (QsCurves, filled by qs_curves() in host_tables.cpp) and copied to the device.
// Layout [curve 0..2][integrand 0..7].
// ----------------------------------------------------------------------------
struct QsCurves {
  double dmin[3][8], dmax[3][8], a0[3][8], a1[3][8], b1[3][8];
  double tdmin[3][8], tdmax[3][8], ta0[3][8], ta1[3][8], tb1[3][8];
};
MFB_HD double qs_curve(double a0, double a1, double b1, double l) { return pow(10.0, (a0 + a1 * l) / (1.0 + b1 * l)); }

// dim: 1 line, 2 quadrilateral; f: integrand 1/r^f; tel: Telles-mapped rule
MFB_HD int qs_estimate(const QsCurves& p, int dim, int f, double d, const double* bx, bool tel) {
  int res;
  if (d <= 2.0) {
    double l = log10(d);
    const double(*dmin)[8] = tel ? p.tdmin : p.dmin;
    const double(*dmax)[8] = tel ? p.tdmax : p.dmax;
    const double(*a0)[8] = tel ? p.ta0 : p.a0;
    const double(*a1)[8] = tel ? p.ta1 : p.a1;
    const double(*b1)[8] = tel ? p.tb1 : p.b1;
    double N1, N2;
    if (dim == 1 && !(fabs(bx[0]) < 1.0)) {
      if (d <= dmin[1][f]) return 0;
      N2 = (d >= dmax[1][f]) ? 2.0 : qs_curve(a0[1][f], a1[1][f], b1[1][f], l);
      res = (int)ceil(N2);
    } else {
      if (d <= dmin[0][f]) return 0;
      N1 = (d >= dmax[0][f]) ? 2.0 : qs_curve(a0[0][f], a1[0][f], b1[0][f], l);
      if (d <= dmin[1][f]) return 0;
      N2 = (d >= dmax[1][f]) ? 2.0 : qs_curve(a0[1][f], a1[1][f], b1[1][f], l);
      if (dim == 1) res = (int)ceil(bx[0] * bx[0] * (N2 - N1) + N1);
      else res = (int)ceil((bx[0] * bx[0]) * (bx[1] * bx[1]) * (N2 - N1) + N1);
    }
  } else {
    if (d >= p.dmax[2][f]) {
      res = 2;
    } else {
      double v = qs_curve(p.a0[2][f], p.a1[2][f], p.b1[2][f], log10(d));
      res = (int)(v < 0 ? -floor(-v + 0.5) : floor(v + 0.5));
    }
  }
  return res > 30 ? 0 : res;
}

// ----------------------------------------------------------------------------
// Nearest element point, fbem_nearest_element_point_bem (geometry.f90:5519-5566)
// with the node guess (4263-4316), the Newton-type minimisation (5107-5408,
// evaluated in double-double where the reference uses binary128) and the
// sampling fallback (4329-4441, 4574-4787).
// ----------------------------------------------------------------------------
MFB_HD bool in_quad(double x1, double x2) {
  return !(x1 < -1.0 - kXiTol || x1 > 1.0 + kXiTol || x2 < -1.0 - kXiTol || x2 > 1.0 + kXiTol);
}
MFB_HD bool on_quad_edge(double x1, double x2) {
  if (!in_quad(x1, x2)) return false;
  return x1 < -1.0 + kXiTol || x1 > 1.0 - kXiTol || x2 < -1.0 + kXiTol || x2 > 1.0 - kXiTol;
}

MFB_HD double dd_dist(const dd r[3]) { return dd_round(dd_sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2])); }

MFB_HD void nearest_l3(const double* x /*3x3*/, double cl, const double* p, double* barxi, double* rmin,
                       double* d, int* method) {
  // nodes
  const double xin[3] = {-1.0, 1.0, 0.0};
  int nn = 0;
  double rm = 0;
  for (int k = 0; k < 3; ++k) {
    double v0 = x[3 * k] - p[0], v1 = x[3 * k + 1] - p[1], v2 = x[3 * k + 2] - p[2];
    double rr = sqrt(v0 * v0 + v1 * v1 + v2 * v2);
    if (k == 0 || rr < rm) { rm = rr; nn = k; }
  }
  *barxi = xin[nn];
  *rmin = rm;
  *d = rm / cl;
  if (!(*d < 1.0)) { *method = 1; return; }
  // minimisation, geometry.f90:5211-5287
  double h[22], eh[22];
  h[1] = (*barxi < -1.0 || *barxi > 1.0) ? 0.0 : *barxi;
  int k = 1, info = 0;
  double bx = 0;
  while (info == 0) {
    dd q = dd_from(h[k]);
    dd ph[3], dp[3];
    phi_l3<dd>(q, ph);
    dphi_l3<dd>(q, dp);
    dd xb[3] = {dd_from(0), dd_from(0), dd_from(0)}, db[3] = {dd_from(0), dd_from(0), dd_from(0)};
    for (int i = 0; i < 3; ++i)
      for (int c = 0; c < 3; ++c) {
        xb[c] = xb[c] + ddmul(ph[i], x[3 * i + c]);
        db[c] = db[c] + ddmul(dp[i], x[3 * i + c]);
      }
    dd ab = dd_from(0), bb = dd_from(0);
    for (int c = 0; c < 3; ++c) {
      dd a = xb[c] - db[c] * q - dd_from(p[c]);
      ab = ab + a * db[c];
      bb = bb + db[c] * db[c];
    }
    h[k + 1] = dd_round(-(ab / bb));
    eh[k] = fabs(h[k + 1] - h[k]) * 0.5;
    if (eh[k] <= 1e-14) { bx = h[k + 1]; info = 1; }
    else if (k == 20) { bx = h[k + 1]; info = 2; }
    else if (k > 5) {
      if (eh[k] > eh[k - 2]) { bx = h[k + 1]; info = 3; }
      else ++k;
    } else ++k;
  }
  if (info == 1) {
    if (bx < -1.0 || bx > 1.0) {
      bx = -1.0;
      dd r[3];
      for (int c = 0; c < 3; ++c) r[c] = dd_from(x[c]) - dd_from(p[c]);
      double r1 = dd_dist(r);
      for (int c = 0; c < 3; ++c) r[c] = dd_from(x[3 + c]) - dd_from(p[c]);
      dd r2 = dd_sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
      if (dd_lt(r2, dd_from(r1))) bx = 1.0;
    }
    dd ph[3];
    phi_l3<dd>(dd_from(bx), ph);
    dd r[3] = {dd_from(0), dd_from(0), dd_from(0)};
    for (int i = 0; i < 3; ++i)
      for (int c = 0; c < 3; ++c) r[c] = r[c] + ddmul(ph[i], x[3 * i + c]);
    for (int c = 0; c < 3; ++c) r[c] = r[c] - dd_from(p[c]);
    *barxi = bx;
    *rmin = dd_dist(r);
    *method = 2;
  } else {
    // sampling (25, 14, 2)
    const int ns = 25, nrs = 14, nit = 2;
    double xm = 0, rr = 0;
    for (int kk = 0; kk <= ns + 1; ++kk) {
      double xi = -1.0 + 2.0 / (double)(ns + 1) * (double)kk;
      double ph[3];
      phi_l3<double>(xi, ph);
      double v[3] = {0, 0, 0};
      for (int j = 0; j < 3; ++j)
        for (int c = 0; c < 3; ++c) v[c] = v[c] + ph[j] * x[3 * j + c];
      for (int c = 0; c < 3; ++c) v[c] = v[c] - p[c];
      double r = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
      if (kk == 0 || r < rr) { xm = xi; rr = r; }
    }
    double xo = xm, width = 2.0 / (double)(ns + 1);
    for (int l = 1; l <= nit; ++l) {
      for (int kk = 1; kk <= nrs; ++kk) {
        double xi = xo - width + (2.0 * width) / (double)(nrs + 1) * (double)kk;
        if (xi > -1.0 && xi < 1.0) {
          double ph[3];
          phi_l3<double>(xi, ph);
          double v[3] = {0, 0, 0};
          for (int j = 0; j < 3; ++j)
            for (int c = 0; c < 3; ++c) v[c] = v[c] + ph[j] * x[3 * j + c];
          for (int c = 0; c < 3; ++c) v[c] = v[c] - p[c];
          double r = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
          if (r < rr) { xm = xi; rr = r; }
        }
      }
      xo = xm;
      width = 2.0 * width / (double)(nrs + 1);
    }
    *barxi = xm;
    *rmin = rr;
    *method = 3;
  }
  *d = *rmin / cl;
}

MFB_HD void nearest_q8(const double* x /*8x3*/, double cl, const double* p, double bx[2], double* rmin, double* d,
                       int* method) {
  int nn = 0;
  double rm = 0;
  for (int k = 0; k < 8; ++k) {
    double v0 = x[3 * k] - p[0], v1 = x[3 * k + 1] - p[1], v2 = x[3 * k + 2] - p[2];
    double rr = sqrt(v0 * v0 + v1 * v1 + v2 * v2);
    if (k == 0 || rr < rm) { rm = rr; nn = k; }
  }
  bx[0] = q8xi(nn, 0);
  bx[1] = q8xi(nn, 1);
  *rmin = rm;
  *d = rm / cl;
  if (!(*d < 1.0)) { *method = 1; return; }
  double h0[22], h1[22], eh[22];
  if (!in_quad(bx[0], bx[1])) { h0[1] = 0.0; h1[1] = 0.0; }
  else { h0[1] = bx[0]; h1[1] = bx[1]; }
  int k = 1, info = 0;
  while (info == 0) {
    dd q1 = dd_from(h0[k]), q2 = dd_from(h1[k]);
    dd ph[8], d1[8], d2[8];
    phi_q8<dd>(q1, q2, ph);
    dphi_q8<dd>(q1, q2, d1, d2);
    dd xb[3], b[3], c[3];
    for (int cc = 0; cc < 3; ++cc) xb[cc] = b[cc] = c[cc] = dd_from(0);
    for (int i = 0; i < 8; ++i)
      for (int cc = 0; cc < 3; ++cc) {
        xb[cc] = xb[cc] + ddmul(ph[i], x[3 * i + cc]);
        b[cc] = b[cc] + ddmul(d1[i], x[3 * i + cc]);
        c[cc] = c[cc] + ddmul(d2[i], x[3 * i + cc]);
      }
    dd bb = dd_from(0), cc_ = dd_from(0), bc = dd_from(0), ab = dd_from(0), ac = dd_from(0);
    for (int cc = 0; cc < 3; ++cc) {
      dd a = xb[cc] - b[cc] * q1 - c[cc] * q2 - dd_from(p[cc]);
      bb = bb + b[cc] * b[cc];
      cc_ = cc_ + c[cc] * c[cc];
      bc = bc + b[cc] * c[cc];
      ab = ab + a * b[cc];
      ac = ac + a * c[cc];
    }
    dd det = bb * cc_ - bc * bc;
    h0[k + 1] = dd_round(-((ab * cc_ - bc * ac) / det));
    h1[k + 1] = dd_round(-((bb * ac - ab * bc) / det));
    double e0 = h0[k + 1] - h0[k], e1 = h1[k + 1] - h1[k];
    eh[k] = sqrt(e0 * e0 + e1 * e1) * 0.5;
    if (eh[k] <= 1e-14) { bx[0] = h0[k + 1]; bx[1] = h1[k + 1]; info = 1; }
    else if (k == 20) { bx[0] = h0[k + 1]; bx[1] = h1[k + 1]; info = 2; }
    else if (k > 5) {
      if (eh[k] >= eh[k - 2]) { bx[0] = h0[k + 1]; bx[1] = h1[k + 1]; info = 3; }
      else ++k;
    } else ++k;
  }
  if (info == 1) {
    if (!in_quad(bx[0], bx[1])) {
      double rme[4], bxe[4];
      for (int ke = 0; ke < 4; ++ke) {
        double xe[9];
        for (int n = 0; n < 3; ++n)
          for (int c = 0; c < 3; ++c) xe[3 * n + c] = x[3 * q8edge(ke, n) + c];
        double cle = length_l3(xe, 1e-12);
        double de;
        int me;
        nearest_l3(xe, cle, p, &bxe[ke], &rme[ke], &de, &me);
      }
      int ke = 0;
      for (int j = 1; j < 4; ++j)
        if (rme[j] < rme[ke]) ke = j;
      dd ph[3];
      phi_l3<dd>(dd_from(bxe[ke]), ph);
      double b0 = 0.0, b1 = 0.0;
      for (int n = 0; n < 3; ++n) {
        int nd = q8edge(ke, n);
        b0 = dd_round(dd_from(b0) + ddmul(ph[n], q8xi(nd, 0)));
        b1 = dd_round(dd_from(b1) + ddmul(ph[n], q8xi(nd, 1)));
      }
      bx[0] = b0;
      bx[1] = b1;
    }
    dd ph[8];
    phi_q8<dd>(dd_from(bx[0]), dd_from(bx[1]), ph);
    dd r[3] = {dd_from(0), dd_from(0), dd_from(0)};
    for (int i = 0; i < 8; ++i)
      for (int c = 0; c < 3; ++c) r[c] = r[c] + ddmul(ph[i], x[3 * i + c]);
    for (int c = 0; c < 3; ++c) r[c] = r[c] - dd_from(p[c]);
    *rmin = dd_dist(r);
    *method = 2;
  } else {
    const int ns = 25, nrs = 14, nit = 2;
    double xm0 = 0, xm1 = 0, rr = 0;
    for (int k1 = 0; k1 <= ns + 1; ++k1) {
      double x1 = -1.0 + 2.0 * (double)k1 / (double)(ns + 1);
      for (int k2 = 0; k2 <= ns + 1; ++k2) {
        double x2 = -1.0 + 2.0 * (double)k2 / (double)(ns + 1);
        double ph[8];
        phi_q8<double>(x1, x2, ph);
        double v[3] = {0, 0, 0};
        for (int j = 0; j < 8; ++j)
          for (int c = 0; c < 3; ++c) v[c] = v[c] + ph[j] * x[3 * j + c];
        for (int c = 0; c < 3; ++c) v[c] = v[c] - p[c];
        double r = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        if ((k1 == 0 && k2 == 0) || r < rr) { xm0 = x1; xm1 = x2; rr = r; }
      }
    }
    double xo0 = xm0, xo1 = xm1, width = 2.0 / (double)(ns + 1);
    for (int l = 1; l <= nit; ++l) {
      for (int k1 = 1; k1 <= nrs; ++k1) {
        double x1 = xo0 + 2.0 * ((double)k1 - (double)(nrs + 1) / 2.0) / (double)(nrs + 1) * width;
        if (x1 > -1.0 && x1 < 1.0) {
          for (int k2 = 1; k2 <= nrs; ++k2) {
            double x2 = xo1 + 2.0 * ((double)k2 - (double)(nrs + 1) / 2.0) / (double)(nrs + 1) * width;
            if (x2 > -1.0 && x2 < 1.0) {
              double ph[8];
              phi_q8<double>(x1, x2, ph);
              double v[3] = {0, 0, 0};
              for (int j = 0; j < 8; ++j)
                for (int c = 0; c < 3; ++c) v[c] = v[c] + ph[j] * x[3 * j + c];
              for (int c = 0; c < 3; ++c) v[c] = v[c] - p[c];
              double r = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
              if (r < rr) { xm0 = x1; xm1 = x2; rr = r; }
            }
          }
        }
      }
      xo0 = xm0;
      xo1 = xm1;
      width = width / (double)(nrs + 1);
      width = 2.0 * width / (double)(nrs + 1);
    }
    bx[0] = xm0;
    bx[1] = xm1;
    *rmin = rr;
    *method = 3;
  }
  *d = *rmin / cl;
}

// fbem_obtain_element_subdivision_coordinates (geometry.f90:2591-2697)
MFB_HD void subdiv_q8(const double* x, const double* xs /*4x2*/, double* out /*8x3*/) {
  for (int k = 0; k < 8; ++k) {
    double s[4];
    phi_q4(q8xi(k, 0), q8xi(k, 1), s);
    double a = 0, b = 0;
    for (int i = 0; i < 4; ++i) {
      a = a + s[i] * xs[2 * i];
      b = b + s[i] * xs[2 * i + 1];
    }
    double ph[8];
    phi_q8<double>(a, b, ph);
    for (int c = 0; c < 3; ++c) out[3 * k + c] = 0.0;
    for (int i = 0; i < 8; ++i)
      for (int c = 0; c < 3; ++c) out[3 * k + c] = out[3 * k + c] + ph[i] * x[3 * i + c];
  }
}
MFB_HD void subdiv_l3(const double* x, double s0, double s1, double* out /*3x3*/) {
  const double xin[3] = {-1.0, 1.0, 0.0};
  for (int k = 0; k < 3; ++k) {
    double a = 0.5 * xin[k];
    double xi = 0.0;
    xi = xi + (0.5 - a) * s0;
    xi = xi + (0.5 + a) * s1;
    double ph[3];
    phi_l3<double>(xi, ph);
    for (int c = 0; c < 3; ++c) out[3 * k + c] = 0.0;
    for (int i = 0; i < 3; ++i)
      for (int c = 0; c < 3; ++c) out[3 * k + c] = out[3 * k + c] + ph[i] * x[3 * i + c];
  }
}

}  // namespace mfb
