// Oracle (test infrastructure only): element geometry helpers - characteristic
// length, bounding ball, nearest element point (nodes / binary128 minimisation /
// sampling), subdivision coordinates and the polar transformation.
#include "orc.h"
#include <cmath>

namespace orc {

static inline quad qsqrt(quad v) {
  if (v <= 0) return 0;
  quad s = (quad)std::sqrt((double)v);
  s = (s + v / s) / (quad)2;
  s = (s + v / s) / (quad)2;
  return s;
}

// ---------------------------------------------------------------------------
// fbem_jacobian3d_1d (geometry.f90:1469-1504) and fbem_length3d with rule=0
// (adaptive tolerance mode, geometry.f90:2794-2882)
// ---------------------------------------------------------------------------
static double jacobian3d_line3(const double x[3][3], double xi) {
  double d[3];
  dphi_line3(xi, d);
  double t[3] = {0, 0, 0};
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) t[j] = t[j] + d[i] * x[i][j];
  return std::sqrt(t[0] * t[0] + t[1] * t[1] + t[2] * t[2]);
}

double length3d_line3(const double x[3][3], double tol) {
  double ltol = (tol <= 0.0) ? 1e-6 : tol;
  const int step = 3, nr = 32;
  double err = ltol + 1.0;
  double length = jacobian3d_line3(x, gl11_xi(1, 1)) * gl11_w(1, 1);
  int j = 1 + step;
  while (err >= ltol) {
    double old = length;
    length = 0.0;
    for (int i = 1; i <= j; ++i) length = length + jacobian3d_line3(x, gl11_xi(i, j)) * gl11_w(i, j);
    err = std::fabs((old - length) / length);
    j = j + step;
    if (j >= nr) {
      length = 0.0;
      for (int i = 1; i <= nr - 1; ++i)
        length = length + jacobian3d_line3(x, gl11_xi(i, nr - 1)) * gl11_w(i, nr - 1);
      old = length;
      length = 0.0;
      for (int i = 1; i <= nr; ++i) length = length + jacobian3d_line3(x, gl11_xi(i, nr)) * gl11_w(i, nr);
      break;
    }
  }
  return length;
}

// fbem_characteristic_length (geometry.f90:3357-3389): longest edge length
double characteristic_length_quad8(const double x[8][3], double tol) {
  double lmax = 0.0;
  for (int e = 0; e < 4; ++e) {
    double xe[3][3];
    for (int n = 0; n < 3; ++n)
      for (int c = 0; c < 3; ++c) xe[n][c] = x[quad8_edge_node[e][n]][c];
    double l = length3d_line3(xe, tol);
    if (e == 0 || l > lmax) lmax = l;
  }
  return lmax;
}
double characteristic_length_line3(const double x[3][3], double tol) { return length3d_line3(x, tol); }

// fbem_geometry_element_ball (geometry.f90:3904-4235), quadrilateral branch
void element_ball_quad8(const double x[8][3], int glp, double centre[3], double* radius) {
  double esize = 0.0, xm[3] = {0, 0, 0};
  for (int k1 = 1; k1 <= glp; ++k1)
    for (int k2 = 1; k2 <= glp; ++k2) {
      double xi[2] = {gl11_xi(k1, glp), gl11_xi(k2, glp)};
      double w1 = gl11_w(k1, glp), w2 = gl11_w(k2, glp);
      double phi[8], d1[8], d2[8];
      phi_quad8(xi, phi);
      dphi_quad8(xi, d1, d2);
      double xp[3] = {0, 0, 0}, T1[3] = {0, 0, 0}, T2[3] = {0, 0, 0};
      for (int k = 0; k < 8; ++k)
        for (int c = 0; c < 3; ++c) {
          xp[c] = xp[c] + phi[k] * x[k][c];
          T1[c] = T1[c] + d1[k] * x[k][c];
          T2[c] = T2[c] + d2[k] * x[k][c];
        }
      double N[3] = {T1[1] * T2[2] - T1[2] * T2[1], T1[2] * T2[0] - T1[0] * T2[2],
                     T1[0] * T2[1] - T1[1] * T2[0]};
      double jg = std::sqrt(N[0] * N[0] + N[1] * N[1] + N[2] * N[2]);
      double jw = jg * w1 * w2;
      esize = esize + jw;
      for (int c = 0; c < 3; ++c) xm[c] = xm[c] + xp[c] * jw;
    }
  for (int c = 0; c < 3; ++c) centre[c] = xm[c] / esize;
  double r = 0.0;
  for (int k = 0; k < 8; ++k) {
    double v[3] = {x[k][0] - centre[0], x[k][1] - centre[1], x[k][2] - centre[2]};
    double t = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    if (r < t) r = t;
  }
  for (int k1 = 1; k1 <= glp; ++k1)
    for (int k2 = 1; k2 <= glp; ++k2) {
      double xi[2] = {gl11_xi(k1, glp), gl11_xi(k2, glp)};
      double phi[8];
      phi_quad8(xi, phi);
      double xp[3] = {0, 0, 0};
      for (int k = 0; k < 8; ++k)
        for (int c = 0; c < 3; ++c) xp[c] = xp[c] + phi[k] * x[k][c];
      double v[3] = {xp[0] - centre[0], xp[1] - centre[1], xp[2] - centre[2]};
      double t = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
      if (r < t) r = t;
    }
  *radius = r;
}

// ---------------------------------------------------------------------------
// Nearest element point
// ---------------------------------------------------------------------------
static bool check_xi(double xi) { return !(xi < -1.0 - check_xi_tolerance || xi > 1.0 + check_xi_tolerance); }
static bool check_xi1xi2_quad(const double xi[2]) {
  return !(xi[0] < -1.0 - check_xi_tolerance || xi[0] > 1.0 + check_xi_tolerance ||
           xi[1] < -1.0 - check_xi_tolerance || xi[1] > 1.0 + check_xi_tolerance);
}
// shape_functions.f90:1111-1146
bool check_xi1xi2_edge_quad(const double xi[2]) {
  if (!check_xi1xi2_quad(xi)) return false;
  return (xi[0] < -1.0 + check_xi_tolerance || xi[0] > 1.0 - check_xi_tolerance ||
          xi[1] < -1.0 + check_xi_tolerance || xi[1] > 1.0 - check_xi_tolerance);
}

// fbem_nearest_xi_nodes (geometry.f90:4263-4316)
static void nearest_xi_nodes_quad8(const double x[8][3], const double p[3], double xi[2], double* r) {
  int nn = 0;
  double rm = 0;
  for (int k = 0; k < 8; ++k) {
    double v[3] = {x[k][0] - p[0], x[k][1] - p[1], x[k][2] - p[2]};
    double rr = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    if (k == 0 || rr < rm) { rm = rr; nn = k; }
  }
  xi[0] = quad8_xi_nodes[nn][0];
  xi[1] = quad8_xi_nodes[nn][1];
  *r = rm;
}
static void nearest_xi_nodes_line3(const double x[3][3], const double p[3], double* xi, double* r) {
  static const double xin[3] = {-1.0, 1.0, 0.0};
  int nn = 0;
  double rm = 0;
  for (int k = 0; k < 3; ++k) {
    double v[3] = {x[k][0] - p[0], x[k][1] - p[1], x[k][2] - p[2]};
    double rr = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    if (k == 0 || rr < rm) { rm = rr; nn = k; }
  }
  *xi = xin[nn];
  *r = rm;
}

// nearest_minimization_iteration_1d (geometry.f90:5072-5105), binary128
static double min_iter_1d(const double x[3][3], const double xi_[3], double barxi) {
  quad phi[3], dphi[3];
  phi_line3_q((quad)barxi, phi);
  dphi_line3_q((quad)barxi, dphi);
  quad xb[3] = {0, 0, 0}, db[3] = {0, 0, 0};
  for (int k = 0; k < 3; ++k)
    for (int c = 0; c < 3; ++c) {
      xb[c] = xb[c] + phi[k] * (quad)x[k][c];
      db[c] = db[c] + dphi[k] * (quad)x[k][c];
    }
  quad a[3], ab = 0, bb = 0;
  for (int c = 0; c < 3; ++c) a[c] = xb[c] - db[c] * (quad)barxi - (quad)xi_[c];
  for (int c = 0; c < 3; ++c) { ab += a[c] * db[c]; bb += db[c] * db[c]; }
  return (double)(-ab / bb);
}

// nearest_minimization_iteration_2d (geometry.f90:5107-5150), binary128
static void min_iter_2d(const double x[8][3], const double xi_[3], const double bx[2], double nb[2]) {
  quad q[2] = {(quad)bx[0], (quad)bx[1]};
  quad phi[8], d1[8], d2[8];
  phi_quad8_q(q, phi);
  dphi_quad8_q(q, d1, d2);
  quad xb[3] = {0, 0, 0}, b[3] = {0, 0, 0}, c[3] = {0, 0, 0};
  for (int i = 0; i < 8; ++i)
    for (int k = 0; k < 3; ++k) {
      xb[k] = xb[k] + phi[i] * (quad)x[i][k];
      b[k] = b[k] + d1[i] * (quad)x[i][k];
      c[k] = c[k] + d2[i] * (quad)x[i][k];
    }
  quad a[3];
  for (int k = 0; k < 3; ++k) a[k] = xb[k] - b[k] * q[0] - c[k] * q[1] - (quad)xi_[k];
  quad bb = 0, cc = 0, bc = 0, ab = 0, ac = 0;
  for (int k = 0; k < 3; ++k) {
    bb += b[k] * b[k];
    cc += c[k] * c[k];
    bc += b[k] * c[k];
    ab += a[k] * b[k];
    ac += a[k] * c[k];
  }
  quad det = bb * cc - bc * bc;
  nb[0] = (double)(-(ab * cc - bc * ac) / det);
  nb[1] = (double)(-(bb * ac - ab * bc) / det);
}

// fbem_nearest_minimization_1d (geometry.f90:5211-5287)
static void nearest_min_1d(const double x[3][3], const double xi_[3], double error, int nmax, double* barxi,
                           double* rmin, int* info) {
  double hist[64], eh[64];
  hist[1] = (*barxi < -1.0 || *barxi > 1.0) ? 0.0 : *barxi;
  int k = 1;
  *info = 0;
  while (*info == 0) {
    hist[k + 1] = min_iter_1d(x, xi_, hist[k]);
    eh[k] = std::fabs(hist[k + 1] - hist[k]) * 0.5;
    if (eh[k] <= error) {
      *barxi = hist[k + 1];
      *info = 1;
    } else if (k == nmax) {
      *barxi = hist[k + 1];
      *info = 2;
    } else if (k > 5) {
      if (eh[k] > eh[k - 2]) { *barxi = hist[k + 1]; *info = 3; }
      else k = k + 1;
    } else {
      k = k + 1;
    }
  }
  if (*info == 1) {
    if (*barxi < -1.0 || *barxi > 1.0) {
      *barxi = -1.0;
      quad r[3];
      for (int c = 0; c < 3; ++c) r[c] = (quad)x[0][c] - (quad)xi_[c];
      *rmin = (double)qsqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
      for (int c = 0; c < 3; ++c) r[c] = (quad)x[1][c] - (quad)xi_[c];
      if (qsqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]) < (quad)(*rmin)) *barxi = 1.0;
    }
    quad phi[3];
    phi_line3_q((quad)(*barxi), phi);
    quad r[3] = {0, 0, 0};
    for (int kk = 0; kk < 3; ++kk)
      for (int c = 0; c < 3; ++c) r[c] = r[c] + phi[kk] * (quad)x[kk][c];
    for (int c = 0; c < 3; ++c) r[c] = r[c] - (quad)xi_[c];
    *rmin = (double)qsqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
  }
}

// fbem_nearest_xi (geometry.f90:4329-4441), 1D sampling
static void nearest_xi_sampling_line3(const double x[3][3], const double p[3], int ns, int nrs, int nit, double* xi_out,
                                      double* r_out) {
  double ximin = 0, rmin = 0;
  for (int k = 0; k <= ns + 1; ++k) {
    double xi = -1.0 + 2.0 / (double)(ns + 1) * (double)k;
    double phi[3];
    phi_line3(xi, phi);
    double xp[3] = {0, 0, 0};
    for (int j = 0; j < 3; ++j)
      for (int c = 0; c < 3; ++c) xp[c] = xp[c] + phi[j] * x[j][c];
    double v[3] = {xp[0] - p[0], xp[1] - p[1], xp[2] - p[2]};
    double r = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    if (k == 0) { ximin = xi; rmin = r; }
    if (r < rmin) { ximin = xi; rmin = r; }
  }
  double xold = ximin;
  double width = 2.0 / (double)(ns + 1);
  for (int l = 1; l <= nit; ++l) {
    for (int k = 1; k <= nrs; ++k) {
      double xi = xold - width + (2.0 * width) / (double)(nrs + 1) * (double)k;
      if (xi > -1.0 && xi < 1.0) {
        double phi[3];
        phi_line3(xi, phi);
        double xp[3] = {0, 0, 0};
        for (int j = 0; j < 3; ++j)
          for (int c = 0; c < 3; ++c) xp[c] = xp[c] + phi[j] * x[j][c];
        double v[3] = {xp[0] - p[0], xp[1] - p[1], xp[2] - p[2]};
        double r = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        if (r < rmin) { ximin = xi; rmin = r; }
      }
    }
    xold = ximin;
    width = 2.0 * width / (double)(nrs + 1);
  }
  *xi_out = ximin;
  *r_out = rmin;
}

// fbem_nearest_xi1xi2 (geometry.f90:4574-4787), quadrilateral branch
static void nearest_xi_sampling_quad8(const double x[8][3], const double p[3], int ns, int nrs, int nit,
                                      double xi_out[2], double* r_out) {
  double xm[2] = {0, 0}, rm = 0;
  for (int k1 = 0; k1 <= ns + 1; ++k1) {
    double xi[2];
    xi[0] = -1.0 + 2.0 * (double)k1 / (double)(ns + 1);
    for (int k2 = 0; k2 <= ns + 1; ++k2) {
      xi[1] = -1.0 + 2.0 * (double)k2 / (double)(ns + 1);
      double phi[8];
      phi_quad8(xi, phi);
      double xp[3] = {0, 0, 0};
      for (int j = 0; j < 8; ++j)
        for (int c = 0; c < 3; ++c) xp[c] = xp[c] + phi[j] * x[j][c];
      double v[3] = {xp[0] - p[0], xp[1] - p[1], xp[2] - p[2]};
      double r = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
      if (k1 == 0 && k2 == 0) { xm[0] = xi[0]; xm[1] = xi[1]; rm = r; }
      if (r < rm) { xm[0] = xi[0]; xm[1] = xi[1]; rm = r; }
    }
  }
  double xo[2] = {xm[0], xm[1]};
  double width = 2.0 / (double)(ns + 1);
  for (int l = 1; l <= nit; ++l) {
    for (int k1 = 1; k1 <= nrs; ++k1) {
      double xi[2];
      xi[0] = xo[0] + 2.0 * ((double)k1 - (double)(nrs + 1) / 2.0) / (double)(nrs + 1) * width;
      if (xi[0] > -1.0 && xi[0] < 1.0) {
        for (int k2 = 1; k2 <= nrs; ++k2) {
          xi[1] = xo[1] + 2.0 * ((double)k2 - (double)(nrs + 1) / 2.0) / (double)(nrs + 1) * width;
          if (xi[1] > -1.0 && xi[1] < 1.0) {
            double phi[8];
            phi_quad8(xi, phi);
            double xp[3] = {0, 0, 0};
            for (int j = 0; j < 8; ++j)
              for (int c = 0; c < 3; ++c) xp[c] = xp[c] + phi[j] * x[j][c];
            double v[3] = {xp[0] - p[0], xp[1] - p[1], xp[2] - p[2]};
            double r = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
            if (r < rm) { xm[0] = xi[0]; xm[1] = xi[1]; rm = r; }
          }
        }
      }
    }
    xo[0] = xm[0];
    xo[1] = xm[1];
    width = width / (double)(nrs + 1);
    width = 2.0 * width / (double)(nrs + 1);
  }
  xi_out[0] = xm[0];
  xi_out[1] = xm[1];
  *r_out = rm;
}

// fbem_nearest_element_point_bem (geometry.f90:5519-5566), line3
void nearest_element_point_line3(const double x[3][3], double cl, const double xi_[3], double* barxi,
                                 double* rmin, double* d, int* method) {
  nearest_xi_nodes_line3(x, xi_, barxi, rmin);
  *d = *rmin / cl;
  if (*d < 1.0) {
    int info;
    nearest_min_1d(x, xi_, 1e-14, 20, barxi, rmin, &info);
    if (info != 1) {
      nearest_xi_sampling_line3(x, xi_, 25, 14, 2, barxi, rmin);
      *method = 3;
    } else {
      *method = 2;
    }
    *d = *rmin / cl;
  } else {
    *method = 1;
  }
}

// fbem_nearest_minimization_2d (geometry.f90:5289-5408)
static void nearest_min_2d(const double x[8][3], const double xi_[3], double error, int nmax, double barxi[2],
                           double* rmin, int* info) {
  double hist[64][2], eh[64];
  if (!check_xi1xi2_quad(barxi)) { hist[1][0] = 0.0; hist[1][1] = 0.0; }
  else { hist[1][0] = barxi[0]; hist[1][1] = barxi[1]; }
  int k = 1;
  *info = 0;
  while (*info == 0) {
    min_iter_2d(x, xi_, hist[k], hist[k + 1]);
    double a = hist[k + 1][0] - hist[k][0], b = hist[k + 1][1] - hist[k][1];
    eh[k] = std::sqrt(a * a + b * b) * 0.5;
    if (eh[k] <= error) {
      barxi[0] = hist[k + 1][0]; barxi[1] = hist[k + 1][1];
      *info = 1;
    } else if (k == nmax) {
      barxi[0] = hist[k + 1][0]; barxi[1] = hist[k + 1][1];
      *info = 2;
    } else if (k > 5) {
      if (eh[k] >= eh[k - 2]) { barxi[0] = hist[k + 1][0]; barxi[1] = hist[k + 1][1]; *info = 3; }
      else k = k + 1;
    } else {
      k = k + 1;
    }
  }
  if (*info == 1) {
    if (!check_xi1xi2_quad(barxi)) {
      double rme[4], bxe[4];
      for (int ke = 0; ke < 4; ++ke) {
        double xe[3][3];
        for (int n = 0; n < 3; ++n)
          for (int c = 0; c < 3; ++c) xe[n][c] = x[quad8_edge_node[ke][n]][c];
        double cl = characteristic_length_line3(xe, 1e-12);
        double dd;
        int m;
        nearest_element_point_line3(xe, cl, xi_, &bxe[ke], &rme[ke], &dd, &m);
      }
      int ke = 0;
      for (int j = 1; j < 4; ++j)
        if (rme[j] < rme[ke]) ke = j;
      quad phi[3];
      phi_line3_q((quad)bxe[ke], phi);
      barxi[0] = 0.0;
      barxi[1] = 0.0;
      for (int n = 0; n < 3; ++n) {
        const double* xn = quad8_xi_nodes[quad8_edge_node[ke][n]];
        barxi[0] = (double)((quad)barxi[0] + phi[n] * (quad)xn[0]);
        barxi[1] = (double)((quad)barxi[1] + phi[n] * (quad)xn[1]);
      }
    }
    quad q[2] = {(quad)barxi[0], (quad)barxi[1]};
    quad phi[8];
    phi_quad8_q(q, phi);
    quad r[3] = {0, 0, 0};
    for (int kk = 0; kk < 8; ++kk)
      for (int c = 0; c < 3; ++c) r[c] = r[c] + phi[kk] * (quad)x[kk][c];
    for (int c = 0; c < 3; ++c) r[c] = r[c] - (quad)xi_[c];
    *rmin = (double)qsqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
  }
}

// fbem_nearest_element_point_bem (geometry.f90:5519-5566), quad8
void nearest_element_point_quad8(const double x[8][3], double cl, const double xi_[3], double barxi[2],
                                 double* rmin, double* d, int* method) {
  nearest_xi_nodes_quad8(x, xi_, barxi, rmin);
  *d = *rmin / cl;
  if (*d < 1.0) {
    int info;
    nearest_min_2d(x, xi_, 1e-14, 20, barxi, rmin, &info);
    if (info != 1) {
      nearest_xi_sampling_quad8(x, xi_, 25, 14, 2, barxi, rmin);
      *method = 3;
    } else {
      *method = 2;
    }
    *d = *rmin / cl;
  } else {
    *method = 1;
  }
}

// fbem_obtain_element_subdivision_coordinates (geometry.f90:2591-2697)
void subdivision_coords_quad8(const double x[8][3], const double xi_s[4][2], double x_s[8][3]) {
  for (int k = 0; k < 8; ++k) {
    double phis[4];
    phi_quad4(quad8_xi_nodes[k], phis);
    double xi[2] = {0, 0};
    for (int i = 0; i < 4; ++i) {
      xi[0] = xi[0] + phis[i] * xi_s[i][0];
      xi[1] = xi[1] + phis[i] * xi_s[i][1];
    }
    double phi[8];
    phi_quad8(xi, phi);
    for (int c = 0; c < 3; ++c) x_s[k][c] = 0.0;
    for (int i = 0; i < 8; ++i)
      for (int c = 0; c < 3; ++c) x_s[k][c] = x_s[k][c] + phi[i] * x[i][c];
  }
}
void subdivision_coords_line3(const double x[3][3], const double xi_s[2], double x_s[3][3]) {
  static const double xin[3] = {-1.0, 1.0, 0.0};
  for (int k = 0; k < 3; ++k) {
    double a = 0.5 * xin[k];
    double phis[2] = {0.5 - a, 0.5 + a};
    double xi = 0.0;
    for (int i = 0; i < 2; ++i) xi = xi + phis[i] * xi_s[i];
    double phi[3];
    phi_line3(xi, phi);
    for (int c = 0; c < 3; ++c) x_s[k][c] = 0.0;
    for (int i = 0; i < 3; ++i)
      for (int c = 0; c < 3; ++c) x_s[k][c] = x_s[k][c] + phi[i] * x[i][c];
  }
}

// ---------------------------------------------------------------------------
// Polar transformation, polar_transformation.f90:251-546 (quadrilaterals)
// ---------------------------------------------------------------------------
void polar_setup_quad(const double xi_i[2], int* nsubtri, int st[8], double th[8][2], double thp[8][2]) {
  const double t = check_xi_tolerance;
  int n = 0;
  if (!check_xi1xi2_edge_quad(xi_i)) {
    n = 8;
    for (int k = 0; k < 8; ++k) st[k] = k + 1;
  } else {
    if (xi_i[0] <= -1.0 + t && xi_i[1] <= -1.0 + t) { n = 2; st[0] = 4; st[1] = 5; }
    if (xi_i[0] >= 1.0 - t && xi_i[1] <= -1.0 + t) { n = 2; st[0] = 6; st[1] = 7; }
    if (xi_i[0] >= 1.0 - t && xi_i[1] >= 1.0 - t) { n = 2; st[0] = 8; st[1] = 1; }
    if (xi_i[0] <= -1.0 + t && xi_i[1] >= 1.0 - t) { n = 2; st[0] = 2; st[1] = 3; }
    if (n == 0) {
      if (xi_i[1] <= -1.0 + t) { n = 4; st[0] = 4; st[1] = 5; st[2] = 6; st[3] = 7; }
      if (xi_i[0] >= 1.0 - t) { n = 4; st[0] = 6; st[1] = 7; st[2] = 8; st[3] = 1; }
      if (xi_i[1] >= 1.0 - t) { n = 4; st[0] = 8; st[1] = 1; st[2] = 2; st[3] = 3; }
      if (xi_i[0] <= -1.0 + t) { n = 4; st[0] = 2; st[1] = 3; st[2] = 4; st[3] = 5; }
    }
  }
  *nsubtri = n;
  const double x1 = xi_i[0], x2 = xi_i[1];
  for (int k = 0; k < n; ++k) {
    double a, b;
    switch (st[k]) {
      case 1: {
        double t1 = c_pi - std::asin((-1.0 - x2) / std::sqrt((-1.0 - x1) * (-1.0 - x1) + (-1.0 - x2) * (-1.0 - x2)));
        a = t1; b = 1.5 * c_pi;
        th[k][0] = a; th[k][1] = b;
        thp[k][0] = (1.0 + x2) * std::log(std::tan(0.5 * (a - c_pi)));
        thp[k][1] = (1.0 + x2) * std::log(std::tan(0.5 * (b - c_pi)));
        break;
      }
      case 2: {
        double t2 = c_2pi + std::asin((-1.0 - x2) / std::sqrt((1.0 - x1) * (1.0 - x1) + (-1.0 - x2) * (-1.0 - x2)));
        a = 1.5 * c_pi; b = t2;
        th[k][0] = a; th[k][1] = b;
        thp[k][0] = (1.0 + x2) * std::log(std::tan(0.5 * (a - c_pi)));
        thp[k][1] = (1.0 + x2) * std::log(std::tan(0.5 * (b - c_pi)));
        break;
      }
      case 3: {
        double t2 = c_2pi + std::asin((-1.0 - x2) / std::sqrt((1.0 - x1) * (1.0 - x1) + (-1.0 - x2) * (-1.0 - x2)));
        a = t2; b = c_2pi;
        th[k][0] = a; th[k][1] = b;
        thp[k][0] = (1.0 - x1) * std::log(std::tan(0.5 * (a + c_pi_2)));
        thp[k][1] = (1.0 - x1) * std::log(std::tan(0.5 * (b + c_pi_2)));
        break;
      }
      case 4: {
        double t3 = std::asin((1.0 - x2) / std::sqrt((1.0 - x1) * (1.0 - x1) + (1.0 - x2) * (1.0 - x2)));
        a = 0.0; b = t3;
        th[k][0] = a; th[k][1] = b;
        thp[k][0] = (1.0 - x1) * std::log(std::tan(0.5 * (a + c_pi_2)));
        thp[k][1] = (1.0 - x1) * std::log(std::tan(0.5 * (b + c_pi_2)));
        break;
      }
      case 5: {
        double t3 = std::asin((1.0 - x2) / std::sqrt((1.0 - x1) * (1.0 - x1) + (1.0 - x2) * (1.0 - x2)));
        a = t3; b = c_pi_2;
        th[k][0] = a; th[k][1] = b;
        thp[k][0] = (1.0 - x2) * std::log(std::tan(0.5 * a));
        thp[k][1] = (1.0 - x2) * std::log(std::tan(0.5 * b));
        break;
      }
      case 6: {
        double t4 = c_pi - std::asin((1.0 - x2) / std::sqrt((-1.0 - x1) * (-1.0 - x1) + (1.0 - x2) * (1.0 - x2)));
        a = c_pi_2; b = t4;
        th[k][0] = a; th[k][1] = b;
        thp[k][0] = (1.0 - x2) * std::log(std::tan(0.5 * a));
        thp[k][1] = (1.0 - x2) * std::log(std::tan(0.5 * b));
        break;
      }
      case 7: {
        double t4 = c_pi - std::asin((1.0 - x2) / std::sqrt((-1.0 - x1) * (-1.0 - x1) + (1.0 - x2) * (1.0 - x2)));
        a = t4; b = c_pi;
        th[k][0] = a; th[k][1] = b;
        thp[k][0] = (1.0 + x1) * std::log(std::tan(0.5 * (a - c_pi_2)));
        thp[k][1] = (1.0 + x1) * std::log(std::tan(0.5 * (b - c_pi_2)));
        break;
      }
      default: {  // 8
        double t1 = c_pi - std::asin((-1.0 - x2) / std::sqrt((-1.0 - x1) * (-1.0 - x1) + (-1.0 - x2) * (-1.0 - x2)));
        a = c_pi; b = t1;
        th[k][0] = a; th[k][1] = b;
        thp[k][0] = (1.0 + x1) * std::log(std::tan(0.5 * (a - c_pi_2)));
        thp[k][1] = (1.0 + x1) * std::log(std::tan(0.5 * (b - c_pi_2)));
        break;
      }
    }
  }
}

void polar_angular_quad(const double xi_i[2], int s, double thetap, double* theta, double* rhoij) {
  switch (s) {
    case 1: case 2:
      *theta = 2.0 * std::atan(std::exp(thetap / (1.0 + xi_i[1]))) + c_pi;
      *rhoij = (-1.0 - xi_i[1]) / std::sin(*theta);
      break;
    case 3: case 4:
      *theta = 2.0 * std::atan(std::exp(thetap / (1.0 - xi_i[0]))) - c_pi_2;
      *rhoij = (1.0 - xi_i[0]) / std::cos(*theta);
      break;
    case 5: case 6:
      *theta = 2.0 * std::atan(std::exp(thetap / (1.0 - xi_i[1])));
      *rhoij = (1.0 - xi_i[1]) / std::sin(*theta);
      break;
    default:
      *theta = 2.0 * std::atan(std::exp(thetap / (1.0 + xi_i[0]))) + c_pi_2;
      *rhoij = (-1.0 - xi_i[0]) / std::cos(*theta);
      break;
  }
}

}  // namespace orc
