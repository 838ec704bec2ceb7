// Oracle (test infrastructure only): staela / harela SBIE element integration,
// free terms, the region builders' collocation loops and the equation scatter,
// plus the C entry points the Python tests load with ctypes.
#include "orc.h"
#include <cmath>
#include <cstring>
#include <map>
#include <algorithm>
#include <type_traits>
#include <omp.h>

namespace orc {

// ---------------------------------------------------------------------------
// Element prepared for integration: fbem_bem_element subset
// (lib/fbem/src/bem_general.f90:51-107) for continuous quad8 elements, with the
// precalculated datasets of init_precalculated_datasets (bem_general.f90:163-759).
// phi^p == phi^s here (same quad8 functional interpolation, delta=0).
// ---------------------------------------------------------------------------
struct Elem {
  double x[8][3];
  double cl;
  int gln_far;
  double bc[3], br;
  int n_ps;
  int ps_gln[16], ps_ngp[16], ps_off[16];
  int ps_gln_max;
  std::vector<double> px, pn, pphijw;  // [off+kip][3], [3], [8]
};

static void init_precalculated(Elem& e, int n_ps, const int* ps_gln) {
  e.n_ps = n_ps;
  int off = 0;
  e.ps_gln_max = 0;
  for (int i = 0; i < n_ps; ++i) {
    e.ps_gln[i] = ps_gln[i];
    e.ps_ngp[i] = ps_gln[i] * ps_gln[i];
    e.ps_off[i] = off;
    off += e.ps_ngp[i];
    if (ps_gln[i] > e.ps_gln_max) e.ps_gln_max = ps_gln[i];
  }
  e.px.assign(off * 3, 0.0);
  e.pn.assign(off * 3, 0.0);
  e.pphijw.assign(off * 8, 0.0);
  for (int i = 0; i < n_ps; ++i) {
    int g = e.ps_gln[i];
    for (int k1 = 1; k1 <= g; ++k1)
      for (int k2 = 1; k2 <= g; ++k2) {
        int kt = e.ps_off[i] + (k2 - 1) + (k1 - 1) * g;
        double xi[2] = {gl11_xi(k1, g), gl11_xi(k2, g)};
        double w1 = gl11_w(k1, g), w2 = gl11_w(k2, g);
        double phi[8], d1[8], d2[8];
        phi_quad8(xi, phi);
        dphi_quad8(xi, d1, d2);
        double xp[3] = {0, 0, 0}, T1[3] = {0, 0, 0}, T2[3] = {0, 0, 0};
        for (int k = 0; k < 8; ++k)
          for (int c = 0; c < 3; ++c) {
            xp[c] = xp[c] + phi[k] * e.x[k][c];
            T1[c] = T1[c] + d1[k] * e.x[k][c];
            T2[c] = T2[c] + d2[k] * e.x[k][c];
          }
        double N[3] = {T1[1] * T2[2] - T1[2] * T2[1], T1[2] * T2[0] - T1[0] * T2[2],
                       T1[0] * T2[1] - T1[1] * T2[0]};
        double j = std::sqrt(N[0] * N[0] + N[1] * N[1] + N[2] * N[2]);
        for (int c = 0; c < 3; ++c) {
          e.px[kt * 3 + c] = xp[c];
          e.pn[kt * 3 + c] = N[c] / j;
        }
        for (int k = 0; k < 8; ++k) e.pphijw[kt * 8 + k] = phi[k] * j * w1 * w2;
      }
  }
}

// ---------------------------------------------------------------------------
// Harmonic parameters: fbem_bem_harela3d_calculate_parameters
// (bem_harela3d.f90:143-287), u*/t* coefficient subset.
// ---------------------------------------------------------------------------
struct HarPar {
  cplx k1, k2, c1, c2;
  cplx psi[6], chi[6], T1[10], T2[9], T3[9];
  cplx cte_u, cte_t;
  // d* / s* (HBIE) coefficients
  cplx S1[11], S2[11], S3[12], S4[10], S5[11];
  cplx cte_d, cte_s;
};
static HarPar harela_parameters(cplx lambda, cplx mu, double rho, double omega) {
  HarPar p;
  const cplx I(0.0, 1.0);
  cplx c1 = std::sqrt((lambda + 2.0 * mu) / rho);
  cplx c2 = std::sqrt(mu / rho);
  cplx k1 = omega / c1, k2 = omega / c2;
  p.c1 = c1; p.c2 = c2; p.k1 = k1; p.k2 = k2;
  cplx c1p2 = c1 * c1, c2p2 = c2 * c2, c1p3 = c1p2 * c1, c1p4 = c1p2 * c1p2;
  cplx k2p2 = k2 * k2;
  cplx ik1 = I * k1, ik2 = I * k2;
  cplx ik1p2 = ik1 * ik1, ik2p2 = ik2 * ik2;
  cplx r = c2p2 / c1p2;
  double om2 = omega * omega;
  p.psi[0] = 0.5 * (1.0 + r);
  p.psi[1] = -1.0 / 3.0 * (2.0 / c2 + c2p2 / c1p3) * I * omega;
  p.psi[2] = I * k1 / k2p2;
  p.psi[3] = 1.0 / ik2;
  p.psi[4] = 1.0 / k2p2;
  p.psi[5] = -1.0 / k2p2;
  p.chi[0] = -0.5 * (1.0 - r);
  p.chi[1] = -r;
  p.chi[2] = -3.0 * r / ik1;
  p.chi[3] = 3.0 / ik2;
  p.chi[4] = -3.0 * r / ik1p2;
  p.chi[5] = 3.0 / ik2p2;
  p.T1[0] = 3.0 * (r - 1.0);
  p.T1[1] = -0.25 * (1.0 / c2p2 - c2p2 / c1p4) * om2;
  p.T1[2] = -2.0 * I * k1 * r;
  p.T1[3] = 2.0 * I * k2;
  p.T1[4] = -12.0 * r;
  p.T1[5] = 12.0;
  p.T1[6] = -r * 30.0 / ik1;
  p.T1[7] = 30.0 / ik2;
  p.T1[8] = -r * 30.0 / ik1p2;
  p.T1[9] = 30.0 / ik2p2;
  p.T2[0] = -r;
  p.T2[1] = -0.25 * (1.0 / c2p2 + c2p2 / c1p4) * om2;
  p.T2[2] = -I * k2;
  p.T2[3] = 2.0 * r;
  p.T2[4] = -3.0;
  p.T2[5] = r * 6.0 / ik1;
  p.T2[6] = -6.0 / ik2;
  p.T2[7] = r * 6.0 / ik1p2;
  p.T2[8] = -6.0 / ik2p2;
  p.T3[0] = r;
  p.T3[1] = 0.25 * (3.0 * c2p2 / c1p4 - 2.0 / c1p2 + 1.0 / c2p2) * om2;
  p.T3[2] = (2.0 * r - 1.0) * I * k1;
  p.T3[3] = 4.0 * r - 1.0;
  p.T3[4] = -2.0;
  p.T3[5] = r * 6.0 / ik1;
  p.T3[6] = -6.0 / ik2;
  p.T3[7] = r * 6.0 / ik1p2;
  p.T3[8] = -6.0 / ik2p2;
  p.cte_u = c_1_4pi / mu;
  p.cte_t = cplx(c_1_4pi, 0.0);
  // S1..S5 (bem_harela3d.f90:219-279)
  cplx k1p2 = k1 * k1, q = k1p2 / k2p2, c1p5 = c1p4 * c1, c2p3 = c2p2 * c2;
  double om3 = om2 * omega;
  p.S1[0] = 3.0 * (1.0 - 2.0 * r);
  p.S1[1] = -0.5 * c2p2 / c1p4 * om2;
  p.S1[2] = k2p2;
  p.S1[3] = 4.0 * I * k1 * q;
  p.S1[4] = -7.0 * I * k2;
  p.S1[5] = 24.0 * q;
  p.S1[6] = -27.0;
  p.S1[7] = 60.0 * q / ik1;
  p.S1[8] = -60.0 / ik2;
  p.S1[9] = 60.0 * q / ik1p2;
  p.S1[10] = -60.0 / ik2p2;
  p.S2[0] = 6.0 * r;
  p.S2[1] = (0.5 / c2p2 + 1.5 * c2p2 / c1p4 - 1.0 / c1p2) * om2;
  p.S2[2] = 2.0 * c2p2 / c1p4 * (c1p2 / c2p2 - 2.0) * om2;
  p.S2[3] = 2.0 * I * c2p2 / c1p3 * (8.0 - 3.0 * c1p2 / c2p2) * omega;
  p.S2[4] = -4.0 * I * k2;
  p.S2[5] = 6.0 * r * (6.0 - c1p2 / c2p2);
  p.S2[6] = -24.0;
  p.S2[7] = r * 60.0 / ik1;
  p.S2[8] = -60.0 / ik2;
  p.S2[9] = 60.0 / ik2p2;
  p.S2[10] = -60.0 / ik2p2;
  p.S3[0] = 30.0 * (1.0 - r);
  p.S3[1] = 1.5 * (1.0 / c2p2 - c2p2 / c1p4) * om2;
  p.S3[2] = -4.0 * r * k1p2;
  p.S3[3] = 4.0 * k2p2;
  p.S3[4] = 40.0 * r * I * k1;
  p.S3[5] = -40.0 * I * k2;
  p.S3[6] = 180.0 * r;
  p.S3[7] = -180.0;
  p.S3[8] = 420.0 * r / ik1;
  p.S3[9] = -420.0 / ik2;
  p.S3[10] = 420.0 / ik2p2;
  p.S3[11] = -420.0 / ik2p2;
  p.S4[0] = 2.0 * r;
  p.S4[1] = 0.5 * (c2p2 / c1p4 + 1.0 / c2p2) * om2;
  p.S4[2] = -2.0 / 5.0 * (1.0 / c2p3 + 2.0 / 3.0 * c2p2 / c1p5) * I * om3;
  p.S4[3] = 2.0 * I * k2;
  p.S4[4] = -4.0 * r;
  p.S4[5] = 6.0;
  p.S4[6] = -12.0 * r / ik1;
  p.S4[7] = 12.0 / ik2;
  p.S4[8] = -12.0 / ik2p2;
  p.S4[9] = 12.0 / ik2p2;
  p.S5[0] = 2.0 * (1.0 - 3.0 * r);
  p.S5[1] = (-2.0 / c1p2 + 0.5 / c2p2 + 0.5 * c2p2 / c1p4) * om2;
  p.S5[2] = (8.0 / 3.0 / c1p3 + 4.0 / 15.0 / c2p3 - 1.0 / c1 / c2p2 - 24.0 / 15.0 * c2p2 / c1p5) * I * om3;
  p.S5[3] = (-4.0 / c1p2 + 1.0 / c2p2 + 4.0 * c2p2 / c1p4) * om2;
  p.S5[4] = 4.0 * I * (1.0 / c1 - 2.0 * c2p2 / c1p3) * omega;
  p.S5[5] = 4.0 * (1.0 - 3.0 * r);
  p.S5[6] = 4.0;
  p.S5[7] = 12.0 * I * k1 / k2p2;
  p.S5[8] = -12.0 * I / k2;
  p.S5[9] = 12.0 / k2p2;
  p.S5[10] = -12.0 / k2p2;
  p.cte_d = cplx(c_1_4pi, 0.0);
  p.cte_s = c_1_4pi * mu;
  return p;
}

// Per integration point evaluation of the fundamental solutions without their
// constants. Static: bem_staela3d.f90:622-633; harmonic: bem_harela3d.f90:654-688.
struct StaelaK {
  typedef double T;
  static constexpr int F = 5;  // quasi-singular estimate for 1/r^5 integrands
  double cteu1, cteu2, ctet1, ctet2, mu, nu;
  StaelaK(double mu_, double nu_) : mu(mu_), nu(nu_) {
    cteu1 = 1.0 / (16.0 * c_pi * mu * (1.0 - nu));
    cteu2 = 3.0 - 4.0 * nu;
    ctet1 = -1.0 / (8.0 * c_pi * (1.0 - nu));
    ctet2 = 1.0 - 2.0 * nu;
  }
  T cu() const { return cteu1; }
  T ct() const { return ctet1; }
  inline void eval(const double rv[3], const double n[3], T fu[3][3], T ft[3][3]) const {
    double r = std::sqrt(rv[0] * rv[0] + rv[1] * rv[1] + rv[2] * rv[2]);
    double d1r = 1.0 / r, d1r2 = d1r * d1r;
    double drdx[3] = {rv[0] * d1r, rv[1] * d1r, rv[2] * d1r};
    double drdn = drdx[0] * n[0] + drdx[1] * n[1] + drdx[2] * n[2];
    for (int il = 0; il < 3; ++il)
      for (int ik = 0; ik < 3; ++ik) {
        double dk = (il == ik) ? 1.0 : 0.0;
        fu[il][ik] = d1r * (cteu2 * dk + drdx[il] * drdx[ik]);
        ft[il][ik] = d1r2 * ((ctet2 * dk + 3.0 * drdx[il] * drdx[ik]) * drdn +
                             ctet2 * (n[il] * drdx[ik] - n[ik] * drdx[il]));
      }
  }
};
struct HarelaK {
  typedef cplx T;
  static constexpr int F = 5;
  HarPar p;
  explicit HarelaK(const HarPar& pp) : p(pp) {}
  T cu() const { return p.cte_u; }
  T ct() const { return p.cte_t; }
  inline void coeffs(double r, cplx& psi, cplx& chi, cplx& TT1, cplx& TT2, cplx& TT3, double& d1r1,
                     double& d1r2, bool full) const {
    d1r1 = 1.0 / r;
    d1r2 = d1r1 * d1r1;
    double d1r3 = d1r2 * d1r1, d1r4 = d1r3 * d1r1;
    const cplx I(0.0, 1.0);
    cplx z[2] = {-I * p.k1 * r, -I * p.k2 * r};
    cplx E[7][2];
    zexp_decomposed(2, z, E);
    for (int j = 0; j < 2; ++j) {
      E[2][j] = E[2][j] * d1r1;
      E[3][j] = E[3][j] * d1r2;
      E[4][j] = E[4][j] * d1r3;
      E[5][j] = E[5][j] * d1r4;
    }
    psi = p.psi[0] * d1r1 + p.psi[1] + E[2][1] + p.psi[2] * E[3][0] + p.psi[3] * E[3][1] + p.psi[4] * E[4][0] +
          p.psi[5] * E[4][1];
    chi = p.chi[0] * d1r1 + p.chi[1] * E[2][0] + E[2][1] + p.chi[2] * E[3][0] + p.chi[3] * E[3][1] +
          p.chi[4] * E[4][0] + p.chi[5] * E[4][1];
    if (full) {
      TT1 = p.T1[0] * d1r2 + p.T1[1] + p.T1[2] * E[2][0] + p.T1[3] * E[2][1] + p.T1[4] * E[3][0] +
            p.T1[5] * E[3][1] + p.T1[6] * E[4][0] + p.T1[7] * E[4][1] + p.T1[8] * E[5][0] + p.T1[9] * E[5][1];
      TT2 = p.T2[0] * d1r2 + p.T2[1] + p.T2[2] * E[2][1] + p.T2[3] * E[3][0] + p.T2[4] * E[3][1] +
            p.T2[5] * E[4][0] + p.T2[6] * E[4][1] + p.T2[7] * E[5][0] + p.T2[8] * E[5][1];
      TT3 = p.T3[0] * d1r2 + p.T3[1] + p.T3[2] * E[2][0] + p.T3[3] * E[3][0] + p.T3[4] * E[3][1] +
            p.T3[5] * E[4][0] + p.T3[6] * E[4][1] + p.T3[7] * E[5][0] + p.T3[8] * E[5][1];
    } else {  // regular parts only (bem_harela3d.f90 sbie_int)
      TT1 = p.T1[1] + p.T1[2] * E[2][0] + p.T1[3] * E[2][1] + p.T1[4] * E[3][0] + p.T1[5] * E[3][1] +
            p.T1[6] * E[4][0] + p.T1[7] * E[4][1] + p.T1[8] * E[5][0] + p.T1[9] * E[5][1];
      TT2 = p.T2[1] + p.T2[2] * E[2][1] + p.T2[3] * E[3][0] + p.T2[4] * E[3][1] + p.T2[5] * E[4][0] +
            p.T2[6] * E[4][1] + p.T2[7] * E[5][0] + p.T2[8] * E[5][1];
      TT3 = p.T3[1] + p.T3[2] * E[2][0] + p.T3[3] * E[3][0] + p.T3[4] * E[3][1] + p.T3[5] * E[4][0] +
            p.T3[6] * E[4][1] + p.T3[7] * E[5][0] + p.T3[8] * E[5][1];
    }
  }
  inline void eval(const double rv[3], const double n[3], T fu[3][3], T ft[3][3]) const {
    double r = std::sqrt(rv[0] * rv[0] + rv[1] * rv[1] + rv[2] * rv[2]);
    cplx psi, chi, TT1, TT2, TT3;
    double d1r1, d1r2;
    coeffs(r, psi, chi, TT1, TT2, TT3, d1r1, d1r2, true);
    double drdx[3] = {rv[0] * d1r1, rv[1] * d1r1, rv[2] * d1r1};
    double drdn = drdx[0] * n[0] + drdx[1] * n[1] + drdx[2] * n[2];
    for (int il = 0; il < 3; ++il)
      for (int ik = 0; ik < 3; ++ik) {
        double dk = (il == ik) ? 1.0 : 0.0;
        fu[il][ik] = psi * dk - chi * drdx[il] * drdx[ik];
        ft[il][ik] = TT1 * drdx[il] * drdx[ik] * drdn + TT2 * (drdn * dk + drdx[ik] * n[il]) + TT3 * drdx[il] * n[ik];
      }
  }
};

// HBIE kernels at a point x_i with unit normal n_i, exterior integration.
// eval() returns s* (integrated with phi^p into m) in the slot of t* and d*
// (with phi^s into l) in the slot of u*, so ext_pre / ext_st / ext_adp
// integrate them unchanged: m takes the place of h (constant ct(), sign
// reversed with the element) and l that of g (constant cu()).
// Static: bem_staela3d.f90:4376-4446; harmonic: bem_harela3d.f90:2573-2662.
struct StaelaHK {
  typedef double T;
  static constexpr int F = 7;  // quasi-singular estimate for 1/r^7 integrands
  double nu, cted1, cted2, ctes1, ctes2, ctes3, ni[3];
  StaelaHK(double mu, double nu_, const double n_i[3]) : nu(nu_) {
    cted1 = -1.0 / (8.0 * c_pi * (1.0 - nu));
    cted2 = 1.0 - 2.0 * nu;
    ctes1 = mu / (4.0 * c_pi * (1.0 - nu));
    ctes2 = 1.0 - 2.0 * nu;
    ctes3 = 1.0 - 4.0 * nu;
    for (int c = 0; c < 3; ++c) ni[c] = n_i[c];
  }
  T cu() const { return cted1; }
  T ct() const { return ctes1; }
  inline void eval(const double rv[3], const double n[3], T fd[3][3], T fs[3][3]) const {
    double r = std::sqrt(rv[0] * rv[0] + rv[1] * rv[1] + rv[2] * rv[2]);
    double d1r = 1.0 / r, d1r2 = d1r * d1r, d1r3 = d1r2 * d1r;
    double drdx[3] = {rv[0] * d1r, rv[1] * d1r, rv[2] * d1r};
    double drdn = drdx[0] * n[0] + drdx[1] * n[1] + drdx[2] * n[2];
    double drdni = -(drdx[0] * ni[0] + drdx[1] * ni[1] + drdx[2] * ni[2]);
    double nni = n[0] * ni[0] + n[1] * ni[1] + n[2] * ni[2];
    for (int il = 0; il < 3; ++il)
      for (int ik = 0; ik < 3; ++ik) {
        double dk = (il == ik) ? 1.0 : 0.0;
        fd[il][ik] = d1r2 * ((cted2 * dk + 3.0 * drdx[il] * drdx[ik]) * drdni +
                             cted2 * (ni[il] * drdx[ik] - ni[ik] * drdx[il]));
        fs[il][ik] = d1r3 * (3.0 * (5.0 * drdx[il] * drdx[ik] - nu * dk) * drdn * drdni +
                             3.0 * ctes2 * (drdx[ik] * ni[il] * drdn - drdx[il] * n[ik] * drdni) +
                             3.0 * nu * (drdx[il] * ni[ik] * drdn - drdx[ik] * n[il] * drdni) +
                             (3.0 * nu * drdx[il] * drdx[ik] + ctes2 * dk) * nni + ctes2 * n[il] * ni[ik] -
                             ctes3 * n[ik] * ni[il]);
      }
  }
};
struct HarelaHK {
  typedef cplx T;
  static constexpr int F = 7;
  HarPar p;
  double ni[3];
  HarelaHK(const HarPar& pp, const double n_i[3]) : p(pp) {
    for (int c = 0; c < 3; ++c) ni[c] = n_i[c];
  }
  T cu() const { return p.cte_d; }
  T ct() const { return p.cte_s; }
  inline void eval(const double rv[3], const double n[3], T fd[3][3], T fs[3][3]) const {
    double r = std::sqrt(rv[0] * rv[0] + rv[1] * rv[1] + rv[2] * rv[2]);
    double d1r1 = 1.0 / r, d1r2 = d1r1 * d1r1, d1r3 = d1r2 * d1r1, d1r4 = d1r3 * d1r1, d1r5 = d1r4 * d1r1;
    double drdx[3] = {rv[0] * d1r1, rv[1] * d1r1, rv[2] * d1r1};
    double drdn = drdx[0] * n[0] + drdx[1] * n[1] + drdx[2] * n[2];
    double drdni = -(drdx[0] * ni[0] + drdx[1] * ni[1] + drdx[2] * ni[2]);
    double nni = n[0] * ni[0] + n[1] * ni[1] + n[2] * ni[2];
    const cplx I(0.0, 1.0);
    cplx z[2] = {-I * p.k1 * r, -I * p.k2 * r};
    cplx E[7][2];
    zexp_decomposed(2, z, E);
    for (int j = 0; j < 2; ++j) {
      E[2][j] = E[2][j] * d1r1;
      E[3][j] = E[3][j] * d1r2;
      E[4][j] = E[4][j] * d1r3;
      E[5][j] = E[5][j] * d1r4;
      E[6][j] = E[6][j] * d1r5;
    }
    cplx TT1 = p.T1[0] * d1r2 + p.T1[1] + p.T1[2] * E[2][0] + p.T1[3] * E[2][1] + p.T1[4] * E[3][0] +
               p.T1[5] * E[3][1] + p.T1[6] * E[4][0] + p.T1[7] * E[4][1] + p.T1[8] * E[5][0] + p.T1[9] * E[5][1];
    cplx TT2 = p.T2[0] * d1r2 + p.T2[1] + p.T2[2] * E[2][1] + p.T2[3] * E[3][0] + p.T2[4] * E[3][1] +
               p.T2[5] * E[4][0] + p.T2[6] * E[4][1] + p.T2[7] * E[5][0] + p.T2[8] * E[5][1];
    cplx TT3 = p.T3[0] * d1r2 + p.T3[1] + p.T3[2] * E[2][0] + p.T3[3] * E[3][0] + p.T3[4] * E[3][1] +
               p.T3[5] * E[4][0] + p.T3[6] * E[4][1] + p.T3[7] * E[5][0] + p.T3[8] * E[5][1];
    cplx S1 = p.S1[0] * d1r3 + p.S1[1] * d1r1 + p.S1[2] * E[2][1] + p.S1[3] * E[3][0] + p.S1[4] * E[3][1] +
              p.S1[5] * E[4][0] + p.S1[6] * E[4][1] + p.S1[7] * E[5][0] + p.S1[8] * E[5][1] + p.S1[9] * E[6][0] +
              p.S1[10] * E[6][1];
    cplx S2 = p.S2[0] * d1r3 + p.S2[1] * d1r1 + p.S2[2] * E[2][0] + p.S2[3] * E[3][0] + p.S2[4] * E[3][1] +
              p.S2[5] * E[4][0] + p.S2[6] * E[4][1] + p.S2[7] * E[5][0] + p.S2[8] * E[5][1] + p.S2[9] * E[6][0] +
              p.S2[10] * E[6][1];
    cplx S3 = p.S3[0] * d1r3 + p.S3[1] * d1r1 + p.S3[2] * E[2][0] + p.S3[3] * E[2][1] + p.S3[4] * E[3][0] +
              p.S3[5] * E[3][1] + p.S3[6] * E[4][0] + p.S3[7] * E[4][1] + p.S3[8] * E[5][0] + p.S3[9] * E[5][1] +
              p.S3[10] * E[6][0] + p.S3[11] * E[6][1];
    cplx S4 = p.S4[0] * d1r3 + p.S4[1] * d1r1 + p.S4[2] + p.S4[3] * E[3][1] + p.S4[4] * E[4][0] +
              p.S4[5] * E[4][1] + p.S4[6] * E[5][0] + p.S4[7] * E[5][1] + p.S4[8] * E[6][0] + p.S4[9] * E[6][1];
    cplx S5 = p.S5[0] * d1r3 + p.S5[1] * d1r1 + p.S5[2] + p.S5[3] * E[2][0] + p.S5[4] * E[3][0] +
              p.S5[5] * E[4][0] + p.S5[6] * E[4][1] + p.S5[7] * E[5][0] + p.S5[8] * E[5][1] + p.S5[9] * E[6][0] +
              p.S5[10] * E[6][1];
    for (int il = 0; il < 3; ++il)
      for (int ik = 0; ik < 3; ++ik) {
        double dk = (il == ik) ? 1.0 : 0.0;
        fd[il][ik] = TT1 * drdx[il] * drdx[ik] * drdni - TT2 * (-drdni * dk + drdx[il] * ni[ik]) -
                     TT3 * drdx[ik] * ni[il];
        fs[il][ik] = S1 * (drdx[il] * ni[ik] * drdn - drdx[ik] * n[il] * drdni - dk * drdn * drdni +
                           drdx[il] * drdx[ik] * nni) +
                     S2 * (drdx[ik] * ni[il] * drdn - drdx[il] * n[ik] * drdni) +
                     S3 * drdx[il] * drdx[ik] * drdn * drdni + S4 * (dk * nni + ni[ik] * n[il]) + S5 * n[ik] * ni[il];
      }
  }
};

// Kernel at the integration point x for the collocation point x_i: the
// full-space kernels depend on x - x_i only; the half-space complementary
// kernel (HscK, below) overloads this with the absolute coordinates.
template <class K>
inline void kernel_at(const K& k, const double x[3], const double x_i[3], const double n[3],
                      typename K::T fu[3][3], typename K::T ft[3][3]) {
  double rv[3] = {x[0] - x_i[0], x[1] - x_i[1], x[2] - x_i[2]};
  k.eval(rv, n, fu, ft);
}

template <class K>
struct HG {
  typename K::T h[8][3][3], g[8][3][3];
  void zero() {
    for (int a = 0; a < 8; ++a)
      for (int b = 0; b < 3; ++b)
        for (int c = 0; c < 3; ++c) h[a][b][c] = g[a][b][c] = 0.0;
  }
};

// sbie_ext_pre: bem_staela3d.f90:592-650 / bem_harela3d.f90:628-700
template <class K>
static void ext_pre(const K& k, int ps, const Elem& e, bool reverse, const double x_i[3], HG<K>& out) {
  out.zero();
  for (int kip = 0; kip < e.ps_ngp[ps]; ++kip) {
    int kt = e.ps_off[ps] + kip;
    const double* x = &e.px[kt * 3];
    const double* n = &e.pn[kt * 3];
    const double* pj = &e.pphijw[kt * 8];
    typename K::T fu[3][3], ft[3][3];
    kernel_at(k, x, x_i, n, fu, ft);
    for (int il = 0; il < 3; ++il)
      for (int ik = 0; ik < 3; ++ik)
        for (int a = 0; a < 8; ++a) {
          out.h[a][il][ik] = out.h[a][il][ik] + ft[il][ik] * pj[a];
          out.g[a][il][ik] = out.g[a][il][ik] + fu[il][ik] * pj[a];
        }
  }
  for (int a = 0; a < 8; ++a)
    for (int il = 0; il < 3; ++il)
      for (int ik = 0; ik < 3; ++ik) {
        out.h[a][il][ik] = k.ct() * out.h[a][il][ik];
        out.g[a][il][ik] = k.cu() * out.g[a][il][ik];
        if (reverse) out.h[a][il][ik] = -out.h[a][il][ik];
      }
}

// sbie_ext_st (quadrilateral branch): bem_staela3d.f90:654-969 / bem_harela3d.f90:702-1048
template <class K>
static void ext_st(const K& k, const Elem& e, bool reverse, const double xi_s[4][2], const double x_i[3],
                   const double barxip[2], double barr, int gln, HG<K>& out) {
  out.zero();
  Telles tp1 = telles11(barxip[0], barr), tp2 = telles11(barxip[1], barr);
  for (int k1 = 1; k1 <= gln; ++k1) {
    double g1 = gl11_xi(k1, gln), w1 = gl11_w(k1, gln);
    double xip1, jt1;
    telles_xi_jac(tp1, g1, xip1, jt1);
    for (int k2 = 1; k2 <= gln; ++k2) {
      double g2 = gl11_xi(k2, gln), w2 = gl11_w(k2, gln);
      double xip2, jt2;
      telles_xi_jac(tp2, g2, xip2, jt2);
      double xip[2] = {xip1, xip2};
      double sp[4], sd1[4], sd2[4];
      phi_quad4(xip, sp);
      dphi_quad4(xip, sd1, sd2);
      double xi[2] = {0, 0}, dx1[2] = {0, 0}, dx2[2] = {0, 0};
      for (int q = 0; q < 4; ++q)
        for (int c = 0; c < 2; ++c) {
          xi[c] = xi[c] + sp[q] * xi_s[q][c];
          dx1[c] = dx1[c] + sd1[q] * xi_s[q][c];
          dx2[c] = dx2[c] + sd2[q] * xi_s[q][c];
        }
      double js = dx1[0] * dx2[1] - dx1[1] * dx2[0];
      double phi[8], d1[8], d2[8];
      phi_quad8(xi, phi);
      dphi_quad8(xi, d1, d2);
      double x[3] = {0, 0, 0}, T1[3] = {0, 0, 0}, T2[3] = {0, 0, 0};
      for (int q = 0; q < 8; ++q)
        for (int c = 0; c < 3; ++c) {
          x[c] = x[c] + phi[q] * e.x[q][c];
          T1[c] = T1[c] + d1[q] * e.x[q][c];
          T2[c] = T2[c] + d2[q] * e.x[q][c];
        }
      double N[3] = {T1[1] * T2[2] - T1[2] * T2[1], T1[2] * T2[0] - T1[0] * T2[2],
                     T1[0] * T2[1] - T1[1] * T2[0]};
      double jg = std::sqrt(N[0] * N[0] + N[1] * N[1] + N[2] * N[2]);
      double n[3] = {N[0] / jg, N[1] / jg, N[2] / jg};
      double jw = jg * js * jt1 * jt2 * w1 * w2;
      double pj[8];
      for (int q = 0; q < 8; ++q) pj[q] = phi[q] * jw;
      typename K::T fu[3][3], ft[3][3];
      kernel_at(k, x, x_i, n, fu, ft);
      for (int il = 0; il < 3; ++il)
        for (int ik = 0; ik < 3; ++ik)
          for (int a = 0; a < 8; ++a) {
            out.h[a][il][ik] = out.h[a][il][ik] + ft[il][ik] * pj[a];
            out.g[a][il][ik] = out.g[a][il][ik] + fu[il][ik] * pj[a];
          }
    }
  }
  for (int a = 0; a < 8; ++a)
    for (int il = 0; il < 3; ++il)
      for (int ik = 0; ik < 3; ++ik) {
        out.h[a][il][ik] = k.ct() * out.h[a][il][ik];
        out.g[a][il][ik] = k.cu() * out.g[a][il][ik];
        if (reverse) out.h[a][il][ik] = -out.h[a][il][ik];
      }
}

struct AdpStats { long leaves = 0, points = 0, maxdepth_hits = 0; };

// sbie_ext_adp: bem_staela3d.f90:973-1096 / bem_harela3d.f90:1050-1172
template <class K>
static void ext_adp(const K& k, const Elem& e, bool reverse, double xi_s[4][2], const double x_i[3],
                    const QsParams& qsp, int ks, int ns, HG<K>& acc, AdpStats* st, const double* x_near = nullptr) {
  // x_near: the point whose nearest element point drives the subdivision (the
  // collocation point, or its image for the half-space complementary kernel,
  // bem_staela3d.f90:8411-8412)
  const double* xn = x_near ? x_near : x_i;
  double barxip[2], rmin, d;
  int method;
  if (ks == 1) {
    acc.zero();
    xi_s[0][0] = -1; xi_s[0][1] = -1;
    xi_s[1][0] = 1;  xi_s[1][1] = -1;
    xi_s[2][0] = 1;  xi_s[2][1] = 1;
    xi_s[3][0] = -1; xi_s[3][1] = 1;
    nearest_element_point_quad8(e.x, e.cl, xn, barxip, &rmin, &d, &method);
  } else {
    double x_s[8][3];
    subdivision_coords_quad8(e.x, xi_s, x_s);
    double cl = characteristic_length_quad8(x_s, 1e-12);
    nearest_element_point_quad8(x_s, cl, xn, barxip, &rmin, &d, &method);
  }
  int gln_near = qs_n_estimation_telles(2, K::F, qsp, d, barxip);
  bool subdivide = false;
  if (ks == ns) {
    if (gln_near == 0) { gln_near = 30; if (st) st->maxdepth_hits++; }
  } else if (gln_near == 0) {
    subdivide = true;
  }
  if (subdivide) {
    double t[4][2];
    double c[2] = {0.25 * (xi_s[0][0] + xi_s[1][0] + xi_s[2][0] + xi_s[3][0]),
                   0.25 * (xi_s[0][1] + xi_s[1][1] + xi_s[2][1] + xi_s[3][1])};
    for (int q = 0; q < 2; ++q) {
      t[0][q] = xi_s[0][q]; t[1][q] = 0.5 * (xi_s[0][q] + xi_s[1][q]); t[2][q] = c[q]; t[3][q] = 0.5 * (xi_s[0][q] + xi_s[3][q]);
    }
    ext_adp(k, e, reverse, t, x_i, qsp, ks + 1, ns, acc, st, x_near);
    for (int q = 0; q < 2; ++q) {
      t[0][q] = 0.5 * (xi_s[0][q] + xi_s[1][q]); t[1][q] = xi_s[1][q]; t[2][q] = 0.5 * (xi_s[1][q] + xi_s[2][q]); t[3][q] = c[q];
    }
    ext_adp(k, e, reverse, t, x_i, qsp, ks + 1, ns, acc, st, x_near);
    for (int q = 0; q < 2; ++q) {
      t[0][q] = c[q]; t[1][q] = 0.5 * (xi_s[1][q] + xi_s[2][q]); t[2][q] = xi_s[2][q]; t[3][q] = 0.5 * (xi_s[2][q] + xi_s[3][q]);
    }
    ext_adp(k, e, reverse, t, x_i, qsp, ks + 1, ns, acc, st, x_near);
    for (int q = 0; q < 2; ++q) {
      t[0][q] = 0.5 * (xi_s[0][q] + xi_s[3][q]); t[1][q] = c[q]; t[2][q] = 0.5 * (xi_s[2][q] + xi_s[3][q]); t[3][q] = xi_s[3][q];
    }
    ext_adp(k, e, reverse, t, x_i, qsp, ks + 1, ns, acc, st, x_near);
  } else {
    double barr = telles_barr_any(d);
    int gln = std::max(gln_near, e.gln_far);
    HG<K> tmp;
    ext_st(k, e, reverse, xi_s, x_i, barxip, barr, gln, tmp);
    if (st) { st->leaves++; st->points += (long)gln * gln; }
    for (int a = 0; a < 8; ++a)
      for (int il = 0; il < 3; ++il)
        for (int ik = 0; ik < 3; ++ik) {
          acc.h[a][il][ik] = acc.h[a][il][ik] + tmp.h[a][il][ik];
          acc.g[a][il][ik] = acc.g[a][il][ik] + tmp.g[a][il][ik];
        }
  }
}

// fbem_bem_staela3d_sbie_int_li (bem_staela3d.f90:2245-2376), line3 edge
static void int_li(const double xn[3][3], double xi_s[2], const double x_i[3], int ngp_min, const QsParams& qsp,
                   int ks, int ns, double hli[3][3]) {
  double x_s[3][3];
  if (ks == 1) {
    xi_s[0] = -1.0;
    xi_s[1] = 1.0;
    std::memcpy(x_s, xn, sizeof(x_s));
  } else {
    subdivision_coords_line3(xn, xi_s, x_s);
  }
  double cl = characteristic_length_line3(x_s, 1e-12);
  double barxip, rmin, d;
  int method;
  nearest_element_point_line3(x_s, cl, x_i, &barxip, &rmin, &d, &method);
  int gln_near = qs_n_estimation_telles(1, 1, qsp, d, &barxip);
  bool subdivide = false;
  if (ks == ns) {
    if (gln_near == 0) gln_near = 30;
  } else if (gln_near == 0) {
    subdivide = true;
  }
  if (subdivide) {
    double t[2];
    t[0] = xi_s[0]; t[1] = 0.5 * (xi_s[0] + xi_s[1]);
    int_li(xn, t, x_i, ngp_min, qsp, ks + 1, ns, hli);
    t[0] = 0.5 * (xi_s[0] + xi_s[1]); t[1] = xi_s[1];
    int_li(xn, t, x_i, ngp_min, qsp, ks + 1, ns, hli);
  } else {
    double ht[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    int gln = std::max(gln_near, ngp_min);
    double barr = telles_barr_any(d);
    Telles tp = telles11(barxip, barr);
    for (int kip = 1; kip <= gln; ++kip) {
      double gm = gl11_xi(kip, gln), w = gl11_w(kip, gln);
      double xip, jt;
      telles_xi_jac(tp, gm, xip, jt);
      double xi = 0.5 * (1.0 - xip) * xi_s[0] + 0.5 * (1.0 + xip) * xi_s[1];
      double js = 0.5 * (xi_s[1] - xi_s[0]);
      double phi[3], dphi[3];
      phi_line3(xi, phi);
      dphi_line3(xi, dphi);
      double x[3] = {0, 0, 0}, T[3] = {0, 0, 0};
      for (int q = 0; q < 3; ++q)
        for (int c = 0; c < 3; ++c) {
          x[c] = x[c] + phi[q] * xn[q][c];
          T[c] = T[c] + dphi[q] * xn[q][c];
        }
      double jg = std::sqrt(T[0] * T[0] + T[1] * T[1] + T[2] * T[2]);
      double t[3] = {T[0] / jg, T[1] / jg, T[2] / jg};
      double rv[3] = {x[0] - x_i[0], x[1] - x_i[1], x[2] - x_i[2]};
      double r = std::sqrt(rv[0] * rv[0] + rv[1] * rv[1] + rv[2] * rv[2]);
      double dr1 = 1.0 / r;
      double jw = jg * js * jt * w;
      ht[0][1] = ht[0][1] - dr1 * t[2] * jw;
      ht[0][2] = ht[0][2] + dr1 * t[1] * jw;
      ht[1][2] = ht[1][2] - dr1 * t[0] * jw;
    }
    ht[1][0] = -ht[0][1];
    ht[2][0] = -ht[0][2];
    ht[2][1] = -ht[1][2];
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) hli[a][b] = hli[a][b] + ht[a][b];
  }
}

// Shared surface-integral driver of sbie_int: bem_staela3d.f90:1100-1381 and
// bem_harela3d.f90:1174-1472 (polar coordinates, CPV regularisation, line
// integrals for the strongly singular part).
template <class K>
static void sbie_int(const K& k, const Elem& e, bool reverse, const double xi_i[2], HG<K>& out);

template <>
void sbie_int<StaelaK>(const StaelaK& k, const Elem& e, bool reverse, const double xi_i[2], HG<StaelaK>& out);
template <>
void sbie_int<HarelaK>(const HarelaK& k, const Elem& e, bool reverse, const double xi_i[2], HG<HarelaK>& out);

static void line_integrals(const Elem& e, const double x_i[3], int nsub, const int* st, double hli[3][3]) {
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b) hli[a][b] = 0.0;
  QsParams qsp;
  qs_calculate_parameters(1e-15, qsp);
  for (int ke = 1; ke <= 4; ++ke) {
    bool integ = false;
    for (int s = 0; s < nsub; ++s)
      if (st[s] == 2 * ke - 1 || st[s] == 2 * ke) { integ = true; break; }
    if (!integ) continue;
    double xe[3][3];
    for (int q = 0; q < 3; ++q)
      for (int c = 0; c < 3; ++c) xe[q][c] = e.x[quad8_edge_node[ke - 1][q]][c];
    double xs[2];
    int_li(xe, xs, x_i, 5, qsp, 1, 16, hli);
  }
}

template <class K, class PointFn>
static void polar_loop(const Elem& e, const double xi_i[2], const double x_i[3], PointFn fn, int* nsub_out,
                       int st_out[8]) {
  int nsub, st[8];
  double th[8][2], thp[8][2];
  polar_setup_quad(xi_i, &nsub, st, th, thp);
  for (int s = 0; s < nsub; ++s) {
    double ti = th[s][0], tf = th[s][1], tpi = thp[s][0], tpf = thp[s][1];
    const int ngp_rho = 15;
    int ngp_theta = 5 + (int)std::lround(25.0 * (tf - ti) / c_pi_2);
    for (int kt = 1; kt <= ngp_theta; ++kt) {
      double tpp = gl01_xi(kt, ngp_theta), wa = gl01_w(kt, ngp_theta);
      double jtp = (tpf - tpi);
      double tp = jtp * tpp + tpi;
      double theta, rhoij;
      polar_angular_quad(xi_i, st[s], tp, &theta, &rhoij);
      double ct = std::cos(theta), sn = std::sin(theta);
      for (int kr = 1; kr <= ngp_rho; ++kr) {
        double rhop = gl01_xi(kr, ngp_rho), wr = gl01_w(kr, ngp_rho);
        double rho = rhoij * rhop;
        double xi[2] = {xi_i[0] + rho * ct, xi_i[1] + rho * sn};
        double phi[8], d1[8], d2[8];
        phi_quad8(xi, phi);
        dphi_quad8(xi, d1, d2);
        double x[3] = {0, 0, 0}, T1[3] = {0, 0, 0}, T2[3] = {0, 0, 0};
        for (int q = 0; q < 8; ++q)
          for (int c = 0; c < 3; ++c) {
            x[c] = x[c] + phi[q] * e.x[q][c];
            T1[c] = T1[c] + d1[q] * e.x[q][c];
            T2[c] = T2[c] + d2[q] * e.x[q][c];
          }
        double N[3] = {T1[1] * T2[2] - T1[2] * T2[1], T1[2] * T2[0] - T1[0] * T2[2],
                       T1[0] * T2[1] - T1[1] * T2[0]};
        double jg = std::sqrt(N[0] * N[0] + N[1] * N[1] + N[2] * N[2]);
        double n[3] = {N[0] / jg, N[1] / jg, N[2] / jg};
        double rv[3] = {x[0] - x_i[0], x[1] - x_i[1], x[2] - x_i[2]};
        double jw = jg * rho * jtp * wa * wr;
        fn(x, rv, n, phi, jw);
      }
    }
  }
  *nsub_out = nsub;
  for (int s = 0; s < nsub; ++s) st_out[s] = st[s];
}

template <>
void sbie_int<StaelaK>(const StaelaK& k, const Elem& e, bool reverse, const double xi_i[2], HG<StaelaK>& out) {
  out.zero();
  double phii[8];
  phi_quad8(xi_i, phii);
  double x_i[3] = {0, 0, 0};
  for (int q = 0; q < 8; ++q)
    for (int c = 0; c < 3; ++c) x_i[c] = x_i[c] + phii[q] * e.x[q][c];
  int nsub, st[8];
  auto fn = [&](const double*, const double rv[3], const double n[3], const double phi[8], double jw) {
    double r = std::sqrt(rv[0] * rv[0] + rv[1] * rv[1] + rv[2] * rv[2]);
    double d1r = 1.0 / r, d1r2 = d1r * d1r;
    double drdx[3] = {rv[0] * d1r, rv[1] * d1r, rv[2] * d1r};
    double drdn = drdx[0] * n[0] + drdx[1] * n[1] + drdx[2] * n[2];
    double pj[8];
    for (int q = 0; q < 8; ++q) pj[q] = phi[q] * jw;
    for (int il = 0; il < 3; ++il)
      for (int ik = 0; ik < 3; ++ik) {
        double dk = (il == ik) ? 1.0 : 0.0;
        double fu = d1r * (k.cteu2 * dk + drdx[il] * drdx[ik]);
        double ft = d1r2 * drdn * (k.ctet2 * dk + 3.0 * drdx[il] * drdx[ik]);
        for (int a = 0; a < 8; ++a) {
          out.h[a][il][ik] = out.h[a][il][ik] + ft * pj[a];
          out.g[a][il][ik] = out.g[a][il][ik] + fu * pj[a];
        }
        ft = d1r2 * k.ctet2 * (n[il] * drdx[ik] - n[ik] * drdx[il]);
        for (int a = 0; a < 8; ++a) out.h[a][il][ik] = out.h[a][il][ik] + ft * (phi[a] - phii[a]) * jw;
      }
  };
  polar_loop<StaelaK>(e, xi_i, x_i, fn, &nsub, st);
  double hli[3][3];
  line_integrals(e, x_i, nsub, st, hli);
  for (int il = 0; il < 3; ++il)
    for (int ik = 0; ik < 3; ++ik)
      for (int a = 0; a < 8; ++a) out.h[a][il][ik] = out.h[a][il][ik] + phii[a] * k.ctet2 * hli[il][ik];
  for (int a = 0; a < 8; ++a)
    for (int il = 0; il < 3; ++il)
      for (int ik = 0; ik < 3; ++ik) {
        out.h[a][il][ik] = k.ctet1 * out.h[a][il][ik];
        out.g[a][il][ik] = k.cteu1 * out.g[a][il][ik];
        if (reverse) out.h[a][il][ik] = -out.h[a][il][ik];
      }
}

template <>
void sbie_int<HarelaK>(const HarelaK& k, const Elem& e, bool reverse, const double xi_i[2], HG<HarelaK>& out) {
  out.zero();
  double phii[8];
  phi_quad8(xi_i, phii);
  double x_i[3] = {0, 0, 0};
  for (int q = 0; q < 8; ++q)
    for (int c = 0; c < 3; ++c) x_i[c] = x_i[c] + phii[q] * e.x[q][c];
  int nsub, st[8];
  const HarPar& p = k.p;
  auto fn = [&](const double*, const double rv[3], const double n[3], const double phi[8], double jw) {
    double r = std::sqrt(rv[0] * rv[0] + rv[1] * rv[1] + rv[2] * rv[2]);
    cplx psi, chi, TT1, TT2, TT3;
    double dr1, dr2;
    k.coeffs(r, psi, chi, TT1, TT2, TT3, dr1, dr2, false);
    double drdx[3] = {rv[0] * dr1, rv[1] * dr1, rv[2] * dr1};
    double drdn = drdx[0] * n[0] + drdx[1] * n[1] + drdx[2] * n[2];
    double pj[8];
    for (int q = 0; q < 8; ++q) pj[q] = phi[q] * jw;
    for (int il = 0; il < 3; ++il)
      for (int ik = 0; ik < 3; ++ik) {
        double dk = (il == ik) ? 1.0 : 0.0;
        cplx fu = psi * dk - chi * drdx[il] * drdx[ik];
        cplx ft = (TT1 + p.T1[0] * dr2) * drdx[il] * drdx[ik] * drdn + (TT2 + p.T2[0] * dr2) * drdn * dk +
                  TT2 * drdx[ik] * n[il] + TT3 * drdx[il] * n[ik];
        for (int a = 0; a < 8; ++a) {
          out.h[a][il][ik] = out.h[a][il][ik] + ft * pj[a];
          out.g[a][il][ik] = out.g[a][il][ik] + fu * pj[a];
        }
        ft = p.T2[0] * dr2 * (n[il] * drdx[ik] - n[ik] * drdx[il]);
        for (int a = 0; a < 8; ++a) out.h[a][il][ik] = out.h[a][il][ik] + ft * (phi[a] - phii[a]) * jw;
      }
  };
  polar_loop<HarelaK>(e, xi_i, x_i, fn, &nsub, st);
  double hli[3][3];
  line_integrals(e, x_i, nsub, st, hli);
  for (int il = 0; il < 3; ++il)
    for (int ik = 0; ik < 3; ++ik)
      for (int a = 0; a < 8; ++a) out.h[a][il][ik] = out.h[a][il][ik] + phii[a] * p.T2[0] * hli[il][ik];
  for (int a = 0; a < 8; ++a)
    for (int il = 0; il < 3; ++il)
      for (int ik = 0; ik < 3; ++ik) {
        out.h[a][il][ik] = p.cte_t * out.h[a][il][ik];
        out.g[a][il][ik] = p.cte_u * out.g[a][il][ik];
        if (reverse) out.h[a][il][ik] = -out.h[a][il][ik];
      }
}

// Pair classes reported for tests: precalculated rule index 0..n_ps-1,
// CLS_ADP for adaptive subdivision, CLS_SING for interior integration.
enum { CLS_ADP = 100, CLS_SING = 101 };

// sbie_auto: bem_staela3d.f90:524-589 / bem_harela3d.f90:1474-1538
template <class K>
static int sbie_auto(const K& k, const Elem& e, bool reverse, const double x_i[3], const QsParams& qsp, int ns,
                     HG<K>& out, AdpStats* st) {
  double r[3] = {e.bc[0] - x_i[0], e.bc[1] - x_i[1], e.bc[2] - x_i[2]};
  double rmin = std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]) - e.br;
  double barxi[2], d;
  int delta;
  if (rmin > 4.0 * e.br) {
    delta = 0;
    barxi[0] = barxi[1] = 0.0;
    d = rmin / e.cl;
  } else {
    int method;
    nearest_element_point_quad8(e.x, e.cl, x_i, barxi, &rmin, &d, &method);
    delta = (d <= 1e-12) ? 1 : 0;
  }
  if (delta == 1) {
    sbie_int<K>(k, e, reverse, barxi, out);
    return CLS_SING;
  }
  int gln_near = qs_n_estimation_standard(2, K::F, qsp, d, barxi);
  int gln = std::max(e.gln_far, gln_near);
  if (gln <= e.ps_gln_max && gln_near > 0) {
    int ps = 0;
    for (int i = 0; i < e.n_ps; ++i)
      if (e.ps_gln[i] >= gln) { ps = i; break; }
    ext_pre<K>(k, ps, e, reverse, x_i, out);
    return ps;
  }
  double xi_s[4][2];
  ext_adp<K>(k, e, reverse, xi_s, x_i, qsp, 1, ns, out, st);
  return CLS_ADP;
}

// ---------------------------------------------------------------------------
// HBIE interior integration: the collocation point lies inside the element
// (never at an edge: the HBIE is collocated at non-nodal points). Polar
// integration of the regularised integrands around xi_i plus line integrals
// over the four edges for the parts reduced by Stokes' theorem.
// Static: fbem_bem_staela3d_hbie_int (bem_staela3d.f90:4918-5353);
// harmonic: fbem_bem_harela3d_hbie_int (bem_harela3d.f90:3169-3630).
// HG<K>.h receives m (integrated with phi^p), HG<K>.g receives l (phi^s).
// ---------------------------------------------------------------------------
static thread_local int g_hbie_err = 0;  // 1: an HBIE collocation point at an element edge

struct HbieLi {
  double lli[3][3], mli1, mli2[3], mli3[3][3], mli4[3], mli5[3][3][3];
  void zero() { std::memset(this, 0, sizeof(*this)); }
};

// fbem_bem_staela3d_hbie_int_li (bem_staela3d.f90:5356-5578): all line
// integrals of one line3 edge, adaptive Telles + bisection, 1/r^2 estimate
static void hbie_int_li(const double xn[3][3], double xi_s[2], const double x_i[3], const double n_i[3], int ngp_min,
                        const QsParams& qsp, int ks, int ns, HbieLi& L) {
  double x_s[3][3];
  if (ks == 1) {
    xi_s[0] = -1.0;
    xi_s[1] = 1.0;
    std::memcpy(x_s, xn, sizeof(x_s));
  } else {
    subdivision_coords_line3(xn, xi_s, x_s);
  }
  double cl = characteristic_length_line3(x_s, 1e-12);
  double barxip, rmin, d;
  int method;
  nearest_element_point_line3(x_s, cl, x_i, &barxip, &rmin, &d, &method);
  int gln_near = qs_n_estimation_telles(1, 2, qsp, d, &barxip);
  bool subdivide = false;
  if (ks == ns) {
    if (gln_near == 0) gln_near = 30;
  } else if (gln_near == 0) {
    subdivide = true;
  }
  if (subdivide) {
    double t[2];
    t[0] = xi_s[0]; t[1] = 0.5 * (xi_s[0] + xi_s[1]);
    hbie_int_li(xn, t, x_i, n_i, ngp_min, qsp, ks + 1, ns, L);
    t[0] = 0.5 * (xi_s[0] + xi_s[1]); t[1] = xi_s[1];
    hbie_int_li(xn, t, x_i, n_i, ngp_min, qsp, ks + 1, ns, L);
    return;
  }
  HbieLi T;
  T.zero();
  int gln = std::max(gln_near, ngp_min);
  Telles tp = telles11(barxip, telles_barr_any(d));
  for (int kip = 1; kip <= gln; ++kip) {
    double gm = gl11_xi(kip, gln), w = gl11_w(kip, gln);
    double xip, jt;
    telles_xi_jac(tp, gm, xip, jt);
    double xi = 0.5 * (1.0 - xip) * xi_s[0] + 0.5 * (1.0 + xip) * xi_s[1];
    double js = 0.5 * (xi_s[1] - xi_s[0]);
    double phi[3], dphi[3];
    phi_line3(xi, phi);
    dphi_line3(xi, dphi);
    double x[3] = {0, 0, 0}, Tg[3] = {0, 0, 0};
    for (int q = 0; q < 3; ++q)
      for (int c = 0; c < 3; ++c) {
        x[c] = x[c] + phi[q] * xn[q][c];
        Tg[c] = Tg[c] + dphi[q] * xn[q][c];
      }
    double jg = std::sqrt(Tg[0] * Tg[0] + Tg[1] * Tg[1] + Tg[2] * Tg[2]);
    double t[3] = {Tg[0] / jg, Tg[1] / jg, Tg[2] / jg};
    double rv[3] = {x[0] - x_i[0], x[1] - x_i[1], x[2] - x_i[2]};
    double r = std::sqrt(rv[0] * rv[0] + rv[1] * rv[1] + rv[2] * rv[2]);
    double dr1 = 1.0 / r, dr3 = 1.0 / (r * r * r);
    double drdx[3] = {rv[0] * dr1, rv[1] * dr1, rv[2] * dr1};
    double jw = jg * js * jt * w;
    T.lli[0][1] = T.lli[0][1] - dr1 * t[2] * jw;
    T.lli[0][2] = T.lli[0][2] + dr1 * t[1] * jw;
    T.lli[1][2] = T.lli[1][2] - dr1 * t[0] * jw;
    double rxni[3] = {rv[1] * n_i[2] - rv[2] * n_i[1], rv[2] * n_i[0] - rv[0] * n_i[2], rv[0] * n_i[1] - rv[1] * n_i[0]};
    double rxnit = rxni[0] * t[0] + rxni[1] * t[1] + rxni[2] * t[2];
    T.mli1 = T.mli1 + dr3 * rxnit * jw;
    for (int a = 0; a < 3; ++a)
      for (int b = a; b < 3; ++b) T.mli3[a][b] = T.mli3[a][b] + dr3 * rxnit * drdx[a] * drdx[b] * jw;
    for (int ik = 0; ik < 3; ++ik) {
      double ek[3] = {0, 0, 0};
      ek[ik] = 1.0;
      double ekxni[3] = {ek[1] * n_i[2] - ek[2] * n_i[1], ek[2] * n_i[0] - ek[0] * n_i[2],
                         ek[0] * n_i[1] - ek[1] * n_i[0]};
      double ekxnit = ekxni[0] * t[0] + ekxni[1] * t[1] + ekxni[2] * t[2];
      double rxek[3] = {rv[1] * ek[2] - rv[2] * ek[1], rv[2] * ek[0] - rv[0] * ek[2], rv[0] * ek[1] - rv[1] * ek[0]};
      double rxekt = rxek[0] * t[0] + rxek[1] * t[1] + rxek[2] * t[2];
      T.mli2[ik] = T.mli2[ik] + dr1 * ekxnit * jw;
      T.mli4[ik] = T.mli4[ik] + dr3 * rxekt * jw;
      for (int a = 0; a < 3; ++a)
        for (int b = a; b < 3; ++b) T.mli5[a][b][ik] = T.mli5[a][b][ik] + dr1 * ekxnit * drdx[a] * drdx[b] * jw;
    }
  }
  T.lli[1][0] = -T.lli[0][1];
  T.lli[2][0] = -T.lli[0][2];
  T.lli[2][1] = -T.lli[1][2];
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < a; ++b) {
      T.mli3[a][b] = T.mli3[b][a];
      for (int k = 0; k < 3; ++k) T.mli5[a][b][k] = T.mli5[b][a][k];
    }
  for (int a = 0; a < 3; ++a) {
    L.mli2[a] = L.mli2[a] + T.mli2[a];
    L.mli4[a] = L.mli4[a] + T.mli4[a];
    for (int b = 0; b < 3; ++b) {
      L.lli[a][b] = L.lli[a][b] + T.lli[a][b];
      L.mli3[a][b] = L.mli3[a][b] + T.mli3[a][b];
      for (int k = 0; k < 3; ++k) L.mli5[a][b][k] = L.mli5[a][b][k] + T.mli5[a][b][k];
    }
  }
  L.mli1 = L.mli1 + T.mli1;
}

// Collocation point data of the interior integration: x_i, the unit normal
// n_i, phi(xi_i) and psi_i, the shape functions' tangential gradient at xi_i
// in the orthogonal frame v1 = t1, v2 = n_i x t1 (bem_staela3d.f90:5022-5118).
struct HbieAt {
  double x_i[3], n_i[3], phi_i[8], psi_i[8][3];
};
static void hbie_at(const Elem& e, const double xi_i[2], HbieAt& a) {
  double d1[8], d2[8];
  phi_quad8(xi_i, a.phi_i);
  dphi_quad8(xi_i, d1, d2);
  double T1[3] = {0, 0, 0}, T2[3] = {0, 0, 0};
  for (int c = 0; c < 3; ++c) a.x_i[c] = 0.0;
  for (int q = 0; q < 8; ++q)
    for (int c = 0; c < 3; ++c) {
      a.x_i[c] = a.x_i[c] + a.phi_i[q] * e.x[q][c];
      T1[c] = T1[c] + d1[q] * e.x[q][c];
      T2[c] = T2[c] + d2[q] * e.x[q][c];
    }
  double N[3] = {T1[1] * T2[2] - T1[2] * T2[1], T1[2] * T2[0] - T1[0] * T2[2], T1[0] * T2[1] - T1[1] * T2[0]};
  double jg = std::sqrt(N[0] * N[0] + N[1] * N[1] + N[2] * N[2]);
  for (int c = 0; c < 3; ++c) a.n_i[c] = N[c] / jg;
  double jxi1 = std::sqrt(T1[0] * T1[0] + T1[1] * T1[1] + T1[2] * T1[2]);
  double jxi2 = std::sqrt(T2[0] * T2[0] + T2[1] * T2[1] + T2[2] * T2[2]);
  double t1[3] = {T1[0] / jxi1, T1[1] / jxi1, T1[2] / jxi1}, t2[3] = {T2[0] / jxi2, T2[1] / jxi2, T2[2] / jxi2};
  const double* ni = a.n_i;
  double v1[3] = {t1[0], t1[1], t1[2]};
  double v2[3] = {ni[1] * t1[2] - ni[2] * t1[1], ni[2] * t1[0] - ni[0] * t1[2], ni[0] * t1[1] - ni[1] * t1[0]};
  double M11 = 1.0, M12 = v1[0] * t2[0] + v1[1] * t2[1] + v1[2] * t2[2], M21 = 0.0,
         M22 = v2[0] * t2[0] + v2[1] * t2[1] + v2[2] * t2[2];
  double det = M11 * M22 - M12 * M21;
  double x11 = M22 / (jxi1 * det), x12 = -M12 / (jxi1 * det), x21 = -M21 / (jxi2 * det), x22 = M11 / (jxi2 * det);
  for (int k = 0; k < 8; ++k)
    for (int c = 0; c < 3; ++c)
      a.psi_i[k][c] = (d1[k] * x11 + d2[k] * x21) * v1[c] + (d1[k] * x12 + d2[k] * x22) * v2[c];
}

static void hbie_edges(const Elem& e, const HbieAt& a, HbieLi& L) {
  L.zero();
  QsParams qsp;
  qs_calculate_parameters(1e-15, qsp);
  for (int ke = 0; ke < 4; ++ke) {
    double xe[3][3];
    for (int q = 0; q < 3; ++q)
      for (int c = 0; c < 3; ++c) xe[q][c] = e.x[quad8_edge_node[ke][q]][c];
    double xs[2];
    hbie_int_li(xe, xs, a.x_i, a.n_i, 5, qsp, 1, 16, L);
  }
}

static void hbie_int(const StaelaHK& k, const Elem& e, bool reverse, const double xi_i[2], HG<StaelaHK>& out) {
  out.zero();
  if (check_xi1xi2_edge_quad(xi_i)) {
    g_hbie_err = 1;
    return;
  }
  HbieAt a;
  hbie_at(e, xi_i, a);
  const double nu = k.nu, cted2 = k.cted2, ctes2 = k.ctes2, ctes3 = k.ctes3;
  const double* ni = a.n_i;
  int nsub, st[8];
  auto fn = [&](const double*, const double rv[3], const double n[3], const double phi[8], double jw) {
    double r = std::sqrt(rv[0] * rv[0] + rv[1] * rv[1] + rv[2] * rv[2]);
    double d1r = 1.0 / r, d1r2 = d1r * d1r, d1r3 = d1r2 * d1r;
    double drdx[3] = {rv[0] * d1r, rv[1] * d1r, rv[2] * d1r};
    double drdn = drdx[0] * n[0] + drdx[1] * n[1] + drdx[2] * n[2];
    double drdni = -(drdx[0] * ni[0] + drdx[1] * ni[1] + drdx[2] * ni[2]);
    double nni = n[0] * ni[0] + n[1] * ni[1] + n[2] * ni[2];
    double pj[8], reg[8], psn[8];
    for (int q = 0; q < 8; ++q) {
      pj[q] = phi[q] * jw;
      reg[q] = phi[q] - a.phi_i[q] - a.psi_i[q][0] * rv[0] - a.psi_i[q][1] * rv[1] - a.psi_i[q][2] * rv[2];
      psn[q] = a.psi_i[q][0] * n[0] + a.psi_i[q][1] * n[1] + a.psi_i[q][2] * n[2];
    }
    for (int il = 0; il < 3; ++il)
      for (int ik = 0; ik < 3; ++ik) {
        double dk = (il == ik) ? 1.0 : 0.0;
        // L1
        double fd = d1r2 * ((cted2 * dk + 3.0 * drdx[il] * drdx[ik]) * drdni +
                            cted2 * ((ni[il] - n[il]) * drdx[ik] - (ni[ik] - n[ik]) * drdx[il]));
        for (int q = 0; q < 8; ++q) out.g[q][il][ik] = out.g[q][il][ik] + fd * pj[q];
        // L21
        if (il != ik) {
          fd = d1r2 * cted2 * (n[il] * drdx[ik] - n[ik] * drdx[il]);
          for (int q = 0; q < 8; ++q) out.g[q][il][ik] = out.g[q][il][ik] + fd * (phi[q] - a.phi_i[q]) * jw;
        }
        // M1
        double fs = 3.0 * d1r3 * drdn * drdni * (5.0 * drdx[il] * drdx[ik] - nu * dk);
        for (int q = 0; q < 8; ++q) out.h[q][il][ik] = out.h[q][il][ik] + fs * pj[q];
        if (il == ik) {
          // M21, M221, M231
          fs = ctes2 * d1r3 * nni;
          for (int q = 0; q < 8; ++q) out.h[q][il][ik] = out.h[q][il][ik] + fs * reg[q] * jw;
          fs = -ctes2 * 3.0 * d1r3 * drdn * drdni;
          for (int q = 0; q < 8; ++q) out.h[q][il][ik] = out.h[q][il][ik] + a.phi_i[q] * fs * jw;
          fs = -ctes2 * d1r2 * drdni;
          for (int q = 0; q < 8; ++q) out.h[q][il][ik] = out.h[q][il][ik] + fs * psn[q] * jw;
        }
        // M31
        fs = d1r3 * (3.0 * ctes2 * (drdx[ik] * ni[il] * drdn - drdx[il] * n[ik] * drdni) +
                     3.0 * nu * (drdx[il] * ni[ik] * drdn - drdx[ik] * n[il] * drdni) +
                     3.0 * nu * drdx[il] * drdx[ik] * nni + ctes2 * ni[ik] * n[il] - ctes3 * ni[il] * n[ik]);
        for (int q = 0; q < 8; ++q) out.h[q][il][ik] = out.h[q][il][ik] + fs * reg[q] * jw;
        // M321
        fs = d1r3 * (-15.0 * nu * drdx[il] * drdx[ik] * drdn * drdni +
                     3.0 * nu * drdx[ik] * (ni[il] * drdn - n[il] * drdni) +
                     3.0 * ctes2 * drdx[il] * (ni[ik] * drdn - n[ik] * drdni));
        for (int q = 0; q < 8; ++q) out.h[q][il][ik] = out.h[q][il][ik] + a.phi_i[q] * fs * jw;
        // M331
        for (int ij = 0; ij < 3; ++ij) {
          double djk = (ij == ik) ? 1.0 : 0.0;
          fs = d1r2 * (drdx[ij] * (3.0 * ctes2 * (drdx[ik] * ni[il] * drdn - drdx[il] * n[ik] * drdni) +
                                   3.0 * nu * (drdx[il] * ni[ik] * drdn - drdx[ik] * n[il] * drdni) -
                                   3.0 * nu * drdx[il] * n[ik] * drdni) -
                       ((1.0 - 3.0 * nu) * ni[il] * drdx[ij] + nu * ni[ij] * drdx[il]) * (n[ik] - ni[ik] * nni) +
                       ctes2 * ni[ik] * drdx[ij] * (n[il] - ni[il] * nni) -
                       nu * (dk + ni[il] * ni[ik]) * n[ij] * drdni - nu * (djk - ni[ij] * ni[ik]) * n[il] * drdni);
          for (int q = 0; q < 8; ++q) out.h[q][il][ik] = out.h[q][il][ik] + a.psi_i[q][ij] * fs * jw;
        }
      }
  };
  polar_loop<StaelaHK>(e, xi_i, a.x_i, fn, &nsub, st);
  HbieLi L;
  hbie_edges(e, a, L);
  for (int il = 0; il < 3; ++il)
    for (int ik = 0; ik < 3; ++ik) {
      double dk = (il == ik) ? 1.0 : 0.0;
      for (int q = 0; q < 8; ++q) {
        const double ph = a.phi_i[q];
        const double* ps = a.psi_i[q];
        out.g[q][il][ik] = out.g[q][il][ik] + ph * cted2 * L.lli[il][ik];  // L22
        double v = out.h[q][il][ik];
        if (il == ik) {
          v = v + ph * ctes2 * L.mli1;                                  // M222
          for (int ij = 0; ij < 3; ++ij) v = v + ps[ij] * ctes2 * L.mli2[ij];  // M232
        }
        v = v + ph * 3.0 * nu * L.mli3[il][ik];          // M322
        v = v + ph * ctes2 * ni[ik] * L.mli4[il];        // M323
        v = v - ph * ctes3 * ni[il] * L.mli4[ik];        // M324
        for (int ij = 0; ij < 3; ++ij) {
          double djk = (ij == ik) ? 1.0 : 0.0;
          v = v + ps[ij] * nu * L.mli5[ij][il][ik];                               // M332
          v = v + ps[ij] * nu * (dk + ni[il] * ni[ik]) * L.mli2[ij];              // M333
          v = v + ps[ij] * nu * (djk - ni[ij] * ni[ik]) * L.mli2[il];             // M334
        }
        out.h[q][il][ik] = v;
      }
    }
  for (int q = 0; q < 8; ++q)
    for (int il = 0; il < 3; ++il)
      for (int ik = 0; ik < 3; ++ik) {
        out.h[q][il][ik] = k.ctes1 * out.h[q][il][ik];
        out.g[q][il][ik] = k.cted1 * out.g[q][il][ik];
        if (reverse) out.g[q][il][ik] = -out.g[q][il][ik];
      }
}

static void hbie_int(const HarelaHK& k, const Elem& e, bool reverse, const double xi_i[2], HG<HarelaHK>& out) {
  out.zero();
  if (check_xi1xi2_edge_quad(xi_i)) {
    g_hbie_err = 1;
    return;
  }
  HbieAt a;
  hbie_at(e, xi_i, a);
  const HarPar& p = k.p;
  const double* ni = a.n_i;
  const cplx I(0.0, 1.0);
  const cplx S1o3 = p.S1[0] / 3.0;
  int nsub, st[8];
  auto fn = [&](const double*, const double rv[3], const double n[3], const double phi[8], double jw) {
    double r = std::sqrt(rv[0] * rv[0] + rv[1] * rv[1] + rv[2] * rv[2]);
    double dr1 = 1.0 / r, dr2 = dr1 * dr1, dr3 = dr2 * dr1, dr4 = dr3 * dr1, dr5 = dr4 * dr1;
    double drdx[3] = {rv[0] * dr1, rv[1] * dr1, rv[2] * dr1};
    double drdn = drdx[0] * n[0] + drdx[1] * n[1] + drdx[2] * n[2];
    double drdni = -(drdx[0] * ni[0] + drdx[1] * ni[1] + drdx[2] * ni[2]);
    double nni = n[0] * ni[0] + n[1] * ni[1] + n[2] * ni[2];
    double pj[8], reg[8], psn[8];
    for (int q = 0; q < 8; ++q) {
      pj[q] = phi[q] * jw;
      reg[q] = phi[q] - a.phi_i[q] - a.psi_i[q][0] * rv[0] - a.psi_i[q][1] * rv[1] - a.psi_i[q][2] * rv[2];
      psn[q] = a.psi_i[q][0] * n[0] + a.psi_i[q][1] * n[1] + a.psi_i[q][2] * n[2];
    }
    cplx z[2] = {-I * p.k1 * r, -I * p.k2 * r};
    cplx E[7][2];
    zexp_decomposed(2, z, E);
    for (int j = 0; j < 2; ++j) {
      E[2][j] = E[2][j] * dr1;
      E[3][j] = E[3][j] * dr2;
      E[4][j] = E[4][j] * dr3;
      E[5][j] = E[5][j] * dr4;
      E[6][j] = E[6][j] * dr5;
    }
    // regular parts only (the 1/r^2 and 1/r^3 terms are regularised below)
    cplx TT1 = p.T1[1] + p.T1[2] * E[2][0] + p.T1[3] * E[2][1] + p.T1[4] * E[3][0] + p.T1[5] * E[3][1] +
               p.T1[6] * E[4][0] + p.T1[7] * E[4][1] + p.T1[8] * E[5][0] + p.T1[9] * E[5][1];
    cplx TT2 = p.T2[1] + p.T2[2] * E[2][1] + p.T2[3] * E[3][0] + p.T2[4] * E[3][1] + p.T2[5] * E[4][0] +
               p.T2[6] * E[4][1] + p.T2[7] * E[5][0] + p.T2[8] * E[5][1];
    cplx TT3 = p.T3[1] + p.T3[2] * E[2][0] + p.T3[3] * E[3][0] + p.T3[4] * E[3][1] + p.T3[5] * E[4][0] +
               p.T3[6] * E[4][1] + p.T3[7] * E[5][0] + p.T3[8] * E[5][1];
    cplx S1 = p.S1[1] * dr1 + p.S1[2] * E[2][1] + p.S1[3] * E[3][0] + p.S1[4] * E[3][1] + p.S1[5] * E[4][0] +
              p.S1[6] * E[4][1] + p.S1[7] * E[5][0] + p.S1[8] * E[5][1] + p.S1[9] * E[6][0] + p.S1[10] * E[6][1];
    cplx S2 = p.S2[1] * dr1 + p.S2[2] * E[2][0] + p.S2[3] * E[3][0] + p.S2[4] * E[3][1] + p.S2[5] * E[4][0] +
              p.S2[6] * E[4][1] + p.S2[7] * E[5][0] + p.S2[8] * E[5][1] + p.S2[9] * E[6][0] + p.S2[10] * E[6][1];
    cplx S3 = p.S3[1] * dr1 + p.S3[2] * E[2][0] + p.S3[3] * E[2][1] + p.S3[4] * E[3][0] + p.S3[5] * E[3][1] +
              p.S3[6] * E[4][0] + p.S3[7] * E[4][1] + p.S3[8] * E[5][0] + p.S3[9] * E[5][1] + p.S3[10] * E[6][0] +
              p.S3[11] * E[6][1];
    cplx S4 = p.S4[1] * dr1 + p.S4[2] + p.S4[3] * E[3][1] + p.S4[4] * E[4][0] + p.S4[5] * E[4][1] +
              p.S4[6] * E[5][0] + p.S4[7] * E[5][1] + p.S4[8] * E[6][0] + p.S4[9] * E[6][1];
    cplx S5 = p.S5[1] * dr1 + p.S5[2] + p.S5[3] * E[2][0] + p.S5[4] * E[3][0] + p.S5[5] * E[4][0] +
              p.S5[6] * E[4][1] + p.S5[7] * E[5][0] + p.S5[8] * E[5][1] + p.S5[9] * E[6][0] + p.S5[10] * E[6][1];
    for (int il = 0; il < 3; ++il)
      for (int ik = 0; ik < 3; ++ik) {
        double dk = (il == ik) ? 1.0 : 0.0;
        cplx fd = (TT1 + p.T1[0] * dr2) * drdx[il] * drdx[ik] * drdni + (TT2 + p.T2[0] * dr2) * dk * drdni -
                  TT2 * drdx[il] * ni[ik] - TT3 * drdx[ik] * ni[il] +
                  p.T2[0] * dr2 * ((ni[il] - n[il]) * drdx[ik] - (ni[ik] - n[ik]) * drdx[il]);
        cplx fs = S1 * (drdx[il] * ni[ik] * drdn - drdx[ik] * n[il] * drdni - dk * drdn * drdni +
                        drdx[il] * drdx[ik] * nni) +
                  S2 * (drdx[ik] * ni[il] * drdn - drdx[il] * n[ik] * drdni) + S3 * drdx[il] * drdx[ik] * drdn * drdni +
                  S4 * (dk * nni + ni[ik] * n[il]) + S5 * n[ik] * ni[il] - dk * p.S1[0] * dr3 * drdn * drdni +
                  p.S3[0] * dr3 * drdx[il] * drdx[ik] * drdn * drdni;
        for (int q = 0; q < 8; ++q) {
          out.h[q][il][ik] = out.h[q][il][ik] + fs * pj[q];
          out.g[q][il][ik] = out.g[q][il][ik] + fd * pj[q];
        }
        // L21
        if (il != ik) {
          fd = p.T2[0] * dr2 * (n[il] * drdx[ik] - n[ik] * drdx[il]);
          for (int q = 0; q < 8; ++q) out.g[q][il][ik] = out.g[q][il][ik] + fd * (phi[q] - a.phi_i[q]) * jw;
        }
        if (il == ik) {
          // M21, M221, M231
          fs = p.S4[0] * dr3 * nni;
          for (int q = 0; q < 8; ++q) out.h[q][il][ik] = out.h[q][il][ik] + fs * reg[q] * jw;
          fs = -p.S4[0] * 3.0 * dr3 * drdn * drdni;
          for (int q = 0; q < 8; ++q) out.h[q][il][ik] = out.h[q][il][ik] + a.phi_i[q] * fs * jw;
          fs = -p.S4[0] * dr2 * drdni;
          for (int q = 0; q < 8; ++q) out.h[q][il][ik] = out.h[q][il][ik] + fs * psn[q] * jw;
        }
        // M31
        fs = dr3 * (p.S2[0] * (drdx[ik] * ni[il] * drdn - drdx[il] * n[ik] * drdni) +
                    p.S1[0] * (drdx[il] * ni[ik] * drdn - drdx[ik] * n[il] * drdni) +
                    p.S1[0] * drdx[il] * drdx[ik] * nni + p.S4[0] * ni[ik] * n[il] + p.S5[0] * ni[il] * n[ik]);
        for (int q = 0; q < 8; ++q) out.h[q][il][ik] = out.h[q][il][ik] + fs * reg[q] * jw;
        // M321
        fs = dr3 * (-5.0 * p.S1[0] * drdx[il] * drdx[ik] * drdn * drdni +
                    p.S1[0] * drdx[ik] * (ni[il] * drdn - n[il] * drdni) +
                    p.S2[0] * drdx[il] * (ni[ik] * drdn - n[ik] * drdni));
        for (int q = 0; q < 8; ++q) out.h[q][il][ik] = out.h[q][il][ik] + a.phi_i[q] * fs * jw;
        // M331
        for (int ij = 0; ij < 3; ++ij) {
          double djk = (ij == ik) ? 1.0 : 0.0;
          fs = dr2 * (drdx[ij] * (p.S2[0] * (drdx[ik] * ni[il] * drdn - drdx[il] * n[ik] * drdni) +
                                  p.S1[0] * (drdx[il] * ni[ik] * drdn - drdx[ik] * n[il] * drdni) -
                                  p.S1[0] * drdx[il] * n[ik] * drdni) -
                      ((S1o3 - p.S5[0]) * ni[il] * drdx[ij] + S1o3 * ni[ij] * drdx[il]) * (n[ik] - ni[ik] * nni) +
                      p.S4[0] * ni[ik] * drdx[ij] * (n[il] - ni[il] * nni) -
                      S1o3 * (dk + ni[il] * ni[ik]) * n[ij] * drdni - S1o3 * (djk - ni[ij] * ni[ik]) * n[il] * drdni);
          for (int q = 0; q < 8; ++q) out.h[q][il][ik] = out.h[q][il][ik] + a.psi_i[q][ij] * fs * jw;
        }
      }
  };
  polar_loop<HarelaHK>(e, xi_i, a.x_i, fn, &nsub, st);
  HbieLi L;
  hbie_edges(e, a, L);
  for (int il = 0; il < 3; ++il)
    for (int ik = 0; ik < 3; ++ik) {
      double dk = (il == ik) ? 1.0 : 0.0;
      for (int q = 0; q < 8; ++q) {
        const double ph = a.phi_i[q];
        const double* ps = a.psi_i[q];
        out.g[q][il][ik] = out.g[q][il][ik] + ph * p.T2[0] * L.lli[il][ik];  // L22
        cplx v = out.h[q][il][ik];
        if (il == ik) {
          v = v + ph * p.S4[0] * L.mli1;                                     // M222
          for (int ij = 0; ij < 3; ++ij) v = v + ps[ij] * p.S4[0] * L.mli2[ij];  // M232
        }
        v = v + ph * p.S1[0] * L.mli3[il][ik];          // M322
        v = v + ph * p.S4[0] * ni[ik] * L.mli4[il];     // M323
        v = v + ph * p.S5[0] * ni[il] * L.mli4[ik];     // M324
        for (int ij = 0; ij < 3; ++ij) {
          double djk = (ij == ik) ? 1.0 : 0.0;
          v = v + ps[ij] * S1o3 * L.mli5[ij][il][ik];                    // M332
          v = v + ps[ij] * S1o3 * (dk + ni[il] * ni[ik]) * L.mli2[ij];   // M333
          v = v + ps[ij] * S1o3 * (djk - ni[ij] * ni[ik]) * L.mli2[il];  // M334
        }
        out.h[q][il][ik] = v;
      }
    }
  for (int q = 0; q < 8; ++q)
    for (int il = 0; il < 3; ++il)
      for (int ik = 0; ik < 3; ++ik) {
        out.h[q][il][ik] = p.cte_s * out.h[q][il][ik];
        out.g[q][il][ik] = p.cte_d * out.g[q][il][ik];
        if (reverse) out.g[q][il][ik] = -out.g[q][il][ik];
      }
}

// hbie_auto (bem_staela3d.f90:4307-4373 / bem_harela3d.f90:3632-3697): the
// classification of sbie_auto with the 1/r^7 estimate. A point on the element
// (d <= 1e-12) takes the interior integration when `interior` is set (HBIE
// collocation on the boundary); internal points pass false and get zero
// kernels with CLS_SING, which they report.
template <class K>
static int hbie_auto(const K& k, const Elem& e, bool reverse, const double x_i[3], const QsParams& qsp, int ns,
                     HG<K>& out, bool interior = false, AdpStats* st = nullptr) {
  double r[3] = {e.bc[0] - x_i[0], e.bc[1] - x_i[1], e.bc[2] - x_i[2]};
  double rmin = std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]) - e.br;
  double barxi[2] = {0.0, 0.0}, d;
  if (rmin > 4.0 * e.br) {
    d = rmin / e.cl;
  } else {
    int method;
    nearest_element_point_quad8(e.x, e.cl, x_i, barxi, &rmin, &d, &method);
    if (d <= 1e-12) {
      if (interior) hbie_int(k, e, reverse, barxi, out);
      else out.zero();
      return CLS_SING;
    }
  }
  int gln_near = qs_n_estimation_standard(2, K::F, qsp, d, barxi);
  int gln = std::max(e.gln_far, gln_near);
  if (gln <= e.ps_gln_max && gln_near > 0) {
    int ps = 0;
    for (int i = 0; i < e.n_ps; ++i)
      if (e.ps_gln[i] >= gln) { ps = i; break; }
    ext_pre<K>(k, ps, e, reverse, x_i, out);
    return ps;
  }
  double xi_s[4][2];
  ext_adp<K>(k, e, reverse, xi_s, x_i, qsp, 1, ns, out, st);
  return CLS_ADP;
}

// fbem_bem_harela3d_shbie_auto (bem_harela3d.f90:4888-4957): SBIE and HBIE
// kernels at one collocation point, classified once with the HBIE's 1/r^7
// estimate: interior integration of both, one precalculated rule for both
// (shbie_ext_pre, bem_harela3d.f90:4781-4886), or each kernel's own adaptive
// subdivision.
static int shbie_auto(const HarelaK& k, const HarelaHK& kh, const Elem& e, bool reverse, const double x_i[3],
                      const QsParams& qsp, int ns, HG<HarelaK>& hg, HG<HarelaHK>& ml, AdpStats* st) {
  double r[3] = {e.bc[0] - x_i[0], e.bc[1] - x_i[1], e.bc[2] - x_i[2]};
  double rmin = std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]) - e.br;
  double barxi[2] = {0.0, 0.0}, d;
  if (rmin > 4.0 * e.br) {
    d = rmin / e.cl;
  } else {
    int method;
    nearest_element_point_quad8(e.x, e.cl, x_i, barxi, &rmin, &d, &method);
    if (d <= 1e-12) {
      sbie_int<HarelaK>(k, e, reverse, barxi, hg);
      hbie_int(kh, e, reverse, barxi, ml);
      return CLS_SING;
    }
  }
  int gln_near = qs_n_estimation_standard(2, HarelaHK::F, qsp, d, barxi);
  int gln = std::max(e.gln_far, gln_near);
  if (gln <= e.ps_gln_max && gln_near > 0) {
    int ps = 0;
    for (int i = 0; i < e.n_ps; ++i)
      if (e.ps_gln[i] >= gln) { ps = i; break; }
    ext_pre<HarelaK>(k, ps, e, reverse, x_i, hg);
    ext_pre<HarelaHK>(kh, ps, e, reverse, x_i, ml);
    return ps;
  }
  double xi_s[4][2];
  ext_adp<HarelaK>(k, e, reverse, xi_s, x_i, qsp, 1, ns, hg, st);
  ext_adp<HarelaHK>(kh, e, reverse, xi_s, x_i, qsp, 1, ns, ml, st);
  return CLS_ADP;
}

// ---------------------------------------------------------------------------
// Half-space complementary kernel (static): the part of Mindlin's fundamental
// solution for the half-space x3 >= xp with a traction-free surface x3 = xp
// (outward unit normal (0, 0, -1)) that is added to Kelvin's full-space
// solution. fbem_bem_staela3d_hsc_sbie, bem_staela3d.f90:7438-7563, with its
// constants applied per point. As written there, the image point is
// (x_i1, x_i2, -x_i3) (the reflection in x3 = 0) while c and z are measured
// from x3 = xp: both agree for the plane x3 = 0. u[il][ik], t[il][ik]: load
// direction il, observed component ik.
// ---------------------------------------------------------------------------
static thread_local int g_hs_err = 0;  // 1: a point below the free surface; 2: a singular element off it

struct HscK {
  typedef double T;
  static constexpr int F = 5;
  double mu, nu, xp;
  HscK(double mu_, double nu_, double xp_) : mu(mu_), nu(nu_), xp(xp_) {}
  double cu() const { return 1.0; }
  double ct() const { return 1.0; }
  void eval_at(const double x[3], const double x_i[3], const double n[3], double u[3][3], double t[3][3]) const {
    if (x_i[2] < xp || x[2] < xp) g_hs_err = 1;
    const double c1 = 1.0 - nu, c2 = 1.0 - 2.0 * nu, c3 = 3.0 - 2.0 * nu, c4 = 3.0 - 4.0 * nu, c5 = 5.0 - 4.0 * nu;
    const double c = x_i[2] - xp, z = x[2] - xp;
    const double rv[3] = {x[0] - x_i[0], x[1] - x_i[1], x[2] - x_i[2]};
    const double r = std::sqrt(rv[0] * rv[0] + rv[1] * rv[1]);
    const double rpv[3] = {x[0] - x_i[0], x[1] - x_i[1], x[2] + x_i[2]};
    const double rp = std::sqrt(rpv[0] * rpv[0] + rpv[1] * rpv[1] + rpv[2] * rpv[2]);
    const double rp2 = rp * rp, rp3 = rp2 * rp, rp5 = rp3 * rp2, rp7 = rp5 * rp2;
    const double zc = z + c, q = rp + z + c;
    const double r1 = rv[0] * rv[0], r2 = rv[1] * rv[1];
    // load along the normal, local cylindrical axes (r, theta, x3)
    double un[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, sn[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    un[2][0] = r * (c4 * (z - c) / rp3 - 4.0 * c1 * c2 / rp / q + 6.0 * c * z * zc / rp5);
    un[2][2] = (8.0 * (c1 * c1) - c4) / rp + (c4 * (zc * zc) - 2.0 * c * z) / rp3 + 6.0 * c * z * (zc * zc) / rp5;
    sn[0][0] = -c2 * (z + 7.0 * c) / rp3 + 4.0 * c1 * c2 / rp / q +
               (6.0 * c * c2 * (zc * zc) - 6.0 * (c * c) * zc - 3.0 * c4 * (r * r) * (z - c)) / rp5 -
               30.0 * c * (r * r) * z * zc / rp7;
    sn[0][2] = r * (c2 / rp3 - (3.0 * c4 * z * zc - 3.0 * c * (3.0 * z + c)) / rp5 - 30.0 * c * z * (zc * zc) / rp7);
    sn[2][0] = sn[0][2];
    sn[1][1] = c2 * (c4 * zc - 6.0 * c) / rp3 - 4.0 * c1 * c2 / rp / q + 6.0 * c2 * c * (zc * zc) / rp5 -
               6.0 * (c * c) * zc / rp5;
    sn[2][2] = c2 * (z - c) / rp3 - (3.0 * c4 * z * (zc * zc) - 3.0 * c * zc * (5.0 * z - c)) / rp5 -
               30.0 * c * z * (zc * zc * zc) / rp7;
    // to global axes: L (.) L^T with L the rotation by theta about x3
    const double th = std::atan2(x[1] - x_i[1], x[0] - x_i[0]);
    const double L[3][3] = {{std::cos(th), -std::sin(th), 0.0}, {std::sin(th), std::cos(th), 0.0}, {0.0, 0.0, 1.0}};
    auto rot = [&](double a[3][3]) {
      double tmp[3][3], out[3][3];
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
          double v = 0.0;
          for (int k = 0; k < 3; ++k) v = v + a[i][k] * L[j][k];
          tmp[i][j] = v;
        }
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
          double v = 0.0;
          for (int k = 0; k < 3; ++k) v = v + L[i][k] * tmp[k][j];
          out[i][j] = v;
        }
      std::memcpy(a, out, sizeof(out));
    };
    rot(un);
    rot(sn);
    // loads tangent to the surface, global axes
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) u[i][j] = 0.0;
    const double q2 = q * q;
    u[0][0] = 1.0 / rp + c4 * r1 / rp3 + 2.0 * c * z / rp3 * (1.0 - 3.0 * r1 / rp2) + 4.0 * c1 * c2 / q * (1.0 - r1 / rp / q);
    u[0][1] = rv[0] * rv[1] * (c4 / rp3 - 6.0 * c * z / rp5 - 4.0 * c1 * c2 / rp / q2);
    u[0][2] = rv[0] * (c4 * (z - c) / rp3 - 6.0 * c * z * zc / rp5 + 4.0 * c1 * c2 / rp / q);
    u[1][0] = rv[0] * rv[1] * (c4 / rp3 - 6.0 * c * z / rp5 - 4.0 * c1 * c2 / rp / q2);
    u[1][1] = 1.0 / rp + c4 * r2 / rp3 + 2.0 * c * z / rp3 * (1.0 - 3.0 * r2 / rp2) + 4.0 * c1 * c2 / q * (1.0 - r2 / rp / q);
    u[1][2] = rv[1] * (c4 * (z - c) / rp3 - 6.0 * c * z * zc / rp5 + 4.0 * c1 * c2 / rp / q);
    double sg[3][3][3];  // sg[i][j][k]: stress ij of the load along k
    std::memset(sg, 0, sizeof(sg));
    const double b1 = 3.0 * rp + z + c;
    sg[0][0][0] = rv[0] * (c2 * c5 / rp3 - 3.0 * c4 * r1 / rp5 - 4.0 * c1 * c2 / rp / q2 * (3.0 - r1 * b1 / rp2 / q) +
                           6.0 * c / rp5 * (3.0 * c - c3 * zc + 5.0 * r1 * z / rp2));
    sg[1][1][0] = rv[0] * (c2 * c4 / rp3 - 3.0 * c4 * r2 / rp5 - 4.0 * c1 * c2 / rp / q2 * (1.0 - r2 * b1 / rp2 / q) +
                           6.0 * c / rp5 * (c - c2 * zc + 5.0 * r2 * z / rp2));
    sg[2][2][0] = rv[0] * (-c2 / rp3 - 3.0 * c4 * (zc * zc) / rp5 + 6.0 * c / rp5 * (c + c2 * zc + 5.0 * z * (zc * zc) / rp2));
    sg[1][2][0] = rv[0] * rv[1] * (-3.0 * c4 * zc / rp5 + 6.0 * c / rp5 * (c2 + 5.0 * z * zc / rp2));
    sg[2][0][0] = c2 * (z - c) / rp3 - 3.0 * c4 * r1 * zc / rp5 - 6.0 * c / rp5 * (z * zc - c2 * r1 - 5.0 * r1 * z * zc / rp2);
    sg[0][1][0] = rv[1] * (c2 / rp3 - 3.0 * c4 * r1 / rp5 - 4.0 * c1 * c2 / rp / q2 * (1.0 - r1 * b1 / rp2 / q) -
                           6.0 * c * z / rp5 * (1.0 - 5.0 * r1 / rp2));
    sg[2][1][0] = sg[1][2][0];
    sg[0][2][0] = sg[2][0][0];
    sg[1][0][0] = sg[0][1][0];
    sg[0][0][1] = rv[1] * (c2 * c4 / rp3 - 3.0 * c4 * r1 / rp5 - 4.0 * c1 * c2 / rp / q2 * (1.0 - r1 * b1 / rp2 / q) +
                           6.0 * c / rp5 * (c - c2 * zc + 5.0 * r1 * z / rp2));
    sg[1][1][1] = rv[1] * (c2 * c5 / rp3 - 3.0 * c4 * r2 / rp5 - 4.0 * c1 * c2 / rp / q2 * (3.0 - r2 * b1 / rp2 / q) +
                           6.0 * c / rp5 * (3.0 * c - c3 * zc + 5.0 * r2 * z / rp2));
    sg[2][2][1] = rv[1] * (-c2 / rp3 - 3.0 * c4 * (zc * zc) / rp5 + 6.0 * c / rp5 * (c + c2 * zc + 5.0 * z * (zc * zc) / rp2));
    sg[0][2][1] = rv[0] * rv[1] * (-3.0 * c4 * zc / rp5 + 6.0 * c / rp5 * (c2 + 5.0 * z * zc / rp2));
    sg[2][1][1] = c2 * (z - c) / rp3 - 3.0 * c4 * r2 * zc / rp5 - 6.0 * c / rp5 * (z * zc - c2 * r2 - 5.0 * r2 * z * zc / rp2);
    sg[1][0][1] = rv[0] * (c2 / rp3 - 3.0 * c4 * r2 / rp5 - 4.0 * c1 * c2 / rp / q2 * (1.0 - r2 * b1 / rp2 / q) -
                           6.0 * c * z / rp5 * (1.0 - 5.0 * r2 / rp2));
    sg[2][0][1] = sg[0][2][1];
    sg[1][2][1] = sg[2][1][1];
    sg[0][1][1] = sg[1][0][1];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) sg[i][j][2] = sn[i][j];
    const double cu_ = 16.0 * c_pi * c1 * mu, cs_ = 8.0 * c_pi * c1;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) u[i][j] = (u[i][j] + un[i][j]) / cu_;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j)
        for (int k = 0; k < 3; ++k) sg[i][j][k] = sg[i][j][k] / cs_;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) t[i][j] = sg[j][0][i] * n[0] + sg[j][1][i] * n[1] + sg[j][2][i] * n[2];
  }
};
inline void kernel_at(const HscK& k, const double x[3], const double x_i[3], const double n[3], double fu[3][3],
                      double ft[3][3]) {
  k.eval_at(x, x_i, n, fu, ft);
}

// ---------------------------------------------------------------------------
// Complementary HBIE kernels d*, s* of the half-space (static) at an internal
// point: fbem_bem_staela3d_hsc_hbie (bem_staela3d.f90:10882-11102) builds them
// from the first and mixed second derivatives of the complementary u* with
// respect to the field point x and the source point x_i. Here those
// derivatives come from forward-mode differentiation (a jet carrying the value,
// the gradients in x and x_i and the mixed Hessian block) of u* written in
// Cartesian form, then the same steps: sigma* = C : grad_x u*, its x_i
// derivative, d*_lkp / s*_lkp = C applied to the x_i gradients, contracted with
// n_i. z and z_i are measured from the plane x3 = xp, R the distance to the
// image (x_i1, x_i2, 2 xp - x_i3).
// ---------------------------------------------------------------------------
struct Jet {
  double v, gx[3], gi[3], H[3][3];  // value, d/dx, d/dx_i, d2/(dx_j dx_i_p)
};
static inline Jet jconst(double c) {
  Jet r{};
  r.v = c;
  return r;
}
static inline Jet operator+(const Jet& a, const Jet& b) {
  Jet r;
  r.v = a.v + b.v;
  for (int j = 0; j < 3; ++j) {
    r.gx[j] = a.gx[j] + b.gx[j];
    r.gi[j] = a.gi[j] + b.gi[j];
    for (int p = 0; p < 3; ++p) r.H[j][p] = a.H[j][p] + b.H[j][p];
  }
  return r;
}
static inline Jet operator*(double c, const Jet& a) {
  Jet r;
  r.v = c * a.v;
  for (int j = 0; j < 3; ++j) {
    r.gx[j] = c * a.gx[j];
    r.gi[j] = c * a.gi[j];
    for (int p = 0; p < 3; ++p) r.H[j][p] = c * a.H[j][p];
  }
  return r;
}
static inline Jet operator-(const Jet& a, const Jet& b) { return a + (-1.0) * b; }
static inline Jet operator+(const Jet& a, double c) { Jet r = a; r.v = r.v + c; return r; }
static inline Jet operator*(const Jet& a, const Jet& b) {
  Jet r;
  r.v = a.v * b.v;
  for (int j = 0; j < 3; ++j) {
    r.gx[j] = a.v * b.gx[j] + a.gx[j] * b.v;
    r.gi[j] = a.v * b.gi[j] + a.gi[j] * b.v;
  }
  for (int j = 0; j < 3; ++j)
    for (int p = 0; p < 3; ++p)
      r.H[j][p] = a.v * b.H[j][p] + a.H[j][p] * b.v + a.gx[j] * b.gi[p] + a.gi[p] * b.gx[j];
  return r;
}
// g(a) for a scalar function with derivatives d1 = g'(a.v), d2 = g''(a.v)
static inline Jet jchain(const Jet& a, double g, double d1, double d2) {
  Jet r;
  r.v = g;
  for (int j = 0; j < 3; ++j) {
    r.gx[j] = d1 * a.gx[j];
    r.gi[j] = d1 * a.gi[j];
  }
  for (int j = 0; j < 3; ++j)
    for (int p = 0; p < 3; ++p) r.H[j][p] = d1 * a.H[j][p] + d2 * a.gx[j] * a.gi[p];
  return r;
}
static inline Jet jinv(const Jet& a) { const double q = 1.0 / a.v; return jchain(a, q, -q * q, 2.0 * q * q * q); }
static inline Jet jsqrt(const Jet& a) {
  const double s = std::sqrt(a.v);
  return jchain(a, s, 0.5 / s, -0.25 / (s * a.v));
}

// Complementary u*[l][k] (load direction l, component k, without the factor
// 1 / (16 pi mu (1 - nu))) in Cartesian form: the tangential-load rows of
// hsc_sbie (bem_staela3d.f90:7438-7563) and the normal-load row with the
// radial component r F written as (x - x_i) F.
static void hsc_u_jets(double nu, const Jet x[3], const Jet xi[3], double xp, Jet u[3][3]) {
  const double c1 = 1.0 - nu, c2 = 1.0 - 2.0 * nu, c4 = 3.0 - 4.0 * nu;
  const Jet rx = x[0] - xi[0], ry = x[1] - xi[1];
  const Jet z = x[2] + (-xp), c = xi[2] + (-xp), zc = z + c;
  const Jet rp = jsqrt(rx * rx + ry * ry + zc * zc);
  const Jet irp = jinv(rp), irp2 = irp * irp, irp3 = irp2 * irp, irp5 = irp3 * irp2;
  const Jet q = rp + zc, iq = jinv(q), iq2 = iq * iq;
  const Jet cz = c * z;
  const double k12 = 4.0 * c1 * c2;
  const Jet rr[2] = {rx, ry};
  for (int a = 0; a < 2; ++a) {
    const Jet ra2 = rr[a] * rr[a];
    u[a][a] = irp + (c4 * ra2) * irp3 + (2.0 * cz) * irp3 * (jconst(1.0) - (3.0 * ra2) * irp2) +
              (k12 * iq) * (jconst(1.0) - ra2 * irp * iq);
    u[a][2] = rr[a] * ((c4 * (z - c)) * irp3 - (6.0 * cz * zc) * irp5 + (k12 * irp) * iq);
    u[2][a] = rr[a] * ((c4 * (z - c)) * irp3 - (k12 * irp) * iq + (6.0 * cz * zc) * irp5);
  }
  u[0][1] = rx * ry * (c4 * irp3 - (6.0 * cz) * irp5 - (k12 * irp) * iq2);
  u[1][0] = u[0][1];
  u[2][2] = (8.0 * c1 * c1 - c4) * irp + (c4 * zc * zc - 2.0 * cz) * irp3 + (6.0 * cz * zc * zc) * irp5;
}

struct HscHK {
  typedef double T;
  static constexpr int F = 7;
  double mu, nu, xp, ni[3];
  HscHK(double mu_, double nu_, double xp_, const double n_i[3]) : mu(mu_), nu(nu_), xp(xp_) {
    for (int c = 0; c < 3; ++c) ni[c] = n_i[c];
  }
  double cu() const { return 1.0; }
  double ct() const { return 1.0; }
  // fd = d*, fs = s* (load direction il, component ik), constants included
  void eval_at(const double xq[3], const double x_i[3], const double n[3], double fd[3][3], double fs[3][3]) const {
    if (x_i[2] < xp || xq[2] < xp) g_hs_err = 1;
    Jet x[3], xi[3];
    for (int c = 0; c < 3; ++c) {
      x[c] = jconst(xq[c]);
      x[c].gx[c] = 1.0;
      xi[c] = jconst(x_i[c]);
      xi[c].gi[c] = 1.0;
    }
    Jet u[3][3];
    hsc_u_jets(nu, x, xi, xp, u);
    const double Ku = 1.0 / (16.0 * c_pi * mu * (1.0 - nu)), lam = 2.0 * mu * nu / (1.0 - 2.0 * nu);
    // d/dx_i of t* = sigma*(x) n with sigma*_{l,kj} = lam d_kj div u_l + mu (u_lk,j + u_lj,k)
    double dt[3][3][3];  // dt[l][k][p]
    for (int l = 0; l < 3; ++l)
      for (int k = 0; k < 3; ++k)
        for (int p = 0; p < 3; ++p) {
          double div = 0.0;
          for (int m = 0; m < 3; ++m) div = div + u[l][m].H[m][p];
          double v = 0.0;
          for (int j = 0; j < 3; ++j) {
            double sg = mu * (u[l][k].H[j][p] + u[l][j].H[k][p]);
            if (j == k) sg = sg + lam * div;
            v = v + sg * n[j];
          }
          dt[l][k][p] = Ku * v;
        }
    for (int l = 0; l < 3; ++l)
      for (int k = 0; k < 3; ++k) {
        double dv = 0.0, sv = 0.0;
        for (int p = 0; p < 3; ++p) {
          double dl = mu * Ku * (u[l][k].gi[p] + u[p][k].gi[l]);
          double sl = mu * (dt[l][k][p] + dt[p][k][l]);
          if (l == p) {
            double tr = 0.0, ts = 0.0;
            for (int j = 0; j < 3; ++j) {
              tr = tr + u[j][k].gi[j];
              ts = ts + dt[j][k][j];
            }
            dl = dl + lam * Ku * tr;
            sl = sl + lam * ts;
          }
          dv = dv + dl * ni[p];
          sv = sv + sl * ni[p];
        }
        fd[l][k] = dv;
        fs[l][k] = sv;
      }
  }
};
inline void kernel_at(const HscHK& k, const double x[3], const double x_i[3], const double n[3], double fu[3][3],
                      double ft[3][3]) {
  k.eval_at(x, x_i, n, fu, ft);
}

// fbem_bem_staela3d_hsc_sbie_int (bem_staela3d.f90:8624-8833): element on the
// free surface containing the collocation point. h is minus the full-space h
// (the complete traction kernel vanishes on the free surface); g integrates
// the complementary displacement kernel restricted to the surface with the
// same polar rule as the full-space singular integration.
static void hsc_int(const StaelaK& kf, const HscK& k, const Elem& e, bool reverse, const double xi_i[2], HG<HscK>& out) {
  out.zero();
  for (int q = 0; q < 8; ++q)
    if (std::fabs(e.x[q][2] - k.xp) > 1e-12) g_hs_err = 2;
  HG<StaelaK> full;
  sbie_int<StaelaK>(kf, e, reverse, xi_i, full);
  for (int a = 0; a < 8; ++a)
    for (int il = 0; il < 3; ++il)
      for (int ik = 0; ik < 3; ++ik) out.h[a][il][ik] = -full.h[a][il][ik];
  double phii[8];
  phi_quad8(xi_i, phii);
  double x_i[3] = {0, 0, 0};
  for (int q = 0; q < 8; ++q)
    for (int c = 0; c < 3; ++c) x_i[c] = x_i[c] + phii[q] * e.x[q][c];
  const double nu = k.nu, xp = k.xp;
  auto fn = [&](const double* x, const double rv[3], const double*, const double phi[8], double jw) {
    double r = std::sqrt(rv[0] * rv[0] + rv[1] * rv[1] + rv[2] * rv[2]);
    double d1r = 1.0 / r;
    double dr[3] = {rv[0] * d1r, rv[1] * d1r, rv[2] * d1r};
    const double a = 3.0 - 4.0 * nu, b = 4.0 * (1.0 - nu) * (1.0 - 2.0 * nu), s = r + x[2] - xp;
    double gk[3][3];
    gk[0][0] = d1r + a * (dr[0] * dr[0]) * d1r + b / s * (1.0 - (dr[0] * dr[0]) * r / s);
    gk[0][1] = a * dr[0] * dr[1] * d1r - b * dr[0] * dr[1] * r / (s * s);
    gk[0][2] = a * dr[0] * dr[2] * d1r + b * dr[0] / s;
    gk[1][0] = a * dr[0] * dr[1] * d1r - b * dr[0] * dr[1] * r / (s * s);
    gk[1][1] = d1r + a * (dr[1] * dr[1]) * d1r + b / s * (1.0 - (dr[1] * dr[1]) * r / s);
    gk[1][2] = a * dr[1] * dr[2] * d1r + b * dr[1] / s;
    gk[2][0] = a * dr[0] * dr[2] * d1r - b * dr[0] / s;
    gk[2][1] = a * dr[1] * dr[2] * d1r - b * dr[1] / s;
    gk[2][2] = (8.0 * ((1.0 - nu) * (1.0 - nu)) - a) * d1r + a * (dr[2] * dr[2]) * d1r;
    for (int il = 0; il < 3; ++il)
      for (int ik = 0; ik < 3; ++ik)
        for (int q = 0; q < 8; ++q) out.g[q][il][ik] = out.g[q][il][ik] + gk[il][ik] * (phi[q] * jw);
  };
  int nsub, st[8];
  polar_loop<HscK>(e, xi_i, x_i, fn, &nsub, st);
  const double cg = 16.0 * c_pi * k.mu * (1.0 - nu);
  for (int q = 0; q < 8; ++q)
    for (int il = 0; il < 3; ++il)
      for (int ik = 0; ik < 3; ++ik) out.g[q][il][ik] = out.g[q][il][ik] / cg;
}

// fbem_bem_staela3d_hsc_sbie_auto (bem_staela3d.f90:9047-9118): sbie_auto's
// classification on the image of the collocation point in the free surface,
// the kernel evaluated at the collocation point itself.
static int hsc_auto(const StaelaK& kf, const HscK& k, const Elem& e, bool reverse, const double x_i[3],
                    const QsParams& qsp, int ns, HG<HscK>& out, AdpStats* st) {
  const double xq[3] = {x_i[0], x_i[1], 2.0 * k.xp - x_i[2]};
  double r[3] = {e.bc[0] - xq[0], e.bc[1] - xq[1], e.bc[2] - xq[2]};
  double rmin = std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]) - e.br;
  double barxi[2], d;
  int delta;
  if (rmin > 4.0 * e.br) {
    delta = 0;
    barxi[0] = barxi[1] = 0.0;
    d = rmin / e.cl;
  } else {
    int method;
    nearest_element_point_quad8(e.x, e.cl, xq, barxi, &rmin, &d, &method);
    delta = (d <= 1e-12) ? 1 : 0;
  }
  if (delta == 1) {
    hsc_int(kf, k, e, reverse, barxi, out);
    return CLS_SING;
  }
  int gln_near = qs_n_estimation_standard(2, HscK::F, qsp, d, barxi);
  int gln = std::max(e.gln_far, gln_near);
  if (gln <= e.ps_gln_max && gln_near > 0) {
    int ps = 0;
    for (int i = 0; i < e.n_ps; ++i)
      if (e.ps_gln[i] >= gln) { ps = i; break; }
    ext_pre<HscK>(k, ps, e, reverse, x_i, out);
    return ps;
  }
  double xi_s[4][2];
  ext_adp<HscK>(k, e, reverse, xi_s, x_i, qsp, 1, ns, out, st, xq);
  return CLS_ADP;
}

// fbem_bem_staela3d_hsc_hbie_auto (bem_staela3d.f90:11573-11645): hbie_auto's
// classification (1/r^7 estimate) on the image of the point; a point on an
// element of the free surface (image on the element) cannot be integrated
// (the reference stops): g_hs_err = 2.
static int hsc_hbie_auto(const HscHK& k, const Elem& e, bool reverse, const double x_i[3], const QsParams& qsp,
                         int ns, HG<HscHK>& out, AdpStats* st) {
  const double xq[3] = {x_i[0], x_i[1], 2.0 * k.xp - x_i[2]};
  double r[3] = {e.bc[0] - xq[0], e.bc[1] - xq[1], e.bc[2] - xq[2]};
  double rmin = std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]) - e.br;
  double barxi[2], d;
  if (rmin > 4.0 * e.br) {
    barxi[0] = barxi[1] = 0.0;
    d = rmin / e.cl;
  } else {
    int method;
    nearest_element_point_quad8(e.x, e.cl, xq, barxi, &rmin, &d, &method);
    if (d <= 1e-12) {
      g_hs_err = 2;
      out.zero();
      return CLS_SING;
    }
  }
  int gln_near = qs_n_estimation_standard(2, HscHK::F, qsp, d, barxi);
  int gln = std::max(e.gln_far, gln_near);
  if (gln <= e.ps_gln_max && gln_near > 0) {
    int ps = 0;
    for (int i = 0; i < e.n_ps; ++i)
      if (e.ps_gln[i] >= gln) { ps = i; break; }
    ext_pre<HscHK>(k, ps, e, reverse, x_i, out);
    return ps;
  }
  double xi_s[4][2];
  ext_adp<HscHK>(k, e, reverse, xi_s, x_i, qsp, 1, ns, out, st, xq);
  return CLS_ADP;
}

// ---------------------------------------------------------------------------
// Free term: V. Mantic's formula, bem_staela3d.f90:228-405 (real nu) and
// bem_harela3d.f90:365-542 (complex nu): identical algorithm.
// Returns false when the normals/tangents configuration is invalid (the
// reference stops there).
// ---------------------------------------------------------------------------
template <typename T>
static bool freeterm(int ne, const double* n, const double* t, double tol, T nu, T c[3][3]) {
  double ltol = (tol < 1e-12 || tol > 1e-3) ? 1e-6 : tol;
  std::vector<double> ln(3 * (ne + 2)), lt(3 * (ne + 2)), lti(3 * ne);
  auto LN = [&](int k, int c) -> double& { return ln[3 * k + c]; };
  auto LT = [&](int k, int c) -> double& { return lt[3 * k + c]; };
  for (int ki = 1; ki <= ne; ++ki)
    for (int c = 0; c < 3; ++c) { LN(ki, c) = n[3 * (ki - 1) + c]; LT(ki, c) = t[3 * (ki - 1) + c]; }
  std::vector<int> tc(ne + 1);
  std::vector<double> theta(ne + 1);
  for (int ki = 1; ki <= ne - 1; ++ki) {
    double e1[3] = {LT(ki, 0), LT(ki, 1), LT(ki, 2)}, e3[3] = {LN(ki, 0), LN(ki, 1), LN(ki, 2)};
    double e2[3] = {e3[1] * e1[2] - e3[2] * e1[1], e3[2] * e1[0] - e3[0] * e1[2], e3[0] * e1[1] - e3[1] * e1[0]};
    for (int kj = 1; kj <= ne; ++kj) {
      lti[3 * (kj - 1) + 0] = e1[0] * LT(kj, 0) + e1[1] * LT(kj, 1) + e1[2] * LT(kj, 2);
      lti[3 * (kj - 1) + 1] = e2[0] * LT(kj, 0) + e2[1] * LT(kj, 1) + e2[2] * LT(kj, 2);
      lti[3 * (kj - 1) + 2] = e3[0] * LT(kj, 0) + e3[1] * LT(kj, 1) + e3[2] * LT(kj, 2);
    }
    int nc = 0;
    for (int kj = ki + 1; kj <= ne; ++kj)
      if (std::fabs(lti[3 * (kj - 1) + 2]) <= ltol) tc[++nc] = kj;
    if (nc == 0) return false;
    for (int kj = 1; kj <= nc; ++kj) {
      int j = tc[kj];
      theta[j] = std::atan2(lti[3 * (j - 1) + 1], lti[3 * (j - 1) + 0]);
      if (theta[j] < 0.0) theta[j] = theta[j] + 2.0 * c_pi;
    }
    double mt = theta[tc[1]];
    int mk = tc[1];
    for (int kj = 2; kj <= nc; ++kj)
      if (theta[tc[kj]] < mt) { mt = theta[tc[kj]]; mk = tc[kj]; }
    for (int c = 0; c < 3; ++c) {
      std::swap(LT(ki + 1, c), LT(mk, c));
      std::swap(LN(ki + 1, c), LN(mk, c));
    }
  }
  for (int c = 0; c < 3; ++c) {
    LN(0, c) = LN(ne, c); LT(0, c) = LT(ne, c);
    LN(ne + 1, c) = LN(1, c); LT(ne + 1, c) = LT(1, c);
  }
  double sum_a = 0.0;
  for (int ki = 1; ki <= ne; ++ki) {
    double nx[3] = {LN(ki - 1, 1) * LN(ki, 2) - LN(ki - 1, 2) * LN(ki, 1),
                    LN(ki - 1, 2) * LN(ki, 0) - LN(ki - 1, 0) * LN(ki, 2),
                    LN(ki - 1, 0) * LN(ki, 1) - LN(ki - 1, 1) * LN(ki, 0)};
    double s = nx[0] * LT(ki, 0) + nx[1] * LT(ki, 1) + nx[2] * LT(ki, 2);
    if (s < 0.0) s = -1.0;
    if (s > 0.0) s = 1.0;
    double ndn = LN(ki - 1, 0) * LN(ki, 0) + LN(ki - 1, 1) * LN(ki, 1) + LN(ki - 1, 2) * LN(ki, 2);
    if (ndn > 1.0) ndn = 1.0;
    sum_a = sum_a + s * std::acos(ndn);
  }
  double cp = 1.0 / (4.0 * c_pi) * (2.0 * c_pi + sum_a);
  double sb[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  for (int ki = 1; ki <= ne; ++ki) {
    double rmr[3] = {LT(ki + 1, 0) - LT(ki, 0), LT(ki + 1, 1) - LT(ki, 1), LT(ki + 1, 2) - LT(ki, 2)};
    double rx[3] = {rmr[1] * LN(ki, 2) - rmr[2] * LN(ki, 1), rmr[2] * LN(ki, 0) - rmr[0] * LN(ki, 2),
                    rmr[0] * LN(ki, 1) - rmr[1] * LN(ki, 0)};
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) sb[a][b] = sb[a][b] + rx[a] * LN(ki, b);
  }
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b) {
      c[a][b] = -1.0 / (8.0 * c_pi * (1.0 - nu)) * sb[a][b];
      if (a == b) c[a][b] = c[a][b] + cp;
    }
  return true;
}

// ---------------------------------------------------------------------------
// Problem: the host-side data the Fortran keeps in problem_variables for one
// ordinary BE boundary of continuous quad8 elements in a full-space region.
// ---------------------------------------------------------------------------
struct Colloc {
  double x[3];
  int node;     // collocation node (rows)
  int kind;     // 0 SBIE (nodal), 1 SBIE MCA, 2 HBIE, 3 SBIE + HBIE (Burton & Miller) at one point,
                // 4 SBIE and HBIE of a crack-like node, 5 the HBIE part of 'dual_bm_mixed'
                // (beta alpha HBIE at its own point; the node's SBIE at its kind 0 / 1 point)
  int elem, kn; // element/local node it was taken from
  double xi[2];
  double n[3];  // unit normal at xi (HBIE kinds)
};

struct Problem {
  int nn, ne;
  std::vector<double> X;     // 3*nn
  std::vector<int> conn;     // 8*ne
  std::vector<int> ctype;    // 3*nn
  std::vector<cplx> cvalue;  // 3*nn
  double qsi_re, geo_tol;
  int ns_max, n_ps;
  int ps_gln[16];
  QsParams qsp;
  std::vector<Elem> el;
  std::vector<int> node_order;                   // DOF order
  std::vector<int> dof;                          // nn*3 -> 0-based DOF index
  std::vector<std::vector<std::pair<int, int>>> node_el;  // (element, local)
  std::vector<char> in_boundary;
  std::vector<double> delta_mca;                 // 8*ne
  std::vector<double> n_gn, tbp_gn, tbm_gn;      // 8*ne*3
  std::vector<Colloc> cps;
  std::vector<std::vector<int>> node_cps;        // collocation points per node
  int ndof;
  // region space (read_regions.f90:130-200): hs_n = 0 full space, else the
  // half-space with hyperplane normal hs_n (+-1..3), coordinate hs_x and
  // boundary condition hs_bc (1: traction-free surface)
  int hs_n = 0, hs_bc = 1;
  double hs_x = 0.0;
  // BEM formulation per node (src/read_bem_formulation_selected_nodes.f90:
  // 70-260, ordinary boundary of continuous elements): 0 the default SBIE
  // (assign_default_bem_formulation.f90:76-93), 1 'hbie' (HBIE alone at
  // non-nodal points), 2 'dual_bm_same' (SBIE and HBIE at the same non-nodal
  // point, Burton & Miller combination with weight alpha); delta_hbie moves
  // the point into each element of the node
  std::vector<int> form;
  std::vector<double> alpha, delta_hbie;
  // crack-like boundary (src/read_boundaries.f90:105): its elements, and
  // their nodes with two faces (build_auxiliary_variables_mechanics_static.f90:
  // 150-181): face 2's boundary conditions and DOF (dof2: the face-2 column,
  // equal to the row of the node's second (HBIE) equation)
  std::vector<char> crack_el, crack;
  std::vector<int> ctype2, dof2;
  std::vector<cplx> cvalue2;
};

static void build(Problem& P) {
  const int nn = P.nn, ne = P.ne;
  P.el.resize(ne);
  for (int e = 0; e < ne; ++e) {
    Elem& E = P.el[e];
    for (int k = 0; k < 8; ++k)
      for (int c = 0; c < 3; ++c) E.x[k][c] = P.X[3 * P.conn[8 * e + k] + c];
    // build_data_of_be_elements.f90:52-96
    E.cl = characteristic_length_quad8(E.x, 1e-9);
    bool ok;
    int n1 = qs_phijac_ngp_2d_quad8(E.x, P.qsi_re, &ok);
    int n2 = qs_phijac_ngp_2d_quad8(E.x, P.qsi_re, &ok);
    E.gln_far = std::max(n1, n2);
    element_ball_quad8(E.x, E.gln_far, E.bc, &E.br);
    init_precalculated(E, P.n_ps, P.ps_gln);
  }
  // node -> elements (increasing element order)
  P.node_el.assign(nn, {});
  for (int e = 0; e < ne; ++e)
    for (int k = 0; k < 8; ++k) P.node_el[P.conn[8 * e + k]].push_back({e, k});
  // mesh boundary (data_structures.f90:1433-1495): edges with one element
  std::map<std::pair<int, int>, int> edge_count;
  for (int e = 0; e < ne; ++e)
    for (int ke = 0; ke < 4; ++ke) {
      int a = P.conn[8 * e + quad8_edge_node[ke][0]], b = P.conn[8 * e + quad8_edge_node[ke][1]];
      edge_count[{std::min(a, b), std::max(a, b)}]++;
    }
  P.in_boundary.assign(nn, 0);
  for (int e = 0; e < ne; ++e)
    for (int ke = 0; ke < 4; ++ke) {
      int a = P.conn[8 * e + quad8_edge_node[ke][0]], b = P.conn[8 * e + quad8_edge_node[ke][1]];
      if (edge_count[{std::min(a, b), std::max(a, b)}] == 1)
        for (int q = 0; q < 3; ++q) P.in_boundary[P.conn[8 * e + quad8_edge_node[ke][q]]] = 1;
    }
  // assign_default_bem_formulation.f90:76-93
  P.delta_mca.assign(8 * ne, 0.0);
  for (int s = 0; s < nn; ++s)
    if (P.in_boundary[s])
      for (auto& pr : P.node_el[s]) P.delta_mca[8 * pr.first + pr.second] = 0.05;
  // geometrical node normals/tangents (build_data_at_geometrical_nodes.f90:177-222)
  P.n_gn.assign(8 * ne * 3, 0.0);
  P.tbp_gn.assign(8 * ne * 3, 0.0);
  P.tbm_gn.assign(8 * ne * 3, 0.0);
  for (int e = 0; e < ne; ++e)
    for (int k = 0; k < 8; ++k) {
      double d1[8], d2[8];
      dphi_quad8(quad8_xi_nodes[k], d1, d2);
      double T1[3] = {0, 0, 0}, T2[3] = {0, 0, 0};
      for (int i = 0; i < 8; ++i)
        for (int c = 0; c < 3; ++c) { T1[c] = T1[c] + d1[i] * P.el[e].x[i][c]; T2[c] = T2[c] + d2[i] * P.el[e].x[i][c]; }
      double N[3] = {T1[1] * T2[2] - T1[2] * T2[1], T1[2] * T2[0] - T1[0] * T2[2], T1[0] * T2[1] - T1[1] * T2[0]};
      double tmp = std::sqrt(N[0] * N[0] + N[1] * N[1] + N[2] * N[2]);
      for (int c = 0; c < 3; ++c) P.n_gn[(8 * e + k) * 3 + c] = N[c] / tmp;
      double n1 = std::sqrt(T1[0] * T1[0] + T1[1] * T1[1] + T1[2] * T1[2]);
      double n2 = std::sqrt(T2[0] * T2[0] + T2[1] * T2[1] + T2[2] * T2[2]);
      double t1[3] = {T1[0] / n1, T1[1] / n1, T1[2] / n1}, t2[3] = {T2[0] / n2, T2[1] / n2, T2[2] / n2};
      // geometry.f90:833-873 quadrilateral branch
      static const int sp[8][2] = {{1, 2}, {2, -1}, {-1, -2}, {-2, 1}, {1, -1}, {2, -2}, {-1, 1}, {-2, 2}};
      for (int c = 0; c < 3; ++c) {
        int a = sp[k][0], b = sp[k][1];
        double va = (std::abs(a) == 1 ? t1[c] : t2[c]) * (a > 0 ? 1.0 : -1.0);
        double vb = (std::abs(b) == 1 ? t1[c] : t2[c]) * (b > 0 ? 1.0 : -1.0);
        P.tbp_gn[(8 * e + k) * 3 + c] = va;
        P.tbm_gn[(8 * e + k) * 3 + c] = vb;
      }
    }
  P.form.assign(nn, 0);
  P.alpha.assign(nn, 1.0);
  P.delta_hbie.assign(nn, 0.22540333);
  P.crack_el.assign(ne, 0);
  P.crack.assign(nn, 0);
  P.ctype2.assign(3 * nn, 1);
  P.cvalue2.assign(3 * nn, cplx(0.0, 0.0));
}

// DOF numbering, build_auxiliary_variables_mechanics_static.f90:60-181: nodes
// in element order (first appearance); an ordinary node takes rows / columns
// r, r+1, r+2; a node of a crack-like boundary r..r+5 with row(k, eq) =
// r + 2k + eq - 1 and col(k, face) = r + 2k + face - 1.
static void build_dofs(Problem& P) {
  const int nn = P.nn, ne = P.ne;
  P.dof.assign(3 * nn, -1);
  P.dof2.assign(3 * nn, -1);
  P.node_order.clear();
  std::vector<char> used(nn, 0);
  int row = 0;
  for (int e = 0; e < ne; ++e)
    for (int k = 0; k < 8; ++k) {
      int s = P.conn[8 * e + k];
      if (used[s]) continue;
      used[s] = 1;
      P.node_order.push_back(s);
      if (P.crack[s]) {
        for (int c = 0; c < 3; ++c) {
          P.dof[3 * s + c] = row + 2 * c;
          P.dof2[3 * s + c] = row + 2 * c + 1;
        }
        row += 6;
      } else {
        for (int c = 0; c < 3; ++c) P.dof[3 * s + c] = row++;
      }
    }
  P.ndof = row;
}

// Collocation points in the collocation loop order
// (build_lse_mechanics_bem_staela.f90:761-1034): per element and local node,
// the node's nodal SBIE point (once), SBIE-MCA point or HBIE point. HBIE
// points: xi moved from the element edge by delta_hbie
// (src/build_data_at_collocation_points.f90:148-160) and the unit normal there
// (:368-376).
// HBIE point of element e's local node k: xi moved from the edge by dl
// (fbem_move_xi1xi2_from_edge), x there and the element's unit normal.
static void hbie_point(const Problem& P, int e, int k, double dl, Colloc& cp) {
  double xi[2] = {quad8_xi_nodes[k][0], quad8_xi_nodes[k][1]};
  if (check_xi1xi2_edge_quad(xi)) { xi[0] = xi[0] * (1.0 - dl); xi[1] = xi[1] * (1.0 - dl); }
  double d1[8], d2[8], phi[8];
  dphi_quad8(xi, d1, d2);
  phi_quad8(xi, phi);
  double T1[3] = {0, 0, 0}, T2[3] = {0, 0, 0}, x[3] = {0, 0, 0};
  for (int q = 0; q < 8; ++q)
    for (int c = 0; c < 3; ++c) {
      T1[c] = T1[c] + d1[q] * P.el[e].x[q][c];
      T2[c] = T2[c] + d2[q] * P.el[e].x[q][c];
      x[c] = x[c] + phi[q] * P.el[e].x[q][c];
    }
  double N[3] = {T1[1] * T2[2] - T1[2] * T2[1], T1[2] * T2[0] - T1[0] * T2[2], T1[0] * T2[1] - T1[1] * T2[0]};
  double jn = std::sqrt(N[0] * N[0] + N[1] * N[1] + N[2] * N[2]);
  for (int c = 0; c < 3; ++c) {
    cp.n[c] = N[c] / jn;
    cp.x[c] = x[c];
  }
  cp.xi[0] = xi[0];
  cp.xi[1] = xi[1];
}

static void build_colloc(Problem& P) {
  const int nn = P.nn, ne = P.ne;
  P.cps.clear();
  std::vector<char> coll(nn, 0);
  P.node_cps.assign(nn, {});
  for (int e = 0; e < ne; ++e)
    for (int k = 0; k < 8; ++k) {
      int s = P.conn[8 * e + k];
      Colloc cp;
      cp.node = s; cp.elem = e; cp.kn = k;
      cp.n[0] = cp.n[1] = cp.n[2] = 0.0;
      double xi[2] = {quad8_xi_nodes[k][0], quad8_xi_nodes[k][1]};
      if (P.form[s] == 3 && !P.crack[s]) {
        // 'dual_bm_mixed': the HBIE at its own point of this element (kind 5,
        // weight beta alpha), the SBIE at the node's usual point below
        // (src/read_bem_formulation_selected_nodes.f90:243-295)
        Colloc hb = cp;
        hb.kind = 5;
        hbie_point(P, e, k, P.delta_hbie[s], hb);
        P.node_cps[s].push_back((int)P.cps.size());
        P.cps.push_back(hb);
      }
      if ((P.form[s] != 0 && P.form[s] != 3) || P.crack[s]) {
        // crack-like nodes: SBIE and HBIE at the same MCA point, each its own
        // equation (dual BEM, assign_default_bem_formulation.f90:94-128)
        double dl = P.delta_hbie[s];
        if (check_xi1xi2_edge_quad(xi)) { xi[0] = xi[0] * (1.0 - dl); xi[1] = xi[1] * (1.0 - dl); }
        cp.kind = P.crack[s] ? 4 : (P.form[s] == 1 ? 2 : 3);
        double d1[8], d2[8];
        dphi_quad8(xi, d1, d2);
        double T1[3] = {0, 0, 0}, T2[3] = {0, 0, 0};
        for (int q = 0; q < 8; ++q)
          for (int c = 0; c < 3; ++c) {
            T1[c] = T1[c] + d1[q] * P.el[e].x[q][c];
            T2[c] = T2[c] + d2[q] * P.el[e].x[q][c];
          }
        double N[3] = {T1[1] * T2[2] - T1[2] * T2[1], T1[2] * T2[0] - T1[0] * T2[2], T1[0] * T2[1] - T1[1] * T2[0]};
        double jn = std::sqrt(N[0] * N[0] + N[1] * N[1] + N[2] * N[2]);
        for (int c = 0; c < 3; ++c) cp.n[c] = N[c] / jn;
      } else if (!P.in_boundary[s]) {
        if (coll[s]) continue;
        coll[s] = 1;
        cp.kind = 0;
      } else {
        // fbem_move_xi1xi2_from_edge (geometry.f90:5631-5659)
        double dl = P.delta_mca[8 * e + k];
        if (check_xi1xi2_edge_quad(xi)) { xi[0] = xi[0] * (1.0 - dl); xi[1] = xi[1] * (1.0 - dl); }
        cp.kind = 1;
      }
      cp.xi[0] = xi[0]; cp.xi[1] = xi[1];
      double phi[8];
      phi_quad8(xi, phi);
      double x[3] = {0, 0, 0};
      for (int q = 0; q < 8; ++q)
        for (int c = 0; c < 3; ++c) x[c] = x[c] + phi[q] * P.el[e].x[q][c];
      for (int c = 0; c < 3; ++c) cp.x[c] = x[c];
      P.node_cps[s].push_back((int)P.cps.size());
      P.cps.push_back(cp);
    }
}

// Scatter one (collocation point, integration element) block into the row
// buffer of one equation of the point's node: assemble_bem_staela_equation.f90:
// 69-124 and assemble_bem_harela_equation.f90:78-150. Face 1 of the element's
// nodes takes (hp, gp); on a crack-like element face 2 takes (hm, gm) too.
template <typename T>
static void scatter4(const Problem& P, int e, const T hp[8][3][3], const T gp[8][3][3], const T hm[8][3][3],
                     const T gm[8][3][3], T* rowbuf /*3*ndof*/, T* brow /*3*/) {
  auto val = [](const cplx& v) -> T {
    if constexpr (std::is_same<T, double>::value) return v.real();
    else return v;
  };
  const bool ck = P.crack_el[e] != 0;
  for (int il = 0; il < 3; ++il)
    for (int ik = 0; ik < 3; ++ik)
      for (int kn = 0; kn < 8; ++kn) {
        int s = P.conn[8 * e + kn];
        int col = P.dof[3 * s + ik];
        T cv = val(P.cvalue[3 * s + ik]);
        if (P.ctype[3 * s + ik] == 0) {
          rowbuf[il * P.ndof + col] = rowbuf[il * P.ndof + col] - gp[kn][il][ik];
          brow[il] = brow[il] - hp[kn][il][ik] * cv;
        } else {
          rowbuf[il * P.ndof + col] = rowbuf[il * P.ndof + col] + hp[kn][il][ik];
          brow[il] = brow[il] + gp[kn][il][ik] * cv;
        }
        if (ck) {
          int col2 = P.dof2[3 * s + ik];
          T cv2 = val(P.cvalue2[3 * s + ik]);
          if (P.ctype2[3 * s + ik] == 0) {
            rowbuf[il * P.ndof + col2] = rowbuf[il * P.ndof + col2] - gm[kn][il][ik];
            brow[il] = brow[il] - hm[kn][il][ik] * cv2;
          } else {
            rowbuf[il * P.ndof + col2] = rowbuf[il * P.ndof + col2] + hm[kn][il][ik];
            brow[il] = brow[il] + gm[kn][il][ik] * cv2;
          }
        }
      }
}
// integration kernels: face 2 of a crack-like element sees the reversed
// normal, hm = -h, gm = g (build_lse_mechanics_bem_staela.f90:883-887)
template <typename T>
static void scatter(const Problem& P, int e, const T h[8][3][3], const T g[8][3][3], T* rowbuf, T* brow) {
  if (!P.crack_el[e]) {
    scatter4<T>(P, e, h, g, h, g, rowbuf, brow);
    return;
  }
  T hm[8][3][3];
  for (int a = 0; a < 8; ++a)
    for (int il = 0; il < 3; ++il)
      for (int ik = 0; ik < 3; ++ik) hm[a][il][ik] = -h[a][il][ik];
  scatter4<T>(P, e, h, g, hm, g, rowbuf, brow);
}

// Free-term contribution for collocation node s (first element of the
// collocation order carries it), build_lse_mechanics_bem_staela.f90:152-549.
template <class K>
static bool free_terms_for_node(const Problem& P, int s, typename K::T nu, typename K::T beta, typename K::T* rowbuf,
                                typename K::T* brow, typename K::T* rowbuf2, typename K::T* brow2) {
  typedef typename K::T T;
  for (int ci : P.node_cps[s]) {
    const Colloc& cp = P.cps[ci];
    HG<K> hg;
    hg.zero();
    if (cp.kind == 4) {
      // crack-like point (dual BEM): SBIE equation 1/2 phi on both faces' u,
      // HBIE equation -1/2 phi on face 1's t, +1/2 phi on face 2's t
      // (build_lse_mechanics_bem_staela.f90:181-204)
      double pphi[8];
      phi_quad8(cp.xi, pphi);
      HG<K> z, l1, l2;
      z.zero();
      l1.zero();
      l2.zero();
      for (int il = 0; il < 3; ++il)
        for (int a = 0; a < 8; ++a) {
          hg.h[a][il][il] = 0.5 * pphi[a];
          l1.g[a][il][il] = -0.5 * pphi[a];
          l2.g[a][il][il] = 0.5 * pphi[a];
        }
      scatter4<T>(P, cp.elem, hg.h, z.g, hg.h, z.g, rowbuf, brow);
      scatter4<T>(P, cp.elem, z.h, l1.g, z.h, l2.g, rowbuf2, brow2);
      continue;
    }
    if (cp.kind == 0) {
      int nce = (int)P.node_el[s].size();
      std::vector<double> nset(3 * nce), tset(3 * nce);
      for (int j = 0; j < nce; ++j) {
        int e = P.node_el[s][j].first, k = P.node_el[s][j].second;
        for (int c = 0; c < 3; ++c) {
          nset[3 * j + c] = P.n_gn[(8 * e + k) * 3 + c];
          tset[3 * j + c] = P.tbp_gn[(8 * e + k) * 3 + c];
        }
      }
      T C[3][3];
      if (!freeterm<T>(nce, nset.data(), tset.data(), P.geo_tol, nu, C)) return false;
      for (int il = 0; il < 3; ++il)
        for (int ik = 0; ik < 3; ++ik) hg.h[cp.kn][il][ik] = hg.h[cp.kn][il][ik] + C[il][ik];
    } else {
      double pphi[8];
      phi_quad8(cp.xi, pphi);
      // SBIE at a non-nodal point: 1/2 phi(xi_i) on h; HBIE: -1/2 phi(xi_i) on
      // l, which is g ('hbie', dual = 0) or weighted by beta into g (Burton &
      // Miller) (build_lse_mechanics_bem_staela.f90:181-211,440-489,
      // build_lse_mechanics_bem_harela.f90:316-360,598-681)
      if (cp.kind != 2 && cp.kind != 5)
        for (int il = 0; il < 3; ++il)
          for (int a = 0; a < 8; ++a) hg.h[a][il][il] = hg.h[a][il][il] + 0.5 * pphi[a];
      if (cp.kind >= 2) {
        const T w = cp.kind == 2 ? (T)1.0 : beta * P.alpha[s];
        for (int il = 0; il < 3; ++il)
          for (int a = 0; a < 8; ++a) hg.g[a][il][il] = hg.g[a][il][il] + w * (-0.5 * pphi[a]);
      }
    }
    // half-space with a traction-free surface: a collocation point on the
    // surface takes twice the free term (build_lse_mechanics_bem_staela.f90:502-513,
    // build_lse_mechanics_bem_harela.f90:688-697)
    if (P.hs_n != 0) {
      const int ax = std::abs(P.hs_n) - 1;
      if (cp.x[ax] - P.hs_x <= 1e-12 / P.el[cp.elem].cl && P.hs_bc == 1)
        for (int a = 0; a < 8; ++a)
          for (int il = 0; il < 3; ++il)
            for (int ik = 0; ik < 3; ++ik) hg.h[a][il][ik] = 2.0 * hg.h[a][il][ik];
    }
    scatter<T>(P, cp.elem, hg.h, hg.g, rowbuf, brow);
  }
  return true;
}

// The region builder's collocation loop for one BE region. mkh(n_i) makes the
// HBIE kernel at a point with unit normal n_i; bm is the Burton & Miller
// factor besides the node's alpha: 1 static (h + alpha m,
// build_lse_mechanics_bem_staela.f90:835-841), i / c2 harmonic with c2 the
// complex S-wave speed (h + alpha i / c2 m, build_lse_mechanics_bem_harela.f90:
// 1174-1181). stats: [0..2] SBIE precalculated / adaptive / singular pairs,
// [3] adaptive leaves, [4] their points, [5] maximum-depth hits, [6..7]
// complementary adaptive / singular pairs, [8..10] HBIE precalculated /
// adaptive / singular pairs.
template <class K, class KH, class MKH>
static int assemble(const Problem& P, const K& k, MKH mkh, typename K::T bm, typename K::T nu, typename K::T* A,
                    typename K::T* b, int nthreads, long* stats) {
  typedef typename K::T T;
  constexpr bool kHarmonic = std::is_same<K, HarelaK>::value;
  const int n = P.ndof;
  int nord = (int)P.node_order.size();
  int bad = 0;
  bool has_hbie = false;
  for (int f : P.form) has_hbie = has_hbie || f != 0;
  for (char c : P.crack) has_hbie = has_hbie || c != 0;
  if (has_hbie && P.hs_n != 0) return -5;
  long s_leaves = 0, s_points = 0, s_maxd = 0, s_sing = 0, s_adp = 0, s_pre = 0, s_hsing = 0, s_hadp = 0;
  long s_bpre = 0, s_badp = 0, s_bsing = 0;
  int hs_err = 0, hb_err = 0;
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel reduction(+ : bad, s_leaves, s_points, s_maxd, s_sing, s_adp, s_pre, s_hsing, s_hadp, s_bpre, \
                               s_badp, s_bsing) reduction(max : hs_err, hb_err)
  {
    g_hs_err = 0;
    g_hbie_err = 0;
    std::vector<T> rowbuf(3 * (size_t)n), rowbuf2;
    AdpStats st;
    auto count = [&](int cls, long& sing, long& adp, long& pre) {
      if (cls == CLS_SING) sing++;
      else if (cls == CLS_ADP) adp++;
      else pre++;
    };
#pragma omp for schedule(dynamic, 1)
    for (int oi = 0; oi < nord; ++oi) {
      int s = P.node_order[oi];
      std::fill(rowbuf.begin(), rowbuf.end(), (T)0);
      if (P.crack[s]) rowbuf2.assign(3 * (size_t)n, (T)0);
      T brow[3] = {(T)0, (T)0, (T)0}, brow2[3] = {(T)0, (T)0, (T)0};
      for (int e = 0; e < P.ne; ++e) {
        for (int ci : P.node_cps[s]) {
          const Colloc& cp = P.cps[ci];
          HG<K> hg;
          if (cp.kind == 4) {
            // dual BEM: the SBIE into the node's first equation, the HBIE into
            // its second, each with both faces of a crack-like element
            // (build_lse_mechanics_bem_staela.f90:783-830,1000-1010)
            KH kh = mkh(cp.n);
            HG<KH> ml;
            if constexpr (kHarmonic) {
              int c = shbie_auto(k, kh, P.el[e], false, cp.x, P.qsp, P.ns_max, hg, ml, &st);
              count(c, s_sing, s_adp, s_pre);
              count(c, s_bsing, s_badp, s_bpre);
            } else {
              count(sbie_auto<K>(k, P.el[e], false, cp.x, P.qsp, P.ns_max, hg, &st), s_sing, s_adp, s_pre);
              count(hbie_auto<KH>(kh, P.el[e], false, cp.x, P.qsp, P.ns_max, ml, true, &st), s_bsing, s_badp, s_bpre);
            }
            scatter<T>(P, e, hg.h, hg.g, rowbuf.data(), brow);
            scatter<T>(P, e, ml.h, ml.g, rowbuf2.data(), brow2);
            continue;
          }
          if (cp.kind <= 1) {
            count(sbie_auto<K>(k, P.el[e], false, cp.x, P.qsp, P.ns_max, hg, &st), s_sing, s_adp, s_pre);
            if constexpr (std::is_same<K, StaelaK>::value) {
              // half-space region: h, g of the complementary kernel added to the
              // full-space ones (build_lse_mechanics_bem_staela.f90:861-875)
              if (P.hs_n != 0) {
                HscK kc(k.mu, k.nu, P.hs_x);
                HG<HscK> hp;
                int c2 = hsc_auto(k, kc, P.el[e], false, cp.x, P.qsp, P.ns_max, hp, &st);
                if (c2 == CLS_SING) s_hsing++;
                else if (c2 == CLS_ADP) s_hadp++;
                for (int a = 0; a < 8; ++a)
                  for (int il = 0; il < 3; ++il)
                    for (int ik = 0; ik < 3; ++ik) {
                      hg.h[a][il][ik] = hg.h[a][il][ik] + hp.h[a][il][ik];
                      hg.g[a][il][ik] = hg.g[a][il][ik] + hp.g[a][il][ik];
                    }
              }
            }
          } else {
            KH kh = mkh(cp.n);
            HG<KH> ml;
            T w = (T)1.0;
            if (cp.kind == 5) {
              // 'dual_bm_mixed': the HBIE alone at its own point, weighted by
              // beta alpha (separate hbie_auto in both builders,
              // build_lse_mechanics_bem_staela.f90:938-997,
              // build_lse_mechanics_bem_harela.f90:1244-1284)
              count(hbie_auto<KH>(kh, P.el[e], false, cp.x, P.qsp, P.ns_max, ml, true, &st), s_bsing, s_badp, s_bpre);
              hg.zero();
              w = bm * P.alpha[s];
            } else if (cp.kind == 2) {
              // 'hbie': h = m, g = l
              count(hbie_auto<KH>(kh, P.el[e], false, cp.x, P.qsp, P.ns_max, ml, true, &st), s_bsing, s_badp, s_bpre);
              hg.zero();
            } else {
              w = bm * P.alpha[s];
              if constexpr (kHarmonic) {
                int c = shbie_auto(k, kh, P.el[e], false, cp.x, P.qsp, P.ns_max, hg, ml, &st);
                count(c, s_sing, s_adp, s_pre);
                count(c, s_bsing, s_badp, s_bpre);
              } else {
                count(sbie_auto<K>(k, P.el[e], false, cp.x, P.qsp, P.ns_max, hg, &st), s_sing, s_adp, s_pre);
                count(hbie_auto<KH>(kh, P.el[e], false, cp.x, P.qsp, P.ns_max, ml, true, &st), s_bsing, s_badp,
                      s_bpre);
              }
            }
            for (int a = 0; a < 8; ++a)
              for (int il = 0; il < 3; ++il)
                for (int ik = 0; ik < 3; ++ik) {
                  hg.h[a][il][ik] = hg.h[a][il][ik] + w * ml.h[a][il][ik];
                  hg.g[a][il][ik] = hg.g[a][il][ik] + w * ml.g[a][il][ik];
                }
          }
          scatter<T>(P, e, hg.h, hg.g, rowbuf.data(), brow);
        }
      }
      if (!free_terms_for_node<K>(P, s, nu, bm, rowbuf.data(), brow, rowbuf2.data(), brow2)) bad++;
      for (int il = 0; il < 3; ++il) {
        int r = P.dof[3 * s + il];
        for (int c = 0; c < n; ++c) A[(size_t)c * n + r] = A[(size_t)c * n + r] + rowbuf[(size_t)il * n + c];
        b[r] = b[r] + brow[il];
        if (P.crack[s]) {
          int r2 = P.dof2[3 * s + il];
          for (int c = 0; c < n; ++c) A[(size_t)c * n + r2] = A[(size_t)c * n + r2] + rowbuf2[(size_t)il * n + c];
          b[r2] = b[r2] + brow2[il];
        }
      }
    }
    s_leaves += st.leaves;
    s_points += st.points;
    s_maxd += st.maxdepth_hits;
    hs_err = std::max(hs_err, g_hs_err);
    hb_err = std::max(hb_err, g_hbie_err);
  }
  if (stats) {
    stats[0] = s_pre; stats[1] = s_adp; stats[2] = s_sing; stats[3] = s_leaves; stats[4] = s_points; stats[5] = s_maxd;
    stats[6] = s_hadp; stats[7] = s_hsing;
    stats[8] = s_bpre; stats[9] = s_badp; stats[10] = s_bsing;
  }
  if (hs_err) return -1 - hs_err;
  if (hb_err) return -6;
  return bad ? -1 : 0;
}

// Internal points: calculate_internal_points_mechanics_bem_{staela,harela}
// (src/calculate_internal_points_mechanics_static.f90:188-502,
// src/calculate_internal_points_mechanics_bem_harela.f90:22-505) for ordinary
// BE boundaries without symmetry planes, body loads or incident field:
//   u_il(x_i)      = sum_e sum_kn g(kn,il,ik) t_ik - h(kn,il,ik) u_ik
//   sigma_il,kc    = sum_e sum_kn l(kn,il,ik) t_ik - m(kn,il,ik) u_ik, n_i = e_kc
// with sbie_auto / hbie_auto at x_i; a point at a boundary node (distance /
// csize of the node's first element < 1e-12) takes the node's displacement and
// zero stresses (calculate_internal_points_mechanics_bem_harela.f90:190-208).
// A crack-like element adds face 2's terms with its reversed kernels, + g t2
// + h u2 and + l t2 + m u2 (calculate_internal_points_mechanics_static.f90:
// 320-354,431-465); u2, t2 [nn][3] (null without cracks).
// out[ip][4][3]: [0] displacement, [1 + kc] sigma(:, kc). Returns the index + 1
// of the first point that lies on an element away from its nodes or at a
// node of a crack-like boundary, else 0.
template <class K, class KH, class MKH>
static int internal_points(const Problem& P, const K& k, MKH mkh, int nip, const double* xip,
                           const typename K::T* u, const typename K::T* t, const typename K::T* u2,
                           const typename K::T* t2, typename K::T* out, int nthreads) {
  typedef typename K::T T;
  std::vector<int> efirst(P.nn, -1);
  for (int e = 0; e < P.ne; ++e)
    for (int kn = 0; kn < 8; ++kn)
      if (efirst[P.conn[8 * e + kn]] < 0) efirst[P.conn[8 * e + kn]] = e;
  std::vector<int> on_elem(nip, 0);
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1)
  for (int ip = 0; ip < nip; ++ip) {
    const double* xi = xip + 3 * (size_t)ip;
    T acc[4][3];
    for (int a = 0; a < 4; ++a)
      for (int c = 0; c < 3; ++c) acc[a][c] = (T)0;
    int on_node = -1;
    for (int sn = 0; sn < P.nn; ++sn) {
      if (efirst[sn] < 0) continue;
      double rd[3] = {xi[0] - P.X[3 * sn], xi[1] - P.X[3 * sn + 1], xi[2] - P.X[3 * sn + 2]};
      if (std::sqrt(rd[0] * rd[0] + rd[1] * rd[1] + rd[2] * rd[2]) / P.el[efirst[sn]].cl < 1e-12) on_node = sn;
    }
    if (on_node < 0) {
      for (int e = 0; e < P.ne && !on_elem[ip]; ++e) {
        const int* cn = &P.conn[8 * e];
        HG<K> hg;
        if (sbie_auto<K>(k, P.el[e], false, xi, P.qsp, P.ns_max, hg, nullptr) == CLS_SING) {
          on_elem[ip] = 1;
          break;
        }
        const bool ck = P.crack_el[e] != 0 && u2 && t2;
        if constexpr (std::is_same<K, StaelaK>::value) {
          // half-space: the complementary kernels added to the full-space
          // ones (calculate_internal_points_mechanics_static.f90:288-310,
          // 401-418): hsc_sbie_auto for u, hsc_hbie_auto for sigma
          if (P.hs_n != 0) {
            HscK kc(k.mu, k.nu, P.hs_x);
            HG<HscK> hp;
            hsc_auto(k, kc, P.el[e], false, xi, P.qsp, P.ns_max, hp, nullptr);
            for (int a = 0; a < 8; ++a)
              for (int il = 0; il < 3; ++il)
                for (int ik = 0; ik < 3; ++ik) {
                  hg.h[a][il][ik] = hg.h[a][il][ik] + hp.h[a][il][ik];
                  hg.g[a][il][ik] = hg.g[a][il][ik] + hp.g[a][il][ik];
                }
          }
        }
        for (int il = 0; il < 3; ++il)
          for (int ik = 0; ik < 3; ++ik)
            for (int kn = 0; kn < 8; ++kn) {
              acc[0][il] = acc[0][il] + hg.g[kn][il][ik] * t[3 * cn[kn] + ik] - hg.h[kn][il][ik] * u[3 * cn[kn] + ik];
              if (ck)
                acc[0][il] = acc[0][il] + hg.g[kn][il][ik] * t2[3 * cn[kn] + ik] +
                             hg.h[kn][il][ik] * u2[3 * cn[kn] + ik];
            }
        for (int kc = 0; kc < 3; ++kc) {
          double ni[3] = {0.0, 0.0, 0.0};
          ni[kc] = 1.0;
          KH kh = mkh(ni);
          HG<KH> ml;
          hbie_auto<KH>(kh, P.el[e], false, xi, P.qsp, P.ns_max, ml);
          if constexpr (std::is_same<K, StaelaK>::value) {
            if (P.hs_n != 0) {
              HscHK kc(k.mu, k.nu, P.hs_x, ni);
              HG<HscHK> mp;
              hsc_hbie_auto(kc, P.el[e], false, xi, P.qsp, P.ns_max, mp, nullptr);
              for (int a = 0; a < 8; ++a)
                for (int il = 0; il < 3; ++il)
                  for (int ik = 0; ik < 3; ++ik) {
                    ml.h[a][il][ik] = ml.h[a][il][ik] + mp.h[a][il][ik];
                    ml.g[a][il][ik] = ml.g[a][il][ik] + mp.g[a][il][ik];
                  }
            }
          }
          for (int il = 0; il < 3; ++il)
            for (int ik = 0; ik < 3; ++ik)
              for (int kn = 0; kn < 8; ++kn) {
                acc[1 + kc][il] =
                    acc[1 + kc][il] + ml.g[kn][il][ik] * t[3 * cn[kn] + ik] - ml.h[kn][il][ik] * u[3 * cn[kn] + ik];
                if (ck)
                  acc[1 + kc][il] = acc[1 + kc][il] + ml.g[kn][il][ik] * t2[3 * cn[kn] + ik] +
                                    ml.h[kn][il][ik] * u2[3 * cn[kn] + ik];
              }
        }
      }
    } else if (P.crack[on_node]) {
      on_elem[ip] = 1;
    } else {
      for (int c = 0; c < 3; ++c) acc[0][c] = u[3 * on_node + c];
    }
    for (int a = 0; a < 4; ++a)
      for (int c = 0; c < 3; ++c) out[12 * (size_t)ip + 3 * a + c] = acc[a][c];
  }
  for (int ip = 0; ip < nip; ++ip)
    if (on_elem[ip]) return ip + 1;
  return 0;
}

}  // namespace orc

using namespace orc;

extern "C" {

void* orc_problem_new(int nn, const double* X, int ne, const int* conn, const int* ctype, const double* cvalue,
                      double qsi_re, int ns_max, int n_ps, const int* ps_gln, double geo_tol) {
  Problem* P = new Problem();
  P->nn = nn; P->ne = ne;
  P->X.assign(X, X + 3 * nn);
  P->conn.assign(conn, conn + 8 * ne);
  P->ctype.assign(ctype, ctype + 3 * nn);
  P->cvalue.resize(3 * nn);
  for (int i = 0; i < 3 * nn; ++i) P->cvalue[i] = cplx(cvalue[2 * i], cvalue[2 * i + 1]);
  P->qsi_re = qsi_re; P->ns_max = ns_max; P->n_ps = n_ps; P->geo_tol = geo_tol;
  for (int i = 0; i < n_ps; ++i) P->ps_gln[i] = ps_gln[i];
  qs_calculate_parameters(qsi_re, P->qsp);
  build(*P);
  build_dofs(*P);
  build_colloc(*P);
  return P;
}
// Crack-like boundary: crack_el [ne] marks its elements (their nodes get two
// faces), ctype2 [nn][3] and cvalue2 [nn][3] (complex) the boundary conditions
// of face 2 (face 1: the problem's ctype / cvalue). Renumbers the DOF and
// rebuilds the collocation points. Returns -1 if a crack node also belongs
// to an ordinary element (a node lies in one boundary, data_structures.f90:
// 1433-1452).
int orc_problem_set_crack(void* h, const char* crack_el, const int* ctype2, const double* cvalue2) {
  Problem* P = (Problem*)h;
  std::vector<char> cn(P->nn, 0), on(P->nn, 0);
  for (int e = 0; e < P->ne; ++e)
    for (int k = 0; k < 8; ++k) (crack_el[e] ? cn : on)[P->conn[8 * e + k]] = 1;
  for (int s = 0; s < P->nn; ++s)
    if (cn[s] && on[s]) return -1;
  P->crack_el.assign(crack_el, crack_el + P->ne);
  P->crack = cn;
  for (int i = 0; i < 3 * P->nn; ++i) {
    P->ctype2[i] = ctype2[i];
    P->cvalue2[i] = cplx(cvalue2[2 * i], cvalue2[2 * i + 1]);
  }
  build_dofs(*P);
  build_colloc(*P);
  return 0;
}
void orc_dof2_map(void* h, int* dof2 /*3*nn*/) {
  Problem* P = (Problem*)h;
  for (int i = 0; i < 3 * P->nn; ++i) dof2[i] = P->dof2[i];
}
// BEM formulation per node (0 default SBIE, 1 'hbie', 2 'dual_bm_same'),
// alpha and delta_hbie per node (null: 1 and 0.22540333, the quadratic
// default of read_bem_formulation_selected_nodes.f90:43); rebuilds the
// collocation points. Returns -1 for a formulation code out of range.
int orc_problem_set_formulation(void* h, const int* form, const double* alpha, const double* delta) {
  Problem* P = (Problem*)h;
  for (int s = 0; s < P->nn; ++s)
    if (form[s] < 0 || form[s] > 3) return -1;
  for (int s = 0; s < P->nn; ++s) {
    P->form[s] = form[s];
    P->alpha[s] = alpha ? alpha[s] : 1.0;
    P->delta_hbie[s] = delta ? delta[s] : 0.22540333;
    // 'dual_bm_mixed' on the mesh boundary: the SBIE's MCA point moves by the
    // quadratic default 0.22540333 instead of the boundary default 0.05
    // (read_bem_formulation_selected_nodes.f90:273-294)
    if (P->in_boundary[s])
      for (auto& pr : P->node_el[s]) P->delta_mca[8 * pr.first + pr.second] = form[s] == 3 ? 0.22540333 : 0.05;
  }
  build_colloc(*P);
  return 0;
}
// unit normals of the collocation points (zero for SBIE points)
void orc_colloc_normals(void* h, double* n /*3*ncp*/) {
  Problem* P = (Problem*)h;
  for (size_t i = 0; i < P->cps.size(); ++i)
    for (int c = 0; c < 3; ++c) n[3 * i + c] = P->cps[i].n[c];
}
// One (collocation point, element) pair of the HBIE kernels at the point's
// normal (m, l laid out [kn][il][ik]), interior integration included.
int orc_pair_hbie_staela(void* hp, int ci, int e, double mu, double nu, double* m, double* l) {
  Problem* P = (Problem*)hp;
  StaelaHK k(mu, nu, P->cps[ci].n);
  HG<StaelaHK> ml;
  g_hbie_err = 0;
  int cls = hbie_auto<StaelaHK>(k, P->el[e], false, P->cps[ci].x, P->qsp, P->ns_max, ml, true);
  std::memcpy(m, ml.h, sizeof(ml.h));
  std::memcpy(l, ml.g, sizeof(ml.g));
  return g_hbie_err ? -6 : cls;
}
int orc_pair_hbie_harela(void* hp, int ci, int e, double lre, double lim, double mre, double mim, double rho,
                         double omega, double* m, double* l) {
  Problem* P = (Problem*)hp;
  HarelaHK k(harela_parameters(cplx(lre, lim), cplx(mre, mim), rho, omega), P->cps[ci].n);
  HG<HarelaHK> ml;
  g_hbie_err = 0;
  int cls = hbie_auto<HarelaHK>(k, P->el[e], false, P->cps[ci].x, P->qsp, P->ns_max, ml, true);
  std::memcpy(m, ml.h, sizeof(ml.h));
  std::memcpy(l, ml.g, sizeof(ml.g));
  return g_hbie_err ? -6 : cls;
}
void orc_problem_free(void* h) { delete (Problem*)h; }
int orc_n_dof(void* h) { return ((Problem*)h)->ndof; }
int orc_n_colloc(void* h) { return (int)((Problem*)h)->cps.size(); }

void orc_dof_map(void* h, int* dof /*3*nn*/, int* order /*nn*/) {
  Problem* P = (Problem*)h;
  for (int i = 0; i < 3 * P->nn; ++i) dof[i] = P->dof[i];
  for (size_t i = 0; i < P->node_order.size(); ++i) order[i] = P->node_order[i];
}
void orc_element_data(void* h, double* cl, int* gln_far, double* ball /*4*ne*/) {
  Problem* P = (Problem*)h;
  for (int e = 0; e < P->ne; ++e) {
    cl[e] = P->el[e].cl;
    gln_far[e] = P->el[e].gln_far;
    for (int c = 0; c < 3; ++c) ball[4 * e + c] = P->el[e].bc[c];
    ball[4 * e + 3] = P->el[e].br;
  }
}
void orc_colloc(void* h, double* x /*3*ncp*/, int* info /*4*ncp: node, kind, elem, kn*/) {
  Problem* P = (Problem*)h;
  for (size_t i = 0; i < P->cps.size(); ++i) {
    for (int c = 0; c < 3; ++c) x[3 * i + c] = P->cps[i].x[c];
    info[4 * i + 0] = P->cps[i].node;
    info[4 * i + 1] = P->cps[i].kind;
    info[4 * i + 2] = P->cps[i].elem;
    info[4 * i + 3] = P->cps[i].kn;
  }
}
void orc_node_geometry(void* h, double* n_gn, double* tbp, double* tbm, char* in_boundary) {
  Problem* P = (Problem*)h;
  std::memcpy(n_gn, P->n_gn.data(), sizeof(double) * P->n_gn.size());
  std::memcpy(tbp, P->tbp_gn.data(), sizeof(double) * P->tbp_gn.size());
  std::memcpy(tbm, P->tbm_gn.data(), sizeof(double) * P->tbm_gn.size());
  std::memcpy(in_boundary, P->in_boundary.data(), P->in_boundary.size());
}

// Region space: n = 0 full space, else the half-space normal (+-1..3), its
// hyperplane coordinate and boundary condition (1 traction-free). The static
// complementary kernel exists for n = -3 only (bem_staela3d.f90:7466-7468);
// the harmonic builder applies the free-term rule alone.
int orc_problem_set_halfspace(void* h, int n, double x, int bc) {
  Problem* P = (Problem*)h;
  if (n < -3 || n > 3 || bc != 1) return -1;
  P->hs_n = n;
  P->hs_x = x;
  P->hs_bc = bc;
  return 0;
}
// One point of the complementary kernel (u, t [3][3]: load, component).
int orc_hsc_point(double mu, double nu, double xp, const double* x_i, const double* x, const double* n, double* u,
                  double* t) {
  HscK k(mu, nu, xp);
  g_hs_err = 0;
  double uu[3][3], tt[3][3];
  k.eval_at(x, x_i, n, uu, tt);
  std::memcpy(u, uu, sizeof(uu));
  std::memcpy(t, tt, sizeof(tt));
  return g_hs_err;
}
// One (collocation point, element) pair of the complementary kernel.
int orc_pair_hsc(void* hp, int ci, int e, double mu, double nu, double* h, double* g) {
  Problem* P = (Problem*)hp;
  StaelaK kf(mu, nu);
  HscK k(mu, nu, P->hs_x);
  HG<HscK> hg;
  g_hs_err = 0;
  int cls = hsc_auto(kf, k, P->el[e], false, P->cps[ci].x, P->qsp, P->ns_max, hg, nullptr);
  std::memcpy(h, hg.h, sizeof(hg.h));
  std::memcpy(g, hg.g, sizeof(hg.g));
  return g_hs_err ? -1 - g_hs_err : cls;
}

int orc_assemble_staela(void* h, double mu, double nu, double* A, double* b, int nthreads, long* stats) {
  Problem* P = (Problem*)h;
  if (P->hs_n != 0 && P->hs_n != -3) return -4;
  StaelaK k(mu, nu);
  auto mkh = [&](const double* ni) { return StaelaHK(mu, nu, ni); };
  return assemble<StaelaK, StaelaHK>(*P, k, mkh, 1.0, nu, A, b, nthreads, stats);
}
// Harmonic assembly; nu is the region's complex-typed Poisson ratio (property_c(3)).
int orc_assemble_harela_nu(void* h, double lre, double lim, double mre, double mim, double rho, double omega,
                           double nure, double nuim, double* A, double* b, int nthreads, long* stats) {
  Problem* P = (Problem*)h;
  HarPar par = harela_parameters(cplx(lre, lim), cplx(mre, mim), rho, omega);
  HarelaK k(par);
  auto mkh = [&](const double* ni) { return HarelaHK(par, ni); };
  return assemble<HarelaK, HarelaHK>(*P, k, mkh, cplx(0.0, 1.0) / par.c2, cplx(nure, nuim), (cplx*)A, (cplx*)b,
                                     nthreads, stats);
}

// One (collocation point, element) pair; h,g laid out [kn][il][ik].
int orc_pair_staela(void* hp, int ci, int e, double mu, double nu, double* h, double* g) {
  Problem* P = (Problem*)hp;
  StaelaK k(mu, nu);
  HG<StaelaK> hg;
  int cls = sbie_auto<StaelaK>(k, P->el[e], false, P->cps[ci].x, P->qsp, P->ns_max, hg, nullptr);
  std::memcpy(h, hg.h, sizeof(hg.h));
  std::memcpy(g, hg.g, sizeof(hg.g));
  return cls;
}
int orc_pair_harela(void* hp, int ci, int e, double lre, double lim, double mre, double mim, double rho,
                    double omega, double* h, double* g) {
  Problem* P = (Problem*)hp;
  HarelaK k(harela_parameters(cplx(lre, lim), cplx(mre, mim), rho, omega));
  HG<HarelaK> hg;
  int cls = sbie_auto<HarelaK>(k, P->el[e], false, P->cps[ci].x, P->qsp, P->ns_max, hg, nullptr);
  std::memcpy(h, hg.h, sizeof(hg.h));
  std::memcpy(g, hg.g, sizeof(hg.g));
  return cls;
}
// Internal points (displacement and stresses), u / t nodal values [nn][3].
int orc_internal_points_staela(void* hp, double mu, double nu, int nip, const double* xip, const double* u,
                               const double* t, const double* u2, const double* t2, double* out, int nthreads) {
  Problem* P = (Problem*)hp;
  if (P->hs_n != 0) {
    // the complementary kernels exist for the half-space x3 >= xp only
    // (fbem_bem_staela3d_hsc_hbie: np = -3); points must lie in it
    if (P->hs_n != -3 || P->hs_bc != 1) return -7;
    for (int ip = 0; ip < nip; ++ip)
      if (xip[3 * ip + 2] < P->hs_x) return -8;
  }
  StaelaK k(mu, nu);
  auto mkh = [&](const double* ni) { return StaelaHK(mu, nu, ni); };
  return internal_points<StaelaK, StaelaHK>(*P, k, mkh, nip, xip, u, t, u2, t2, out, nthreads);
}
int orc_internal_points_harela(void* hp, double lre, double lim, double mre, double mim, double rho, double omega,
                               int nip, const double* xip, const double* u, const double* t, const double* u2,
                               const double* t2, double* out, int nthreads) {
  Problem* P = (Problem*)hp;
  HarPar par = harela_parameters(cplx(lre, lim), cplx(mre, mim), rho, omega);
  HarelaK k(par);
  auto mkh = [&](const double* ni) { return HarelaHK(par, ni); };
  return internal_points<HarelaK, HarelaHK>(*P, k, mkh, nip, xip, (const cplx*)u, (const cplx*)t, (const cplx*)u2,
                                            (const cplx*)t2, (cplx*)out, nthreads);
}
// Complementary HBIE kernels at one point (d, s [3][3]: load il, component
// ik) and the complementary stress sigma[l][k][j] = sigma*_{l,kj} from the
// derivatives of the Cartesian u* (test hooks for the pinning).
int orc_hsc_hbie_point(double mu, double nu, double xp, const double* x_i, const double* n_i, const double* x,
                       const double* n, double* d, double* s) {
  g_hs_err = 0;
  HscHK k(mu, nu, xp, n_i);
  double fd[3][3], fs[3][3];
  k.eval_at(x, x_i, n, fd, fs);
  std::memcpy(d, fd, sizeof(fd));
  std::memcpy(s, fs, sizeof(fs));
  return g_hs_err;
}
void orc_hsc_sigma_ad(double mu, double nu, double xp, const double* x_i, const double* xq, double* sig) {
  Jet x[3], xi[3];
  for (int c = 0; c < 3; ++c) {
    x[c] = jconst(xq[c]);
    x[c].gx[c] = 1.0;
    xi[c] = jconst(x_i[c]);
    xi[c].gi[c] = 1.0;
  }
  Jet u[3][3];
  hsc_u_jets(nu, x, xi, xp, u);
  const double Ku = 1.0 / (16.0 * c_pi * mu * (1.0 - nu)), lam = 2.0 * mu * nu / (1.0 - 2.0 * nu);
  for (int l = 0; l < 3; ++l) {
    const double div = u[l][0].gx[0] + u[l][1].gx[1] + u[l][2].gx[2];
    for (int k = 0; k < 3; ++k)
      for (int j = 0; j < 3; ++j)
        sig[9 * l + 3 * k + j] = Ku * ((j == k ? lam * div : 0.0) + mu * (u[l][k].gx[j] + u[l][j].gx[k]));
  }
}
// Harmonic parameter block for tests: k1,k2,c1,c2,psi(6),chi(6),T1(10),T2(9),T3(9),cte_u,cte_t (complex)
void orc_harela_parameters(double lre, double lim, double mre, double mim, double rho, double omega, double* out) {
  HarPar p = harela_parameters(cplx(lre, lim), cplx(mre, mim), rho, omega);
  cplx* o = (cplx*)out;
  int i = 0;
  o[i++] = p.k1; o[i++] = p.k2; o[i++] = p.c1; o[i++] = p.c2;
  for (int j = 0; j < 6; ++j) o[i++] = p.psi[j];
  for (int j = 0; j < 6; ++j) o[i++] = p.chi[j];
  for (int j = 0; j < 10; ++j) o[i++] = p.T1[j];
  for (int j = 0; j < 9; ++j) o[i++] = p.T2[j];
  for (int j = 0; j < 9; ++j) o[i++] = p.T3[j];
  o[i++] = p.cte_u; o[i++] = p.cte_t;
}

void orc_gauss_tables(double* gl11x, double* gl11w, double* gl01x, double* gl01w) {
  const GaussTables& g = gauss();
  std::memcpy(gl11x, g.gl11_xi, sizeof(g.gl11_xi));
  std::memcpy(gl11w, g.gl11_w, sizeof(g.gl11_w));
  std::memcpy(gl01x, g.gl01_xi, sizeof(g.gl01_xi));
  std::memcpy(gl01w, g.gl01_w, sizeof(g.gl01_w));
}
void orc_qs_parameters(double re, double* out /*10*24*/) {
  QsParams p;
  qs_calculate_parameters(re, p);
  const double* arrs[10] = {&p.dmin[0][0], &p.dmax[0][0], &p.alpha0[0][0], &p.alpha1[0][0], &p.beta1[0][0],
                            &p.t_dmin[0][0], &p.t_dmax[0][0], &p.t_alpha0[0][0], &p.t_alpha1[0][0], &p.t_beta1[0][0]};
  for (int a = 0; a < 10; ++a)
    for (int i = 0; i < 24; ++i) out[24 * a + i] = arrs[a][i];
}
int orc_qs_estimate(int telles, int dim, int f, double re, double d, const double* barxi) {
  QsParams p;
  qs_calculate_parameters(re, p);
  return telles ? qs_n_estimation_telles(dim, f, p, d, barxi) : qs_n_estimation_standard(dim, f, p, d, barxi);
}
void orc_zexp(double zr, double zi, double* E /*7 complex*/) {
  cplx z(zr, zi), e[7][2];
  zexp_decomposed(1, &z, e);
  for (int k = 0; k < 7; ++k) { E[2 * k] = e[k][0].real(); E[2 * k + 1] = e[k][0].imag(); }
}
void orc_nearest_quad8(const double* x /*8x3*/, double cl, const double* p, double* barxi, double* rmin, double* d,
                       int* method) {
  double xx[8][3];
  std::memcpy(xx, x, sizeof(xx));
  nearest_element_point_quad8(xx, cl, p, barxi, rmin, d, method);
}
int orc_freeterm(int ne, const double* n, const double* t, double tol, double nu, double* c) {
  double C[3][3];
  bool ok = freeterm<double>(ne, n, t, tol, nu, C);
  std::memcpy(c, C, sizeof(C));
  return ok ? 0 : -1;
}

}  // extern "C"
