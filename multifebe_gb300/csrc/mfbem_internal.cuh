// Internal points: calculate_internal_points_mechanics_bem_{staela,harela}
// (src/calculate_internal_points_mechanics_static.f90:188-502,
// src/calculate_internal_points_mechanics_bem_harela.f90:22-505), the step
// after the solve. Displacement and stress tensor at points inside the region
// from the nodal solution, for ordinary BE boundaries without symmetry planes,
// body loads or incident field:
//   u_il        = sum_e sum_kn g(kn,il,ik) t_ik - h(kn,il,ik) u_ik      (sbie_auto)
//   sigma_il,kc = sum_e sum_kn l(kn,il,ik) t_ik - m(kn,il,ik) u_ik      (hbie_auto, n_i = e_kc)
// with the HBIE kernels d* (l) and s* (m) of bem_staela3d.f90:4376-4446 and
// bem_harela3d.f90:2573-2662, classified like sbie_auto with the 1/r^7
// quasi-singular estimate. A point at a boundary node (distance / csize of the
// node's first element < 1e-12) takes the node's displacement and zero
// stresses (calculate_internal_points_mechanics_bem_harela.f90:190-208).
//
// Layout of the work: the shape-function weights of every quadrature point are
// contracted with the element's nodal values first (t_w = sum_kn phi_kn J w t_kn,
// the same for u), so no 8x3x3 kernel block is formed; one warp per (point,
// frequency) walks the elements with the precalculated rules, and one thread per
// quasi-singular (point, element) pair walks the subdivision tree, writing its
// 12 sums to a slot that the warp adds in element order (deterministic). FP64:
// this runs once per solution, not per sweep step.
#pragma once

namespace mfb {

// d* / s* coefficients of fbem_bem_harela3d_calculate_parameters (bem_harela3d.f90:219-283)
// (ic2 = i / c2, the Burton & Miller factor of the harmonic builder)
struct HarParH {
  cd S1[11], S2[11], S3[12], S4[10], S5[11];
  cd cte_d, cte_s, ic2;
};
__host__ __device__ inline HarParH harela_hbie_params(cd lambda, cd mu, double rho, double omega) {
  HarParH p;
  const cd I = mk(0.0, 1.0);
  cd c1 = csqrt_((lambda + 2.0 * mu) / rho), c2 = csqrt_(mu / rho);
  cd k1 = omega / c1, k2 = omega / c2;
  cd c1p2 = c1 * c1, c2p2 = c2 * c2, c1p3 = c1p2 * c1, c1p4 = c1p2 * c1p2, c1p5 = c1p4 * c1, c2p3 = c2p2 * c2;
  cd k1p2 = k1 * k1, k2p2 = k2 * k2, q = k1p2 / k2p2;
  cd ik1 = I * k1, ik2 = I * k2, ik1p2 = ik1 * ik1, ik2p2 = ik2 * ik2;
  cd r = c2p2 / c1p2;
  const double om2 = omega * omega, om3 = om2 * omega;
  p.S1[0] = 3.0 * (1.0 - 2.0 * r);
  p.S1[1] = -0.5 * c2p2 / c1p4 * om2;
  p.S1[2] = k2p2;
  p.S1[3] = 4.0 * I * k1 * q;
  p.S1[4] = -7.0 * I * k2;
  p.S1[5] = 24.0 * q;
  p.S1[6] = mk(-27.0);
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
  p.S2[6] = mk(-24.0);
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
  p.S3[7] = mk(-180.0);
  p.S3[8] = 420.0 * r / ik1;
  p.S3[9] = -420.0 / ik2;
  p.S3[10] = 420.0 / ik2p2;
  p.S3[11] = -420.0 / ik2p2;
  p.S4[0] = 2.0 * r;
  p.S4[1] = 0.5 * (c2p2 / c1p4 + 1.0 / c2p2) * om2;
  p.S4[2] = -2.0 / 5.0 * (1.0 / c2p3 + 2.0 / 3.0 * c2p2 / c1p5) * I * om3;
  p.S4[3] = 2.0 * I * k2;
  p.S4[4] = -4.0 * r;
  p.S4[5] = mk(6.0);
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
  p.S5[6] = mk(4.0);
  p.S5[7] = 12.0 * I * k1 / k2p2;
  p.S5[8] = -12.0 * I / k2;
  p.S5[9] = 12.0 / k2p2;
  p.S5[10] = -12.0 / k2p2;
  p.cte_d = mk(k1_4Pi);
  p.cte_s = k1_4Pi * mu;
  p.ic2 = I / c2;
  return p;
}

// E_2..E_6 of z (numerical.f90:1258-1331), as zexp_2to5 plus E_6
__device__ __forceinline__ void zexp_2to6(const ZexpSteps& steps, cd z, cd E[7]) {
  const double az2 = z.re * z.re + z.im * z.im;
  cd z2 = z * z, z3 = z2 * z, z4 = z3 * z, z5 = z4 * z;
  if (az2 <= 1.0) {
    const int N = zexp_nterms(steps, az2) + 6;
    cd t = mk(1.0);
    for (int k = N; k >= 7; --k) t = 1.0 + t * z * (1.0 / (double)k);
    E[6] = ((z5 * z) * (1.0 / 720.0)) * t;
    E[5] = E[6] + z5 * (1.0 / 120.0);
    E[4] = E[5] + z4 * (1.0 / 24.0);
    E[3] = E[4] + z3 * (1.0 / 6.0);
    E[2] = E[3] + z2 * 0.5;
  } else {
    E[2] = (cexp_(z) - 1.0) - z;
    E[3] = E[2] - 0.5 * z2;
    E[4] = E[3] - (1.0 / 6.0) * z3;
    E[5] = E[4] - (1.0 / 24.0) * z4;
    E[6] = E[5] - (1.0 / 120.0) * z5;
  }
}

// The contraction of one quadrature point: u-part (SBIE) and sigma-part (HBIE
// with the three unit normals), already multiplied by the nodal values' weighted
// sums ut (tractions) and uu (displacements). rs = -1 for a reversed element.
struct IpStatic {
  typedef double T;
  StaelaP k;
  double nu, cted1, cted2, ctes1, ctes2, ctes3, mu = 0.0;
  __device__ void sbie(int, const double*, const double rv[3], const double n[3], const T ut[3], const T uu[3], double rs,
                       T du[3]) const {
    double fu[9], ft[9];
    staela_point(k, rv, n, fu, ft);
#pragma unroll
    for (int il = 0; il < 3; ++il) {
      double g = 0.0, h = 0.0;
#pragma unroll
      for (int ik = 0; ik < 3; ++ik) {
        g += fu[3 * il + ik] * ut[ik];
        h += ft[3 * il + ik] * uu[ik];
      }
      du[il] += k.cteu1 * g - rs * k.ctet1 * h;
    }
  }
  __device__ void hbie(int, const double*, const double rv[3], const double n[3], const T ut[3], const T uu[3], double rs,
                       T sg[3][3]) const {
    const double r = sqrt(rv[0] * rv[0] + rv[1] * rv[1] + rv[2] * rv[2]);
    const double d1r = 1.0 / r, d1r2 = d1r * d1r, d1r3 = d1r2 * d1r;
    const double dr[3] = {rv[0] * d1r, rv[1] * d1r, rv[2] * d1r};
    const double drdn = dr[0] * n[0] + dr[1] * n[1] + dr[2] * n[2];
#pragma unroll 1
    for (int kc = 0; kc < 3; ++kc) {
      const double drdni = -dr[kc], nni = n[kc];
#pragma unroll
      for (int il = 0; il < 3; ++il) {
        double l = 0.0, m = 0.0;
#pragma unroll
        for (int ik = 0; ik < 3; ++ik) {
          const double dk = il == ik ? 1.0 : 0.0, nil = il == kc ? 1.0 : 0.0, nik = ik == kc ? 1.0 : 0.0;
          const double fd = d1r2 * ((cted2 * dk + 3.0 * dr[il] * dr[ik]) * drdni + cted2 * (nil * dr[ik] - nik * dr[il]));
          const double fs = d1r3 * (3.0 * (5.0 * dr[il] * dr[ik] - nu * dk) * drdn * drdni +
                                    3.0 * ctes2 * (dr[ik] * nil * drdn - dr[il] * n[ik] * drdni) +
                                    3.0 * nu * (dr[il] * nik * drdn - dr[ik] * n[il] * drdni) +
                                    (3.0 * nu * dr[il] * dr[ik] + ctes2 * dk) * nni + ctes2 * n[il] * nik -
                                    ctes3 * n[ik] * nil);
          l += fd * ut[ik];
          m += fs * uu[ik];
        }
        sg[il][kc] += cted1 * l - rs * ctes1 * m;
      }
    }
  }
};

struct IpHarmonic {
  typedef cd T;
  const HarParD* p;
  const HarParH* ph;
  __device__ void sbie(int f, const double*, const double rv[3], const double n[3], const T ut[3], const T uu[3], double rs,
                       T du[3]) const {
    cd fu[9], ft[9];
    harela_point(p[f], rv, n, fu, ft);
#pragma unroll
    for (int il = 0; il < 3; ++il) {
      cd g = mk(0.0), h = mk(0.0);
#pragma unroll
      for (int ik = 0; ik < 3; ++ik) {
        g = g + fu[3 * il + ik] * ut[ik];
        h = h + ft[3 * il + ik] * uu[ik];
      }
      du[il] = du[il] + p[f].cte_u * g - (rs * p[f].cte_t) * h;
    }
  }
  __device__ void hbie(int f, const double*, const double rv[3], const double n[3], const T ut[3], const T uu[3], double rs,
                       T sg[3][3]) const {
    const HarParD& q = p[f];
    const HarParH& s = ph[f];
    const double r = sqrt(rv[0] * rv[0] + rv[1] * rv[1] + rv[2] * rv[2]);
    const double d1r1 = 1.0 / r, d1r2 = d1r1 * d1r1, d1r3 = d1r2 * d1r1, d1r4 = d1r3 * d1r1, d1r5 = d1r4 * d1r1;
    const double dr[3] = {rv[0] * d1r1, rv[1] * d1r1, rv[2] * d1r1};
    const double drdn = dr[0] * n[0] + dr[1] * n[1] + dr[2] * n[2];
    cd a[7], b[7];
    zexp_2to6(q.steps, mk(q.k1.im * r, -q.k1.re * r), a);
    zexp_2to6(q.steps, mk(q.k2.im * r, -q.k2.re * r), b);
    const double sc[7] = {0.0, 0.0, d1r1, d1r2, d1r3, d1r4, d1r5};
#pragma unroll
    for (int j = 2; j < 7; ++j) {
      a[j] = a[j] * sc[j];
      b[j] = b[j] * sc[j];
    }
    const cd TT1 = q.T1[0] * d1r2 + q.T1[1] + q.T1[2] * a[2] + q.T1[3] * b[2] + q.T1[4] * a[3] + q.T1[5] * b[3] +
                   q.T1[6] * a[4] + q.T1[7] * b[4] + q.T1[8] * a[5] + q.T1[9] * b[5];
    const cd TT2 = q.T2[0] * d1r2 + q.T2[1] + q.T2[2] * b[2] + q.T2[3] * a[3] + q.T2[4] * b[3] + q.T2[5] * a[4] +
                   q.T2[6] * b[4] + q.T2[7] * a[5] + q.T2[8] * b[5];
    const cd TT3 = q.T3[0] * d1r2 + q.T3[1] + q.T3[2] * a[2] + q.T3[3] * a[3] + q.T3[4] * b[3] + q.T3[5] * a[4] +
                   q.T3[6] * b[4] + q.T3[7] * a[5] + q.T3[8] * b[5];
    const cd S1 = s.S1[0] * d1r3 + s.S1[1] * d1r1 + s.S1[2] * b[2] + s.S1[3] * a[3] + s.S1[4] * b[3] +
                  s.S1[5] * a[4] + s.S1[6] * b[4] + s.S1[7] * a[5] + s.S1[8] * b[5] + s.S1[9] * a[6] + s.S1[10] * b[6];
    const cd S2 = s.S2[0] * d1r3 + s.S2[1] * d1r1 + s.S2[2] * a[2] + s.S2[3] * a[3] + s.S2[4] * b[3] +
                  s.S2[5] * a[4] + s.S2[6] * b[4] + s.S2[7] * a[5] + s.S2[8] * b[5] + s.S2[9] * a[6] + s.S2[10] * b[6];
    const cd S3 = s.S3[0] * d1r3 + s.S3[1] * d1r1 + s.S3[2] * a[2] + s.S3[3] * b[2] + s.S3[4] * a[3] +
                  s.S3[5] * b[3] + s.S3[6] * a[4] + s.S3[7] * b[4] + s.S3[8] * a[5] + s.S3[9] * b[5] +
                  s.S3[10] * a[6] + s.S3[11] * b[6];
    const cd S4 = s.S4[0] * d1r3 + s.S4[1] * d1r1 + s.S4[2] + s.S4[3] * b[3] + s.S4[4] * a[4] + s.S4[5] * b[4] +
                  s.S4[6] * a[5] + s.S4[7] * b[5] + s.S4[8] * a[6] + s.S4[9] * b[6];
    const cd S5 = s.S5[0] * d1r3 + s.S5[1] * d1r1 + s.S5[2] + s.S5[3] * a[2] + s.S5[4] * a[3] + s.S5[5] * a[4] +
                  s.S5[6] * b[4] + s.S5[7] * a[5] + s.S5[8] * b[5] + s.S5[9] * a[6] + s.S5[10] * b[6];
    const cd cl = s.cte_d, cm = rs * s.cte_s;
#pragma unroll 1
    for (int kc = 0; kc < 3; ++kc) {
      const double drdni = -dr[kc], nni = n[kc];
#pragma unroll
      for (int il = 0; il < 3; ++il) {
        cd l = mk(0.0), m = mk(0.0);
#pragma unroll
        for (int ik = 0; ik < 3; ++ik) {
          const double dk = il == ik ? 1.0 : 0.0, nil = il == kc ? 1.0 : 0.0, nik = ik == kc ? 1.0 : 0.0;
          const cd fd = TT1 * (dr[il] * dr[ik] * drdni) - TT2 * (-drdni * dk + dr[il] * nik) - TT3 * (dr[ik] * nil);
          const cd fs = S1 * (dr[il] * nik * drdn - dr[ik] * n[il] * drdni - dk * drdn * drdni + dr[il] * dr[ik] * nni) +
                        S2 * (dr[ik] * nil * drdn - dr[il] * n[ik] * drdni) + S3 * (dr[il] * dr[ik] * drdn * drdni) +
                        S4 * (dk * nni + nik * n[il]) + S5 * (n[ik] * nil);
          l = l + fd * ut[ik];
          m = m + fs * uu[ik];
        }
        sg[il][kc] = sg[il][kc] + cl * l - cm * m;
      }
    }
  }
};

// Half-space (static, x3 >= xp, traction-free surface): the complementary
// kernels added at internal points (calculate_internal_points_mechanics_static.f90:
// 288-310,401-418). rv is measured from the image of the point (the pairs are
// classified on it, as fbem_bem_staela3d_hsc_sbie_auto / _hsc_hbie_auto do);
// xi is the point. u*, t*: hsc_point (fbem_bem_staela3d_hsc_sbie). d*, s*
// (fbem_bem_staela3d_hsc_hbie, bem_staela3d.f90:10882-11102): built from the
// first and mixed second derivatives of the complementary u* in x and x_i,
// here by forward-mode differentiation of u* in Cartesian form (HJet: value,
// the gradients in x and x_i and the mixed Hessian block).
struct HJet {
  double v, gx[3], gi[3], H[3][3];
};
__device__ __forceinline__ HJet hj_const(double c) {
  HJet r;
  r.v = c;
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    r.gx[j] = r.gi[j] = 0.0;
#pragma unroll
    for (int p = 0; p < 3; ++p) r.H[j][p] = 0.0;
  }
  return r;
}
__device__ __forceinline__ HJet hj_axpy(double a, const HJet& x, const HJet& y) {  // a x + y
  HJet r;
  r.v = a * x.v + y.v;
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    r.gx[j] = a * x.gx[j] + y.gx[j];
    r.gi[j] = a * x.gi[j] + y.gi[j];
#pragma unroll
    for (int p = 0; p < 3; ++p) r.H[j][p] = a * x.H[j][p] + y.H[j][p];
  }
  return r;
}
__device__ __forceinline__ HJet hj_add(const HJet& x, const HJet& y) { return hj_axpy(1.0, x, y); }
__device__ __forceinline__ HJet hj_sub(const HJet& x, const HJet& y) { return hj_axpy(-1.0, y, x); }
__device__ __forceinline__ HJet hj_scale(double a, const HJet& x) { return hj_axpy(a, x, hj_const(0.0)); }
__device__ __forceinline__ HJet hj_mul(const HJet& a, const HJet& b) {
  HJet r;
  r.v = a.v * b.v;
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    r.gx[j] = a.v * b.gx[j] + a.gx[j] * b.v;
    r.gi[j] = a.v * b.gi[j] + a.gi[j] * b.v;
  }
#pragma unroll
  for (int j = 0; j < 3; ++j)
#pragma unroll
    for (int p = 0; p < 3; ++p) r.H[j][p] = a.v * b.H[j][p] + a.H[j][p] * b.v + a.gx[j] * b.gi[p] + a.gi[p] * b.gx[j];
  return r;
}
__device__ __forceinline__ HJet hj_chain(const HJet& a, double g, double d1, double d2) {
  HJet r;
  r.v = g;
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    r.gx[j] = d1 * a.gx[j];
    r.gi[j] = d1 * a.gi[j];
  }
#pragma unroll
  for (int j = 0; j < 3; ++j)
#pragma unroll
    for (int p = 0; p < 3; ++p) r.H[j][p] = d1 * a.H[j][p] + d2 * a.gx[j] * a.gi[p];
  return r;
}
__device__ __forceinline__ HJet hj_inv(const HJet& a) {
  const double q = 1.0 / a.v;
  return hj_chain(a, q, -q * q, 2.0 * q * q * q);
}
__device__ __forceinline__ HJet hj_sqrt(const HJet& a) {
  const double s = sqrt(a.v);
  return hj_chain(a, s, 0.5 / s, -0.25 / (s * a.v));
}
// complementary u*[l][k] without 1 / (16 pi mu (1 - nu)); x, xi seeded jets
__device__ void hsc_u_jets(double nu, const HJet x[3], const HJet xi[3], double xp, HJet u[3][3]) {
  const double c1 = 1.0 - nu, c2 = 1.0 - 2.0 * nu, c4 = 3.0 - 4.0 * nu, k12 = 4.0 * c1 * c2;
  const HJet rx = hj_sub(x[0], xi[0]), ry = hj_sub(x[1], xi[1]);
  const HJet z = hj_axpy(1.0, x[2], hj_const(-xp)), c = hj_axpy(1.0, xi[2], hj_const(-xp)), zc = hj_add(z, c);
  const HJet rp = hj_sqrt(hj_add(hj_add(hj_mul(rx, rx), hj_mul(ry, ry)), hj_mul(zc, zc)));
  const HJet irp = hj_inv(rp), irp2 = hj_mul(irp, irp), irp3 = hj_mul(irp2, irp), irp5 = hj_mul(irp3, irp2);
  const HJet iq = hj_inv(hj_add(rp, zc)), iq2 = hj_mul(iq, iq);
  const HJet cz = hj_mul(c, z), zmc = hj_sub(z, c);
  const HJet one = hj_const(1.0);
  const HJet irpiq = hj_mul(irp, iq);
  // shared radial factors of the tangential / normal loads
  const HJet tA = hj_sub(hj_scale(c4, hj_mul(zmc, irp3)), hj_scale(6.0, hj_mul(hj_mul(cz, zc), irp5)));
  const HJet Bt = hj_axpy(k12, irpiq, tA);   // load tangential, component 3
  const HJet Bn = hj_axpy(-k12, irpiq, hj_axpy(12.0, hj_mul(hj_mul(cz, zc), irp5), tA));  // normal load, components 1, 2
#pragma unroll 1
  for (int a = 0; a < 2; ++a) {
    const HJet ra = a ? ry : rx, ra2 = hj_mul(ra, ra);
    HJet v = hj_add(irp, hj_scale(c4, hj_mul(ra2, irp3)));
    v = hj_add(v, hj_mul(hj_scale(2.0, hj_mul(cz, irp3)), hj_axpy(-3.0, hj_mul(ra2, irp2), one)));
    v = hj_add(v, hj_mul(hj_scale(k12, iq), hj_sub(one, hj_mul(ra2, irpiq))));
    u[a][a] = v;
    u[a][2] = hj_mul(ra, Bt);
    u[2][a] = hj_mul(ra, Bn);
  }
  u[0][1] = hj_mul(hj_mul(rx, ry), hj_sub(hj_sub(hj_scale(c4, irp3), hj_scale(6.0, hj_mul(cz, irp5))),
                                          hj_scale(k12, hj_mul(irp, iq2))));
  u[1][0] = u[0][1];
  const HJet zc2 = hj_mul(zc, zc);
  u[2][2] = hj_add(hj_add(hj_scale(8.0 * c1 * c1 - c4, irp), hj_mul(hj_sub(hj_scale(c4, zc2), hj_scale(2.0, cz)), irp3)),
                   hj_scale(6.0, hj_mul(hj_mul(cz, zc2), irp5)));
}
struct IpHsc {
  typedef double T;
  double mu, nu, xp;
  __device__ void sbie(int, const double* xi, const double rv[3], const double n[3], const T ut[3], const T uu[3],
                       double rs, T du[3]) const {
    const double c = xi[2] - xp;
    double fu[9], ft[9];
    hsc_point(nu, rv[0], rv[1], c, rv[2] - c, rv[2] + 2.0 * xp, n, fu, ft);
    const double cu = 1.0 / (16.0 * kPi * mu * (1.0 - nu)), ct = 1.0 / (8.0 * kPi * (1.0 - nu));
#pragma unroll
    for (int il = 0; il < 3; ++il) {
      double g = 0.0, h = 0.0;
#pragma unroll
      for (int ik = 0; ik < 3; ++ik) {
        g += fu[3 * il + ik] * ut[ik];
        h += ft[3 * il + ik] * uu[ik];
      }
      du[il] += cu * g - rs * ct * h;
    }
  }
  __device__ void hbie(int, const double* xi, const double rv[3], const double n[3], const T ut[3], const T uu[3],
                       double rs, T sg[3][3]) const {
    // x = image + rv
    const double xq[3] = {xi[0] + rv[0], xi[1] + rv[1], 2.0 * xp - xi[2] + rv[2]};
    HJet xj[3], ij[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      xj[c] = hj_const(xq[c]);
      xj[c].gx[c] = 1.0;
      ij[c] = hj_const(xi[c]);
      ij[c].gi[c] = 1.0;
    }
    HJet u[3][3];
    hsc_u_jets(nu, xj, ij, xp, u);
    const double Ku = 1.0 / (16.0 * kPi * mu * (1.0 - nu)), lam = 2.0 * mu * nu / (1.0 - 2.0 * nu);
    // x_i derivative of t* = sigma*(x) n, sigma*_{l,kj} = lam d_kj div u_l + mu (u_lk,j + u_lj,k)
    double dt[3][3][3];
#pragma unroll 1
    for (int l = 0; l < 3; ++l)
#pragma unroll 1
      for (int k = 0; k < 3; ++k)
#pragma unroll 1
        for (int p = 0; p < 3; ++p) {
          const double div = u[l][0].H[0][p] + u[l][1].H[1][p] + u[l][2].H[2][p];
          double v = 0.0;
          for (int j = 0; j < 3; ++j) {
            double sj = mu * (u[l][k].H[j][p] + u[l][j].H[k][p]);
            if (j == k) sj += lam * div;
            v += sj * n[j];
          }
          dt[l][k][p] = Ku * v;
        }
    // d*_lkp, s*_lkp contracted with n_i = e_kc: sg(:, kc) += d ut - rs s uu
#pragma unroll 1
    for (int kc = 0; kc < 3; ++kc)
#pragma unroll 1
      for (int l = 0; l < 3; ++l) {
        double acc = 0.0;
        for (int k = 0; k < 3; ++k) {
          double dl = mu * Ku * (u[l][k].gi[kc] + u[kc][k].gi[l]);
          double sl = mu * (dt[l][k][kc] + dt[kc][k][l]);
          if (l == kc) {
            dl += lam * Ku * (u[0][k].gi[0] + u[1][k].gi[1] + u[2][k].gi[2]);
            sl += lam * (dt[0][k][0] + dt[1][k][1] + dt[2][k][2]);
          }
          acc += dl * ut[k] - rs * sl * uu[k];
        }
        sg[l][kc] += acc;
      }
  }
};

// q: [nf][6] = lambda (re, im), mu (re, im), rho, omega
__global__ void k_harparh(const double* q, int nf, HarParH* out) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nf) return;
  const double* v = q + 6 * f;
  out[f] = harela_hbie_params(mk(v[0], v[1]), mk(v[2], v[3]), v[4], v[5]);
}

// inputs of the internal-point kernels
struct IpArgs {
  int nip, nf;
  const double* xip;     // [nip][3]
  const int* enode;      // [ne][8] 0-based node of each element node
  const double* nodex;   // [nn][3]
  const double* nodecl;  // [nn] csize of the node's first element
  int nn;
  const void* uval;      // [nf][nn][3] T
  const void* tval;      // [nf][nn][3] T
  uint8_t* cls_s;        // [nip][ne]
  uint8_t* cls_h;
  int* onnode;           // [nip] node index or -1
  int* npair;            // [nip] quasi-singular pairs per point, then exclusive offsets [nip+1]
  int* poff;
  int* pair_e;           // [npairs]
  int* pair_ip;
  int* err;              // first point (1-based) on an element away from its nodes, 0 if none
  void* slot;            // [nf][npairs][12] T
  int npairs;
  void* out;             // [nf][nip][12] T: u(3), then sigma(:, kc) for kc = 0..2
  // image pass of a half-space region: pairs classified and integrated from
  // the image (x_i1, x_i2, 2 xp - x_i3) of each point; points at a node add 0
  int image;
  double hs_xp;
};
// the point the pair geometry is measured from: the point, or its image
__device__ __forceinline__ void ip_ref(const IpArgs& a, const double* xi, double xr[3]) {
  xr[0] = xi[0];
  xr[1] = xi[1];
  xr[2] = a.image ? 2.0 * a.hs_xp - xi[2] : xi[2];
}

// point at a node: the last node (in node order) within 1e-12 csize
__global__ void k_ip_onnode(IpArgs a) {
  const int ip = blockIdx.x * blockDim.x + threadIdx.x;
  if (ip >= a.nip) return;
  const double* x = a.xip + 3 * (size_t)ip;
  int last = -1;
  for (int s = 0; s < a.nn; ++s) {
    if (a.nodecl[s] <= 0.0) continue;  // node of no element
    const double r0 = x[0] - a.nodex[3 * s], r1 = x[1] - a.nodex[3 * s + 1], r2 = x[2] - a.nodex[3 * s + 2];
    if (sqrt(r0 * r0 + r1 * r1 + r2 * r2) / a.nodecl[s] < 1e-12) last = s;
  }
  a.onnode[ip] = last;
}

// sbie_auto / hbie_auto classification of every (point, element) pair
__global__ void k_ip_classify(DMesh m, IpArgs a, const QsCurves* __restrict__ qs) {
  const long long total = (long long)a.nip * m.ne;
  for (long long id = blockIdx.x * (long long)blockDim.x + threadIdx.x; id < total;
       id += (long long)gridDim.x * blockDim.x) {
    const int ip = (int)(id / m.ne), e = (int)(id % m.ne);
    double xi[3];
    ip_ref(a, a.xip + 3 * (size_t)ip, xi);
    const double* b = m.ball + 4 * (size_t)e;
    const double r0 = b[0] - xi[0], r1 = b[1] - xi[1], r2 = b[2] - xi[2];
    double rmin = sqrt(r0 * r0 + r1 * r1 + r2 * r2) - b[3];
    double bx[2] = {0.0, 0.0}, d;
    bool sing = false;
    if (rmin > 4.0 * b[3]) {
      d = rmin / m.cl[e];
    } else {
      int method;
      nearest_q8(m.ex + 24 * (size_t)e, m.cl[e], xi, bx, &rmin, &d, &method);
      sing = d <= 1e-12;
    }
    uint8_t c[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      if (sing) {
        c[h] = CLS_SING;
        continue;
      }
      const int gn = qs_estimate(*qs, 2, h ? 7 : 5, d, bx, false);
      const int gln = max(m.gln_far[e], gn);
      c[h] = CLS_ADP;
      if (gln <= m.ps_gln_max && gn > 0)
        for (int i = 0; i < m.nps; ++i)
          if (m.ps_gln[i] >= gln) { c[h] = (uint8_t)i; break; }
    }
    a.cls_s[id] = c[0];
    a.cls_h[id] = c[1];
  }
}

// quasi-singular pairs per point (one warp per point); a singular pair of a
// point that is not at a node records the point in err
__global__ void k_ip_count(DMesh m, IpArgs a) {
  const int ip = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), l = threadIdx.x & 31;
  if (ip >= a.nip) return;
  int cnt = 0, sing = 0;
  if (a.onnode[ip] < 0)
    for (int e = l; e < m.ne; e += 32) {
      const size_t id = (size_t)ip * m.ne + e;
      const uint8_t s = a.cls_s[id], h = a.cls_h[id];
      if (s == CLS_SING || h == CLS_SING) sing = 1;
      else if (s == CLS_ADP || h == CLS_ADP) ++cnt;
    }
  for (int o = 16; o > 0; o >>= 1) {
    cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    sing |= __shfl_xor_sync(0xffffffffu, sing, o);
  }
  if (l == 0) {
    a.npair[ip] = sing ? 0 : cnt;
    if (sing) atomicMin(a.err, ip + 1);
  }
}
__global__ void k_ip_fill(DMesh m, IpArgs a) {
  const int ip = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), l = threadIdx.x & 31;
  if (ip >= a.nip || a.onnode[ip] >= 0) return;
  int o = a.poff[ip];
  const int o1 = a.poff[ip + 1];
  for (int e0 = 0; e0 < m.ne && o < o1; e0 += 32) {
    const int e = e0 + l;
    bool q = false;
    if (e < m.ne) {
      const size_t id = (size_t)ip * m.ne + e;
      const uint8_t s = a.cls_s[id], h = a.cls_h[id];
      q = s != CLS_SING && h != CLS_SING && (s == CLS_ADP || h == CLS_ADP);
    }
    const unsigned mq = __ballot_sync(0xffffffffu, q);
    if (q) {
      const int j = o + __popc(mq & ((1u << l) - 1u));
      a.pair_e[j] = e;
      a.pair_ip[j] = ip;
    }
    o += __popc(mq);
  }
}

// weighted sums of the element's nodal values at one quadrature point
template <typename T>
__device__ __forceinline__ void ip_weights(const T* un, const T* tn, const double w[8], T uu[3], T ut[3]) {
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    uu[c] = VT<T>::zero();
    ut[c] = VT<T>::zero();
  }
#pragma unroll
  for (int kn = 0; kn < 8; ++kn)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      uu[c] = uu[c] + un[3 * kn + c] * w[kn];
      ut[c] = ut[c] + tn[3 * kn + c] * w[kn];
    }
}

// One quasi-singular (point, element) pair and frequency per thread: the
// subdivision tree of sbie_ext_adp / hbie_ext_adp (bem_staela3d.f90:973-1096,
// 4790-4914) walked depth-first with an explicit stack, every leaf integrated
// with its Telles-mapped rule (sbie_ext_st / hbie_ext_st) as it is reached.
template <class POL>
__global__ void k_ip_adp(DMesh m, IpArgs a, POL pol, const QsCurves* __restrict__ qs) {
  typedef typename POL::T T;
  const long long id = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (id >= (long long)a.npairs * a.nf) return;
  const int pr = (int)(id % a.npairs), f = (int)(id / a.npairs);
  const int ip = a.pair_ip[pr], e = a.pair_e[pr];
  const double* xi = a.xip + 3 * (size_t)ip;
  double xr[3];
  ip_ref(a, xi, xr);
  const double* x = m.ex + 24 * (size_t)e;
  const T* uv = (const T*)a.uval + (size_t)f * a.nn * 3;
  const T* tv = (const T*)a.tval + (size_t)f * a.nn * 3;
  T un[24], tn[24];
  for (int kn = 0; kn < 8; ++kn) {
    const int s = a.enode[8 * e + kn];
    for (int c = 0; c < 3; ++c) {
      un[3 * kn + c] = uv[3 * s + c];
      tn[3 * kn + c] = tv[3 * s + c];
    }
  }
  const double rs = (m.rev[e] & 1) ? -1.0 : 1.0;
  T du[3], sg[3][3];
  for (int c = 0; c < 3; ++c) {
    du[c] = VT<T>::zero();
    for (int k = 0; k < 3; ++k) sg[c][k] = VT<T>::zero();
  }
  const size_t cid = (size_t)ip * m.ne + e;
#pragma unroll 1
  for (int h = 0; h < 2; ++h) {
    if ((h ? a.cls_h[cid] : a.cls_s[cid]) != CLS_ADP) continue;
    const int F = h ? 7 : 5;
    AdpNode st[52];
    int top = 0;
    st[0].xs[0] = -1; st[0].xs[1] = -1; st[0].xs[2] = 1; st[0].xs[3] = -1;
    st[0].xs[4] = 1;  st[0].xs[5] = 1;  st[0].xs[6] = -1; st[0].xs[7] = 1;
    st[0].ks = 1;
    top = 1;
    while (top > 0) {
      const AdpNode nd = st[--top];
      double bx[2], rmin, d;
      int method;
      if (nd.ks == 1) {
        nearest_q8(x, m.cl[e], xr, bx, &rmin, &d, &method);
      } else {
        double xsub[24];
        subdiv_q8(x, nd.xs, xsub);
        nearest_q8(xsub, clen_q8(xsub, 1e-12), xr, bx, &rmin, &d, &method);
      }
      int gn = qs_estimate(*qs, 2, F, d, bx, true);
      bool sub = false;
      if (nd.ks == m.ns_max) {
        if (gn == 0) gn = 30;
      } else if (gn == 0) {
        sub = true;
      }
      if (sub && top + 4 <= 52) {
        const double* s = nd.xs;
        const double c0 = 0.25 * (s[0] + s[2] + s[4] + s[6]), c1 = 0.25 * (s[1] + s[3] + s[5] + s[7]);
        const double q[4][8] = {
            {s[0], s[1], 0.5 * (s[0] + s[2]), 0.5 * (s[1] + s[3]), c0, c1, 0.5 * (s[0] + s[6]), 0.5 * (s[1] + s[7])},
            {0.5 * (s[0] + s[2]), 0.5 * (s[1] + s[3]), s[2], s[3], 0.5 * (s[2] + s[4]), 0.5 * (s[3] + s[5]), c0, c1},
            {c0, c1, 0.5 * (s[2] + s[4]), 0.5 * (s[3] + s[5]), s[4], s[5], 0.5 * (s[4] + s[6]), 0.5 * (s[5] + s[7])},
            {0.5 * (s[0] + s[6]), 0.5 * (s[1] + s[7]), c0, c1, 0.5 * (s[4] + s[6]), 0.5 * (s[5] + s[7]), s[6], s[7]}};
        for (int i = 3; i >= 0; --i) {
          for (int j = 0; j < 8; ++j) st[top].xs[j] = q[i][j];
          st[top].ks = nd.ks + 1;
          ++top;
        }
        continue;
      }
      // leaf: Telles-mapped rule of order max(gn, gln_far) on the sub-square
      const int g = max(gn, m.gln_far[e]);
      const double barr = telles_barr(d);
      const Telles t1 = telles11(bx[0], barr), t2 = telles11(bx[1], barr);
      for (int k1 = 1; k1 <= g; ++k1) {
        double xp1, jt1;
        telles_map(t1, gl11x(k1, g), xp1, jt1);
        for (int k2 = 1; k2 <= g; ++k2) {
          double xp2, jt2;
          telles_map(t2, gl11x(k2, g), xp2, jt2);
          double sp[4], sd1[4], sd2[4];
          phi_q4(xp1, xp2, sp);
          dphi_q4(xp1, xp2, sd1, sd2);
          double xa = 0, xb = 0, a11 = 0, a12 = 0, a21 = 0, a22 = 0;
          for (int qq = 0; qq < 4; ++qq) {
            xa += sp[qq] * nd.xs[2 * qq];
            xb += sp[qq] * nd.xs[2 * qq + 1];
            a11 += sd1[qq] * nd.xs[2 * qq];
            a12 += sd1[qq] * nd.xs[2 * qq + 1];
            a21 += sd2[qq] * nd.xs[2 * qq];
            a22 += sd2[qq] * nd.xs[2 * qq + 1];
          }
          const double js = a11 * a22 - a12 * a21;
          double xq[3], T1[3], T2[3], phi[8], N[3];
          geom_q8(x, xa, xb, xq, T1, T2, phi);
          cross3(T1, T2, N);
          const double jg = norm3(N);
          const double n[3] = {N[0] / jg, N[1] / jg, N[2] / jg};
          const double rv[3] = {xq[0] - xr[0], xq[1] - xr[1], xq[2] - xr[2]};
          const double jw = jg * js * jt1 * jt2 * gl11w(k1, g) * gl11w(k2, g);
          double w[8];
          for (int qq = 0; qq < 8; ++qq) w[qq] = phi[qq] * jw;
          T uu[3], ut[3];
          ip_weights<T>(un, tn, w, uu, ut);
          if (h) pol.hbie(f, xi, rv, n, ut, uu, rs, sg);
          else pol.sbie(f, xi, rv, n, ut, uu, rs, du);
        }
      }
    }
  }
  // the layout of out: u, then sigma(:, kc) for kc = 0..2
  T* sl = (T*)a.slot + ((size_t)f * a.npairs + pr) * 12;
  for (int c = 0; c < 3; ++c) {
    sl[c] = du[c];
    for (int k = 0; k < 3; ++k) sl[3 + 3 * k + c] = sg[c][k];
  }
}

// One warp per (point, frequency): the precalculated-rule pairs of every
// element on the lanes, then the point's quasi-singular slots in element order.
template <class POL, int WPB>
__global__ void __launch_bounds__(WPB * 32) k_ip_reg(DMesh m, IpArgs a, POL pol) {
  typedef typename POL::T T;
  __shared__ T nv[WPB][48];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const long long gw = blockIdx.x * (long long)WPB + w;
  if (gw >= (long long)a.nip * a.nf) return;
  const int ip = (int)(gw % a.nip), f = (int)(gw / a.nip);
  T* o = (T*)a.out + ((size_t)f * a.nip + ip) * 12;
  const T* uv = (const T*)a.uval + (size_t)f * a.nn * 3;
  const T* tv = (const T*)a.tval + (size_t)f * a.nn * 3;
  const int on = a.onnode[ip];
  if (on >= 0) {
    if (lane < 12) o[lane] = (lane < 3 && !a.image) ? uv[3 * on + lane] : VT<T>::zero();
    return;
  }
  const double* xi = a.xip + 3 * (size_t)ip;
  double xr[3];
  ip_ref(a, xi, xr);
  T du[3], sg[3][3];
  for (int c = 0; c < 3; ++c) {
    du[c] = VT<T>::zero();
    for (int k = 0; k < 3; ++k) sg[c][k] = VT<T>::zero();
  }
  for (int e = 0; e < m.ne; ++e) {
    const size_t cid = (size_t)ip * m.ne + e;
    const uint8_t cs = a.cls_s[cid], ch = a.cls_h[cid];
    if (cs == CLS_SING || ch == CLS_SING) continue;
    if (cs >= CLS_ADP && ch >= CLS_ADP) continue;
    __syncwarp();
    for (int j = lane; j < 48; j += 32) {
      const int kn = (j % 24) / 3, c = j % 3, s = a.enode[8 * e + kn];
      nv[w][j] = j < 24 ? uv[3 * s + c] : tv[3 * s + c];
    }
    __syncwarp();
    const double rs = (m.rev[e] & 1) ? -1.0 : 1.0;
#pragma unroll 1
    for (int h = 0; h < 2; ++h) {
      const uint8_t c = h ? ch : cs;
      if (c >= CLS_ADP) continue;
      const int P = m.ps_gln[c] * m.ps_gln[c];
      for (int k = lane; k < P; k += 32) {
        const size_t pt = (size_t)e * m.ptot + m.ps_off[c] + k;
        const double rv[3] = {m.px[3 * pt] - xr[0], m.px[3 * pt + 1] - xr[1], m.px[3 * pt + 2] - xr[2]};
        const double n[3] = {m.pn[3 * pt], m.pn[3 * pt + 1], m.pn[3 * pt + 2]};
        double wq[8];
        for (int q = 0; q < 8; ++q) wq[q] = m.pphi[8 * pt + q];
        T uu[3], ut[3];
        ip_weights<T>(nv[w], nv[w] + 24, wq, uu, ut);
        if (h) pol.hbie(f, xi, rv, n, ut, uu, rs, sg);
        else pol.sbie(f, xi, rv, n, ut, uu, rs, du);
      }
    }
  }
  T acc[12];
  for (int c = 0; c < 3; ++c) {
    acc[c] = du[c];
    for (int k = 0; k < 3; ++k) acc[3 + 3 * k + c] = sg[c][k];
  }
  for (int j = 0; j < 12; ++j)
    for (int off = 16; off > 0; off >>= 1) acc[j] = acc[j] + shfl_x(acc[j], off);
  if (lane == 0) {
    const T* sl = (const T*)a.slot;
    for (int pr = a.poff[ip]; pr < a.poff[ip + 1]; ++pr)
      for (int j = 0; j < 12; ++j) acc[j] = acc[j] + sl[((size_t)f * a.npairs + pr) * 12 + j];
    for (int j = 0; j < 12; ++j) o[j] = acc[j];
  }
}

}  // namespace mfb
