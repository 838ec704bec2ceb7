// Per-integration-point evaluation of the fundamental solutions (without their
// constant factors), device side.
//   static (Kelvin):      lib/fbem/src/bem_staela3d.f90:622-633
//   time-harmonic (Stokes): lib/fbem/src/bem_harela3d.f90:654-688, with the
//   decomposed exponential E_n(z) of lib/fbem/src/numerical.f90:1258-1331
#pragma once
#include "dev_complex.cuh"

namespace mfb {

struct StaelaP {
  double cteu1, cteu2, ctet1, ctet2;
};

// Number of series terms of numerical.f90:1286-1290 for 1e-6 < |z| <= 1:
// n = nint(10^(1.176 + 0.175 log10|z|)), a step function of |z|. Its steps sit
// at |z| = ((k + 1/2) / 10^1.176)^(1/0.175); the table holds their squares
// (filled on the host by zexp_thresholds()), so the device decides n with four
// comparisons on |z|^2 instead of evaluating log10 and pow in FP64.
struct ZexpSteps {
  double t2[16];  // t2[k-1]: |z|^2 at which n becomes k+1 (k = 1..14), t2[14] = +inf
};
__host__ inline ZexpSteps zexp_thresholds() {
  ZexpSteps s;
  const double c = pow(10.0, 1.176);
  for (int k = 1; k <= 14; ++k) {
    double t = pow((k + 0.5) / c, 1.0 / 0.175);
    s.t2[k - 1] = t * t;
  }
  s.t2[14] = s.t2[15] = 1e300;
  return s;
}
__device__ __forceinline__ int zexp_nterms(const ZexpSteps& s, double az2) {
  if (az2 <= 1e-12) return 1;
  // smallest k with az2 < t2[k-1] gives n = k (n = 15 above the last step)
  int lo = 0, hi = 15;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (az2 < s.t2[mid]) hi = mid;
    else lo = mid + 1;
  }
  return lo + 1;
}

// u* / t* coefficient block of fbem_bem_harela3d_parameters (bem_harela3d.f90:118-134)
struct HarParD {
  cd k1, k2;
  cd psi[6], chi[6];
  cd T1[10], T2[9], T3[9];
  cd cte_u, cte_t;
  ZexpSteps steps;
};

__host__ __device__ inline StaelaP staela_params(double mu, double nu) {
  StaelaP p;
  p.cteu1 = 1.0 / (16.0 * kPi * mu * (1.0 - nu));
  p.cteu2 = 3.0 - 4.0 * nu;
  p.ctet1 = -1.0 / (8.0 * kPi * (1.0 - nu));
  p.ctet2 = 1.0 - 2.0 * nu;
  return p;
}

// fbem_bem_harela3d_calculate_parameters (bem_harela3d.f90:143-287), u*/t* part
__host__ __device__ inline HarParD harela_params(cd lambda, cd mu, double rho, double omega) {
  HarParD p;
  const cd I = mk(0.0, 1.0);
  cd c1 = csqrt_((lambda + 2.0 * mu) / rho);
  cd c2 = csqrt_(mu / rho);
  cd k1 = omega / c1, k2 = omega / c2;
  p.k1 = k1;
  p.k2 = k2;
  cd c1p2 = c1 * c1, c2p2 = c2 * c2, c1p3 = c1p2 * c1, c1p4 = c1p2 * c1p2;
  cd k2p2 = k2 * k2;
  cd ik1 = I * k1, ik2 = I * k2, ik1p2 = ik1 * ik1, ik2p2 = ik2 * ik2;
  cd r = c2p2 / c1p2;
  double om2 = omega * omega;
  p.psi[0] = 0.5 * (1.0 + r);
  p.psi[1] = (-1.0 / 3.0 * (2.0 / c2 + c2p2 / c1p3)) * I * omega;
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
  p.T1[5] = mk(12.0);
  p.T1[6] = -r * 30.0 / ik1;
  p.T1[7] = 30.0 / ik2;
  p.T1[8] = -r * 30.0 / ik1p2;
  p.T1[9] = 30.0 / ik2p2;
  p.T2[0] = -r;
  p.T2[1] = -0.25 * (1.0 / c2p2 + c2p2 / c1p4) * om2;
  p.T2[2] = -I * k2;
  p.T2[3] = 2.0 * r;
  p.T2[4] = mk(-3.0);
  p.T2[5] = r * 6.0 / ik1;
  p.T2[6] = -6.0 / ik2;
  p.T2[7] = r * 6.0 / ik1p2;
  p.T2[8] = -6.0 / ik2p2;
  p.T3[0] = r;
  p.T3[1] = 0.25 * (3.0 * c2p2 / c1p4 - 2.0 / c1p2 + 1.0 / c2p2) * om2;
  p.T3[2] = (2.0 * r - 1.0) * I * k1;
  p.T3[3] = 4.0 * r - 1.0;
  p.T3[4] = mk(-2.0);
  p.T3[5] = r * 6.0 / ik1;
  p.T3[6] = -6.0 / ik2;
  p.T3[7] = r * 6.0 / ik1p2;
  p.T3[8] = -6.0 / ik2p2;
  p.cte_u = k1_4Pi / mu;
  p.cte_t = mk(k1_4Pi);
  return p;
}

// E_2..E_5 of z (numerical.f90:1258-1331): E_n(z) = e^z - sum_{k<n} z^k/k!.
// For |z|<=1 the reference sums the series tail from k=n+6 down to 6; the same
// terms are summed here in nested (Horner) form.
__device__ __forceinline__ void zexp_2to5(const ZexpSteps& steps, cd z, cd& E2, cd& E3, cd& E4, cd& E5) {
  double az2 = z.re * z.re + z.im * z.im;
  cd z2 = z * z, z3 = z2 * z, z4 = z3 * z;
  if (az2 <= 1.0) {
    int N = zexp_nterms(steps, az2) + 6;
    cd t = mk(1.0);
    for (int k = N; k >= 7; --k) t = 1.0 + t * z * (1.0 / (double)k);
    cd z5 = z4 * z, z6 = z5 * z;
    cd e6 = (z6 * (1.0 / 720.0)) * t;
    E5 = e6 + z5 * (1.0 / 120.0);
    E4 = E5 + z4 * (1.0 / 24.0);
    E3 = E4 + z3 * (1.0 / 6.0);
    E2 = E3 + z2 * 0.5;
  } else {
    cd e0 = cexp_(z);
    cd e1 = e0 - 1.0;
    E2 = e1 - z;
    E3 = E2 - 0.5 * z2;
    E4 = E3 - (1.0 / 6.0) * z3;
    E5 = E4 - (1.0 / 24.0) * z4;
  }
}

// Regular-point harmonic fundamental solutions: fu[3*il+ik] = u*_{il,ik}/cte_u,
// ft[...] = t*_{il,ik}/cte_t.  With full == false the 1/r^2 terms of TT1..TT3
// are dropped (bem_harela3d.f90 sbie_int); the caller adds them back.
__device__ __forceinline__ void harela_coeffs(const HarParD& p, double r, cd& psi, cd& chi, cd& TT1, cd& TT2,
                                              cd& TT3, double& d1r1, double& d1r2, bool full) {
  d1r1 = 1.0 / r;
  d1r2 = d1r1 * d1r1;
  double d1r3 = d1r2 * d1r1, d1r4 = d1r3 * d1r1;
  cd z1 = mk(p.k1.im * r, -p.k1.re * r);  // -i k1 r
  cd z2 = mk(p.k2.im * r, -p.k2.re * r);
  cd a2, a3, a4, a5, b2, b3, b4, b5;
  zexp_2to5(p.steps, z1, a2, a3, a4, a5);
  zexp_2to5(p.steps, z2, b2, b3, b4, b5);
  a2 = a2 * d1r1; b2 = b2 * d1r1;
  a3 = a3 * d1r2; b3 = b3 * d1r2;
  a4 = a4 * d1r3; b4 = b4 * d1r3;
  a5 = a5 * d1r4; b5 = b5 * d1r4;
  psi = p.psi[0] * d1r1 + p.psi[1] + b2 + p.psi[2] * a3 + p.psi[3] * b3 + p.psi[4] * a4 + p.psi[5] * b4;
  chi = p.chi[0] * d1r1 + p.chi[1] * a2 + b2 + p.chi[2] * a3 + p.chi[3] * b3 + p.chi[4] * a4 + p.chi[5] * b4;
  TT1 = p.T1[1] + p.T1[2] * a2 + p.T1[3] * b2 + p.T1[4] * a3 + p.T1[5] * b3 + p.T1[6] * a4 + p.T1[7] * b4 +
        p.T1[8] * a5 + p.T1[9] * b5;
  TT2 = p.T2[1] + p.T2[2] * b2 + p.T2[3] * a3 + p.T2[4] * b3 + p.T2[5] * a4 + p.T2[6] * b4 + p.T2[7] * a5 +
        p.T2[8] * b5;
  TT3 = p.T3[1] + p.T3[2] * a2 + p.T3[3] * a3 + p.T3[4] * b3 + p.T3[5] * a4 + p.T3[6] * b4 + p.T3[7] * a5 +
        p.T3[8] * b5;
  if (full) {
    TT1 = TT1 + p.T1[0] * d1r2;
    TT2 = TT2 + p.T2[0] * d1r2;
    TT3 = TT3 + p.T3[0] * d1r2;
  }
}

__device__ __forceinline__ void harela_point(const HarParD& p, const double rv[3], const double n[3], cd fu[9],
                                             cd ft[9]) {
  double r = sqrt(rv[0] * rv[0] + rv[1] * rv[1] + rv[2] * rv[2]);
  cd psi, chi, TT1, TT2, TT3;
  double d1r1, d1r2;
  harela_coeffs(p, r, psi, chi, TT1, TT2, TT3, d1r1, d1r2, true);
  double dr[3] = {rv[0] * d1r1, rv[1] * d1r1, rv[2] * d1r1};
  double drdn = dr[0] * n[0] + dr[1] * n[1] + dr[2] * n[2];
#pragma unroll
  for (int il = 0; il < 3; ++il)
#pragma unroll
    for (int ik = 0; ik < 3; ++ik) {
      double rr = dr[il] * dr[ik];
      cd u = -(chi * rr);
      cd t = TT1 * (rr * drdn) + TT2 * (dr[ik] * n[il]) + TT3 * (dr[il] * n[ik]);
      if (il == ik) {
        u = u + psi;
        t = t + TT2 * drdn;
      }
      fu[3 * il + ik] = u;
      ft[3 * il + ik] = t;
    }
}

__device__ __forceinline__ void staela_point(const StaelaP& k, const double rv[3], const double n[3], double fu[9],
                                             double ft[9]) {
  double r = sqrt(rv[0] * rv[0] + rv[1] * rv[1] + rv[2] * rv[2]);
  double d1r = 1.0 / r, d1r2 = d1r * d1r;
  double dr[3] = {rv[0] * d1r, rv[1] * d1r, rv[2] * d1r};
  double drdn = dr[0] * n[0] + dr[1] * n[1] + dr[2] * n[2];
#pragma unroll
  for (int il = 0; il < 3; ++il)
#pragma unroll
    for (int ik = 0; ik < 3; ++ik) {
      double dk = (il == ik) ? 1.0 : 0.0;
      fu[3 * il + ik] = d1r * (k.cteu2 * dk + dr[il] * dr[ik]);
      ft[3 * il + ik] = d1r2 * ((k.ctet2 * dk + 3.0 * dr[il] * dr[ik]) * drdn + k.ctet2 * (n[il] * dr[ik] - n[ik] * dr[il]));
    }
}

// Complementary part of Mindlin's fundamental solution for the half-space
// x3 >= xp with the traction-free surface x3 = xp (fbem_bem_staela3d_hsc_sbie,
// bem_staela3d.f90:7438-7563), without its constants: fu = 16 pi mu (1 - nu) u,
// ft = 8 pi (1 - nu) t, [3 * load + component]. Inputs: the horizontal offsets
// rv1, rv2 of x from x_i, c = x_i3 - xp, z = x3 - xp, and rpz, the vertical
// offset of x from the image point as the reference forms it (x3 + x_i3). The
// normal load's cylindrical fields are turned to global axes with
// cos = rv1 / r, sin = rv2 / r (cos = 1, sin = 0 on the axis r = 0, where
// the reference's atan2 gives theta = 0).
__device__ __forceinline__ void hsc_point(double nu, double rv1, double rv2, double c, double z, double rpz,
                                          const double n[3], double fu[9], double ft[9]) {
  const double c1 = 1.0 - nu, c2 = 1.0 - 2.0 * nu, c3 = 3.0 - 2.0 * nu, c4 = 3.0 - 4.0 * nu, c5 = 5.0 - 4.0 * nu;
  const double k12 = 4.0 * c1 * c2;
  const double a1 = rv1 * rv1, a2 = rv2 * rv2, rh2 = a1 + a2;
  const double rp = sqrt(rh2 + rpz * rpz);
  const double rp2 = rp * rp, i1 = 1.0 / rp, i2 = 1.0 / rp2, i3 = i1 * i2, i5 = i3 * i2, i7 = i5 * i2;
  const double zc = z + c, q = rp + zc, iq = 1.0 / q, b1 = 3.0 * rp + zc;
  const double K = k12 * i1 * iq * iq;  // 4 c1 c2 / (rp q^2)
  // tangential loads (l = 0, 1): displacements
  const double A = c4 * i3 - 6.0 * c * z * i5 - K;
  const double B = c4 * (z - c) * i3 - 6.0 * c * z * zc * i5 + k12 * i1 * iq;
  const double rv[2] = {rv1, rv2}, aa[2] = {a1, a2};
  for (int l = 0; l < 2; ++l) {
    const double a = rv[l], b = rv[1 - l], al = aa[l], bl = aa[1 - l];
    fu[3 * l + l] = i1 + c4 * al * i3 + 2.0 * c * z * i3 * (1.0 - 3.0 * al * i2) + k12 * iq * (1.0 - al * i1 * iq);
    fu[3 * l + 1 - l] = rv1 * rv2 * A;
    fu[3 * l + 2] = a * B;
    // stresses of the load along l: along (l), across (m) and vertical (3)
    const double sll = a * (c2 * c5 * i3 - 3.0 * c4 * al * i5 - K * (3.0 - al * b1 * i2 * iq) +
                            6.0 * c * i5 * (3.0 * c - c3 * zc + 5.0 * al * z * i2));
    const double smm = a * (c2 * c4 * i3 - 3.0 * c4 * bl * i5 - K * (1.0 - bl * b1 * i2 * iq) +
                            6.0 * c * i5 * (c - c2 * zc + 5.0 * bl * z * i2));
    const double s33 = a * (-c2 * i3 - 3.0 * c4 * zc * zc * i5 + 6.0 * c * i5 * (c + c2 * zc + 5.0 * z * zc * zc * i2));
    const double sm3 = rv1 * rv2 * (-3.0 * c4 * zc * i5 + 6.0 * c * i5 * (c2 + 5.0 * z * zc * i2));
    const double sl3 = c2 * (z - c) * i3 - 3.0 * c4 * al * zc * i5 - 6.0 * c * i5 * (z * zc - c2 * al - 5.0 * al * z * zc * i2);
    const double slm = b * (c2 * i3 - 3.0 * c4 * al * i5 - K * (1.0 - al * b1 * i2 * iq) - 6.0 * c * z * i5 * (1.0 - 5.0 * al * i2));
    const double nl = n[l], nm = n[1 - l], n3 = n[2];
    ft[3 * l + l] = sll * nl + slm * nm + sl3 * n3;
    ft[3 * l + 1 - l] = slm * nl + smm * nm + sm3 * n3;
    ft[3 * l + 2] = sl3 * nl + sm3 * nm + s33 * n3;
  }
  // normal load (l = 2)
  const double V = c4 * (z - c) * i3 - k12 * i1 * iq + 6.0 * c * z * zc * i5;
  fu[6] = rv1 * V;
  fu[7] = rv2 * V;
  fu[8] = (8.0 * c1 * c1 - c4) * i1 + (c4 * zc * zc - 2.0 * c * z) * i3 + 6.0 * c * z * zc * zc * i5;
  const double srr = -c2 * (z + 7.0 * c) * i3 + k12 * i1 * iq +
                     (6.0 * c * c2 * zc * zc - 6.0 * c * c * zc - 3.0 * c4 * rh2 * (z - c)) * i5 - 30.0 * c * rh2 * z * zc * i7;
  const double stt = c2 * (c4 * zc - 6.0 * c) * i3 - k12 * i1 * iq + 6.0 * c2 * c * zc * zc * i5 - 6.0 * c * c * zc * i5;
  const double s33 = c2 * (z - c) * i3 - (3.0 * c4 * z * zc * zc - 3.0 * c * zc * (5.0 * z - c)) * i5 - 30.0 * c * z * zc * zc * zc * i7;
  const double E = c2 * i3 - (3.0 * c4 * z * zc - 3.0 * c * (3.0 * z + c)) * i5 - 30.0 * c * z * zc * zc * i7;
  double cc = 1.0, ss = 0.0, cs = 0.0;
  if (rh2 > 0.0) {
    const double ir2 = 1.0 / rh2;
    cc = a1 * ir2;
    ss = a2 * ir2;
    cs = rv1 * rv2 * ir2;
  }
  const double sxx = cc * srr + ss * stt, syy = ss * srr + cc * stt, sxy = cs * (srr - stt);
  const double sxz = rv1 * E, syz = rv2 * E;
  ft[6] = sxx * n[0] + sxy * n[1] + sxz * n[2];
  ft[7] = sxy * n[0] + syy * n[1] + syz * n[2];
  ft[8] = sxz * n[0] + syz * n[1] + s33 * n[2];
}

// The complementary displacement kernel on the free surface itself, as the
// singular integration of fbem_bem_staela3d_hsc_sbie_int integrates it
// (bem_staela3d.f90:8815-8829), times 16 pi mu (1 - nu): r = |x - x_i|,
// dr = (x - x_i) / r, z = x3 - xp.
__device__ __forceinline__ void hsc_surface_g(double nu, double r, const double dr[3], double z, double fu[9]) {
  const double a = 3.0 - 4.0 * nu, b = 4.0 * (1.0 - nu) * (1.0 - 2.0 * nu), d1r = 1.0 / r;
  const double is = 1.0 / (r + z);
  fu[0] = d1r + a * dr[0] * dr[0] * d1r + b * is * (1.0 - dr[0] * dr[0] * r * is);
  fu[1] = a * dr[0] * dr[1] * d1r - b * dr[0] * dr[1] * r * is * is;
  fu[2] = a * dr[0] * dr[2] * d1r + b * dr[0] * is;
  fu[3] = fu[1];
  fu[4] = d1r + a * dr[1] * dr[1] * d1r + b * is * (1.0 - dr[1] * dr[1] * r * is);
  fu[5] = a * dr[1] * dr[2] * d1r + b * dr[1] * is;
  fu[6] = a * dr[0] * dr[2] * d1r - b * dr[0] * is;
  fu[7] = a * dr[1] * dr[2] * d1r - b * dr[1] * is;
  fu[8] = (8.0 * (1.0 - nu) * (1.0 - nu) - a) * d1r + a * dr[2] * dr[2] * d1r;
}

}  // namespace mfb
