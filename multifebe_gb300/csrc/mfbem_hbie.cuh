// HBIE (traction boundary integral equation) collocated on the boundary: the
// 'hbie' and 'dual_bm_same' (Burton & Miller) formulations of ordinary
// boundaries (src/read_bem_formulation_selected_nodes.f90:70-260) in both
// region builders. The HBIE collocation points (element(se)%x_i_hbie, one per
// element of each node, moved into the element) form their own view of the
// mesh with their own pair lists, classified like hbie_auto with the 1/r^7
// estimate (bem_staela3d.f90:4307-4373, bem_harela3d.f90:3632-3697):
//   regular / adaptive pairs  k_reg / k_adp with the PolHbie* policies below
//                             (d* into l, s* into m: hbie_ext_pre / _ext_st);
//   singular pairs            k_hsing, the interior (hypersingular)
//                             integration of hbie_int (bem_staela3d.f90:
//                             4918-5353, bem_harela3d.f90:3169-3630);
//   free terms                k_hfree (-1/2 phi(xi_i) on l, and 1/2 phi(xi_i)
//                             on h for Burton & Miller).
// Each point's equation is h = m, g = l ('hbie'), or adds beta (m, l) to the
// SBIE at the same point (Burton & Miller, 'dual_bm_same') or to the node's
// SBIE at its own nodal / MCA point ('dual_bm_mixed', whose SBIE points sit in
// the SBIE view): beta = alpha in the static builder
// (build_lse_mechanics_bem_staela.f90:835-841), alpha i / c2 in the harmonic
// one (build_lse_mechanics_bem_harela.f90:1174-1181, c2 the complex S-wave
// speed). beta is folded into the integrands here, so the rows of both views
// simply add into A and b. Crack-like nodes put their HBIE in rows of their
// own (k_hfree and the scatter).
#pragma once

namespace mfb {

// HBIE points weighted by the Burton & Miller factor beta alpha: kind 3
// ('dual_bm_same') and 5 ('dual_bm_mixed'); kinds 2 ('hbie') and 4
// (crack-like node) take weight 1.
__host__ __device__ __forceinline__ bool hbie_weighted(int kind) { return kind == 3 || kind == 5; }

// d* (fd, integrated into l) and s* (fs, into m) at one point for the
// collocation normal ni, without their constants.
// Static: bem_staela3d.f90:4376-4446 (cted1, ctes1 applied by the flush).
__device__ __forceinline__ void hbie_point_s(double nu, double cted2, double ctes2, double ctes3, const double rv[3],
                                             const double n[3], const double ni[3], double fd[9], double fs[9]) {
  const double r = sqrt(rv[0] * rv[0] + rv[1] * rv[1] + rv[2] * rv[2]);
  const double d1r = 1.0 / r, d1r2 = d1r * d1r, d1r3 = d1r2 * d1r;
  const double dr[3] = {rv[0] * d1r, rv[1] * d1r, rv[2] * d1r};
  const double drdn = dr[0] * n[0] + dr[1] * n[1] + dr[2] * n[2];
  const double drdni = -(dr[0] * ni[0] + dr[1] * ni[1] + dr[2] * ni[2]);
  const double nni = n[0] * ni[0] + n[1] * ni[1] + n[2] * ni[2];
#pragma unroll
  for (int il = 0; il < 3; ++il)
#pragma unroll
    for (int ik = 0; ik < 3; ++ik) {
      const double dk = il == ik ? 1.0 : 0.0;
      fd[3 * il + ik] = d1r2 * ((cted2 * dk + 3.0 * dr[il] * dr[ik]) * drdni + cted2 * (ni[il] * dr[ik] - ni[ik] * dr[il]));
      fs[3 * il + ik] = d1r3 * (3.0 * (5.0 * dr[il] * dr[ik] - nu * dk) * drdn * drdni +
                                3.0 * ctes2 * (dr[ik] * ni[il] * drdn - dr[il] * n[ik] * drdni) +
                                3.0 * nu * (dr[il] * ni[ik] * drdn - dr[ik] * n[il] * drdni) +
                                (3.0 * nu * dr[il] * dr[ik] + ctes2 * dk) * nni + ctes2 * n[il] * ni[ik] -
                                ctes3 * n[ik] * ni[il]);
    }
}

// E_n-decomposed coefficient functions of d* and s* (bem_harela3d.f90:
// 2573-2662). With `full` the 1/r^2 (T) and 1/r^3 (S) terms are included; the
// interior integration takes the regular parts only (bem_harela3d.f90:3480-3500).
struct HbieCoefH {
  cd TT1, TT2, TT3, S1, S2, S3, S4, S5;
};
__device__ __forceinline__ void hbie_coef_h(const HarParD& q, const HarParH& s, double r, bool full, HbieCoefH& c) {
  const double d1r1 = 1.0 / r, d1r2 = d1r1 * d1r1, d1r3 = d1r2 * d1r1, d1r4 = d1r3 * d1r1, d1r5 = d1r4 * d1r1;
  cd a[7], b[7];
  zexp_2to6(q.steps, mk(q.k1.im * r, -q.k1.re * r), a);
  zexp_2to6(q.steps, mk(q.k2.im * r, -q.k2.re * r), b);
  const double sc[7] = {0.0, 0.0, d1r1, d1r2, d1r3, d1r4, d1r5};
#pragma unroll
  for (int j = 2; j < 7; ++j) {
    a[j] = a[j] * sc[j];
    b[j] = b[j] * sc[j];
  }
  const double f2 = full ? d1r2 : 0.0, f3 = full ? d1r3 : 0.0;
  c.TT1 = q.T1[0] * f2 + q.T1[1] + q.T1[2] * a[2] + q.T1[3] * b[2] + q.T1[4] * a[3] + q.T1[5] * b[3] + q.T1[6] * a[4] +
          q.T1[7] * b[4] + q.T1[8] * a[5] + q.T1[9] * b[5];
  c.TT2 = q.T2[0] * f2 + q.T2[1] + q.T2[2] * b[2] + q.T2[3] * a[3] + q.T2[4] * b[3] + q.T2[5] * a[4] + q.T2[6] * b[4] +
          q.T2[7] * a[5] + q.T2[8] * b[5];
  c.TT3 = q.T3[0] * f2 + q.T3[1] + q.T3[2] * a[2] + q.T3[3] * a[3] + q.T3[4] * b[3] + q.T3[5] * a[4] + q.T3[6] * b[4] +
          q.T3[7] * a[5] + q.T3[8] * b[5];
  c.S1 = s.S1[0] * f3 + s.S1[1] * d1r1 + s.S1[2] * b[2] + s.S1[3] * a[3] + s.S1[4] * b[3] + s.S1[5] * a[4] +
         s.S1[6] * b[4] + s.S1[7] * a[5] + s.S1[8] * b[5] + s.S1[9] * a[6] + s.S1[10] * b[6];
  c.S2 = s.S2[0] * f3 + s.S2[1] * d1r1 + s.S2[2] * a[2] + s.S2[3] * a[3] + s.S2[4] * b[3] + s.S2[5] * a[4] +
         s.S2[6] * b[4] + s.S2[7] * a[5] + s.S2[8] * b[5] + s.S2[9] * a[6] + s.S2[10] * b[6];
  c.S3 = s.S3[0] * f3 + s.S3[1] * d1r1 + s.S3[2] * a[2] + s.S3[3] * b[2] + s.S3[4] * a[3] + s.S3[5] * b[3] +
         s.S3[6] * a[4] + s.S3[7] * b[4] + s.S3[8] * a[5] + s.S3[9] * b[5] + s.S3[10] * a[6] + s.S3[11] * b[6];
  c.S4 = s.S4[0] * f3 + s.S4[1] * d1r1 + s.S4[2] + s.S4[3] * b[3] + s.S4[4] * a[4] + s.S4[5] * b[4] + s.S4[6] * a[5] +
         s.S4[7] * b[5] + s.S4[8] * a[6] + s.S4[9] * b[6];
  c.S5 = s.S5[0] * f3 + s.S5[1] * d1r1 + s.S5[2] + s.S5[3] * a[2] + s.S5[4] * a[3] + s.S5[5] * a[4] + s.S5[6] * b[4] +
         s.S5[7] * a[5] + s.S5[8] * b[5] + s.S5[9] * a[6] + s.S5[10] * b[6];
}

// Harmonic d* and s* at one point for the collocation normal ni (constants
// cte_d, cte_s applied by the flush).
__device__ __forceinline__ void hbie_point_h(const HarParD& q, const HarParH& s, const double rv[3], const double n[3],
                                             const double ni[3], cd fd[9], cd fs[9]) {
  const double r = sqrt(rv[0] * rv[0] + rv[1] * rv[1] + rv[2] * rv[2]);
  HbieCoefH c;
  hbie_coef_h(q, s, r, true, c);
  const double d1r = 1.0 / r;
  const double dr[3] = {rv[0] * d1r, rv[1] * d1r, rv[2] * d1r};
  const double drdn = dr[0] * n[0] + dr[1] * n[1] + dr[2] * n[2];
  const double drdni = -(dr[0] * ni[0] + dr[1] * ni[1] + dr[2] * ni[2]);
  const double nni = n[0] * ni[0] + n[1] * ni[1] + n[2] * ni[2];
#pragma unroll
  for (int il = 0; il < 3; ++il)
#pragma unroll
    for (int ik = 0; ik < 3; ++ik) {
      const double dk = il == ik ? 1.0 : 0.0;
      fd[3 * il + ik] = c.TT1 * (dr[il] * dr[ik] * drdni) - c.TT2 * (-drdni * dk + dr[il] * ni[ik]) - c.TT3 * (dr[ik] * ni[il]);
      fs[3 * il + ik] = c.S1 * (dr[il] * ni[ik] * drdn - dr[ik] * n[il] * drdni - dk * drdn * drdni + dr[il] * dr[ik] * nni) +
                        c.S2 * (dr[ik] * ni[il] * drdn - dr[il] * n[ik] * drdni) + c.S3 * (dr[il] * dr[ik] * drdn * drdni) +
                        c.S4 * (dk * nni + ni[ik] * n[il]) + c.S5 * (n[ik] * ni[il]);
    }
}

// Policies of k_reg / k_adp for the HBIE view: fu <- beta d*, ft <- beta s*;
// cte_u / cte_t are d*'s and s*'s constants; the flush reverses m with the
// element as hbie_ext_pre does (bem_staela3d.f90:4443). d* is not symmetric:
// all nine components are kept (NG = 9).
struct PolHbieStatic {
  typedef double T;
  static constexpr int NG = 9;
  double nu, cted1, cted2, ctes1, ctes2, ctes3;
  const double* cpn;    // [ncp][3] collocation normals
  const double* cpa;    // [ncp] Burton & Miller alpha
  const int* cpk;       // [ncp] kind: 2 HBIE alone, 3 Burton & Miller, 4 crack-like, 5 'dual_bm_mixed'
  __device__ T cte_t(int) const { return ctes1; }
  __device__ T cte_u(int) const { return cted1; }
  __device__ T cpv(int) const { return 0.0; }
  __device__ void point(int, int cp, const double rv[3], const double n[3], T fu[9], T ft[9]) const {
    hbie_point_s(nu, cted2, ctes2, ctes3, rv, n, cpn + 3 * (size_t)cp, fu, ft);
    if (hbie_weighted(cpk[cp])) {
      const double b = cpa[cp];
#pragma unroll
      for (int q = 0; q < 9; ++q) {
        fu[q] = b * fu[q];
        ft[q] = b * ft[q];
      }
    }
  }
};
struct PolHbieHarmonic {
  typedef cd T;
  static constexpr int NG = 9;
  const HarParD* p;
  const HarParH* ph;
  const double* cpn;
  const double* cpa;
  const int* cpk;
  __device__ T cte_t(int f) const { return ph[f].cte_s; }
  __device__ T cte_u(int f) const { return ph[f].cte_d; }
  __device__ T cpv(int) const { return mk(0.0); }
  __device__ void point(int f, int cp, const double rv[3], const double n[3], T fu[9], T ft[9]) const {
    hbie_point_h(p[f], ph[f], rv, n, cpn + 3 * (size_t)cp, fu, ft);
    if (hbie_weighted(cpk[cp])) {
      const cd b = cpa[cp] * ph[f].ic2;
#pragma unroll
      for (int q = 0; q < 9; ++q) {
        fu[q] = b * fu[q];
        ft[q] = b * ft[q];
      }
    }
  }
};
__host__ __device__ inline PolHbieStatic hbie_static_policy(double mu, double nu) {
  PolHbieStatic p{};
  p.nu = nu;
  p.cted1 = -1.0 / (8.0 * kPi * (1.0 - nu));
  p.cted2 = 1.0 - 2.0 * nu;
  p.ctes1 = mu / (4.0 * kPi * (1.0 - nu));
  p.ctes2 = 1.0 - 2.0 * nu;
  p.ctes3 = 1.0 - 4.0 * nu;
  return p;
}

// ---------------------------------------------------------------- singular pairs
// The interior integration written once for both kernels. With the
// coefficients of the 1/r^2 terms of d* (T1s, T2s) and the 1/r^3 terms of s*
// (S1s..S5s) -- static: 3, 1-2nu, 3nu, 3(1-2nu), 15, 1-2nu, -(1-4nu) with
// constants cted1, ctes1 (bem_staela3d.f90:5208-5275); harmonic: T1(1),
// T2(1), S1(1)..S5(1) with cte_d, cte_s and the regular parts of the
// E_n-decomposed functions (bem_harela3d.f90:3478-3593) -- one polar point
// contributes
//   l(kn) += fd w(kn) + fc wd(kn)
//   m(kn) += fsA w(kn) + fsR wd(kn) + phi_i(kn) P + psi_i(kn) . Q
// with w = phi jw, wd = (phi - phi_i) jw and the pair-level sums
//   P   = sum (M221 + M321) jw,
//   Q_j = sum (M231 n_j + M331_j - (M21 + M31) rv_j) jw,
// since phi - phi_i - psi_i . rv = (phi - phi_i) - psi_i . rv and phi_i, psi_i
// are constant over the pair. The edge line integrals enter P, Q and l at
// the flush.
template <typename T>
struct HsCoef {
  T T1s, T2s, S1s, S2s, S3s, S4s, S5s, cte_d, cte_s, bm;
};
struct HsStatic {
  typedef double T;
  static constexpr bool kDyn = false;
  double nu, cted1, cted2, ctes1, ctes2, ctes3;
  __device__ HsCoef<double> coef(int) const {
    return HsCoef<double>{3.0, cted2, 3.0 * nu, 3.0 * ctes2, 15.0, ctes2, -ctes3, cted1, ctes1, 1.0};
  }
  __device__ void dyn(int, double, HbieCoefH&) const {}
};
struct HsHarmonic {
  typedef cd T;
  static constexpr bool kDyn = true;
  const HarParD* p;
  const HarParH* ph;
  __device__ HsCoef<cd> coef(int f) const {
    const HarParD& q = p[f];
    const HarParH& s = ph[f];
    return HsCoef<cd>{q.T1[0], q.T2[0], s.S1[0], s.S2[0], s.S3[0], s.S4[0], s.S5[0], s.cte_d, s.cte_s, s.ic2};
  }
  __device__ void dyn(int f, double r, HbieCoefH& c) const { hbie_coef_h(p[f], ph[f], r, false, c); }
};

template <typename T>
struct alignas(16) ComboH {
  T A[9], R[9], D[9], C[9], PQ[36];
  double w[8], wd[8];
  int pair;
};
__device__ __forceinline__ double dyn_pick(const HbieCoefH&, double, double) { return 0.0; }

// One polar point: the 72 per-point values of the combination above.
template <class HS>
__device__ __forceinline__ void hsing_point(const HS& hs, int f, const HsCoef<typename HS::T>& k, const double rv[3],
                                            const double n[3], const double ni[3], double jw, ComboH<typename HS::T>& o) {
  typedef typename HS::T T;
  const double r = sqrt(rv[0] * rv[0] + rv[1] * rv[1] + rv[2] * rv[2]);
  const double d1r = 1.0 / r, d2 = d1r * d1r, d3 = d2 * d1r;
  const double dr[3] = {rv[0] * d1r, rv[1] * d1r, rv[2] * d1r};
  const double drdn = dr[0] * n[0] + dr[1] * n[1] + dr[2] * n[2];
  const double drdni = -(dr[0] * ni[0] + dr[1] * ni[1] + dr[2] * ni[2]);
  const double nni = n[0] * ni[0] + n[1] * ni[1] + n[2] * ni[2];
  const T z = VT<T>::zero();
  T TT1 = z, TT2 = z, TT3 = z, S1 = z, S2 = z, S3 = z, S4 = z, S5 = z;
  if constexpr (HS::kDyn) {
    HbieCoefH c;
    hs.dyn(f, r, c);
    TT1 = c.TT1; TT2 = c.TT2; TT3 = c.TT3;
    S1 = c.S1; S2 = c.S2; S3 = c.S3; S4 = c.S4; S5 = c.S5;
  }
  const T S1o3 = k.S1s * (1.0 / 3.0);
#pragma unroll 1
  for (int il = 0; il < 3; ++il)
#pragma unroll 1
    for (int ik = 0; ik < 3; ++ik) {
      const int q = 3 * il + ik;
      const double dk = il == ik ? 1.0 : 0.0;
      const double rr = dr[il] * dr[ik];
      // l: regular + the 1/r^2 part with (n_i - n), and L21 with (phi - phi_i)
      T fd = (TT1 + k.T1s * d2) * (rr * drdni) + (TT2 + k.T2s * d2) * (dk * drdni) - TT2 * (dr[il] * ni[ik]) -
             TT3 * (dr[ik] * ni[il]) + k.T2s * (d2 * ((ni[il] - n[il]) * dr[ik] - (ni[ik] - n[ik]) * dr[il]));
      o.D[q] = fd;
      o.C[q] = il != ik ? k.T2s * (d2 * (n[il] * dr[ik] - n[ik] * dr[il])) : z;
      // m with phi jw: regular parts, M1
      const double a1 = dr[il] * ni[ik] * drdn - dr[ik] * n[il] * drdni;  // S1 (and M31) bracket
      const double a2 = dr[ik] * ni[il] * drdn - dr[il] * n[ik] * drdni;  // S2 bracket
      o.A[q] = S1 * (a1 - dk * drdn * drdni + rr * nni) + S2 * a2 + S3 * (rr * drdn * drdni) +
               S4 * (dk * nni + ni[ik] * n[il]) + S5 * (n[ik] * ni[il]) - k.S1s * (dk * d3 * drdn * drdni) +
               k.S3s * (d3 * rr * drdn * drdni);
      // M21 + M31: with (phi - phi_i - psi_i . rv) jw
      T fr = d3 * (k.S2s * a2 + k.S1s * a1 + k.S1s * (rr * nni) + k.S4s * (ni[ik] * n[il]) + k.S5s * (ni[il] * n[ik]));
      if (il == ik) fr = fr + k.S4s * (d3 * nni);
      o.R[q] = fr;
      // M221 + M321: with phi_i jw
      T fp = d3 * (k.S1s * (-5.0 * rr * drdn * drdni) + k.S1s * (dr[ik] * (ni[il] * drdn - n[il] * drdni)) +
                   k.S2s * (dr[il] * (ni[ik] * drdn - n[ik] * drdni)));
      if (il == ik) fp = fp - k.S4s * (3.0 * d3 * drdn * drdni);
      o.PQ[q] = fp * jw;
      // M231 (psi_i . n), M331 (psi_i_j) and the -psi_i . rv part of M21 + M31
      const T fnn = il == ik ? -(k.S4s * (d2 * drdni)) : z;
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        const double djk = j == ik ? 1.0 : 0.0;
        T fj = d2 * (dr[j] * (k.S2s * a2 + k.S1s * a1 - k.S1s * (dr[il] * n[ik] * drdni)) -
                     ((S1o3 - k.S5s) * (ni[il] * dr[j]) + S1o3 * (ni[j] * dr[il])) * (n[ik] - ni[ik] * nni) +
                     k.S4s * (ni[ik] * dr[j] * (n[il] - ni[il] * nni)) - S1o3 * ((dk + ni[il] * ni[ik]) * n[j] * drdni) -
                     S1o3 * ((djk - ni[j] * ni[ik]) * n[il] * drdni));
        o.PQ[9 + 3 * q + j] = (fnn * n[j] + fj - fr * rv[j]) * jw;
      }
    }
}

// Scatter one HBIE singular pair (final m, l of this lane's outputs) into A, b.
// On a crack-like element face 2 takes -m and l at the next column.
template <typename T>
__device__ __forceinline__ void hsing_scatter(const DMesh& m, int dn, int e, int o, T v, double* Af, size_t lda, T bc[3]) {
  const int ck = m.rev[e] >> 1;
  if (o < 72) {
    const int kn = o / 9, il = (o % 9) / 3, ik = o % 3;
    const size_t row = dn_row(m, dn, il);
    for (int fc = 0; fc <= ck; ++fc, v = -v) {
      const int dof = m.edof[8 * e + kn] + (ik << ck) + fc;
      if (m.dct[dof] == 1) addA(Af, (size_t)dof * lda + row, v);
      else bc[il] = bc[il] - v * cval(m.dcv, dof, v);
    }
  } else {
    const int q = o - 72, kn = q / 9, il = (q % 9) / 3, ik = q % 3;
    const size_t row = dn_row(m, dn, il);
    for (int fc = 0; fc <= ck; ++fc) {
      const int dof = m.edof[8 * e + kn] + (ik << ck) + fc;
      if (m.dct[dof] == 0) addA(Af, (size_t)dof * lda + row, -v);
      else bc[il] = bc[il] + v * cval(m.dcv, dof, v);
    }
  }
}

// One warp per (dnode, frequency) walks the HBIE singular pairs of the node's
// collocation points (one per point: the element holding it). Phase 1: one
// lane per polar point forms ComboH; phase 2: lanes own the outputs
// o = lane + 32 j (m: o < 72, l: o >= 72) and the 36 pair sums P, Q.
template <class HS>
__global__ void __launch_bounds__(32) k_hsing(DMesh m, HS hs, int nf, double* A, size_t lda, size_t astride, double* b,
                                              size_t bstride) {
  typedef typename HS::T T;
  constexpr int NA = 5;  // 144 outputs over 32 lanes
  __shared__ ComboH<T> S[32];
  __shared__ T pq[36];
  __shared__ double ex[8 + 24 + 3 + 52];  // phi_i, psi_i, n_i, line integrals of the pair being flushed
  const int lane = threadIdx.x & 31;
  const long long gw = blockIdx.x;
  if (gw >= (long long)m.ndn * nf) return;
  const int dn = (int)(gw % m.ndn), f = (int)(gw / m.ndn);
  const HsCoef<T> k = hs.coef(f);
  const T z = VT<T>::zero();
  double* Af = A + astride * f;
  for (int cp = m.dn_cp[dn]; cp < m.dn_cp[dn + 1]; ++cp) {
    const int q0 = m.sing_start[cp], q1 = m.sing_start[cp + 1];
    if (q0 == q1) continue;
    const T beta = hbie_weighted(m.cp_kind[cp]) ? k.bm * m.cp_alpha[cp] : VT<T>::zero() + 1.0;
    const long long P0 = m.sing_pt[q0], Q = m.sing_pt[q1] - P0;
    int cur = -1;
    T acc[NA], as0 = z, as1 = z;
    for (int j = 0; j < NA; ++j) acc[j] = z;
    auto flush = [&](int qp) {
      // pair sums + edge line integrals (bem_staela3d.f90:5308-5345), then scale and scatter
      const double* D = m.sing_d + (size_t)qp * SING_D;
      const double* X = m.hsing_x + (size_t)qp * HSING_X;
      if (lane < 8) ex[lane] = D[5 + lane];
      for (int t = lane; t < 79; t += 32) ex[8 + t] = X[t];
      __syncwarp();
      const double* ni = ex + 8 + HX_N;
      const double* L = ex + 8 + HX_LLI - 0;
      const T S1o3 = k.S1s * (1.0 / 3.0);
      for (int s = lane; s < 36; s += 32) {
        T v = s == lane ? as0 : as1;
        if (s < 9) {
          const int il = s / 3, ik = s % 3;
          const double dk = il == ik ? 1.0 : 0.0;
          v = v + k.S4s * (dk * L[HX_M1 - HX_LLI]) + k.S1s * L[HX_M3 - HX_LLI + s] +
              k.S4s * (ni[ik] * L[HX_M4 - HX_LLI + il]) + k.S5s * (ni[il] * L[HX_M4 - HX_LLI + ik]);
        } else {
          const int qq = (s - 9) / 3, j = (s - 9) % 3, il = qq / 3, ik = qq % 3;
          const double dk = il == ik ? 1.0 : 0.0, djk = j == ik ? 1.0 : 0.0;
          v = v + k.S4s * (dk * L[HX_M2 - HX_LLI + j]) +
              S1o3 * (L[HX_M5 - HX_LLI + 9 * j + 3 * il + ik] + (dk + ni[il] * ni[ik]) * L[HX_M2 - HX_LLI + j] +
                      (djk - ni[j] * ni[ik]) * L[HX_M2 - HX_LLI + il]);
        }
        pq[s] = v;
      }
      __syncwarp();
      const int e = m.sing_e[qp];
      const bool rev = (m.rev[e] & 1) != 0;
      const T cs = k.cte_s * beta, cl = k.cte_d * beta;
      T bc[3] = {z, z, z};
      for (int j = 0; j < NA; ++j) {
        const int o = lane + 32 * j;
        if (o >= 144) break;
        T v = acc[j];
        if (o < 72) {
          const int kn = o / 9, qq = o % 9;
          const double* ps = ex + 8 + HX_PSI + 3 * kn;
          v = v + ex[kn] * pq[qq] + ps[0] * pq[9 + 3 * qq] + ps[1] * pq[10 + 3 * qq] + ps[2] * pq[11 + 3 * qq];
          v = v * cs;
        } else {
          const int kn = (o - 72) / 9, qq = (o - 72) % 9;
          v = v + ex[kn] * (k.T2s * L[qq]);  // L22
          v = v * cl;
          if (rev) v = -v;
        }
        hsing_scatter(m, dn, e, o, v, Af, lda, bc);
      }
      for (int il = 0; il < 3; ++il)
        for (int o = 16; o > 0; o >>= 1) bc[il] = bc[il] + shfl_x(bc[il], o);
      if (lane == 0) {
        double* bf = b + bstride * f;
        for (int il = 0; il < 3; ++il) addA(bf, dn_row(m, dn, il), bc[il]);
      }
      __syncwarp();
    };
    for (long long base = 0; base < Q; base += 32) {
      const long long c = base + lane;
      if (c < Q) {
        const int qp = find_le(m.sing_pt, q0, q1, P0 + c);
        double rv[3], n[3], w[8], wd[8];
        if (m.sing_geo) {
          const long long g = P0 + c, np = m.nsing_pts;
          const double* G = m.sing_geo;
          rv[0] = G[g]; rv[1] = G[np + g]; rv[2] = G[2 * np + g];
          n[0] = G[3 * np + g]; n[1] = G[4 * np + g]; n[2] = G[5 * np + g];
          for (int p = 0; p < 8; ++p) {
            w[p] = G[(6 + p) * np + g];
            wd[p] = G[(14 + p) * np + g];
          }
        } else {
          sing_point(m, qp, (int)(P0 + c - m.sing_pt[qp]), rv, n, w, wd);
        }
        double jw = 0.0;
        for (int p = 0; p < 8; ++p) {
          jw += w[p];
          S[lane].w[p] = w[p];
          S[lane].wd[p] = wd[p];
        }
        const double* ni = m.hsing_x + (size_t)qp * HSING_X + HX_N;
        const double nv[3] = {ni[0], ni[1], ni[2]};
        hsing_point(hs, f, k, rv, n, nv, jw, S[lane]);
        S[lane].pair = qp;
      }
      __syncwarp();
      const int nt = (int)min((long long)32, Q - base);
      for (int t = 0; t < nt; ++t) {
        const int qp = S[t].pair;
        if (qp != cur) {
          if (cur >= 0) flush(cur);
          cur = qp;
          for (int j = 0; j < NA; ++j) acc[j] = z;
          as0 = as1 = z;
        }
#pragma unroll
        for (int j = 0; j < NA; ++j) {
          const int o = lane + 32 * j;
          if (o < 144) {
            if (o < 72) {
              const int kn = o / 9, qq = o % 9;
              acc[j] = acc[j] + S[t].A[qq] * S[t].w[kn] + S[t].R[qq] * S[t].wd[kn];
            } else {
              const int kn = (o - 72) / 9, qq = (o - 72) % 9;
              acc[j] = acc[j] + S[t].D[qq] * S[t].w[kn] + S[t].C[qq] * S[t].wd[kn];
            }
          }
        }
        as0 = as0 + S[t].PQ[lane];
        if (lane < 4) as1 = as1 + S[t].PQ[32 + lane];
      }
      __syncwarp();
    }
    if (cur >= 0) flush(cur);
  }
}

// Free terms of the HBIE view's points (build_lse_mechanics_bem_staela.f90:
// 181-211,459-489, build_lse_mechanics_bem_harela.f90:316-360,629-681): -1/2
// phi(xi_i) on l (taken as g: weight 1 for HBIE alone, beta for Burton &
// Miller) and, for Burton & Miller, the SBIE's 1/2 phi(xi_i) on h. A point of
// a crack-like boundary (cp_kind 4, dual BEM) carries both equations of its
// node: the SBIE (rows one below the HBIE's) takes 1/2 phi(xi_i) on both
// faces' u, the HBIE -1/2 phi(xi_i) on face 1's t and +1/2 phi(xi_i) on face
// 2's t (staela.f90:195-204). One thread per (dnode, frequency).
template <typename T>
__global__ void k_hfree(DMesh m, const HarParH* ph, int nf, double* A, size_t lda, size_t astride, double* b,
                        size_t bstride) {
  const long long id = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (id >= (long long)m.ndn * nf) return;
  const int dn = (int)(id % m.ndn), f = (int)(id / m.ndn);
  if (m.dn_cp[dn] == m.dn_cp[dn + 1]) return;
  double* Af = A + astride * f;
  double* bf = b + bstride * f;
  const T z = VT<T>::zero();
  T bc[3] = {z, z, z}, bs[3] = {z, z, z};
  bool crack = false;
  for (int cp = m.dn_cp[dn]; cp < m.dn_cp[dn + 1]; ++cp) {
    const int e = m.cp_elem[cp];
    if (m.cp_kind[cp] == 4) {
      crack = true;
      double phi[8];
      phi_q8<double>(m.cp_xi[2 * cp], m.cp_xi[2 * cp + 1], phi);
      for (int kn = 0; kn < 8; ++kn)
        for (int il = 0; il < 3; ++il) {
          const size_t row = dn_row(m, dn, il);
          for (int fc = 0; fc < 2; ++fc) {
            const int dof = m.edof[8 * e + kn] + 2 * il + fc;
            const T v = z + 0.5 * phi[kn];
            if (m.dct[dof] == 1) addA(Af, (size_t)dof * lda + row - 1, v);
            else bs[il] = bs[il] - v * cval(m.dcv, dof, z);
            const T g = z + (fc ? 0.5 : -0.5) * phi[kn];
            if (m.dct[dof] == 0) addA(Af, (size_t)dof * lda + row, -g);
            else bc[il] = bc[il] + g * cval(m.dcv, dof, z);
          }
        }
      continue;
    }
    // Burton & Miller: the SBIE's 1/2 phi(xi_i) on h here too ('dual_bm_same';
    // 'dual_bm_mixed' has it at its own SBIE point in the SBIE view)
    const bool bm = m.cp_kind[cp] == 3;
    T beta = z + 1.0;
    if (hbie_weighted(m.cp_kind[cp])) {
      if constexpr (std::is_same<T, cd>::value) beta = ph[f].ic2 * m.cp_alpha[cp];
      else beta = z + m.cp_alpha[cp];
    }
    double phi[8];
    phi_q8<double>(m.cp_xi[2 * cp], m.cp_xi[2 * cp + 1], phi);
    for (int kn = 0; kn < 8; ++kn)
      for (int il = 0; il < 3; ++il) {
        const size_t row = dn_row(m, dn, il);
        const int dof = m.edof[8 * e + kn] + il;
        if (bm) {
          const T v = z + 0.5 * phi[kn];
          if (m.dct[dof] == 1) addA(Af, (size_t)dof * lda + row, v);
          else bc[il] = bc[il] - v * cval(m.dcv, dof, z);
        }
        const T g = beta * (-0.5 * phi[kn]);
        if (m.dct[dof] == 0) addA(Af, (size_t)dof * lda + row, -g);
        else bc[il] = bc[il] + g * cval(m.dcv, dof, z);
      }
  }
  for (int il = 0; il < 3; ++il) {
    addA(bf, dn_row(m, dn, il), bc[il]);
    if (crack) addA(bf, dn_row(m, dn, il) - 1, bs[il]);
  }
}

}  // namespace mfb
