// Per-frequency assembly kernels. One warp owns one DOF-order node ("dnode",
// the 3 rows of its equations) for one frequency, walks the node's collocation
// points and their pair lists in element order, and adds the integrated
// (kn, il, ik) blocks into A and b with the scatter of
// assemble_bem_{staela,harela}_equation (ordinary BE boundary,
// src/assemble_bem_staela_equation.f90:69-98). Rows are owned by exactly one
// warp, so no atomics are used and the summation order is fixed.
//
// Each kernel runs in two phases per batch of 32 quadrature points:
//   phase 1: one lane per point evaluates geometry and the fundamental
//            solutions (fu, ft) and stores them with phi*J*w in shared memory;
//   phase 2: all lanes walk the 32 points in order; lane l owns the outputs
//            o = l, l+32, ... (o = hg*72 + kn*9 + il*3 + ik) of the current
//            pair and accumulates fs[o] * phiJw[kn]; a pair change flushes.
#pragma once
#include "bem_common.h"
#include "dev_complex.cuh"
#include "dev_point.cuh"
#include "mfbem_dev.h"
#include "dev_df64.cuh"

namespace mfb {

template <typename T> struct VT;
template <> struct VT<double> {
  __device__ static double zero() { return 0.0; }
};
template <> struct VT<cd> {
  __device__ static cd zero() { return mk(0.0, 0.0); }
};
__device__ __forceinline__ double shfl_x(double v, int o) { return __shfl_xor_sync(0xffffffffu, v, o); }
__device__ __forceinline__ cd shfl_x(cd v, int o) { return mk(shfl_x(v.re, o), shfl_x(v.im, o)); }
__device__ __forceinline__ double cval(const double* dcv, int dof, double) { return dcv[2 * (size_t)dof]; }
__device__ __forceinline__ cd cval(const double* dcv, int dof, cd) { return mk(dcv[2 * (size_t)dof], dcv[2 * (size_t)dof + 1]); }
__device__ __forceinline__ void addA(double* A, size_t idx, double v) { A[idx] += v; }
__device__ __forceinline__ void addA(double* A, size_t idx, cd v) {
  double2* p = reinterpret_cast<double2*>(A) + idx;
  double2 a = *p;
  a.x += v.re;
  a.y += v.im;
  *p = a;
}

// Kernel family policies -----------------------------------------------------
struct PolStatic {
  typedef double T;
  static constexpr int NG = 6;  // independent components of g per node (u* symmetric)
  StaelaP k;
  double nu = 0.0, mu = 0.0;
  __device__ T cte_t(int) const { return k.ctet1; }
  __device__ T cte_u(int) const { return k.cteu1; }
  __device__ T cpv(int) const { return k.ctet2; }  // coefficient of the CPV/line-integral part
  __device__ void point(int, int, const double rv[3], const double n[3], T fu[9], T ft[9]) const {
    staela_point(k, rv, n, fu, ft);
  }
  // singular (interior) integration: regular parts and the CPV integrand
  __device__ void point_sing(int, int, const double rv[3], const double n[3], T fu[9], T ft[9], T fc[9]) const {
    double r = sqrt(rv[0] * rv[0] + rv[1] * rv[1] + rv[2] * rv[2]);
    double d1r = 1.0 / r, d1r2 = d1r * d1r;
    double dr[3] = {rv[0] * d1r, rv[1] * d1r, rv[2] * d1r};
    double drdn = dr[0] * n[0] + dr[1] * n[1] + dr[2] * n[2];
    for (int il = 0; il < 3; ++il)
      for (int ik = 0; ik < 3; ++ik) {
        double dk = (il == ik) ? 1.0 : 0.0;
        fu[3 * il + ik] = d1r * (k.cteu2 * dk + dr[il] * dr[ik]);
        ft[3 * il + ik] = d1r2 * drdn * (k.ctet2 * dk + 3.0 * dr[il] * dr[ik]);
        fc[3 * il + ik] = d1r2 * k.ctet2 * (n[il] * dr[ik] - n[ik] * dr[il]);
      }
  }
};
struct HarParH;
struct PolHarmonic {
  typedef cd T;
  static constexpr int NG = 6;
  const HarParD* p;  // one parameter block per frequency
  const HarParH* ph = nullptr;  // d* / s* parameters per frequency (HBIE points only)
  __device__ T cte_t(int f) const { return p[f].cte_t; }
  __device__ T cte_u(int f) const { return p[f].cte_u; }
  __device__ T cpv(int f) const { return p[f].T2[0]; }
  __device__ void point(int f, int, const double rv[3], const double n[3], T fu[9], T ft[9]) const {
    harela_point(p[f], rv, n, fu, ft);
  }
  __device__ void point_sing(int f, int, const double rv[3], const double n[3], T fu[9], T ft[9], T fc[9]) const {
    const HarParD& q = p[f];
    double r = sqrt(rv[0] * rv[0] + rv[1] * rv[1] + rv[2] * rv[2]);
    cd psi, chi, TT1, TT2, TT3;
    double d1r1, d1r2;
    harela_coeffs(q, r, psi, chi, TT1, TT2, TT3, d1r1, d1r2, false);
    double dr[3] = {rv[0] * d1r1, rv[1] * d1r1, rv[2] * d1r1};
    double drdn = dr[0] * n[0] + dr[1] * n[1] + dr[2] * n[2];
    cd A1 = TT1 + q.T1[0] * d1r2, A2 = TT2 + q.T2[0] * d1r2;
    cd c2 = q.T2[0] * d1r2;
    for (int il = 0; il < 3; ++il)
      for (int ik = 0; ik < 3; ++ik) {
        double rr = dr[il] * dr[ik];
        cd u = -(chi * rr);
        cd t = A1 * (rr * drdn) + TT2 * (dr[ik] * n[il]) + TT3 * (dr[il] * n[ik]);
        if (il == ik) {
          u = u + psi;
          t = t + A2 * drdn;
        }
        fu[3 * il + ik] = u;
        ft[3 * il + ik] = t;
        fc[3 * il + ik] = c2 * (n[il] * dr[ik] - n[ik] * dr[il]);
      }
  }
};

// Half-space complementary kernel (static, traction-free surface x3 = xp):
// the pair lists of these policies are classified on the images of the
// collocation points, so rv = x - image; c[cp] = x_i3 - xp of the original
// point. u* of this kernel is not symmetric: all nine g components are kept.
struct PolHsc {
  typedef double T;
  static constexpr int NG = 9;
  StaelaP k;
  const double* c;  // [ncp]
  double xp, nu;
  __device__ T cte_t(int) const { return -k.ctet1; }  // 1 / (8 pi (1 - nu))
  __device__ T cte_u(int) const { return k.cteu1; }   // 1 / (16 pi mu (1 - nu))
  __device__ T cpv(int) const { return 0.0; }
  __device__ void point(int, int cp, const double rv[3], const double n[3], T fu[9], T ft[9]) const {
    const double ci = c[cp];
    // z = x3 - xp; the image's vertical offset as x3 + x_i3 (reflection in x3 = 0)
    hsc_point(nu, rv[0], rv[1], ci, rv[2] - ci, rv[2] + 2.0 * xp, n, fu, ft);
  }
};
// Singular pairs of the complementary kernel (collocation point and element on
// the free surface): h is minus the full-space singular h (CPV and line
// integrals included), g the surface restriction of the complementary
// displacement kernel on the same polar rule. rv = x - x_i here.
struct PolHscSing {
  typedef double T;
  static constexpr int NG = 9;
  StaelaP k;
  const double* c;
  double nu;
  __device__ T cte_t(int) const { return k.ctet1; }
  __device__ T cte_u(int) const { return k.cteu1; }
  __device__ T cpv(int) const { return -k.ctet2; }
  __device__ void point_sing(int, int cp, const double rv[3], const double n[3], T fu[9], T ft[9], T fc[9]) const {
    double r = sqrt(rv[0] * rv[0] + rv[1] * rv[1] + rv[2] * rv[2]);
    double d1r = 1.0 / r, d1r2 = d1r * d1r;
    double dr[3] = {rv[0] * d1r, rv[1] * d1r, rv[2] * d1r};
    double drdn = dr[0] * n[0] + dr[1] * n[1] + dr[2] * n[2];
    for (int il = 0; il < 3; ++il)
      for (int ik = 0; ik < 3; ++ik) {
        double dk = (il == ik) ? 1.0 : 0.0;
        ft[3 * il + ik] = -(d1r2 * drdn * (k.ctet2 * dk + 3.0 * dr[il] * dr[ik]));
        fc[3 * il + ik] = -(d1r2 * k.ctet2 * (n[il] * dr[ik] - n[ik] * dr[il]));
      }
    hsc_surface_g(nu, r, dr, rv[2] + c[cp], fu);
  }
};

// Outputs of one pair handled by the lanes of a warp: o = lane + 32 j, j < 4.
// o < 72: h(kn, il, ik), kn = o / 9; o >= 72: g(kn, s) with s one of the six
// (il <= ik) components (u* is symmetric, so g(kn, il, ik) = g(kn, ik, il)).
constexpr int kOut = 120;
constexpr int kAcc = 4;
// outputs and accumulators per lane for NG g components per node
template <int NG> struct GOut {
  static constexpr int out = 72 + 8 * NG;
  static constexpr int acc = (out + 31) / 32;
};
__device__ __forceinline__ int sym_il(int s) { return s < 3 ? 0 : (s < 5 ? 1 : 2); }
__device__ __forceinline__ int sym_ik(int s) { return s < 3 ? s : (s < 5 ? s - 2 : 2); }

// Shared flush: scale, reverse, scatter one pair's outputs of this lane set.
template <class POL>
__device__ __forceinline__ void flush_pair(const DMesh& m, const POL& pol, int f, int dn, int e,
                                           typename POL::T* acc, double* A, size_t lda, size_t astride,
                                           double* b, size_t bstride, const double* hli_phi /* or null */) {
  typedef typename POL::T T;
  constexpr int NG = POL::NG;
  const int lane = threadIdx.x & 31;
  T bc[3] = {VT<T>::zero(), VT<T>::zero(), VT<T>::zero()};
  const int rv = m.rev[e];
  const bool rev = (rv & 1) != 0;
  // crack-like element: face 2 (reversed normal) takes -h and g at the next
  // column (build_lse_mechanics_bem_staela.f90:883-887)
  const int ck = rv >> 1;
  double* Af = A + astride * f;
  for (int j = 0; j < GOut<NG>::acc; ++j) {
    int o = lane + 32 * j;
    if (o >= GOut<NG>::out) break;
    T v = acc[j];
    if (o < 72) {
      int kn = o / 9, il = (o % 9) / 3, ik = o % 3;
      if (hli_phi) v = v + hli_phi[9 + kn] * pol.cpv(f) * hli_phi[3 * il + ik];
      v = v * pol.cte_t(f);
      if (rev) v = -v;
      const size_t row = dn_row(m, dn, il);
      for (int fc = 0; fc <= ck; ++fc, v = -v) {
        const int dof = m.edof[8 * e + kn] + (ik << ck) + fc;
        if (m.dct[dof] == 1) addA(Af, (size_t)dof * lda + row, v);
        else bc[il] = bc[il] - v * cval(m.dcv, dof, v);
      }
    } else {
      int q = o - 72, kn = q / NG, sidx = q % NG;
      int il = NG == 6 ? sym_il(sidx) : sidx / 3, ik = NG == 6 ? sym_ik(sidx) : sidx % 3;
      v = v * pol.cte_u(f);
      for (int t = 0; t < (il == ik || NG == 9 ? 1 : 2); ++t) {
        int r_ = t ? ik : il, c_ = t ? il : ik;
        const size_t row = dn_row(m, dn, r_);
        for (int fc = 0; fc <= ck; ++fc) {
          const int dof = m.edof[8 * e + kn] + (c_ << ck) + fc;
          if (m.dct[dof] == 0) addA(Af, (size_t)dof * lda + row, -v);
          else bc[r_] = bc[r_] + v * cval(m.dcv, dof, v);
        }
      }
    }
  }
  for (int il = 0; il < 3; ++il)
    for (int o = 16; o > 0; o >>= 1) bc[il] = bc[il] + shfl_x(bc[il], o);
  if (lane == 0) {
    double* bf = b + bstride * f;
    for (int il = 0; il < 3; ++il) addA(bf, dn_row(m, dn, il), bc[il]);
  }
  __syncwarp();
}

template <typename T, int NG = 6>
struct alignas(16) Combo {
  T fu[NG], ft[9];
  double w[8];
  int pair;
};
template <typename T, int NG = 6>
struct alignas(16) ComboS {
  T fu[NG], ft[9], fc[9];
  double w[8], wd[8];
  int pair;
};
// keep the NG independent components of u* (six of a symmetric one)
template <int NG, typename T>
__device__ __forceinline__ void store_u(T* dst, const T fu[9]) {
  if (NG == 6) {
    dst[0] = fu[0]; dst[1] = fu[1]; dst[2] = fu[2]; dst[3] = fu[4]; dst[4] = fu[5]; dst[5] = fu[8];
  } else {
    for (int q = 0; q < 9; ++q) dst[q] = fu[q];
  }
}

__device__ __forceinline__ int find_le(const long long* a, int lo, int hi, long long v) {
  // largest j in [lo, hi) with a[j] <= v
  while (hi - lo > 1) {
    int mid = (lo + hi) >> 1;
    if (a[mid] <= v) lo = mid;
    else hi = mid;
  }
  return lo;
}

template <int NG, typename T>
__device__ __forceinline__ void accumulate(T* acc, const T* fug, const T* ft, const double* w) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int j = 0; j < GOut<NG>::acc; ++j) {
    int o = lane + 32 * j;
    if (o < GOut<NG>::out) {
      T v;
      int kn;
      if (o < 72) {
        kn = o / 9;
        v = ft[o % 9];
      } else {
        kn = (o - 72) / NG;
        v = fug[(o - 72) % NG];
      }
      acc[j] = acc[j] + v * w[kn];
    }
  }
}

// ---------------------------------------------------------------- regular pairs
template <class POL, int WPB>
__global__ void __launch_bounds__(WPB * 32) k_reg(DMesh m, POL pol, int nf, double* A, size_t lda, size_t astride,
                                                  double* b, size_t bstride) {
  typedef typename POL::T T;
  constexpr int NG = POL::NG, NA = GOut<NG>::acc;
  __shared__ Combo<T, NG> sm[WPB][32];
  const int lane = threadIdx.x & 31, w = threadIdx.x / 32;
  const long long gw = blockIdx.x * (long long)WPB + w;
  if (gw >= (long long)m.ndn * nf) return;
  const int dn = (int)(gw % m.ndn), f = (int)(gw / m.ndn);
  Combo<T, NG>* S = sm[w];
  for (int cp = m.dn_cp[dn]; cp < m.dn_cp[dn + 1]; ++cp) {
    const int s0 = m.reg_start[cp], s1 = m.reg_start[cp + 1];
    if (s0 == s1) continue;
    const double* xi = m.cpx + 3 * (size_t)cp;
    const long long P0 = m.reg_pt[s0], Q = m.reg_pt[s1] - P0;
    int cur = -1;
    T acc[NA];
    for (int j = 0; j < NA; ++j) acc[j] = VT<T>::zero();
    for (long long base = 0; base < Q; base += 32) {
      long long c = base + lane;
      if (c < Q) {
        int jp = find_le(m.reg_pt, s0, s1, P0 + c);
        int pr = m.reg_pair[jp];
        int e = pr & 0xFFFFFF, ps = pr >> 24;
        size_t pt = (size_t)e * m.ptot + m.ps_off[ps] + (size_t)(P0 + c - m.reg_pt[jp]);
        double rv[3] = {m.px[3 * pt] - xi[0], m.px[3 * pt + 1] - xi[1], m.px[3 * pt + 2] - xi[2]};
        double n[3] = {m.pn[3 * pt], m.pn[3 * pt + 1], m.pn[3 * pt + 2]};
        T fu9[9];
        pol.point(f, cp, rv, n, fu9, S[lane].ft);
        store_u<NG>(S[lane].fu, fu9);
        for (int k = 0; k < 8; ++k) S[lane].w[k] = m.pphi[8 * pt + k];
        S[lane].pair = jp;
      }
      __syncwarp();
      int nt = (int)min((long long)32, Q - base);
      for (int t = 0; t < nt; ++t) {
        int jp = S[t].pair;
        if (jp != cur) {
          if (cur >= 0) flush_pair(m, pol, f, dn, m.reg_pair[cur] & 0xFFFFFF, acc, A, lda, astride, b, bstride, nullptr);
          cur = jp;
          for (int j = 0; j < NA; ++j) acc[j] = VT<T>::zero();
        }
        accumulate<NG>(acc, S[t].fu, S[t].ft, S[t].w);
      }
      __syncwarp();
    }
    if (cur >= 0) flush_pair(m, pol, f, dn, m.reg_pair[cur] & 0xFFFFFF, acc, A, lda, astride, b, bstride, nullptr);
  }
}

// ---------------------------------------------------------------- adaptive pairs
// Geometry of point k of leaf l (adaptive pair a): Telles maps, sub-square to
// element coordinates, element geometry (sbie_ext_st, bem_staela3d.f90:654-969).
__device__ __forceinline__ void leaf_point(const DMesh& m, int l, int a, int k, const double* xi, double rv[3],
                                           double n[3], double w[8]) {
  int e = m.adp_e[a];
  int g = m.leaf_gln[l];
  int k1 = k / g + 1, k2 = k % g + 1;
  const double* L = m.leaf + (size_t)l * LEAF_D;
  Telles t1{L[8], L[9], L[10], L[11]}, t2{L[12], L[13], L[14], L[15]};
  double xp1, jt1, xp2, jt2;
  telles_map(t1, gl11x(k1, g), xp1, jt1);
  telles_map(t2, gl11x(k2, g), xp2, jt2);
  double sp[4], sd1[4], sd2[4];
  phi_q4(xp1, xp2, sp);
  dphi_q4(xp1, xp2, sd1, sd2);
  double xa = 0, xb = 0, a11 = 0, a12 = 0, a21 = 0, a22 = 0;
  for (int q = 0; q < 4; ++q) {
    xa = xa + sp[q] * L[2 * q];
    xb = xb + sp[q] * L[2 * q + 1];
    a11 = a11 + sd1[q] * L[2 * q];
    a12 = a12 + sd1[q] * L[2 * q + 1];
    a21 = a21 + sd2[q] * L[2 * q];
    a22 = a22 + sd2[q] * L[2 * q + 1];
  }
  double js = a11 * a22 - a12 * a21;
  double xq[3], T1[3], T2[3], phi[8], N[3];
  geom_q8(m.ex + 24 * (size_t)e, xa, xb, xq, T1, T2, phi);
  cross3(T1, T2, N);
  double jg = norm3(N);
  n[0] = N[0] / jg;
  n[1] = N[1] / jg;
  n[2] = N[2] / jg;
  rv[0] = xq[0] - xi[0];
  rv[1] = xq[1] - xi[1];
  rv[2] = xq[2] - xi[2];
  double jw = jg * js * jt1 * jt2 * gl11w(k1, g) * gl11w(k2, g);
  for (int q = 0; q < 8; ++q) w[q] = phi[q] * jw;
}

template <class POL, int WPB>
__global__ void __launch_bounds__(WPB * 32) k_adp(DMesh m, POL pol, int nf, double* A, size_t lda, size_t astride,
                                                  double* b, size_t bstride) {
  typedef typename POL::T T;
  constexpr int NG = POL::NG, NA = GOut<NG>::acc;
  __shared__ Combo<T, NG> sm[WPB][32];
  const int lane = threadIdx.x & 31, w = threadIdx.x / 32;
  const long long gw = blockIdx.x * (long long)WPB + w;
  if (gw >= (long long)m.ndn * nf) return;
  const int dn = (int)(gw % m.ndn), f = (int)(gw / m.ndn);
  Combo<T, NG>* S = sm[w];
  for (int cp = m.dn_cp[dn]; cp < m.dn_cp[dn + 1]; ++cp) {
    const int a0 = m.adp_start[cp], a1 = m.adp_start[cp + 1];
    if (a0 == a1) continue;
    const int l0 = m.adp_leaf[a0], l1 = m.adp_leaf[a1];
    const double* xi = m.cpx + 3 * (size_t)cp;
    const long long P0 = m.leaf_pt[l0], Q = m.leaf_pt[l1] - P0;
    int cur = -1;
    T acc[NA];
    for (int j = 0; j < NA; ++j) acc[j] = VT<T>::zero();
    for (long long base = 0; base < Q; base += 32) {
      long long c = base + lane;
      if (c < Q) {
        int l = find_le(m.leaf_pt, l0, l1, P0 + c);
        int a = m.leaf_pair[l];
        if (m.leaf_geo) {
          const long long g = P0 + c, np = m.nleaf_pts;
          const double* G = m.leaf_geo;
          double rv[3] = {G[g], G[np + g], G[2 * np + g]};
          double n[3] = {G[3 * np + g], G[4 * np + g], G[5 * np + g]};
          T fu9[9];
          pol.point(f, cp, rv, n, fu9, S[lane].ft);
          store_u<NG>(S[lane].fu, fu9);
          for (int q = 0; q < 8; ++q) S[lane].w[q] = G[(6 + q) * np + g];
        } else {
          double rv[3], n[3], w[8];
          leaf_point(m, l, a, (int)(P0 + c - m.leaf_pt[l]), xi, rv, n, w);
          T fu9[9];
          pol.point(f, cp, rv, n, fu9, S[lane].ft);
          store_u<NG>(S[lane].fu, fu9);
          for (int q = 0; q < 8; ++q) S[lane].w[q] = w[q];
        }
        S[lane].pair = a;
      }
      __syncwarp();
      int nt = (int)min((long long)32, Q - base);
      for (int t = 0; t < nt; ++t) {
        int a = S[t].pair;
        if (a != cur) {
          if (cur >= 0) flush_pair(m, pol, f, dn, m.adp_e[cur], acc, A, lda, astride, b, bstride, nullptr);
          cur = a;
          for (int j = 0; j < NA; ++j) acc[j] = VT<T>::zero();
        }
        accumulate<NG>(acc, S[t].fu, S[t].ft, S[t].w);
      }
      __syncwarp();
    }
    if (cur >= 0) flush_pair(m, pol, f, dn, m.adp_e[cur], acc, A, lda, astride, b, bstride, nullptr);
  }
}

// ---------------------------------------------------------------- singular pairs
// Geometry of polar point k of singular pair q (sbie_int, bem_staela3d.f90:1100-1381).
__device__ __forceinline__ void sing_point(const DMesh& m, int q, int k, double rv[3], double n[3], double w[8],
                                           double wd[8]) {
  const double* D = m.sing_d + (size_t)q * SING_D;
  const int* I = m.sing_i + (size_t)q * SING_I;
  int s = 0;
  while (s + 1 < I[0] && I[17 + s + 1] <= k) ++s;
  int kk = k - I[17 + s];
  int ngt = I[9 + s];
  int kt = kk / 15 + 1, kr = kk % 15 + 1;
  double xi_i[2] = {D[0], D[1]};
  double tpi = D[38 + 2 * s], tpf = D[39 + 2 * s];
  double tpp = gl01x(kt, ngt), wa = gl01w(kt, ngt);
  double jtp = tpf - tpi;
  double tp = jtp * tpp + tpi;
  double theta, rhoij;
  polar_angular(xi_i, I[1 + s], tp, &theta, &rhoij);
  double sn, cs;
  sincos(theta, &sn, &cs);
  double rho = rhoij * gl01x(kr, 15);
  double xq[3], T1[3], T2[3], phi[8], N[3];
  int e = m.sing_e[q];
  geom_q8(m.ex + 24 * (size_t)e, xi_i[0] + rho * cs, xi_i[1] + rho * sn, xq, T1, T2, phi);
  cross3(T1, T2, N);
  double jg = norm3(N);
  n[0] = N[0] / jg;
  n[1] = N[1] / jg;
  n[2] = N[2] / jg;
  rv[0] = xq[0] - D[2];
  rv[1] = xq[1] - D[3];
  rv[2] = xq[2] - D[4];
  double jw = jg * rho * jtp * wa * gl01w(kr, 15);
  for (int p = 0; p < 8; ++p) {
    w[p] = phi[p] * jw;
    wd[p] = (phi[p] - D[5 + p]) * jw;
  }
}

// once per mesh: the singular and adaptive-leaf point geometry for all frequencies
__global__ void k_sing_geo(DMesh m) {
  long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (g >= m.nsing_pts) return;
  int q = find_le(m.sing_pt, 0, (int)m.nsing, g);
  double rv[3], n[3], w[8], wd[8];
  sing_point(m, q, (int)(g - m.sing_pt[q]), rv, n, w, wd);
  const long long np = m.nsing_pts;
  for (int c = 0; c < 3; ++c) {
    m.sing_geo[c * np + g] = rv[c];
    m.sing_geo[(3 + c) * np + g] = n[c];
  }
  for (int p = 0; p < 8; ++p) {
    m.sing_geo[(6 + p) * np + g] = w[p];
    m.sing_geo[(14 + p) * np + g] = wd[p];
  }
}
__global__ void k_leaf_geo(DMesh m) {
  long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (g >= m.nleaf_pts) return;
  int l = find_le(m.leaf_pt, 0, (int)m.nleaf, g);
  int a = m.leaf_pair[l];
  double rv[3], n[3], w[8];
  leaf_point(m, l, a, (int)(g - m.leaf_pt[l]), m.cpx + 3 * (size_t)m.adp_cp[a], rv, n, w);
  const long long np = m.nleaf_pts;
  for (int c = 0; c < 3; ++c) {
    m.leaf_geo[c * np + g] = rv[c];
    m.leaf_geo[(3 + c) * np + g] = n[c];
  }
  for (int p = 0; p < 8; ++p) m.leaf_geo[(6 + p) * np + g] = w[p];
}

template <class POL, int WPB>
__global__ void __launch_bounds__(WPB * 32) k_sing(DMesh m, POL pol, int nf, double* A, size_t lda, size_t astride,
                                                   double* b, size_t bstride) {
  typedef typename POL::T T;
  constexpr int NG = POL::NG, NA = GOut<NG>::acc;
  __shared__ ComboS<T, NG> sm[WPB][32];
  __shared__ double hp[WPB][17];  // hli[9], phi_i[8] of the pair being flushed
  const int lane = threadIdx.x & 31, w = threadIdx.x / 32;
  const long long gw = blockIdx.x * (long long)WPB + w;
  if (gw >= (long long)m.ndn * nf) return;
  const int dn = (int)(gw % m.ndn), f = (int)(gw / m.ndn);
  ComboS<T, NG>* S = sm[w];
  for (int cp = m.dn_cp[dn]; cp < m.dn_cp[dn + 1]; ++cp) {
    const int q0 = m.sing_start[cp], q1 = m.sing_start[cp + 1];
    if (q0 == q1) continue;
    const long long P0 = m.sing_pt[q0], Q = m.sing_pt[q1] - P0;
    int cur = -1;
    T acc[NA], acd[NA];
    for (int j = 0; j < NA; ++j) acc[j] = acd[j] = VT<T>::zero();
    for (long long base = 0; base < Q; base += 32) {
      long long c = base + lane;
      if (c < Q) {
        int q = find_le(m.sing_pt, q0, q1, P0 + c);
        double rv[3], n[3];
        if (m.sing_geo) {
          const long long g = P0 + c, np = m.nsing_pts;
          const double* G = m.sing_geo;
          rv[0] = G[g]; rv[1] = G[np + g]; rv[2] = G[2 * np + g];
          n[0] = G[3 * np + g]; n[1] = G[4 * np + g]; n[2] = G[5 * np + g];
          for (int p = 0; p < 8; ++p) {
            S[lane].w[p] = G[(6 + p) * np + g];
            S[lane].wd[p] = G[(14 + p) * np + g];
          }
        } else {
          sing_point(m, q, (int)(P0 + c - m.sing_pt[q]), rv, n, S[lane].w, S[lane].wd);
        }
        T fu9[9];
        pol.point_sing(f, cp, rv, n, fu9, S[lane].ft, S[lane].fc);
        store_u<NG>(S[lane].fu, fu9);
        S[lane].pair = q;
      }
      __syncwarp();
      int nt = (int)min((long long)32, Q - base);
      for (int t = 0; t < nt; ++t) {
        int q = S[t].pair;
        if (q != cur) {
          if (cur >= 0) {
            for (int j = 0; j < NA; ++j) acc[j] = acc[j] + acd[j];
            flush_pair(m, pol, f, dn, m.sing_e[cur], acc, A, lda, astride, b, bstride, hp[w]);
          }
          cur = q;
          for (int j = 0; j < NA; ++j) acc[j] = acd[j] = VT<T>::zero();
          if (lane < 17) {
            const double* D = m.sing_d + (size_t)q * SING_D;
            hp[w][lane] = lane < 9 ? D[13 + lane] : D[5 + lane - 9];
          }
          __syncwarp();
        }
        accumulate<NG>(acc, S[t].fu, S[t].ft, S[t].w);
        // CPV integrand with (phi - phi_i): h outputs only
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          int o = lane + 32 * j;
          if (o < 72) {
            int kn = o / 9, qq = o % 9;
            acd[j] = acd[j] + S[t].fc[qq] * S[t].wd[kn];
          }
        }
      }
      __syncwarp();
    }
    if (cur >= 0) {
      for (int j = 0; j < NA; ++j) acc[j] = acc[j] + acd[j];
      flush_pair(m, pol, f, dn, m.sing_e[cur], acc, A, lda, astride, b, bstride, hp[w]);
    }
  }
}

// ---------------------------------------------------------------- free terms
__device__ __forceinline__ double one_minus(const double* nu, double) { return 1.0 - nu[0]; }
__device__ __forceinline__ cd one_minus(const double* nu, cd) { return mk(1.0 - nu[0], -nu[1]); }
__device__ __forceinline__ double fr(double x, double) { return x; }
__device__ __forceinline__ cd fr(double x, cd) { return mk(x, 0.0); }

// Free terms of build_lse_mechanics_bem_{staela,harela} (staela.f90:152-549):
// nodal SBIE points get Mantic's C (cp I - sum_b / (8 pi (1-nu))) on their own
// columns; SBIE-MCA points get 1/2 phi(xi_i) on the diagonal blocks of their
// element's nodes. One thread per (dnode, frequency).
template <class POL>
__global__ void k_free(DMesh m, POL pol, const double* nu /* complex, per frequency */, int nf, double* A, size_t lda,
                       size_t astride, double* b, size_t bstride, int* err) {
  typedef typename POL::T T;
  long long id = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (id >= (long long)m.ndn * nf) return;
  int dn = (int)(id % m.ndn), f = (int)(id / m.ndn);
  if (m.dn_cp[dn] == m.dn_cp[dn + 1]) return;
  double* Af = A + astride * f;
  double* bf = b + bstride * f;
  const T z = VT<T>::zero();
  T bc[3] = {z, z, z};
  for (int cp = m.dn_cp[dn]; cp < m.dn_cp[dn + 1]; ++cp) {
    int e = m.cp_elem[cp], kn0 = m.cp_kn[cp];
    // half-space: a collocation point on the traction-free surface takes twice
    // its free term (build_lse_mechanics_bem_staela.f90:502-513,
    // build_lse_mechanics_bem_harela.f90:688-697)
    const double two =
        (m.hs_ax >= 0 && m.cpx[3 * (size_t)cp + m.hs_ax] - m.hs_x <= 1e-12 / m.cl[e]) ? 2.0 : 1.0;
    if (m.cp_kind[cp] == 0) {
      if (!m.ft_ok[cp]) { atomicExch(err, 1); continue; }
      const double* F = m.ft + (size_t)cp * FT_D;
      T onemnu = one_minus(nu + 2 * f, z);
      T q = -1.0 / ((8.0 * kPi) * onemnu);
      for (int il = 0; il < 3; ++il) {
        const size_t row = dn_row(m, dn, il);
        for (int ik = 0; ik < 3; ++ik) {
          T C = q * F[1 + 3 * il + ik];
          if (il == ik) C = C + F[0];
          C = C * two;
          int dof = m.edof[8 * e + kn0] + ik;
          if (m.dct[dof] == 1) addA(Af, (size_t)dof * lda + row, C);
          else bc[il] = bc[il] - C * cval(m.dcv, dof, z);
        }
      }
    } else {
      double phi[8];
      phi_q8<double>(m.cp_xi[2 * cp], m.cp_xi[2 * cp + 1], phi);
      for (int kn = 0; kn < 8; ++kn)
        for (int il = 0; il < 3; ++il) {
          const size_t row = dn_row(m, dn, il);
          T v = fr(0.5 * phi[kn] * two, z);
          int dof = m.edof[8 * e + kn] + il;
          if (m.dct[dof] == 1) addA(Af, (size_t)dof * lda + row, v);
          else bc[il] = bc[il] - v * cval(m.dcv, dof, z);
        }
    }
  }
  for (int il = 0; il < 3; ++il) addA(bf, dn_row(m, dn, il), bc[il]);
}

// ============================================================================
// Mixed-precision regular pairs (time-harmonic). Only x - x_i is formed in
// binary64; the distance, the decomposed exponentials E_n of both wavenumbers,
// the linear combinations forming psi, chi, TT1..TT3, the fundamental solutions
// and the quadrature sums run in double-float arithmetic (dev_df64.cuh) on the
// FP32 pipe. Used by the mixed sweep only: regular (far-field) pairs have smooth
// integrands, and double-float keeps them at ~1e-14 relative; singular and
// quasi-singular pairs stay FP64.
// ============================================================================

// Coefficients of one frequency in double-float. The five combinations
// X = psi, chi, TT1, TT2, TT3 of bem_harela3d.f90:654-688 are written as
//   X = c0[X] r^-p + c1[X] + sum_{w=1,2} sum_{n=2..5} cm[w][n-2][X] E_n(-i k_w r) r^-(n-1)
// (p = 1 for psi and chi, 2 for TT1..TT3); cm holds the reference's psi(6),
// chi(6), T1(10), T2(9), T3(9) at the places of the terms they multiply and
// zero elsewhere, so one loop over (w, n) evaluates all five.
struct HarParF {
  cf k1, k2, cte_u, cte_t;
  cf c0[5], c1[5];
  cf cm[2][4][5];
  unsigned nz[2][4];  // bit t set: cm[w][n][t] is not structurally zero
  float t2[16];       // E_n series-length steps on |z|^2 (ZexpSteps as binary32)
};
__global__ void k_harpar_f(const HarParD* p, HarParF* out, int nf) {
  int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nf) return;
  const HarParD& P = p[f];
  HarParF o;
  auto c = [](const cd& v) { return cf_from(v.re, v.im); };
  const cf Z = cf_zero(), ONE = cf{ff{1.0f, 0.0f}, ff_zero()};
  o.k1 = c(P.k1);
  o.k2 = c(P.k2);
  o.cte_u = c(P.cte_u);
  o.cte_t = c(P.cte_t);
  // targets 0 psi, 1 chi, 2 TT1, 3 TT2, 4 TT3
  o.c0[0] = c(P.psi[0]); o.c0[1] = c(P.chi[0]); o.c0[2] = c(P.T1[0]); o.c0[3] = c(P.T2[0]); o.c0[4] = c(P.T3[0]);
  o.c1[0] = c(P.psi[1]); o.c1[1] = Z;           o.c1[2] = c(P.T1[1]); o.c1[3] = c(P.T2[1]); o.c1[4] = c(P.T3[1]);
  // wavenumber k1 (w = 0), n = 2..5
  const cf k1t[4][5] = {{Z, c(P.chi[1]), c(P.T1[2]), Z, c(P.T3[2])},
                        {c(P.psi[2]), c(P.chi[2]), c(P.T1[4]), c(P.T2[3]), c(P.T3[3])},
                        {c(P.psi[4]), c(P.chi[4]), c(P.T1[6]), c(P.T2[5]), c(P.T3[5])},
                        {Z, Z, c(P.T1[8]), c(P.T2[7]), c(P.T3[7])}};
  // wavenumber k2 (w = 1)
  const cf k2t[4][5] = {{ONE, ONE, c(P.T1[3]), c(P.T2[2]), Z},
                        {c(P.psi[3]), c(P.chi[3]), c(P.T1[5]), c(P.T2[4]), c(P.T3[4])},
                        {c(P.psi[5]), c(P.chi[5]), c(P.T1[7]), c(P.T2[6]), c(P.T3[6])},
                        {Z, Z, c(P.T1[9]), c(P.T2[8]), c(P.T3[8])}};
  for (int n = 0; n < 4; ++n) {
    o.nz[0][n] = o.nz[1][n] = 0u;
    for (int t = 0; t < 5; ++t) {
      o.cm[0][n][t] = k1t[n][t];
      o.cm[1][n][t] = k2t[n][t];
      if (k1t[n][t].re.hi != 0.0f || k1t[n][t].im.hi != 0.0f) o.nz[0][n] |= 1u << t;
      if (k2t[n][t].re.hi != 0.0f || k2t[n][t].im.hi != 0.0f) o.nz[1][n] |= 1u << t;
    }
  }
  for (int i = 0; i < 16; ++i) o.t2[i] = (float)P.steps.t2[i];
  out[f] = o;
}
// binary64 dataset arrays (phi*J*w, unit normals) as double-float, once per mesh
__global__ void k_pphi_f(const double* pphi, ff* out, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    out[i] = ff_from(pphi[i]);
}

__device__ __forceinline__ int zexp_nterms_f(const float* t2, float az2) {
  if (az2 <= 1e-12f) return 1;
  int lo = 0, hi = 15;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (az2 < t2[mid]) hi = mid;
    else lo = mid + 1;
  }
  return lo + 1;
}

// E_2..E_5 of z in double-float. |z| <= 1: the series of numerical.f90:1286-1301
// with the same number of terms, E_6 = z^6/6! t, t = sum_{m=0..M} c_m z^m,
// c_m = 6!/(6+m)!: the terms m <= 6 in double-float (Horner), the tail m >= 7
// in FP32 -- it is at most 720/13! = 1.2e-7 of t, so its FP32 rounding stays
// near 1e-14 of t (and 3e-15 of E_5). |z| > 1: e^z minus its leading terms.
__device__ __forceinline__ void zexp_2to5_ff(const float* t2, cf z, cf& E2, cf& E3, cf& E4, cf& E5) {
  const float az2 = __fmaf_rn(z.re.hi, z.re.hi, __fmul_rn(z.im.hi, z.im.hi));
  cf z2 = cf_mul(z, z), z3 = cf_mul(z2, z), z4 = cf_mul(z3, z);
  if (az2 <= 1.0f) {
    const int M = zexp_nterms_f(t2, az2);
    const int H = M < 6 ? M : 6;
    // tail / z^7 in FP32
    float qr = 0.0f, qi = 0.0f;
    const float zr = z.re.hi, zi = z.im.hi;
    if (M >= 7) {
      qr = c_df.zc32[M];
#pragma unroll 1
      for (int m = M - 1; m >= 7; --m) {
        const float nr = __fmaf_rn(qr, zr, __fmaf_rn(-qi, zi, c_df.zc32[m]));
        qi = __fmaf_rn(qr, zi, __fmul_rn(qi, zr));
        qr = nr;
      }
    }
    cf t = cf{c_df.zc[H], ff_zero()};
#pragma unroll 1
    for (int m = H - 1; m >= 0; --m) {
      t = cf_mul(t, z);
      t.re = ff_add(t.re, c_df.zc[m]);
    }
    cf z5 = cf_mul(z4, z), z6 = cf_mul(z5, z);
    if (M >= 7) {
      // z^7 q in FP32, added to the double-float head
      const float z7r = __fmaf_rn(z6.re.hi, zr, -__fmul_rn(z6.im.hi, zi));
      const float z7i = __fmaf_rn(z6.re.hi, zi, __fmul_rn(z6.im.hi, zr));
      t.re = ff_add(t.re, ff{__fmaf_rn(z7r, qr, -__fmul_rn(z7i, qi)), 0.0f});
      t.im = ff_add(t.im, ff{__fmaf_rn(z7r, qi, __fmul_rn(z7i, qr)), 0.0f});
    }
    cf e6 = cf_mul(cf_scale(z6, c_df.inv_fact[6]), t);
    E5 = cf_add(e6, cf_scale(z5, c_df.inv_fact[5]));
    E4 = cf_add(E5, cf_scale(z4, c_df.inv_fact[4]));
    E3 = cf_add(E4, cf_scale(z3, c_df.inv_fact[3]));
    E2 = cf_add(E3, cf_scale(z2, c_df.inv_fact[2]));
  } else {
    ff ex = ff_exp(z.re), sn, cs;
    ff_sincos(z.im, &sn, &cs);
    cf e0 = cf{ff_mul(ex, cs), ff_mul(ex, sn)};
    e0.re = ff_sub(e0.re, ff{1.0f, 0.0f});
    E2 = cf_add(e0, cf_neg(z));
    E3 = cf_add(E2, cf_neg(cf_scale(z2, c_df.inv_fact[2])));
    E4 = cf_add(E3, cf_neg(cf_scale(z3, c_df.inv_fact[3])));
    E5 = cf_add(E4, cf_neg(cf_scale(z4, c_df.inv_fact[4])));
  }
}

__device__ __forceinline__ ff sel3(const ff v[3], int i) { return i == 0 ? v[0] : (i == 1 ? v[1] : v[2]); }
__device__ __forceinline__ cf sel4(cf a, cf b, cf c, cf d, int i) { return i == 0 ? a : (i == 1 ? b : (i == 2 ? c : d)); }

// u*, t* (without constants) at one regular point (bem_harela3d.f90:654-688),
// all in double-float, written to fu6 (the six il <= ik components of u*) and
// ft (9). Loops are kept rolled: the kernel is bound by instruction fetch when
// this function is fully unrolled.
__device__ __forceinline__ void harela_point_ff(const HarParF& q, const ff rv[3], const ff n[3], cf* fu6, cf* ft) {
  const ff r2 = ff_add(ff_add(ff_mul(rv[0], rv[0]), ff_mul(rv[1], rv[1])), ff_mul(rv[2], rv[2]));
  const ff r = ff_sqrt(r2);
  const ff d1r1 = ff_rcp(r), d1r2 = ff_mul(d1r1, d1r1);
  cf X[5];
#pragma unroll
  for (int t = 0; t < 5; ++t) X[t] = cf_add(cf_scale(q.c0[t], t < 2 ? d1r1 : d1r2), q.c1[t]);
#pragma unroll 1
  for (int w = 0; w < 2; ++w) {
    const cf k = w ? q.k2 : q.k1;
    const cf z = cf{ff_mul(k.im, r), ff_neg(ff_mul(k.re, r))};  // -i k r
    cf e2, e3, e4, e5;
    zexp_2to5_ff(q.t2, z, e2, e3, e4, e5);
    ff rp = d1r1;
#pragma unroll 1
    for (int nn = 0; nn < 4; ++nn) {
      const cf src = cf_scale(sel4(e2, e3, e4, e5, nn), rp);
      const unsigned nzm = q.nz[w][nn];
#pragma unroll
      for (int t = 0; t < 5; ++t)
        if (nzm & (1u << t)) acc_cmac(X[t], q.cm[w][nn][t], src);
      rp = ff_mul(rp, d1r1);
    }
  }
  const cf psi = cf_norm(X[0]), chi = cf_norm(X[1]), T1 = cf_norm(X[2]), T2 = cf_norm(X[3]), T3 = cf_norm(X[4]);
  const ff dr[3] = {ff_mul(rv[0], d1r1), ff_mul(rv[1], d1r1), ff_mul(rv[2], d1r1)};
  const ff drdn = ff_add(ff_add(ff_mul(dr[0], n[0]), ff_mul(dr[1], n[1])), ff_mul(dr[2], n[2]));
#pragma unroll 1
  for (int c = 0; c < 9; ++c) {
    const int il = c / 3, ik = c - 3 * il;
    const ff dri = sel3(dr, il), drk = sel3(dr, ik), ni = sel3(n, il), nk = sel3(n, ik);
    const ff rr = ff_mul(dri, drk);
    const ff s1 = il == ik ? ff_add(ff_mul(drk, ni), drdn) : ff_mul(drk, ni);
    cf t = cf_zero();
    acc_cmac_r(t, T1, ff_mul(rr, drdn));
    acc_cmac_r(t, T2, s1);
    acc_cmac_r(t, T3, ff_mul(dri, nk));
    ft[c] = cf_norm(t);
    if (ik >= il) {
      cf u = cf_neg(cf_scale(chi, rr));
      if (il == ik) u = cf_add(u, psi);
      fu6[ik + (il == 1 ? 2 : (il == 2 ? 3 : 0))] = u;
    }
  }
}

template <bool SING> struct alignas(16) ComboF;
template <> struct alignas(16) ComboF<false> {
  cf fu[6], ft[9];
  ff w[8];
  int pair;
};
template <> struct alignas(16) ComboF<true> {
  cf fu[6], ft[9], fc[9];
  ff w[8], wd[8];
  int pair;
};

__device__ __forceinline__ cf cf_sub(cf a, cf b) { return cf_add(a, cf_neg(b)); }
__device__ __forceinline__ cf cval_f(const ff* dcv_f, int dof) { return cf{dcv_f[2 * (size_t)dof], dcv_f[2 * (size_t)dof + 1]}; }
// df64 complex entry {re.hi, re.lo, im.hi, im.lo} += v
// A(idx) += v: the pair's double-float sum rounded once to binary64
__device__ __forceinline__ void addAc(double2* A, size_t idx, cf v) {
  double2 a = A[idx];
  a.x += ff_to(v.re);
  a.y += ff_to(v.im);
  A[idx] = a;
}
__device__ __forceinline__ void add3(cf bc[3], int i, cf v) {
  if (i == 0) bc[0] = cf_add(bc[0], v);
  else if (i == 1) bc[1] = cf_add(bc[1], v);
  else bc[2] = cf_add(bc[2], v);
}

// scale, reverse and scatter this lane's outputs of one pair (the scatter of
// flush_pair in double-float; rows 3 dn + il: never used on a region with
// crack-like boundaries): A entries added to the binary64 system,
// prescribed values into the lane's b partial sums bc. hp (singular pairs only): static
// line integrals hli[9] and phi_i[8] of the pair; their CPV part
// T2[0] hli(il,ik) phi_i(kn) is added to the h outputs.
__device__ __forceinline__ void flush_pair_ff(const DMesh& m, const HarParF& q, const ff* dcv_f, int dn, int e,
                                              const cf acc[kAcc], double2* Ac, size_t lda, cf bc[3], const ff* hp) {
  const int lane = threadIdx.x & 31;
  const bool rev = (m.rev[e] & 1) != 0;
#pragma unroll 1
  for (int j = 0; j < kAcc; ++j) {
    const int o = lane + 32 * j;
    if (o >= kOut) break;
    cf aj = cf_norm(sel4(acc[0], acc[1], acc[2], acc[3], j));
    if (o < 72) {
      const int kn = o / 9, il = (o % 9) / 3, ik = o % 3;
      if (hp) aj = cf_add(aj, cf_scale(q.c0[3], ff_mul(hp[9 + kn], hp[3 * il + ik])));
      cf v = cf_mul(aj, q.cte_t);
      if (rev) v = cf_neg(v);
      const int dof = m.edof[8 * e + kn] + ik;
      if (m.dct[dof] == 1) addAc(Ac, (size_t)dof * lda + 3 * (size_t)dn + il, v);
      else add3(bc, il, cf_neg(cf_mul(v, cval_f(dcv_f, dof))));
    } else {
      const int qq = o - 72, kn = qq / 6, sidx = qq % 6, il = sym_il(sidx), ik = sym_ik(sidx);
      const cf v = cf_mul(aj, q.cte_u);
      for (int t = 0; t < (il == ik ? 1 : 2); ++t) {
        const int r_ = t ? ik : il, c_ = t ? il : ik;
        const int dof = m.edof[8 * e + kn] + c_;
        if (m.dct[dof] == 0) addAc(Ac, (size_t)dof * lda + 3 * (size_t)dn + r_, cf_neg(v));
        else add3(bc, r_, cf_mul(v, cval_f(dcv_f, dof)));
      }
    }
  }
}

// Singular (polar) points: the regular parts of u*, t* and the CPV integrand
// (PolHarmonic::point_sing) in double-float. TT2, TT3 without their 1/r^2
// terms; those form fc = T2[0]/r^2 (n_il dr_ik - n_ik dr_il), integrated with
// (phi - phi_i) J w.
__device__ __forceinline__ void harela_point_sing_ff(const HarParF& q, const ff rv[3], const ff n[3], cf* fu6, cf* ft,
                                                     cf* fc) {
  const ff r2 = ff_add(ff_add(ff_mul(rv[0], rv[0]), ff_mul(rv[1], rv[1])), ff_mul(rv[2], rv[2]));
  const ff r = ff_sqrt(r2);
  const ff d1r1 = ff_rcp(r), d1r2 = ff_mul(d1r1, d1r1);
  cf X[5];
#pragma unroll
  for (int t = 0; t < 5; ++t) X[t] = t < 3 ? cf_add(cf_scale(q.c0[t], t < 2 ? d1r1 : d1r2), q.c1[t]) : q.c1[t];
#pragma unroll 1
  for (int w = 0; w < 2; ++w) {
    const cf k = w ? q.k2 : q.k1;
    const cf z = cf{ff_mul(k.im, r), ff_neg(ff_mul(k.re, r))};
    cf e2, e3, e4, e5;
    zexp_2to5_ff(q.t2, z, e2, e3, e4, e5);
    ff rp = d1r1;
#pragma unroll 1
    for (int nn = 0; nn < 4; ++nn) {
      const cf src = cf_scale(sel4(e2, e3, e4, e5, nn), rp);
      const unsigned nzm = q.nz[w][nn];
#pragma unroll
      for (int t = 0; t < 5; ++t)
        if (nzm & (1u << t)) acc_cmac(X[t], q.cm[w][nn][t], src);
      rp = ff_mul(rp, d1r1);
    }
  }
  const cf psi = cf_norm(X[0]), chi = cf_norm(X[1]), T1 = cf_norm(X[2]), T2 = cf_norm(X[3]), T3 = cf_norm(X[4]);
  const cf c2 = cf_scale(q.c0[3], d1r2);
  const cf T2f = cf_add(T2, c2);
  const ff dr[3] = {ff_mul(rv[0], d1r1), ff_mul(rv[1], d1r1), ff_mul(rv[2], d1r1)};
  const ff drdn = ff_add(ff_add(ff_mul(dr[0], n[0]), ff_mul(dr[1], n[1])), ff_mul(dr[2], n[2]));
#pragma unroll 1
  for (int c = 0; c < 9; ++c) {
    const int il = c / 3, ik = c - 3 * il;
    const ff dri = sel3(dr, il), drk = sel3(dr, ik), ni = sel3(n, il), nk = sel3(n, ik);
    const ff rr = ff_mul(dri, drk);
    const ff a = ff_mul(drk, ni), bq = ff_mul(dri, nk);
    cf t = cf_scale(T1, ff_mul(rr, drdn));
    t = cf_fma_r(T2, a, t);
    t = cf_fma_r(T3, bq, t);
    if (il == ik) t = cf_fma_r(T2f, drdn, t);
    ft[c] = t;
    fc[c] = cf_scale(c2, ff_sub(a, bq));
    if (ik >= il) {
      cf u = cf_neg(cf_scale(chi, rr));
      if (il == ik) u = cf_add(u, psi);
      fu6[ik + (il == 1 ? 2 : (il == 2 ? 3 : 0))] = u;
    }
  }
}

// Pair lists walked by the mixed kernels: regular pairs (precalculated element
// datasets), adaptive pairs (subdivision leaves) and singular pairs (polar points).
enum MixKind { MIX_REG = 0, MIX_ADP = 1, MIX_SING = 2 };

// Mixed-precision pair kernels (time-harmonic): one warp per (DOF node,
// frequency), the two-phase scheme of k_reg, all arithmetic after x - x_i in
// double-float; each pair's sums are rounded once to binary64 and added to
// the system Ac (complex entries, stride astride_e per frequency; the warp
// owns its node's rows, so no other warp writes them). dsf: df64 copies of phi*J*w [ne][ptot][8], unit
// normals [ne][ptot][3] and prescribed values [ndof][2]; gf: df64 copy of the
// frequency-independent point geometry (leaf_geo for adaptive, sing_geo for
// singular pairs), component-major.
template <int KIND, int WPB>
__global__ void __launch_bounds__(WPB * 32, 4) k_mixed(DMesh m, const HarParF* pf, const ff* dsf, const ff* gf, int nf,
                                                       double2* Ac, size_t lda, size_t astride_e, double* b,
                                                       size_t bstride) {
  constexpr bool SG = KIND == MIX_SING;
  __shared__ ComboF<SG> sm[WPB][32];
  __shared__ ff hps[WPB][SG ? 17 : 1];
  const int lane = threadIdx.x & 31, w = threadIdx.x / 32;
  const long long gw = blockIdx.x * (long long)WPB + w;
  if (gw >= (long long)m.ndn * nf) return;
  const int dn = (int)(gw % m.ndn), f = (int)(gw / m.ndn);
  ComboF<SG>* S = sm[w];
  const HarParF& Q = pf[f];
  const ff* pphi_f = dsf;
  const ff* pn_f = dsf + 8LL * m.ne * m.ptot;
  const ff* dcv_f = pn_f + 3LL * m.ne * m.ptot;
  double2* Acf = Ac + astride_e * f;
  cf bc[3] = {cf_zero(), cf_zero(), cf_zero()};
  // this lane's output slots: byte offset of its kernel value in the point's
  // ComboF (t* or u* component) << 4 | element node; -1 past the 120 outputs.
  // One path for both kinds, so no slot diverges between t* and u* lanes.
  int slot[kAcc];
#pragma unroll
  for (int j = 0; j < kAcc; ++j) {
    const int o = lane + 32 * j;
    if (o < 72) slot[j] = (int)((offsetof(ComboF<SG>, ft) + sizeof(cf) * (o % 9)) << 4) | (o / 9);
    else if (o < kOut) slot[j] = (int)((offsetof(ComboF<SG>, fu) + sizeof(cf) * ((o - 72) % 6)) << 4) | ((o - 72) / 6);
    else slot[j] = -1;
  }
  for (int cp = m.dn_cp[dn]; cp < m.dn_cp[dn + 1]; ++cp) {
    int s0, s1;
    const long long* pts;
    if (KIND == MIX_REG) {
      s0 = m.reg_start[cp]; s1 = m.reg_start[cp + 1]; pts = m.reg_pt;
    } else if (KIND == MIX_ADP) {
      const int a0 = m.adp_start[cp], a1 = m.adp_start[cp + 1];
      if (a0 == a1) continue;
      s0 = m.adp_leaf[a0]; s1 = m.adp_leaf[a1]; pts = m.leaf_pt;
    } else {
      s0 = m.sing_start[cp]; s1 = m.sing_start[cp + 1]; pts = m.sing_pt;
    }
    if (s0 == s1) continue;
    const double* xi = m.cpx + 3 * (size_t)cp;
    const long long P0 = pts[s0], Qn = pts[s1] - P0;
    int cur = -1;
    cf acc[kAcc];
    for (int j = 0; j < kAcc; ++j) acc[j] = cf_zero();
    for (long long base = 0; base < Qn; base += 32) {
      const long long c = base + lane;
      if (c < Qn) {
        const int jl = find_le(pts, s0, s1, P0 + c);
        ff rv[3], n[3];
        if (KIND == MIX_REG) {
          const int pr = m.reg_pair[jl];
          const int e = pr & 0xFFFFFF, ps = pr >> 24;
          const size_t pt = (size_t)e * m.ptot + m.ps_off[ps] + (size_t)(P0 + c - m.reg_pt[jl]);
          rv[0] = ff_from(m.px[3 * pt] - xi[0]);
          rv[1] = ff_from(m.px[3 * pt + 1] - xi[1]);
          rv[2] = ff_from(m.px[3 * pt + 2] - xi[2]);
          n[0] = pn_f[3 * pt]; n[1] = pn_f[3 * pt + 1]; n[2] = pn_f[3 * pt + 2];
          for (int k = 0; k < 8; ++k) S[lane].w[k] = pphi_f[8 * pt + k];
          S[lane].pair = jl;
        } else {
          const long long g = P0 + c, np = SG ? m.nsing_pts : m.nleaf_pts;
#pragma unroll
          for (int k = 0; k < 3; ++k) {
            rv[k] = gf[k * np + g];
            n[k] = gf[(3 + k) * np + g];
          }
          for (int k = 0; k < 8; ++k) S[lane].w[k] = gf[(6 + k) * np + g];
          if constexpr (SG) {
            for (int k = 0; k < 8; ++k) S[lane].wd[k] = gf[(14 + k) * np + g];
          }
          S[lane].pair = SG ? jl : m.leaf_pair[jl];
        }
        if constexpr (SG) harela_point_sing_ff(Q, rv, n, S[lane].fu, S[lane].ft, S[lane].fc);
        else harela_point_ff(Q, rv, n, S[lane].fu, S[lane].ft);
      }
      __syncwarp();
      const int nt = (int)min((long long)32, Qn - base);
      // one extra step after the last point flushes the last pair (single call site)
      const int tend = (base + 32 >= Qn) ? nt + 1 : nt;
#pragma unroll 1
      for (int t = 0; t < tend; ++t) {
        const int jp = t < nt ? S[t].pair : -1;
        if (jp != cur) {
          if (cur >= 0) {
            const int e = KIND == MIX_REG ? (m.reg_pair[cur] & 0xFFFFFF) : (KIND == MIX_ADP ? m.adp_e[cur] : m.sing_e[cur]);
            flush_pair_ff(m, Q, dcv_f, dn, e, acc, Acf, lda, bc, SG ? hps[w] : nullptr);
          }
          cur = jp;
          for (int j = 0; j < kAcc; ++j) acc[j] = cf_zero();
          if constexpr (SG) {
            __syncwarp();
            if (jp >= 0 && lane < 17) {
              const double* D = m.sing_d + (size_t)jp * SING_D;
              hps[w][lane] = ff_from(lane < 9 ? D[13 + lane] : D[5 + lane - 9]);
            }
            __syncwarp();
          }
        }
        if (t < nt) {
          const char* St = reinterpret_cast<const char*>(&S[t]);
#pragma unroll
          for (int j = 0; j < kAcc; ++j) {
            const int sl = slot[j];
            if (sl >= 0) {
              // compensated accumulation (lo unnormalised until the flush)
              const int kn = sl & 15;
              acc_cmac_r(acc[j], *reinterpret_cast<const cf*>(St + (sl >> 4)), S[t].w[kn]);
              if constexpr (SG) {
                const int o = lane + 32 * j;
                if (o < 72) acc_cmac_r(acc[j], S[t].fc[o % 9], S[t].wd[kn]);
              }
            }
          }
        }
      }
      __syncwarp();
    }
  }
  // b: one warp reduction per DOF node
  double* bf = b + bstride * f;
#pragma unroll 1
  for (int il = 0; il < 3; ++il) {
    cf v = il == 0 ? bc[0] : (il == 1 ? bc[1] : bc[2]);
#pragma unroll 1
    for (int o = 16; o > 0; o >>= 1) {
      cf u;
      u.re.hi = __shfl_xor_sync(0xffffffffu, v.re.hi, o);
      u.re.lo = __shfl_xor_sync(0xffffffffu, v.re.lo, o);
      u.im.hi = __shfl_xor_sync(0xffffffffu, v.im.hi, o);
      u.im.lo = __shfl_xor_sync(0xffffffffu, v.im.lo, o);
      v = cf_add(v, u);
    }
    if (lane == 0) {
      bf[2 * (3 * (size_t)dn + il)] += ff_to(v.re);
      bf[2 * (3 * (size_t)dn + il) + 1] += ff_to(v.im);
    }
  }
}

}  // namespace mfb
