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
  StaelaP k;
  __device__ T cte_t(int) const { return k.ctet1; }
  __device__ T cte_u(int) const { return k.cteu1; }
  __device__ T cpv(int) const { return k.ctet2; }  // coefficient of the CPV/line-integral part
  __device__ void point(int, const double rv[3], const double n[3], T fu[9], T ft[9]) const {
    staela_point(k, rv, n, fu, ft);
  }
  // singular (interior) integration: regular parts and the CPV integrand
  __device__ void point_sing(int, const double rv[3], const double n[3], T fu[9], T ft[9], T fc[9]) const {
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
struct PolHarmonic {
  typedef cd T;
  const HarParD* p;  // one parameter block per frequency
  __device__ T cte_t(int f) const { return p[f].cte_t; }
  __device__ T cte_u(int f) const { return p[f].cte_u; }
  __device__ T cpv(int f) const { return p[f].T2[0]; }
  __device__ void point(int f, const double rv[3], const double n[3], T fu[9], T ft[9]) const {
    harela_point(p[f], rv, n, fu, ft);
  }
  __device__ void point_sing(int f, const double rv[3], const double n[3], T fu[9], T ft[9], T fc[9]) const {
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

// Outputs of one pair handled by the lanes of a warp: o = lane + 32 j, j < 4.
// o < 72: h(kn, il, ik), kn = o / 9; o >= 72: g(kn, s) with s one of the six
// (il <= ik) components (u* is symmetric, so g(kn, il, ik) = g(kn, ik, il)).
constexpr int kOut = 120;
constexpr int kAcc = 4;
__device__ __forceinline__ int sym_il(int s) { return s < 3 ? 0 : (s < 5 ? 1 : 2); }
__device__ __forceinline__ int sym_ik(int s) { return s < 3 ? s : (s < 5 ? s - 2 : 2); }

// Shared flush: scale, reverse, scatter one pair's outputs of this lane set.
template <class POL>
__device__ __forceinline__ void flush_pair(const DMesh& m, const POL& pol, int f, int dn, int e,
                                           typename POL::T acc[kAcc], double* A, size_t lda, size_t astride,
                                           double* b, size_t bstride, const double* hli_phi /* or null */) {
  typedef typename POL::T T;
  const int lane = threadIdx.x & 31;
  T bc[3] = {VT<T>::zero(), VT<T>::zero(), VT<T>::zero()};
  const bool rev = m.rev[e] != 0;
  double* Af = A + astride * f;
  for (int j = 0; j < kAcc; ++j) {
    int o = lane + 32 * j;
    if (o >= kOut) break;
    T v = acc[j];
    if (o < 72) {
      int kn = o / 9, il = (o % 9) / 3, ik = o % 3;
      if (hli_phi) v = v + hli_phi[9 + kn] * pol.cpv(f) * hli_phi[3 * il + ik];
      v = v * pol.cte_t(f);
      if (rev) v = -v;
      int dof = m.edof[8 * e + kn] + ik;
      size_t row = 3 * (size_t)dn + il;
      if (m.dct[dof] == 1) addA(Af, (size_t)dof * lda + row, v);
      else bc[il] = bc[il] - v * cval(m.dcv, dof, v);
    } else {
      int q = o - 72, kn = q / 6, sidx = q % 6, il = sym_il(sidx), ik = sym_ik(sidx);
      v = v * pol.cte_u(f);
      for (int t = 0; t < (il == ik ? 1 : 2); ++t) {
        int r_ = t ? ik : il, c_ = t ? il : ik;
        int dof = m.edof[8 * e + kn] + c_;
        size_t row = 3 * (size_t)dn + r_;
        if (m.dct[dof] == 0) addA(Af, (size_t)dof * lda + row, -v);
        else bc[r_] = bc[r_] + v * cval(m.dcv, dof, v);
      }
    }
  }
  for (int il = 0; il < 3; ++il)
    for (int o = 16; o > 0; o >>= 1) bc[il] = bc[il] + shfl_x(bc[il], o);
  if (lane == 0) {
    double* bf = b + bstride * f;
    for (int il = 0; il < 3; ++il) addA(bf, 3 * (size_t)dn + il, bc[il]);
  }
  __syncwarp();
}

template <typename T>
struct alignas(16) Combo {
  T fu[6], ft[9];
  double w[8];
  int pair;
};
template <typename T>
struct alignas(16) ComboS {
  T fu[6], ft[9], fc[9];
  double w[8], wd[8];
  int pair;
};
// keep the six independent components of the symmetric u*
template <typename T>
__device__ __forceinline__ void store_u6(T* dst, const T fu[9]) {
  dst[0] = fu[0]; dst[1] = fu[1]; dst[2] = fu[2]; dst[3] = fu[4]; dst[4] = fu[5]; dst[5] = fu[8];
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

template <typename T>
__device__ __forceinline__ void accumulate(T acc[kAcc], const T* fu6, const T* ft, const double* w) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int j = 0; j < kAcc; ++j) {
    int o = lane + 32 * j;
    if (o < kOut) {
      T v;
      int kn;
      if (o < 72) {
        kn = o / 9;
        v = ft[o % 9];
      } else {
        kn = (o - 72) / 6;
        v = fu6[(o - 72) % 6];
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
  __shared__ Combo<T> sm[WPB][32];
  const int lane = threadIdx.x & 31, w = threadIdx.x / 32;
  const long long gw = blockIdx.x * (long long)WPB + w;
  if (gw >= (long long)m.ndn * nf) return;
  const int dn = (int)(gw % m.ndn), f = (int)(gw / m.ndn);
  Combo<T>* S = sm[w];
  for (int cp = m.dn_cp[dn]; cp < m.dn_cp[dn + 1]; ++cp) {
    const int s0 = m.reg_start[cp], s1 = m.reg_start[cp + 1];
    if (s0 == s1) continue;
    const double* xi = m.cpx + 3 * (size_t)cp;
    const long long P0 = m.reg_pt[s0], Q = m.reg_pt[s1] - P0;
    int cur = -1;
    T acc[kAcc];
    for (int j = 0; j < kAcc; ++j) acc[j] = VT<T>::zero();
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
        pol.point(f, rv, n, fu9, S[lane].ft);
        store_u6(S[lane].fu, fu9);
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
          for (int j = 0; j < kAcc; ++j) acc[j] = VT<T>::zero();
        }
        accumulate(acc, S[t].fu, S[t].ft, S[t].w);
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
  __shared__ Combo<T> sm[WPB][32];
  const int lane = threadIdx.x & 31, w = threadIdx.x / 32;
  const long long gw = blockIdx.x * (long long)WPB + w;
  if (gw >= (long long)m.ndn * nf) return;
  const int dn = (int)(gw % m.ndn), f = (int)(gw / m.ndn);
  Combo<T>* S = sm[w];
  for (int cp = m.dn_cp[dn]; cp < m.dn_cp[dn + 1]; ++cp) {
    const int a0 = m.adp_start[cp], a1 = m.adp_start[cp + 1];
    if (a0 == a1) continue;
    const int l0 = m.adp_leaf[a0], l1 = m.adp_leaf[a1];
    const double* xi = m.cpx + 3 * (size_t)cp;
    const long long P0 = m.leaf_pt[l0], Q = m.leaf_pt[l1] - P0;
    int cur = -1;
    T acc[kAcc];
    for (int j = 0; j < kAcc; ++j) acc[j] = VT<T>::zero();
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
          pol.point(f, rv, n, fu9, S[lane].ft);
          store_u6(S[lane].fu, fu9);
          for (int q = 0; q < 8; ++q) S[lane].w[q] = G[(6 + q) * np + g];
        } else {
          double rv[3], n[3], w[8];
          leaf_point(m, l, a, (int)(P0 + c - m.leaf_pt[l]), xi, rv, n, w);
          T fu9[9];
          pol.point(f, rv, n, fu9, S[lane].ft);
          store_u6(S[lane].fu, fu9);
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
          for (int j = 0; j < kAcc; ++j) acc[j] = VT<T>::zero();
        }
        accumulate(acc, S[t].fu, S[t].ft, S[t].w);
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
  __shared__ ComboS<T> sm[WPB][32];
  __shared__ double hp[WPB][17];  // hli[9], phi_i[8] of the pair being flushed
  const int lane = threadIdx.x & 31, w = threadIdx.x / 32;
  const long long gw = blockIdx.x * (long long)WPB + w;
  if (gw >= (long long)m.ndn * nf) return;
  const int dn = (int)(gw % m.ndn), f = (int)(gw / m.ndn);
  ComboS<T>* S = sm[w];
  for (int cp = m.dn_cp[dn]; cp < m.dn_cp[dn + 1]; ++cp) {
    const int q0 = m.sing_start[cp], q1 = m.sing_start[cp + 1];
    if (q0 == q1) continue;
    const long long P0 = m.sing_pt[q0], Q = m.sing_pt[q1] - P0;
    int cur = -1;
    T acc[kAcc], acd[kAcc];
    for (int j = 0; j < kAcc; ++j) acc[j] = acd[j] = VT<T>::zero();
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
        pol.point_sing(f, rv, n, fu9, S[lane].ft, S[lane].fc);
        store_u6(S[lane].fu, fu9);
        S[lane].pair = q;
      }
      __syncwarp();
      int nt = (int)min((long long)32, Q - base);
      for (int t = 0; t < nt; ++t) {
        int q = S[t].pair;
        if (q != cur) {
          if (cur >= 0) {
            for (int j = 0; j < kAcc; ++j) acc[j] = acc[j] + acd[j];
            flush_pair(m, pol, f, dn, m.sing_e[cur], acc, A, lda, astride, b, bstride, hp[w]);
          }
          cur = q;
          for (int j = 0; j < kAcc; ++j) acc[j] = acd[j] = VT<T>::zero();
          if (lane < 17) {
            const double* D = m.sing_d + (size_t)q * SING_D;
            hp[w][lane] = lane < 9 ? D[13 + lane] : D[5 + lane - 9];
          }
          __syncwarp();
        }
        accumulate(acc, S[t].fu, S[t].ft, S[t].w);
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
      for (int j = 0; j < kAcc; ++j) acc[j] = acc[j] + acd[j];
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
  double* Af = A + astride * f;
  double* bf = b + bstride * f;
  const T z = VT<T>::zero();
  T bc[3] = {z, z, z};
  for (int cp = m.dn_cp[dn]; cp < m.dn_cp[dn + 1]; ++cp) {
    int e = m.cp_elem[cp], kn0 = m.cp_kn[cp];
    if (m.cp_kind[cp] == 0) {
      if (!m.ft_ok[cp]) { atomicExch(err, 1); continue; }
      const double* F = m.ft + (size_t)cp * FT_D;
      T onemnu = one_minus(nu + 2 * f, z);
      T q = -1.0 / ((8.0 * kPi) * onemnu);
      for (int il = 0; il < 3; ++il) {
        size_t row = 3 * (size_t)dn + il;
        for (int ik = 0; ik < 3; ++ik) {
          T C = q * F[1 + 3 * il + ik];
          if (il == ik) C = C + F[0];
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
          size_t row = 3 * (size_t)dn + il;
          T v = fr(0.5 * phi[kn], z);
          int dof = m.edof[8 * e + kn] + il;
          if (m.dct[dof] == 1) addA(Af, (size_t)dof * lda + row, v);
          else bc[il] = bc[il] - v * cval(m.dcv, dof, z);
        }
    }
  }
  for (int il = 0; il < 3; ++il) addA(bf, 3 * (size_t)dn + il, bc[il]);
}

// ============================================================================
// Mixed-precision regular pairs (time-harmonic). The exponential decomposition
// E_n and the geometry stay in binary64; the linear combinations forming psi,
// chi, TT1..TT3, the fundamental solutions and the quadrature sums run in
// double-float arithmetic (dev_df64.cuh) on the FP32 pipe. Used by the mixed
// sweep only: regular (far-field) pairs have smooth integrands, and double-float
// keeps them at ~1e-14 relative; singular and quasi-singular pairs stay FP64.
// ============================================================================

struct HarParF {
  cf psi[6], chi[6], T1[10], T2[9], T3[9];
};
__global__ void k_harpar_f(const HarParD* p, HarParF* out, int nf) {
  int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nf) return;
  HarParF o;
  for (int i = 0; i < 6; ++i) o.psi[i] = cf_from(p[f].psi[i].re, p[f].psi[i].im);
  for (int i = 0; i < 6; ++i) o.chi[i] = cf_from(p[f].chi[i].re, p[f].chi[i].im);
  for (int i = 0; i < 10; ++i) o.T1[i] = cf_from(p[f].T1[i].re, p[f].T1[i].im);
  for (int i = 0; i < 9; ++i) o.T2[i] = cf_from(p[f].T2[i].re, p[f].T2[i].im);
  for (int i = 0; i < 9; ++i) o.T3[i] = cf_from(p[f].T3[i].re, p[f].T3[i].im);
  out[f] = o;
}
// phi*J*w of the element datasets as double-float, once per mesh
__global__ void k_pphi_f(const double* pphi, ff* out, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    out[i] = ff_from(pphi[i]);
}

__device__ __forceinline__ cf cfc(const cd& v) { return cf_from(v.re, v.im); }

// u*, t* (without constants) at one regular point, df64 combination stage
__device__ __forceinline__ void harela_point_f(const HarParD& p, const HarParF& q, const double rv[3], const double n[3],
                                               cf fu6[6], cf ft[9]) {
  double r = sqrt(rv[0] * rv[0] + rv[1] * rv[1] + rv[2] * rv[2]);
  double d1r1 = 1.0 / r, d1r2 = d1r1 * d1r1, d1r3 = d1r2 * d1r1, d1r4 = d1r3 * d1r1;
  cd z1 = mk(p.k1.im * r, -p.k1.re * r), z2 = mk(p.k2.im * r, -p.k2.re * r);
  cd a2, a3, a4, a5, b2, b3, b4, b5;
  zexp_2to5(p.steps, z1, a2, a3, a4, a5);
  zexp_2to5(p.steps, z2, b2, b3, b4, b5);
  cf A2 = cfc(a2 * d1r1), A3 = cfc(a3 * d1r2), A4 = cfc(a4 * d1r3), A5 = cfc(a5 * d1r4);
  cf B2 = cfc(b2 * d1r1), B3 = cfc(b3 * d1r2), B4 = cfc(b4 * d1r3), B5 = cfc(b5 * d1r4);
  ff D1 = ff_from(d1r1), D2 = ff_from(d1r2);
  cf psi = cf_add(cf_add(cf_scale(q.psi[0], D1), q.psi[1]), B2);
  psi = cf_fma(q.psi[2], A3, psi);
  psi = cf_fma(q.psi[3], B3, psi);
  psi = cf_fma(q.psi[4], A4, psi);
  psi = cf_fma(q.psi[5], B4, psi);
  cf chi = cf_add(cf_add(cf_scale(q.chi[0], D1), B2), cf_mul(q.chi[1], A2));
  chi = cf_fma(q.chi[2], A3, chi);
  chi = cf_fma(q.chi[3], B3, chi);
  chi = cf_fma(q.chi[4], A4, chi);
  chi = cf_fma(q.chi[5], B4, chi);
  cf T1 = cf_add(cf_scale(q.T1[0], D2), q.T1[1]);
  T1 = cf_fma(q.T1[2], A2, T1);
  T1 = cf_fma(q.T1[3], B2, T1);
  T1 = cf_fma(q.T1[4], A3, T1);
  T1 = cf_fma(q.T1[5], B3, T1);
  T1 = cf_fma(q.T1[6], A4, T1);
  T1 = cf_fma(q.T1[7], B4, T1);
  T1 = cf_fma(q.T1[8], A5, T1);
  T1 = cf_fma(q.T1[9], B5, T1);
  cf T2 = cf_add(cf_scale(q.T2[0], D2), q.T2[1]);
  T2 = cf_fma(q.T2[2], B2, T2);
  T2 = cf_fma(q.T2[3], A3, T2);
  T2 = cf_fma(q.T2[4], B3, T2);
  T2 = cf_fma(q.T2[5], A4, T2);
  T2 = cf_fma(q.T2[6], B4, T2);
  T2 = cf_fma(q.T2[7], A5, T2);
  T2 = cf_fma(q.T2[8], B5, T2);
  cf T3 = cf_add(cf_scale(q.T3[0], D2), q.T3[1]);
  T3 = cf_fma(q.T3[2], A2, T3);
  T3 = cf_fma(q.T3[3], A3, T3);
  T3 = cf_fma(q.T3[4], B3, T3);
  T3 = cf_fma(q.T3[5], A4, T3);
  T3 = cf_fma(q.T3[6], B4, T3);
  T3 = cf_fma(q.T3[7], A5, T3);
  T3 = cf_fma(q.T3[8], B5, T3);
  double drd[3] = {rv[0] * d1r1, rv[1] * d1r1, rv[2] * d1r1};
  double drdn_d = drd[0] * n[0] + drd[1] * n[1] + drd[2] * n[2];
  ff dr[3] = {ff_from(drd[0]), ff_from(drd[1]), ff_from(drd[2])};
  ff nn[3] = {ff_from(n[0]), ff_from(n[1]), ff_from(n[2])};
  ff drdn = ff_from(drdn_d);
  cf T2dn = cf_scale(T2, drdn);
  int s = 0;
#pragma unroll
  for (int il = 0; il < 3; ++il)
#pragma unroll
    for (int ik = 0; ik < 3; ++ik) {
      ff rr = ff_mul(dr[il], dr[ik]);
      cf t = cf_scale(T1, ff_mul(rr, drdn));
      t = cf_fma_r(T2, ff_mul(dr[ik], nn[il]), t);
      t = cf_fma_r(T3, ff_mul(dr[il], nn[ik]), t);
      if (il == ik) t = cf_add(t, T2dn);
      ft[3 * il + ik] = t;
      if (ik >= il) {
        cf u = cf_neg(cf_scale(chi, rr));
        if (il == ik) u = cf_add(u, psi);
        fu6[s++] = u;
      }
    }
}

struct alignas(16) ComboF {
  cf fu[6], ft[9];
  ff w[8];
  int pair;
};

template <int WPB>
__global__ void __launch_bounds__(WPB * 32) k_reg_mixed(DMesh m, PolHarmonic pol, const HarParF* pf, const ff* pphi_f,
                                                        int nf, double* A, size_t lda, size_t astride, double* b,
                                                        size_t bstride) {
  __shared__ ComboF sm[WPB][32];
  const int lane = threadIdx.x & 31, w = threadIdx.x / 32;
  const long long gw = blockIdx.x * (long long)WPB + w;
  if (gw >= (long long)m.ndn * nf) return;
  const int dn = (int)(gw % m.ndn), f = (int)(gw / m.ndn);
  ComboF* S = sm[w];
  const HarParD& P = pol.p[f];
  const HarParF& Q = pf[f];
  for (int cp = m.dn_cp[dn]; cp < m.dn_cp[dn + 1]; ++cp) {
    const int s0 = m.reg_start[cp], s1 = m.reg_start[cp + 1];
    if (s0 == s1) continue;
    const double* xi = m.cpx + 3 * (size_t)cp;
    const long long P0 = m.reg_pt[s0], Qn = m.reg_pt[s1] - P0;
    int cur = -1;
    cf acc[kAcc];
    for (int j = 0; j < kAcc; ++j) acc[j] = cf_zero();
    for (long long base = 0; base < Qn; base += 32) {
      long long c = base + lane;
      if (c < Qn) {
        int jp = find_le(m.reg_pt, s0, s1, P0 + c);
        int pr = m.reg_pair[jp];
        int e = pr & 0xFFFFFF, ps = pr >> 24;
        size_t pt = (size_t)e * m.ptot + m.ps_off[ps] + (size_t)(P0 + c - m.reg_pt[jp]);
        double rv[3] = {m.px[3 * pt] - xi[0], m.px[3 * pt + 1] - xi[1], m.px[3 * pt + 2] - xi[2]};
        double n[3] = {m.pn[3 * pt], m.pn[3 * pt + 1], m.pn[3 * pt + 2]};
        harela_point_f(P, Q, rv, n, S[lane].fu, S[lane].ft);
        for (int k = 0; k < 8; ++k) S[lane].w[k] = pphi_f[8 * pt + k];
        S[lane].pair = jp;
      }
      __syncwarp();
      int nt = (int)min((long long)32, Qn - base);
      for (int t = 0; t < nt; ++t) {
        int jp = S[t].pair;
        if (jp != cur) {
          if (cur >= 0) {
            cd a[kAcc];
            for (int j = 0; j < kAcc; ++j) a[j] = mk(ff_to(acc[j].re), ff_to(acc[j].im));
            flush_pair(m, pol, f, dn, m.reg_pair[cur] & 0xFFFFFF, a, A, lda, astride, b, bstride, nullptr);
          }
          cur = jp;
          for (int j = 0; j < kAcc; ++j) acc[j] = cf_zero();
        }
#pragma unroll
        for (int j = 0; j < kAcc; ++j) {
          int o = lane + 32 * j;
          if (o < kOut) {
            cf v;
            int kn;
            if (o < 72) {
              kn = o / 9;
              v = S[t].ft[o % 9];
            } else {
              kn = (o - 72) / 6;
              v = S[t].fu[(o - 72) % 6];
            }
            acc[j] = cf_fma_r(v, S[t].w[kn], acc[j]);
          }
        }
      }
      __syncwarp();
    }
    if (cur >= 0) {
      cd a[kAcc];
      for (int j = 0; j < kAcc; ++j) a[j] = mk(ff_to(acc[j].re), ff_to(acc[j].im));
      flush_pair(m, pol, f, dn, m.reg_pair[cur] & 0xFFFFFF, a, A, lda, astride, b, bstride, nullptr);
    }
  }
}

}  // namespace mfb
