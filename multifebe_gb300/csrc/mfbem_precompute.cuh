// Frequency-independent, once-per-mesh device work: Gauss-point datasets of
// every element (bem_general.f90:163-759), classification of every
// (collocation point, element) pair as in sbie_auto (bem_staela3d.f90:524-589),
// subdivision trees of the adaptive pairs (sbie_ext_adp, bem_staela3d.f90:973-1096),
// polar layouts and static line integrals of the singular pairs
// (sbie_int / sbie_int_li, bem_staela3d.f90:1100-1381, 2245-2376) and the
// geometric part of the free terms (bem_staela3d.f90:228-405).
#pragma once
#include "bem_common.h"
#include "mfbem_dev.h"

namespace mfb {

// ---------------------------------------------------------------- datasets
__global__ void k_datasets(DMesh m) {
  const int e = blockIdx.x;
  const double* x = m.ex + 24 * (size_t)e;
  for (int t = threadIdx.x; t < m.ptot; t += blockDim.x) {
    int ps = 0;
    while (ps + 1 < m.nps && m.ps_off[ps + 1] <= t) ++ps;
    int g = m.ps_gln[ps];
    int kt = t - m.ps_off[ps];
    int k1 = kt / g + 1, k2 = kt % g + 1;  // kt = (k2-1) + (k1-1)*g
    double x1 = gl11x(k1, g), x2 = gl11x(k2, g), w1 = gl11w(k1, g), w2 = gl11w(k2, g);
    double xp[3], T1[3], T2[3], phi[8], N[3];
    geom_q8(x, x1, x2, xp, T1, T2, phi);
    cross3(T1, T2, N);
    double j = norm3(N);
    size_t o = (size_t)e * m.ptot + t;
    for (int c = 0; c < 3; ++c) {
      m.px[3 * o + c] = xp[c];
      m.pn[3 * o + c] = N[c] / j;
    }
    for (int k = 0; k < 8; ++k) m.pphi[8 * o + k] = phi[k] * j * w1 * w2;
  }
}

// ---------------------------------------------------------------- classification
__global__ void k_classify(DMesh m, const QsCurves* __restrict__ qs) {
  const long long total = (long long)m.ncp * m.ne;
  for (long long id = blockIdx.x * (long long)blockDim.x + threadIdx.x; id < total;
       id += (long long)gridDim.x * blockDim.x) {
    int cp = (int)(id / m.ne), e = (int)(id % m.ne);
    const double* xi = m.cpx + 3 * (size_t)cp;
    const double* b = m.ball + 4 * (size_t)e;
    double r0 = b[0] - xi[0], r1 = b[1] - xi[1], r2 = b[2] - xi[2];
    double rmin = sqrt(r0 * r0 + r1 * r1 + r2 * r2) - b[3];
    double bx[2] = {0.0, 0.0}, d;
    uint8_t c;
    bool sing = false;
    if (rmin > 4.0 * b[3]) {
      d = rmin / m.cl[e];
    } else {
      int method;
      nearest_q8(m.ex + 24 * (size_t)e, m.cl[e], xi, bx, &rmin, &d, &method);
      sing = (d <= 1e-12);
    }
    if (sing) {
      c = CLS_SING;
    } else {
      int gn = qs_estimate(*qs, 2, m.fcls, d, bx, false);
      int gln = max(m.gln_far[e], gn);
      if (gln <= m.ps_gln_max && gn > 0) {
        int ps = 0;
        for (int i = 0; i < m.nps; ++i)
          if (m.ps_gln[i] >= gln) { ps = i; break; }
        c = (uint8_t)ps;
      } else {
        c = CLS_ADP;
      }
    }
    m.cls[id] = c;
  }
}

// per collocation point: number of regular / adaptive / singular pairs and of
// regular Gauss points (one warp per point)
__global__ void k_count(DMesh m, int* nreg, int* nadp, int* nsing, long long* npts) {
  int cp = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  int lane = threadIdx.x & 31;
  if (cp >= m.ncp) return;
  int a = 0, b = 0, c = 0;
  long long p = 0;
  const uint8_t* row = m.cls + (size_t)cp * m.ne;
  for (int e = lane; e < m.ne; e += 32) {
    uint8_t k = row[e];
    if (k == CLS_ADP) ++b;
    else if (k == CLS_SING) ++c;
    else { ++a; p += (long long)m.ps_gln[k] * m.ps_gln[k]; }
  }
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    b += __shfl_xor_sync(0xffffffffu, b, o);
    c += __shfl_xor_sync(0xffffffffu, c, o);
    p += __shfl_xor_sync(0xffffffffu, p, o);
  }
  if (lane == 0) { nreg[cp] = a; nadp[cp] = b; nsing[cp] = c; npts[cp] = p; }
}

// single-block exclusive scan of n values into out[0..n] (out[n] = total)
template <typename TI, typename TO>
__global__ void k_scan(const TI* in, TO* out, int n) {
  __shared__ TO part[1024];
  __shared__ TO carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < n; base += 1024) {
    int i = base + threadIdx.x;
    TO v = (i < n) ? (TO)in[i] : (TO)0;
    part[threadIdx.x] = v;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {
      TO t = (threadIdx.x >= (unsigned)off) ? part[threadIdx.x - off] : (TO)0;
      __syncthreads();
      part[threadIdx.x] += t;
      __syncthreads();
    }
    if (i < n) out[i] = carry + part[threadIdx.x] - v;
    __syncthreads();
    if (threadIdx.x == 1023) carry += part[1023];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[n] = carry;
}

// fill the per-point lists in element order (one warp per collocation point)
__global__ void k_fill(DMesh m, const long long* pts_base, int* adp_cp, int* sing_cp) {
  int cp = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  int lane = threadIdx.x & 31;
  if (cp >= m.ncp) return;
  const uint8_t* row = m.cls + (size_t)cp * m.ne;
  int ra = m.reg_start[cp], rb = m.adp_start[cp], rc = m.sing_start[cp];
  long long pb = pts_base[cp];
  const unsigned lt = (1u << lane) - 1u;
  for (int e0 = 0; e0 < m.ne; e0 += 32) {
    int e = e0 + lane;
    uint8_t k = (e < m.ne) ? row[e] : (uint8_t)253;
    bool isr = (e < m.ne) && k != CLS_ADP && k != CLS_SING;
    bool isa = (e < m.ne) && k == CLS_ADP;
    bool iss = (e < m.ne) && k == CLS_SING;
    unsigned mr = __ballot_sync(0xffffffffu, isr), ma = __ballot_sync(0xffffffffu, isa),
             ms = __ballot_sync(0xffffffffu, iss);
    long long np = isr ? (long long)m.ps_gln[k] * m.ps_gln[k] : 0;
    // inclusive scan of np over the warp
    long long inc = np;
    for (int o = 1; o < 32; o <<= 1) {
      long long t = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= o) inc += t;
    }
    if (isr) {
      int j = ra + __popc(mr & lt);
      m.reg_pair[j] = e | ((int)k << 24);
      m.reg_pt[j] = pb + inc - np;
    }
    if (isa) { int j = rb + __popc(ma & lt); m.adp_e[j] = e; adp_cp[j] = cp; }
    if (iss) { int j = rc + __popc(ms & lt); m.sing_e[j] = e; sing_cp[j] = cp; }
    ra += __popc(mr);
    rb += __popc(ma);
    rc += __popc(ms);
    pb += __shfl_sync(0xffffffffu, inc, 31);
  }
}

// ---------------------------------------------------------------- adaptive subdivision
// Depth-first traversal of sbie_ext_adp's 1/4 subdivision tree with an explicit
// stack; children are visited in the reference's order (subquads 1..4).
struct AdpNode {
  double xs[8];
  int ks;
};
template <bool WRITE>
__device__ int adp_traverse(const DMesh& m, const QsCurves& qs, int e, const double* xi, double* leaf_out,
                            int* gln_out, int* pair_out, int pair_id, long long* npts = nullptr) {
  AdpNode st[52];
  int top = 0;
  const double* x = m.ex + 24 * (size_t)e;
  st[top].xs[0] = -1; st[top].xs[1] = -1; st[top].xs[2] = 1; st[top].xs[3] = -1;
  st[top].xs[4] = 1;  st[top].xs[5] = 1;  st[top].xs[6] = -1; st[top].xs[7] = 1;
  st[top].ks = 1;
  ++top;
  int nleaf = 0;
  while (top > 0) {
    AdpNode nd = st[--top];
    double bx[2], rmin, d;
    int method;
    if (nd.ks == 1) {
      nearest_q8(x, m.cl[e], xi, bx, &rmin, &d, &method);
    } else {
      double xsub[24];
      subdiv_q8(x, nd.xs, xsub);
      double cl = clen_q8(xsub, 1e-12);
      nearest_q8(xsub, cl, xi, bx, &rmin, &d, &method);
    }
    int gn = qs_estimate(qs, 2, m.fadp, d, bx, true);
    bool sub = false;
    if (nd.ks == m.ns_max) {
      if (gn == 0) gn = 30;
    } else if (gn == 0) {
      sub = true;
    }
    if (sub && top + 4 <= 52) {
      const double* s = nd.xs;
      double c0 = 0.25 * (s[0] + s[2] + s[4] + s[6]), c1 = 0.25 * (s[1] + s[3] + s[5] + s[7]);
      AdpNode ch[4];
      // SUBQUAD 1..4 as in bem_staela3d.f90:1050-1077
      double q[4][8] = {
          {s[0], s[1], 0.5 * (s[0] + s[2]), 0.5 * (s[1] + s[3]), c0, c1, 0.5 * (s[0] + s[6]), 0.5 * (s[1] + s[7])},
          {0.5 * (s[0] + s[2]), 0.5 * (s[1] + s[3]), s[2], s[3], 0.5 * (s[2] + s[4]), 0.5 * (s[3] + s[5]), c0, c1},
          {c0, c1, 0.5 * (s[2] + s[4]), 0.5 * (s[3] + s[5]), s[4], s[5], 0.5 * (s[4] + s[6]), 0.5 * (s[5] + s[7])},
          {0.5 * (s[0] + s[6]), 0.5 * (s[1] + s[7]), c0, c1, 0.5 * (s[4] + s[6]), 0.5 * (s[5] + s[7]), s[6], s[7]}};
      for (int i = 3; i >= 0; --i) {
        for (int j = 0; j < 8; ++j) st[top].xs[j] = q[i][j];
        st[top].ks = nd.ks + 1;
        ++top;
      }
      (void)ch;
    } else {
      if (WRITE) {
        double barr = telles_barr(d);
        int gln = max(gn, m.gln_far[e]);
        Telles t1 = telles11(bx[0], barr), t2 = telles11(bx[1], barr);
        double* L = leaf_out + (size_t)nleaf * LEAF_D;
        for (int j = 0; j < 8; ++j) L[j] = nd.xs[j];
        L[8] = t1.a; L[9] = t1.b; L[10] = t1.c; L[11] = t1.d;
        L[12] = t2.a; L[13] = t2.b; L[14] = t2.c; L[15] = t2.d;
        gln_out[nleaf] = gln;
        pair_out[nleaf] = pair_id;
      }
      if (npts) {
        const long long g = max(gn, m.gln_far[e]);
        *npts += g * g;
      }
      ++nleaf;
    }
  }
  return nleaf;
}

__global__ void k_adp_count(DMesh m, const QsCurves* qs, const int* adp_cp, int* nleaf) {
  long long a = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (a >= m.nadp) return;
  int cp = adp_cp[a], e = m.adp_e[a];
  nleaf[a] = adp_traverse<false>(m, *qs, e, m.cpx + 3 * (size_t)cp, nullptr, nullptr, nullptr, 0);
}
__global__ void k_adp_fill(DMesh m, const QsCurves* qs, const int* adp_cp) {
  long long a = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (a >= m.nadp) return;
  int cp = adp_cp[a], e = m.adp_e[a];
  int l0 = m.adp_leaf[a];
  adp_traverse<true>(m, *qs, e, m.cpx + 3 * (size_t)cp, m.leaf + (size_t)l0 * LEAF_D, m.leaf_gln + l0,
                     m.leaf_pair + l0, (int)a);
}
__global__ void k_leaf_points(DMesh m, long long* npts) {
  long long l = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (l >= m.nleaf) return;
  long long g = m.leaf_gln[l];
  npts[l] = g * g;
}

// ---------------------------------------------------------------- singular pairs
// Polar layout (polar_transformation.f90:251-500) of a quadrilateral around xi_i.
__device__ void polar_setup(const double xi[2], int* nsub, int st[8], double th[8][2], double thp[8][2]) {
  const double t = kXiTol;
  int n = 0;
  if (!on_quad_edge(xi[0], xi[1])) {
    n = 8;
    for (int k = 0; k < 8; ++k) st[k] = k + 1;
  } else {
    if (xi[0] <= -1.0 + t && xi[1] <= -1.0 + t) { n = 2; st[0] = 4; st[1] = 5; }
    if (xi[0] >= 1.0 - t && xi[1] <= -1.0 + t) { n = 2; st[0] = 6; st[1] = 7; }
    if (xi[0] >= 1.0 - t && xi[1] >= 1.0 - t) { n = 2; st[0] = 8; st[1] = 1; }
    if (xi[0] <= -1.0 + t && xi[1] >= 1.0 - t) { n = 2; st[0] = 2; st[1] = 3; }
    if (n == 0) {
      if (xi[1] <= -1.0 + t) { n = 4; st[0] = 4; st[1] = 5; st[2] = 6; st[3] = 7; }
      if (xi[0] >= 1.0 - t) { n = 4; st[0] = 6; st[1] = 7; st[2] = 8; st[3] = 1; }
      if (xi[1] >= 1.0 - t) { n = 4; st[0] = 8; st[1] = 1; st[2] = 2; st[3] = 3; }
      if (xi[0] <= -1.0 + t) { n = 4; st[0] = 2; st[1] = 3; st[2] = 4; st[3] = 5; }
    }
  }
  *nsub = n;
  const double x1 = xi[0], x2 = xi[1];
  auto th1 = [&]() { return kPi - asin((-1.0 - x2) / sqrt((-1.0 - x1) * (-1.0 - x1) + (-1.0 - x2) * (-1.0 - x2))); };
  auto th2 = [&]() { return k2Pi + asin((-1.0 - x2) / sqrt((1.0 - x1) * (1.0 - x1) + (-1.0 - x2) * (-1.0 - x2))); };
  auto th3 = [&]() { return asin((1.0 - x2) / sqrt((1.0 - x1) * (1.0 - x1) + (1.0 - x2) * (1.0 - x2))); };
  auto th4 = [&]() { return kPi - asin((1.0 - x2) / sqrt((-1.0 - x1) * (-1.0 - x1) + (1.0 - x2) * (1.0 - x2))); };
  for (int k = 0; k < n; ++k) {
    double a = 0, b = 0, f = 0, sh = 0;
    switch (st[k]) {
      case 1: a = th1(); b = 1.5 * kPi; f = 1.0 + x2; sh = -kPi; break;
      case 2: a = 1.5 * kPi; b = th2(); f = 1.0 + x2; sh = -kPi; break;
      case 3: a = th2(); b = k2Pi; f = 1.0 - x1; sh = kPi2; break;
      case 4: a = 0.0; b = th3(); f = 1.0 - x1; sh = kPi2; break;
      case 5: a = th3(); b = kPi2; f = 1.0 - x2; sh = 0.0; break;
      case 6: a = kPi2; b = th4(); f = 1.0 - x2; sh = 0.0; break;
      case 7: a = th4(); b = kPi; f = 1.0 + x1; sh = -kPi2; break;
      default: a = kPi; b = th1(); f = 1.0 + x1; sh = -kPi2; break;
    }
    th[k][0] = a;
    th[k][1] = b;
    if (sh == 0.0) {
      thp[k][0] = f * log(tan(0.5 * a));
      thp[k][1] = f * log(tan(0.5 * b));
    } else {
      thp[k][0] = f * log(tan(0.5 * (a + sh)));
      thp[k][1] = f * log(tan(0.5 * (b + sh)));
    }
  }
}

// polar_transformation.f90:501-546
__device__ __forceinline__ void polar_angular(const double xi[2], int s, double tp, double* theta, double* rho) {
  if (s <= 2) {
    *theta = 2.0 * atan(exp(tp / (1.0 + xi[1]))) + kPi;
    *rho = (-1.0 - xi[1]) / sin(*theta);
  } else if (s <= 4) {
    *theta = 2.0 * atan(exp(tp / (1.0 - xi[0]))) - kPi2;
    *rho = (1.0 - xi[0]) / cos(*theta);
  } else if (s <= 6) {
    *theta = 2.0 * atan(exp(tp / (1.0 - xi[1])));
    *rho = (1.0 - xi[1]) / sin(*theta);
  } else {
    *theta = 2.0 * atan(exp(tp / (1.0 + xi[0]))) + kPi2;
    *rho = (-1.0 - xi[0]) / cos(*theta);
  }
}

// Line integral eps_ijk e_k.t/r over one line3 edge with adaptive Telles +
// bisection (fbem_bem_staela3d_sbie_int_li, bem_staela3d.f90:2245-2376).
__device__ void line_integral(const double* xe, const double* xi_, const QsCurves& q15, double hli[9]) {
  struct It {
    double s0, s1;
    int ks;
  };
  It st[20];
  int top = 0;
  st[top++] = It{-1.0, 1.0, 1};
  while (top > 0) {
    It it = st[--top];
    double xs[9];
    if (it.ks == 1) {
      for (int j = 0; j < 9; ++j) xs[j] = xe[j];
    } else {
      subdiv_l3(xe, it.s0, it.s1, xs);
    }
    double cl = length_l3(xs, 1e-12);
    double bx, rmin, d;
    int method;
    nearest_l3(xs, cl, xi_, &bx, &rmin, &d, &method);
    int gn = qs_estimate(q15, 1, 1, d, &bx, true);
    bool sub = false;
    if (it.ks == 16) {
      if (gn == 0) gn = 30;
    } else if (gn == 0) {
      sub = true;
    }
    if (sub && top + 2 <= 20) {
      double mid = 0.5 * (it.s0 + it.s1);
      st[top++] = It{mid, it.s1, it.ks + 1};
      st[top++] = It{it.s0, mid, it.ks + 1};
    } else {
      int gln = max(gn, 5);
      double barr = telles_barr(d);
      Telles t = telles11(bx, barr);
      double h01 = 0, h02 = 0, h12 = 0;
      for (int k = 1; k <= gln; ++k) {
        double xip, jt;
        telles_map(t, gl11x(k, gln), xip, jt);
        double w = gl11w(k, gln);
        double xi = 0.5 * (1.0 - xip) * it.s0 + 0.5 * (1.0 + xip) * it.s1;
        double js = 0.5 * (it.s1 - it.s0);
        double ph[3], dp[3];
        phi_l3<double>(xi, ph);
        dphi_l3<double>(xi, dp);
        double xp[3] = {0, 0, 0}, T[3] = {0, 0, 0};
        for (int q = 0; q < 3; ++q)
          for (int c = 0; c < 3; ++c) {
            xp[c] = xp[c] + ph[q] * xe[3 * q + c];
            T[c] = T[c] + dp[q] * xe[3 * q + c];
          }
        double jg = norm3(T);
        double tt[3] = {T[0] / jg, T[1] / jg, T[2] / jg};
        double rv[3] = {xp[0] - xi_[0], xp[1] - xi_[1], xp[2] - xi_[2]};
        double dr1 = 1.0 / norm3(rv);
        double jw = jg * js * jt * w;
        h01 = h01 - dr1 * tt[2] * jw;
        h02 = h02 + dr1 * tt[1] * jw;
        h12 = h12 - dr1 * tt[0] * jw;
      }
      hli[1] += h01; hli[2] += h02; hli[5] += h12;
      hli[3] += -h01; hli[6] += -h02; hli[7] += -h12;
    }
  }
}

__global__ void k_sing_prep(DMesh m, const QsCurves* q15, const int* sing_cp, long long* npts) {
  long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q >= m.nsing) return;
  int cp = sing_cp[q], e = m.sing_e[q];
  const double* x = m.ex + 24 * (size_t)e;
  double bx[2], rmin, d;
  int method;
  nearest_q8(x, m.cl[e], m.cpx + 3 * (size_t)cp, bx, &rmin, &d, &method);
  double* D = m.sing_d + (size_t)q * SING_D;
  int* I = m.sing_i + (size_t)q * SING_I;
  D[0] = bx[0];
  D[1] = bx[1];
  double phi[8];
  phi_q8<double>(bx[0], bx[1], phi);
  double xi_[3] = {0, 0, 0};
  for (int k = 0; k < 8; ++k)
    for (int c = 0; c < 3; ++c) xi_[c] = xi_[c] + phi[k] * x[3 * k + c];
  for (int c = 0; c < 3; ++c) D[2 + c] = xi_[c];
  for (int k = 0; k < 8; ++k) D[5 + k] = phi[k];
  int nsub, st[8];
  double th[8][2], thp[8][2];
  polar_setup(bx, &nsub, st, th, thp);
  double hli[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  for (int ke = 1; ke <= 4; ++ke) {
    bool integ = false;
    for (int s = 0; s < nsub; ++s)
      if (st[s] == 2 * ke - 1 || st[s] == 2 * ke) integ = true;
    if (!integ) continue;
    double xe[9];
    for (int n = 0; n < 3; ++n)
      for (int c = 0; c < 3; ++c) xe[3 * n + c] = x[3 * q8edge(ke - 1, n) + c];
    line_integral(xe, xi_, *q15, hli);
  }
  for (int j = 0; j < 9; ++j) D[13 + j] = hli[j];
  I[0] = nsub;
  int off = 0;
  for (int s = 0; s < 8; ++s) {
    int ng = 0;
    if (s < nsub) {
      D[22 + 2 * s] = th[s][0];
      D[23 + 2 * s] = th[s][1];
      D[38 + 2 * s] = thp[s][0];
      D[39 + 2 * s] = thp[s][1];
      double v = 25.0 * (th[s][1] - th[s][0]) / kPi2;
      ng = 5 + (int)(v < 0 ? -floor(-v + 0.5) : floor(v + 0.5));
      I[1 + s] = st[s];
    } else {
      I[1 + s] = 0;
    }
    I[9 + s] = ng;
    I[17 + s] = off;
    off += ng * 15;
  }
  I[25] = off;
  npts[q] = off;
}

// ---------------------------------------------------------------- HBIE singular pairs
// All line integrals of the HBIE interior integration over one line3 edge,
// adaptive Telles + bisection with the 1/r^2 estimate
// (fbem_bem_staela3d_hbie_int_li, bem_staela3d.f90:5356-5578). L: lli[3][3],
// mli1, mli2[3], mli3[3][3], mli4[3], mli5[3][3][3] (HX_* offsets - HX_LLI).
__device__ void hbie_line_integrals(const double* xe, const double* xi_, const double* ni, const QsCurves& q15,
                                    double* L) {
  struct It {
    double s0, s1;
    int ks;
  };
  It st[20];
  int top = 0;
  st[top++] = It{-1.0, 1.0, 1};
  while (top > 0) {
    It it = st[--top];
    double xs[9];
    if (it.ks == 1) {
      for (int j = 0; j < 9; ++j) xs[j] = xe[j];
    } else {
      subdiv_l3(xe, it.s0, it.s1, xs);
    }
    double cl = length_l3(xs, 1e-12);
    double bx, rmin, d;
    int method;
    nearest_l3(xs, cl, xi_, &bx, &rmin, &d, &method);
    int gn = qs_estimate(q15, 1, 2, d, &bx, true);
    bool sub = false;
    if (it.ks == 16) {
      if (gn == 0) gn = 30;
    } else if (gn == 0) {
      sub = true;
    }
    if (sub && top + 2 <= 20) {
      double mid = 0.5 * (it.s0 + it.s1);
      st[top++] = It{mid, it.s1, it.ks + 1};
      st[top++] = It{it.s0, mid, it.ks + 1};
      continue;
    }
    int gln = max(gn, 5);
    Telles t = telles11(bx, telles_barr(d));
    double T[52];
    for (int j = 0; j < 52; ++j) T[j] = 0.0;
    for (int k = 1; k <= gln; ++k) {
      double xip, jt;
      telles_map(t, gl11x(k, gln), xip, jt);
      double w = gl11w(k, gln);
      double xi = 0.5 * (1.0 - xip) * it.s0 + 0.5 * (1.0 + xip) * it.s1;
      double js = 0.5 * (it.s1 - it.s0);
      double ph[3], dp[3];
      phi_l3<double>(xi, ph);
      dphi_l3<double>(xi, dp);
      double xp[3] = {0, 0, 0}, Tg[3] = {0, 0, 0};
      for (int q = 0; q < 3; ++q)
        for (int c = 0; c < 3; ++c) {
          xp[c] = xp[c] + ph[q] * xe[3 * q + c];
          Tg[c] = Tg[c] + dp[q] * xe[3 * q + c];
        }
      double jg = norm3(Tg);
      double tt[3] = {Tg[0] / jg, Tg[1] / jg, Tg[2] / jg};
      double rv[3] = {xp[0] - xi_[0], xp[1] - xi_[1], xp[2] - xi_[2]};
      double r = norm3(rv);
      double dr1 = 1.0 / r, dr3 = 1.0 / (r * r * r);
      double dr[3] = {rv[0] * dr1, rv[1] * dr1, rv[2] * dr1};
      double jw = jg * js * jt * w;
      T[1] = T[1] - dr1 * tt[2] * jw;
      T[2] = T[2] + dr1 * tt[1] * jw;
      T[5] = T[5] - dr1 * tt[0] * jw;
      double rxni[3] = {rv[1] * ni[2] - rv[2] * ni[1], rv[2] * ni[0] - rv[0] * ni[2], rv[0] * ni[1] - rv[1] * ni[0]};
      double rxnit = rxni[0] * tt[0] + rxni[1] * tt[1] + rxni[2] * tt[2];
      T[9] = T[9] + dr3 * rxnit * jw;
      for (int a = 0; a < 3; ++a)
        for (int b = a; b < 3; ++b) T[13 + 3 * a + b] = T[13 + 3 * a + b] + dr3 * rxnit * dr[a] * dr[b] * jw;
      for (int ik = 0; ik < 3; ++ik) {
        // (e_k x n_i).t and (r x e_k).t
        const int i1 = (ik + 1) % 3, i2 = (ik + 2) % 3;
        double ekxnit = ni[i1] * tt[i2] - ni[i2] * tt[i1];
        double rxekt = rv[i2] * tt[i1] - rv[i1] * tt[i2];
        T[10 + ik] = T[10 + ik] + dr1 * ekxnit * jw;
        T[22 + ik] = T[22 + ik] + dr3 * rxekt * jw;
        for (int a = 0; a < 3; ++a)
          for (int b = a; b < 3; ++b)
            T[25 + 9 * a + 3 * b + ik] = T[25 + 9 * a + 3 * b + ik] + dr1 * ekxnit * dr[a] * dr[b] * jw;
      }
    }
    T[3] = -T[1];
    T[6] = -T[2];
    T[7] = -T[5];
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < a; ++b) {
        T[13 + 3 * a + b] = T[13 + 3 * b + a];
        for (int k = 0; k < 3; ++k) T[25 + 9 * a + 3 * b + k] = T[25 + 9 * b + 3 * a + k];
      }
    for (int j = 0; j < 52; ++j) L[j] += T[j];
  }
}

// Extras of the HBIE singular pairs (after k_sing_prep has laid out the polar
// rule and x_i): the unit normal n_i and psi_i, the shape functions'
// tangential gradient in the orthogonal frame v1 = t1, v2 = n_i x t1 at xi_i
// (bem_staela3d.f90:5022-5118), and the line integrals of all four edges.
__global__ void k_hsing_prep(DMesh m, const QsCurves* q15) {
  long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q >= m.nsing) return;
  const int e = m.sing_e[q];
  const double* x = m.ex + 24 * (size_t)e;
  const double* D = m.sing_d + (size_t)q * SING_D;
  double* X = m.hsing_x + (size_t)q * HSING_X;
  double d1[8], d2[8];
  dphi_q8<double>(D[0], D[1], d1, d2);
  double T1[3] = {0, 0, 0}, T2[3] = {0, 0, 0};
  for (int k = 0; k < 8; ++k)
    for (int c = 0; c < 3; ++c) {
      T1[c] = T1[c] + d1[k] * x[3 * k + c];
      T2[c] = T2[c] + d2[k] * x[3 * k + c];
    }
  double N[3];
  cross3(T1, T2, N);
  double jg = norm3(N);
  double ni[3] = {N[0] / jg, N[1] / jg, N[2] / jg};
  double j1 = norm3(T1), j2 = norm3(T2);
  double t1[3] = {T1[0] / j1, T1[1] / j1, T1[2] / j1}, t2[3] = {T2[0] / j2, T2[1] / j2, T2[2] / j2};
  double v2[3];
  cross3(ni, t1, v2);
  double M12 = t1[0] * t2[0] + t1[1] * t2[1] + t1[2] * t2[2], M22 = v2[0] * t2[0] + v2[1] * t2[1] + v2[2] * t2[2];
  double det = M22;  // M11 = 1, M21 = 0
  double x11 = M22 / (j1 * det), x12 = -M12 / (j1 * det), x21 = 0.0 / (j2 * det), x22 = 1.0 / (j2 * det);
  for (int c = 0; c < 3; ++c) X[HX_N + c] = ni[c];
  for (int k = 0; k < 8; ++k)
    for (int c = 0; c < 3; ++c)
      X[HX_PSI + 3 * k + c] = (d1[k] * x11 + d2[k] * x21) * t1[c] + (d1[k] * x12 + d2[k] * x22) * v2[c];
  double L[52];
  for (int j = 0; j < 52; ++j) L[j] = 0.0;
  for (int ke = 0; ke < 4; ++ke) {
    double xe[9];
    for (int n = 0; n < 3; ++n)
      for (int c = 0; c < 3; ++c) xe[3 * n + c] = x[3 * q8edge(ke, n) + c];
    hbie_line_integrals(xe, D + 2, ni, *q15, L);
  }
  for (int j = 0; j < 52; ++j) X[HX_LLI + j] = L[j];
}

// ---------------------------------------------------------------- free terms
// Mantic's C-matrix (bem_staela3d.f90:228-405) for the nodal-SBIE collocation
// points; stores the solid-angle term cp and sum_b (C = cp I - sum_b/(8 pi (1-nu))).
__global__ void k_ft_prep(DMesh m) {
  int cp = blockIdx.x * blockDim.x + threadIdx.x;
  if (cp >= m.ncp) return;
  double* F = m.ft + (size_t)cp * FT_D;
  if (m.cp_kind[cp] != 0) {
    for (int j = 0; j < FT_D; ++j) F[j] = 0.0;
    m.ft_ok[cp] = 1;
    return;
  }
  const int MX = 16;
  int i0 = m.inc_start[cp], ne = m.inc_start[cp + 1] - i0;
  if (ne > MX || ne < 1) { m.ft_ok[cp] = 0; return; }
  double ln[MX + 2][3], lt[MX + 2][3];
  for (int k = 0; k < ne; ++k) {
    int ek = m.inc_el[i0 + k];
    for (int c = 0; c < 3; ++c) {
      ln[k + 1][c] = m.n_gn[3 * (size_t)ek + c];
      lt[k + 1][c] = m.tbp_gn[3 * (size_t)ek + c];
    }
  }
  double ltol = (m.geo_tol < 1e-12 || m.geo_tol > 1e-3) ? 1e-6 : m.geo_tol;
  for (int ki = 1; ki <= ne - 1; ++ki) {
    double e1[3] = {lt[ki][0], lt[ki][1], lt[ki][2]}, e3[3] = {ln[ki][0], ln[ki][1], ln[ki][2]}, e2[3];
    e2[0] = e3[1] * e1[2] - e3[2] * e1[1];
    e2[1] = e3[2] * e1[0] - e3[0] * e1[2];
    e2[2] = e3[0] * e1[1] - e3[1] * e1[0];
    int nc = 0, mk_ = -1;
    double mt = 0;
    for (int kj = ki + 1; kj <= ne; ++kj) {
      double l3 = e3[0] * lt[kj][0] + e3[1] * lt[kj][1] + e3[2] * lt[kj][2];
      if (fabs(l3) <= ltol) {
        double l1 = e1[0] * lt[kj][0] + e1[1] * lt[kj][1] + e1[2] * lt[kj][2];
        double l2 = e2[0] * lt[kj][0] + e2[1] * lt[kj][1] + e2[2] * lt[kj][2];
        double th = atan2(l2, l1);
        if (th < 0.0) th = th + 2.0 * kPi;
        if (nc == 0 || th < mt) { mt = th; mk_ = kj; }
        ++nc;
      }
    }
    if (nc == 0) { m.ft_ok[cp] = 0; return; }
    for (int c = 0; c < 3; ++c) {
      double t = lt[ki + 1][c]; lt[ki + 1][c] = lt[mk_][c]; lt[mk_][c] = t;
      t = ln[ki + 1][c]; ln[ki + 1][c] = ln[mk_][c]; ln[mk_][c] = t;
    }
  }
  for (int c = 0; c < 3; ++c) {
    ln[0][c] = ln[ne][c]; lt[0][c] = lt[ne][c];
    ln[ne + 1][c] = ln[1][c]; lt[ne + 1][c] = lt[1][c];
  }
  double sa = 0.0;
  for (int ki = 1; ki <= ne; ++ki) {
    double nx[3] = {ln[ki - 1][1] * ln[ki][2] - ln[ki - 1][2] * ln[ki][1],
                    ln[ki - 1][2] * ln[ki][0] - ln[ki - 1][0] * ln[ki][2],
                    ln[ki - 1][0] * ln[ki][1] - ln[ki - 1][1] * ln[ki][0]};
    double s = nx[0] * lt[ki][0] + nx[1] * lt[ki][1] + nx[2] * lt[ki][2];
    if (s < 0.0) s = -1.0;
    if (s > 0.0) s = 1.0;
    double ndn = ln[ki - 1][0] * ln[ki][0] + ln[ki - 1][1] * ln[ki][1] + ln[ki - 1][2] * ln[ki][2];
    if (ndn > 1.0) ndn = 1.0;
    sa = sa + s * acos(ndn);
  }
  F[0] = 1.0 / (4.0 * kPi) * (2.0 * kPi + sa);
  double sb[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  for (int ki = 1; ki <= ne; ++ki) {
    double rr[3] = {lt[ki + 1][0] - lt[ki][0], lt[ki + 1][1] - lt[ki][1], lt[ki + 1][2] - lt[ki][2]};
    double rx[3] = {rr[1] * ln[ki][2] - rr[2] * ln[ki][1], rr[2] * ln[ki][0] - rr[0] * ln[ki][2],
                    rr[0] * ln[ki][1] - rr[1] * ln[ki][0]};
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) sb[3 * a + b] = sb[3 * a + b] + rx[a] * ln[ki][b];
  }
  for (int j = 0; j < 9; ++j) F[1 + j] = sb[j];
  m.ft_ok[cp] = 1;
}

// ---------------------------------------------------------------- half-space
// Images of the collocation points in the free surface x3 = xp, on which the
// complementary kernel's pairs are classified (fbem_bem_staela3d_hsc_sbie_auto,
// bem_staela3d.f90:9074-9075), and c = x_i3 - xp of the points themselves.
__global__ void k_hs_image(const double* cpx, int ncp, double xp, double* img, double* c) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ncp) return;
  img[3 * (size_t)i] = cpx[3 * (size_t)i];
  img[3 * (size_t)i + 1] = cpx[3 * (size_t)i + 1];
  img[3 * (size_t)i + 2] = 2.0 * xp - cpx[3 * (size_t)i + 2];
  c[i] = cpx[3 * (size_t)i + 2] - xp;
}
// Configurations the reference stops on (bem_staela3d.f90:7466-7476,8700-8705):
// bit 0, an element node or collocation point outside the half-space; bit 1,
// an element holding a collocation point of the free surface (a singular pair
// of the complementary kernel) that does not lie on the surface.
__global__ void k_hs_check(DMesh mh, const double* c, double xp, int* err) {
  const long long n1 = 8LL * mh.ne, n2 = n1 + mh.ncp, n3 = n2 + mh.nsing;
  long long id = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (id >= n3) return;
  if (id < n1) {
    if (mh.ex[3 * id + 2] < xp) atomicOr(err, 1);
  } else if (id < n2) {
    if (c[id - n1] < 0.0) atomicOr(err, 1);
  } else {
    const int e = mh.sing_e[id - n2];
    for (int k = 0; k < 8; ++k)
      if (fabs(mh.ex[24 * (size_t)e + 3 * k + 2] - xp) > 1e-12) atomicOr(err, 2);
  }
}

}  // namespace mfb
