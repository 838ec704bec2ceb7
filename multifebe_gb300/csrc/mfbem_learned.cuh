// Learned quadrature for near-singular (quasi-singular) pairs: a small MLP
// predicts, for a (collocation point, element) pair, the relative integration
// error of each rule of a fixed family -- graded subdivision of depth D
// (D = 0..4) toward the nearest point (each level splits the square holding
// it into four and keeps the other three as leaves: 3D + 1 leaves) with a
// Telles-mapped g x g Gauss rule on every leaf, the leaf rule of sbie_ext_st
// (bem_staela3d.f90:654-969) -- and the cheapest rule whose predicted error
// meets the tolerance replaces the reference's adaptive subdivision
// (sbie_ext_adp, bem_staela3d.f90:973-1096) for that pair; pairs with no such
// rule keep the reference rule. Included into mfbem_abi.cu.
//
// Training data come from the method itself: seeded random quad8 elements and
// points, each candidate rule's h/g blocks compared with a converged rule
// (D = 9, g = 30, checked against D = 9, g = 24). Training, inference and the
// gradients are this file's own kernels (FP32 weights, tanh hidden layers).
#pragma once

namespace mfb {

constexpr int QL_NF = 8;    // features
constexpr int QL_NT = 7;    // reference adaptive rule at qsi_relative_error 1e-3 .. 1e-9
constexpr int QL_NG = 9;    // Gauss orders per level
constexpr int QL_NL = 5;    // graded subdivision depths 0..4
constexpr int QL_DCONV = 9; // depth of the converged rule
constexpr int QL_NC = QL_NT + QL_NL * QL_NG;
constexpr int QL_H = 64;    // hidden width (3 hidden layers)
// candidate c < QL_NT: the reference rule (sbie_ext_adp) at tolerance 10^-(3+c);
// c >= QL_NT: graded depth D = (c - QL_NT) / QL_NG, order c_ql_g[(c - QL_NT) % QL_NG]
__constant__ int c_ql_g[QL_NG] = {3, 4, 6, 8, 10, 12, 16, 20, 30};
static const int h_ql_g[QL_NG] = {3, 4, 6, 8, 10, 12, 16, 20, 30};
// parameter layout: W1[H][NF] b1[H] W2[H][H] b2[H] W3[H][H] b3[H] W4[NC][H] b4[NC]
constexpr int QL_W1 = 0, QL_B1 = QL_W1 + QL_H * QL_NF, QL_W2 = QL_B1 + QL_H, QL_B2 = QL_W2 + QL_H * QL_H,
              QL_W3 = QL_B2 + QL_H, QL_B3 = QL_W3 + QL_H * QL_H, QL_W4 = QL_B3 + QL_H, QL_B4 = QL_W4 + QL_NC * QL_H,
              QL_NW = QL_B4 + QL_NC;

// ---------------------------------------------------------------- features
// Pair features, normalised to O(1): log10 of the nearest-point distance over
// the element size, log10 of the aspect ratio, the nearest point's local
// coordinates, kernel type (0 static, 1 harmonic), wavenumber x element size,
// curvature (mid-side node offset from the corner chords over the size),
// log10 of the element size.
__device__ void ql_features(const double* x, double cl, const double* xi, int kt, double kcl, float f[QL_NF],
                            double* d_out, double bx_out[2]) {
  double bx[2], rmin, d;
  int method;
  nearest_q8(x, cl, xi, bx, &rmin, &d, &method);
  auto dist = [&](int a, int b) {
    double s = 0;
    for (int c = 0; c < 3; ++c) s += (x[3 * a + c] - x[3 * b + c]) * (x[3 * a + c] - x[3 * b + c]);
    return sqrt(s);
  };
  // mid-lines: nodes 8 (-1,0) - 6 (1,0) and 5 (0,-1) - 7 (0,1) (0-based 7-5, 4-6)
  const double l1 = dist(7, 5), l2 = dist(4, 6);
  const double asp = fmax(l1, l2) / fmax(fmin(l1, l2), 1e-300);
  double curv = 0.0;
  for (int k = 0; k < 4; ++k) {
    const int a = k, b = (k + 1) & 3, mnode = 4 + k;
    double s = 0;
    for (int c = 0; c < 3; ++c) {
      const double v = x[3 * mnode + c] - 0.5 * (x[3 * a + c] + x[3 * b + c]);
      s += v * v;
    }
    curv = fmax(curv, sqrt(s) / cl);
  }
  f[0] = (float)(log10(fmax(d, 1e-6)) + 1.5);
  f[1] = (float)(log10(asp) / 0.3);
  f[2] = (float)bx[0];
  f[3] = (float)bx[1];
  f[4] = (float)kt;
  f[5] = (float)(kcl / 0.5);
  f[6] = (float)(curv / 0.2);
  f[7] = (float)log10(cl);
  if (d_out) *d_out = d;
  if (bx_out) { bx_out[0] = bx[0]; bx_out[1] = bx[1]; }
}

// ---------------------------------------------------------------- MLP
__device__ __forceinline__ void ql_forward1(const float* w, const float* f, float* out) {
  float a[QL_H], b[QL_H];
  for (int j = 0; j < QL_H; ++j) {
    float z = w[QL_B1 + j];
    for (int i = 0; i < QL_NF; ++i) z = fmaf(w[QL_W1 + j * QL_NF + i], f[i], z);
    a[j] = tanhf(z);
  }
  for (int j = 0; j < QL_H; ++j) {
    float z = w[QL_B2 + j];
    for (int i = 0; i < QL_H; ++i) z = fmaf(w[QL_W2 + j * QL_H + i], a[i], z);
    b[j] = tanhf(z);
  }
  for (int j = 0; j < QL_H; ++j) {
    float z = w[QL_B3 + j];
    for (int i = 0; i < QL_H; ++i) z = fmaf(w[QL_W3 + j * QL_H + i], b[i], z);
    a[j] = tanhf(z);
  }
  for (int c = 0; c < QL_NC; ++c) {
    float z = w[QL_B4 + c];
    for (int i = 0; i < QL_H; ++i) z = fmaf(w[QL_W4 + c * QL_H + i], a[i], z);
    out[c] = z;
  }
}

// Batched forward (+ backward) on 128 samples per CTA: weights and per-sample
// activations in shared memory ([unit][sample], conflict-free), one thread per
// sample for the layer sums, the weight gradients as block-level products
// summed over the CTA's samples and added atomically. Loss: mean over valid
// samples and outputs of (out - y)^2.
constexpr int QL_BT = 128;
constexpr size_t ql_smem_bytes() {
  return sizeof(float) * ((size_t)QL_NW + 3 * (size_t)QL_H * QL_BT + (size_t)QL_NC * QL_BT + (size_t)QL_NF * QL_BT);
}
template <bool BWD>
__global__ void __launch_bounds__(QL_BT) k_mlp(const float* w, const float* feat, const float* y, const int* valid,
                                               int n, const int* idx, int nb, float inv_count, float* out, float* grad,
                                               float* loss) {
  extern __shared__ __align__(16) float qs[];
  float* W = qs;
  float* A1 = W + QL_NW;
  float* A2 = A1 + QL_H * QL_BT;
  float* A3 = A2 + QL_H * QL_BT;
  float* D4 = A3 + QL_H * QL_BT;
  float* X = D4 + QL_NC * QL_BT;
  const int t = threadIdx.x;
  for (int i = t; i < QL_NW; i += QL_BT) W[i] = w[i];
  const int q = blockIdx.x * QL_BT + t;  // position in the batch
  const bool live = q < nb;
  const int s = live ? (idx ? idx[q] : q) : 0;
  const float vs = (live && (!valid || valid[s])) ? 1.0f : 0.0f;
  for (int i = 0; i < QL_NF; ++i) X[i * QL_BT + t] = live ? feat[(size_t)s * QL_NF + i] : 0.0f;
  __syncthreads();
  // forward
  for (int j = 0; j < QL_H; ++j) {
    float z = W[QL_B1 + j];
    for (int i = 0; i < QL_NF; ++i) z = fmaf(W[QL_W1 + j * QL_NF + i], X[i * QL_BT + t], z);
    A1[j * QL_BT + t] = tanhf(z);
  }
  for (int j = 0; j < QL_H; ++j) {
    float z = W[QL_B2 + j];
    for (int i = 0; i < QL_H; ++i) z = fmaf(W[QL_W2 + j * QL_H + i], A1[i * QL_BT + t], z);
    A2[j * QL_BT + t] = tanhf(z);
  }
  for (int j = 0; j < QL_H; ++j) {
    float z = W[QL_B3 + j];
    for (int i = 0; i < QL_H; ++i) z = fmaf(W[QL_W3 + j * QL_H + i], A2[i * QL_BT + t], z);
    A3[j * QL_BT + t] = tanhf(z);
  }
  float lsum = 0.0f;
  for (int c = 0; c < QL_NC; ++c) {
    float z = W[QL_B4 + c];
    for (int i = 0; i < QL_H; ++i) z = fmaf(W[QL_W4 + c * QL_H + i], A3[i * QL_BT + t], z);
    if (out && live) out[(size_t)q * QL_NC + c] = z;
    float dl = 0.0f;
    if (BWD) {
      const float e = (z - y[(size_t)s * QL_NC + c]) * vs;
      lsum += e * e;
      dl = 2.0f * e * inv_count;
    }
    D4[c * QL_BT + t] = dl;
  }
  if (!BWD) return;
  for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
  if ((t & 31) == 0) atomicAdd(loss, lsum * inv_count);
  __syncthreads();
  // layer 4 gradients, delta3 = W4^T d4 * (1 - a3^2)
  for (int e = t; e < QL_NC * QL_H; e += QL_BT) {
    const int c = e / QL_H, i = e % QL_H;
    float g = 0.0f;
    for (int k = 0; k < QL_BT; ++k) g = fmaf(D4[c * QL_BT + k], A3[i * QL_BT + k], g);
    atomicAdd(grad + QL_W4 + e, g);
  }
  for (int c = t; c < QL_NC; c += QL_BT) {
    float g = 0.0f;
    for (int k = 0; k < QL_BT; ++k) g += D4[c * QL_BT + k];
    atomicAdd(grad + QL_B4 + c, g);
  }
  float d3[QL_H];
  for (int i = 0; i < QL_H; ++i) {
    float g = 0.0f;
    for (int c = 0; c < QL_NC; ++c) g = fmaf(W[QL_W4 + c * QL_H + i], D4[c * QL_BT + t], g);
    const float a = A3[i * QL_BT + t];
    d3[i] = g * (1.0f - a * a);
  }
  __syncthreads();
  for (int i = 0; i < QL_H; ++i) A3[i * QL_BT + t] = d3[i];  // A3 now holds delta3
  __syncthreads();
  // layer 3 gradients from delta3 and a2, then delta2
  for (int e = t; e < QL_H * QL_H; e += QL_BT) {
    const int j = e / QL_H, i = e % QL_H;
    float g = 0.0f;
    for (int k = 0; k < QL_BT; ++k) g = fmaf(A3[j * QL_BT + k], A2[i * QL_BT + k], g);
    atomicAdd(grad + QL_W3 + e, g);
  }
  for (int j = t; j < QL_H; j += QL_BT) {
    float g = 0.0f;
    for (int k = 0; k < QL_BT; ++k) g += A3[j * QL_BT + k];
    atomicAdd(grad + QL_B3 + j, g);
  }
  for (int i = 0; i < QL_H; ++i) {
    float g = 0.0f;
    for (int j = 0; j < QL_H; ++j) g = fmaf(W[QL_W3 + j * QL_H + i], A3[j * QL_BT + t], g);
    const float a = A2[i * QL_BT + t];
    d3[i] = g * (1.0f - a * a);
  }
  __syncthreads();
  for (int i = 0; i < QL_H; ++i) A2[i * QL_BT + t] = d3[i];  // delta2
  __syncthreads();
  for (int e = t; e < QL_H * QL_H; e += QL_BT) {
    const int j = e / QL_H, i = e % QL_H;
    float g = 0.0f;
    for (int k = 0; k < QL_BT; ++k) g = fmaf(A2[j * QL_BT + k], A1[i * QL_BT + k], g);
    atomicAdd(grad + QL_W2 + e, g);
  }
  for (int j = t; j < QL_H; j += QL_BT) {
    float g = 0.0f;
    for (int k = 0; k < QL_BT; ++k) g += A2[j * QL_BT + k];
    atomicAdd(grad + QL_B2 + j, g);
  }
  for (int i = 0; i < QL_H; ++i) {
    float g = 0.0f;
    for (int j = 0; j < QL_H; ++j) g = fmaf(W[QL_W2 + j * QL_H + i], A2[j * QL_BT + t], g);
    const float a = A1[i * QL_BT + t];
    d3[i] = g * (1.0f - a * a);
  }
  __syncthreads();
  for (int i = 0; i < QL_H; ++i) A1[i * QL_BT + t] = d3[i];  // delta1
  __syncthreads();
  for (int e = t; e < QL_H * QL_NF; e += QL_BT) {
    const int j = e / QL_NF, i = e % QL_NF;
    float g = 0.0f;
    for (int k = 0; k < QL_BT; ++k) g = fmaf(A1[j * QL_BT + k], X[i * QL_BT + k], g);
    atomicAdd(grad + QL_W1 + e, g);
  }
  for (int j = t; j < QL_H; j += QL_BT) {
    float g = 0.0f;
    for (int k = 0; k < QL_BT; ++k) g += A1[j * QL_BT + k];
    atomicAdd(grad + QL_B1 + j, g);
  }
}

// Adam (Kingma & Ba, 2015) step t (1-based)
__global__ void k_adam(float* w, const float* g, float* m, float* v, int n, float lr, float b1, float b2, float eps,
                       int t) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.0f - b1) * gi, vi = b2 * v[i] + (1.0f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  const float mh = mi / (1.0f - powf(b1, (float)t)), vh = vi / (1.0f - powf(b2, (float)t));
  w[i] -= lr * mh / (sqrtf(vh) + eps);
}
// mini-batch indices of step `step`: splitmix64 of (seed, step, i)
__device__ __forceinline__ unsigned long long ql_mix(unsigned long long z) {
  z += 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
__global__ void k_ql_batch(int* idx, int nb, int n, unsigned long long seed, int step) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nb) return;
  idx[i] = (int)(ql_mix(seed ^ ql_mix((unsigned long long)step * 1000003ULL + (unsigned long long)i)) % (unsigned long long)n);
}

// ---------------------------------------------------------------- rule evaluation
// Leaf (sub-square xs, Telles maps toward the nearest point of the sub-element)
// in the layout of the adaptive leaves (LEAF_D doubles)
__device__ void ql_leaf(const double* x, const double xs[8], const double* xi, double* L) {
  double xsub[24], bx[2], rmin, d;
  int method;
  subdiv_q8(x, xs, xsub);
  const double cl = clen_q8(xsub, 1e-12);
  nearest_q8(xsub, cl, xi, bx, &rmin, &d, &method);
  const double barr = telles_barr(d);
  const Telles t1 = telles11(bx[0], barr), t2 = telles11(bx[1], barr);
  for (int j = 0; j < 8; ++j) L[j] = xs[j];
  L[8] = t1.a; L[9] = t1.b; L[10] = t1.c; L[11] = t1.d;
  L[12] = t2.a; L[13] = t2.b; L[14] = t2.c; L[15] = t2.d;
}
// Sub-square j (of 3D + 1) of the graded subdivision of depth D toward the
// local point bx: level l splits the current square (side 2^(1-l)) into its
// four quadrants; the quadrant holding bx is split again, the other three are
// leaves j = 3l .. 3l + 2 (quadrants in SUBQUAD order); the last square is
// leaf 3D. Corners in the order of the root square.
__device__ void ql_graded(int D, int j, const double bx[2], double xs[8]) {
  double u0 = -1.0, v0 = -1.0, h = 2.0;
  const double b0 = fmin(1.0, fmax(-1.0, bx[0])), b1 = fmin(1.0, fmax(-1.0, bx[1]));
  for (int l = 0; l < D; ++l) {
    const double hh = 0.5 * h;
    const int qa = b0 < u0 + hh ? 0 : 1, qb = b1 < v0 + hh ? 0 : 1;
    const int keep = qb * 2 + qa;  // quadrant holding bx
    if (j >= 3 * l && j < 3 * l + 3) {
      int k = j - 3 * l, q = 0;
      for (int c = 0; c < 4; ++c)
        if (c != keep) {
          if (k == 0) { q = c; break; }
          --k;
        }
      const double a = u0 + (q & 1) * hh, b = v0 + (q >> 1) * hh;
      xs[0] = a; xs[1] = b; xs[2] = a + hh; xs[3] = b; xs[4] = a + hh; xs[5] = b + hh; xs[6] = a; xs[7] = b + hh;
      return;
    }
    u0 += qa * hh;
    v0 += qb * hh;
    h = hh;
  }
  xs[0] = u0; xs[1] = v0; xs[2] = u0 + h; xs[3] = v0; xs[4] = u0 + h; xs[5] = v0 + h; xs[6] = u0; xs[7] = v0 + h;
}
__host__ __device__ constexpr int ql_nleaf(int D) { return 3 * D + 1; }

// geometry of point k (of g x g) of a leaf: x - x_i, unit normal, phi J w
__device__ void ql_point(const double* x, const double* L, int g, int k, const double* xi, double rv[3], double n[3],
                         double w[8]) {
  const int k1 = k / g + 1, k2 = k % g + 1;
  const Telles t1{L[8], L[9], L[10], L[11]}, t2{L[12], L[13], L[14], L[15]};
  double xp1, jt1, xp2, jt2;
  telles_map(t1, gl11x(k1, g), xp1, jt1);
  telles_map(t2, gl11x(k2, g), xp2, jt2);
  double sp[4], sd1[4], sd2[4];
  phi_q4(xp1, xp2, sp);
  dphi_q4(xp1, xp2, sd1, sd2);
  double xa = 0, xb = 0, a11 = 0, a12 = 0, a21 = 0, a22 = 0;
  for (int q = 0; q < 4; ++q) {
    xa += sp[q] * L[2 * q];
    xb += sp[q] * L[2 * q + 1];
    a11 += sd1[q] * L[2 * q];
    a12 += sd1[q] * L[2 * q + 1];
    a21 += sd2[q] * L[2 * q];
    a22 += sd2[q] * L[2 * q + 1];
  }
  const double js = a11 * a22 - a12 * a21;
  double xq[3], T1[3], T2[3], phi[8], N[3];
  geom_q8(x, xa, xb, xq, T1, T2, phi);
  cross3(T1, T2, N);
  const double jg = norm3(N);
  for (int c = 0; c < 3; ++c) {
    n[c] = N[c] / jg;
    rv[c] = xq[c] - xi[c];
  }
  const double jw = jg * js * jt1 * jt2 * gl11w(k1, g) * gl11w(k2, g);
  for (int q = 0; q < 8; ++q) w[q] = phi[q] * jw;
}

// Warp-cooperative integration of the full h(kn,il,ik), g(kn,il,ik) blocks
// (72 + 72 values, without the kernels' constant factors) over nleaf leaves
// with per-leaf orders gl[] (prefix sums of the point counts in pref[]).
// Lane l returns outputs o = l + 32 j (j < 5, o < 144) in acc[j].
template <typename T>
struct QlCombo {
  T fu[9], ft[9];
  double w[8];
};
template <class KER, typename T>
__device__ void ql_integrate(const KER& ker, const double* x, const double* xi, const double* leaves, const int* gl,
                             const int* pref, int nleaf, QlCombo<T>* S, T acc[5]) {
  const int lane = threadIdx.x & 31;
  for (int j = 0; j < 5; ++j) acc[j] = VT<T>::zero();
  const int total = pref[nleaf];
  for (int base = 0; base < total; base += 32) {
    const int p = base + lane;
    if (p < total) {
      int lf = 0;
      while (lf + 1 < nleaf && pref[lf + 1] <= p) ++lf;
      double rv[3], n[3];
      ql_point(x, leaves + (size_t)lf * LEAF_D, gl[lf], p - pref[lf], xi, rv, n, S[lane].w);
      ker.point(rv, n, S[lane].fu, S[lane].ft);
    }
    __syncwarp();
    const int nt = min(32, total - base);
    for (int t = 0; t < nt; ++t) {
#pragma unroll
      for (int j = 0; j < 5; ++j) {
        const int o = lane + 32 * j;
        if (o < 144) {
          const int oo = o < 72 ? o : o - 72, kn = oo / 9, c = oo % 9;
          acc[j] = acc[j] + (o < 72 ? S[t].ft[c] : S[t].fu[c]) * S[t].w[kn];
        }
      }
    }
    __syncwarp();
  }
}
struct QlStatic {
  StaelaP k;
  __device__ void point(const double rv[3], const double n[3], double fu[9], double ft[9]) const {
    staela_point(k, rv, n, fu, ft);
  }
};
struct QlHarmonic {
  const HarParD* p;
  __device__ void point(const double rv[3], const double n[3], cd fu[9], cd ft[9]) const {
    harela_point(*p, rv, n, fu, ft);
  }
};
__device__ __forceinline__ double qabs2(double v) { return v * v; }
__device__ __forceinline__ double qabs2(cd v) { return v.re * v.re + v.im * v.im; }

// max over the h and g blocks of the relative Frobenius distance of acc to ref
template <typename T>
__device__ double ql_relerr(const T acc[5], const T ref[5]) {
  const int lane = threadIdx.x & 31;
  double dh = 0, nh = 0, dg = 0, ng = 0;
  for (int j = 0; j < 5; ++j) {
    const int o = lane + 32 * j;
    if (o >= 144) break;
    const double dd = qabs2(acc[j] - ref[j]), rr = qabs2(ref[j]);
    if (o < 72) { dh += dd; nh += rr; }
    else { dg += dd; ng += rr; }
  }
  for (int o = 16; o > 0; o >>= 1) {
    dh += __shfl_xor_sync(0xffffffffu, dh, o);
    nh += __shfl_xor_sync(0xffffffffu, nh, o);
    dg += __shfl_xor_sync(0xffffffffu, dg, o);
    ng += __shfl_xor_sync(0xffffffffu, ng, o);
  }
  return fmax(sqrt(dh / fmax(nh, 1e-300)), sqrt(dg / fmax(ng, 1e-300)));
}

// Labels of random pairs, one warp per sample (WPB warps per CTA): features,
// and for every candidate rule its log10 relative error against the converged
// rule and its quadrature point count (reference-rule candidates beyond
// QL_MAXREF leaves get error 10 and cost -1).
constexpr int QL_MAXREF = 128;  // adaptive leaves kept for a reference-rule candidate
template <int WPB, bool HARM>
__global__ void __launch_bounds__(WPB * 32) k_ql_label(int n, const double* ex, const double* pts, const double* cl,
                                                       const int* gln_far, const double* kcl, const HarParD* par,
                                                       const QsCurves* qsc, int ns_max, double* scratch, float* feat,
                                                       float* logerr, int* cost, int* valid) {
  typedef typename std::conditional<HARM, cd, double>::type T;
  __shared__ QlCombo<T> S[WPB][32];
  __shared__ double LV[WPB][64 * LEAF_D];
  __shared__ int GL[WPB][QL_MAXREF], PF[WPB][QL_MAXREF + 1];
  const int lane = threadIdx.x & 31, w = threadIdx.x / 32;
  const int s = blockIdx.x * WPB + w;
  if (s >= n) return;
  const double* x = ex + 24 * (size_t)s;
  const double* xi = pts + 3 * (size_t)s;
  typename std::conditional<HARM, QlHarmonic, QlStatic>::type ker;
  if constexpr (HARM) ker.p = par + s;
  else ker.k = staela_params(1.0, 0.3);
  double bx[2] = {0.0, 0.0};
  if (lane == 0) {
    float f[QL_NF];
    ql_features(x, cl[s], xi, HARM ? 1 : 0, HARM ? kcl[s] : 0.0, f, nullptr, bx);
    for (int i = 0; i < QL_NF; ++i) feat[(size_t)s * QL_NF + i] = f[i];
  }
  bx[0] = __shfl_sync(0xffffffffu, bx[0], 0);
  bx[1] = __shfl_sync(0xffffffffu, bx[1], 0);
  // converged rule: graded depth QL_DCONV, g = 30, checked against g = 24
  const int ncv = ql_nleaf(QL_DCONV);
  for (int j = lane; j < ncv; j += 32) {
    double xs[8];
    ql_graded(QL_DCONV, j, bx, xs);
    ql_leaf(x, xs, xi, &LV[w][j * LEAF_D]);
  }
  T ref[5], acc[5];
  for (int pass = 0; pass < 2; ++pass) {
    const int g = pass == 0 ? 30 : 24;
    if (lane == 0) {
      PF[w][0] = 0;
      for (int j = 0; j < ncv; ++j) { GL[w][j] = g; PF[w][j + 1] = PF[w][j] + g * g; }
    }
    __syncwarp();
    ql_integrate(ker, x, xi, LV[w], GL[w], PF[w], ncv, S[w], pass == 0 ? ref : acc);
    __syncwarp();
  }
  const double cerr = ql_relerr(acc, ref);
  if (lane == 0) valid[s] = cerr < 1e-10 ? 1 : 0;
  // errors below the converged rule's own accuracy are not resolved: clamp at 1e-10
  auto put = [&](int c, double e, int pts_) {
    if (lane == 0) {
      logerr[(size_t)s * QL_NC + c] = (float)fmin(1.0, log10(fmax(e, 1e-10)));
      cost[(size_t)s * QL_NC + c] = pts_;
    }
  };
  // candidates 0 .. QL_NT-1: the reference adaptive rule at 1e-3 .. 1e-9
  DMesh fm;
  memset(&fm, 0, sizeof(fm));
  fm.ex = ex;
  fm.cl = cl;
  fm.gln_far = gln_far;
  fm.ns_max = ns_max;
  fm.fcls = fm.fadp = 5;  // SBIE kernels: the 1/r^5 estimate
  double* lbuf = scratch + (size_t)s * QL_MAXREF * LEAF_D;
  for (int r = 0; r < QL_NT; ++r) {
    int cnt = 0;
    __syncwarp();
    if (lane == 0) {
      cnt = adp_traverse<false>(fm, qsc[r], s, xi, nullptr, nullptr, nullptr, 0);
      if (cnt <= QL_MAXREF) {
        int pr[QL_MAXREF];
        adp_traverse<true>(fm, qsc[r], s, xi, lbuf, GL[w], pr, 0);
        PF[w][0] = 0;
        for (int j = 0; j < cnt; ++j) PF[w][j + 1] = PF[w][j] + GL[w][j] * GL[w][j];
      }
    }
    cnt = __shfl_sync(0xffffffffu, cnt, 0);
    __syncwarp();
    if (cnt <= QL_MAXREF) {
      ql_integrate(ker, x, xi, lbuf, GL[w], PF[w], cnt, S[w], acc);
      put(r, ql_relerr(acc, ref), PF[w][cnt]);
    } else {
      put(r, 10.0, -1);
    }
  }
  // candidates QL_NT ..: graded rules
  for (int lev = 0; lev < QL_NL; ++lev) {
    const int nl = ql_nleaf(lev);
    __syncwarp();
    for (int j = lane; j < nl; j += 32) {
      double xs[8];
      ql_graded(lev, j, bx, xs);
      ql_leaf(x, xs, xi, &LV[w][j * LEAF_D]);
    }
    for (int gi = 0; gi < QL_NG; ++gi) {
      const int g = c_ql_g[gi];
      if (lane == 0) {
        PF[w][0] = 0;
        for (int j = 0; j < nl; ++j) { GL[w][j] = g; PF[w][j + 1] = PF[w][j] + g * g; }
      }
      __syncwarp();
      ql_integrate(ker, x, xi, LV[w], GL[w], PF[w], nl, S[w], acc);
      put(QL_NT + lev * QL_NG + gi, ql_relerr(acc, ref), nl * g * g);
      __syncwarp();
    }
  }
}

// ---------------------------------------------------------------- mesh leaves
// Rule choice of every adaptive pair of a mesh: the cheapest candidate whose
// predicted log10 error is <= log10_tol (reference-rule candidates costed by
// their exact point count), else -1 (the mesh's own reference rule); leaf
// count of the choice. qt: the QL_NT tolerance curves of the reference-rule candidates.
__global__ void k_ql_choose(DMesh m, const QsCurves* qsc, const QsCurves* qt, const float* w, float log10_tol, int kt,
                            double kcl, int* choice, int* nleaf) {
  const long long a = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (a >= m.nadp) return;
  const int e = m.adp_e[a], cp = m.adp_cp[a];
  const double* x = m.ex + 24 * (size_t)e;
  const double* xi = m.cpx + 3 * (size_t)cp;
  float f[QL_NF], o[QL_NC];
  ql_features(x, m.cl[e], xi, kt, kcl, f, nullptr, nullptr);
  ql_forward1(w, f, o);
  int best = -1;
  long long bcost = 0;
  int bleaf = 0;
  for (int c = 0; c < QL_NC; ++c) {
    if (o[c] > log10_tol) continue;
    long long cost;
    int nl;
    if (c < QL_NT) {
      cost = 0;
      nl = adp_traverse<false>(m, qt[c], e, xi, nullptr, nullptr, nullptr, 0, &cost);
    } else {
      const int lev = (c - QL_NT) / QL_NG, g = c_ql_g[(c - QL_NT) % QL_NG];
      nl = ql_nleaf(lev);
      cost = (long long)nl * g * g;
    }
    if (best < 0 || cost < bcost) { best = c; bcost = cost; bleaf = nl; }
  }
  choice[a] = best;
  nleaf[a] = best >= 0 ? bleaf : adp_traverse<false>(m, *qsc, e, xi, nullptr, nullptr, nullptr, 0);
}
__global__ void k_ql_fill(DMesh m, const QsCurves* qsc, const QsCurves* qt, const int* choice) {
  const long long a = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (a >= m.nadp) return;
  const int e = m.adp_e[a], cp = m.adp_cp[a];
  const double* x = m.ex + 24 * (size_t)e;
  const double* xi = m.cpx + 3 * (size_t)cp;
  const int l0 = m.adp_leaf[a];
  const int c = choice[a];
  if (c < QL_NT) {
    adp_traverse<true>(m, c < 0 ? *qsc : qt[c], e, xi, m.leaf + (size_t)l0 * LEAF_D, m.leaf_gln + l0,
                       m.leaf_pair + l0, (int)a);
    return;
  }
  const int lev = (c - QL_NT) / QL_NG, g = c_ql_g[(c - QL_NT) % QL_NG], nl = ql_nleaf(lev);
  float f[QL_NF];
  double bx[2];
  ql_features(x, m.cl[e], xi, 0, 0.0, f, nullptr, bx);
  for (int j = 0; j < nl; ++j) {
    double xs[8];
    ql_graded(lev, j, bx, xs);
    ql_leaf(x, xs, xi, m.leaf + (size_t)(l0 + j) * LEAF_D);
    m.leaf_gln[l0 + j] = g;
    m.leaf_pair[l0 + j] = (int)a;
  }
}

}  // namespace mfb
