// Dense LU with partial pivoting (LAPACK getrf semantics: row interchanges
// recorded in ipiv, unit lower L and upper U overwrite A) and the triangular
// solves of getrs, for a batch of column-major matrices with a common size.
// Replaces the LAPACK calls of src/solve_lse_r.f90:137,189 and
// src/solve_lse_c.f90:124,176.
//
// Right-looking blocked algorithm, panel width NB:
//   panel   column-by-column partial pivoting inside the panel (k_panel_*),
//   laswp   the panel's interchanges applied to the other columns,
//   trsm    U12 = L11^{-1} A12,
//   update  A22 -= L21 U12 (a GEMM; issued by the host layer).
#pragma once
#include <cuda_runtime.h>
#include "dev_complex.cuh"

namespace mfb {

// scalar traits ---------------------------------------------------------------
template <typename S> struct Sc;
template <> struct Sc<double> {
  typedef double R;
  __device__ static double zero() { return 0.0; }
  __device__ static double one() { return 1.0; }
  __device__ static double abs1(double a) { return fabs(a); }
  __device__ static double mul(double a, double b) { return a * b; }
  __device__ static double sub(double a, double b) { return a - b; }
  __device__ static double add(double a, double b) { return a + b; }
  __device__ static double div(double a, double b) { return a / b; }
  __device__ static double rcp(double a) { return 1.0 / a; }
  __device__ static bool iszero(double a) { return a == 0.0; }
};
template <> struct Sc<float> {
  typedef float R;
  __device__ static float zero() { return 0.0f; }
  __device__ static float one() { return 1.0f; }
  __device__ static float abs1(float a) { return fabsf(a); }
  __device__ static float mul(float a, float b) { return a * b; }
  __device__ static float sub(float a, float b) { return a - b; }
  __device__ static float add(float a, float b) { return a + b; }
  __device__ static float div(float a, float b) { return a / b; }
  __device__ static float rcp(float a) { return 1.0f / a; }
  __device__ static bool iszero(float a) { return a == 0.0f; }
};
template <> struct Sc<double2> {
  typedef double R;
  __device__ static double2 zero() { return make_double2(0.0, 0.0); }
  __device__ static double2 one() { return make_double2(1.0, 0.0); }
  // |re| + |im|, the pivot measure of LAPACK's izamax (dcabs1)
  __device__ static double abs1(double2 a) { return fabs(a.x) + fabs(a.y); }
  __device__ static double2 mul(double2 a, double2 b) { return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
  __device__ static double2 sub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
  __device__ static double2 add(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
  __device__ static double2 div(double2 a, double2 b) {
    cd q = mk(a.x, a.y) / mk(b.x, b.y);
    return make_double2(q.re, q.im);
  }
  __device__ static double2 rcp(double2 a) { return div(one(), a); }
  __device__ static bool iszero(double2 a) { return a.x == 0.0 && a.y == 0.0; }
};
template <> struct Sc<float2> {
  typedef float R;
  __device__ static float2 zero() { return make_float2(0.f, 0.f); }
  __device__ static float2 one() { return make_float2(1.f, 0.f); }
  __device__ static float abs1(float2 a) { return fabsf(a.x) + fabsf(a.y); }
  __device__ static float2 mul(float2 a, float2 b) { return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
  __device__ static float2 sub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
  __device__ static float2 add(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
  __device__ static float2 div(float2 a, float2 b) {
    if (fabsf(b.x) >= fabsf(b.y)) {
      float r = b.y / b.x, den = b.x + b.y * r;
      return make_float2((a.x + a.y * r) / den, (a.y - a.x * r) / den);
    }
    float r = b.x / b.y, den = b.y + b.x * r;
    return make_float2((a.x * r + a.y) / den, (a.y * r - a.x) / den);
  }
  __device__ static float2 rcp(float2 a) { return div(one(), a); }
  __device__ static bool iszero(float2 a) { return a.x == 0.f && a.y == 0.f; }
};

// ---------------------------------------------------------------------------
// Panel factorisation, one CTA per matrix (used where the panel's arithmetic
// is cheap relative to synchronisation: FP32 and small FP64 problems).
// A: batch of matrices at A + b*strideA; panel = columns [k, k+nb).
// ipiv (1-based global row indices) at ipiv + b*n; info (first zero pivot).
// ---------------------------------------------------------------------------
template <typename S, int NT>
__global__ void __launch_bounds__(NT) k_panel_cta(S* A, long long strideA, int lda, int n, int k, int nb, int* ipiv,
                                                  int* info) {
  typedef typename Sc<S>::R R;
  const int bidx = blockIdx.x;
  S* M = A + strideA * bidx;
  int* piv = ipiv + (size_t)n * bidx;
  __shared__ R sv[NT / 32];
  __shared__ int si[NT / 32];
  __shared__ int sp;
  __shared__ S prow[128];
  const int lane = threadIdx.x & 31, wid = threadIdx.x / 32;
  const int kend = min(k + nb, n);
  for (int j = k; j < kend; ++j) {
    // argmax |A(i,j)|, i >= j (first index on ties, as i?amax)
    R best = -1;
    int bi = j;
    for (int i = j + threadIdx.x; i < n; i += NT) {
      R v = Sc<S>::abs1(M[(size_t)j * lda + i]);
      if (v > best) { best = v; bi = i; }
    }
    for (int o = 16; o > 0; o >>= 1) {
      R ov = __shfl_xor_sync(0xffffffffu, best, o);
      int oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
    }
    if (lane == 0) { sv[wid] = best; si[wid] = bi; }
    __syncthreads();
    if (threadIdx.x == 0) {
      R b0 = sv[0];
      int i0 = si[0];
      for (int w = 1; w < NT / 32; ++w)
        if (sv[w] > b0 || (sv[w] == b0 && si[w] < i0)) { b0 = sv[w]; i0 = si[w]; }
      sp = i0;
      piv[j] = i0 + 1;
      if (Sc<S>::iszero(M[(size_t)j * lda + i0]) && info[bidx] == 0) info[bidx] = j + 1;
    }
    __syncthreads();
    const int p = sp;
    // swap rows j and p inside the panel and keep the pivot row in shared memory
    for (int c = k + threadIdx.x; c < kend; c += NT) {
      S a = M[(size_t)c * lda + j], bb = M[(size_t)c * lda + p];
      M[(size_t)c * lda + j] = bb;
      M[(size_t)c * lda + p] = a;
      prow[c - k] = bb;
    }
    __syncthreads();
    S dj = prow[j - k];
    if (!Sc<S>::iszero(dj)) {
      S r = Sc<S>::rcp(dj);
      for (int i = j + 1 + threadIdx.x; i < n; i += NT) {
        S l = Sc<S>::mul(M[(size_t)j * lda + i], r);
        M[(size_t)j * lda + i] = l;
        for (int c = j + 1; c < kend; ++c) M[(size_t)c * lda + i] = Sc<S>::sub(M[(size_t)c * lda + i], Sc<S>::mul(l, prow[c - k]));
      }
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// Multi-CTA panel step for one column j (FP64 problems, where a single SM's
// FP64 rate would serialise the panel). Two launches per column:
//   k_pcol_pivot:  one CTA per matrix, pivot search, ipiv, interchange in the panel
//   k_pcol_update: G CTAs per matrix, scale column j and rank-1 update of the
//                  panel columns j+1..k+nb-1 over row chunks
// ---------------------------------------------------------------------------
template <typename S, int NT>
__global__ void __launch_bounds__(NT) k_pcol_pivot(S* A, long long strideA, int lda, int n, int k, int nb, int j,
                                                   int* ipiv, int* info) {
  typedef typename Sc<S>::R R;
  const int bidx = blockIdx.x;
  S* M = A + strideA * bidx;
  __shared__ R sv[NT / 32];
  __shared__ int si[NT / 32];
  __shared__ int sp;
  const int lane = threadIdx.x & 31, wid = threadIdx.x / 32;
  R best = -1;
  int bi = j;
  for (int i = j + threadIdx.x; i < n; i += NT) {
    R v = Sc<S>::abs1(M[(size_t)j * lda + i]);
    if (v > best) { best = v; bi = i; }
  }
  for (int o = 16; o > 0; o >>= 1) {
    R ov = __shfl_xor_sync(0xffffffffu, best, o);
    int oi = __shfl_xor_sync(0xffffffffu, bi, o);
    if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
  }
  if (lane == 0) { sv[wid] = best; si[wid] = bi; }
  __syncthreads();
  if (threadIdx.x == 0) {
    R b0 = sv[0];
    int i0 = si[0];
    for (int w = 1; w < NT / 32; ++w)
      if (sv[w] > b0 || (sv[w] == b0 && si[w] < i0)) { b0 = sv[w]; i0 = si[w]; }
    sp = i0;
    ipiv[(size_t)n * bidx + j] = i0 + 1;
    if (Sc<S>::iszero(M[(size_t)j * lda + i0]) && info[bidx] == 0) info[bidx] = j + 1;
  }
  __syncthreads();
  const int p = sp;
  if (p != j) {
    const int kend = min(k + nb, n);
    for (int c = k + threadIdx.x; c < kend; c += NT) {
      S a = M[(size_t)c * lda + j];
      M[(size_t)c * lda + j] = M[(size_t)c * lda + p];
      M[(size_t)c * lda + p] = a;
    }
  }
}
template <typename S, int NT>
__global__ void __launch_bounds__(NT) k_pcol_update(S* A, long long strideA, int lda, int n, int k, int nb, int j) {
  const int bidx = blockIdx.y;
  S* M = A + strideA * bidx;
  const int kend = min(k + nb, n);
  __shared__ S prow[128];
  for (int c = j + threadIdx.x; c < kend; c += NT) prow[c - j] = M[(size_t)c * lda + j];
  __syncthreads();
  S dj = prow[0];
  if (Sc<S>::iszero(dj)) return;
  S r = Sc<S>::rcp(dj);
  for (int i = j + 1 + blockIdx.x * NT + threadIdx.x; i < n; i += gridDim.x * NT) {
    S l = Sc<S>::mul(M[(size_t)j * lda + i], r);
    M[(size_t)j * lda + i] = l;
    for (int c = j + 1; c < kend; ++c) M[(size_t)c * lda + i] = Sc<S>::sub(M[(size_t)c * lda + i], Sc<S>::mul(l, prow[c - j]));
  }
}

// Apply the panel interchanges (rows k..k+nb-1 with ipiv) to the columns
// outside the panel: one thread per column.
template <typename S>
__global__ void k_laswp(S* A, long long strideA, int lda, int n, int k, int nb, const int* ipiv) {
  const int bidx = blockIdx.y;
  S* M = A + strideA * bidx;
  const int* piv = ipiv + (size_t)n * bidx;
  const int kend = min(k + nb, n);
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  int nout = n - (kend - k);
  if (c >= nout) return;
  int col = c < k ? c : c + (kend - k);
  S* Ac = M + (size_t)col * lda;
  for (int j = k; j < kend; ++j) {
    int p = piv[j] - 1;
    if (p != j) {
      S t = Ac[j];
      Ac[j] = Ac[p];
      Ac[p] = t;
    }
  }
}

// U12 = L11^{-1} A12 (L11 unit lower, nb x nb at (k,k)); one thread per column.
template <typename S>
__global__ void k_trsm_llu(S* A, long long strideA, int lda, int n, int k, int nb) {
  const int bidx = blockIdx.y;
  S* M = A + strideA * bidx;
  const int kend = min(k + nb, n), w = kend - k;
  extern __shared__ unsigned char smraw[];
  S* L = reinterpret_cast<S*>(smraw);  // w x w
  for (int t = threadIdx.x; t < w * w; t += blockDim.x) {
    int i = t % w, jj = t / w;
    L[t] = M[(size_t)(k + jj) * lda + k + i];
  }
  __syncthreads();
  int col = kend + blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= n) return;
  S* Ac = M + (size_t)col * lda + k;
  S x[128];
  for (int i = 0; i < w; ++i) x[i] = Ac[i];
  for (int jj = 0; jj < w; ++jj)
    for (int i = jj + 1; i < w; ++i) x[i] = Sc<S>::sub(x[i], Sc<S>::mul(L[jj * w + i], x[jj]));
  for (int i = 0; i < w; ++i) Ac[i] = x[i];
}

// ---------------------------------------------------------------------------
// getrs (no transpose) for one right-hand side per matrix, blocked by TB rows:
//   k_rhs_swap:     apply all interchanges to b (sequential, one thread per matrix)
//   k_trsv_diag:    solve the TB x TB diagonal block (one CTA per matrix)
//   k_trsv_update:  b[rest] -= A[rest, blk] x[blk] (GEMV, many CTAs)
// ---------------------------------------------------------------------------
template <typename S>
__global__ void k_rhs_swap(S* b, long long strideb, int n, const int* ipiv, int nbatch) {
  int bidx = blockIdx.x * blockDim.x + threadIdx.x;
  if (bidx >= nbatch) return;
  S* x = b + strideb * bidx;
  const int* piv = ipiv + (size_t)n * bidx;
  for (int j = 0; j < n; ++j) {
    int p = piv[j] - 1;
    if (p != j) {
      S t = x[j];
      x[j] = x[p];
      x[p] = t;
    }
  }
}
// lower (unit) forward / upper backward solve of the diagonal block [r0, r0+w)
template <typename S, bool LOWER>
__global__ void k_trsv_diag(const S* A, long long strideA, int lda, S* b, long long strideb, int r0, int w) {
  const int bidx = blockIdx.x;
  const S* M = A + strideA * bidx;
  S* x = b + strideb * bidx;
  __shared__ S xs[256];
  if ((int)threadIdx.x < w) xs[threadIdx.x] = x[r0 + threadIdx.x];
  __syncthreads();
  if (LOWER) {
    for (int j = 0; j < w; ++j) {
      S xj = xs[j];
      int i = threadIdx.x;
      if (i > j && i < w) xs[i] = Sc<S>::sub(xs[i], Sc<S>::mul(M[(size_t)(r0 + j) * lda + r0 + i], xj));
      __syncthreads();
    }
  } else {
    for (int j = w - 1; j >= 0; --j) {
      if (threadIdx.x == 0) xs[j] = Sc<S>::div(xs[j], M[(size_t)(r0 + j) * lda + r0 + j]);
      __syncthreads();
      S xj = xs[j];
      int i = threadIdx.x;
      if (i < j) xs[i] = Sc<S>::sub(xs[i], Sc<S>::mul(M[(size_t)(r0 + j) * lda + r0 + i], xj));
      __syncthreads();
    }
  }
  if ((int)threadIdx.x < w) x[r0 + threadIdx.x] = xs[threadIdx.x];
}
// rows [i0, i1) -= A[rows, r0:r0+w] x[r0:r0+w]
template <typename S>
__global__ void k_trsv_update(const S* A, long long strideA, int lda, S* b, long long strideb, int r0, int w, int i0,
                              int i1) {
  const int bidx = blockIdx.y;
  const S* M = A + strideA * bidx;
  S* x = b + strideb * bidx;
  __shared__ S xs[256];
  if ((int)threadIdx.x < w) xs[threadIdx.x] = x[r0 + threadIdx.x];
  __syncthreads();
  int i = i0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= i1) return;
  S acc = Sc<S>::zero();
  for (int j = 0; j < w; ++j) acc = Sc<S>::add(acc, Sc<S>::mul(M[(size_t)(r0 + j) * lda + i], xs[j]));
  x[i] = Sc<S>::sub(x[i], acc);
}

}  // namespace mfb
