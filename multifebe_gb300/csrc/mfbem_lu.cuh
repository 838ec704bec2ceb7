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
#include <cooperative_groups.h>

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
  __device__ static double conj(double a) { return a; }
  __device__ static double from(double v) { return v; }
  __device__ static double re(double a) { return a; }
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
  __device__ static float conj(float a) { return a; }
  __device__ static float from(double v) { return (float)v; }
  __device__ static float re(float a) { return a; }
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
  __device__ static double2 conj(double2 a) { return make_double2(a.x, -a.y); }
  __device__ static double2 from(double v) { return make_double2(v, 0.0); }
  __device__ static double re(double2 a) { return a.x; }
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
  __device__ static float2 conj(float2 a) { return make_float2(a.x, -a.y); }
  __device__ static float2 from(double v) { return make_float2((float)v, 0.f); }
  __device__ static float re(float2 a) { return a.x; }
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

// ---------------------------------------------------------------------------
// Cooperative panel factorisation: the panel columns [k, k+kb) of each matrix
// are split by rows over G CTAs (row chunk of `chunk` rows each) and held in
// shared memory for the whole panel; per column one barrier among the matrix's
// G CTAs exchanges the chunk-local pivot candidates. Launched with
// cudaLaunchCooperativeKernel, so all CTAs are co-resident; every barrier wait
// is bounded (about a second), after which the kernel sets *err and returns.
//
// Per column j (global row/column jj = k + j):
//   every CTA   argmax |A(i,jj)| (LAPACK's |re|+|im| for complex) over its rows
//               i >= jj, publishes (value, row, the row's kb panel values); the
//               owner of row jj publishes that row too (slot jj % 2)
//   barrier
//   every CTA   picks the winner (largest value, smallest row on ties), swaps
//               the two rows inside its chunk where it owns them, then scales
//               column jj below the diagonal and updates columns jj+1.. of its rows
// Counters ctr[matrix] count barrier arrivals over the whole factorisation
// (zeroed once per getrf), so the target of column jj is (jj + 1) * G.
// ---------------------------------------------------------------------------
constexpr long long kCoopSpin = 1LL << 24;

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

template <typename S, int NT>
__global__ void __launch_bounds__(NT) k_panel_coop(S* A, long long strideA, int lda, int n, int k, int kb, int G,
                                                   int chunk, int b0, int* ipiv, int* info, unsigned* ctr, S* xrow,
                                                   typename Sc<S>::R* xval, int* xidx, int* err, long long spin) {
  typedef typename Sc<S>::R R;
  extern __shared__ __align__(16) unsigned char smraw[];
  S* pan = reinterpret_cast<S*>(smraw);  // [kb][chunk]
  S* prow = pan + (size_t)kb * chunk;     // [kb] pivot row
  __shared__ R sv[NT / 32];
  __shared__ int si[NT / 32], sg[NT / 32];
  __shared__ int s_ok, s_p, s_g;
  const int mat = b0 + blockIdx.x / G, g = blockIdx.x % G;
  const int lane = threadIdx.x & 31, wid = threadIdx.x / 32;
  S* M = A + strideA * mat;
  int* piv = ipiv + (size_t)n * mat;
  const int r0 = k + g * chunk, r1 = min(n, r0 + chunk), nr = max(0, r1 - r0);
  // exchange slots of this matrix: [2][G][kb] rows, [2][G] values / indices, then
  // [2][kb] for the current diagonal row (stored at candidate index G)
  S* XR = xrow + (size_t)(mat) * 2 * (G + 1) * kb;
  R* XV = xval + (size_t)(mat) * 2 * G;
  int* XI = xidx + (size_t)(mat) * 2 * G;
  for (int t = threadIdx.x; t < kb * nr; t += NT) {
    const int c = t / nr, i = t - c * nr;
    pan[(size_t)c * chunk + i] = M[(size_t)(k + c) * lda + r0 + i];
  }
  __syncthreads();
  for (int j = 0; j < kb; ++j) {
    const int jj = k + j, slot = jj & 1;
    // chunk-local candidate
    R best = -1;
    int bi = -1;
    for (int i = max(jj, r0) - r0 + threadIdx.x; i < nr; i += NT) {
      const R v = Sc<S>::abs1(pan[(size_t)j * chunk + i]);
      if (v > best) { best = v; bi = r0 + i; }
    }
    for (int o = 16; o > 0; o >>= 1) {
      const R ov = __shfl_xor_sync(0xffffffffu, best, o);
      const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (ov > best || (ov == best && oi >= 0 && (bi < 0 || oi < bi))) { best = ov; bi = oi; }
    }
    if (lane == 0) { sv[wid] = best; si[wid] = bi; }
    __syncthreads();
    if (threadIdx.x == 0) {
      R b_ = sv[0];
      int i_ = si[0];
      for (int w = 1; w < NT / 32; ++w)
        if (sv[w] > b_ || (sv[w] == b_ && si[w] >= 0 && (i_ < 0 || si[w] < i_))) { b_ = sv[w]; i_ = si[w]; }
      XV[slot * G + g] = b_;
      XI[slot * G + g] = i_;
      s_p = i_;
    }
    __syncthreads();
    const int myc = s_p;
    if (myc >= 0 && (int)threadIdx.x < kb)
      XR[((size_t)slot * (G + 1) + g) * kb + threadIdx.x] = pan[(size_t)threadIdx.x * chunk + (myc - r0)];
    if (jj >= r0 && jj < r1 && (int)threadIdx.x < kb)
      XR[((size_t)slot * (G + 1) + G) * kb + threadIdx.x] = pan[(size_t)threadIdx.x * chunk + (jj - r0)];
    // barrier among the G CTAs of this matrix
    __syncthreads();
    if (threadIdx.x == 0) {
      __threadfence();
      atomicAdd(ctr + mat, 1u);
      const unsigned target = (unsigned)(jj + 1) * (unsigned)G;
      long long it = 0;
      int ok = 1;
      const long long lim = spin > 0 ? spin : kCoopSpin;
      while (ld_acquire_u32(ctr + mat) < target) {
        if (++it > lim) { ok = 0; atomicExch(err, 1); break; }
        __nanosleep(32);
      }
      __threadfence();
      s_ok = ok;
    }
    __syncthreads();
    if (!s_ok) return;
    // winner over the G candidates (parallel loads, block argmax)
    {
      R b_ = -1;
      int i_ = -1, g_ = 0;
      for (int q = threadIdx.x; q < G; q += NT) {
        const R v = __ldcg(XV + slot * G + q);
        const int ix = __ldcg(XI + slot * G + q);
        if (ix >= 0 && (v > b_ || (v == b_ && ix < i_))) { b_ = v; i_ = ix; g_ = q; }
      }
      for (int o = 16; o > 0; o >>= 1) {
        const R ov = __shfl_xor_sync(0xffffffffu, b_, o);
        const int oi = __shfl_xor_sync(0xffffffffu, i_, o);
        const int og = __shfl_xor_sync(0xffffffffu, g_, o);
        if (oi >= 0 && (ov > b_ || (ov == b_ && (i_ < 0 || oi < i_)))) { b_ = ov; i_ = oi; g_ = og; }
      }
      if (lane == 0) { sv[wid] = b_; si[wid] = i_; sg[wid] = g_; }
      __syncthreads();
      if (threadIdx.x == 0) {
        R bb = sv[0];
        int ii = si[0], gg = sg[0];
        for (int w = 1; w < NT / 32; ++w)
          if (si[w] >= 0 && (sv[w] > bb || (sv[w] == bb && (ii < 0 || si[w] < ii)))) { bb = sv[w]; ii = si[w]; gg = sg[w]; }
        s_p = ii;
        s_g = gg;
      }
      __syncthreads();
    }
    const int p = s_p;
    if ((int)threadIdx.x < kb)
      prow[threadIdx.x] = __ldcg(XR + ((size_t)slot * (G + 1) + s_g) * kb + threadIdx.x);
    __syncthreads();
    if (g == 0 && threadIdx.x == 0) {
      piv[jj] = p + 1;
      if (Sc<S>::iszero(prow[j]) && info[mat] == 0) info[mat] = jj + 1;
    }
    if (p != jj) {
      // row p <- old row jj, row jj <- pivot row, where this CTA owns them
      if (p >= r0 && p < r1 && (int)threadIdx.x < kb)
        pan[(size_t)threadIdx.x * chunk + (p - r0)] = __ldcg(XR + ((size_t)slot * (G + 1) + G) * kb + threadIdx.x);
      if (jj >= r0 && jj < r1 && (int)threadIdx.x < kb) pan[(size_t)threadIdx.x * chunk + (jj - r0)] = prow[threadIdx.x];
    }
    __syncthreads();
    const S dj = prow[j];
    if (!Sc<S>::iszero(dj)) {
      const S rcp = Sc<S>::rcp(dj);
      for (int i = max(jj + 1, r0) - r0 + threadIdx.x; i < nr; i += NT) {
        const S l = Sc<S>::mul(pan[(size_t)j * chunk + i], rcp);
        pan[(size_t)j * chunk + i] = l;
        for (int c = j + 1; c < kb; ++c)
          pan[(size_t)c * chunk + i] = Sc<S>::sub(pan[(size_t)c * chunk + i], Sc<S>::mul(l, prow[c]));
      }
    }
    __syncthreads();
  }
  for (int t = threadIdx.x; t < kb * nr; t += NT) {
    const int c = t / nr, i = t - c * nr;
    M[(size_t)(k + c) * lda + r0 + i] = pan[(size_t)c * chunk + i];
  }
}

// ---------------------------------------------------------------------------
// Cluster panel: the same algorithm as k_panel_coop with the G CTAs of a
// matrix forming one thread-block cluster (cluster rank = row chunk): the
// per-column exchange goes through distributed shared memory and the
// hardware cluster barrier instead of global memory and a spin on a counter.
// Candidate slots are double-buffered by column parity, so one cluster
// barrier per column suffices: a slot written at column j + 2 is read by
// everyone before the barrier of column j + 1.
// ---------------------------------------------------------------------------
template <typename S, int NT>
__global__ void __launch_bounds__(NT) k_panel_cluster(S* A, long long strideA, int lda, int n, int k, int kb,
                                                      int chunk, int* ipiv, int* info) {
  namespace cg = cooperative_groups;
  typedef typename Sc<S>::R R;
  cg::cluster_group cl = cg::this_cluster();
  const int G = (int)cl.num_blocks(), g = (int)cl.block_rank();
  extern __shared__ __align__(16) unsigned char smraw[];
  S* pan = reinterpret_cast<S*>(smraw);  // [kb][chunk]
  S* prow = pan + (size_t)kb * chunk;     // [kb] pivot row
  S* xrow = prow + 32;                    // [2][2][32]: slot parity x {candidate row, row jj}
  R* xval = reinterpret_cast<R*>(xrow + 2 * 2 * 32);  // [2]
  int* xidx = reinterpret_cast<int*>(xval + 2);        // [2]
  __shared__ R sv[NT / 32];
  __shared__ int si[NT / 32];
  __shared__ int s_p;
  const int mat = blockIdx.x / G;
  const int lane = threadIdx.x & 31, wid = threadIdx.x / 32;
  S* M = A + strideA * mat;
  int* piv = ipiv + (size_t)n * mat;
  const int r0 = k + g * chunk, r1 = min(n, r0 + chunk), nr = max(0, r1 - r0);
  for (int t = threadIdx.x; t < kb * nr; t += NT) {
    const int c = t / nr, i = t - c * nr;
    pan[(size_t)c * chunk + i] = M[(size_t)(k + c) * lda + r0 + i];
  }
  __syncthreads();
  for (int j = 0; j < kb; ++j) {
    const int jj = k + j, slot = j & 1;
    R best = -1;
    int bi = -1;
    for (int i = max(jj, r0) - r0 + threadIdx.x; i < nr; i += NT) {
      const R v = Sc<S>::abs1(pan[(size_t)j * chunk + i]);
      if (v > best) { best = v; bi = r0 + i; }
    }
    for (int o = 16; o > 0; o >>= 1) {
      const R ov = __shfl_xor_sync(0xffffffffu, best, o);
      const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (ov > best || (ov == best && oi >= 0 && (bi < 0 || oi < bi))) { best = ov; bi = oi; }
    }
    if (lane == 0) { sv[wid] = best; si[wid] = bi; }
    __syncthreads();
    // the CTA's candidate: warp 0 reduces the warps' (larger |a|, then the
    // smaller row; no row = -1 loses), then stages it and row jj
    if (wid == 0) {
      R v = lane < NT / 32 ? sv[lane] : (R)-1;
      int ix = lane < NT / 32 ? si[lane] : -1;
      for (int o = 16; o > 0; o >>= 1) {
        const R ov = __shfl_xor_sync(0xffffffffu, v, o);
        const int oi = __shfl_xor_sync(0xffffffffu, ix, o);
        if (oi >= 0 && (ix < 0 || ov > v || (ov == v && oi < ix))) { v = ov; ix = oi; }
      }
      if (lane == 0) {
        xval[slot] = v;
        xidx[slot] = ix;
      }
      if (lane < kb) {
        if (ix >= 0) xrow[(slot * 2 + 0) * 32 + lane] = pan[(size_t)lane * chunk + (ix - r0)];
        if (jj >= r0 && jj < r1) xrow[(slot * 2 + 1) * 32 + lane] = pan[(size_t)lane * chunk + (jj - r0)];
      }
    }
    cl.sync();
    // winner over the cluster's candidates: warp 0 reads the G ranks' slots of
    // distributed shared memory in parallel (one lane each), reduces with the
    // same order, fetches the pivot row and interchanges rows p and jj
    if (wid == 0) {
      R v = (R)-1;
      int ix = -1, gq = lane;
      if (lane < G) {
        v = cl.map_shared_rank(xval, lane)[slot];
        ix = cl.map_shared_rank(xidx, lane)[slot];
      }
      for (int o = 16; o > 0; o >>= 1) {
        const R ov = __shfl_xor_sync(0xffffffffu, v, o);
        const int oi = __shfl_xor_sync(0xffffffffu, ix, o);
        const int og = __shfl_xor_sync(0xffffffffu, gq, o);
        if (oi >= 0 && (ix < 0 || ov > v || (ov == v && oi < ix))) { v = ov; ix = oi; gq = og; }
      }
      const int own = (jj - k) / chunk;  // rank owning row jj
      if (lane < kb) {
        const S pr = cl.map_shared_rank(xrow, gq)[(slot * 2 + 0) * 32 + lane];
        prow[lane] = pr;
        if (ix != jj) {
          if (ix >= r0 && ix < r1)
            pan[(size_t)lane * chunk + (ix - r0)] = cl.map_shared_rank(xrow, own)[(slot * 2 + 1) * 32 + lane];
          if (jj >= r0 && jj < r1) pan[(size_t)lane * chunk + (jj - r0)] = pr;
        }
      }
      if (lane == 0) s_p = ix;
    }
    __syncthreads();
    const int p = s_p;
    if (g == 0 && threadIdx.x == 0) {
      piv[jj] = p + 1;
      if (Sc<S>::iszero(prow[j]) && info[mat] == 0) info[mat] = jj + 1;
    }
    const S dj = prow[j];
    if (!Sc<S>::iszero(dj)) {
      const S rcp = Sc<S>::rcp(dj);
      for (int i = max(jj + 1, r0) - r0 + threadIdx.x; i < nr; i += NT) {
        const S l = Sc<S>::mul(pan[(size_t)j * chunk + i], rcp);
        pan[(size_t)j * chunk + i] = l;
        for (int c = j + 1; c < kb; ++c)
          pan[(size_t)c * chunk + i] = Sc<S>::sub(pan[(size_t)c * chunk + i], Sc<S>::mul(l, prow[c]));
      }
    }
    __syncthreads();
  }
  for (int t = threadIdx.x; t < kb * nr; t += NT) {
    const int c = t / nr, i = t - c * nr;
    M[(size_t)(k + c) * lda + r0 + i] = pan[(size_t)c * chunk + i];
  }
  // no CTA may exit while others can still read its shared memory
  cl.sync();
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

// U12 = L11^{-1} A12 for the columns [c0, c1) (L11 unit lower, w x w at (k,k),
// w <= 32). A CTA of trsm_cols<S>() threads stages a 32-row tile of as many
// columns (coalesced along each column), thread t solves column t in shared
// memory, and the tile is written back.
template <typename S> __host__ __device__ constexpr int trsm_cols() { return sizeof(S) > 8 ? 32 : 64; }
template <typename S>
__global__ void __launch_bounds__(trsm_cols<S>()) k_trsm_cols(S* A, long long strideA, int lda, int k, int w, int c0,
                                                              int c1) {
  constexpr int NC = trsm_cols<S>();
  const int bidx = blockIdx.y;
  S* M = A + strideA * bidx;
  __shared__ S L[32 * 32];
  __shared__ S T[NC * 33];  // [column][row], padded
  const int cb = c0 + blockIdx.x * NC;
  const int ncol = min(NC, c1 - cb);
  for (int t = threadIdx.x; t < w * w; t += NC) {
    const int i = t % w, jj = t / w;
    L[t] = M[(size_t)(k + jj) * lda + k + i];
  }
  // the 32 rows of one column are contiguous
  for (int t = threadIdx.x; t < 32 * ncol; t += NC) {
    const int i = t & 31, c = t >> 5;
    if (i < w) T[c * 33 + i] = M[(size_t)(cb + c) * lda + k + i];
  }
  __syncthreads();
  const int c = threadIdx.x;
  if (c < ncol) {
    S* x = T + c * 33;
    if (w == 32) {
      // full panel width: the column in registers, the substitution unrolled
      // (L read from shared memory as a broadcast, no read-modify-write of x)
      S xr[32];
#pragma unroll
      for (int i = 0; i < 32; ++i) xr[i] = x[i];
#pragma unroll
      for (int jj = 0; jj < 32; ++jj)
#pragma unroll
        for (int i = jj + 1; i < 32; ++i) xr[i] = Sc<S>::sub(xr[i], Sc<S>::mul(L[jj * 32 + i], xr[jj]));
#pragma unroll
      for (int i = 0; i < 32; ++i) x[i] = xr[i];
    } else {
      for (int jj = 0; jj < w; ++jj) {
        const S xj = x[jj];
        for (int i = jj + 1; i < w; ++i) x[i] = Sc<S>::sub(x[i], Sc<S>::mul(L[jj * w + i], xj));
      }
    }
  }
  __syncthreads();
  for (int t = threadIdx.x; t < 32 * ncol; t += NC) {
    const int i = t & 31, cc = t >> 5;
    if (i < w) M[(size_t)(cb + cc) * lda + k + i] = T[cc * 33 + i];
  }
}

// Diagonal block solve of getrs by one warp: the w x w block (w <= 64) staged
// in shared memory, lane l holding rows l and l + 32 of the block; the solved
// component is broadcast by a shuffle, no block-wide barrier per row.
// LOWER: unit lower forward substitution; else upper backward substitution.
template <typename S> __device__ __forceinline__ S shfl_s(S v, int src);
template <> __device__ __forceinline__ float2 shfl_s(float2 v, int src) {
  return make_float2(__shfl_sync(0xffffffffu, v.x, src), __shfl_sync(0xffffffffu, v.y, src));
}
template <> __device__ __forceinline__ double2 shfl_s(double2 v, int src) {
  return make_double2(__shfl_sync(0xffffffffu, v.x, src), __shfl_sync(0xffffffffu, v.y, src));
}
template <> __device__ __forceinline__ float shfl_s(float v, int src) { return __shfl_sync(0xffffffffu, v, src); }
template <> __device__ __forceinline__ double shfl_s(double v, int src) { return __shfl_sync(0xffffffffu, v, src); }

// Stage the w x w diagonal block at (r0, r0) into D[col * 65 + row] with 128
// threads, eight loads in flight per thread before their stores (the block is
// usually cold in L2; one load per iteration would serialise on its latency).
template <typename S>
__device__ __forceinline__ void stage_diag64(const S* M, int lda, int r0, int w, S* D) {
  for (int t0 = threadIdx.x; t0 < w * 64; t0 += 128 * 8) {
    S v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int t = t0 + 128 * u, i = t & 63, j = t >> 6;
      if (t < w * 64 && i < w) v[u] = M[(size_t)(r0 + j) * lda + r0 + i];
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int t = t0 + 128 * u, i = t & 63, j = t >> 6;
      if (t < w * 64 && i < w) D[j * 65 + i] = v[u];
    }
  }
}

template <typename S, bool LOWER>
__global__ void __launch_bounds__(128) k_trsv_diag64(const S* A, long long strideA, int lda, S* b, long long strideb,
                                                     int r0, int w) {
  const int bidx = blockIdx.x;
  const S* M = A + strideA * bidx;
  S* xg = b + strideb * bidx;
  extern __shared__ __align__(16) unsigned char smraw[];
  S* D = reinterpret_cast<S*>(smraw);  // [col][row], w x w, padded to 65 rows
  stage_diag64(M, lda, r0, w, D);
  __syncthreads();
  if (threadIdx.x >= 32) return;
  const int l = threadIdx.x;
  S x0 = l < w ? xg[r0 + l] : Sc<S>::zero();
  S x1 = l + 32 < w ? xg[r0 + l + 32] : Sc<S>::zero();
  if (LOWER) {
    for (int j = 0; j < w; ++j) {
      const S xj = shfl_s(j < 32 ? x0 : x1, j & 31);
      if (l > j && l < w) x0 = Sc<S>::sub(x0, Sc<S>::mul(D[j * 65 + l], xj));
      if (l + 32 > j && l + 32 < w) x1 = Sc<S>::sub(x1, Sc<S>::mul(D[j * 65 + l + 32], xj));
    }
  } else {
    for (int j = w - 1; j >= 0; --j) {
      if (j < 32) { if (l == j) x0 = Sc<S>::div(x0, D[j * 65 + j]); }
      else { if (l + 32 == j) x1 = Sc<S>::div(x1, D[j * 65 + j]); }
      const S xj = shfl_s(j < 32 ? x0 : x1, j & 31);
      if (l < j) x0 = Sc<S>::sub(x0, Sc<S>::mul(D[j * 65 + l], xj));
      if (l + 32 < j) x1 = Sc<S>::sub(x1, Sc<S>::mul(D[j * 65 + l + 32], xj));
    }
  }
  if (l < w) xg[r0 + l] = x0;
  if (l + 32 < w) xg[r0 + l + 32] = x1;
}

// ---------------------------------------------------------------------------
// Inner panel without row interchanges (the mixed path's first attempt; its
// factors are only a preconditioner for FP64 refinement, which falls back to
// partial pivoting when it stalls), one launch: every CTA factorises the
// kb x kb diagonal block in shared memory (the same operations in the same
// order, so every copy is bitwise the one written back), takes the
// reciprocals of U11's diagonal, then solves its 128 rows of
// L21 = A21 inv(U11), one thread per row. No cross-CTA pivot search per
// column and no launch between the diagonal block and its rows (a separate
// diagonal kernel cost one dependent launch per 32 columns). The factorised
// block goes back in place only after every CTA has read the original: each
// CTA takes a ticket from cnt[b] after its load, and the last one writes and
// resets the counter (zero on entry, zero on exit). A zero or non-finite
// pivot sets info and leaves the rows as they are.
// Grid: (max(1, ceil((r1 - r0) / 128)), batch).
// ---------------------------------------------------------------------------
template <typename S>
__global__ void __launch_bounds__(128) k_panel_nopiv(S* A, long long sA, int lda, int k, int kb, int r0, int r1,
                                                     int* info, int* cnt) {
  __shared__ S D[32 * 33];
  __shared__ S ur[32];  // reciprocals of U11's diagonal: the row chains multiply, no division
  __shared__ int s_bad, s_last;
  const int b = blockIdx.y, t = threadIdx.x;
  S* M = A + sA * b;
  for (int e = t; e < kb * kb; e += 128) {
    const int i = e % kb, c = e / kb;
    D[c * 33 + i] = M[(size_t)(k + c) * lda + k + i];
  }
  if (t == 0) s_bad = 0;
  __syncthreads();
  if (t == 0) s_last = atomicAdd(cnt + b, 1) == (int)gridDim.x - 1;
  for (int j = 0; j < kb; ++j) {
    const S d = D[j * 33 + j];
    const float m = (float)Sc<S>::abs1(d);
    if (!(m > 0.0f) || !isfinite(m)) {
      if (t == 0) {
        s_bad = 1;
        if (s_last && info[b] == 0) info[b] = k + j + 1;
      }
      break;
    }
    const S rcp = Sc<S>::rcp(d);
    for (int i = j + 1 + t; i < kb; i += 128) D[j * 33 + i] = Sc<S>::mul(D[j * 33 + i], rcp);
    __syncthreads();
    const int w = kb - j - 1;
    for (int e = t; e < w * w; e += 128) {
      const int i = j + 1 + e % w, c = j + 1 + e / w;
      D[c * 33 + i] = Sc<S>::sub(D[c * 33 + i], Sc<S>::mul(D[j * 33 + i], D[c * 33 + j]));
    }
    __syncthreads();
  }
  __syncthreads();
  if (s_last) {
    for (int e = t; e < kb * kb; e += 128) {
      const int i = e % kb, c = e / kb;
      M[(size_t)(k + c) * lda + k + i] = D[c * 33 + i];
    }
    if (t == 0) cnt[b] = 0;
  }
  if (s_bad) return;
  if (t < kb) ur[t] = Sc<S>::rcp(D[t * 33 + t]);
  __syncthreads();
  const int row = r0 + blockIdx.x * 128 + t;
  if (row >= r1) return;
  S x[32];
#pragma unroll
  for (int j = 0; j < 32; ++j)
    if (j < kb) x[j] = M[(size_t)(k + j) * lda + row];
#pragma unroll
  for (int j = 0; j < 32; ++j) {
    if (j < kb) {
      S v = x[j];
#pragma unroll
      for (int c = 0; c < j; ++c) v = Sc<S>::sub(v, Sc<S>::mul(x[c], D[j * 33 + c]));
      x[j] = Sc<S>::mul(v, ur[j]);
    }
  }
#pragma unroll
  for (int j = 0; j < 32; ++j)
    if (j < kb) M[(size_t)(k + j) * lda + row] = x[j];
}

// ---------------------------------------------------------------------------
// Triangular solve of getrs in one launch per triangle (no counterpart in the
// reference, which calls ?getrs): the rows are cut in blocks of 64; a CTA takes
// work items (system, block) in solve order from a global counter, adds the
// contributions of the blocks already solved as their ready flags appear
// (L or U read once, 64 contiguous entries per column), solves its 64 x 64
// diagonal block in one warp (shuffles) and publishes x and its flag. Items are
// claimed in dependency order, so every block an item waits for is held by a
// CTA that is already running: no co-residency is needed. Waits on flags are
// bounded; a wait that gives up sets *err and the CTA publishes its block
// anyway, so every other wait ends too.
// LOWER: unit lower L, forward; else upper U with its diagonal, backward.
// ready[b * nb + blk] must be 0 and *counter 0 on entry. Dynamic shared
// memory: trsv_sf_smem<S>() bytes.
// ---------------------------------------------------------------------------
constexpr long long kTrsvSpin = 1LL << 22;
template <typename S>
constexpr size_t trsv_sf_smem() {
  return sizeof(S) * (64 * 65 + 4 * 64 + 64 + 64);
}
__device__ __forceinline__ int ld_acquire_s32(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
// Loads of the factors issued where they stand in the program: the
// prefetch of the next solved block's tile must leave before the wait on
// that block's flag (a plain load may be scheduled next to its first use,
// behind the wait). The factors are read-only during the solve.
__device__ __forceinline__ float ld_pinned(const float* p) {
  float v;
  asm volatile("ld.global.nc.f32 %0, [%1];" : "=f"(v) : "l"(p));
  return v;
}
__device__ __forceinline__ double ld_pinned(const double* p) {
  double v;
  asm volatile("ld.global.nc.f64 %0, [%1];" : "=d"(v) : "l"(p));
  return v;
}
__device__ __forceinline__ float2 ld_pinned(const float2* p) {
  float2 v;
  asm volatile("ld.global.nc.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "l"(p));
  return v;
}
__device__ __forceinline__ double2 ld_pinned(const double2* p) {
  double2 v;
  asm volatile("ld.global.nc.v2.f64 {%0, %1}, [%2];" : "=d"(v.x), "=d"(v.y) : "l"(p));
  return v;
}
template <typename S, bool LOWER>
__global__ void __launch_bounds__(256) k_trsv_sf(const S* A, long long sA, int lda, int n, S* x, long long sx,
                                                 int batch, int nb, unsigned* counter, int* ready, int* err,
                                                 long long spin) {
  // dynamic shared memory: D [64 x 65] (diagonal block, column-major), part [4][64],
  // xs [64] (the solved block being applied), rinv [64] (reciprocals of U's
  // diagonal, formed before the wait so that no division lies on the chain)
  extern __shared__ __align__(16) unsigned char sfraw[];
  S* D = reinterpret_cast<S*>(sfraw);
  S (*part)[64] = reinterpret_cast<S (*)[64]>(D + 64 * 65);
  S* xs = D + 64 * 65 + 4 * 64;
  S* rinv = xs + 64;
  __shared__ int s_item, s_end;
  const int t = threadIdx.x, row = t & 63, grp = t >> 6;
  const long long lim = spin > 0 ? spin : kTrsvSpin;
  for (;;) {
    if (t == 0) s_item = (int)atomicAdd(counter, 1u);
    __syncthreads();
    const int item = s_item;
    if (item >= nb * batch) break;
    const int b = item % batch, q = item / batch;
    const int blk = LOWER ? q : nb - 1 - q;
    const int r0 = blk * 64, w = min(64, n - r0);
    const S* M = A + sA * b;
    S* xb = x + sx * b;
    // this thread's 16 entries (row, columns grp + 4i) of the next solved
    // block's tile: loaded before that block is published (the factors do not
    // depend on it), so applying a newly solved block costs one load of its
    // 64 values and 16 FMAs
    S mreg[16];
    auto load_tile = [&](int qq) {
      const int jb = LOWER ? qq : nb - 1 - qq;
      const int c0 = jb * 64, wc = min(64, n - c0);
#pragma unroll
      for (int i = 0; i < 16; ++i) {
        const int c = grp + 4 * i;
        mreg[i] = (row < w && c < wc) ? ld_pinned(M + (size_t)(c0 + c) * lda + r0 + row) : Sc<S>::zero();
      }
    };
    if (q > 0) load_tile(0);
    // diagonal block into shared memory (used after the contributions); the
    // upper triangle's rows scaled by the reciprocals of U's diagonal, so
    // that the substitution chain below carries no multiplication by them
    if (!LOWER) {
      if (t < w) rinv[t] = Sc<S>::rcp(M[(size_t)(r0 + t) * lda + r0 + t]);
      __syncthreads();
    }
    for (int e = t; e < 64 * 64; e += 256) {
      const int i = e & 63, j = e >> 6;
      if (i < w && j < w) {
        const S v = M[(size_t)(r0 + j) * lda + r0 + i];
        D[j * 65 + i] = LOWER ? v : Sc<S>::mul(v, rinv[i]);
      }
    }
    // contributions of the solved blocks, in the order they were solved:
    // thread 0 waits for the next one, then takes every later one already
    // published too, so a CTA that is behind catches up with one barrier
    S acc = Sc<S>::zero();
    for (int done = 0; done < q;) {
      if (t == 0) {
        long long it = 0;
        const int jb0 = LOWER ? done : nb - 1 - done;
        while (ld_acquire_s32(ready + (size_t)b * nb + jb0) == 0) {
          if (++it > lim) {
            atomicExch(err, 1);
            break;
          }
          if (it > 64) __nanosleep(64);
        }
        int e = done + 1;
        while (e < q && ld_acquire_s32(ready + (size_t)b * nb + (LOWER ? e : nb - 1 - e)) != 0) ++e;
        s_end = e;
      }
      __syncthreads();
      const int end = s_end;
      for (int qq = done; qq < end; ++qq) {
        const int jb = LOWER ? qq : nb - 1 - qq;
        const int c0 = jb * 64, wc = min(64, n - c0);
        if (t < 64) xs[t] = t < wc ? __ldcg(xb + c0 + t) : Sc<S>::zero();
        __syncthreads();
#pragma unroll
        for (int i = 0; i < 16; ++i) acc = Sc<S>::add(acc, Sc<S>::mul(mreg[i], xs[grp + 4 * i]));
        __syncthreads();
        if (qq + 1 < q) load_tile(qq + 1);
      }
      done = end;
    }
    part[grp][row] = acc;
    __syncthreads();
    if (t < 32) {
      const int l = t;
      S x0 = Sc<S>::zero(), x1 = Sc<S>::zero();
      if (l < w) x0 = Sc<S>::sub(xb[r0 + l], Sc<S>::add(Sc<S>::add(part[0][l], part[1][l]), Sc<S>::add(part[2][l], part[3][l])));
      if (l + 32 < w)
        x1 = Sc<S>::sub(xb[r0 + l + 32], Sc<S>::add(Sc<S>::add(part[0][l + 32], part[1][l + 32]),
                                                    Sc<S>::add(part[2][l + 32], part[3][l + 32])));
      if (LOWER) {
        for (int j = 0; j < w; ++j) {
          const S xj = shfl_s(j < 32 ? x0 : x1, j & 31);
          if (l > j && l < w) x0 = Sc<S>::sub(x0, Sc<S>::mul(D[j * 65 + l], xj));
          if (l + 32 > j && l + 32 < w) x1 = Sc<S>::sub(x1, Sc<S>::mul(D[j * 65 + l + 32], xj));
        }
      } else {
        // rows pre-scaled: x_l = y_l / u_ll - sum_{j > l} (u_lj / u_ll) x_j
        if (l < w) x0 = Sc<S>::mul(x0, rinv[l]);
        if (l + 32 < w) x1 = Sc<S>::mul(x1, rinv[l + 32]);
        for (int j = w - 1; j >= 0; --j) {
          const S xj = shfl_s(j < 32 ? x0 : x1, j & 31);
          if (l < j) x0 = Sc<S>::sub(x0, Sc<S>::mul(D[j * 65 + l], xj));
          if (l + 32 < j) x1 = Sc<S>::sub(x1, Sc<S>::mul(D[j * 65 + l + 32], xj));
        }
      }
      if (l < w) xb[r0 + l] = x0;
      if (l + 32 < w) xb[r0 + l + 32] = x1;
      __threadfence();
      __syncwarp();
      if (l == 0) atomicExch(ready + (size_t)b * nb + blk, 1);
    }
    __syncthreads();
  }
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
#pragma unroll 8
  for (int j = 0; j < w; ++j) acc = Sc<S>::add(acc, Sc<S>::mul(M[(size_t)(r0 + j) * lda + i], xs[j]));
  x[i] = Sc<S>::sub(x[i], acc);
}

}  // namespace mfb
