// solve_lse_r / solve_lse_c with every option of the reference
// (src/solve_lse_r.f90:25-232, src/solve_lse_c.f90:25-219), all on the device:
//
//   lse_scaling    ?geequ row / column scale factors and ?laqge's decision
//                  (equed N/R/C/B, thresholds 0.1 and safe-min / precision);
//                  b scaled by r before the solve, x by c after it
//   factorize      ?getrf (getrf_batched)
//   lse_condition  ?gecon: one-norm of the (scaled) matrix and the ?lacn2
//                  estimate of ||inv(A)||_1 from solves with L, U, U^H, L^H
//   (solve)        ?getrs (getrs_batched)
//   lse_refine     ?gerfs: residual with the unfactorised matrix, componentwise
//                  backward error, at most five correction steps while it
//                  halves, forward-error bound by ?lacn2 with solves by A^H
//
// The one-norm estimator is Higham's refinement of Hager's method (LAPACK
// ?lacn2, Higham, ACM TOMS 14(4), 1988). Its control flow, a handful of
// scalar decisions per step, runs on the host over device-resident vectors;
// every vector operation is a kernel. ?gecon's triangular solves are ?latrs,
// which rescales to avoid overflow; the solves here are plain substitutions,
// identical whenever ?latrs does not rescale (always, for matrices whose
// inverse norm stays far below the overflow threshold).
#pragma once
#include <climits>
#include <cstring>

namespace mfb {

// ---------------------------------------------------------------------------
// Conjugate-transposed triangular solves with the LU factors: U^H forward
// (lower, non-unit) and L^H backward (upper, unit), blocked by 64 rows like
// getrs_batched's solves.
// ---------------------------------------------------------------------------
template <typename S, bool LH>
__global__ void __launch_bounds__(128) k_trsv_diag64_h(const S* A, long long strideA, int lda, S* b,
                                                       long long strideb, int r0, int w) {
  const S* M = A + strideA * blockIdx.x;
  S* xg = b + strideb * blockIdx.x;
  extern __shared__ __align__(16) unsigned char smraw[];
  S* D = reinterpret_cast<S*>(smraw);  // D[col * 65 + row] = A(r0 + row, r0 + col)
  stage_diag64(M, lda, r0, w, D);
  __syncthreads();
  if (threadIdx.x >= 32) return;
  const int l = threadIdx.x;
  S x0 = l < w ? xg[r0 + l] : Sc<S>::zero();
  S x1 = l + 32 < w ? xg[r0 + l + 32] : Sc<S>::zero();
  if (!LH) {
    // x_j /= conj(U_jj); x_i -= conj(U_ji) x_j for i > j (U_ji = D[i * 65 + j])
    for (int j = 0; j < w; ++j) {
      if (j < 32) { if (l == j) x0 = Sc<S>::div(x0, Sc<S>::conj(D[j * 65 + j])); }
      else { if (l + 32 == j) x1 = Sc<S>::div(x1, Sc<S>::conj(D[j * 65 + j])); }
      const S xj = shfl_s(j < 32 ? x0 : x1, j & 31);
      if (l > j && l < w) x0 = Sc<S>::sub(x0, Sc<S>::mul(Sc<S>::conj(D[l * 65 + j]), xj));
      if (l + 32 > j && l + 32 < w) x1 = Sc<S>::sub(x1, Sc<S>::mul(Sc<S>::conj(D[(l + 32) * 65 + j]), xj));
    }
  } else {
    // unit diagonal; x_i -= conj(L_ji) x_j for i < j
    for (int j = w - 1; j >= 0; --j) {
      const S xj = shfl_s(j < 32 ? x0 : x1, j & 31);
      if (l < j) x0 = Sc<S>::sub(x0, Sc<S>::mul(Sc<S>::conj(D[l * 65 + j]), xj));
      if (l + 32 < j) x1 = Sc<S>::sub(x1, Sc<S>::mul(Sc<S>::conj(D[(l + 32) * 65 + j]), xj));
    }
  }
  if (l < w) xg[r0 + l] = x0;
  if (l + 32 < w) xg[r0 + l + 32] = x1;
}

// rows [i0, i1): x_i -= sum_j conj(A(r0 + j, i)) x_{r0 + j}; one warp per row,
// reading column i's block rows contiguously
template <typename S>
__global__ void k_trsv_update_h(const S* A, long long strideA, int lda, S* b, long long strideb, int r0, int w,
                                int i0, int i1) {
  const S* M = A + strideA * blockIdx.y;
  S* x = b + strideb * blockIdx.y;
  __shared__ S xs[64];
  if ((int)threadIdx.x < w) xs[threadIdx.x] = x[r0 + threadIdx.x];
  __syncthreads();
  const int l = threadIdx.x & 31;
  const int i = i0 + blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (i >= i1) return;
  const S* col = M + (size_t)i * lda + r0;
  S acc = Sc<S>::zero();
  if (l < w) acc = Sc<S>::mul(Sc<S>::conj(col[l]), xs[l]);
  if (l + 32 < w) acc = Sc<S>::add(acc, Sc<S>::mul(Sc<S>::conj(col[l + 32]), xs[l + 32]));
  for (int o = 16; o > 0; o >>= 1) acc = Sc<S>::add(acc, shfl_s(acc, l ^ o));
  if (l == 0) x[i] = Sc<S>::sub(x[i], acc);
}

// inverse of the getrs row permutation: out[perm[i]] = x[i]
template <typename S>
__global__ void k_scatter_perm(const S* x, long long sx, const int* perm, int n, S* out) {
  const int bi = blockIdx.y, i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  out[(size_t)n * bi + perm[(size_t)n * bi + i]] = x[sx * bi + i];
}
// the interchanges in reverse order (one thread per right-hand side), for n
// too large for k_perm's shared-memory index array
template <typename S>
__global__ void k_rhs_swap_rev(S* b, long long sb, int n, const int* ipiv, long long sP, int nbatch) {
  const int bi = blockIdx.x * blockDim.x + threadIdx.x;
  if (bi >= nbatch) return;
  S* x = b + sb * bi;
  const int* piv = ipiv + sP * bi;
  for (int j = n - 1; j >= 0; --j) {
    const int p = piv[j] - 1;
    if (p != j) {
      S t = x[j];
      x[j] = x[p];
      x[p] = t;
    }
  }
}

enum TrOp { TR_L = 0, TR_U = 1, TR_UH = 2, TR_LH = 3 };

// one triangular solve with the factors in A (no permutation)
template <typename S>
static int trsv_op(cudaStream_t st, const S* A, long long sA, int lda, int n, S* b, long long sb, int batch, int op) {
  const int TB = 64;
  const size_t dsm = (size_t)TB * 65 * sizeof(S);
  const void* kd = op == TR_L ? (const void*)k_trsv_diag64<S, true>
                   : op == TR_U ? (const void*)k_trsv_diag64<S, false>
                   : op == TR_UH ? (const void*)k_trsv_diag64_h<S, false> : (const void*)k_trsv_diag64_h<S, true>;
  if (raise_smem_limit(kd)) return fail(MFBEM_ECUDA, "shared-memory limit of the triangular solve");
  const int last = ((n - 1) / TB) * TB;
  const bool fwd = op == TR_L || op == TR_UH;
  for (int k = 0; k < n; k += TB) {
    const int r0 = fwd ? k : last - k;
    const int w = std::min(TB, n - r0);
    const int i0 = fwd ? r0 + w : 0, i1 = fwd ? n : r0;
    switch (op) {
      case TR_L: k_trsv_diag64<S, true><<<batch, 128, dsm, st>>>(A, sA, lda, b, sb, r0, w); break;
      case TR_U: k_trsv_diag64<S, false><<<batch, 128, dsm, st>>>(A, sA, lda, b, sb, r0, w); break;
      case TR_UH: k_trsv_diag64_h<S, false><<<batch, 128, dsm, st>>>(A, sA, lda, b, sb, r0, w); break;
      default: k_trsv_diag64_h<S, true><<<batch, 128, dsm, st>>>(A, sA, lda, b, sb, r0, w); break;
    }
    ++g_launches;
    if (i1 > i0) {
      if (op <= TR_U)
        k_trsv_update<S><<<dim3(nblk(i1 - i0, 256), batch), 256, 0, st>>>(A, sA, lda, b, sb, r0, w, i0, i1);
      else
        k_trsv_update_h<S><<<dim3(nblk(i1 - i0, 8), batch), 256, 0, st>>>(A, sA, lda, b, sb, r0, w, i0, i1);
      ++g_launches;
    }
  }
  CK(cudaGetLastError());
  return 0;
}

// getrs with trans = 'C' (complex) / 'T' (real): x = P^T L^-H U^-H b
template <typename S>
static int getrs_conj(cudaStream_t st, const S* A, int lda, int n, const int* ipiv, S* b, long long sb, int batch) {
  int rc = trsv_op<S>(st, A, 0, lda, n, b, sb, batch, TR_UH);
  if (!rc) rc = trsv_op<S>(st, A, 0, lda, n, b, sb, batch, TR_LH);
  if (rc) return rc;
  const size_t psm = (size_t)n * sizeof(int);
  if (psm <= 200 * 1024) {
    if ((rc = ensure(g_rs_ws, (size_t)batch * n * (sizeof(int) + sizeof(S)) + 256))) return rc;
    if (psm > 48 * 1024 && raise_smem_limit((const void*)k_perm)) return fail(MFBEM_ECUDA, "shared-memory limit of the row permutation");
    int* perm = (int*)g_rs_ws.p;
    S* tmp = (S*)((char*)g_rs_ws.p + ((size_t)batch * n * sizeof(int) + 255) / 256 * 256);
    k_perm<<<batch, 256, psm, st>>>(ipiv, 0, n, perm); ++g_launches;
    k_scatter_perm<S><<<dim3(nblk(n, 256), batch), 256, 0, st>>>(b, sb, perm, n, tmp); ++g_launches;
    k_scatter_back<S><<<dim3(nblk(n, 256), batch), 256, 0, st>>>(tmp, n, b, sb); ++g_launches;
  } else {
    k_rhs_swap_rev<S><<<nblk(batch, 64), 64, 0, st>>>(b, sb, n, ipiv, 0, batch); ++g_launches;
  }
  CK(cudaGetLastError());
  return 0;
}

// ---------------------------------------------------------------------------
// ?geequ / ?laqge
// ---------------------------------------------------------------------------
// DLAMCH('S') and 1 / DLAMCH('S')
constexpr double kSafeMin = 2.2250738585072014e-308;
constexpr double kBigNum = 1.0 / 2.2250738585072014e-308;
// DLAMCH('E') (relative machine precision, rounding) and DLAMCH('P') = 2 E
constexpr double kEps = 1.1102230246251565e-16;
constexpr double kPrec = 2.220446049250313e-16;

// the absolute value ?geequ / ?gerfs use: |re| + |im| (CABS1) for complex
template <typename S> __device__ __forceinline__ double abs1d(S a) { return (double)Sc<S>::abs1(a); }
// the modulus (Fortran ABS of a complex): ?lacn2 and ?gecon's column sums
__device__ __forceinline__ double absm(double a) { return fabs(a); }
__device__ __forceinline__ double absm(double2 a) { return hypot(a.x, a.y); }

// row maxima over column chunks; non-negative doubles order as their bits
template <typename S>
__global__ void k_absmax_rows(const S* A, int lda, int n, int cols_per_chunk, unsigned long long* R) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int j0 = blockIdx.y * cols_per_chunk, j1 = min(n, j0 + cols_per_chunk);
  double m = 0.0;
  for (int j = j0; j < j1; ++j) m = fmax(m, abs1d(A[(size_t)j * lda + i]));
  atomicMax(R + i, (unsigned long long)__double_as_longlong(m));
}
// column maxima of |a_ij| * r_i (one warp per column)
template <typename S>
__global__ void k_absmax_cols(const S* A, int lda, int n, const double* r, unsigned long long* C) {
  const int j = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), l = threadIdx.x & 31;
  if (j >= n) return;
  double m = 0.0;
  for (int i = l; i < n; i += 32) m = fmax(m, abs1d(A[(size_t)j * lda + i]) * r[i]);
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if (l == 0) C[j] = (unsigned long long)__double_as_longlong(m);
}
// ?geequ's reduction of the maxima v[0..n): out = {cnd, max}, info = info_base +
// first zero index (1-based) or 0; v[i] <- 1 / min(max(v[i], smlnum), bignum)
__global__ void k_eq_finish(unsigned long long* vb, double* v, int n, int info_base, double* out, int* info) {
  __shared__ double smin[1024], smax[1024];
  __shared__ int szero[1024];
  double mn = kBigNum, mx = 0.0;
  int z = INT_MAX;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double a = __longlong_as_double((long long)vb[i]);
    mn = fmin(mn, a);
    mx = fmax(mx, a);
    if (a == 0.0 && i < z) z = i;
  }
  smin[threadIdx.x] = mn;
  smax[threadIdx.x] = mx;
  szero[threadIdx.x] = z;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) {
      smin[threadIdx.x] = fmin(smin[threadIdx.x], smin[threadIdx.x + s]);
      smax[threadIdx.x] = fmax(smax[threadIdx.x], smax[threadIdx.x + s]);
      szero[threadIdx.x] = min(szero[threadIdx.x], szero[threadIdx.x + s]);
    }
    __syncthreads();
  }
  const double rcmin = smin[0], rcmax = smax[0];
  if (rcmin == 0.0) {
    if (threadIdx.x == 0) *info = info_base + szero[0] + 1;
    return;
  }
  for (int i = threadIdx.x; i < n; i += blockDim.x)
    v[i] = 1.0 / fmin(fmax(__longlong_as_double((long long)vb[i]), kSafeMin), kBigNum);
  if (threadIdx.x == 0) {
    out[0] = fmax(rcmin, kSafeMin) / fmin(rcmax, kBigNum);
    out[1] = rcmax;
    *info = 0;
  }
}
// ?laqge's scaling: mode 'C' a_ij *= c_j, 'R' a_ij *= r_i, 'B' a_ij *= (c_j r_i)
template <typename S>
__global__ void k_laqge(S* A, int lda, int n, const double* r, const double* c, int mode) {
  const long long nn = (long long)n * n;
  for (long long id = blockIdx.x * (long long)blockDim.x + threadIdx.x; id < nn; id += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(id % n), j = (int)(id / n);
    const double s = mode == 'C' ? c[j] : (mode == 'R' ? r[i] : c[j] * r[i]);
    S& a = A[(size_t)j * lda + i];
    a = Sc<S>::mul(a, Sc<S>::from(s));
  }
}
// b(:, k) *= s(:) for every right-hand side
template <typename S>
__global__ void k_rows_scale(S* b, int n, int nrhs, const double* s) {
  const long long t = (long long)n * nrhs;
  for (long long id = blockIdx.x * (long long)blockDim.x + threadIdx.x; id < t; id += (long long)gridDim.x * blockDim.x)
    b[id] = Sc<S>::mul(b[id], Sc<S>::from(s[id % n]));
}

// one-norm of A, the column sums of moduli as src/solve_lse_c.f90:140-147 (one
// warp per column, maximum through the bit order of non-negative doubles)
template <typename S>
__global__ void k_norm1(const S* A, int lda, int n, unsigned long long* out) {
  const int j = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), l = threadIdx.x & 31;
  if (j >= n) return;
  double s = 0.0;
  for (int i = l; i < n; i += 32) s += absm(A[(size_t)j * lda + i]);
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (l == 0) atomicMax(out, (unsigned long long)__double_as_longlong(s));
}

// ---------------------------------------------------------------------------
// vector kernels of ?lacn2 and ?gerfs (one block; n is a matrix dimension)
// ---------------------------------------------------------------------------
// out = {sum |x_i|, max |x_i|, first index of the maximum, value at q}; MODE 0
// the modulus (?lacn2: dasum / dzsum1, idamax / izmax1), MODE 1 CABS1
// (?gerfs' normalisation). out[3] = x_q (real) or |x_q| (complex).
template <typename S, int MODE>
__global__ void k_vstats(const S* x, int n, int q, double* out) {
  __shared__ double ss[1024], sm[1024];
  __shared__ int si[1024];
  double s = 0.0, m = -1.0;
  int mi = 0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double a = MODE ? abs1d(x[i]) : absm(x[i]);
    s += a;
    if (a > m) { m = a; mi = i; }
  }
  ss[threadIdx.x] = s;
  sm[threadIdx.x] = m;
  si[threadIdx.x] = mi;
  __syncthreads();
  for (int h = blockDim.x / 2; h > 0; h >>= 1) {
    if ((int)threadIdx.x < h) {
      ss[threadIdx.x] += ss[threadIdx.x + h];
      const double m2 = sm[threadIdx.x + h];
      const int i2 = si[threadIdx.x + h];
      if (m2 > sm[threadIdx.x] || (m2 == sm[threadIdx.x] && i2 < si[threadIdx.x])) {
        sm[threadIdx.x] = m2;
        si[threadIdx.x] = i2;
      }
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[0] = ss[0];
    out[1] = sm[0];
    out[2] = (double)si[0];
    out[3] = (q >= 0 && q < n) ? (sizeof(S) == 8 ? Sc<S>::re(x[q]) : absm(x[q])) : 0.0;
  }
}
template <typename S>
__global__ void k_vfill(S* x, int n, double v) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) x[i] = Sc<S>::from(v);
}
template <typename S>
__global__ void k_vunit(S* x, int n, int j) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) x[i] = Sc<S>::from(i == j ? 1.0 : 0.0);
}
// x_i = (-1)^i (1 + i / (n - 1))
template <typename S>
__global__ void k_valt(S* x, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) x[i] = Sc<S>::from((i & 1 ? -1.0 : 1.0) * (1.0 + (double)i / (double)(n - 1)));
}
// complex: x_i / |x_i| (1 where |x_i| <= safe-min)
__global__ void k_vsign_c(double2* x, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double a = hypot(x[i].x, x[i].y);
  x[i] = a > kSafeMin ? make_double2(x[i].x / a, x[i].y / a) : make_double2(1.0, 0.0);
}
// real: sign vector s_i = +-1; apply 0: flag = some s_i differs from isgn_i;
// apply 1: x = s, isgn = s
__global__ void k_vsign_r(double* x, int* isgn, int n, int apply, int* flag) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int s = x[i] >= 0.0 ? 1 : -1;
  if (apply) {
    x[i] = (double)s;
    isgn[i] = s;
  } else if (s != isgn[i]) {
    *flag = 1;
  }
}
template <typename S>
__global__ void k_vmulw(S* x, const double* w, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) x[i] = Sc<S>::mul(x[i], Sc<S>::from(w[i]));
}
template <typename S>
__global__ void k_vaxpy(S* x, const S* d, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) x[i] = Sc<S>::add(x[i], d[i]);
}
// sum_k |a_ik| |x_k| over column chunks (?gerfs), partial sums part[chunk][i]
template <typename S>
__global__ void k_absAx(const S* A, int lda, int n, const S* x, int cols_per_chunk, double* part) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int j0 = blockIdx.y * cols_per_chunk, j1 = min(n, j0 + cols_per_chunk);
  double s = 0.0;
  for (int k = j0; k < j1; ++k) s += abs1d(A[(size_t)k * lda + i]) * abs1d(x[k]);
  part[(size_t)blockIdx.y * n + i] = s;
}
// w_i = |b_i| + sum of the partials; out[0] = the componentwise backward error
// max_i |r_i| / w_i (with ?gerfs' safe-min guard)
template <typename S>
__global__ void k_berr(const S* R, const S* b, const double* part, int nch, int n, double safe1, double safe2,
                       double* w, double* out) {
  __shared__ double sm[1024];
  double m = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    double wi = abs1d(b[i]);
    for (int c = 0; c < nch; ++c) wi += part[(size_t)c * n + i];
    w[i] = wi;
    const double ar = abs1d(R[i]);
    m = fmax(m, wi > safe2 ? ar / wi : (ar + safe1) / (wi + safe1));
  }
  sm[threadIdx.x] = m;
  __syncthreads();
  for (int h = blockDim.x / 2; h > 0; h >>= 1) {
    if ((int)threadIdx.x < h) sm[threadIdx.x] = fmax(sm[threadIdx.x], sm[threadIdx.x + h]);
    __syncthreads();
  }
  if (threadIdx.x == 0) out[0] = sm[0];
}
// ?gerfs' weights of the forward-error bound: |r_i| + (n+1) eps w_i (+ safe1)
template <typename S>
__global__ void k_ferr_w(const S* R, double* w, int n, double nzeps, double safe1, double safe2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double ar = abs1d(R[i]);
  w[i] = w[i] > safe2 ? ar + nzeps * w[i] : ar + nzeps * w[i] + safe1;
}

// ---------------------------------------------------------------------------
// host drivers
// ---------------------------------------------------------------------------
struct LseWork {
  cudaStream_t st;
  double* red;  // device scalars [8]
  int* flag;    // device int [2]
};

template <typename S>
static int vstats(const LseWork& w, const S* x, int n, int q, int mode, double h[4]) {
  if (mode) k_vstats<S, 1><<<1, 1024, 0, w.st>>>(x, n, q, w.red);
  else k_vstats<S, 0><<<1, 1024, 0, w.st>>>(x, n, q, w.red);
  ++g_launches;
  CK(cudaMemcpyAsync(h, w.red, 4 * sizeof(double), cudaMemcpyDeviceToHost, w.st));
  CK(cudaStreamSynchronize(w.st));
  return 0;
}
template <typename S> static void vsign(const LseWork& w, S* x, int* isgn, int n);
template <> void vsign<double2>(const LseWork& w, double2* x, int*, int n) {
  k_vsign_c<<<nblk(n, 256), 256, 0, w.st>>>(x, n); ++g_launches;
}
template <> void vsign<double>(const LseWork& w, double* x, int* isgn, int n) {
  k_vsign_r<<<nblk(n, 256), 256, 0, w.st>>>(x, isgn, n, 1, w.flag); ++g_launches;
}

// ?lacn2 with the reverse communication unrolled: apply(kase, x) overwrites x
// by A x (kase 1) or A^H x (kase 2); est receives the estimate of ||A||_1.
// x, v: n-vectors, isgn: n ints (real case).
template <typename S, class F>
static int lacn2(const LseWork& w, int n, S* x, S* v, int* isgn, F apply, double* est) {
  const bool cplx = sizeof(S) == 16;
  const unsigned g = nblk(n, 256);
  double h[4];
  int rc;
  k_vfill<S><<<g, 256, 0, w.st>>>(x, n, 1.0 / n); ++g_launches;
  if ((rc = apply(1, x))) return rc;
  if (n == 1) {
    if ((rc = vstats<S>(w, x, n, 0, 0, h))) return rc;
    *est = h[0];
    return 0;
  }
  if ((rc = vstats<S>(w, x, n, -1, 0, h))) return rc;
  double e = h[0];
  vsign<S>(w, x, isgn, n);
  if ((rc = apply(2, x)) || (rc = vstats<S>(w, x, n, -1, 0, h))) return rc;
  int j = (int)h[2], iter = 2;
  for (;;) {
    k_vunit<S><<<g, 256, 0, w.st>>>(x, n, j); ++g_launches;
    if ((rc = apply(1, x))) return rc;
    CK(cudaMemcpyAsync(v, x, sizeof(S) * n, cudaMemcpyDeviceToDevice, w.st));
    const double eold = e;
    if ((rc = vstats<S>(w, x, n, -1, 0, h))) return rc;
    e = h[0];
    if (!cplx) {  // repeated sign vector: converged
      int f = 0;
      CK(cudaMemsetAsync(w.flag, 0, sizeof(int), w.st));
      k_vsign_r<<<g, 256, 0, w.st>>>((double*)x, isgn, n, 0, w.flag); ++g_launches;
      CK(cudaMemcpyAsync(&f, w.flag, sizeof(int), cudaMemcpyDeviceToHost, w.st));
      CK(cudaStreamSynchronize(w.st));
      if (!f) break;
    }
    if (e <= eold) break;
    vsign<S>(w, x, isgn, n);
    if ((rc = apply(2, x))) return rc;
    const int jlast = j;
    if ((rc = vstats<S>(w, x, n, jlast, 0, h))) return rc;
    j = (int)h[2];
    if (h[3] != h[1] && iter < 5) {
      ++iter;
      continue;
    }
    break;
  }
  k_valt<S><<<g, 256, 0, w.st>>>(x, n); ++g_launches;
  if ((rc = apply(1, x)) || (rc = vstats<S>(w, x, n, -1, 0, h))) return rc;
  const double temp = 2.0 * (h[0] / (3.0 * n));
  if (temp > e) {
    CK(cudaMemcpyAsync(v, x, sizeof(S) * n, cudaMemcpyDeviceToDevice, w.st));
    e = temp;
  }
  *est = e;
  return 0;
}

// ?geequ + ?laqge on the device matrix A; r, c (device) receive the factors.
// Returns a positive ?geequ info (zero row i, or zero column n + j) through
// *info, else sets *equed.
template <typename S>
static int equilibrate(const LseWork& w, S* A, int n, double* r, double* c, unsigned long long* bits, int* info,
                       char* equed) {
  CK(cudaMemsetAsync(bits, 0, sizeof(unsigned long long) * n, w.st));
  const int ch = 64, cpc = (n + ch - 1) / ch;
  k_absmax_rows<S><<<dim3(nblk(n, 256), ch), 256, 0, w.st>>>(A, n, n, cpc, bits); ++g_launches;
  int* dinfo = w.flag;
  k_eq_finish<<<1, 1024, 0, w.st>>>(bits, r, n, 0, w.red, dinfo); ++g_launches;
  double h[4];
  CK(cudaMemcpyAsync(h, w.red, 2 * sizeof(double), cudaMemcpyDeviceToHost, w.st));
  CK(cudaMemcpyAsync(info, dinfo, sizeof(int), cudaMemcpyDeviceToHost, w.st));
  CK(cudaStreamSynchronize(w.st));
  if (*info) return 0;
  const double rowcnd = h[0], amax = h[1];
  k_absmax_cols<S><<<nblk(n, 8), 256, 0, w.st>>>(A, n, n, r, bits); ++g_launches;
  k_eq_finish<<<1, 1024, 0, w.st>>>(bits, c, n, n, w.red, dinfo); ++g_launches;
  CK(cudaMemcpyAsync(h, w.red, 2 * sizeof(double), cudaMemcpyDeviceToHost, w.st));
  CK(cudaMemcpyAsync(info, dinfo, sizeof(int), cudaMemcpyDeviceToHost, w.st));
  CK(cudaStreamSynchronize(w.st));
  if (*info) return 0;
  const double colcnd = h[0];
  // ?laqge
  const double small = kSafeMin / kPrec, large = 1.0 / small;
  char e;
  if (rowcnd >= 0.1 && amax >= small && amax <= large) e = colcnd >= 0.1 ? 'N' : 'C';
  else e = colcnd >= 0.1 ? 'R' : 'B';
  if (e != 'N') {
    k_laqge<S><<<152 * 8, 256, 0, w.st>>>(A, n, n, r, c, e); ++g_launches;
  }
  *equed = e;
  CK(cudaGetLastError());
  return 0;
}

// ?gecon (one-norm) from the factors in LU and the one-norm of the
// unfactorised matrix Ao
template <typename S>
static int gecon1(const LseWork& w, const S* Ao, const S* LU, int n, S* x, S* v, int* isgn,
                  unsigned long long* bits, double* rcond) {
  CK(cudaMemsetAsync(bits, 0, sizeof(unsigned long long), w.st));
  k_norm1<S><<<nblk(n, 8), 256, 0, w.st>>>(Ao, n, n, bits); ++g_launches;
  unsigned long long ab = 0;
  CK(cudaMemcpyAsync(&ab, bits, sizeof(ab), cudaMemcpyDeviceToHost, w.st));
  CK(cudaStreamSynchronize(w.st));
  double anorm;
  std::memcpy(&anorm, &ab, sizeof(double));
  *rcond = 0.0;
  if (n == 0) { *rcond = 1.0; return 0; }
  if (anorm == 0.0) return 0;
  auto apply = [&](int kase, S* y) -> int {
    int rc = trsv_op<S>(w.st, LU, 0, n, n, y, n, 1, kase == 1 ? TR_L : TR_UH);
    if (!rc) rc = trsv_op<S>(w.st, LU, 0, n, n, y, n, 1, kase == 1 ? TR_U : TR_LH);
    return rc;
  };
  double ainv = 0.0;
  int rc = lacn2<S>(w, n, x, v, isgn, apply, &ainv);
  if (rc) return rc;
  if (ainv != 0.0) *rcond = (1.0 / ainv) / anorm;
  return 0;
}

// ?gerfs (no transpose) for one right-hand side: X refined in place,
// ferr / berr as LAPACK returns them. Work: R, y, v (n each), wts, part
// (64 n doubles), isgn (n ints).
template <typename S>
static int gerfs1(const LseWork& w, const S* Ao, const S* LU, const int* ipiv, int n, const S* B, S* X, S* R, S* y,
                  S* v, int* isgn, double* wts, double* part, double* ferr, double* berr) {
  const double nz = n + 1, safe1 = nz * kSafeMin, safe2 = safe1 / kEps;
  const int ch = 64, cpc = (n + ch - 1) / ch;
  const unsigned g = nblk(n, 256);
  double lstres = 3.0, h[4];
  int count = 1, rc;
  for (;;) {
    CK(cudaMemcpyAsync(R, B, sizeof(S) * n, cudaMemcpyDeviceToDevice, w.st));
    if ((rc = gemv_res<S>(w.st, n, Ao, n, 0, X, 0, R, 0, 1))) return rc;
    k_absAx<S><<<dim3(g, ch), 256, 0, w.st>>>(Ao, n, n, X, cpc, part); ++g_launches;
    k_berr<S><<<1, 1024, 0, w.st>>>(R, B, part, ch, n, safe1, safe2, wts, w.red); ++g_launches;
    CK(cudaMemcpyAsync(h, w.red, sizeof(double), cudaMemcpyDeviceToHost, w.st));
    CK(cudaStreamSynchronize(w.st));
    *berr = h[0];
    if (h[0] > kEps && 2.0 * h[0] <= lstres && count <= 5) {
      CK(cudaMemcpyAsync(y, R, sizeof(S) * n, cudaMemcpyDeviceToDevice, w.st));
      if ((rc = getrs_batched<S>(w.st, LU, 0, n, n, ipiv, 0, y, n, 1))) return rc;
      k_vaxpy<S><<<g, 256, 0, w.st>>>(X, y, n); ++g_launches;
      lstres = h[0];
      ++count;
      continue;
    }
    break;
  }
  k_ferr_w<S><<<g, 256, 0, w.st>>>(R, wts, n, nz * kEps, safe1, safe2); ++g_launches;
  auto apply = [&](int kase, S* z) -> int {
    int rc2 = 0;
    if (kase == 1) {
      rc2 = getrs_conj<S>(w.st, LU, n, n, ipiv, z, n, 1);
      k_vmulw<S><<<g, 256, 0, w.st>>>(z, wts, n); ++g_launches;
    } else {
      k_vmulw<S><<<g, 256, 0, w.st>>>(z, wts, n); ++g_launches;
      rc2 = getrs_batched<S>(w.st, LU, 0, n, n, ipiv, 0, z, n, 1);
    }
    return rc2;
  };
  double f = 0.0;
  if ((rc = lacn2<S>(w, n, y, v, isgn, apply, &f))) return rc;
  if ((rc = vstats<S>(w, X, n, -1, 1, h))) return rc;
  *ferr = h[1] != 0.0 ? f / h[1] : f;
  return 0;
}

// ---------------------------------------------------------------------------
// mfbem_solve_{r,c}: the drop-in (host arrays in and out)
// ---------------------------------------------------------------------------
struct LseReport {
  double rcond = NAN;
  std::vector<double> ferr, berr;
};
static thread_local LseReport g_lse;

struct SolveCtx {
  cudaStream_t st = nullptr;
  DevBuf A, b, ipiv, info, Ao, bc, wv;
};
// one context per device ordinal (the stream belongs to it)
static std::map<int, SolveCtx*> g_solve;
static std::mutex g_solve_mu;
static int solve_ctx(SolveCtx** out) {
  std::lock_guard<std::mutex> lk(g_solve_mu);
  int nd = 0;
  if (cudaGetDeviceCount(&nd) != cudaSuccess || nd == 0) return fail(MFBEM_ECUDA, "no CUDA device");
  const int dev = cur_dev();
  auto it = g_solve.find(dev);
  if (it == g_solve.end()) {
    int rc = init_tables();
    if (rc) return rc;
    SolveCtx* c = new SolveCtx();
    CK(cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking));
    it = g_solve.emplace(dev, c).first;
  }
  *out = it->second;
  return 0;
}

// Pivots handed back by a caller (factorize = 0) must be what getrf leaves:
// 1-based, row j interchanged with ipiv(j) in [j, n]; any other value would
// make the row interchanges of the solve read and write outside the vectors.
static int check_ipiv(int32_t n, const int32_t* ipiv) {
  for (int32_t j = 0; j < n; ++j)
    if (ipiv[j] < j + 1 || ipiv[j] > n)
      return fail(MFBEM_EARG, "ipiv(" + std::to_string(j + 1) + ") = " + std::to_string(ipiv[j]) +
                                  " is not a pivot of getrf (must lie in [" + std::to_string(j + 1) + ", n])");
  return 0;
}

template <typename S>
static int solve_dropin(int32_t n, double* A, int32_t* ipiv, int32_t aodim, double* Ao, char* equed, double* r,
                        double* c, int32_t n_rhs, double* b, int32_t factorize, int32_t scaling, int32_t condition,
                        int32_t refine) {
  g_err.clear();
  g_lse = LseReport();
  if (n <= 0 || !A || !ipiv || n_rhs < 0 || (n_rhs > 0 && !b)) return fail(MFBEM_EARG, "invalid argument");
  // src/solve_lse_r.f90:70-78: Ao is used only with condition or refine, and then its dimension must be n
  if ((condition || refine) && (aodim != n || !Ao)) return fail(MFBEM_EARG, "invalid value of Aodim");
  if (scaling && (!equed || !r || !c)) return fail(MFBEM_EARG, "scaling needs equed, r and c");
  if (scaling && !factorize && *equed != 'N' && *equed != 'R' && *equed != 'C' && *equed != 'B')
    return fail(MFBEM_EARG, "invalid value of equed");
  if (!factorize && check_ipiv(n, ipiv)) return MFBEM_EARG;
  SolveCtx* cx;
  int rc = solve_ctx(&cx);
  if (rc) return rc;
  std::lock_guard<std::mutex> lk(g_solve_mu);
  const size_t es = sizeof(S), nn = (size_t)n * n, nr = (size_t)std::max(1, n_rhs);
  const bool keep_ao = condition || refine;
  // vector work: x, v, R, y (n S each), r, c, wts (n doubles), part (64 n),
  // bits (n u64), isgn (n ints), scalars
  const size_t wbytes = 4 * n * es + (3 + 64) * (size_t)n * 8 + (size_t)n * 8 + (size_t)n * 4 + 256;
  if ((rc = ensure(cx->A, nn * es)) || (rc = ensure(cx->b, (size_t)n * nr * es)) ||
      (rc = ensure(cx->ipiv, sizeof(int) * n)) || (rc = ensure(cx->info, sizeof(int) * 4)) ||
      (rc = ensure(cx->wv, wbytes)) || (keep_ao && (rc = ensure(cx->Ao, nn * es))) ||
      (refine && (rc = ensure(cx->bc, (size_t)n * nr * es))))
    return rc;
  cudaStream_t st = cx->st;
  S* dA = (S*)cx->A.p;
  S* dAo = keep_ao ? (S*)cx->Ao.p : nullptr;
  int* dp = (int*)cx->ipiv.p;
  int* di = (int*)cx->info.p;
  char* wp = (char*)cx->wv.p;
  S* vx = (S*)wp; S* vv = vx + n; S* vR = vv + n; S* vy = vR + n;
  double* dr = (double*)(vy + n);
  double* dc = dr + n;
  double* wts = dc + n;
  double* part = wts + n;
  unsigned long long* bits = (unsigned long long*)(part + 64 * (size_t)n);
  int* isgn = (int*)(bits + n);
  double* red = (double*)(((uintptr_t)(isgn + n) + 63) / 64 * 64);
  LseWork w{st, red, di + 2};
  if ((rc = trsv_err_reset(st))) return rc;
  CK(cudaMemcpyAsync(dA, A, nn * es, cudaMemcpyHostToDevice, st));
  char eq = scaling ? *equed : 'N';
  if (factorize) {
    if (scaling) {
      int einfo = 0;
      if ((rc = equilibrate<S>(w, dA, n, dr, dc, bits, &einfo, &eq))) return rc;
      if (einfo) return fail(einfo, "scaling has failed: ?geequ info " + std::to_string(einfo));
      CK(cudaMemcpyAsync(r, dr, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
      CK(cudaMemcpyAsync(c, dc, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
      *equed = eq;
    }
    if (keep_ao) {
      CK(cudaMemcpyAsync(dAo, dA, nn * es, cudaMemcpyDeviceToDevice, st));
      CK(cudaMemcpyAsync(Ao, dAo, nn * es, cudaMemcpyDeviceToHost, st));
    }
    if ((rc = getrf_batched<S>(st, dA, 0, n, n, 1, dp, di))) return rc;
    int info = 0;
    CK(cudaMemcpyAsync(A, dA, nn * es, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(ipiv, dp, sizeof(int) * n, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(&info, di, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (info > 0) return fail(info, "singular matrix: zero pivot U(info,info)");
  } else {
    CK(cudaMemcpyAsync(dp, ipiv, sizeof(int) * n, cudaMemcpyHostToDevice, st));
    if (scaling) {
      CK(cudaMemcpyAsync(dr, r, sizeof(double) * n, cudaMemcpyHostToDevice, st));
      CK(cudaMemcpyAsync(dc, c, sizeof(double) * n, cudaMemcpyHostToDevice, st));
    }
    if (refine) CK(cudaMemcpyAsync(dAo, Ao, nn * es, cudaMemcpyHostToDevice, st));
  }
  if (condition && factorize) {
    double rcond = 0.0;
    if ((rc = gecon1<S>(w, dAo, dA, n, vx, vv, isgn, bits, &rcond))) return rc;
    g_lse.rcond = rcond;
  }
  if (n_rhs > 0) {
    S* db = (S*)cx->b.p;
    CK(cudaMemcpyAsync(db, b, (size_t)n * n_rhs * es, cudaMemcpyHostToDevice, st));
    if (scaling && (eq == 'R' || eq == 'B')) {
      k_rows_scale<S><<<152 * 4, 256, 0, st>>>(db, n, n_rhs, dr); ++g_launches;
    }
    S* dbc = refine ? (S*)cx->bc.p : nullptr;
    if (refine) CK(cudaMemcpyAsync(dbc, db, (size_t)n * n_rhs * es, cudaMemcpyDeviceToDevice, st));
    if ((rc = getrs_batched<S>(st, dA, 0, n, n, dp, 0, db, n, n_rhs))) return rc;
    if (refine) {
      g_lse.ferr.assign(n_rhs, 0.0);
      g_lse.berr.assign(n_rhs, 0.0);
      for (int j = 0; j < n_rhs; ++j)
        if ((rc = gerfs1<S>(w, dAo, dA, dp, n, dbc + (size_t)j * n, db + (size_t)j * n, vR, vy, vv, isgn, wts, part,
                            &g_lse.ferr[j], &g_lse.berr[j])))
          return rc;
    }
    if (scaling && (eq == 'C' || eq == 'B')) {
      k_rows_scale<S><<<152 * 4, 256, 0, st>>>(db, n, n_rhs, dc); ++g_launches;
    }
    CK(cudaMemcpyAsync(b, db, (size_t)n * n_rhs * es, cudaMemcpyDeviceToHost, st));
  }
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(st));
  return trsv_err_check(st);
}

extern "C" int mfbem_solve_r(int32_t n, double* A, int32_t* ipiv, int32_t aodim, double* Ao, char* equed, double* r,
                             double* c, int32_t n_rhs, double* b, int32_t factorize, int32_t scaling,
                             int32_t condition, int32_t refine) {
  return solve_dropin<double>(n, A, ipiv, aodim, Ao, equed, r, c, n_rhs, b, factorize, scaling, condition, refine);
}
extern "C" int mfbem_solve_c(int32_t n, double* A, int32_t* ipiv, int32_t aodim, double* Ao, char* equed, double* r,
                             double* c, int32_t n_rhs, double* b, int32_t factorize, int32_t scaling,
                             int32_t condition, int32_t refine) {
  return solve_dropin<double2>(n, A, ipiv, aodim, Ao, equed, r, c, n_rhs, b, factorize, scaling, condition, refine);
}
extern "C" int mfbem_solve_report(double* rcond, int32_t n_rhs, double* ferr, double* berr) {
  if (rcond) *rcond = g_lse.rcond;
  for (int j = 0; j < n_rhs; ++j) {
    if (ferr) ferr[j] = j < (int)g_lse.ferr.size() ? g_lse.ferr[j] : NAN;
    if (berr) berr[j] = j < (int)g_lse.berr.size() ? g_lse.berr[j] : NAN;
  }
  return 0;
}

}  // namespace mfb
