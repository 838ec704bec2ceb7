// Dense solves behind mfbem_solve_{r,c}, mfbem_sweep_harela and
// mfbem_solve_staela (included into mfbem_abi.cu).
#pragma once

// The dynamic shared-memory limit is a process-wide attribute of a kernel:
// raise it once to the device's opt-in maximum (a per-call value would race
// between concurrent sweeps with different sizes).
static int raise_smem_limit(const void* f) {
  static std::mutex mu;
  static std::vector<const void*> done;
  std::lock_guard<std::mutex> lk(mu);
  for (const void* d : done)
    if (d == f) return 0;
  int dev = 0, mx = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&mx, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  cudaFuncAttributes fa;
  cudaFuncGetAttributes(&fa, f);
  const int lim = mx - (int)fa.sharedSizeBytes;
  if (cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, lim) != cudaSuccess) {
    cudaGetLastError();
    return -1;
  }
  done.push_back(f);
  return 0;
}

// ---------------------------------------------------------------------------
// GEMM dispatch for the trailing update A22 -= L21 U12 (plain library GEMM)
// ---------------------------------------------------------------------------
// ipiv[b][j] = j + 1
__global__ void k_ipiv_identity(int* ipiv, int n) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < n) ipiv[(size_t)n * blockIdx.y + j] = j + 1;
}

// Compute type of the single-precision trailing updates of the mixed LU:
// 0 SIMT FP32 (k_gemm_simt), 1 tcgen05 TF32, one pass (TF32-accurate factors;
// refinement in FP64 restores the accuracy and escalates to SIMT FP32 when it
// stalls), 3 tcgen05 3xTF32 (FP32-accurate factors at tensor-core speed).
// The tensor-core kernels take the complex updates (tc_min_depth below); the
// real ones run on SIMT FP32.
// Default 3; MFBEM_FP32_GEMM=simt|tf32|tc3 overrides.
static thread_local int g_c32_mode = 3;
static int c32_default() {
  const char* e = getenv("MFBEM_FP32_GEMM");
  const std::string v = e ? e : "tc3";
  return v == "simt" ? 0 : (v == "tf32" ? 1 : 3);
}
// modes 1 and 3: the tcgen05 kernels (mfbem_tc.cuh) for the complex trailing
// updates; their timeout flag and pre-split operand tiles, per host thread
static thread_local DevBuf g_tc_err, g_tc_ws;

// C -= A B (complex64, batched): split A and B into pre-tiled hi / lo TF32
// words once, then the bulk-copy / tcgen05 pipeline per 128 x 128 tile of C~.
static int tc_cgemm_run(cudaStream_t st, const float2* A, int lda, long long sA, const float2* B, int ldb,
                        long long sB, float2* C, int ldc, long long sC, int m, int n, int k, int batch, DevBuf& ws,
                        int* err, int passes = 3) {
  const int nmt = (m + TC_BM / 2 - 1) / (TC_BM / 2), nnt = (n + TC_BN - 1) / TC_BN, nkc = (k + TQ / 2 - 1) / (TQ / 2);
  if (nmt == 0 || nnt == 0 || nkc == 0) return 0;
  const size_t wa = (size_t)batch * nmt * nkc * TQ_TW, wb = (size_t)batch * nnt * nkc * TQ_TW;
  int rc = ensure(ws, sizeof(uint32_t) * 2 * (wa + wb));
  if (rc) return rc;
  // column tiles of 256 (M 128 x N 256 MMAs, two CTAs per SM) unless the
  // update is narrower; MFBEM_TC_BN=128 selects the 128-column tiles
  static const int bn_env = [] {
    const char* e = getenv("MFBEM_TC_BN");
    return e ? atoi(e) : 256;
  }();
  const bool wide = bn_env != 128 && nnt > 1;
  if (raise_smem_limit(wide ? (const void*)k_tc_cgemm_bulk<2> : (const void*)k_tc_cgemm_bulk<1>))
    return fail(MFBEM_ECUDA, "shared-memory limit of the tcgen05 GEMM");
  uint32_t* ahi = (uint32_t*)ws.p;
  uint32_t* alo = ahi + wa;
  uint32_t* bhi = alo + wa;
  uint32_t* blo = bhi + wb;
  // one block per tile (wa / TQ_TW and wb / TQ_TW tiles)
  k_tc_prep_a<<<(unsigned)(wa / TQ_TW), 256, 0, st>>>(A, lda, sA, m, k, nmt, nkc, batch, ahi, alo);
  ++g_launches;
  k_tc_prep_b<<<(unsigned)(wb / TQ_TW), 256, 0, st>>>(B, ldb, sB, k, n, nnt, nkc, batch, bhi, blo);
  ++g_launches;
  if (wide)
    k_tc_cgemm_bulk<2><<<dim3(nmt, (nnt + 1) / 2, batch), 128, tc_smem_bulk<2>(), st>>>(
        ahi, alo, bhi, blo, nmt, nnt, nkc, C, ldc, sC, m, n, err, g_spin_limit.load(), passes);
  else
    k_tc_cgemm_bulk<1><<<dim3(nmt, nnt, batch), 128, tc_smem_bulk<1>(), st>>>(ahi, alo, bhi, blo, nmt, nnt, nkc, C, ldc,
                                                                           sC, m, n, err, g_spin_limit.load(), passes);
  ++g_launches;
  CK(cudaGetLastError());
  return 0;
}

// SIMT update C -= A B (any of the four scalar types, batched): a 64 x 64
// tile of C per 256-thread CTA, 4 x 4 outputs per thread, K staged in shared
// memory 16 at a time; accumulation in the scalar's own precision (binary64
// FMA on the FP64 pipe for double / double2).
__device__ __forceinline__ double2 zfma(double2 a, double2 b, double2 c) {
  return make_double2(fma(a.x, b.x, fma(-a.y, b.y, c.x)), fma(a.x, b.y, fma(a.y, b.x, c.y)));
}
__device__ __forceinline__ double zfma(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float2 zfma(float2 a, float2 b, float2 c) {
  return make_float2(fmaf(a.x, b.x, fmaf(-a.y, b.y, c.x)), fmaf(a.x, b.y, fmaf(a.y, b.x, c.y)));
}
__device__ __forceinline__ float zfma(float a, float b, float c) { return fmaf(a, b, c); }
template <typename S>
__global__ void __launch_bounds__(256) k_gemm_simt(const S* A, int lda, long long sA, const S* B, int ldb,
                                                   long long sB, S* C, int ldc, long long sC, int m, int n, int k) {
  __shared__ S As[16][64 + 1];
  __shared__ S Bs[16][64 + 1];
  const int b = blockIdx.z, tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  const int i0 = blockIdx.x * 64, j0 = blockIdx.y * 64;
  const S* Ab = A + sA * b;
  const S* Bb = B + sB * b;
  S acc[4][4];
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) acc[u][v] = Sc<S>::zero();
  for (int l0 = 0; l0 < k; l0 += 16) {
    for (int q = threadIdx.x; q < 16 * 64; q += 256) {
      const int ii = q % 64, ll = q / 64;
      As[ll][ii] = (i0 + ii < m && l0 + ll < k) ? Ab[(size_t)(l0 + ll) * lda + i0 + ii] : Sc<S>::zero();
      const int jj = q / 16, lb = q % 16;
      Bs[lb][jj] = (j0 + jj < n && l0 + lb < k) ? Bb[(size_t)(j0 + jj) * ldb + l0 + lb] : Sc<S>::zero();
    }
    __syncthreads();
#pragma unroll 4
    for (int ll = 0; ll < 16; ++ll) {
      S a[4], bv[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) a[u] = As[ll][tx + 16 * u];
#pragma unroll
      for (int v = 0; v < 4; ++v) bv[v] = Bs[ll][ty + 16 * v];
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) acc[u][v] = zfma(a[u], bv[v], acc[u][v]);
    }
    __syncthreads();
  }
  S* Cb = C + sC * b;
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int i = i0 + tx + 16 * u, j = j0 + ty + 16 * v;
      if (i < m && j < n) Cb[(size_t)j * ldc + i] = Sc<S>::sub(Cb[(size_t)j * ldc + i], acc[u][v]);
    }
}
template <typename S>
static int gemm_simt(cudaStream_t st, int m, int n, int k, const S* A, int lda, long long sA, const S* B, int ldb,
                     long long sB, S* C, int ldc, long long sC, int batch) {
  if (m <= 0 || n <= 0 || k <= 0) return 0;
  k_gemm_simt<S><<<dim3(nblk(m, 64), nblk(n, 64), batch), 256, 0, st>>>(A, lda, sA, B, ldb, sB, C, ldc, sC, m, n, k);
  ++g_launches;
  CK(cudaGetLastError());
  return 0;
}
// ---------------------------------------------------------------------------
// FP64 trailing updates C -= A B of the plain LU (batched, column-major):
// mode 0 (default) the FP64-accurate Ozaki-scheme kernels on the bf16 tensor
// cores (mfbem_oz.cuh); mode 1 this library's binary64 SIMT kernel
// (k_dgemm_simt, FMA on the FP64 pipe). MFBEM_FP64_GEMM=oz|dfma overrides.
// ---------------------------------------------------------------------------
static int f64_default() {
  const char* e = getenv("MFBEM_FP64_GEMM");
  return (e && std::string(e) == "dfma") ? 1 : 0;
}
static thread_local DevBuf g_oz_ws, g_oz_err;

template <bool CPLX>
static int oz_gemm_run(cudaStream_t st, const typename OzT<CPLX>::S* A, int lda, long long sA,
                       const typename OzT<CPLX>::S* B, int ldb, long long sB, typename OzT<CPLX>::S* C, int ldc,
                       long long sC, int m, int n, int k, int batch) {
  typedef typename OzT<CPLX>::S S;
  if (m <= 0 || n <= 0 || k <= 0 || batch <= 0) return 0;
  constexpr int W = CPLX ? 2 : 1;  // real K per complex K
  const int kmax = OZ_MAXK / W;
  if (k > kmax) {  // exactness bound of the level accumulators: split K
    for (int k0 = 0; k0 < k; k0 += kmax) {
      const int kk = std::min(kmax, k - k0);
      int rc = oz_gemm_run<CPLX>(st, A + (size_t)k0 * lda, lda, sA, B + k0, ldb, sB, C, ldc, sC, m, n, kk, batch);
      if (rc) return rc;
    }
    return 0;
  }
  const int mr = W * m, Kr = W * k;
  const int nmt = (mr + OZ_BM - 1) / OZ_BM, nnt = (n + OZ_BN - 1) / OZ_BN, nkc = (Kr + OZ_KC - 1) / OZ_KC;
  const size_t wa = (size_t)batch * nmt * nkc * OZ_S * OZ_TWA, wb = (size_t)batch * nnt * nkc * OZ_S * OZ_TWB;
  const size_t ne = (size_t)batch * nmt * OZ_BM, nf = (size_t)batch * nnt * OZ_BN;
  int rc = ensure(g_oz_ws, sizeof(uint32_t) * (wa + wb) + sizeof(int) * (ne + nf) + 256);
  if (rc) return rc;
  if (!g_oz_err.p) return fail(MFBEM_ECUDA, "Ozaki GEMM: error flag not set up");
  if (raise_smem_limit((const void*)k_oz_gemm)) return fail(MFBEM_ECUDA, "shared-memory limit of the Ozaki GEMM");
  uint32_t* at = (uint32_t*)g_oz_ws.p;
  uint32_t* bt = at + wa;
  int* erow = (int*)(bt + wb);
  int* fcol = erow + ne;
  k_oz_split<CPLX><<<dim3(nmt + nnt, batch), 256, 0, st>>>(A, lda, sA, m, B, ldb, sB, n, k, nmt, nnt, nkc, at, erow,
                                                            bt, fcol);
  ++g_launches;
  k_oz_gemm<<<dim3(nmt, nnt, batch), 128, OZ_SMEM, st>>>(at, bt, erow, fcol, nmt, nnt, nkc, (double*)C,
                                                        (long long)W * ldc, (long long)W * sC, mr, n,
                                                        (int*)g_oz_err.p, g_spin_limit.load());
  ++g_launches;
  CK(cudaGetLastError());
  return 0;
}
// the Ozaki kernels' timeout flag: zeroed before a factorisation, read after it
static int oz_err_reset(cudaStream_t st) {
  int rc = ensure(g_oz_err, sizeof(int));
  if (rc) return rc;
  CK(cudaMemsetAsync(g_oz_err.p, 0, sizeof(int), st));
  return 0;
}
static int oz_err_check(cudaStream_t st) {
  int e = 0;
  CK(cudaMemcpyAsync(&e, g_oz_err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  if (e) return fail(MFBEM_ETIMEOUT, "FP64 trailing update: a tensor-core completion wait timed out");
  return 0;
}

// Below this many real multiply-adds an update goes to the binary64 SIMT
// kernel even in mode 0: the Ozaki path's fixed cost (operand split, TMEM
// allocation, binary64 epilogue; about 30-40 µs) exceeds the SIMT kernel's
// time there (small static systems, the depth-16 updates inside an outer block).
constexpr double kOzMinMacs = 16777216.0;  // 2^24
// smallest update depth taken by the Ozaki scheme (MFBEM_OZ_MIN_K; 0, the
// default: any depth above the size threshold). Sending the depth-16 and
// depth-32 updates to the binary64 SIMT kernel instead made the plain
// factorisation slower (20 cube systems 232.8 -> 317 ms, the 14883-row patch
// 676 -> 795 ms at depth < 33).
static int oz_min_depth() {
  static const int v = [] {
    const char* e = getenv("MFBEM_OZ_MIN_K");
    return e ? std::max(0, atoi(e)) : 0;
  }();
  return v;
}
template <typename S>
static int f64_gemm(cudaStream_t st, int m, int n, int k, const S* A, int lda, long long sA, const S* B, int ldb,
                    long long sB, S* C, int ldc, long long sC, int batch) {
  if (m <= 0 || n <= 0 || k <= 0) return 0;
  const double macs = (double)m * n * k * batch * (std::is_same<S, double2>::value ? 4.0 : 1.0);
  if (f64_default() == 1 || macs < kOzMinMacs || k < oz_min_depth())
    return gemm_simt<S>(st, m, n, k, A, lda, sA, B, ldb, sB, C, ldc, sC, batch);
  return oz_gemm_run<std::is_same<S, double2>::value>(st, A, lda, sA, B, ldb, sB, C, ldc, sC, m, n, k, batch);
}
// smallest depth of a complex update that goes to the tensor cores: 32 (the
// updates inside an outer block too) for a batch of systems, 64 for a single
// system, whose depth-32 updates ran faster on the SIMT kernel (88.8 against
// 91.4 ms for the factorisation of one 14883-row system); MFBEM_TC_MIN_K
// overrides
static int tc_min_depth(int batch) {
  const char* e = getenv("MFBEM_TC_MIN_K");
  return e ? std::max(1, atoi(e)) : (batch > 1 ? 32 : 64);
}
// C -= A B (batched) in the scalar type of the factorisation, as configured
// above: FP64 (plain LU) or FP32 (mixed LU)
static int gemm_sb(cudaStream_t st, int m, int n, int k, const double* A, int lda, long long sA, const double* B,
                   int ldb, long long sB, double* C, int ldc, long long sC, int batch) {
  return f64_gemm<double>(st, m, n, k, A, lda, sA, B, ldb, sB, C, ldc, sC, batch);
}
static int gemm_sb(cudaStream_t st, int m, int n, int k, const double2* A, int lda, long long sA, const double2* B,
                   int ldb, long long sB, double2* C, int ldc, long long sC, int batch) {
  return f64_gemm<double2>(st, m, n, k, A, lda, sA, B, ldb, sB, C, ldc, sC, batch);
}
static int gemm_sb(cudaStream_t st, int m, int n, int k, const float* A, int lda, long long sA, const float* B,
                   int ldb, long long sB, float* C, int ldc, long long sC, int batch) {
  return gemm_simt<float>(st, m, n, k, A, lda, sA, B, ldb, sB, C, ldc, sC, batch);
}
static int gemm_sb(cudaStream_t st, int m, int n, int k, const float2* A, int lda, long long sA, const float2* B,
                   int ldb, long long sB, float2* C, int ldc, long long sC, int batch) {
  const int mode = g_c32_mode;
  if ((mode == 3 || mode == 1) && g_tc_err.p && k >= tc_min_depth(batch))
    return tc_cgemm_run(st, A, lda, sA, B, ldb, sB, C, ldc, sC, m, n, k, batch, g_tc_ws, (int*)g_tc_err.p,
                        mode == 3 ? 3 : 1);
  return gemm_simt<float2>(st, m, n, k, A, lda, sA, B, ldb, sB, C, ldc, sC, batch);
}

// ---------------------------------------------------------------------------
// TRSM of the plain LU's row panel, U12 = inv(L11) A12 with L11 the kb x kb
// unit lower block at (k, k): on the tensor cores as the FP64-accurate update
// A12 := 0 - (-inv(L11)) A12 (k_trtri_neg, k_take_zero, then the Ozaki GEMM)
// when the panel row is long; the substitution kernel k_trsm_cols otherwise.
// ---------------------------------------------------------------------------
// T[b] = -inv(L11) (column-major, ld 32): one warp per (column j, matrix),
// lane i holding x_i of column j; the forward substitution runs as kb steps
// of one multiply-add per lane (x_c broadcast by a shuffle), so each lane's
// dependent chain is kb operations long, and the columns run on separate
// SMs (binary64 arithmetic is slow on this GPU; long chains of it on one SM
// were the cost here).
template <typename S>
__global__ void __launch_bounds__(32) k_trtri_neg(const S* A, long long sA, int lda, int k, int kb, S* T) {
  const int j = blockIdx.x, b = blockIdx.y, i = threadIdx.x;
  const S* M = A + sA * b;
  S x = (i == j) ? Sc<S>::one() : Sc<S>::zero();
  for (int c = j; c < kb - 1; ++c) {
    const S xc = shfl_s(x, c);
    if (i > c && i < kb) x = Sc<S>::sub(x, Sc<S>::mul(M[(size_t)(k + c) * lda + k + i], xc));
  }
  T[1024 * (size_t)b + j * 32 + i] = Sc<S>::sub(Sc<S>::zero(), x);
}
// W[b] (kb x nc, ld kb) = A[k:k+kb, c0:c0+nc]; that block of A set to zero
template <typename S>
__global__ void k_take_zero(S* A, long long sA, int lda, int k, int kb, int c0, int nc, int batch, S* W) {
  const long long tot = (long long)batch * nc * kb;
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < tot; g += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(g % kb);
    const long long r = g / kb;
    const int c = (int)(r % nc), b = (int)(r / nc);
    S* a = A + sA * b + (size_t)(c0 + c) * lda + k + i;
    W[g] = *a;
    *a = Sc<S>::zero();
  }
}
static thread_local DevBuf g_trsm_ws;

// Row interchanges of the mixed path's FP32 factorisation: none first (the
// factors only precondition the FP64 refinement; the panel then needs no
// pivot search across CTAs), partial pivoting when a zero pivot appears or
// the refinement stalls (the handle remembers it for later solves of the
// mesh). MFBEM_PIVOT=partial|none overrides. The plain path always pivots.
static thread_local bool g_nopiv = false;
static int pivot_default() {
  const char* e = getenv("MFBEM_PIVOT");
  if (!e) return -1;
  return std::string(e) == "none" ? 1 : 0;
}

// Panel width of the binary64 factorisations: 16 below n = 8192 (measured on
// GB300: the 3462-DOF complex sweep factorises 5 % faster than with 32), 32
// above (the 14883-DOF system 4 % faster than with 16); MFBEM_PANEL_NB (8, 16
// or 32) overrides.
static int panel_nb_f64(int n) {
  const char* e = getenv("MFBEM_PANEL_NB");
  const int v = e ? atoi(e) : (n < 8192 ? 16 : 32);
  return (v == 8 || v == 16) ? v : 32;
}

template <typename S> struct IsF64 { static const bool v = false; };
template <> struct IsF64<double> { static const bool v = true; };
template <> struct IsF64<double2> { static const bool v = true; };

// Workspace of the cooperative panel (barrier counters, candidate exchange,
// error flag); per host thread, so concurrent sweeps do not share it
static thread_local DevBuf g_lu_ws, g_pn_ws;
// Concurrent sweeps (mfbem_sweep_harela_batch): a cooperative panel launch
// waits on its own CTAs only, and two of them sharing the SMs could each hold
// part of the machine; so under concurrency the panels run one at a time
// (mutex held until the panel kernel has finished).
static std::mutex g_coop_mu;
static thread_local bool g_concurrent = false;

// Plan of the cooperative panel for n x n matrices in a batch: G CTAs per
// matrix (panel rows split in G chunks held in shared memory, at most
// kCoopBytes per CTA so that two CTAs share an SM), launched in groups of
// `group` matrices whose CTAs are all co-resident. Returns false when the
// device cannot hold one matrix's CTAs at once (the caller then uses the
// per-column panel).
struct CoopPlan {
  int G = 0, group = 0;
  size_t smem = 0;
};
template <typename S>
static bool coop_plan(int n, int nb, int batch, CoopPlan* pl) {
  constexpr size_t kCoopBytes = 96 * 1024;
  int dev = 0, nsm = 0, coop = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return false;
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
  if (!coop || nsm <= 0) return false;
  const size_t es = sizeof(S);
  const int gmin = (int)(((size_t)n * nb * es + kCoopBytes - 1) / kCoopBytes);
  // about one CTA per SM in total (barrier cost grows with G), at least 64 rows each
  int G = std::max(gmin, std::min((n + 63) / 64, std::max(1, nsm / std::max(1, batch))));
  G = std::max(1, std::min(G, n));
  const int chunk = (n + G - 1) / G;
  const size_t smem = ((size_t)nb * chunk + nb) * es;
  if (raise_smem_limit((const void*)k_panel_coop<S, 256>)) return false;
  int bps = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_panel_coop<S, 256>, 256, smem) != cudaSuccess || bps < 1) {
    cudaGetLastError();
    return false;
  }
  const int cap = bps * nsm;
  if (G > cap) return false;
  pl->G = G;
  pl->group = std::max(1, std::min(batch, cap / G));
  pl->smem = smem;
  return true;
}

// Blocked right-looking getrf for a batch of n x n matrices (stride sA).
template <typename S>
static int getrf_batched(cudaStream_t st, S* A, long long sA, int lda, int n, int batch,
                         int* ipiv, int* info, int nbo = 128) {
  // panel width: the L11 block of the TRSM lives in shared memory (<= 16 KB);
  // MFBEM_PANEL_NB (8, 16 or 32) overrides for the binary64 factorisations
  const int nb = IsF64<S>::v ? panel_nb_f64(n) : 32;
  CK(cudaMemsetAsync(info, 0, sizeof(int) * batch, st));
  // pivots start as the identity: a panel that gives up on a bounded wait
  // leaves valid row indices behind for the interchanges that follow
  k_ipiv_identity<<<dim3(nblk(n, 256), batch), 256, 0, st>>>(ipiv, n); ++g_launches;
  typedef typename Sc<S>::R R;
  const bool tc = (g_c32_mode == 3 || g_c32_mode == 1) && std::is_same<S, float2>::value;
  // single precision only: the mixed path's unpivoted first attempt
  const bool nopiv = g_nopiv && !IsF64<S>::v;
  int* pn_cnt = nullptr;  // tickets of k_panel_nopiv, one per matrix
  if (nopiv) {
    int rc = ensure(g_pn_ws, sizeof(int) * batch);
    if (rc) return rc;
    pn_cnt = (int*)g_pn_ws.p;
    CK(cudaMemsetAsync(pn_cnt, 0, sizeof(int) * batch, st));
  }
  const bool oz = IsF64<S>::v && f64_default() == 0;
  if (oz) {
    int rc = oz_err_reset(st);
    if (rc) return rc;
  }
  if (tc) {
    int rc = ensure(g_tc_err, sizeof(int));
    if (rc) return rc;
    CK(cudaMemsetAsync(g_tc_err.p, 0, sizeof(int), st));
  }
  // cluster panel: 8 CTAs per matrix in a thread-block cluster when a matrix's
  // panel rows fit their shared memory (about 200 KB each)
  constexpr int GC = 8;
  auto cl_smem = [&](int rows) {
    const int ch = (rows + GC - 1) / GC;
    return ((size_t)nb * ch + 32 + 4 * 32) * sizeof(S) + 2 * sizeof(R) + 2 * sizeof(int) + 16;
  };
  bool use_cl = cl_smem(n) <= 200 * 1024 && !raise_smem_limit((const void*)k_panel_cluster<S, 256>);
  if (use_cl) {
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = GC;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(GC * batch);
    cfg.blockDim = dim3(256);
    cfg.dynamicSmemBytes = cl_smem(n);
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int ncl = 0;
    if (cudaOccupancyMaxActiveClusters(&ncl, (void*)k_panel_cluster<S, 256>, &cfg) != cudaSuccess || ncl < 1) {
      cudaGetLastError();
      use_cl = false;
    }
  }
  CoopPlan pl;
  const bool coop = !use_cl && coop_plan<S>(n, nb, batch, &pl);
  unsigned* ctr = nullptr;
  S* xrow = nullptr;
  R* xval = nullptr;
  int *xidx = nullptr, *derr = nullptr;
  if (coop) {
    const size_t nctr = (size_t)batch, nrow = (size_t)batch * 2 * (pl.G + 1) * nb, nval = (size_t)batch * 2 * pl.G;
    size_t off_row = ((nctr + 1) * sizeof(unsigned) + 255) / 256 * 256;
    size_t off_val = off_row + (nrow * sizeof(S) + 255) / 256 * 256;
    size_t off_idx = off_val + (nval * sizeof(R) + 255) / 256 * 256;
    size_t total = off_idx + nval * sizeof(int);
    int rc = ensure(g_lu_ws, total);
    if (rc) return rc;
    char* w = (char*)g_lu_ws.p;
    ctr = (unsigned*)w;
    derr = (int*)(ctr + nctr);
    xrow = (S*)(w + off_row);
    xval = (R*)(w + off_val);
    xidx = (int*)(w + off_idx);
    CK(cudaMemsetAsync(w, 0, (nctr + 1) * sizeof(unsigned), st));
  }
  // FP64 without the cooperative panel: spread the panel's rank-1 updates over
  // many SMs per column (one SM's FP64 rate would serialise the panel); FP32:
  // one CTA per matrix and panel.
  const bool multi = IsF64<S>::v;
  int G = std::max(1, std::min(64, (n / 128) * 2 / std::max(1, batch) + 1));
  // U12 of an inner panel: columns [c0, c1) of rows [k, k + kb)
  auto trsm = [&](int k, int kb, int c0, int c1) -> int {
    const int nc = c1 - c0;
    if (nc <= 0) return 0;
    if constexpr (IsF64<S>::v) {
      const double macs = (double)kb * kb * nc * batch * (std::is_same<S, double2>::value ? 4.0 : 1.0);
      if (oz && nc >= 128 && macs >= kOzMinMacs / 4 && kb >= oz_min_depth()) {
        const size_t tb = sizeof(S) * 1024 * (size_t)batch, wb = sizeof(S) * (size_t)kb * nc * batch;
        int rc = ensure(g_trsm_ws, tb + wb);
        if (rc) return rc;
        S* T = (S*)g_trsm_ws.p;
        S* W = (S*)((char*)g_trsm_ws.p + tb);
        k_trtri_neg<S><<<dim3(32, batch), 32, 0, st>>>(A, sA, lda, k, kb, T); ++g_launches;
        k_take_zero<S><<<(unsigned)std::min<long long>(nblk((long long)batch * nc * kb, 256), 152 * 16), 256, 0, st>>>(
            A, sA, lda, k, kb, c0, nc, batch, W);
        ++g_launches;
        return oz_gemm_run<std::is_same<S, double2>::value>(st, T, 32, 1024, W, kb, (long long)kb * nc,
                                                            A + k + (size_t)c0 * lda, lda, sA, kb, nc, kb, batch);
      }
    }
    k_trsm_cols<S><<<dim3(nblk(nc, trsm_cols<S>()), batch), trsm_cols<S>(), 0, st>>>(A, sA, lda, k, kb, c0, c1);
    ++g_launches;
    return 0;
  };
  // Two-level blocking: outer blocks of NBO columns are factorised with inner
  // panels of nb columns (updates restricted to the outer block), then one
  // trailing GEMM of depth NBO updates the rest of the matrix.
  const int NBO = std::max(nb, nbo);
  for (int K = 0; K < n; K += NBO) {
    const int KE = std::min(n, K + NBO);
    for (int k = K; k < KE; k += nb) {
      const int kb = std::min(nb, KE - k);
      if (nopiv) {
        const unsigned gr = std::max(1u, nblk(n - k - kb, 128));
        k_panel_nopiv<S><<<dim3(gr, batch), 128, 0, st>>>(A, sA, lda, k, kb, k + kb, n, info, pn_cnt);
        ++g_launches;
      } else if (use_cl) {
        const int chunk = (n - k + GC - 1) / GC;
        cudaLaunchConfig_t cfg = {};
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = GC;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.gridDim = dim3(GC * batch);
        cfg.blockDim = dim3(256);
        cfg.dynamicSmemBytes = cl_smem(n - k);
        cfg.stream = st;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        CK(cudaLaunchKernelEx(&cfg, k_panel_cluster<S, 256>, A, sA, lda, n, k, kb, chunk, ipiv, info));
        ++g_launches;
      } else if (coop) {
        const int chunk = (n - k + pl.G - 1) / pl.G;
        for (int b0 = 0; b0 < batch; b0 += pl.group) {
          const int nbm = std::min(pl.group, batch - b0);
          int Gp = pl.G, ck = chunk, kk = k, kbb = kb, nn_ = n, ldaa = lda, bb0 = b0;
          long long sAA = sA;
          long long spin = g_spin_limit.load();
          void* args[] = {&A, &sAA, &ldaa, &nn_, &kk, &kbb, &Gp, &ck, &bb0, &ipiv, &info, &ctr, &xrow, &xval, &xidx, &derr,
                          &spin};
          std::unique_lock<std::mutex> lk(g_coop_mu, std::defer_lock);
          if (g_concurrent) lk.lock();
          CK(cudaLaunchCooperativeKernel((const void*)k_panel_coop<S, 256>, dim3(pl.G * nbm), dim3(256), args,
                                         ((size_t)kb * chunk + kb) * sizeof(S), st));
          ++g_launches;
          if (g_concurrent) CK(cudaStreamSynchronize(st));
        }
      } else if (multi) {
        for (int j = k; j < k + kb; ++j) {
          k_pcol_pivot<S, 256><<<batch, 256, 0, st>>>(A, sA, lda, n, k, kb, j, ipiv, info); ++g_launches;
          int rows = n - j - 1;
          int g = std::max(1, std::min(G, (rows + 255) / 256));
          k_pcol_update<S, 256><<<dim3(g, batch), 256, 0, st>>>(A, sA, lda, n, k, kb, j); ++g_launches;
        }
      } else {
        k_panel_cta<S, 512><<<batch, 512, 0, st>>>(A, sA, lda, n, k, kb, ipiv, info); ++g_launches;
      }
      int nout = n - kb;
      if (nout > 0 && !nopiv) { k_laswp<S><<<dim3(nblk(nout, 128), batch), 128, 0, st>>>(A, sA, lda, n, k, kb, ipiv); ++g_launches; }
      if (k + kb < KE) {
        // inside the outer block: U12 and the update of columns [k+kb, KE)
        const int nc = KE - k - kb;
        CKG(trsm(k, kb, k + kb, KE));
        CKG(gemm_sb(st, n - k - kb, nc, kb, A + k + kb + (size_t)k * lda, lda, sA, A + k + (size_t)(k + kb) * lda, lda,
                    sA, A + (k + kb) + (size_t)(k + kb) * lda, lda, sA, batch));
      }
    }
    if (KE < n) {
      // U12 of the outer block (rows [K, KE), columns [KE, n)), blocked by nb
      const int nc = n - KE;
      for (int k = K; k < KE; k += nb) {
        const int kb = std::min(nb, KE - k);
        CKG(trsm(k, kb, KE, n));
        if (k + kb < KE)
          CKG(gemm_sb(st, KE - k - kb, nc, kb, A + k + kb + (size_t)k * lda, lda, sA, A + k + (size_t)KE * lda, lda, sA,
                      A + (k + kb) + (size_t)KE * lda, lda, sA, batch));
      }
      // trailing update of depth KE - K
      CKG(gemm_sb(st, nc, nc, KE - K, A + KE + (size_t)K * lda, lda, sA, A + K + (size_t)KE * lda, lda, sA,
                  A + KE + (size_t)KE * lda, lda, sA, batch));
    }
  }
  CK(cudaGetLastError());
  if (coop) {
    int e = 0;
    CK(cudaMemcpyAsync(&e, derr, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (e) return fail(MFBEM_ETIMEOUT, "LU panel: a barrier wait timed out");
  }
  if (oz) {
    int rc = oz_err_check(st);
    if (rc) return rc;
  }
  if (tc) {
    int e = 0;
    CK(cudaMemcpyAsync(&e, g_tc_err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (e) return fail(MFBEM_ETIMEOUT, "LU trailing update: a tensor-core completion wait timed out");
  }
  return 0;
}

// ---------------------------------------------------------------------------
// Autotuner of the mixed LU's outer block width (64, 128 or 256 columns: the
// depth of the trailing GEMMs against the number of panel steps), per scalar
// type, size class (n rounded up to 512), batch and GEMM compute type. The
// first factorisation of a class times the candidates on a seeded random
// batch of that size (partial pivoting; the operation count is what is timed)
// and caches the fastest.
// MFBEM_AUTOTUNE=0 keeps 128.
// ---------------------------------------------------------------------------
template <typename S> __device__ __forceinline__ S rnd_val(unsigned long long h);
template <> __device__ __forceinline__ float rnd_val<float>(unsigned long long h) {
  return (float)((h >> 40) & 0xFFFFFF) / 16777216.0f - 0.5f;
}
template <> __device__ __forceinline__ float2 rnd_val<float2>(unsigned long long h) {
  return make_float2((float)((h >> 40) & 0xFFFFFF) / 16777216.0f - 0.5f, (float)((h >> 8) & 0xFFFFFF) / 16777216.0f - 0.5f);
}
template <typename S>
__global__ void k_tune_fill(S* A, long long total) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
    unsigned long long z = (unsigned long long)i * 0x9E3779B97F4A7C15ULL + 0x632BE59BD9B4E019ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    z ^= z >> 31;
    A[i] = rnd_val<S>(z);
  }
}
static std::mutex g_tune_mu;
static std::map<std::tuple<int, int, int, int>, int> g_tune;
template <typename S>
static int tuned_nbo(cudaStream_t st, int n, int batch, int* ipiv, int* info, int* out) {
  *out = 128;
  const char* e = getenv("MFBEM_AUTOTUNE");
  if (e && std::string(e) == "0") return 0;
  const auto key = std::make_tuple((int)sizeof(S), (n + 511) / 512, batch, g_c32_mode * 2 + (g_nopiv ? 1 : 0));
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune.find(key);
    if (it != g_tune.end()) { *out = it->second; return 0; }
  }
  const long long nn = (long long)n * n;
  S* T = nullptr;
  if (cudaMalloc(&T, sizeof(S) * nn * batch) != cudaSuccess) {
    cudaGetLastError();
    return 0;  // no room to tune: keep the default
  }
  cudaEvent_t t0, t1;
  cudaEventCreate(&t0);
  cudaEventCreate(&t1);
  const int cand[3] = {64, 128, 256};
  float best = 1e30f;
  int bn = 128, rc = 0;
  for (int c = 0; c < 3 && !rc; ++c) {
    k_tune_fill<S><<<152 * 8, 256, 0, st>>>(T, nn * batch); ++g_launches;
    cudaEventRecord(t0, st);
    rc = getrf_batched<S>(st, T, nn, n, n, batch, ipiv, info, cand[c]);
    cudaEventRecord(t1, st);
    cudaEventSynchronize(t1);
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, t0, t1);
    if (!rc && ms < best) { best = ms; bn = cand[c]; }
  }
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  cudaFree(T);
  if (rc) return rc;
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune[key] = bn;
  *out = bn;
  return 0;
}

// getrs (no transpose) for one right-hand side per batch entry.
// A: batch stride sA (0 = shared factors), ipiv stride sP, b stride sb.
template <typename S>
__global__ void k_rhs_swap2(S* b, long long sb, int n, const int* ipiv, long long sP, int nbatch) {
  int bi = blockIdx.x * blockDim.x + threadIdx.x;
  if (bi >= nbatch) return;
  S* x = b + sb * bi;
  const int* piv = ipiv + sP * bi;
  for (int j = 0; j < n; ++j) {
    int p = piv[j] - 1;
    if (p != j) {
      S t = x[j];
      x[j] = x[p];
      x[p] = t;
    }
  }
}
// The row interchanges of getrs as one permutation: a single thread per
// matrix replays the n swaps on an index array in shared memory, then the
// right-hand sides are gathered in parallel.
__global__ void k_perm(const int* ipiv, long long sP, int n, int* perm) {
  extern __shared__ int pm[];
  const int bi = blockIdx.x;
  const int* piv = ipiv + sP * bi;
  for (int i = threadIdx.x; i < n; i += blockDim.x) pm[i] = i;
  __syncthreads();
  if (threadIdx.x == 0)
    for (int j = 0; j < n; ++j) {
      const int p = piv[j] - 1;
      if (p != j) {
        const int t = pm[j];
        pm[j] = pm[p];
        pm[p] = t;
      }
    }
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) perm[(size_t)n * bi + i] = pm[i];
}
template <typename S>
__global__ void k_gather_perm(const S* x, long long sx, const int* perm, int n, S* out) {
  const int bi = blockIdx.y, i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  out[(size_t)n * bi + i] = x[sx * bi + perm[(size_t)n * bi + i]];
}
template <typename S>
__global__ void k_scatter_back(const S* tmp, int n, S* x, long long sx) {
  const int bi = blockIdx.y, i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  x[sx * bi + i] = tmp[(size_t)n * bi + i];
}
static thread_local DevBuf g_rs_ws, g_sf_ws, g_sf_err;
// triangular solves of getrs: one launch per triangle (default) or one pair of
// launches per 64-row block (MFBEM_TRSV=blocked)
static bool trsv_sync_free() {
  const char* e = getenv("MFBEM_TRSV");
  return !(e && std::string(e) == "blocked");
}
// the timeout flag of the one-launch triangular solves: zeroed before a
// solve (all its getrs calls), read after it
static int trsv_err_reset(cudaStream_t st) {
  int rc = ensure(g_sf_err, sizeof(int));
  if (rc) return rc;
  CK(cudaMemsetAsync(g_sf_err.p, 0, sizeof(int), st));
  return 0;
}
static int trsv_err_check(cudaStream_t st) {
  int e = 0;
  CK(cudaMemcpyAsync(&e, g_sf_err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  if (e) return fail(MFBEM_ETIMEOUT, "triangular solve: a wait on a solved block timed out");
  return 0;
}

// no_interchanges: the factors come from the unpivoted factorisation (ipiv is
// the identity), so the permutation step is skipped
template <typename S>
static int getrs_batched(cudaStream_t st, const S* A, long long sA, int lda, int n, const int* ipiv, long long sP,
                         S* b, long long sb, int batch, bool no_interchanges = false) {
  // diagonal blocks of TB rows solved by one warp (k_trsv_diag64), the rows
  // below / above updated by a GEMV over the solved block
  const int TB = 64;
  const size_t dsm = (size_t)TB * 65 * sizeof(S);
  if (raise_smem_limit((const void*)k_trsv_diag64<S, true>) || raise_smem_limit((const void*)k_trsv_diag64<S, false>))
    return fail(MFBEM_ECUDA, "shared-memory limit of the triangular solve");
  const size_t psm = (size_t)n * sizeof(int);
  bool gathered = no_interchanges;
  if (!gathered && psm <= 200 * 1024) {
    int rc = ensure(g_rs_ws, (size_t)batch * n * (sizeof(int) + sizeof(S)) + 256);
    if (rc) return rc;
    if (psm > 48 * 1024 && raise_smem_limit((const void*)k_perm)) return fail(MFBEM_ECUDA, "shared-memory limit of the row permutation");
    int* perm = (int*)g_rs_ws.p;
    S* tmp = (S*)((char*)g_rs_ws.p + ((size_t)batch * n * sizeof(int) + 255) / 256 * 256);
    k_perm<<<batch, 256, psm, st>>>(ipiv, sP, n, perm); ++g_launches;
    k_gather_perm<S><<<dim3(nblk(n, 256), batch), 256, 0, st>>>(b, sb, perm, n, tmp); ++g_launches;
    k_scatter_back<S><<<dim3(nblk(n, 256), batch), 256, 0, st>>>(tmp, n, b, sb); ++g_launches;
    gathered = true;
  }
  if (!gathered) { k_rhs_swap2<S><<<nblk(batch, 64), 64, 0, st>>>(b, sb, n, ipiv, sP, batch); ++g_launches; }
  if (trsv_sync_free()) {
    // one launch per triangle (k_trsv_sf): ready flags [batch][nb] and a counter
    const int nb = (n + 63) / 64;
    int rc = ensure(g_sf_ws, sizeof(int) * ((size_t)batch * nb + 1));
    if (rc) return rc;
    if (!g_sf_err.p) return fail(MFBEM_ECUDA, "triangular solve: error flag not set up");
    int* ready = (int*)g_sf_ws.p;
    unsigned* ctr = (unsigned*)(ready + (size_t)batch * nb);
    int* err = (int*)g_sf_err.p;
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const unsigned g = (unsigned)std::max(1, std::min(batch * nb, 2 * nsm));
    constexpr size_t smem = trsv_sf_smem<S>();
    if (raise_smem_limit((const void*)k_trsv_sf<S, true>) || raise_smem_limit((const void*)k_trsv_sf<S, false>))
      return fail(MFBEM_ECUDA, "shared-memory limit of the triangular solve");
    CK(cudaMemsetAsync(g_sf_ws.p, 0, sizeof(int) * ((size_t)batch * nb + 1), st));
    k_trsv_sf<S, true><<<g, 256, smem, st>>>(A, sA, lda, n, b, sb, batch, nb, ctr, ready, err, g_spin_limit.load());
    ++g_launches;
    CK(cudaMemsetAsync(g_sf_ws.p, 0, sizeof(int) * ((size_t)batch * nb + 1), st));
    k_trsv_sf<S, false><<<g, 256, smem, st>>>(A, sA, lda, n, b, sb, batch, nb, ctr, ready, err, g_spin_limit.load());
    ++g_launches;
    CK(cudaGetLastError());
    return 0;
  }
  for (int r0 = 0; r0 < n; r0 += TB) {
    int w = std::min(TB, n - r0);
    k_trsv_diag64<S, true><<<batch, 128, dsm, st>>>(A, sA, lda, b, sb, r0, w); ++g_launches;
    if (r0 + w < n) { k_trsv_update<S><<<dim3(nblk(n - r0 - w, 256), batch), 256, 0, st>>>(A, sA, lda, b, sb, r0, w, r0 + w, n); ++g_launches; }
  }
  int last = ((n - 1) / TB) * TB;
  for (int r0 = last; r0 >= 0; r0 -= TB) {
    int w = std::min(TB, n - r0);
    k_trsv_diag64<S, false><<<batch, 128, dsm, st>>>(A, sA, lda, b, sb, r0, w); ++g_launches;
    if (r0 > 0) { k_trsv_update<S><<<dim3(nblk(r0, 256), batch), 256, 0, st>>>(A, sA, lda, b, sb, r0, w, 0, r0); ++g_launches; }
  }
  CK(cudaGetLastError());
  return 0;
}


// ---------------------------------------------------------------------------
// Mixed precision: FP32 factors + FP64 iterative refinement on the FP64 system.
// ---------------------------------------------------------------------------
template <typename SD, typename SF>
__global__ void k_demote(const SD* a, SF* out, long long n);
template <>
__global__ void k_demote<double2, float2>(const double2* a, float2* out, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    out[i] = make_float2((float)a[i].x, (float)a[i].y);
}
template <>
__global__ void k_demote<double, float>(const double* a, float* out, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    out[i] = (float)a[i];
}
__device__ __forceinline__ double amag(double a) { return fabs(a); }
__device__ __forceinline__ double amag(double2 a) { return hypot(a.x, a.y); }
__device__ __forceinline__ double amag(float a) { return fabsf(a); }
__device__ __forceinline__ double amag(float2 a) { return hypotf(a.x, a.y); }

// FP32 copy of the FP64 systems and their row sums of |a_ij| (for the
// infinity norm), in one pass: a CTA covers 256 rows x 128 columns, coalesced
// along the rows; the moduli are taken in binary32 (the norm only scales the
// stopping test) and the partial sums are added atomically.
template <typename SD, typename SF>
__global__ void __launch_bounds__(256) k_demote_rowabs(const SD* A, SF* A32, long long sA, int lda, int n, double* rows);
template <>
__global__ void __launch_bounds__(256) k_demote_rowabs<double2, float2>(const double2* A, float2* A32, long long sA,
                                                                        int lda, int n, double* rows) {
  const int b = blockIdx.z, i = blockIdx.x * 256 + threadIdx.x;
  if (i >= n) return;
  const int j0 = blockIdx.y * 128, j1 = min(n, j0 + 128);
  const double2* M = A + sA * b;
  float2* M32 = A32 + sA * b;
  float s = 0.0f;
  for (int j = j0; j < j1; ++j) {
    const double2 v = M[(size_t)j * lda + i];
    const float2 f = make_float2((float)v.x, (float)v.y);
    M32[(size_t)j * lda + i] = f;
    s += hypotf(f.x, f.y);
  }
  atomicAdd(rows + (size_t)n * b + i, (double)s);
}
template <>
__global__ void __launch_bounds__(256) k_demote_rowabs<double, float>(const double* A, float* A32, long long sA,
                                                                      int lda, int n, double* rows) {
  const int b = blockIdx.z, i = blockIdx.x * 256 + threadIdx.x;
  if (i >= n) return;
  const int j0 = blockIdx.y * 128, j1 = min(n, j0 + 128);
  const double* M = A + sA * b;
  float* M32 = A32 + sA * b;
  float s = 0.0f;
  for (int j = j0; j < j1; ++j) {
    const float f = (float)M[(size_t)j * lda + i];
    M32[(size_t)j * lda + i] = f;
    s += fabsf(f);
  }
  atomicAdd(rows + (size_t)n * b + i, (double)s);
}

// infinity norm of each batch's matrix: row sums of |a_ij|, then max
template <typename S>
__global__ void k_rowabs(const S* A, long long sA, int lda, int n, double* rows) {
  int b = blockIdx.y;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const S* M = A + sA * b;
  double s = 0.0;
  for (int j = 0; j < n; ++j) s += amag(M[(size_t)j * lda + i]);
  rows[(size_t)n * b + i] = s;
}
template <typename S>
__global__ void k_vecmax(const S* v, long long sv, int n, double* out, int slot, int nslots) {
  int b = blockIdx.x;
  const S* x = v + sv * b;
  double m = 0.0;
  // the maximum propagates NaN (fmax would drop it and hide a diverged vector)
  auto mx = [](double a, double b) { return (b > a || b != b) ? b : a; };
  for (int i = threadIdx.x; i < n; i += blockDim.x) m = mx(m, amag(x[i]));
  for (int o = 16; o > 0; o >>= 1) m = mx(m, __shfl_xor_sync(0xffffffffu, m, o));
  __shared__ double sm[32];
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x / 32] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)blockDim.x / 32; ++w) m = mx(m, sm[w]);
    m = mx(m, sm[0]);
    out[(size_t)nslots * b + slot] = m;
  }
}
// scaled demotion of the residual: r32 = r / ||r||
template <typename SD, typename SF>
__global__ void k_scale_demote(const SD* r, long long sr, SF* out, long long so, int n, const double* nrm,
                               int nslots, int slot);
template <>
__global__ void k_scale_demote<double2, float2>(const double2* r, long long sr, float2* out, long long so, int n,
                                                const double* nrm, int nslots, int slot) {
  int b = blockIdx.y, i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = nrm[(size_t)nslots * b + slot];
  double inv = s > 0.0 ? 1.0 / s : 0.0;
  double2 v = r[sr * b + i];
  out[so * b + i] = make_float2((float)(v.x * inv), (float)(v.y * inv));
}
template <>
__global__ void k_scale_demote<double, float>(const double* r, long long sr, float* out, long long so, int n,
                                              const double* nrm, int nslots, int slot) {
  int b = blockIdx.y, i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = nrm[(size_t)nslots * b + slot];
  double inv = s > 0.0 ? 1.0 / s : 0.0;
  out[so * b + i] = (float)(r[sr * b + i] * inv);
}
// x += ||r|| d  (FP64 update with the FP32 correction)
template <typename SD, typename SF>
__global__ void k_update(SD* x, long long sx, const SF* d, long long sd, int n, const double* nrm, int nslots,
                         int slot, const int* active);
template <>
__global__ void k_update<double2, float2>(double2* x, long long sx, const float2* d, long long sd, int n,
                                          const double* nrm, int nslots, int slot, const int* active) {
  int b = blockIdx.y, i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || !active[b]) return;
  double s = nrm[(size_t)nslots * b + slot];
  float2 v = d[sd * b + i];
  double2 xo = x[sx * b + i];
  x[sx * b + i] = make_double2(xo.x + s * (double)v.x, xo.y + s * (double)v.y);
}
template <>
__global__ void k_update<double, float>(double* x, long long sx, const float* d, long long sd, int n,
                                        const double* nrm, int nslots, int slot, const int* active) {
  int b = blockIdx.y, i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || !active[b]) return;
  double s = nrm[(size_t)nslots * b + slot];
  x[sx * b + i] += s * (double)d[sd * b + i];
}
template <typename SD>
__global__ void k_copy_vec(const SD* a, SD* b, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    b[i] = a[i];
}

// ---------------------------------------------------------------------------
// Batched FP64 GEMV of the refinement: y = y - A x (residual, y holding b on
// entry) or y = A x, column-major n x n systems. Pass 1: per (row block of
// 256, column chunk of GV_CH, system) the partial sum over the chunk's
// columns, one thread per row (coalesced column reads, the chunk of x staged
// in shared memory, four independent FMA chains); pass 2: the partials of
// each row added in chunk order, so the result does not depend on scheduling.
// ---------------------------------------------------------------------------
constexpr int GV_CH = 256;
__device__ __forceinline__ double2 vadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double vadd(double a, double b) { return a + b; }
template <typename S>
__global__ void __launch_bounds__(256) k_gemv_part(const S* A, long long sA, int lda, int n, const S* x, long long sx,
                                                   S* part) {
  __shared__ S xs[GV_CH];
  const int b = blockIdx.z, c = blockIdx.y, i = blockIdx.x * 256 + threadIdx.x;
  const int j0 = c * GV_CH, j1 = min(n, j0 + GV_CH);
  for (int j = j0 + threadIdx.x; j < j1; j += 256) xs[j - j0] = x[sx * b + j];
  __syncthreads();
  if (i >= n) return;
  const S* M = A + sA * b + i;
  S a0 = Sc<S>::zero(), a1 = a0, a2 = a0, a3 = a0;
  int j = j0;
  for (; j + 3 < j1; j += 4) {
    a0 = zfma(M[(size_t)j * lda], xs[j - j0], a0);
    a1 = zfma(M[(size_t)(j + 1) * lda], xs[j + 1 - j0], a1);
    a2 = zfma(M[(size_t)(j + 2) * lda], xs[j + 2 - j0], a2);
    a3 = zfma(M[(size_t)(j + 3) * lda], xs[j + 3 - j0], a3);
  }
  for (; j < j1; ++j) a0 = zfma(M[(size_t)j * lda], xs[j - j0], a0);
  part[((size_t)b * gridDim.y + c) * n + i] = vadd(vadd(a0, a1), vadd(a2, a3));
}
template <typename S>
__global__ void k_gemv_sum(const S* part, int nch, int n, S* y, long long sy, int residual) {
  const int b = blockIdx.y, i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  S s = Sc<S>::zero();
  for (int c = 0; c < nch; ++c) s = vadd(s, part[((size_t)b * nch + c) * n + i]);
  y[sy * b + i] = residual ? Sc<S>::sub(y[sy * b + i], s) : s;
}
static thread_local DevBuf g_gv_ws;
template <typename S>
static int gemv_run(cudaStream_t st, int n, const S* A, int lda, long long sA, const S* x, long long sx, S* y,
                    long long sy, int batch, int residual) {
  const int nch = (n + GV_CH - 1) / GV_CH;
  int rc = ensure(g_gv_ws, sizeof(S) * (size_t)batch * nch * n);
  if (rc) return rc;
  S* part = (S*)g_gv_ws.p;
  k_gemv_part<S><<<dim3(nblk(n, 256), nch, batch), 256, 0, st>>>(A, sA, lda, n, x, sx, part); ++g_launches;
  k_gemv_sum<S><<<dim3(nblk(n, 256), batch), 256, 0, st>>>(part, nch, n, y, sy, residual); ++g_launches;
  CK(cudaGetLastError());
  return 0;
}
// r = r - A x (r holds b on entry)
template <typename S>
static int gemv_res(cudaStream_t st, int n, const S* A, int lda, long long sA, const S* x, long long sx, S* r,
                    long long sr, int batch) {
  return gemv_run<S>(st, n, A, lda, sA, x, sx, r, sr, batch, 1);
}
// y = A x
template <typename S>
static int gemv_apply(cudaStream_t st, int n, const S* A, int lda, long long sA, const S* x, long long sx, S* y,
                      long long sy, int batch) {
  return gemv_run<S>(st, n, A, lda, sA, x, sx, y, sy, batch, 0);
}

#include "mfbem_lse.cuh"

// ---------------------------------------------------------------------------
// GMRES-based iterative refinement (Carson & Higham, SIAM J. Sci. Comput. 40(2),
// 2018): each correction d solves A d = r by GMRES in FP64, left-preconditioned
// with the FP32 (or TF32-updated) LU factors, M^-1 A d = M^-1 r. Batched over
// the systems of a sweep; the small Hessenberg least-squares problems run on
// the host with Givens rotations; orthogonalisation is classical Gram-Schmidt
// applied twice.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double2 cdot_term(double2 a, double2 b) {  // conj(a) * b
  return make_double2(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ double cdot_term(double a, double b) { return a * b; }
__device__ __forceinline__ double2 add2(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double add2(double a, double b) { return a + b; }
__device__ __forceinline__ double2 shfl_dn(double2 v, int o) {
  return make_double2(__shfl_down_sync(0xffffffffu, v.x, o), __shfl_down_sync(0xffffffffu, v.y, o));
}
__device__ __forceinline__ double shfl_dn(double v, int o) { return __shfl_down_sync(0xffffffffu, v, o); }
__device__ __forceinline__ double2 zmul(double2 a, double2 b) { return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
__device__ __forceinline__ double zmul(double a, double b) { return a * b; }

// out[b][i] = V_i^H w (i < nv), V_i = V + b*sVb + i*n, w = W + b*sW
template <typename SD>
__global__ void k_bdot(const SD* V, long long sVb, int nv, const SD* W, long long sW, int n, SD* out, int ldo) {
  const int i = blockIdx.x, b = blockIdx.y;
  const SD* v = V + sVb * b + (long long)i * n;
  const SD* w = W + sW * b;
  SD acc = Sc<SD>::zero();
  for (int k = threadIdx.x; k < n; k += blockDim.x) acc = add2(acc, cdot_term(v[k], w[k]));
  for (int o = 16; o > 0; o >>= 1) acc = add2(acc, shfl_dn(acc, o));
  __shared__ SD sm[32];
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x / 32] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    SD t = sm[0];
    for (int q = 1; q < (int)blockDim.x / 32; ++q) t = add2(t, sm[q]);
    out[(size_t)ldo * b + i] = t;
  }
}
__device__ __forceinline__ double2 rscal(double2 a, double f) { return make_double2(a.x * f, a.y * f); }
__device__ __forceinline__ double rscal(double a, double f) { return a * f; }

// w[b] += sign * sum_{i<nv} V_i c[b][i]  (sign -1: Gram-Schmidt; +1: x += V y)
template <typename SD>
__global__ void k_bcomb(SD* W, long long sW, const SD* V, long long sVb, int nv, const SD* c, int ldc, int n,
                        double sign, const int* active) {
  const int b = blockIdx.y, k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n || (active && !active[b])) return;
  const SD* v = V + sVb * b + k;
  SD acc = Sc<SD>::zero();
  for (int i = 0; i < nv; ++i) acc = add2(acc, zmul(v[(long long)i * n], c[(size_t)ldc * b + i]));
  W[sW * b + k] = add2(W[sW * b + k], rscal(acc, sign));
}
// out[b] = in[b] * s[b] (s real)
template <typename SD>
__global__ void k_bscale(const SD* in, long long sIn, SD* out, long long sOut, int n, const double* s) {
  const int b = blockIdx.y, k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  out[sOut * b + k] = rscal(in[sIn * b + k], s[b]);
}
// FP64 out = nrm[b] * (FP64) in32  (promotion of a preconditioner application)
template <typename SD, typename SF>
__global__ void k_promote(const SF* in, long long sIn, SD* out, long long sOut, int n, const double* nrm, int nslots,
                          int slot);
template <>
__global__ void k_promote<double2, float2>(const float2* in, long long sIn, double2* out, long long sOut, int n,
                                           const double* nrm, int nslots, int slot) {
  const int b = blockIdx.y, k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const double s = nrm[(size_t)nslots * b + slot];
  const float2 v = in[sIn * b + k];
  out[sOut * b + k] = make_double2(s * (double)v.x, s * (double)v.y);
}
template <>
__global__ void k_promote<double, float>(const float* in, long long sIn, double* out, long long sOut, int n,
                                         const double* nrm, int nslots, int slot) {
  const int b = blockIdx.y, k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  out[sOut * b + k] = nrm[(size_t)nslots * b + slot] * (double)in[sIn * b + k];
}

// State of the mixed solve of one batch.
template <typename SD, typename SF>
struct MixCtx {
  mfbem_handle* h;
  SD* A;
  SF* A32;
  int* ipiv;
  int n, batch;
  const SD* b;
  SD *x, *r;
  SF* d32;
  double* nrm;
  int* active;
  double tol;
  int it = 0, inner = 0, refactor = 0;
  // the next residual is b itself (x = 0): at the start and after a restart
  bool fresh = true;
  double maxbe = 0.0;
  std::vector<double> be;
  // classical refinement: the estimated forward error of each system relative
  // to x (+inf before the first correction), the last correction's
  // ||d|| / ||x|| (infinity norms) and ||r|| it was scaled by
  std::vector<double> dx, dxraw, rprev;
};
// forward criterion of the classical refinement: the estimated remaining error
// is at most this fraction of x (with the backward-error test it bounds the
// forward error on ill-conditioned systems, where a small backward error alone
// does not). The estimate is the last correction's size, times rho / (1 - rho)
// once two corrections give its contraction rho = ||d_k|| / ||d_k-1|| < 1/2:
// the error left after d_k is about rho ||d_k|| (Higham, Accuracy and
// Stability of Numerical Algorithms, 2nd ed., section 12.1), so a third
// correction whose only purpose would be to show a tiny size is not needed.
constexpr double kFwdTol = 1e-10;

// r = b - A x, backward errors ||r|| / (||A|| ||x|| + ||b||) (infinity norms);
// active[b] = not yet converged. Returns whether all converged.
template <typename SD, typename SF>
static int residual_check(MixCtx<SD, SF>& c, bool first, bool* all) {
  cudaStream_t st = c.h->st;
  const int n = c.n, batch = c.batch;
  const long long nn = (long long)n * n;
  int rc;
  k_copy_vec<SD><<<nblk((long long)n * batch, 256), 256, 0, st>>>(c.b, c.r, (long long)n * batch); ++g_launches;
  if (!first && (rc = gemv_res<SD>(st, n, c.A, n, nn, c.x, n, c.r, n, batch))) return rc;
  k_vecmax<SD><<<batch, 256, 0, st>>>(c.r, n, n, c.nrm, 0, 8); ++g_launches;
  k_vecmax<SD><<<batch, 256, 0, st>>>(c.x, n, n, c.nrm, 1, 8); ++g_launches;
  std::vector<double> hn(8 * (size_t)batch);
  CK(cudaMemcpyAsync(hn.data(), c.nrm, sizeof(double) * 8 * batch, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  c.be.assign(batch, 1.0);
  if ((int)c.dx.size() != batch) c.dx.assign(batch, 1e300);
  if ((int)c.rprev.size() != batch) c.rprev.assign(batch, 0.0);
  std::vector<int> hact(batch);
  c.maxbe = 0.0;
  bool any = false;
  c.fresh = false;
  for (int bi = 0; bi < batch; ++bi) {
    double be = first ? 1.0 : hn[8 * bi + 0] / (hn[8 * bi + 3] * hn[8 * bi + 1] + hn[8 * bi + 2]);
    if (!std::isfinite(be)) be = HUGE_VAL;  // non-finite residual or x: not converged
    c.be[bi] = be;
    c.maxbe = std::max(c.maxbe, be);
    hact[bi] = (!(be <= c.tol) || c.dx[bi] > kFwdTol) ? 1 : 0;
    any = any || hact[bi];
    c.rprev[bi] = hn[8 * bi + 0];
  }
  CK(cudaMemcpyAsync(c.active, hact.data(), sizeof(int) * batch, cudaMemcpyHostToDevice, st));
  *all = !any;
  return 0;
}

// out = M^-1 u for every system (FP64 in and out, FP32 factors): scale by
// ||u||_inf, demote, getrs, promote
template <typename SD, typename SF>
static int precond(MixCtx<SD, SF>& c, const SD* u, SD* out) {
  cudaStream_t st = c.h->st;
  const int n = c.n, batch = c.batch;
  const long long nn = (long long)n * n;
  k_vecmax<SD><<<batch, 256, 0, st>>>(u, n, n, c.nrm, 4, 8); ++g_launches;
  k_scale_demote<SD, SF><<<dim3(nblk(n, 256), batch), 256, 0, st>>>(u, n, c.d32, n, n, c.nrm, 8, 4); ++g_launches;
  int rc = getrs_batched<SF>(st, c.A32, nn, n, n, c.ipiv, n, c.d32, n, batch, g_nopiv);
  if (rc) return rc;
  k_promote<SD, SF><<<dim3(nblk(n, 256), batch), 256, 0, st>>>(c.d32, n, out, n, n, c.nrm, 8, 4); ++g_launches;
  return 0;
}

// Classical refinement x += M^-1 (b - A x). *conv = 1 when every system reaches
// tol; returns early (conv 0) when the contraction per step is slower than 1/4
// twice in a row, or after 30 steps.
template <typename SD, typename SF>
static int refine_classical(MixCtx<SD, SF>& c, int* conv) {
  cudaStream_t st = c.h->st;
  const int n = c.n, batch = c.batch;
  const long long nn = (long long)n * n;
  std::vector<double> prev(batch, 1.0);
  int stall = 0;
  *conv = 0;
  for (int it = 0;; ++it) {
    bool all;
    int rc = residual_check(c, c.fresh, &all);
    if (rc) return rc;
    if (all) { *conv = 1; return 0; }
    bool slow = false;
    for (int bi = 0; bi < batch; ++bi) {
      if (c.be[bi] > c.tol && it >= 2 && c.be[bi] > 0.25 * prev[bi]) slow = true;
      if (c.be[bi] == HUGE_VAL && it >= 1) return 0;  // diverged (non-finite): give up at once
    }
    prev = c.be;
    stall = slow ? stall + 1 : 0;
    if (stall >= 2 || it >= 30) return 0;
    k_scale_demote<SD, SF><<<dim3(nblk(n, 256), batch), 256, 0, st>>>(c.r, n, c.d32, n, n, c.nrm, 8, 0); ++g_launches;
    if ((rc = getrs_batched<SF>(st, c.A32, nn, n, n, c.ipiv, n, c.d32, n, batch, g_nopiv))) return rc;
    k_update<SD, SF><<<dim3(nblk(n, 256), batch), 256, 0, st>>>(c.x, n, c.d32, n, n, c.nrm, 8, 0, c.active); ++g_launches;
    // size of this correction relative to the updated x (for the forward criterion)
    k_vecmax<SF><<<batch, 256, 0, st>>>(c.d32, n, n, c.nrm, 5, 8); ++g_launches;
    k_vecmax<SD><<<batch, 256, 0, st>>>(c.x, n, n, c.nrm, 6, 8); ++g_launches;
    std::vector<double> hn(8 * (size_t)batch);
    CK(cudaMemcpyAsync(hn.data(), c.nrm, sizeof(double) * 8 * batch, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if ((int)c.dxraw.size() != batch) c.dxraw.assign(batch, 1e300);
    for (int bi = 0; bi < batch; ++bi)
      if (c.be[bi] > c.tol || c.dx[bi] > kFwdTol) {
        const double raw = c.rprev[bi] * hn[8 * bi + 5] / std::max(hn[8 * bi + 6], 1e-300);
        const double prev = c.dxraw[bi];
        c.dxraw[bi] = raw;
        double est = raw;
        if (prev < 1e300 && prev > 0.0 && raw / prev < 0.5) est = raw / prev / (1.0 - raw / prev) * raw;
        c.dx[bi] = est;
      }
    ++c.it;
  }
}

// GMRES-IR: up to 10 outer corrections, each a GMRES(m) solve of
// M^-1 A d = M^-1 r to 1e-6 relative (preconditioned residual).
template <typename SD, typename SF>
static int refine_gmres(MixCtx<SD, SF>& c, int* conv) {
  typedef std::complex<double> C;
  cudaStream_t st = c.h->st;
  const int n = c.n, batch = c.batch, m = 20;
  const long long nn = (long long)n * n;
  int rc;
  // work: V [batch][m+1][n], w [batch][n], coefficients [batch][m+1], scales [batch]
  const size_t vbytes = sizeof(SD) * (size_t)batch * (m + 1) * n, wbytes = sizeof(SD) * (size_t)batch * n;
  const size_t cbytes = sizeof(SD) * (size_t)batch * (m + 1), sbytes = sizeof(double) * batch;
  if ((rc = ensure(c.h->gm, vbytes + wbytes + 2 * cbytes + sbytes + 64))) return rc;
  SD* V = (SD*)c.h->gm.p;
  SD* w = (SD*)((char*)V + vbytes);
  SD* hc = (SD*)((char*)w + wbytes);
  SD* hc2 = (SD*)((char*)hc + cbytes);
  double* sc = (double*)((char*)hc2 + cbytes);
  const long long sV = (long long)(m + 1) * n;
  std::vector<SD> hh(batch * (size_t)(m + 1)), hh2(batch * (size_t)(m + 1));
  std::vector<double> hs(batch);
  auto toC = [](const SD& v) -> C {
    if constexpr (std::is_same<SD, double2>::value) return C(v.x, v.y);
    else return C(v, 0.0);
  };
  auto fromC = [](const C& v) -> SD {
    if constexpr (std::is_same<SD, double2>::value) return make_double2(v.real(), v.imag());
    else return v.real();
  };
  *conv = 0;
  c.dx.assign(batch, 0.0);  // GMRES-IR stops on the backward error alone
  for (int outer = 0; outer < 10; ++outer) {
    bool all;
    if ((rc = residual_check(c, c.fresh, &all))) return rc;
    if (all) { *conv = 1; return 0; }
    ++c.it;
    // z = M^-1 r -> V_0 = z / beta
    if ((rc = precond(c, c.r, w))) return rc;
    k_bdot<SD><<<dim3(1, batch), 256, 0, st>>>(w, n, 1, w, n, n, hc, m + 1); ++g_launches;
    CK(cudaMemcpyAsync(hh.data(), hc, cbytes, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    std::vector<double> beta(batch);
    std::vector<int> kb(batch, 0), done(batch, 0);
    std::vector<std::vector<C>> H(batch, std::vector<C>((size_t)(m + 1) * m)), g(batch, std::vector<C>(m + 1));
    std::vector<std::vector<double>> cs(batch, std::vector<double>(m));
    std::vector<std::vector<C>> sn(batch, std::vector<C>(m));
    for (int bi = 0; bi < batch; ++bi) {
      beta[bi] = std::sqrt(std::max(0.0, toC(hh[(size_t)(m + 1) * bi]).real()));
      done[bi] = !(c.be[bi] > c.tol) || beta[bi] == 0.0;
      hs[bi] = beta[bi] > 0.0 ? 1.0 / beta[bi] : 0.0;
      g[bi][0] = beta[bi];
    }
    CK(cudaMemcpyAsync(sc, hs.data(), sbytes, cudaMemcpyHostToDevice, st));
    k_bscale<SD><<<dim3(nblk(n, 256), batch), 256, 0, st>>>(w, n, V, sV, n, sc); ++g_launches;
    int j = 0;
    for (; j < m; ++j) {
      // w = M^-1 A V_j
      if ((rc = gemv_apply<SD>(st, n, c.A, n, nn, V + (long long)j * n, sV, c.r, n, batch))) return rc;
      if ((rc = precond(c, c.r, w))) return rc;
      // classical Gram-Schmidt, twice
      k_bdot<SD><<<dim3(j + 1, batch), 256, 0, st>>>(V, sV, j + 1, w, n, n, hc, m + 1); ++g_launches;
      k_bcomb<SD><<<dim3(nblk(n, 256), batch), 256, 0, st>>>(w, n, V, sV, j + 1, hc, m + 1, n, -1.0, nullptr); ++g_launches;
      k_bdot<SD><<<dim3(j + 1, batch), 256, 0, st>>>(V, sV, j + 1, w, n, n, hc2, m + 1); ++g_launches;
      k_bcomb<SD><<<dim3(nblk(n, 256), batch), 256, 0, st>>>(w, n, V, sV, j + 1, hc2, m + 1, n, -1.0, nullptr); ++g_launches;
      CK(cudaMemcpyAsync(hh.data(), hc, cbytes, cudaMemcpyDeviceToHost, st));
      CK(cudaMemcpyAsync(hh2.data(), hc2, cbytes, cudaMemcpyDeviceToHost, st));
      k_bdot<SD><<<dim3(1, batch), 256, 0, st>>>(w, n, 1, w, n, n, hc, m + 1); ++g_launches;
      std::vector<SD> nw(batch * (size_t)(m + 1));
      CK(cudaMemcpyAsync(nw.data(), hc, cbytes, cudaMemcpyDeviceToHost, st));
      CK(cudaStreamSynchronize(st));
      bool all_done = true;
      for (int bi = 0; bi < batch; ++bi) {
        const double hn1 = std::sqrt(std::max(0.0, toC(nw[(size_t)(m + 1) * bi]).real()));
        hs[bi] = 0.0;
        if (done[bi]) continue;
        C* Hc = &H[bi][(size_t)(m + 1) * j];
        for (int i = 0; i <= j; ++i)
          Hc[i] = toC(hh[(size_t)(m + 1) * bi + i]) + toC(hh2[(size_t)(m + 1) * bi + i]);
        Hc[j + 1] = hn1;
        for (int i = 0; i < j; ++i) {  // previous rotations
          const C a = Hc[i], bq = Hc[i + 1];
          Hc[i] = cs[bi][i] * a + sn[bi][i] * bq;
          Hc[i + 1] = -std::conj(sn[bi][i]) * a + cs[bi][i] * bq;
        }
        const C a = Hc[j];
        const double bq = std::abs(Hc[j + 1]), aa = std::abs(a), t = std::hypot(aa, bq);
        if (t == 0.0) { cs[bi][j] = 1.0; sn[bi][j] = 0.0; }
        else if (aa == 0.0) { cs[bi][j] = 0.0; sn[bi][j] = 1.0; Hc[j] = bq; }
        else {
          const C ph = a / aa;
          cs[bi][j] = aa / t;
          sn[bi][j] = ph * std::conj(Hc[j + 1]) / t;
          Hc[j] = ph * t;
        }
        Hc[j + 1] = 0.0;
        g[bi][j + 1] = -std::conj(sn[bi][j]) * g[bi][j];
        g[bi][j] = cs[bi][j] * g[bi][j];
        kb[bi] = j + 1;
        ++c.inner;
        if (std::abs(g[bi][j + 1]) <= 1e-6 * beta[bi] || hn1 == 0.0) done[bi] = 1;
        else hs[bi] = 1.0 / hn1;
        all_done = all_done && done[bi];
      }
      if (all_done || j + 1 == m) { ++j; break; }
      CK(cudaMemcpyAsync(sc, hs.data(), sbytes, cudaMemcpyHostToDevice, st));
      k_bscale<SD><<<dim3(nblk(n, 256), batch), 256, 0, st>>>(w, n, V + (long long)(j + 1) * n, sV, n, sc); ++g_launches;
    }
    // y = H^-1 g (upper triangular, kb x kb), x += V y
    std::vector<SD> yv(batch * (size_t)(m + 1));
    for (int bi = 0; bi < batch; ++bi) {
      const int k = kb[bi];
      std::vector<C> y(k);
      for (int i = k - 1; i >= 0; --i) {
        C sum = g[bi][i];
        for (int q = i + 1; q < k; ++q) sum -= H[bi][(size_t)(m + 1) * q + i] * y[q];
        y[i] = sum / H[bi][(size_t)(m + 1) * i + i];
      }
      for (int i = 0; i <= m; ++i) yv[(size_t)(m + 1) * bi + i] = fromC(i < k ? y[i] : C(0.0));
    }
    CK(cudaMemcpyAsync(hc, yv.data(), cbytes, cudaMemcpyHostToDevice, st));
    int kmax = 0;
    for (int bi = 0; bi < batch; ++bi) kmax = std::max(kmax, kb[bi]);
    if (kmax > 0) {
      k_bcomb<SD><<<dim3(nblk(n, 256), batch), 256, 0, st>>>(c.x, n, V, sV, kmax, hc, m + 1, n, 1.0, c.active);
      ++g_launches;
    }
  }
  bool all;
  if ((rc = residual_check(c, false, &all))) return rc;
  *conv = all ? 1 : 0;
  return 0;
}

// Solve the batch of FP64 systems (A_f, b_f) in place of x. precision 0: FP64
// LU; 1: FP32 LU + FP64 refinement. Work memory from the handle.
template <typename SD, typename SF>
static int solve_batch(mfbem_handle* h, SD* A, int n, int batch, const SD* b, SD* x, int precision, double tol,
                       mfbem_stats* stats) {
  int rc;
  cudaStream_t st = h->st;
  const long long nn = (long long)n * n;
  if ((rc = ensure(h->ipiv, sizeof(int) * (size_t)n * batch)) || (rc = ensure(h->info, sizeof(int) * (batch + 4))))
    return rc;
  int* ipiv = (int*)h->ipiv.p;
  int* info = (int*)h->info.p;
  if ((rc = trsv_err_reset(st))) return rc;
  cudaEvent_t e0, e1, e2;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventCreate(&e2);
  // mixed: the outer block width of this size class (a first use runs the
  // autotuner, outside the timed factorisation)
  int nbo = 128;
  g_nopiv = false;
  if (precision != 0) {
    g_c32_mode = c32_default();
    if (g_c32_mode == 1 && h->tf32_stalled) g_c32_mode = 0;
    const int pv = pivot_default();
    g_nopiv = pv == 1 || (pv < 0 && !h->nopiv_failed);
    if ((rc = tuned_nbo<SF>(st, n, batch, ipiv, info, &nbo))) return rc;
  }
  cudaEventRecord(e0, st);
  std::vector<int> hinfo(batch);
  if (precision == 0) {
    if ((rc = getrf_batched<SD>(st, A, nn, n, n, batch, ipiv, info))) return rc;
    cudaEventRecord(e1, st);
    k_copy_vec<SD><<<nblk((long long)n * batch, 256), 256, 0, st>>>(b, x, (long long)n * batch); ++g_launches;
    if ((rc = getrs_batched<SD>(st, A, nn, n, n, ipiv, n, x, n, batch))) return rc;
    cudaEventRecord(e2, st);
    CK(cudaMemcpyAsync(hinfo.data(), info, sizeof(int) * batch, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if ((rc = trsv_err_check(st))) return rc;
    stats->refinement_iterations = 0;
  } else {
    // FP32 copy of A, factor
    // work: d32 [batch][n] (SF), then, from a 256-byte boundary (a real FP32
    // vector of odd length would leave the doubles misaligned), nrm [batch][8],
    // rows [batch][n] (double), active [batch] (int)
    const size_t off_nrm = (sizeof(SF) * (size_t)n * batch + 255) / 256 * 256;
    if ((rc = ensure(h->A32, sizeof(SF) * nn * batch)) || (rc = ensure(h->r, sizeof(SD) * (size_t)n * batch)) ||
        (rc = ensure(h->work, off_nrm + sizeof(double) * ((size_t)n * batch + 8 * batch) + 4 * batch)))
      return rc;
    MixCtx<SD, SF> c;
    c.h = h;
    c.A = A;
    c.A32 = (SF*)h->A32.p;
    c.ipiv = ipiv;
    c.n = n;
    c.batch = batch;
    c.b = b;
    c.x = x;
    c.r = (SD*)h->r.p;
    c.d32 = (SF*)h->work.p;
    c.nrm = (double*)((char*)h->work.p + off_nrm);  // [batch][8]: |r|,|x|,|b|,|A|,precond scale
    double* rows = c.nrm + 8 * batch;
    c.active = (int*)(rows + (size_t)n * batch);
    c.tol = tol;
    CK(cudaMemsetAsync(rows, 0, sizeof(double) * (size_t)n * batch, st));
    k_demote_rowabs<SD, SF><<<dim3(nblk(n, 256), nblk(n, 128), batch), 256, 0, st>>>(A, c.A32, nn, n, n, rows); ++g_launches;
    k_vecmax<double><<<batch, 256, 0, st>>>(rows, n, n, c.nrm, 3, 8); ++g_launches;
    k_vecmax<SD><<<batch, 256, 0, st>>>(b, n, n, c.nrm, 2, 8); ++g_launches;
    if ((rc = getrf_batched<SF>(st, c.A32, nn, n, n, batch, ipiv, info, nbo))) return rc;
    if (g_nopiv) {
      // a zero or non-finite pivot without interchanges: factorise again with partial pivoting
      CK(cudaMemcpyAsync(hinfo.data(), info, sizeof(int) * batch, cudaMemcpyDeviceToHost, st));
      CK(cudaStreamSynchronize(st));
      bool bad = false;
      for (int bi = 0; bi < batch; ++bi) bad = bad || hinfo[bi] != 0;
      if (bad) {
        g_nopiv = false;
        h->nopiv_failed = true;
        ++c.refactor;
        k_demote<SD, SF><<<std::min(nblk(nn * batch, 256), 152u * 32u), 256, 0, st>>>(A, c.A32, nn * batch); ++g_launches;
        if ((rc = getrf_batched<SF>(st, c.A32, nn, n, n, batch, ipiv, info, nbo))) return rc;
      }
    }
    cudaEventRecord(e1, st);
    CK(cudaMemsetAsync(x, 0, sizeof(SD) * (size_t)n * batch, st));
    // refinement: precision 1, classical refinement until it converges or
    // stalls; if the factors came from TF32 updates, refactorise with SIMT FP32
    // (one factorisation costs about ten triangular-solve pairs, less than the
    // GMRES steps TF32 factors need on ill-conditioned systems) and refine
    // again; GMRES-IR last. Precision 2: GMRES-IR first, refactorisation if it fails.
    const bool gm_first = precision == 2 || (getenv("MFBEM_REFINE") && std::string(getenv("MFBEM_REFINE")) == "gmres");
    int conv = 0;
    // refactorisation after a stall: with partial pivoting if the factors had
    // none, else with SIMT FP32 updates if they came from single-pass TF32
    auto refactor = [&]() -> int {
      cudaEvent_t f0, f1;
      cudaEventCreate(&f0);
      cudaEventCreate(&f1);
      cudaEventRecord(f0, st);
      if (g_nopiv) {
        g_nopiv = false;
        h->nopiv_failed = true;
      } else {
        g_c32_mode = 0;
        h->tf32_stalled = true;
      }
      ++c.refactor;
      k_demote<SD, SF><<<std::min(nblk(nn * batch, 256), 152u * 32u), 256, 0, st>>>(A, c.A32, nn * batch); ++g_launches;
      int nb2 = 128;
      int r = tuned_nbo<SF>(st, n, batch, ipiv, info, &nb2);
      if (!r) r = getrf_batched<SF>(st, c.A32, nn, n, n, batch, ipiv, info, nb2);
      cudaEventRecord(f1, st);
      cudaEventSynchronize(f1);
      float t = 0.0f;
      cudaEventElapsedTime(&t, f0, f1);
      cudaEventDestroy(f0);
      cudaEventDestroy(f1);
      stats->ms_factor += t;
      stats->ms_solve -= t;
      return r;
    };
    auto restart = [&]() -> int {  // refinement from x = 0 after a refactorisation
      c.fresh = true;
      c.dx.clear();
      c.dxraw.clear();
      c.rprev.clear();
      CK(cudaMemsetAsync(x, 0, sizeof(SD) * (size_t)n * batch, st));
      return 0;
    };
    if (gm_first) {
      if ((rc = refine_gmres(c, &conv))) return rc;
      if (!conv && (g_nopiv || g_c32_mode == 1)) {
        const bool np = g_nopiv;
        if ((rc = refactor()) || (np && (rc = restart()))) return rc;
        if ((rc = refine_gmres(c, &conv))) return rc;
      }
    } else {
      if ((rc = refine_classical(c, &conv))) return rc;
      if (!conv && g_nopiv) {
        if ((rc = refactor()) || (rc = restart())) return rc;
        if ((rc = refine_classical(c, &conv))) return rc;
      }
      if (!conv && g_c32_mode == 1) {
        if ((rc = refactor())) return rc;
        if ((rc = refine_classical(c, &conv))) return rc;
      }
      if (!conv) {
        if ((rc = refine_gmres(c, &conv))) return rc;
      }
    }
    cudaEventRecord(e2, st);
    CK(cudaMemcpyAsync(hinfo.data(), info, sizeof(int) * batch, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    stats->refinement_iterations += c.it;
    stats->gmres_iterations += c.inner;
    stats->refactorizations += c.refactor;
    stats->max_backward_error = std::max(stats->max_backward_error, c.maxbe);
    if ((rc = trsv_err_check(st))) return rc;
    if (!conv) {
      cudaEventDestroy(e0); cudaEventDestroy(e1); cudaEventDestroy(e2);
      return fail(MFBEM_ENOCONV, "iterative refinement did not reach the requested backward error");
    }
  }
  float ms1 = 0, ms2 = 0;
  cudaEventElapsedTime(&ms1, e0, e1);
  cudaEventElapsedTime(&ms2, e1, e2);
  stats->ms_factor += ms1;
  stats->ms_solve += ms2;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaEventDestroy(e2);
  for (int bi = 0; bi < batch; ++bi)
    if (hinfo[bi] > 0) return fail(hinfo[bi], "singular matrix: zero pivot");
  return 0;
}

extern "C" int mfbem_sweep_harela(mfbem_handle* h, const double lambda[2], const double mu[2], double rho,
                                  const double nu[2], int32_t n_freq, const double* omega, int32_t precision,
                                  double rel_tol, double* x_out, int32_t flags, mfbem_stats* stats) {
  g_err.clear();
  if (!h || !lambda || !mu || !nu || !omega || !x_out || n_freq < 1) return fail(MFBEM_EARG, "invalid argument");
  if (int rd = check_dev(h)) return rd;
  if (precision < 0 || precision > 2) return fail(MFBEM_EARG, "precision must be 0, 1 or 2");
  const int n = h->ndof;
  const long long nn = (long long)n * n;
  int rc;
  mfbem_stats s = h->stats;
  s.refinement_iterations = 0;
  s.gmres_iterations = 0;
  s.refactorizations = 0;
  s.max_backward_error = 0.0;
  s.ms_factor = s.ms_solve = 0.0;
  if ((rc = ensure(h->A, sizeof(double2) * nn * n_freq)) || (rc = ensure(h->b, sizeof(double2) * (size_t)n * n_freq)) ||
      (rc = ensure(h->x, sizeof(double2) * (size_t)n * n_freq)) ||
      (rc = ensure(h->par, (sizeof(HarParD) + 6 * sizeof(double)) * n_freq + 2 * sizeof(double) * n_freq)))
    return rc;
  HarParD* dpar = (HarParD*)h->par.p;
  double* dq = (double*)(dpar + n_freq);
  double* dnu = dq + 6 * n_freq;
  std::vector<double> q(6 * (size_t)n_freq), nuv(2 * (size_t)n_freq);
  for (int f = 0; f < n_freq; ++f) {
    double v[6] = {lambda[0], lambda[1], mu[0], mu[1], rho, omega[f]};
    for (int j = 0; j < 6; ++j) q[6 * f + j] = v[j];
    nuv[2 * f] = nu[0];
    nuv[2 * f + 1] = nu[1];
  }
  CK(cudaMemcpyAsync(dq, q.data(), sizeof(double) * q.size(), cudaMemcpyHostToDevice, h->st));
  CK(cudaMemcpyAsync(dnu, nuv.data(), sizeof(double) * nuv.size(), cudaMemcpyHostToDevice, h->st));
  k_harpar<<<nblk(n_freq, 32), 32, 0, h->st>>>(dq, n_freq, dpar, zexp_thresholds()); ++g_launches;
  double2* A = (double2*)h->A.p;
  double2* b = (double2*)h->b.p;
  double2* x = (flags & MFBEM_DEVICE_PTRS) ? (double2*)x_out : (double2*)h->x.p;
  h->last_nf = n_freq;
  // the assembly time covers zeroing the systems too
  cudaEvent_t a0, a1;
  cudaEventCreate(&a0);
  cudaEventCreate(&a1);
  cudaEventRecord(a0, h->st);
  CK(cudaMemsetAsync(A, 0, sizeof(double2) * nn * n_freq, h->st));
  CK(cudaMemsetAsync(b, 0, sizeof(double2) * (size_t)n * n_freq, h->st));
  if ((rc = bm_prepare(h, 1))) return rc;
  PolHarmonic pol;
  pol.p = dpar;
  if ((rc = hbie_params(h, dq, n_freq, &pol.ph))) return rc;
  AsmTimes tm;
  long long l0 = g_launches;
  const HarParF* pf = nullptr;
  const ff* dsf = nullptr;
  const ff *sgf = nullptr, *lgf = nullptr;
  if (precision >= 1) {
    // mixed: regular pairs in double-float (df64 datasets made once per mesh:
    // phi*J*w [ne][ptot][8], unit normals [ne][ptot][3], prescribed values [ndof][2])
    const long long npp = 8LL * h->m.ne * h->m.ptot, nnp = 3LL * h->m.ne * h->m.ptot, ncv = 2LL * n;
    if (h->pphi_f.bytes < sizeof(ff) * (npp + nnp + ncv)) {
      if ((rc = ensure(h->pphi_f, sizeof(ff) * (npp + nnp + ncv)))) return rc;
      ff* d = (ff*)h->pphi_f.p;
      k_pphi_f<<<std::min(nblk(npp, 256), 152u * 16u), 256, 0, h->st>>>(h->m.pphi, d, npp); ++g_launches;
      k_pphi_f<<<std::min(nblk(nnp, 256), 152u * 16u), 256, 0, h->st>>>(h->m.pn, d + npp, nnp); ++g_launches;
      k_pphi_f<<<std::min(nblk(ncv, 256), 152u * 16u), 256, 0, h->st>>>(h->m.dcv, d + npp + nnp, ncv); ++g_launches;
    }
    // df64 copies of the hoisted singular / adaptive point geometry
    const long long ngs = h->m.sing_geo ? 22LL * h->m.nsing_pts : 0, ngl = h->m.leaf_geo ? 14LL * h->m.nleaf_pts : 0;
    if (ngs + ngl > 0 && h->geo_f.bytes < sizeof(ff) * (ngs + ngl)) {
      if ((rc = ensure(h->geo_f, sizeof(ff) * (ngs + ngl)))) return rc;
      ff* d = (ff*)h->geo_f.p;
      if (ngs) { k_pphi_f<<<std::min(nblk(ngs, 256), 152u * 16u), 256, 0, h->st>>>(h->m.sing_geo, d, ngs); ++g_launches; }
      if (ngl) { k_pphi_f<<<std::min(nblk(ngl, 256), 152u * 16u), 256, 0, h->st>>>(h->m.leaf_geo, d + ngs, ngl); ++g_launches; }
    }
    sgf = ngs ? (const ff*)h->geo_f.p : nullptr;
    lgf = ngl ? (const ff*)h->geo_f.p + ngs : nullptr;
    if ((rc = ensure(h->parf, sizeof(HarParF) * n_freq))) return rc;
    k_harpar_f<<<nblk(n_freq, 32), 32, 0, h->st>>>(dpar, (HarParF*)h->parf.p, n_freq); ++g_launches;
    pf = (const HarParF*)h->parf.p;
    dsf = (const ff*)h->pphi_f.p;
  }
  if ((rc = launch_assembly(h, pol, dnu, n_freq, (double*)A, n, 2 * nn, (double*)b, 2 * (size_t)n, &tm, pf, dsf,
                            precision >= 1, sgf, lgf)))
    return rc;
  cudaEventRecord(a1, h->st);
  if ((rc = check_err(h))) return rc;
  float ams = 0;
  cudaEventElapsedTime(&ams, a0, a1);
  cudaEventDestroy(a0);
  cudaEventDestroy(a1);
  s.ms_assemble = ams;
  tm.read(&s);
  rc = solve_batch<double2, float2>(h, A, n, n_freq, b, x, precision, rel_tol, &s);
  s.kernel_launches = g_launches - l0;
  if (rc && rc != MFBEM_ENOCONV) return rc;
  if (!(flags & MFBEM_DEVICE_PTRS)) {
    CK(cudaMemcpyAsync(x_out, x, sizeof(double2) * (size_t)n * n_freq, cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
  }
  h->stats = s;
  if (stats) *stats = s;
  return rc;
}

extern "C" int mfbem_solve_staela(mfbem_handle* h, double mu, double nu, int32_t precision, double rel_tol,
                                  double* x_out, int32_t flags, mfbem_stats* stats) {
  g_err.clear();
  if (!h || !x_out) return fail(MFBEM_EARG, "invalid argument");
  if (int rd = check_dev(h)) return rd;
  if (precision < 0 || precision > 2) return fail(MFBEM_EARG, "precision must be 0, 1 or 2");
  const int n = h->ndof;
  const long long nn = (long long)n * n;
  int rc;
  mfbem_stats s = h->stats;
  s.refinement_iterations = 0;
  s.gmres_iterations = 0;
  s.refactorizations = 0;
  s.max_backward_error = 0.0;
  s.ms_factor = s.ms_solve = 0.0;
  if ((rc = ensure(h->A, sizeof(double) * nn)) || (rc = ensure(h->b, sizeof(double) * n)) ||
      (rc = ensure(h->x, sizeof(double) * n)) || (rc = ensure(h->nu, 2 * sizeof(double))))
    return rc;
  double nuv[2] = {nu, 0.0};
  CK(cudaMemcpyAsync(h->nu.p, nuv, sizeof(nuv), cudaMemcpyHostToDevice, h->st));
  double* A = (double*)h->A.p;
  double* b = (double*)h->b.p;
  double* x = (flags & MFBEM_DEVICE_PTRS) ? x_out : (double*)h->x.p;
  CK(cudaMemsetAsync(A, 0, sizeof(double) * nn, h->st));
  CK(cudaMemsetAsync(b, 0, sizeof(double) * n, h->st));
  if ((rc = hs_prepare_static(h))) return rc;
  if ((rc = bm_prepare(h, 0))) return rc;
  PolStatic pol;
  pol.k = staela_params(mu, nu);
  pol.nu = nu;
  pol.mu = mu;
  AsmTimes tm;
  long long l0 = g_launches;
  if ((rc = launch_assembly(h, pol, (const double*)h->nu.p, 1, A, n, 0, b, 0, &tm))) return rc;
  if ((rc = check_err(h))) return rc;
  tm.read(&s);
  rc = solve_batch<double, float>(h, A, n, 1, b, x, precision, rel_tol, &s);
  s.kernel_launches = g_launches - l0;
  if (rc && rc != MFBEM_ENOCONV) return rc;
  if (!(flags & MFBEM_DEVICE_PTRS)) {
    CK(cudaMemcpyAsync(x_out, x, sizeof(double) * n, cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
  }
  h->stats = s;
  if (stats) *stats = s;
  return rc;
}
