// Complex64 GEMM update C -= A B on the 5th-generation tensor cores (tcgen05,
// kind::tf32) with the 3xTF32 split (A_hi B_hi + A_hi B_lo + A_lo B_hi, each
// operand x = hi + lo with hi = tf32(x)), i.e. FP32-level accuracy: the
// trailing update of the mixed LU. Included into mfbem_abi.cu.
//
// The complex product is one real GEMM of the realified operands:
//   C~ (2m x n)  = C viewed as real, column j = [re C0j, im C0j, re C1j, ...]
//   B~ (2k x n)  = B viewed as real (same memory)
//   A~ (2m x 2k) : A~(2i,2l) = re a_il, A~(2i+1,2l) = im a_il,
//                  A~(2i,2l+1) = -im a_il, A~(2i+1,2l+1) = re a_il
// so C~ -= A~ B~ is C -= A B. Operand tiles live in shared memory in the
// canonical K-major layout without swizzle (8-row x 16-byte core matrices,
// 128 B apart along K, 1024 B apart along M/N); one thread issues
// tcgen05.mma.cta_group::1.kind::tf32 (K 8) into a TMEM accumulator and
// commits to an mbarrier; every warp then reads its 32 TMEM lanes
// (tcgen05.ld 32x32b) and subtracts from C. Two kernels:
//   k_tc_cgemm         each CTA splits and stages its own 128 x 128 tile's
//                      operands (kept as the self-contained variant the
//                      tests compare against);
//   k_tc_cgemm_bulk<NH> the LU's trailing update: operands split once into
//                      tf32 hi / lo tiles by k_tc_prep_a / k_tc_prep_b, copied
//                      by cp.async.bulk into a two-stage pipeline; NH = 2 runs
//                      one M 128 x N 256 MMA per K step (two 128-column
//                      halves in 256 TMEM columns, two CTAs per SM).
// Every wait is bounded: on a timeout the kernel sets *err, waits (bounded)
// for its MMAs, frees its TMEM and returns.
#pragma once
#include <cstdint>

namespace mfb {

constexpr int TC_BM = 128;  // real rows of C~ per CTA (64 complex rows)
constexpr int TC_BN = 128;  // columns per CTA
constexpr int TC_BK = 32;   // real K per chunk (16 complex)
constexpr int TC_TILE_BYTES = TC_BM * TC_BK * 4;  // one operand tile (16 KB); B tile is TC_BN x TC_BK
constexpr int TC_SMEM = 4 * TC_TILE_BYTES + 64;    // A hi/lo, B hi/lo, mbarrier, TMEM address
constexpr int TC_STAGE_BYTES = 4 * TC_TILE_BYTES;  // one pipeline stage: A hi/lo, B hi/lo
constexpr long long TC_SPIN = 1LL << 26;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ uint32_t f2tf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}
// offset in bytes of element (row r, k) of a K-major no-swizzle tile with
// 8 x 16 B core matrices, LBO 128 B (K), SBO 1024 B (rows)
__device__ __forceinline__ uint32_t tc_off(int r, int k) {
  return (uint32_t)((r >> 3) * 1024 + (k >> 2) * 128 + (r & 7) * 16 + (k & 3) * 4);
}
// shared memory descriptor: start address, LBO, SBO (>> 4), version 1, no swizzle
__device__ __forceinline__ uint64_t tc_desc(uint32_t addr) {
  uint64_t d = 0;
  d |= (uint64_t)((addr & 0x3FFFF) >> 4);
  d |= (uint64_t)(128 >> 4) << 16;
  d |= (uint64_t)(1024 >> 4) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}
// instruction descriptor, kind::tf32: D f32, A and B tf32, both K-major, N, M
__host__ __device__ constexpr uint32_t tc_idesc(int m, int n) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

// Spin limit of the waits on mbarriers: TC_SPIN polls with try_wait (which
// itself suspends the thread for a short while); a positive `spin` (set only
// by the failure-detection test hook) instead allows that many non-blocking
// test_wait polls. A wait that gives up makes the kernel set its error flag;
// the waits that then drain the copies and MMAs still in flight use the full
// TC_SPIN.
__device__ __forceinline__ bool tc_wait(uint32_t mbar, uint32_t parity, long long spin = 0) {
  if (spin > 0) {
    for (long long it = 0; it < spin; ++it) {
      uint32_t done;
      asm volatile(
          "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
          : "=r"(done)
          : "r"(mbar), "r"(parity)
          : "memory");
      if (done) return true;
    }
    return false;
  }
  for (long long it = 0; it < TC_SPIN; ++it) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(mbar), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// C (m x n complex, ldc) -= A (m x k, lda) B (k x n, ldb), batch in blockIdx.z
__global__ void __launch_bounds__(128, 1) k_tc_cgemm(const float2* A, int lda, long long sA, const float2* B, int ldb,
                                                     long long sB, float2* C, int ldc, long long sC, int m, int n,
                                                     int k, int* err, long long spin) {
  extern __shared__ __align__(1024) unsigned char tsm[];
  unsigned char* Ahi = tsm;
  unsigned char* Alo = tsm + TC_TILE_BYTES;
  unsigned char* Bhi = tsm + 2 * TC_TILE_BYTES;
  unsigned char* Blo = tsm + 3 * TC_TILE_BYTES;
  uint64_t* mbar = reinterpret_cast<uint64_t*>(tsm + 4 * TC_TILE_BYTES);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(tsm + 4 * TC_TILE_BYTES + 16);
  __shared__ int s_ok;
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  const int bz = blockIdx.z;
  const float2* Ab = A + sA * bz;
  const float2* Bb = B + sB * bz;
  float2* Cb = C + sC * bz;
  const int i0 = blockIdx.x * (TC_BM / 2);  // first complex row
  const int j0 = blockIdx.y * TC_BN;        // first column
  const uint32_t mb = smem_u32(mbar);
  if (t == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mb) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    s_ok = 1;
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)),
                 "r"(TC_BN)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tslot;
  const uint32_t idesc = tc_idesc(TC_BM, TC_BN);
  const int nchunk = (k + TC_BK / 2 - 1) / (TC_BK / 2);
  int phase = 0;
  for (int ch = 0; ch < nchunk && s_ok; ++ch) {
    const int l0 = ch * (TC_BK / 2);
    // Staging walks the tiles in shared-memory word order (32 consecutive
    // words = one 8 x 16 B core matrix), so the stores of a warp are
    // conflict-free; word w: core matrix w / 32 (8 along K per 8-row group),
    // row (w % 32) / 4 inside it, K offset w % 4.
    // A~ tile: 128 rows x 32 K; element (r, kk) comes from a(i0 + r/2, l0 + kk/2)
    for (int w = t; w < TC_BM * TC_BK; w += 128) {
      const int cm = w >> 5, r = ((cm >> 3) << 3) + ((w & 31) >> 2), kk = ((cm & 7) << 2) + (w & 3);
      const int i = i0 + (r >> 1), l = l0 + (kk >> 1);
      float2 a = make_float2(0.0f, 0.0f);
      if (i < m && l < k) a = Ab[(size_t)l * lda + i];
      // (r even, kk even) re, (r odd, kk even) im, (r even, kk odd) -im, (r odd, kk odd) re
      const float v = (kk & 1) ? ((r & 1) ? a.x : -a.y) : ((r & 1) ? a.y : a.x);
      const uint32_t hi = f2tf32(v), lo = f2tf32(v - __uint_as_float(hi));
      reinterpret_cast<uint32_t*>(Ahi)[w] = hi;
      reinterpret_cast<uint32_t*>(Alo)[w] = lo;
    }
    // B~ tile: 128 rows (columns j) x 32 K; element (jj, kk) is component kk&1 of b(l0 + kk/2, j0 + jj)
    for (int w = t; w < TC_BN * TC_BK; w += 128) {
      const int cm = w >> 5, jj = ((cm >> 3) << 3) + ((w & 31) >> 2), kk = ((cm & 7) << 2) + (w & 3);
      const int l = l0 + (kk >> 1), j = j0 + jj;
      float2 b = make_float2(0.0f, 0.0f);
      if (l < k && j < n) b = Bb[(size_t)j * ldb + l];
      const float v = (kk & 1) ? b.y : b.x;
      const uint32_t hi = f2tf32(v), lo = f2tf32(v - __uint_as_float(hi));
      reinterpret_cast<uint32_t*>(Bhi)[w] = hi;
      reinterpret_cast<uint32_t*>(Blo)[w] = lo;
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (t == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t ah = smem_u32(Ahi), al = smem_u32(Alo), bh = smem_u32(Bhi), bl = smem_u32(Blo);
#pragma unroll
      for (int ks = 0; ks < TC_BK / 8; ++ks) {
        const uint32_t ko = ks * 256;  // 8 tf32 = two core matrices along K
        const uint64_t dah = tc_desc(ah + ko), dal = tc_desc(al + ko), dbh = tc_desc(bh + ko), dbl = tc_desc(bl + ko);
        const uint32_t acc0 = (ch > 0 || ks > 0) ? 1u : 0u;
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(
                tmem),
            "l"(dah), "l"(dbh), "r"(idesc), "r"(acc0)
            : "memory");
        asm volatile("tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, 1;" ::"r"(tmem), "l"(dah), "l"(dbl),
                     "r"(idesc)
                     : "memory");
        asm volatile("tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, 1;" ::"r"(tmem), "l"(dal), "l"(dbh),
                     "r"(idesc)
                     : "memory");
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mb)
                   : "memory");
    }
    // the tiles are reused by the next chunk: wait for this chunk's MMAs
    if (!tc_wait(mb, (uint32_t)phase, spin)) {
      if (t == 0) atomicExch(err, 1);
      s_ok = 0;
    }
    phase ^= 1;
    __syncthreads();
  }
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (s_ok && nchunk > 0) {
    // epilogue: warp w reads TMEM lanes 32w..32w+31 (rows of C~), 32 columns at a time
    const int r = 32 * warp + lane;  // real row of the tile
    const int i = i0 + (r >> 1), comp = r & 1;
    for (int c0 = 0; c0 < TC_BN; c0 += 32) {
      uint32_t v[32];
      const uint32_t ta = tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)c0;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,"
          "%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
          : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
            "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]),
            "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]),
            "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
          : "r"(ta)
          : "memory");
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      if (i < m) {
        // all loads first, then the stores (a load / store pair per element
        // would serialise 32 global round trips)
        float* cr = reinterpret_cast<float*>(Cb);
        float cv[32];
#pragma unroll
        for (int q = 0; q < 32; ++q) {
          const int j = j0 + c0 + q;
          cv[q] = j < n ? cr[2 * ((size_t)j * ldc + i) + comp] : 0.0f;
        }
#pragma unroll
        for (int q = 0; q < 32; ++q) {
          const int j = j0 + c0 + q;
          if (j < n) cr[2 * ((size_t)j * ldc + i) + comp] = cv[q] - __uint_as_float(v[q]);
        }
      }
    }
  } else if (!s_ok && threadIdx.x == 0) {
    // the MMAs of the chunk whose wait gave up (phase toggled since): let
    // them finish (full limit) before the TMEM is freed
    tc_wait(mb, (uint32_t)(phase ^ 1));
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC_BN) : "memory");
}

// ---------------------------------------------------------------------------
// Pre-split operands + bulk-copy pipeline. The staging above converts every
// element in every CTA that uses it; the LU's trailing update reuses the same
// L panel (A) and U block (B) across all tiles, so they are split into
// hi / lo TF32 once per update and written pre-tiled in the exact shared-
// memory word order (one 16 KB tile per (row tile, K chunk) / (column tile,
// K chunk)); the GEMM kernel then only streams tiles with cp.async.bulk into
// two stages (mbarrier expect-tx) while the tensor cores work on the other.
// ---------------------------------------------------------------------------
// Tiles of the pipelined kernel: K chunk of TQ real K (16): 128 x 16 words,
// core matrices 128 B apart along K and TQ / 4 * 128 B apart along rows.
constexpr int TQ = 16;
constexpr int TQ_TW = TC_BM * TQ;                  // words per tile (2048)
constexpr int TQ_TILE_BYTES = TQ_TW * 4;           // 8 KB
constexpr int TQ_SBO = TQ / 4 * 128;               // 512 B

__device__ __forceinline__ uint64_t tq_desc(uint32_t addr) {
  uint64_t d = 0;
  d |= (uint64_t)((addr & 0x3FFFF) >> 4);
  d |= (uint64_t)(128 >> 4) << 16;
  d |= (uint64_t)(TQ_SBO >> 4) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}
// word w of a tile <-> element (row, k): core matrix w / 32 (TQ/4 along K per
// 8-row group), row (w % 32) / 4 inside it, K offset w % 4
__device__ __forceinline__ void tq_rk(int w, int& r, int& kk) {
  const int cm = w >> 5;
  r = (cm / (TQ / 4)) * 8 + ((w & 31) >> 2);
  kk = (cm % (TQ / 4)) * 4 + (w & 3);
}

// A~ tiles: [batch][row tile][K chunk][word]. One 256-thread block per tile
// (blockIdx.x = (b * nmt + mt) * nkc + kc), eight words per thread: the tile
// coordinates are decoded once per block, not per word.
__global__ void __launch_bounds__(256) k_tc_prep_a(const float2* A, int lda, long long sA, int m, int k, int nmt,
                                                   int nkc, int batch, uint32_t* hi, uint32_t* lo) {
  const int kc = (int)(blockIdx.x % nkc), tl = (int)(blockIdx.x / nkc), mt = tl % nmt, b = tl / nmt;
  const float2* Ab = A + sA * b;
  const size_t g0 = (size_t)blockIdx.x * TQ_TW;
#pragma unroll 2
  for (int w = threadIdx.x; w < TQ_TW; w += 256) {
    int r, kk;
    tq_rk(w, r, kk);
    const int i = mt * (TC_BM / 2) + (r >> 1), l = kc * (TQ / 2) + (kk >> 1);
    float2 a = make_float2(0.0f, 0.0f);
    if (i < m && l < k) a = Ab[(size_t)l * lda + i];
    const float v = (kk & 1) ? ((r & 1) ? a.x : -a.y) : ((r & 1) ? a.y : a.x);
    const uint32_t h = f2tf32(v);
    hi[g0 + w] = h;
    lo[g0 + w] = f2tf32(v - __uint_as_float(h));
  }
}
// B~ tiles: [batch][column tile][K chunk][word]; element (jj, kk) is component
// kk&1 of b(l, j). One block per tile as k_tc_prep_a.
__global__ void __launch_bounds__(256) k_tc_prep_b(const float2* B, int ldb, long long sB, int k, int n, int nnt,
                                                   int nkc, int batch, uint32_t* hi, uint32_t* lo) {
  const int kc = (int)(blockIdx.x % nkc), tl = (int)(blockIdx.x / nkc), nt = tl % nnt, b = tl / nnt;
  const float2* Bb = B + sB * b;
  const size_t g0 = (size_t)blockIdx.x * TQ_TW;
#pragma unroll 2
  for (int w = threadIdx.x; w < TQ_TW; w += 256) {
    int jj, kk;
    tq_rk(w, jj, kk);
    const int j = nt * TC_BN + jj, l = kc * (TQ / 2) + (kk >> 1);
    float2 bv = make_float2(0.0f, 0.0f);
    if (l < k && j < n) bv = Bb[(size_t)j * ldb + l];
    const float v = (kk & 1) ? bv.y : bv.x;
    const uint32_t h = f2tf32(v);
    hi[g0 + w] = h;
    lo[g0 + w] = f2tf32(v - __uint_as_float(h));
  }
}

__device__ __forceinline__ void tc_bulk(uint32_t dst, const void* src, uint32_t bytes, uint32_t mbar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(mbar)
               : "memory");
}
__device__ __forceinline__ void tc_expect(uint32_t mbar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar), "r"(bytes) : "memory");
}

// C -= A B from pre-split tiles (passes 3: the 3xTF32 products; 1: hi x hi
// only, TF32-accurate); CTA (row tile, column tile of NH x 128 columns,
// batch); thread 0 runs the copy / MMA pipeline (stage s: the A hi / lo tiles
// and NH B hi / lo tiles of 8 KB, "full" barrier fb[s] completed by the bulk
// copies, "free" barrier mb[s] by the MMA commit), all four warps run the
// epilogue. NH = 1: 64 KB of shared memory, three CTAs per SM; NH = 2: one
// M 128 x N 256 MMA per K step (half the shared-memory operand traffic per
// multiply-add of two N 128 MMAs, whose A is read twice), 96 KB and two CTAs
// per SM (2 x 256 TMEM columns). Either way one CTA's epilogue overlaps
// another's MMAs. The B tiles of one column tile's two halves are adjacent
// 128-row blocks of the K-major layout (row group g at g x 512 B), so the
// 256-row operand is the two pre-split tiles copied back to back; a missing
// second half (n <= 128 in the last tile) is not copied and its columns,
// which only feed outputs j >= n, are never stored.
// (NH = 1: registers capped for three CTAs per SM, the shared-memory limit)
template <int NH>
__global__ void __launch_bounds__(128, NH == 1 ? 3 : 2) k_tc_cgemm_bulk(const uint32_t* Ahi, const uint32_t* Alo,
                                                          const uint32_t* Bhi, const uint32_t* Blo, int nmt, int nnt,
                                                          int nkc, float2* C, int ldc, long long sC, int m, int n,
                                                          int* err, long long spin, int passes) {
  constexpr int SB = (2 + 2 * NH) * TQ_TILE_BYTES;  // stage bytes
  constexpr int BN = TC_BN * NH;                     // columns per CTA (TMEM columns)
  extern __shared__ __align__(1024) unsigned char tsm[];
  uint64_t* bars = reinterpret_cast<uint64_t*>(tsm + 2 * SB);  // fb[2], mb[2]
  uint32_t* tslot = reinterpret_cast<uint32_t*>(tsm + 2 * SB + 32);
  __shared__ int s_ok;
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  const int mt = blockIdx.x, nt = blockIdx.y, bz = blockIdx.z;
  const int nh = min(NH, nnt - nt * NH);  // B halves present
  const size_t ta0 = ((size_t)bz * nmt + mt) * nkc * TQ_TW;  // first A tile of this row tile
  const size_t tb0 = ((size_t)bz * nnt + (size_t)nt * NH) * nkc * TQ_TW;
  const uint32_t fb[2] = {smem_u32(bars), smem_u32(bars + 1)}, mb[2] = {smem_u32(bars + 2), smem_u32(bars + 3)};
  const uint32_t st0 = smem_u32(tsm);
  if (t == 0) {
    for (int q = 0; q < 2; ++q) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(fb[q]) : "memory");
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mb[q]) : "memory");
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    s_ok = 1;
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)), "r"(BN)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tslot;
  const uint32_t idesc = tc_idesc(TC_BM, BN);
  int issued = 0;  // chunks whose MMAs were issued (the last commit covers all)
  int loaded = 0;  // chunks whose bulk copies were issued
  int landed = 0;  // chunks whose copies were waited for
  if (t == 0) {
    auto load = [&](int kc, int sidx) {
      const uint32_t d = st0 + sidx * SB;
      tc_expect(fb[sidx], (uint32_t)((2 + 2 * nh) * TQ_TILE_BYTES));
      tc_bulk(d, Ahi + ta0 + (size_t)kc * TQ_TW, TQ_TILE_BYTES, fb[sidx]);
      tc_bulk(d + TQ_TILE_BYTES, Alo + ta0 + (size_t)kc * TQ_TW, TQ_TILE_BYTES, fb[sidx]);
      for (int h = 0; h < nh; ++h) {
        const size_t tb = tb0 + ((size_t)h * nkc + kc) * TQ_TW;
        tc_bulk(d + (2 + h) * TQ_TILE_BYTES, Bhi + tb, TQ_TILE_BYTES, fb[sidx]);
        tc_bulk(d + (2 + NH + h) * TQ_TILE_BYTES, Blo + tb, TQ_TILE_BYTES, fb[sidx]);
      }
      loaded = kc + 1;
    };
    bool ok = true;
    if (nkc > 0) load(0, 0);
    for (int kc = 0; kc < nkc && ok; ++kc) {
      const int s = kc & 1;
      if (kc + 1 < nkc) {
        // stage s^1 was read by the MMAs of chunk kc - 1
        if (kc >= 1 && !tc_wait(mb[s ^ 1], (uint32_t)(((kc - 1) >> 1) & 1), spin)) { ok = false; break; }
        load(kc + 1, s ^ 1);
      }
      if (!tc_wait(fb[s], (uint32_t)((kc >> 1) & 1), spin)) { ok = false; break; }
      landed = kc + 1;
      const uint32_t ah = st0 + s * SB, al = ah + TQ_TILE_BYTES, bh = ah + 2 * TQ_TILE_BYTES,
                     bl = ah + (2 + NH) * TQ_TILE_BYTES;
#pragma unroll
      for (int ks = 0; ks < TQ / 8; ++ks) {
        const uint32_t ko = ks * 256;  // 8 tf32 = two core matrices along K
        const uint64_t dah = tq_desc(ah + ko), dal = tq_desc(al + ko), dbh = tq_desc(bh + ko), dbl = tq_desc(bl + ko);
        const uint32_t acc0 = (kc > 0 || ks > 0) ? 1u : 0u;
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(
                tmem),
            "l"(dah), "l"(dbh), "r"(idesc), "r"(acc0)
            : "memory");
        if (passes == 3) {
          asm volatile("tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, 1;" ::"r"(tmem), "l"(dah), "l"(dbl),
                       "r"(idesc)
                       : "memory");
          asm volatile("tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, 1;" ::"r"(tmem), "l"(dal), "l"(dbh),
                       "r"(idesc)
                       : "memory");
        }
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mb[s])
                   : "memory");
      issued = kc + 1;
    }
    // the last commit covers every earlier MMA
    if (ok && issued > 0 && !tc_wait(mb[(issued - 1) & 1], (uint32_t)(((issued - 1) >> 1) & 1), spin)) ok = false;
    if (!ok) {
      atomicExch(err, 1);
      s_ok = 0;
      // drain (full limit) before the shared memory and the TMEM are given up:
      // the MMAs issued so far, then the bulk copies not yet waited for
      if (issued > 0) tc_wait(mb[(issued - 1) & 1], (uint32_t)(((issued - 1) >> 1) & 1));
      for (int c = landed; c < loaded; ++c) tc_wait(fb[c & 1], (uint32_t)((c >> 1) & 1));
    }
  }
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (s_ok && nkc > 0) {
    const int r = 32 * warp + lane;
    const int i = mt * (TC_BM / 2) + (r >> 1), comp = r & 1;
    float2* Cb = C + sC * bz;
    for (int c0 = 0; c0 < nh * TC_BN; c0 += 32) {
      uint32_t v[32];
      const uint32_t ta = tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)c0;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,"
          "%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
          : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
            "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]),
            "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]),
            "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
          : "r"(ta)
          : "memory");
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      if (i < m) {
        // all loads first, then the stores (a load / store pair per element
        // would serialise 32 global round trips)
        float* cr = reinterpret_cast<float*>(Cb);
        float cv[32];
#pragma unroll
        for (int q = 0; q < 32; ++q) {
          const int j = nt * BN + c0 + q;
          cv[q] = j < n ? cr[2 * ((size_t)j * ldc + i) + comp] : 0.0f;
        }
#pragma unroll
        for (int q = 0; q < 32; ++q) {
          const int j = nt * BN + c0 + q;
          if (j < n) cr[2 * ((size_t)j * ldc + i) + comp] = cv[q] - __uint_as_float(v[q]);
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(BN) : "memory");
}
template <int NH>
constexpr int tc_smem_bulk() {
  return 2 * (2 + 2 * NH) * TQ_TILE_BYTES + 64;
}

}  // namespace mfb
