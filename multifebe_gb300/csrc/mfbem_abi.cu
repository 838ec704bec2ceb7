// C-ABI of the GB300 collocation-BEM library (see include/mfbem.h): handle
// management, the once-per-mesh device precompute, per-frequency assembly,
// and the dense solves. Single translation unit for all device code.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <type_traits>
#include <chrono>
#include <cmath>
#include <complex>
#include <map>
#include <mutex>
#include <thread>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/mfbem.h"
#include "bem_common.h"
#include "dev_complex.cuh"
#include "dev_point.cuh"
#include "mfbem_dev.h"
#include "mfbem_host.h"
#include "mfbem_precompute.cuh"
#include "mfbem_assemble.cuh"
#include "mfbem_internal.cuh"
#include "mfbem_hbie.cuh"
#include "mfbem_lu.cuh"
#include "mfbem_tc.cuh"
#include "mfbem_oz.cuh"

namespace mfb {
static thread_local std::string g_err;
// kernels of this library launched so far by the calling thread (reported
// per call in mfbem_stats; per thread so concurrent sweeps count their own)
static thread_local long long g_launches = 0;
// iteration limit of the bounded device waits (tcgen05 pipeline mbarriers,
// cooperative panel barrier); 0 keeps each kernel's own limit. Only the
// failure-detection test hook mfbem_internal_set_spin_limit changes it.
static std::atomic<long long> g_spin_limit{0};
void set_error(const std::string& s) { g_err = s; }
int fail(int code, const std::string& s) {
  g_err = s;
  return code;
}
}  // namespace mfb

using namespace mfb;

#define CK(call)                                                                                  \
  do {                                                                                            \
    cudaError_t e_ = (call);                                                                      \
    if (e_ != cudaSuccess) return fail(MFBEM_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)
// a library routine returning an MFBEM status: pass a failure on
#define CKG(call)                \
  do {                           \
    int rc_ = (call);            \
    if (rc_) return rc_;         \
  } while (0)

// A device buffer and the device ordinal it was allocated on.
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  int dev = -1;
};

struct mfbem_handle {
  DMesh m;
  // device ordinal the mesh was uploaded on; every call on the handle needs it current
  int dev = 0;
  std::vector<std::pair<void*, size_t>> owned;
  QsCurves* d_qs = nullptr;
  QsCurves* d_q15 = nullptr;
  int ndof = 0, ne = 0, nn = 0;
  // mixed solves: TF32 trailing updates stalled the refinement on this mesh
  // once, so later solves factorise with SIMT FP32 updates from the start
  bool tf32_stalled = false;
  // mixed solves: FP32 factors without row interchanges failed (zero pivot or
  // stalled refinement) on this mesh once, so later solves pivot from the start
  bool nopiv_failed = false;
  cudaStream_t st = nullptr;
  DevBuf A, b, A32, x, r, work, ipiv, info, par, nu, parf, pphi_f, geo_f, gm;
  mfbem_stats stats{};
  // systems of the last mfbem_sweep_harela call (read back by a test hook)
  int last_nf = 0;
  long long pts_reg = 0, pts_adp = 0, pts_sing = 0;
  int* d_err = nullptr;
  // internal points: element -> node (0-based), node position and the csize
  // of the node's first element (-1: node of no element)
  int* enode = nullptr;
  double* nodex = nullptr;
  double* nodecl = nullptr;
  // half-space region (mfbem_set_halfspace): hyperplane normal (0: full
  // space), coordinate; pair lists of the complementary kernel classified on
  // the images of the collocation points (built at the first static assembly)
  int hs_n = 0;
  double hs_x = 0.0;
  bool hs_built = false;
  DMesh mh;
  double* hs_c = nullptr;  // [ncp] x_i3 - hs_x
  long long hs_pts[3] = {0, 0, 0};
  // HBIE collocation (mfbem_mesh_upload_dual): mb, the view of the HBIE
  // points with their pair lists (1/r^7 classification), built at upload;
  // ms[0] / ms[1], the SBIE part of the Burton & Miller points classified
  // like sbie_auto (static) / shbie_auto (harmonic), built at the first
  // assembly of each kind from ms_base (points only)
  bool has_hbie = false, has_bm = false, has_crack = false;
  std::vector<char> crack_node;  // [nn] node of a crack-like boundary
  DMesh mb, ms_base, ms[2];
  bool ms_built[2] = {false, false};
  long long mb_pts[3] = {0, 0, 0}, ms_pts[2][3] = {{0, 0, 0}, {0, 0, 0}};
  DevBuf parh;  // HarParH per frequency of the last harmonic assembly
};

// ---------------------------------------------------------------------------
// Device memory released with a mesh handle is kept for the next handle: a
// caller that uploads, sweeps and releases mesh after mesh (or a harmonic
// driver re-uploading per call) would otherwise pay cudaMalloc / cudaFree of
// several GB per sweep, and cudaFree synchronises the device. Buffers of at
// least 1 MB are cached up to a cap (a quarter of the device memory, or
// MFBEM_DEVICE_CACHE_MB; 0 disables the cache); an allocation takes the
// smallest cached buffer that fits and is at most twice the request.
// mfbem_trim_device_cache() returns everything to the driver. Streams and
// streams of released meshes are reused the same way.
// ---------------------------------------------------------------------------
static std::mutex g_pool_mu;
// cached buffers: size -> (device ordinal, pointer); bytes and cap per device
static std::multimap<size_t, std::pair<int, void*>> g_pool;
static std::map<int, size_t> g_pool_bytes;
static std::map<int, long long> g_pool_cap;
// streams of released meshes: (device, stream)
static std::vector<std::pair<int, cudaStream_t>> g_ctx_pool;

static int cur_dev() {
  int d = 0;
  if (cudaGetDevice(&d) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return d;
}
// runs f with device `dev` current, then restores the caller's device
template <class F>
static void on_device(int dev, F f) {
  const int c = cur_dev();
  if (c != dev) cudaSetDevice(dev);
  f();
  if (c != dev) cudaSetDevice(c);
}
// cap of the cache of the current device (set on its first allocation)
static size_t pool_cap_current(int dev) {
  auto it = g_pool_cap.find(dev);
  if (it == g_pool_cap.end()) {
    long long cap = 0;
    const char* e = getenv("MFBEM_DEVICE_CACHE_MB");
    if (e) {
      cap = std::max(0LL, atoll(e)) << 20;
    } else {
      size_t fr = 0, tot = 0;
      cap = cudaMemGetInfo(&fr, &tot) == cudaSuccess ? (long long)(tot / 4) : 0;
      cudaGetLastError();
    }
    it = g_pool_cap.emplace(dev, cap).first;
  }
  return (size_t)it->second;
}
// a cached buffer of device dev of size in [bytes, 2 bytes], or nullptr; *cap receives its size
static void* pool_take(size_t bytes, int dev, size_t* cap) {
  std::lock_guard<std::mutex> lk(g_pool_mu);
  pool_cap_current(dev);
  for (auto it = g_pool.lower_bound(bytes); it != g_pool.end() && it->first <= 2 * bytes; ++it) {
    if (it->second.first != dev) continue;
    void* p = it->second.second;
    *cap = it->first;
    g_pool_bytes[dev] -= it->first;
    g_pool.erase(it);
    return p;
  }
  return nullptr;
}
// p (on device dev) is idle: the caller has synchronised that device
static void pool_give(void* p, size_t bytes, int dev) {
  if (!p) return;
  {
    std::lock_guard<std::mutex> lk(g_pool_mu);
    auto cap = g_pool_cap.find(dev);
    if (bytes >= (1u << 20) && cap != g_pool_cap.end() && g_pool_bytes[dev] + bytes <= (size_t)cap->second) {
      g_pool.emplace(bytes, std::make_pair(dev, p));
      g_pool_bytes[dev] += bytes;
      return;
    }
  }
  on_device(dev, [&]() { cudaFree(p); });
}
// frees the cached buffers of device dev (every device if dev < 0); g_pool_mu held
static void pool_drop_locked(int dev) {
  for (auto it = g_pool.begin(); it != g_pool.end();) {
    if (dev >= 0 && it->second.first != dev) {
      ++it;
      continue;
    }
    const int d = it->second.first;
    void* q = it->second.second;
    on_device(d, [&]() { cudaFree(q); });
    g_pool_bytes[d] -= it->first;
    it = g_pool.erase(it);
  }
}
static cudaError_t pool_malloc(void** p, size_t bytes, size_t* cap) {
  const int dev = cur_dev();
  if (bytes >= (1u << 20) && (*p = pool_take(bytes, dev, cap))) return cudaSuccess;
  *cap = bytes;
  cudaError_t e = cudaMalloc(p, bytes);
  if (e == cudaErrorMemoryAllocation) {
    // give this device's cache back to the driver and retry once
    cudaGetLastError();
    cudaDeviceSynchronize();
    std::lock_guard<std::mutex> lk(g_pool_mu);
    pool_drop_locked(dev);
    e = cudaMalloc(p, bytes);
  }
  return e;
}
extern "C" int mfbem_trim_device_cache(void) {
  std::lock_guard<std::mutex> lk(g_pool_mu);
  std::vector<int> devs;
  for (auto& kv : g_pool)
    if (std::find(devs.begin(), devs.end(), kv.second.first) == devs.end()) devs.push_back(kv.second.first);
  for (int d : devs) on_device(d, []() { cudaDeviceSynchronize(); });
  pool_drop_locked(-1);
  return 0;
}

static int dalloc(mfbem_handle* h, void** p, size_t bytes) {
  if (bytes == 0) bytes = 16;
  size_t cap = 0;
  cudaError_t e = pool_malloc(p, bytes, &cap);
  if (e != cudaSuccess) return fail(MFBEM_ENOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  h->owned.emplace_back(*p, cap);
  return 0;
}
template <typename T>
static int dupload(mfbem_handle* h, T** dst, const T* src, size_t n) {
  int rc = dalloc(h, (void**)dst, n * sizeof(T));
  if (rc) return rc;
  if (n) CK(cudaMemcpy(*dst, src, n * sizeof(T), cudaMemcpyHostToDevice));
  return 0;
}
// b holds at least `bytes` on the current device (a buffer of another device,
// or one too small, goes back to its device's cache first)
static int ensure(DevBuf& b, size_t bytes) {
  const int dev = cur_dev();
  if (b.p && b.dev == dev && b.bytes >= bytes) return 0;
  if (b.p) {
    // the stream that used it may still run: the cache only takes idle buffers
    on_device(b.dev, []() { cudaDeviceSynchronize(); });
    pool_give(b.p, b.bytes, b.dev);
  }
  b.p = nullptr;
  b.bytes = 0;
  size_t cap = 0;
  cudaError_t e = pool_malloc(&b.p, bytes, &cap);
  if (e != cudaSuccess) return fail(MFBEM_ENOMEM, std::string("cudaMalloc(work): ") + cudaGetErrorString(e));
  b.bytes = cap;
  b.dev = dev;
  return 0;
}
// calls on a handle run on the device it was uploaded on
static int check_dev(const mfbem_handle* h) {
  const int d = cur_dev();
  if (d != h->dev)
    return fail(MFBEM_EARG, "the mesh handle belongs to device " + std::to_string(h->dev) + " but device " +
                                std::to_string(d) + " is current: make its device current (cudaSetDevice) first");
  return 0;
}

static bool g_tables_ready = false;
static std::mutex g_tables_mu;
static int init_tables() {
  std::lock_guard<std::mutex> lk(g_tables_mu);
  if (g_tables_ready) return 0;
  const GLTables& t = host_gauss_tables();
  CK(cudaMemcpyToSymbol(c_gl, &t, sizeof(GLTables)));
  const DfConst dc = df_constants_host();
  CK(cudaMemcpyToSymbol(c_df, &dc, sizeof(DfConst)));
  g_tables_ready = true;
  return 0;
}

static inline unsigned nblk(long long n, int t) { return (unsigned)((n + t - 1) / t); }

extern "C" const char* mfbem_last_error(void) { return g_err.c_str(); }
extern "C" const char* mfbem_version(void) { return "mfbem-gb300 0.1 sm_103a"; }

// Classification of every (collocation point, element) pair of m and the
// pair lists, adaptive subdivision leaves and singular layouts built from it
// (m.cpx: the points the pairs are classified on); hoists the adaptive and
// singular point geometry when it fits. pts: regular / adaptive / singular
// quadrature points.
static int build_pairs(mfbem_handle* h, DMesh& m, long long pts[3]) {
  const int ncp = m.ncp, ne = m.ne;
  int rc;
  if ((rc = dalloc(h, (void**)&m.cls, (size_t)ncp * ne))) return rc;
  // a view may hold no points (every node of the region on another formulation)
  if (ncp > 0) { k_classify<<<std::min(nblk((long long)ncp * ne, 256), 152u * 16u), 256>>>(m, h->d_qs); ++g_launches; }
  // counts and list offsets
  int *nreg, *nadp, *nsing;
  long long* npts;
  if ((rc = dalloc(h, (void**)&nreg, sizeof(int) * ncp)) || (rc = dalloc(h, (void**)&nadp, sizeof(int) * ncp)) ||
      (rc = dalloc(h, (void**)&nsing, sizeof(int) * ncp)) || (rc = dalloc(h, (void**)&npts, sizeof(long long) * ncp)) ||
      (rc = dalloc(h, (void**)&m.reg_start, sizeof(int) * (ncp + 1))) ||
      (rc = dalloc(h, (void**)&m.adp_start, sizeof(int) * (ncp + 1))) ||
      (rc = dalloc(h, (void**)&m.sing_start, sizeof(int) * (ncp + 1)))) {
    return rc;
  }
  long long* pts_base;
  if ((rc = dalloc(h, (void**)&pts_base, sizeof(long long) * (ncp + 1)))) return rc;
  if (ncp > 0) { k_count<<<nblk(ncp, 8), 256>>>(m, nreg, nadp, nsing, npts); ++g_launches; }
  k_scan<int, int><<<1, 1024>>>(nreg, m.reg_start, ncp); ++g_launches;
  k_scan<int, int><<<1, 1024>>>(nadp, m.adp_start, ncp); ++g_launches;
  k_scan<int, int><<<1, 1024>>>(nsing, m.sing_start, ncp); ++g_launches;
  k_scan<long long, long long><<<1, 1024>>>(npts, pts_base, ncp); ++g_launches;
  CK(cudaGetLastError());
  int tot[3];
  long long totp;
  CK(cudaMemcpy(&tot[0], m.reg_start + ncp, sizeof(int), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(&tot[1], m.adp_start + ncp, sizeof(int), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(&tot[2], m.sing_start + ncp, sizeof(int), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(&totp, pts_base + ncp, sizeof(long long), cudaMemcpyDeviceToHost));
  m.nreg = tot[0];
  m.nadp = tot[1];
  m.nsing = tot[2];
  int *adp_cp, *sing_cp;
  if ((rc = dalloc(h, (void**)&m.reg_pair, sizeof(int) * (m.nreg + 1))) ||
      (rc = dalloc(h, (void**)&m.reg_pt, sizeof(long long) * (m.nreg + 1))) ||
      (rc = dalloc(h, (void**)&m.adp_e, sizeof(int) * (m.nadp + 1))) ||
      (rc = dalloc(h, (void**)&adp_cp, sizeof(int) * (m.nadp + 1))) ||
      (rc = dalloc(h, (void**)&m.sing_e, sizeof(int) * (m.nsing + 1))) ||
      (rc = dalloc(h, (void**)&sing_cp, sizeof(int) * (m.nsing + 1)))) {
    return rc;
  }
  if (ncp > 0) { k_fill<<<nblk(ncp, 8), 256>>>(m, pts_base, adp_cp, sing_cp); ++g_launches; }
  CK(cudaMemcpy(m.reg_pt + m.nreg, &totp, sizeof(long long), cudaMemcpyHostToDevice));
  pts[0] = totp;
  // adaptive subdivision leaves
  int* nl;
  if ((rc = dalloc(h, (void**)&nl, sizeof(int) * (m.nadp + 1))) ||
      (rc = dalloc(h, (void**)&m.adp_leaf, sizeof(int) * (m.nadp + 1)))) {
    return rc;
  }
  if (m.nadp > 0) k_adp_count<<<nblk(m.nadp, 64), 64>>>(m, h->d_qs, adp_cp, nl); ++g_launches;
  k_scan<int, int><<<1, 1024>>>(nl, m.adp_leaf, (int)m.nadp); ++g_launches;
  int nleaf = 0;
  CK(cudaMemcpy(&nleaf, m.adp_leaf + m.nadp, sizeof(int), cudaMemcpyDeviceToHost));
  m.nleaf = nleaf;
  long long* lpts;
  if ((rc = dalloc(h, (void**)&m.leaf, sizeof(double) * LEAF_D * (m.nleaf + 1))) ||
      (rc = dalloc(h, (void**)&m.leaf_gln, sizeof(int) * (m.nleaf + 1))) ||
      (rc = dalloc(h, (void**)&m.leaf_pair, sizeof(int) * (m.nleaf + 1))) ||
      (rc = dalloc(h, (void**)&m.leaf_pt, sizeof(long long) * (m.nleaf + 1))) ||
      (rc = dalloc(h, (void**)&lpts, sizeof(long long) * (m.nleaf + 1)))) {
    return rc;
  }
  if (m.nadp > 0) k_adp_fill<<<nblk(m.nadp, 64), 64>>>(m, h->d_qs, adp_cp); ++g_launches;
  if (m.nleaf > 0) k_leaf_points<<<nblk(m.nleaf, 256), 256>>>(m, lpts); ++g_launches;
  k_scan<long long, long long><<<1, 1024>>>(lpts, m.leaf_pt, (int)m.nleaf); ++g_launches;
  CK(cudaMemcpy(&pts[1], m.leaf_pt + m.nleaf, sizeof(long long), cudaMemcpyDeviceToHost));
  // singular pairs
  long long* spts;
  if ((rc = dalloc(h, (void**)&m.sing_d, sizeof(double) * SING_D * (m.nsing + 1))) ||
      (rc = dalloc(h, (void**)&m.sing_i, sizeof(int) * SING_I * (m.nsing + 1))) ||
      (rc = dalloc(h, (void**)&m.sing_pt, sizeof(long long) * (m.nsing + 1))) ||
      (rc = dalloc(h, (void**)&spts, sizeof(long long) * (m.nsing + 1)))) {
    return rc;
  }
  if (m.nsing > 0) k_sing_prep<<<nblk(m.nsing, 64), 64>>>(m, h->d_q15, sing_cp, spts); ++g_launches;
  if (m.hbie) {
    // HBIE view: n_i, psi_i and the edge line integrals of every singular pair
    if ((rc = dalloc(h, (void**)&m.hsing_x, sizeof(double) * HSING_X * (m.nsing + 1)))) return rc;
    if (m.nsing > 0) { k_hsing_prep<<<nblk(m.nsing, 64), 64>>>(m, h->d_q15); ++g_launches; }
  }
  k_scan<long long, long long><<<1, 1024>>>(spts, m.sing_pt, (int)m.nsing); ++g_launches;
  CK(cudaMemcpy(&pts[2], m.sing_pt + m.nsing, sizeof(long long), cudaMemcpyDeviceToHost));
  // hoist the singular / adaptive point geometry out of the frequency loop when
  // it fits a modest share of the device (22 / 14 doubles per point)
  m.adp_cp = adp_cp;
  m.nsing_pts = pts[2];
  m.nleaf_pts = pts[1];
  const size_t geo_budget = (size_t)8 << 30;
  if (m.nsing_pts > 0 && (size_t)m.nsing_pts * 22 * sizeof(double) <= geo_budget) {
    if ((rc = dalloc(h, (void**)&m.sing_geo, (size_t)m.nsing_pts * 22 * sizeof(double)))) return rc;
    k_sing_geo<<<nblk(m.nsing_pts, 128), 128>>>(m); ++g_launches;
  }
  if (m.nleaf_pts > 0 && (size_t)m.nleaf_pts * 14 * sizeof(double) <= geo_budget) {
    if ((rc = dalloc(h, (void**)&m.leaf_geo, (size_t)m.nleaf_pts * 14 * sizeof(double)))) return rc;
    k_leaf_geo<<<nblk(m.nleaf_pts, 128), 128>>>(m); ++g_launches;
  }
  return 0;
}

// ---------------------------------------------------------------------------
// upload + once-per-mesh precompute
// ---------------------------------------------------------------------------
// Collocation points of one view, sorted by DOF-order node (stable: the
// builders' collocation order within a node), uploaded into v's point arrays.
struct HostCP {
  double x[3], xi[2], n[3], alpha;
  int dn, kind, e, kn;
};
static int upload_points(mfbem_handle* h, std::vector<HostCP>& cps, int nn, DMesh& v) {
  std::stable_sort(cps.begin(), cps.end(), [](const HostCP& a, const HostCP& b) { return a.dn < b.dn; });
  const int ncp = (int)cps.size();
  std::vector<int> dn_cp(nn + 1, 0), cp_dn(ncp), cp_kind(ncp), cp_e(ncp), cp_kn(ncp);
  std::vector<double> cpx(3 * (size_t)ncp), cpxi(2 * (size_t)ncp), cpn(3 * (size_t)ncp), cpa(ncp);
  for (int i = 0; i < ncp; ++i) {
    const HostCP& c = cps[i];
    dn_cp[c.dn + 1]++;
    for (int q = 0; q < 3; ++q) {
      cpx[3 * i + q] = c.x[q];
      cpn[3 * i + q] = c.n[q];
    }
    cpxi[2 * i] = c.xi[0];
    cpxi[2 * i + 1] = c.xi[1];
    cp_dn[i] = c.dn;
    cp_kind[i] = c.kind;
    cp_e[i] = c.e;
    cp_kn[i] = c.kn;
    cpa[i] = c.alpha;
  }
  for (int i = 0; i < nn; ++i) dn_cp[i + 1] += dn_cp[i];
  double *dx, *dxi, *dnrm, *da;
  int *ddn, *dk, *de, *dkn, *ddc;
  int rc;
  if ((rc = dupload(h, &dx, cpx.data(), cpx.size())) || (rc = dupload(h, &dxi, cpxi.data(), cpxi.size())) ||
      (rc = dupload(h, &dnrm, cpn.data(), cpn.size())) || (rc = dupload(h, &da, cpa.data(), cpa.size())) ||
      (rc = dupload(h, &ddn, cp_dn.data(), cp_dn.size())) || (rc = dupload(h, &dk, cp_kind.data(), cp_kind.size())) ||
      (rc = dupload(h, &de, cp_e.data(), cp_e.size())) || (rc = dupload(h, &dkn, cp_kn.data(), cp_kn.size())) ||
      (rc = dupload(h, &ddc, dn_cp.data(), dn_cp.size())))
    return rc;
  v.ncp = ncp;
  v.cpx = dx;
  v.cp_xi = dxi;
  v.cp_n = dnrm;
  v.cp_alpha = da;
  v.cp_dn = ddn;
  v.cp_kind = dk;
  v.cp_elem = de;
  v.cp_kn = dkn;
  v.dn_cp = ddc;
  v.inc_start = nullptr;
  v.inc_el = nullptr;
  v.cls = nullptr;
  v.sing_geo = nullptr;
  v.leaf_geo = nullptr;
  v.hsing_x = nullptr;
  v.ft = nullptr;
  v.ft_ok = nullptr;
  return 0;
}

static int upload_impl(const mfbem_mesh_desc* d, const mfbem_dual_desc* dual, mfbem_handle** out);
extern "C" int mfbem_mesh_upload(const mfbem_mesh_desc* d, mfbem_handle** out) { return upload_impl(d, nullptr, out); }
extern "C" int mfbem_mesh_upload_dual(const mfbem_mesh_desc* d, const mfbem_dual_desc* dual, mfbem_handle** out) {
  if (!dual) return fail(MFBEM_EARG, "null dual descriptor");
  return upload_impl(d, dual, out);
}

static int upload_impl(const mfbem_mesh_desc* d, const mfbem_dual_desc* dual, mfbem_handle** out) {
  g_err.clear();
  if (!d || !out) return fail(MFBEM_EARG, "null argument");
  *out = nullptr;
  int dev_count = 0;
  if (cudaGetDeviceCount(&dev_count) != cudaSuccess || dev_count == 0) return fail(MFBEM_ECUDA, "no CUDA device");
  const int nn = d->n_nodes, ne = d->n_elements, ndof = d->n_dof;
  if (nn <= 0 || ne <= 0) return fail(MFBEM_EARG, "empty mesh");
  // crack-like boundaries: their elements and nodes (a node of one carries
  // both faces' unknowns and equations, six rows)
  std::vector<char> ckn(nn, 0);
  int ncrack = 0;
  if (dual && dual->crack_el) {
    if (!dual->ctype2 || !dual->cvalue2) return fail(MFBEM_EARG, "crack_el needs ctype2 and cvalue2");
    std::vector<char> ordn(nn, 0);
    for (int e = 0; e < ne; ++e)
      for (int k = 0; k < 8; ++k) {
        const int s = d->element_node[8 * e + k] - 1;
        if (s < 0 || s >= nn) return fail(MFBEM_EARG, "element_node out of range");
        (dual->crack_el[e] ? ckn : ordn)[s] = 1;
      }
    for (int s = 0; s < nn; ++s) {
      if (ckn[s] && ordn[s])
        return fail(MFBEM_EUNSUPPORTED, "node " + std::to_string(s + 1) +
                                            " belongs to a crack-like and an ordinary element");
      ncrack += ckn[s];
    }
  }
  if (ndof != 3 * nn + 3 * ncrack)
    return fail(MFBEM_EARG, "n_dof must be 3 per node (6 per crack-like node) for one BE region");
  if (d->n_precalsets < 1 || d->n_precalsets > 16) return fail(MFBEM_EARG, "n_precalsets out of range [1,16]");
  if (d->qsi_ns_max < 1 || d->qsi_ns_max > 17) return fail(MFBEM_EUNSUPPORTED, "qsi_ns_max must be in [1,17]");
  for (int i = 0; i < d->n_precalsets; ++i)
    if (d->precalset_gln[i] < 1 || d->precalset_gln[i] > 32 || (i && d->precalset_gln[i] <= d->precalset_gln[i - 1]))
      return fail(MFBEM_EARG, "precalset_gln must be increasing in [1,32]");
  int rc = init_tables();
  if (rc) return rc;
  mfbem_handle* h = new mfbem_handle();
  h->dev = cur_dev();
  h->ndof = ndof;
  h->ne = ne;
  h->nn = nn;
  DMesh& m = h->m;
  std::memset(&m, 0, sizeof(m));
  m.hs_ax = -1;
  m.fcls = m.fadp = 5;
  m.ne = ne;
  m.ndn = nn;
  m.ndof = ndof;
  m.nps = d->n_precalsets;
  m.ns_max = d->qsi_ns_max;
  m.ptot = 0;
  m.ps_gln_max = 0;
  for (int i = 0; i < m.nps; ++i) {
    m.ps_gln[i] = d->precalset_gln[i];
    m.ps_off[i] = m.ptot;
    m.ptot += d->precalset_gln[i] * d->precalset_gln[i];
    m.ps_gln_max = std::max(m.ps_gln_max, d->precalset_gln[i]);
  }
  m.geo_tol = d->geometric_tolerance;
  // --- host bookkeeping (topology only). DOF-order nodes ("dnodes") follow
  // the rows: an ordinary node takes rows r, r+1, r+2 with col == row; a node
  // of a crack-like boundary rows r..r+5, row(k,1) = r + 2(k-1) (SBIE),
  // row(k,2) = row(k,1) + 1 (HBIE) and face f's column of direction k at
  // row(k,1) + f - 1 (build_auxiliary_variables_mechanics_static.f90:146-207).
  std::vector<int> dn_of(nn, -1), rb(nn, 0), by_row(nn);
  for (int s = 0; s < nn; ++s) by_row[s] = s;
  std::stable_sort(by_row.begin(), by_row.end(), [&](int a, int b) { return d->row[3 * a] < d->row[3 * b]; });
  for (int i = 0, next = 1; i < nn; ++i) {
    const int s = by_row[i], r1 = d->row[3 * s], w = ckn[s] ? 2 : 1;
    if (r1 != next || d->row[3 * s + 1] != r1 + w || d->row[3 * s + 2] != r1 + 2 * w) {
      delete h;
      return fail(MFBEM_EARG, ckn[s] ? "the rows of a crack-like node must be r, r+2, r+4 after the previous node's"
                                     : "node rows must be node-wise consecutive triples");
    }
    next = r1 + 3 * w;
    dn_of[s] = i;
    rb[s] = r1 - 1;
    for (int k = 0; k < 3; ++k) {
      int ct = d->ctype[3 * s + k];
      int c = ct == 0 ? d->col[6 * s + 3 + k] : d->col[6 * s + k];
      if ((ct != 0 && ct != 1) || c != r1 + w * k) {
        delete h;
        return fail(MFBEM_EUNSUPPORTED, "only ctype 0/1 with col == row (BE boundary) is supported");
      }
      if (ckn[s] && dual->ctype2[3 * s + k] != 0 && dual->ctype2[3 * s + k] != 1) {
        delete h;
        return fail(MFBEM_EUNSUPPORTED, "ctype2 must be 0 or 1");
      }
    }
  }
  std::vector<int> edof(8 * (size_t)ne), rev(ne, 0);
  for (int e = 0; e < ne; ++e) {
    for (int k = 0; k < 8; ++k) {
      int s = d->element_node[8 * e + k] - 1;
      if (s < 0 || s >= nn) { delete h; return fail(MFBEM_EARG, "element_node out of range"); }
      edof[8 * e + k] = rb[s];
    }
    if (d->reversion) rev[e] = d->reversion[e] ? 1 : 0;
    if (ncrack && dual->crack_el[e]) {
      if (rev[e]) { delete h; return fail(MFBEM_EUNSUPPORTED, "a crack-like element cannot be reversed"); }
      rev[e] = 2;
    }
  }
  std::vector<int> dct(ndof);
  std::vector<double> dcv(2 * (size_t)ndof);
  for (int s = 0; s < nn; ++s)
    for (int k = 0; k < 3; ++k)
      for (int f = 0; f <= (int)ckn[s]; ++f) {
        const int dof = rb[s] + (ckn[s] ? 2 * k + f : k);
        const int* ct = f ? dual->ctype2 : d->ctype;
        const double* cv = f ? dual->cvalue2 : d->cvalue;
        dct[dof] = ct[3 * s + k];
        dcv[2 * dof] = cv[6 * s + 2 * k];
        dcv[2 * dof + 1] = cv[6 * s + 2 * k + 1];
      }
  // formulation per node: 0 SBIE, 1 HBIE alone, 2 Burton & Miller at common points,
  // 3 crack-like node (dual BEM), 4 Burton & Miller with the SBIE at its own point
  std::vector<int> form(nn, 0);
  if (dual) {
    if (!dual->hbie || !dual->dual || !dual->dual_is_common || !dual->alpha || !dual->xi_i_hbie || !dual->x_i_hbie ||
        !dual->n_i_hbie) {
      delete h;
      return fail(MFBEM_EARG, "null member of the dual descriptor");
    }
    for (int s = 0; s < nn; ++s) {
      const int hb = dual->hbie[s], du = dual->dual[s], co = dual->dual_is_common[s];
      if (ckn[s]) {
        // crack-like node: SBIE and HBIE at the same points, each its own
        // equation (fbem_dual_boundary, assign_default_bem_formulation.f90:94-128)
        if (hb != 1 || du != 2 || co != 1) {
          delete h;
          return fail(MFBEM_EARG, "node " + std::to_string(s + 1) +
                                      " of a crack-like boundary needs (hbie, dual, dual_is_common) = (1, 2, 1)");
        }
        form[s] = 3;
        continue;
      }
      if (hb == 0 && du == 0 && co == 0) form[s] = 0;
      else if (hb == 1 && du == 0 && co == 0) form[s] = 1;
      else if (hb == 1 && du == 1 && co == 1) form[s] = 2;
      else if (hb == 1 && du == 1 && co == 0) form[s] = 4;
      else {
        delete h;
        return fail(MFBEM_EUNSUPPORTED, "node " + std::to_string(s + 1) +
                                            ": only SBIE, 'hbie', 'dual_bm_same' and 'dual_bm_mixed' formulations are available");
      }
      if ((form[s] == 2 || form[s] == 4) && !std::isfinite(dual->alpha[s])) {
        delete h;
        return fail(MFBEM_EARG, "Burton & Miller alpha must be finite");
      }
    }
  }
  // collocation points in the builders' collocation order (SBIE view: nodes
  // with the SBIE formulation only)
  struct CP { double x[3], xi[2]; int dn, kind, e, kn; };
  std::vector<CP> cps;
  std::vector<char> col(nn, 0);
  for (int e = 0; e < ne; ++e)
    for (int k = 0; k < 8; ++k) {
      int s = d->element_node[8 * e + k] - 1;
      if (form[s] != 0 && form[s] != 4) continue;  // 'dual_bm_mixed': SBIE here, HBIE in its view
      CP c;
      c.dn = dn_of[s];
      c.e = e;
      c.kn = k;
      if (d->sbie[s] == 0) {
        if (col[s]) continue;
        col[s] = 1;
        c.kind = 0;
        for (int q = 0; q < 3; ++q) c.x[q] = d->x_gn[24 * (size_t)e + 3 * k + q];
        c.xi[0] = q8xi(k, 0);
        c.xi[1] = q8xi(k, 1);
      } else {
        c.kind = 1;
        for (int q = 0; q < 3; ++q) c.x[q] = d->x_i_sbie_mca[24 * (size_t)e + 3 * k + q];
        c.xi[0] = d->xi_i_sbie_mca[16 * (size_t)e + 2 * k];
        c.xi[1] = d->xi_i_sbie_mca[16 * (size_t)e + 2 * k + 1];
      }
      cps.push_back(c);
    }
  std::stable_sort(cps.begin(), cps.end(), [](const CP& a, const CP& b) { return a.dn < b.dn; });
  const int ncp = (int)cps.size();
  m.ncp = ncp;
  std::vector<int> dn_cp(nn + 1, 0);
  for (auto& c : cps) dn_cp[c.dn + 1]++;
  for (int i = 0; i < nn; ++i) dn_cp[i + 1] += dn_cp[i];
  std::vector<double> cpx(3 * (size_t)ncp), cpxi(2 * (size_t)ncp);
  std::vector<int> cp_dn(ncp), cp_kind(ncp), cp_e(ncp), cp_kn(ncp);
  // node -> incident (element, local) in element order
  std::vector<std::vector<int>> inc(nn);
  for (int e = 0; e < ne; ++e)
    for (int k = 0; k < 8; ++k) inc[d->element_node[8 * e + k] - 1].push_back(8 * e + k);
  std::vector<int> node_of_dn(nn);
  for (int s = 0; s < nn; ++s) node_of_dn[dn_of[s]] = s;
  std::vector<int> inc_start(ncp + 1, 0), inc_el;
  for (int i = 0; i < ncp; ++i) {
    const CP& c = cps[i];
    for (int q = 0; q < 3; ++q) cpx[3 * i + q] = c.x[q];
    cpxi[2 * i] = c.xi[0];
    cpxi[2 * i + 1] = c.xi[1];
    cp_dn[i] = c.dn;
    cp_kind[i] = c.kind;
    cp_e[i] = c.e;
    cp_kn[i] = c.kn;
    if (c.kind == 0)
      for (int v : inc[node_of_dn[c.dn]]) inc_el.push_back(v);
    inc_start[i + 1] = (int)inc_el.size();
  }
  // --- device arrays
  double *ex, *cl, *ball, *dcvd, *cpxd, *cpxid, *ngn, *tbp;
  int *gln, *revd, *edofd, *dctd, *cpdn, *cpk, *cpe, *cpkn, *dncp, *incs, *ince;
  if ((rc = dupload(h, &ex, d->x_gn, 24 * (size_t)ne)) || (rc = dupload(h, &cl, d->csize, (size_t)ne)) ||
      (rc = dupload(h, &gln, d->n_phi, (size_t)ne)) || (rc = dupload(h, &ball, d->bball, 4 * (size_t)ne)) ||
      (rc = dupload(h, &revd, rev.data(), rev.size())) || (rc = dupload(h, &edofd, edof.data(), edof.size())) ||
      (rc = dupload(h, &dctd, dct.data(), dct.size())) || (rc = dupload(h, &dcvd, dcv.data(), dcv.size())) ||
      (rc = dupload(h, &cpxd, cpx.data(), cpx.size())) || (rc = dupload(h, &cpxid, cpxi.data(), cpxi.size())) ||
      (rc = dupload(h, &cpdn, cp_dn.data(), cp_dn.size())) || (rc = dupload(h, &cpk, cp_kind.data(), cp_kind.size())) ||
      (rc = dupload(h, &cpe, cp_e.data(), cp_e.size())) || (rc = dupload(h, &cpkn, cp_kn.data(), cp_kn.size())) ||
      (rc = dupload(h, &dncp, dn_cp.data(), dn_cp.size())) || (rc = dupload(h, &incs, inc_start.data(), inc_start.size())) ||
      (rc = dupload(h, &ince, inc_el.data(), inc_el.size())) || (rc = dupload(h, &ngn, d->n_gn, 24 * (size_t)ne)) ||
      (rc = dupload(h, &tbp, d->tbp_gn, 24 * (size_t)ne))) {
    mfbem_mesh_release(h);
    return rc;
  }
  {
    std::vector<int> en(8 * (size_t)ne);
    std::vector<double> nx(3 * (size_t)nn, 0.0), ncl(nn, -1.0);
    for (int e = 0; e < ne; ++e)
      for (int k = 0; k < 8; ++k) {
        const int s = d->element_node[8 * e + k] - 1;
        en[8 * e + k] = s;
        if (ncl[s] < 0.0) {
          ncl[s] = d->csize[e];
          for (int q = 0; q < 3; ++q) nx[3 * s + q] = d->x_gn[24 * (size_t)e + 3 * k + q];
        }
      }
    if ((rc = dupload(h, &h->enode, en.data(), en.size())) || (rc = dupload(h, &h->nodex, nx.data(), nx.size())) ||
        (rc = dupload(h, &h->nodecl, ncl.data(), ncl.size()))) {
      mfbem_mesh_release(h);
      return rc;
    }
  }
  m.ex = ex; m.cl = cl; m.gln_far = gln; m.ball = ball; m.rev = revd; m.edof = edofd;
  m.dct = dctd; m.dcv = dcvd; m.cpx = cpxd; m.cp_xi = cpxid; m.cp_dn = cpdn; m.cp_kind = cpk;
  m.cp_elem = cpe; m.cp_kn = cpkn; m.dn_cp = dncp; m.inc_start = incs; m.inc_el = ince;
  m.n_gn = ngn; m.tbp_gn = tbp;
  // rows of each dnode's equations when crack-like nodes break the 3 dn + il
  // layout: SBIE rows (this view and the SBIE part) and HBIE rows
  int* dn_rb_h = nullptr;
  if (ncrack) {
    std::vector<int> rs(nn), rh(nn);
    for (int s = 0; s < nn; ++s) {
      rs[dn_of[s]] = (rb[s] << 1) | ckn[s];
      rh[dn_of[s]] = ((rb[s] + ckn[s]) << 1) | ckn[s];
    }
    int* dn_rb_s = nullptr;
    if ((rc = dupload(h, &dn_rb_s, rs.data(), rs.size())) || (rc = dupload(h, &dn_rb_h, rh.data(), rh.size()))) {
      mfbem_mesh_release(h);
      return rc;
    }
    m.dn_rb = dn_rb_s;
  }
  QsCurves q = qs_curves(d->qsi_relative_error), q15 = qs_curves(1e-15);
  if ((rc = dupload(h, &h->d_qs, &q, 1)) || (rc = dupload(h, &h->d_q15, &q15, 1)) ||
      (rc = dalloc(h, (void**)&m.px, 3 * sizeof(double) * (size_t)ne * m.ptot)) ||
      (rc = dalloc(h, (void**)&m.pn, 3 * sizeof(double) * (size_t)ne * m.ptot)) ||
      (rc = dalloc(h, (void**)&m.pphi, 8 * sizeof(double) * (size_t)ne * m.ptot)) ||
      (rc = dalloc(h, (void**)&m.ft, sizeof(double) * FT_D * (size_t)ncp)) ||
      (rc = dalloc(h, (void**)&m.ft_ok, sizeof(int) * (size_t)ncp)) ||
      (rc = dalloc(h, (void**)&h->d_err, sizeof(int)))) {
    mfbem_mesh_release(h);
    return rc;
  }
  auto t0 = std::chrono::steady_clock::now();
  k_datasets<<<ne, 128>>>(m); ++g_launches;
  long long pts[3] = {0, 0, 0};
  if ((rc = build_pairs(h, m, pts))) { mfbem_mesh_release(h); return rc; }
  h->pts_reg = pts[0];
  h->pts_adp = pts[1];
  h->pts_sing = pts[2];
  if (ncp > 0) { k_ft_prep<<<nblk(ncp, 128), 128>>>(m); ++g_launches; }
  // HBIE view and the Burton & Miller points' SBIE part
  if (dual) {
    std::vector<HostCP> hb, bm;
    for (int e = 0; e < ne; ++e)
      for (int k = 0; k < 8; ++k) {
        const int s = d->element_node[8 * e + k] - 1;
        if (form[s] == 0) continue;
        HostCP c;
        const double sg = (rev[e] & 1) ? -1.0 : 1.0;
        for (int q = 0; q < 3; ++q) {
          c.x[q] = dual->x_i_hbie[24 * (size_t)e + 3 * k + q];
          c.n[q] = sg * dual->n_i_hbie[24 * (size_t)e + 3 * k + q];
        }
        c.xi[0] = dual->xi_i_hbie[16 * (size_t)e + 2 * k];
        c.xi[1] = dual->xi_i_hbie[16 * (size_t)e + 2 * k + 1];
        if (on_quad_edge(c.xi[0], c.xi[1])) {
          mfbem_mesh_release(h);
          return fail(MFBEM_EARG, "the HBIE cannot be collocated at an element edge (xi_i_hbie on the edge)");
        }
        c.alpha = (form[s] == 2 || form[s] == 4) ? dual->alpha[s] : 1.0;
        c.dn = dn_of[s];
        c.kind = form[s] == 1 ? 2 : (form[s] == 2 ? 3 : (form[s] == 3 ? 4 : 5));
        c.e = e;
        c.kn = k;
        hb.push_back(c);
        if (form[s] == 2 || form[s] == 3) {
          // the SBIE part (Burton & Miller) or equation (crack-like node)
          c.kind = 1;
          bm.push_back(c);
        }
      }
    h->has_hbie = true;
    h->has_bm = !bm.empty();
    h->has_crack = ncrack > 0;
    if (ncrack) h->crack_node = ckn;
    h->mb = m;
    if (ncrack) h->mb.dn_rb = dn_rb_h;
    if ((rc = upload_points(h, hb, nn, h->mb))) { mfbem_mesh_release(h); return rc; }
    h->mb.fcls = h->mb.fadp = 7;
    h->mb.hbie = 1;
    if ((rc = build_pairs(h, h->mb, h->mb_pts))) { mfbem_mesh_release(h); return rc; }
    if (h->has_bm) {
      h->ms_base = m;
      if ((rc = upload_points(h, bm, nn, h->ms_base))) { mfbem_mesh_release(h); return rc; }
      h->ms_base.fadp = 5;
    }
  }
  CK(cudaGetLastError());
  CK(cudaDeviceSynchronize());
  auto t1 = std::chrono::steady_clock::now();
  h->stats.pairs_regular = m.nreg;
  h->stats.pairs_adaptive = m.nadp;
  h->stats.pairs_singular = m.nsing;
  h->stats.points_regular = h->pts_reg;
  h->stats.points_adaptive = h->pts_adp;
  h->stats.points_singular = h->pts_sing;
  h->stats.adaptive_leaves = (int)m.nleaf;
  h->stats.ms_assemble = std::chrono::duration<double, std::milli>(t1 - t0).count();
  {
    std::lock_guard<std::mutex> lk(g_pool_mu);
    for (size_t i = g_ctx_pool.size(); i-- > 0;)
      if (g_ctx_pool[i].first == h->dev) {
        h->st = g_ctx_pool[i].second;
        g_ctx_pool.erase(g_ctx_pool.begin() + i);
        break;
      }
  }
  if (!h->st) CK(cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking));
  *out = h;
  return 0;
}

extern "C" int mfbem_mesh_release(mfbem_handle* h) {
  if (!h) return MFBEM_EARG;
  on_device(h->dev, [&]() {
    cudaDeviceSynchronize();
    for (auto& o : h->owned) pool_give(o.first, o.second, h->dev);
    for (DevBuf* b : {&h->A, &h->b, &h->A32, &h->x, &h->r, &h->work, &h->ipiv, &h->info, &h->par, &h->nu, &h->parf,
                      &h->pphi_f, &h->geo_f, &h->gm, &h->parh})
      pool_give(b->p, b->bytes, b->dev);
    if (h->st) {
      std::lock_guard<std::mutex> lk(g_pool_mu);
      g_ctx_pool.emplace_back(h->dev, h->st);
    }
  });
  delete h;
  return 0;
}

extern "C" int mfbem_set_halfspace(mfbem_handle* h, int32_t n, double x, int32_t bc) {
  g_err.clear();
  if (!h) return fail(MFBEM_EARG, "null argument");
  if (n != 0 && h->has_hbie)
    return fail(MFBEM_EUNSUPPORTED, "HBIE formulations in a half-space region are not available");
  if (n < -3 || n > 3) return fail(MFBEM_EARG, "half-space hyperplane normal must be in -3..3 (0: full space)");
  if (n != 0 && bc != 1)
    return fail(MFBEM_EUNSUPPORTED, "only the traction-free half-space surface (bc = 1) is available");
  if (!std::isfinite(x)) return fail(MFBEM_EARG, "half-space hyperplane coordinate must be finite");
  if (n != h->hs_n || x != h->hs_x) h->hs_built = false;
  h->hs_n = n;
  h->hs_x = x;
  h->m.hs_ax = n == 0 ? -1 : std::abs(n) - 1;
  h->m.hs_x = x;
  return 0;
}

// Test hook: pair counts of the half-space complementary kernel (regular,
// adaptive, singular pairs, adaptive leaves; regular, adaptive, singular
// points), after the first static assembly of a half-space region.
extern "C" int mfbem_internal_hs_counts(mfbem_handle* h, long long* out) {
  if (!h || !out) return fail(MFBEM_EARG, "null argument");
  if (!h->hs_built) return fail(MFBEM_EARG, "no half-space pair lists built");
  out[0] = h->mh.nreg;
  out[1] = h->mh.nadp;
  out[2] = h->mh.nsing;
  out[3] = h->mh.nleaf;
  out[4] = h->hs_pts[0];
  out[5] = h->hs_pts[1];
  out[6] = h->hs_pts[2];
  return 0;
}

extern "C" int mfbem_last_stats(mfbem_handle* h, mfbem_stats* s) {
  if (!h || !s) return fail(MFBEM_EARG, "null argument");
  *s = h->stats;
  return 0;
}

// ---------------------------------------------------------------------------
// assembly into device buffers (nf systems: A at A + f*astride, b at b + f*bstride)
// ---------------------------------------------------------------------------
__global__ void k_harpar(const double* in /*nf x {lre,lim,mre,mim,rho,omega}*/, int nf, HarParD* out,
                         ZexpSteps steps) {
  int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nf) return;
  const double* q = in + 6 * f;
  HarParD p = harela_params(mk(q[0], q[1]), mk(q[2], q[3]), q[4], q[5]);
  p.steps = steps;
  out[f] = p;
}

// Pair lists of the half-space complementary kernel (static builder, plane
// x3 = hs_x): the collocation points' images classified against every element
// like the full-space pairs, once per mesh and hyperplane.
static int hs_prepare_static(mfbem_handle* h) {
  if (h->hs_n == 0 || h->hs_built) return 0;
  if (h->hs_n != -3)
    return fail(MFBEM_EUNSUPPORTED, "the static half-space kernel needs the hyperplane normal n = -3");
  const DMesh& m = h->m;
  DMesh& mh = h->mh;
  mh = m;
  mh.cls = nullptr;
  mh.sing_geo = nullptr;
  mh.leaf_geo = nullptr;
  int rc;
  double* img;
  if ((rc = dalloc(h, (void**)&img, 3 * sizeof(double) * (size_t)m.ncp)) ||
      (rc = dalloc(h, (void**)&h->hs_c, sizeof(double) * (size_t)m.ncp)))
    return rc;
  CK(cudaDeviceSynchronize());
  k_hs_image<<<nblk(m.ncp, 128), 128>>>(m.cpx, m.ncp, h->hs_x, img, h->hs_c); ++g_launches;
  mh.cpx = img;
  if ((rc = build_pairs(h, mh, h->hs_pts))) return rc;
  CK(cudaMemset(h->d_err, 0, sizeof(int)));
  k_hs_check<<<nblk(8LL * m.ne + m.ncp + mh.nsing, 256), 256>>>(mh, h->hs_c, h->hs_x, h->d_err); ++g_launches;
  int e = 0;
  CK(cudaMemcpy(&e, h->d_err, sizeof(int), cudaMemcpyDeviceToHost));
  CK(cudaDeviceSynchronize());
  if (e & 1) return fail(MFBEM_EGEOMETRY, "a node or collocation point lies outside the half-space");
  if (e & 2)
    return fail(MFBEM_EGEOMETRY, "an element holding a collocation point of the free surface does not lie on it");
  h->hs_built = true;
  return 0;
}

// Pair lists of the Burton & Miller points' SBIE part for the static (0) or
// harmonic (1) builder: sbie_auto's classification (1/r^5 estimate) or
// shbie_auto's (the HBIE's 1/r^7 estimate, bem_harela3d.f90:4888-4957); both
// subdivide adaptive pairs with the SBIE's own estimate. Built once per kind.
static int bm_prepare(mfbem_handle* h, int kind) {
  if (!h->has_bm || h->ms_built[kind]) return 0;
  CK(cudaDeviceSynchronize());
  DMesh& v = h->ms[kind];
  v = h->ms_base;
  v.fcls = kind ? 7 : 5;
  v.fadp = 5;
  int rc = build_pairs(h, v, h->ms_pts[kind]);
  if (rc) return rc;
  CK(cudaDeviceSynchronize());
  h->ms_built[kind] = true;
  return 0;
}

// Test hook: pair counts of the HBIE view (regular, adaptive, singular pairs,
// adaptive leaves; regular, adaptive, singular points), then those of the
// Burton & Miller SBIE view of the static and the harmonic builder (zeros
// until built).
extern "C" int mfbem_internal_hbie_counts(mfbem_handle* h, long long* out) {
  if (!h || !out) return fail(MFBEM_EARG, "null argument");
  if (!h->has_hbie) return fail(MFBEM_EARG, "no HBIE collocation points");
  const DMesh* v[3] = {&h->mb, &h->ms[0], &h->ms[1]};
  const long long* p[3] = {h->mb_pts, h->ms_pts[0], h->ms_pts[1]};
  for (int i = 0; i < 3; ++i) {
    const bool b = i == 0 || h->ms_built[i - 1];
    out[7 * i + 0] = b ? v[i]->nreg : 0;
    out[7 * i + 1] = b ? v[i]->nadp : 0;
    out[7 * i + 2] = b ? v[i]->nsing : 0;
    out[7 * i + 3] = b ? v[i]->nleaf : 0;
    for (int j = 0; j < 3; ++j) out[7 * i + 4 + j] = b ? p[i][j] : 0;
  }
  return 0;
}

// Assembly kernels in a fixed order (regular, adaptive, singular, free terms);
// per-kernel device times are recorded with events on the library's stream.
struct AsmTimes {
  cudaEvent_t ev[5];
  bool live = false;
  AsmTimes() {
    for (auto& e : ev) cudaEventCreate(&e);
    live = true;
  }
  ~AsmTimes() {
    if (live)
      for (auto& e : ev) cudaEventDestroy(e);
  }
  void read(mfbem_stats* s) {
    float t[4] = {0, 0, 0, 0};
    for (int i = 0; i < 4; ++i) cudaEventElapsedTime(&t[i], ev[i], ev[i + 1]);
    s->ms_regular = t[0];
    s->ms_adaptive = t[1];
    s->ms_singular = t[2];
    s->ms_free = t[3];
  }
};

template <class POL>
static int launch_assembly(mfbem_handle* h, const POL& pol, const double* d_nu, int nf, double* A, size_t lda,
                           size_t astride, double* b, size_t bstride, AsmTimes* tm = nullptr,
                           const HarParF* pf = nullptr, const ff* dsf = nullptr, bool mixed = false,
                           const ff* sgf = nullptr, const ff* lgf = nullptr) {
  const DMesh& m = h->m;
  constexpr int WPB = 4;
  long long nw = (long long)m.ndn * nf;
  // the double-float kernels write rows 3 dn + il: a region with crack-like
  // boundaries (six rows per crack node) assembles in binary64 only
  if (h->has_crack) mixed = false;
  unsigned g = nblk(nw, WPB);
  // static half-space region: the complementary kernel's pairs follow each
  // full-space stage and add into the same rows
  constexpr bool kStatic = std::is_same<POL, PolStatic>::value;
  const bool hs = kStatic && h->hs_built && h->hs_n == -3;
  const DMesh& mh = h->mh;
  // HBIE points (their own view) and the SBIE part of the Burton & Miller
  // points (the view of this builder's classification)
  const bool hb = h->has_hbie;
  const bool bm = h->has_bm && h->ms_built[kStatic ? 0 : 1];
  if (h->has_bm && !bm) return fail(MFBEM_EARG, "Burton & Miller pair lists not prepared");
  const DMesh& mb = h->mb;
  const DMesh& msv = h->ms[kStatic ? 0 : 1];
  typedef typename std::conditional<kStatic, PolHbieStatic, PolHbieHarmonic>::type PolH;
  typedef typename std::conditional<kStatic, HsStatic, HsHarmonic>::type HsK;
  PolH phb{};
  HsK hsk{};
  if (hb) {
    if constexpr (kStatic) {
      phb = hbie_static_policy(pol.mu, pol.nu);
      hsk.nu = phb.nu; hsk.cted1 = phb.cted1; hsk.cted2 = phb.cted2;
      hsk.ctes1 = phb.ctes1; hsk.ctes2 = phb.ctes2; hsk.ctes3 = phb.ctes3;
    } else {
      if (!pol.ph) return fail(MFBEM_EARG, "HBIE points need the d* / s* parameters");
      phb.p = pol.p;
      phb.ph = pol.ph;
      hsk.p = pol.p;
      hsk.ph = pol.ph;
    }
    phb.cpn = mb.cp_n;
    phb.cpa = mb.cp_alpha;
    phb.cpk = mb.cp_kind;
  }
  PolHsc ph{};
  PolHscSing phs{};
  if constexpr (kStatic) {
    ph.k = pol.k;
    ph.c = h->hs_c;
    ph.xp = h->hs_x;
    ph.nu = pol.nu;
    phs.k = pol.k;
    phs.c = h->hs_c;
    phs.nu = pol.nu;
  }
  CK(cudaMemsetAsync(h->d_err, 0, sizeof(int), h->st));
  if (tm) cudaEventRecord(tm->ev[0], h->st);
  if (m.nreg > 0) {
    if constexpr (std::is_same<POL, PolHarmonic>::value) {
      if (mixed && pf && dsf) {
        k_mixed<MIX_REG, WPB><<<g, WPB * 32, 0, h->st>>>(m, pf, dsf, nullptr, nf, (double2*)A, lda, astride / 2, b,
                                                         bstride);
      } else {
        k_reg<POL, WPB><<<g, WPB * 32, 0, h->st>>>(m, pol, nf, A, lda, astride, b, bstride);
      }
    } else {
      k_reg<POL, WPB><<<g, WPB * 32, 0, h->st>>>(m, pol, nf, A, lda, astride, b, bstride);
    }
    ++g_launches;
  }
  if constexpr (kStatic) {
    if (hs && mh.nreg > 0) {
      k_reg<PolHsc, WPB><<<g, WPB * 32, 0, h->st>>>(mh, ph, nf, A, lda, astride, b, bstride);
      ++g_launches;
    }
  }
  if (bm && msv.nreg > 0) {
    k_reg<POL, WPB><<<g, WPB * 32, 0, h->st>>>(msv, pol, nf, A, lda, astride, b, bstride);
    ++g_launches;
  }
  if (hb && mb.nreg > 0) {
    k_reg<PolH, WPB><<<g, WPB * 32, 0, h->st>>>(mb, phb, nf, A, lda, astride, b, bstride);
    ++g_launches;
  }
  if (tm) cudaEventRecord(tm->ev[1], h->st);
  if (m.nadp > 0) {
    if (mixed && lgf)
      k_mixed<MIX_ADP, WPB><<<g, WPB * 32, 0, h->st>>>(m, pf, dsf, lgf, nf, (double2*)A, lda, astride / 2, b, bstride);
    else k_adp<POL, WPB><<<g, WPB * 32, 0, h->st>>>(m, pol, nf, A, lda, astride, b, bstride);
    ++g_launches;
  }
  if constexpr (kStatic) {
    if (hs && mh.nadp > 0) {
      k_adp<PolHsc, WPB><<<g, WPB * 32, 0, h->st>>>(mh, ph, nf, A, lda, astride, b, bstride);
      ++g_launches;
    }
  }
  if (bm && msv.nadp > 0) {
    k_adp<POL, WPB><<<g, WPB * 32, 0, h->st>>>(msv, pol, nf, A, lda, astride, b, bstride);
    ++g_launches;
  }
  if (hb && mb.nadp > 0) {
    k_adp<PolH, WPB><<<g, WPB * 32, 0, h->st>>>(mb, phb, nf, A, lda, astride, b, bstride);
    ++g_launches;
  }
  if (tm) cudaEventRecord(tm->ev[2], h->st);
  // the singular kernels keep two combo sets per point: 2 warps per block
  if (m.nsing > 0) {
    if (mixed && sgf)
      k_mixed<MIX_SING, 2><<<nblk(nw, 2), 64, 0, h->st>>>(m, pf, dsf, sgf, nf, (double2*)A, lda, astride / 2, b, bstride);
    else k_sing<POL, 2><<<nblk(nw, 2), 64, 0, h->st>>>(m, pol, nf, A, lda, astride, b, bstride);
    ++g_launches;
  }
  if constexpr (kStatic) {
    if (hs && mh.nsing > 0) {
      k_sing<PolHscSing, 2><<<nblk(nw, 2), 64, 0, h->st>>>(mh, phs, nf, A, lda, astride, b, bstride);
      ++g_launches;
    }
  }
  if (bm && msv.nsing > 0) {
    k_sing<POL, 2><<<nblk(nw, 2), 64, 0, h->st>>>(msv, pol, nf, A, lda, astride, b, bstride);
    ++g_launches;
  }
  if (hb && mb.nsing > 0) {
    k_hsing<HsK><<<(unsigned)nw, 32, 0, h->st>>>(mb, hsk, nf, A, lda, astride, b, bstride);
    ++g_launches;
  }
  if (tm) cudaEventRecord(tm->ev[3], h->st);
  k_free<POL><<<nblk(nw, 128), 128, 0, h->st>>>(m, pol, d_nu, nf, A, lda, astride, b, bstride, h->d_err); ++g_launches;
  if (hb) {
    const HarParH* pph = nullptr;
    if constexpr (!kStatic) pph = pol.ph;
    k_hfree<typename POL::T><<<nblk(nw, 128), 128, 0, h->st>>>(mb, pph, nf, A, lda, astride, b, bstride);
    ++g_launches;
  }
  if (tm) cudaEventRecord(tm->ev[4], h->st);
  CK(cudaGetLastError());
  return 0;
}

static int check_err(mfbem_handle* h) {
  int e = 0;
  CK(cudaMemcpyAsync(&e, h->d_err, sizeof(int), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  if (e) return fail(MFBEM_EGEOMETRY, "the normals/tangents configuration at a free-term node is not valid");
  return 0;
}

// host <-> device copies of a column-major lda-strided matrix
static int copy_mat(void* dst, size_t dpitch, const void* src, size_t spitch, size_t rows_bytes, size_t cols,
                    cudaMemcpyKind kind, cudaStream_t st) {
  CK(cudaMemcpy2DAsync(dst, dpitch, src, spitch, rows_bytes, cols, kind, st));
  return 0;
}

template <bool CPLX>
static int assemble_common(mfbem_handle* h, const void* polp, const double* nu_host, double* A, int lda, double* b,
                           int flags) {
  const int n = h->ndof;
  if (lda < n) return fail(MFBEM_EARG, "lda < n_dof");
  if (int rd = check_dev(h)) return rd;
  const size_t es = CPLX ? 16 : 8;
  int rc;
  if ((rc = ensure(h->nu, 2 * sizeof(double)))) return rc;
  CK(cudaMemcpyAsync(h->nu.p, nu_host, 2 * sizeof(double), cudaMemcpyHostToDevice, h->st));
  double *dA, *db;
  size_t dlda;
  const bool dev = flags & MFBEM_DEVICE_PTRS;
  if (dev) {
    dA = A;
    db = b;
    dlda = lda;
    if (flags & MFBEM_OVERWRITE) {
      CK(cudaMemset2DAsync(dA, (size_t)lda * es, 0, n * es, n, h->st));
      CK(cudaMemsetAsync(db, 0, n * es, h->st));
    }
  } else {
    if ((rc = ensure(h->A, (size_t)n * n * es)) || (rc = ensure(h->b, n * es))) return rc;
    h->last_nf = 0;  // the sweep systems are overwritten
    dA = (double*)h->A.p;
    db = (double*)h->b.p;
    dlda = n;
    if (flags & MFBEM_OVERWRITE) {
      CK(cudaMemsetAsync(dA, 0, (size_t)n * n * es, h->st));
      CK(cudaMemsetAsync(db, 0, n * es, h->st));
    } else {
      if ((rc = copy_mat(dA, n * es, A, (size_t)lda * es, n * es, n, cudaMemcpyHostToDevice, h->st))) return rc;
      CK(cudaMemcpyAsync(db, b, n * es, cudaMemcpyHostToDevice, h->st));
    }
  }
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, h->st);
  AsmTimes tm;
  long long l0 = g_launches;
  if (CPLX) rc = launch_assembly(h, *(const PolHarmonic*)polp, (const double*)h->nu.p, 1, dA, dlda, 0, db, 0, &tm);
  else rc = launch_assembly(h, *(const PolStatic*)polp, (const double*)h->nu.p, 1, dA, dlda, 0, db, 0, &tm);
  cudaEventRecord(e1, h->st);
  if (rc) return rc;
  if (!dev) {
    if ((rc = copy_mat(A, (size_t)lda * es, dA, n * es, n * es, n, cudaMemcpyDeviceToHost, h->st))) return rc;
    CK(cudaMemcpyAsync(b, db, n * es, cudaMemcpyDeviceToHost, h->st));
  }
  rc = check_err(h);
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  h->stats.ms_assemble = ms;
  tm.read(&h->stats);
  h->stats.kernel_launches = g_launches - l0;
  return rc;
}

extern "C" int mfbem_assemble_staela(mfbem_handle* h, double mu, double nu, double* A, int32_t lda, double* b,
                                     int32_t flags) {
  g_err.clear();
  if (!h || !A || !b) return fail(MFBEM_EARG, "null argument");
  if (int rd = check_dev(h)) return rd;
  if (int rc = hs_prepare_static(h)) return rc;
  if (int rc = bm_prepare(h, 0)) return rc;
  PolStatic pol;
  pol.k = staela_params(mu, nu);
  pol.nu = nu;
  pol.mu = mu;
  double nuv[2] = {nu, 0.0};
  return assemble_common<false>(h, &pol, nuv, A, lda, b, flags);
}

// d* / s* parameters per frequency (HarParH) from q [nf][6] (lambda, mu, rho,
// omega), for the HBIE points of a harmonic assembly
static int hbie_params(mfbem_handle* h, const double* dq, int nf, const HarParH** out) {
  *out = nullptr;
  if (!h->has_hbie) return 0;
  int rc;
  if ((rc = ensure(h->parh, sizeof(HarParH) * nf))) return rc;
  k_harparh<<<nblk(nf, 32), 32, 0, h->st>>>(dq, nf, (HarParH*)h->parh.p); ++g_launches;
  *out = (const HarParH*)h->parh.p;
  return 0;
}

extern "C" int mfbem_assemble_harela(mfbem_handle* h, const double lambda[2], const double mu[2], double rho,
                                     const double nu[2], double omega, double* A, int32_t lda, double* b,
                                     int32_t flags) {
  g_err.clear();
  if (!h || !A || !b || !lambda || !mu || !nu) return fail(MFBEM_EARG, "null argument");
  int rc;
  if ((rc = ensure(h->par, sizeof(HarParD) + 64))) return rc;
  double q[6] = {lambda[0], lambda[1], mu[0], mu[1], rho, omega};
  double* dq = (double*)((char*)h->par.p + sizeof(HarParD));
  CK(cudaMemcpyAsync(dq, q, sizeof(q), cudaMemcpyHostToDevice, h->st));
  k_harpar<<<1, 32, 0, h->st>>>(dq, 1, (HarParD*)h->par.p, zexp_thresholds()); ++g_launches;
  if ((rc = bm_prepare(h, 1))) return rc;
  PolHarmonic pol;
  pol.p = (const HarParD*)h->par.p;
  if ((rc = hbie_params(h, dq, 1, &pol.ph))) return rc;
  return assemble_common<true>(h, &pol, nu, A, lda, b, flags);
}

// ---------------------------------------------------------------------------
// Internal points (calculate_internal_points_mechanics_bem_{staela,harela})
// ---------------------------------------------------------------------------
struct TmpBufs {
  std::vector<void*> v;
  ~TmpBufs() {
    for (void* p : v) cudaFree(p);
  }
  int get(void** p, size_t bytes) {
    if (cudaMalloc(p, std::max<size_t>(bytes, 16)) != cudaSuccess) {
      cudaGetLastError();
      return fail(MFBEM_ENOMEM, "cudaMalloc (internal points)");
    }
    v.push_back(*p);
    return 0;
  }
};

// One pass of the internal points: classification, quasi-singular pair
// lists, adaptive and precalculated integration; out [nf][nip][12].
template <class POL>
static int ip_pass(mfbem_handle* h, IpArgs a, const POL& pol, TmpBufs& tb, std::vector<typename POL::T>& out) {
  typedef typename POL::T T;
  const DMesh& m = h->m;
  const int n_ip = a.nip, ne = h->ne, nf = a.nf;
  const size_t ob = sizeof(T) * 12 * (size_t)n_ip * nf;
  int rc;
  if ((rc = tb.get((void**)&a.cls_s, (size_t)n_ip * ne)) || (rc = tb.get((void**)&a.cls_h, (size_t)n_ip * ne)) ||
      (rc = tb.get((void**)&a.npair, sizeof(int) * n_ip)) || (rc = tb.get((void**)&a.poff, sizeof(int) * (n_ip + 1))) ||
      (rc = tb.get((void**)&a.err, sizeof(int))) || (rc = tb.get(&a.out, ob)))
    return rc;
  cudaStream_t st = h->st;
  const int big = INT_MAX;
  CK(cudaMemcpyAsync(a.err, &big, sizeof(int), cudaMemcpyHostToDevice, st));
  k_ip_classify<<<std::min(nblk((long long)n_ip * ne, 256), 152u * 16u), 256, 0, st>>>(m, a, h->d_qs); ++g_launches;
  k_ip_count<<<nblk(n_ip, 8), 256, 0, st>>>(m, a); ++g_launches;
  k_scan<int, int><<<1, 1024, 0, st>>>(a.npair, a.poff, n_ip); ++g_launches;
  int np = 0;
  CK(cudaMemcpyAsync(&np, a.poff + n_ip, sizeof(int), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  a.npairs = np;
  if ((rc = tb.get((void**)&a.pair_e, sizeof(int) * (size_t)np)) || (rc = tb.get((void**)&a.pair_ip, sizeof(int) * (size_t)np)) ||
      (rc = tb.get(&a.slot, sizeof(T) * 12 * (size_t)np * nf)))
    return rc;
  k_ip_fill<<<nblk(n_ip, 8), 256, 0, st>>>(m, a); ++g_launches;
  if (np > 0) {
    k_ip_adp<POL><<<nblk((long long)np * nf, 64), 64, 0, st>>>(m, a, pol, h->d_qs); ++g_launches;
  }
  constexpr int WPB = 4;
  k_ip_reg<POL, WPB><<<nblk((long long)n_ip * nf, WPB), WPB * 32, 0, st>>>(m, a, pol); ++g_launches;
  CK(cudaGetLastError());
  out.assign(12 * (size_t)n_ip * nf, T{});
  int err = 0;
  CK(cudaMemcpyAsync(out.data(), a.out, ob, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(&err, a.err, sizeof(int), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  if (err != INT_MAX)
    return fail(MFBEM_EUNSUPPORTED, "internal point " + std::to_string(err - 1) +
                                        (a.image ? " lies on the free surface of the half-space on an element"
                                                 : " lies on the boundary away from a node (needs the singular HBIE "
                                                   "integration)"));
  return 0;
}

template <class POL>
static int internal_points_run(mfbem_handle* h, const POL& pol, int nf, int32_t n_ip, const double* x_ip,
                               const double* u_nodes, const double* t_nodes, const double* u2_nodes,
                               const double* t2_nodes, double* u_ip, double* sigma_ip) {
  typedef typename POL::T T;
  const int nn = h->nn;
  // crack-like boundaries: face 2 sees -h and g of the element, so
  // g t1 - h u1 + g t2 + h u2 = g (t1 + t2) - h (u1 - u2) per node
  // (calculate_internal_points_mechanics_static.f90:320-354, 431-465)
  std::vector<T> ueff, teff;
  if (h->has_crack) {
    if (!u2_nodes || !t2_nodes)
      return fail(MFBEM_EUNSUPPORTED, "a region with crack-like boundaries needs both faces' solution "
                                      "(mfbem_internal_points_faces_staela / _harela)");
    const T* u1 = (const T*)u_nodes;
    const T* t1 = (const T*)t_nodes;
    const T* u2 = (const T*)u2_nodes;
    const T* t2 = (const T*)t2_nodes;
    ueff.assign(u1, u1 + 3 * (size_t)nn);
    teff.assign(t1, t1 + 3 * (size_t)nn);
    for (int s = 0; s < nn; ++s)
      if (h->crack_node[s])
        for (int c = 0; c < 3; ++c) {
          ueff[3 * s + c] = u1[3 * s + c] - u2[3 * s + c];
          teff[3 * s + c] = t1[3 * s + c] + t2[3 * s + c];
        }
    u_nodes = (const double*)ueff.data();
    t_nodes = (const double*)teff.data();
  }
  TmpBufs tb;
  IpArgs a{};
  a.nip = n_ip;
  a.nf = nf;
  a.nn = nn;
  a.enode = h->enode;
  a.nodex = h->nodex;
  a.nodecl = h->nodecl;
  const size_t vb = sizeof(T) * 3 * (size_t)nn * nf;
  int rc;
  if ((rc = tb.get((void**)&a.xip, sizeof(double) * 3 * (size_t)n_ip)) || (rc = tb.get((void**)&a.uval, vb)) ||
      (rc = tb.get((void**)&a.tval, vb)) || (rc = tb.get((void**)&a.onnode, sizeof(int) * n_ip)))
    return rc;
  cudaStream_t st = h->st;
  CK(cudaMemcpyAsync((void*)a.xip, x_ip, sizeof(double) * 3 * (size_t)n_ip, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync((void*)a.uval, u_nodes, vb, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync((void*)a.tval, t_nodes, vb, cudaMemcpyHostToDevice, st));
  k_ip_onnode<<<nblk(n_ip, 128), 128, 0, st>>>(a); ++g_launches;
  std::vector<T> out;
  if ((rc = ip_pass(h, a, pol, tb, out))) return rc;
  // static half-space: the complementary kernels from the points' images
  if constexpr (std::is_same<POL, IpStatic>::value) {
    if (h->hs_n == -3) {
      IpArgs ai = a;
      ai.image = 1;
      ai.hs_xp = h->hs_x;
      IpHsc ph;
      ph.mu = pol.mu;
      ph.nu = pol.nu;
      ph.xp = h->hs_x;
      std::vector<T> out2;
      if ((rc = ip_pass(h, ai, ph, tb, out2))) return rc;
      for (size_t i = 0; i < out.size(); ++i) out[i] = out[i] + out2[i];
    }
  }
  if (h->has_crack) {
    std::vector<int> onn(n_ip);
    CK(cudaMemcpyAsync(onn.data(), a.onnode, sizeof(int) * (size_t)n_ip, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    for (int ip = 0; ip < n_ip; ++ip)
      if (onn[ip] >= 0 && h->crack_node[onn[ip]])
        return fail(MFBEM_EUNSUPPORTED, "internal point " + std::to_string(ip) +
                                            " lies at a node of a crack-like boundary (two faces)");
  }
  T* uo = (T*)u_ip;
  T* so = (T*)sigma_ip;
  for (size_t i = 0; i < (size_t)n_ip * nf; ++i) {
    for (int c = 0; c < 3; ++c) uo[3 * i + c] = out[12 * i + c];
    for (int c = 0; c < 9; ++c) so[9 * i + c] = out[12 * i + 3 + c];
  }
  return 0;
}

static int internal_points_staela(mfbem_handle* h, double mu, double nu, int32_t n_ip, const double* x_ip,
                                  const double* u_nodes, const double* t_nodes, const double* u2_nodes,
                                  const double* t2_nodes, double* u_ip, double* sigma_ip) {
  g_err.clear();
  if (!h || n_ip < 0 || (n_ip > 0 && (!x_ip || !u_nodes || !t_nodes || !u_ip || !sigma_ip)))
    return fail(MFBEM_EARG, "invalid argument");
  if (int rd = check_dev(h)) return rd;
  if (h->hs_n != 0) {
    // the complementary kernels exist for the half-space x3 >= xp only
    // (fbem_bem_staela3d_hsc_sbie / _hsc_hbie: np = -3)
    if (h->hs_n != -3)
      return fail(MFBEM_EUNSUPPORTED, "static half-space internal points need the normal n = -3");
    for (int ip = 0; ip < n_ip; ++ip)
      if (x_ip[3 * (size_t)ip + 2] < h->hs_x)
        return fail(MFBEM_EGEOMETRY, "internal point " + std::to_string(ip) + " lies outside the half-space");
  }
  if (n_ip == 0) return 0;
  IpStatic pol;
  pol.k = staela_params(mu, nu);
  pol.nu = nu;
  pol.mu = mu;
  pol.cted1 = -1.0 / (8.0 * kPi * (1.0 - nu));
  pol.cted2 = 1.0 - 2.0 * nu;
  pol.ctes1 = mu / (4.0 * kPi * (1.0 - nu));
  pol.ctes2 = 1.0 - 2.0 * nu;
  pol.ctes3 = 1.0 - 4.0 * nu;
  return internal_points_run(h, pol, 1, n_ip, x_ip, u_nodes, t_nodes, u2_nodes, t2_nodes, u_ip, sigma_ip);
}
extern "C" int mfbem_internal_points_staela(mfbem_handle* h, double mu, double nu, int32_t n_ip, const double* x_ip,
                                            const double* u_nodes, const double* t_nodes, double* u_ip,
                                            double* sigma_ip) {
  return internal_points_staela(h, mu, nu, n_ip, x_ip, u_nodes, t_nodes, nullptr, nullptr, u_ip, sigma_ip);
}
extern "C" int mfbem_internal_points_faces_staela(mfbem_handle* h, double mu, double nu, int32_t n_ip,
                                                  const double* x_ip, const double* u_nodes, const double* t_nodes,
                                                  const double* u2_nodes, const double* t2_nodes, double* u_ip,
                                                  double* sigma_ip) {
  if (n_ip > 0 && (!u2_nodes || !t2_nodes)) return fail(MFBEM_EARG, "invalid argument");
  return internal_points_staela(h, mu, nu, n_ip, x_ip, u_nodes, t_nodes, u2_nodes, t2_nodes, u_ip, sigma_ip);
}

static int internal_points_harela(mfbem_handle* h, const double lambda[2], const double mu[2], double rho,
                                  double omega, int32_t n_ip, const double* x_ip, const double* u_nodes,
                                  const double* t_nodes, const double* u2_nodes, const double* t2_nodes, double* u_ip,
                                  double* sigma_ip) {
  g_err.clear();
  if (!h || !lambda || !mu || n_ip < 0 || (n_ip > 0 && (!x_ip || !u_nodes || !t_nodes || !u_ip || !sigma_ip)))
    return fail(MFBEM_EARG, "invalid argument");
  if (int rd = check_dev(h)) return rd;
  if (n_ip == 0) return 0;
  TmpBufs tb;
  HarParD* pd;
  HarParH* ph;
  double* dq;
  int rc;
  if ((rc = tb.get((void**)&pd, sizeof(HarParD))) || (rc = tb.get((void**)&ph, sizeof(HarParH))) ||
      (rc = tb.get((void**)&dq, 6 * sizeof(double))))
    return rc;
  const double q[6] = {lambda[0], lambda[1], mu[0], mu[1], rho, omega};
  CK(cudaMemcpyAsync(dq, q, sizeof(q), cudaMemcpyHostToDevice, h->st));
  k_harpar<<<1, 32, 0, h->st>>>(dq, 1, pd, zexp_thresholds()); ++g_launches;
  k_harparh<<<1, 32, 0, h->st>>>(dq, 1, ph); ++g_launches;
  IpHarmonic pol;
  pol.p = pd;
  pol.ph = ph;
  return internal_points_run(h, pol, 1, n_ip, x_ip, u_nodes, t_nodes, u2_nodes, t2_nodes, u_ip, sigma_ip);
}
extern "C" int mfbem_internal_points_harela(mfbem_handle* h, const double lambda[2], const double mu[2], double rho,
                                            double omega, int32_t n_ip, const double* x_ip, const double* u_nodes,
                                            const double* t_nodes, double* u_ip, double* sigma_ip) {
  return internal_points_harela(h, lambda, mu, rho, omega, n_ip, x_ip, u_nodes, t_nodes, nullptr, nullptr, u_ip,
                                sigma_ip);
}
extern "C" int mfbem_internal_points_faces_harela(mfbem_handle* h, const double lambda[2], const double mu[2],
                                                  double rho, double omega, int32_t n_ip, const double* x_ip,
                                                  const double* u_nodes, const double* t_nodes,
                                                  const double* u2_nodes, const double* t2_nodes, double* u_ip,
                                                  double* sigma_ip) {
  if (n_ip > 0 && (!u2_nodes || !t2_nodes)) return fail(MFBEM_EARG, "invalid argument");
  return internal_points_harela(h, lambda, mu, rho, omega, n_ip, x_ip, u_nodes, t_nodes, u2_nodes, t2_nodes, u_ip,
                                sigma_ip);
}

// ---------------------------------------------------------------------------
// Test hook (not part of the reference interface): E_2..E_5 of n values z by
// the binary64 path (zexp_2to5) and the double-float path (zexp_2to5_ff).
// z: [n][2]; e64, e32: [n][4][2] (E2..E5, re/im).
// ---------------------------------------------------------------------------
__global__ void k_zexp_check(const double* z, int n, ZexpSteps steps, double* e64, double* eff) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  cd zz = mk(z[2 * i], z[2 * i + 1]);
  cd E[4];
  zexp_2to5(steps, zz, E[0], E[1], E[2], E[3]);
  float t2[16];
  for (int k = 0; k < 16; ++k) t2[k] = (float)steps.t2[k];
  cf F[4];
  zexp_2to5_ff(t2, cf_from(zz.re, zz.im), F[0], F[1], F[2], F[3]);
  for (int k = 0; k < 4; ++k) {
    e64[8 * i + 2 * k] = E[k].re;
    e64[8 * i + 2 * k + 1] = E[k].im;
    eff[8 * i + 2 * k] = ff_to(F[k].re);
    eff[8 * i + 2 * k + 1] = ff_to(F[k].im);
  }
}
extern "C" int mfbem_internal_zexp(int32_t n, const double* z, double* e64, double* eff) {
  g_err.clear();
  if (n <= 0 || !z || !e64 || !eff) return fail(MFBEM_EARG, "invalid argument");
  int rc = init_tables();
  if (rc) return rc;
  DevBuf dz, d1, d2;
  if ((rc = ensure(dz, 16 * (size_t)n)) || (rc = ensure(d1, 64 * (size_t)n)) || (rc = ensure(d2, 64 * (size_t)n)))
    return rc;
  cudaError_t e = cudaMemcpy(dz.p, z, 16 * (size_t)n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    k_zexp_check<<<nblk(n, 128), 128>>>((const double*)dz.p, n, zexp_thresholds(), (double*)d1.p, (double*)d2.p); ++g_launches;
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(e64, d1.p, 64 * (size_t)n, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(eff, d2.p, 64 * (size_t)n, cudaMemcpyDeviceToHost);
  cudaFree(dz.p);
  cudaFree(d1.p);
  cudaFree(d2.p);
  if (e != cudaSuccess) return fail(MFBEM_ECUDA, std::string("zexp check: ") + cudaGetErrorString(e));
  return 0;
}

#include "mfbem_solve.cuh"
#include "mfbem_learned.cuh"

// Test hook (not part of the reference interface): C -= A B for complex64
// column-major A (m x k), B (k x n), C (m x n) with the tcgen05 3xTF32
// kernels: pre-split tiles + bulk-copy pipeline (staged = 0) or the
// self-staging kernel (staged = 1).
extern "C" int mfbem_internal_tc_cgemm(int32_t m, int32_t n, int32_t k, const float* A, const float* B, float* C,
                                       int32_t staged) {
  g_err.clear();
  if (m <= 0 || n <= 0 || k < 0 || !A || !B || !C) return fail(MFBEM_EARG, "invalid argument");
  int rc;
  DevBuf dA, dB, dC, dE, ws;
  auto cleanup = [&]() {
    for (DevBuf* b : {&dA, &dB, &dC, &dE, &ws})
      if (b->p) cudaFree(b->p);
  };
  const size_t sa = 8 * (size_t)m * std::max(k, 1), sb = 8 * (size_t)std::max(k, 1) * n, sc = 8 * (size_t)m * n;
  if ((rc = ensure(dA, sa)) || (rc = ensure(dB, sb)) || (rc = ensure(dC, sc)) || (rc = ensure(dE, sizeof(int)))) {
    cleanup();
    return rc;
  }
  cudaError_t e = raise_smem_limit((const void*)k_tc_cgemm) ? cudaErrorInvalidValue : cudaSuccess;
  if (e == cudaSuccess && k > 0) e = cudaMemcpy(dA.p, A, 8 * (size_t)m * k, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && k > 0) e = cudaMemcpy(dB.p, B, 8 * (size_t)k * n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dC.p, C, sc, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(dE.p, 0, sizeof(int));
  if (e == cudaSuccess) {
    if (staged) {
      dim3 g(nblk(m, TC_BM / 2), nblk(n, TC_BN), 1);
      k_tc_cgemm<<<g, 128, TC_SMEM>>>((const float2*)dA.p, m, 0, (const float2*)dB.p, std::max(k, 1), 0,
                                      (float2*)dC.p, m, 0, m, n, k, (int*)dE.p, g_spin_limit.load());
      ++g_launches;
    } else if ((rc = tc_cgemm_run(0, (const float2*)dA.p, m, 0, (const float2*)dB.p, std::max(k, 1), 0,
                                  (float2*)dC.p, m, 0, m, n, k, 1, ws, (int*)dE.p))) {
      cleanup();
      return rc;
    }
    e = cudaGetLastError();
  }
  int herr = 0;
  if (e == cudaSuccess) e = cudaMemcpy(C, dC.p, sc, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(&herr, dE.p, sizeof(int), cudaMemcpyDeviceToHost);
  cleanup();
  if (e != cudaSuccess) return fail(MFBEM_ECUDA, std::string("tc cgemm: ") + cudaGetErrorString(e));
  if (herr) return fail(MFBEM_ETIMEOUT, "tc cgemm: an MMA completion wait timed out");
  return 0;
}

// Test hook (not part of the reference interface): C -= A B in FP64 for
// column-major A (m x k), B (k x n), C (m x n), complex (cplx = 1) or real,
// with the plain LU's trailing-update kernels: mode 0 the Ozaki-scheme
// tensor-core kernels, 1 the binary64 SIMT kernel.
extern "C" int mfbem_internal_f64_gemm(int32_t cplx, int32_t m, int32_t n, int32_t k, const double* A,
                                       const double* B, double* C, int32_t mode) {
  g_err.clear();
  if (m <= 0 || n <= 0 || k <= 0 || !A || !B || !C || mode < 0 || mode > 1) return fail(MFBEM_EARG, "invalid argument");
  const size_t es = cplx ? 16 : 8;
  DevBuf dA, dB, dC;
  auto cleanup = [&]() {
    for (DevBuf* b : {&dA, &dB, &dC})
      if (b->p) cudaFree(b->p);
  };
  int rc;
  if ((rc = ensure(dA, es * m * k)) || (rc = ensure(dB, es * k * n)) || (rc = ensure(dC, es * m * n))) {
    cleanup();
    return rc;
  }
  cudaError_t e = cudaMemcpy(dA.p, A, es * m * k, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dB.p, B, es * k * n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dC.p, C, es * m * n, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cleanup();
    return fail(MFBEM_ECUDA, std::string("f64 gemm: ") + cudaGetErrorString(e));
  }
  if (mode == 0) {
    if ((rc = oz_err_reset(0)) == 0)
      rc = cplx ? oz_gemm_run<true>(0, (const double2*)dA.p, m, 0, (const double2*)dB.p, k, 0, (double2*)dC.p, m, 0, m,
                                    n, k, 1)
                : oz_gemm_run<false>(0, (const double*)dA.p, m, 0, (const double*)dB.p, k, 0, (double*)dC.p, m, 0, m,
                                     n, k, 1);
    if (!rc) rc = oz_err_check(0);
  } else {
    if (cplx)
      k_gemm_simt<double2><<<dim3(nblk(m, 64), nblk(n, 64), 1), 256>>>((const double2*)dA.p, m, 0,
                                                                        (const double2*)dB.p, k, 0, (double2*)dC.p, m,
                                                                        0, m, n, k);
    else
      k_gemm_simt<double><<<dim3(nblk(m, 64), nblk(n, 64), 1), 256>>>((const double*)dA.p, m, 0, (const double*)dB.p,
                                                                       k, 0, (double*)dC.p, m, 0, m, n, k);
    ++g_launches;
    rc = cudaGetLastError() == cudaSuccess ? 0 : fail(MFBEM_ECUDA, "f64 gemm launch");
  }
  if (!rc) {
    e = cudaMemcpy(C, dC.p, es * m * n, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) rc = fail(MFBEM_ECUDA, std::string("f64 gemm: ") + cudaGetErrorString(e));
  }
  cleanup();
  return rc;
}

// Test hook (not part of the reference interface): the quasi-singular
// (adaptive) pairs of the mesh's classification. *n_pairs receives their
// number; with xcp and elem given (room for *n_pairs on entry), each pair's
// collocation point (3 doubles) and 0-based element.
extern "C" int mfbem_internal_adaptive_pairs(mfbem_handle* h, int32_t* n_pairs, double* xcp, int32_t* elem) {
  g_err.clear();
  if (!h || !n_pairs) return fail(MFBEM_EARG, "invalid argument");
  if (int rd = check_dev(h)) return rd;
  const int ncp = h->m.ncp, ne = h->m.ne;
  std::vector<uint8_t> cls((size_t)ncp * ne);
  std::vector<double> cpx(3 * (size_t)ncp);
  CK(cudaMemcpy(cls.data(), h->m.cls, cls.size(), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(cpx.data(), h->m.cpx, sizeof(double) * cpx.size(), cudaMemcpyDeviceToHost));
  const int cap = *n_pairs;
  int k = 0;
  for (int c = 0; c < ncp; ++c)
    for (int e = 0; e < ne; ++e)
      if (cls[(size_t)c * ne + e] == CLS_ADP) {
        if (xcp && elem && k < cap) {
          for (int q = 0; q < 3; ++q) xcp[3 * (size_t)k + q] = cpx[3 * (size_t)c + q];
          elem[k] = e;
        }
        ++k;
      }
  *n_pairs = k;
  return 0;
}

// Test hook (not part of the reference interface): sets the iteration limit
// of the bounded device waits (0 restores each kernel's own), so that a test
// can make a wait give up and check the error status, the freed resources
// and the next call. Nothing of the kernels' work is skipped.
extern "C" int mfbem_internal_set_spin_limit(int64_t iterations) {
  if (iterations < 0) return fail(MFBEM_EARG, "negative limit");
  g_spin_limit.store(iterations);
  return 0;
}

// Test hook (not part of the reference interface): system f of the handle's
// last mfbem_sweep_harela call, A (n x n column-major complex128) and b.
// After a mixed-precision sweep A is the assembled binary64 system (its
// factors live in the complex64 copy); after a plain sweep A holds the FP64
// LU factors.
extern "C" int mfbem_internal_sweep_system(mfbem_handle* h, int32_t f, double* A_out, double* b_out) {
  g_err.clear();
  if (!h || !A_out || !b_out || f < 0 || f >= h->last_nf) return fail(MFBEM_EARG, "no such system in the last sweep");
  if (int rd = check_dev(h)) return rd;
  const size_t n = (size_t)h->ndof, nn = n * n;
  CK(cudaMemcpyAsync(A_out, (const double2*)h->A.p + nn * f, sizeof(double2) * nn, cudaMemcpyDeviceToHost, h->st));
  CK(cudaMemcpyAsync(b_out, (const double2*)h->b.p + n * f, sizeof(double2) * n, cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  return 0;
}

// ---------------------------------------------------------------------------
// Batch of harmonic sweeps over meshes of uneven size (no counterpart in the
// reference): every mesh's sweep runs on its own host thread, stream and
// work buffers, so small problems share the GPU instead of running one
// after another. Per mesh i: material lambda[2i..], mu[2i..], rho[i],
// nu[2i..], n_freq[i] frequencies omega[i][...], solutions x_out[i].
// ---------------------------------------------------------------------------
extern "C" int mfbem_sweep_harela_batch(int32_t n_mesh, mfbem_handle* const* hs, const double* lambda,
                                        const double* mu, const double* rho, const double* nu, const int32_t* n_freq,
                                        const double* const* omega, int32_t precision, double rel_tol,
                                        double* const* x_out, int32_t flags, mfbem_stats* stats) {
  g_err.clear();
  if (n_mesh <= 0 || !hs || !lambda || !mu || !rho || !nu || !n_freq || !omega || !x_out)
    return fail(MFBEM_EARG, "invalid argument");
  std::vector<int> rc(n_mesh, 0);
  std::vector<std::string> msg(n_mesh);
  std::vector<mfbem_stats> st(n_mesh);
  int dev = 0;
  cudaGetDevice(&dev);
  std::vector<std::thread> th;
  th.reserve(n_mesh);
  for (int i = 0; i < n_mesh; ++i)
    th.emplace_back([&, i]() {
      cudaSetDevice(dev);
      g_concurrent = n_mesh > 1;
      rc[i] = mfbem_sweep_harela(hs[i], lambda + 2 * i, mu + 2 * i, rho[i], nu + 2 * i, n_freq[i], omega[i], precision,
                                 rel_tol, x_out[i], flags, &st[i]);
      if (rc[i]) msg[i] = g_err;
    });
  for (auto& t : th) t.join();
  if (stats)
    for (int i = 0; i < n_mesh; ++i) stats[i] = st[i];
  for (int i = 0; i < n_mesh; ++i)
    if (rc[i]) return fail(rc[i], "mesh " + std::to_string(i) + ": " + msg[i]);
  return 0;
}

// ---------------------------------------------------------------------------
// Learned quadrature of near-singular pairs (no counterpart in the reference)
// ---------------------------------------------------------------------------
// tolerance curves of the reference-rule candidates (1e-3 .. 1e-9)
static std::vector<QsCurves> ql_tol_curves() {
  std::vector<QsCurves> q(QL_NT);
  for (int r = 0; r < QL_NT; ++r) q[r] = qs_curves(std::pow(10.0, -3.0 - r));
  return q;
}

extern "C" int mfbem_qlearn_label(int32_t n, const double* elem, const double* pts, int32_t kernel, const double* kcl,
                                  float* feat, float* logerr, int32_t* cost, int32_t* valid) {
  g_err.clear();
  if (n <= 0 || !elem || !pts || !feat || !logerr || !cost || !valid || (kernel && !kcl) || kernel < 0 || kernel > 1)
    return fail(MFBEM_EARG, "invalid argument");
  int rc = init_tables();
  if (rc) return rc;
  std::vector<double> cl(n);
  std::vector<int> gf(n);
  for (int s = 0; s < n; ++s) {
    const double* x = elem + 24 * (size_t)s;
    cl[s] = clen_q8(x, 1e-9);
    gf[s] = host_phijac_ngp_q8(x, 1e-6);
  }
  std::vector<HarParD> par;
  if (kernel) {
    // viscoelastic material E = 1, nu = 0.3, rho = 1, xi = 0.02; omega from |k2| cl
    const double E = 1.0, nu = 0.3, rho = 1.0, xi = 0.02;
    const cd mu = mk(E / (2.0 * (1.0 + nu)), 2.0 * xi * E / (2.0 * (1.0 + nu)));
    const cd lam = mu * (2.0 * nu / (1.0 - 2.0 * nu));
    const cd c2 = csqrt_(mu / rho);
    const double ac2 = sqrt(c2.re * c2.re + c2.im * c2.im);
    par.resize(n);
    for (int s = 0; s < n; ++s) {
      par[s] = harela_params(lam, mu, rho, kcl[s] * ac2 / cl[s]);
      par[s].steps = zexp_thresholds();
    }
  }
  const std::vector<QsCurves> q = ql_tol_curves();
  DevBuf b_ex, b_pt, b_cl, b_gf, b_k, b_par, b_q, b_scr, b_f, b_le, b_c, b_v;
  auto cleanup = [&]() {
    for (DevBuf* b : {&b_ex, &b_pt, &b_cl, &b_gf, &b_k, &b_par, &b_q, &b_scr, &b_f, &b_le, &b_c, &b_v})
      if (b->p) cudaFree(b->p);
  };
  if ((rc = ensure(b_ex, 24 * sizeof(double) * n)) || (rc = ensure(b_pt, 3 * sizeof(double) * n)) ||
      (rc = ensure(b_cl, sizeof(double) * n)) || (rc = ensure(b_gf, sizeof(int) * n)) ||
      (rc = ensure(b_k, sizeof(double) * n)) || (rc = ensure(b_par, sizeof(HarParD) * (kernel ? n : 1))) ||
      (rc = ensure(b_q, sizeof(QsCurves) * QL_NT)) || (rc = ensure(b_scr, sizeof(double) * LEAF_D * QL_MAXREF * (size_t)n)) ||
      (rc = ensure(b_f, sizeof(float) * QL_NF * n)) || (rc = ensure(b_le, sizeof(float) * QL_NC * n)) ||
      (rc = ensure(b_c, sizeof(int) * QL_NC * n)) || (rc = ensure(b_v, sizeof(int) * n))) {
    cleanup();
    return rc;
  }
  cudaError_t e = cudaMemcpy(b_ex.p, elem, 24 * sizeof(double) * n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(b_pt.p, pts, 3 * sizeof(double) * n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(b_cl.p, cl.data(), sizeof(double) * n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(b_gf.p, gf.data(), sizeof(int) * n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && kernel) e = cudaMemcpy(b_k.p, kcl, sizeof(double) * n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && kernel) e = cudaMemcpy(b_par.p, par.data(), sizeof(HarParD) * n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(b_q.p, q.data(), sizeof(QsCurves) * QL_NT, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    constexpr int WPB = 2;
    if (kernel)
      k_ql_label<WPB, true><<<nblk(n, WPB), WPB * 32>>>(n, (double*)b_ex.p, (double*)b_pt.p, (double*)b_cl.p,
                                                        (int*)b_gf.p, (double*)b_k.p, (HarParD*)b_par.p,
                                                        (QsCurves*)b_q.p, 16, (double*)b_scr.p, (float*)b_f.p,
                                                        (float*)b_le.p, (int*)b_c.p, (int*)b_v.p);
    else
      k_ql_label<WPB, false><<<nblk(n, WPB), WPB * 32>>>(n, (double*)b_ex.p, (double*)b_pt.p, (double*)b_cl.p,
                                                         (int*)b_gf.p, (double*)b_k.p, (HarParD*)b_par.p,
                                                         (QsCurves*)b_q.p, 16, (double*)b_scr.p, (float*)b_f.p,
                                                         (float*)b_le.p, (int*)b_c.p, (int*)b_v.p);
    ++g_launches;
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(feat, b_f.p, sizeof(float) * QL_NF * n, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(logerr, b_le.p, sizeof(float) * QL_NC * n, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(cost, b_c.p, sizeof(int) * QL_NC * n, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(valid, b_v.p, sizeof(int) * n, cudaMemcpyDeviceToHost);
  cleanup();
  if (e != cudaSuccess) return fail(MFBEM_ECUDA, std::string("qlearn label: ") + cudaGetErrorString(e));
  return 0;
}

extern "C" int32_t mfbem_mlp_size(void) { return QL_NW; }
extern "C" const int32_t* mfbem_mlp_orders(void) { return h_ql_g; }

// MLP loss and gradient over the whole set (forward + backward kernels), or the
// forward outputs only (grad == NULL). y, valid may be NULL for forward only.
static int mlp_run(const float* w, int n, const float* feat, const float* y, const int* valid, float* loss,
                   float* grad, float* out) {
  int rc;
  const bool bwd = grad != nullptr;
  DevBuf bw, bf, by, bv, bg, bl, bo;
  auto cleanup = [&]() {
    for (DevBuf* b : {&bw, &bf, &by, &bv, &bg, &bl, &bo})
      if (b->p) cudaFree(b->p);
  };
  if ((rc = ensure(bw, sizeof(float) * QL_NW)) || (rc = ensure(bf, sizeof(float) * QL_NF * (size_t)n)) ||
      (rc = ensure(by, sizeof(float) * QL_NC * (size_t)n)) || (rc = ensure(bv, sizeof(int) * (size_t)n)) ||
      (rc = ensure(bg, sizeof(float) * QL_NW)) || (rc = ensure(bl, sizeof(float))) ||
      (rc = ensure(bo, sizeof(float) * QL_NC * (size_t)n))) {
    cleanup();
    return rc;
  }
  std::vector<int> ones;
  if (!valid) { ones.assign(n, 1); valid = ones.data(); }
  cudaError_t e = (raise_smem_limit((const void*)k_mlp<true>) || raise_smem_limit((const void*)k_mlp<false>))
                      ? cudaErrorInvalidValue : cudaSuccess;
  if (e == cudaSuccess) e = cudaMemcpy(bw.p, w, sizeof(float) * QL_NW, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(bf.p, feat, sizeof(float) * QL_NF * (size_t)n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && y) e = cudaMemcpy(by.p, y, sizeof(float) * QL_NC * (size_t)n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(bv.p, valid, sizeof(int) * (size_t)n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(bg.p, 0, sizeof(float) * QL_NW);
  if (e == cudaSuccess) e = cudaMemset(bl.p, 0, sizeof(float));
  if (e == cudaSuccess) {
    const float inv = 1.0f / ((float)n * QL_NC);
    if (bwd)
      k_mlp<true><<<nblk(n, QL_BT), QL_BT, ql_smem_bytes()>>>((float*)bw.p, (float*)bf.p, (float*)by.p, (int*)bv.p,
                                                             n, nullptr, n, inv, (float*)bo.p, (float*)bg.p, (float*)bl.p);
    else
      k_mlp<false><<<nblk(n, QL_BT), QL_BT, ql_smem_bytes()>>>((float*)bw.p, (float*)bf.p, nullptr, nullptr, n,
                                                              nullptr, n, inv, (float*)bo.p, nullptr, nullptr);
    ++g_launches;
    e = cudaGetLastError();
  }
  if (e == cudaSuccess && out) e = cudaMemcpy(out, bo.p, sizeof(float) * QL_NC * (size_t)n, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && bwd) e = cudaMemcpy(grad, bg.p, sizeof(float) * QL_NW, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && bwd && loss) e = cudaMemcpy(loss, bl.p, sizeof(float), cudaMemcpyDeviceToHost);
  cleanup();
  if (e != cudaSuccess) return fail(MFBEM_ECUDA, std::string("mlp: ") + cudaGetErrorString(e));
  return 0;
}
extern "C" int mfbem_mlp_forward(const float* w, int32_t n, const float* feat, float* out) {
  g_err.clear();
  if (!w || n <= 0 || !feat || !out) return fail(MFBEM_EARG, "invalid argument");
  return mlp_run(w, n, feat, nullptr, nullptr, nullptr, nullptr, out);
}
extern "C" int mfbem_mlp_loss_grad(const float* w, int32_t n, const float* feat, const float* y, const int32_t* valid,
                                   float* loss, float* grad) {
  g_err.clear();
  if (!w || n <= 0 || !feat || !y || !loss || !grad) return fail(MFBEM_EARG, "invalid argument");
  return mlp_run(w, n, feat, y, valid, loss, grad, nullptr);
}

// Train in place with Adam on mini-batches drawn on the device; loss_hist[s]
// receives the mini-batch loss of step s (may be NULL).
extern "C" int mfbem_mlp_train(float* w, int32_t n, const float* feat, const float* y, const int32_t* valid,
                               int32_t steps, int32_t batch, float lr, uint64_t seed, float* loss_hist) {
  g_err.clear();
  if (!w || n <= 0 || !feat || !y || steps <= 0 || batch <= 0) return fail(MFBEM_EARG, "invalid argument");
  int rc;
  DevBuf bw, bf, by, bv, bg, bm, bvv, bl, bi;
  auto cleanup = [&]() {
    for (DevBuf* b : {&bw, &bf, &by, &bv, &bg, &bm, &bvv, &bl, &bi})
      if (b->p) cudaFree(b->p);
  };
  if ((rc = ensure(bw, sizeof(float) * QL_NW)) || (rc = ensure(bf, sizeof(float) * QL_NF * (size_t)n)) ||
      (rc = ensure(by, sizeof(float) * QL_NC * (size_t)n)) || (rc = ensure(bv, sizeof(int) * (size_t)n)) ||
      (rc = ensure(bg, sizeof(float) * QL_NW)) || (rc = ensure(bm, sizeof(float) * QL_NW)) ||
      (rc = ensure(bvv, sizeof(float) * QL_NW)) || (rc = ensure(bl, sizeof(float) * steps)) ||
      (rc = ensure(bi, sizeof(int) * (size_t)batch))) {
    cleanup();
    return rc;
  }
  std::vector<int> ones;
  if (!valid) { ones.assign(n, 1); valid = ones.data(); }
  cudaError_t e = raise_smem_limit((const void*)k_mlp<true>) ? cudaErrorInvalidValue : cudaSuccess;
  if (e == cudaSuccess) e = cudaMemcpy(bw.p, w, sizeof(float) * QL_NW, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(bf.p, feat, sizeof(float) * QL_NF * (size_t)n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(by.p, y, sizeof(float) * QL_NC * (size_t)n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(bv.p, valid, sizeof(int) * (size_t)n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(bm.p, 0, sizeof(float) * QL_NW);
  if (e == cudaSuccess) e = cudaMemset(bvv.p, 0, sizeof(float) * QL_NW);
  if (e == cudaSuccess) e = cudaMemset(bl.p, 0, sizeof(float) * steps);
  const float inv = 1.0f / ((float)batch * QL_NC);
  for (int t = 0; t < steps && e == cudaSuccess; ++t) {
    k_ql_batch<<<nblk(batch, 256), 256>>>((int*)bi.p, batch, n, (unsigned long long)seed, t); ++g_launches;
    cudaMemsetAsync(bg.p, 0, sizeof(float) * QL_NW);
    k_mlp<true><<<nblk(batch, QL_BT), QL_BT, ql_smem_bytes()>>>((float*)bw.p, (float*)bf.p, (float*)by.p, (int*)bv.p,
                                                               n, (int*)bi.p, batch, inv, nullptr, (float*)bg.p,
                                                               (float*)bl.p + t);
    ++g_launches;
    k_adam<<<nblk(QL_NW, 256), 256>>>((float*)bw.p, (float*)bg.p, (float*)bm.p, (float*)bvv.p, QL_NW, lr, 0.9f, 0.999f,
                                      1e-8f, t + 1);
    ++g_launches;
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(w, bw.p, sizeof(float) * QL_NW, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && loss_hist) e = cudaMemcpy(loss_hist, bl.p, sizeof(float) * steps, cudaMemcpyDeviceToHost);
  cleanup();
  if (e != cudaSuccess) return fail(MFBEM_ECUDA, std::string("mlp train: ") + cudaGetErrorString(e));
  return 0;
}

// Rebuild the adaptive leaves of a mesh with the learned rule choice (w) or
// the reference rule (w == NULL). log10_tol: the largest admissible predicted
// log10 relative error; kernel / kcl: kernel type and wavenumber x element
// size fed to the network. n_learned (optional): pairs that took a learned rule.
extern "C" int mfbem_set_learned_quadrature(mfbem_handle* h, const float* w, double log10_tol, int32_t kernel,
                                            double kcl, int32_t* n_learned) {
  g_err.clear();
  if (!h || kernel < 0 || kernel > 1) return fail(MFBEM_EARG, "invalid argument");
  if (int rd = check_dev(h)) return rd;
  DMesh& m = h->m;
  if (n_learned) *n_learned = 0;
  if (m.nadp == 0) return 0;
  int rc;
  float* dw = nullptr;
  int *choice, *nl;
  if ((rc = dalloc(h, (void**)&choice, sizeof(int) * (m.nadp + 1))) || (rc = dalloc(h, (void**)&nl, sizeof(int) * (m.nadp + 1))))
    return rc;
  QsCurves* qt;
  {
    const std::vector<QsCurves> q = ql_tol_curves();
    if ((rc = dalloc(h, (void**)&qt, sizeof(QsCurves) * QL_NT))) return rc;
    CK(cudaMemcpy(qt, q.data(), sizeof(QsCurves) * QL_NT, cudaMemcpyHostToDevice));
  }
  if (w) {
    if ((rc = dalloc(h, (void**)&dw, sizeof(float) * QL_NW))) return rc;
    CK(cudaMemcpy(dw, w, sizeof(float) * QL_NW, cudaMemcpyHostToDevice));
    k_ql_choose<<<nblk(m.nadp, 64), 64>>>(m, h->d_qs, qt, dw, (float)log10_tol, kernel, kcl, choice, nl); ++g_launches;
  } else {
    // reference rule for every pair
    CK(cudaMemset(choice, 0xff, sizeof(int) * (m.nadp + 1)));
    k_adp_count<<<nblk(m.nadp, 64), 64>>>(m, h->d_qs, m.adp_cp, nl); ++g_launches;
  }
  k_scan<int, int><<<1, 1024>>>(nl, m.adp_leaf, (int)m.nadp); ++g_launches;
  int nleaf = 0;
  CK(cudaMemcpy(&nleaf, m.adp_leaf + m.nadp, sizeof(int), cudaMemcpyDeviceToHost));
  long long* lpts;
  if ((rc = dalloc(h, (void**)&m.leaf, sizeof(double) * LEAF_D * (nleaf + 1))) ||
      (rc = dalloc(h, (void**)&m.leaf_gln, sizeof(int) * (nleaf + 1))) ||
      (rc = dalloc(h, (void**)&m.leaf_pair, sizeof(int) * (nleaf + 1))) ||
      (rc = dalloc(h, (void**)&m.leaf_pt, sizeof(long long) * (nleaf + 1))) ||
      (rc = dalloc(h, (void**)&lpts, sizeof(long long) * (nleaf + 1))))
    return rc;
  m.nleaf = nleaf;
  k_ql_fill<<<nblk(m.nadp, 64), 64>>>(m, h->d_qs, qt, choice); ++g_launches;
  if (m.nleaf > 0) { k_leaf_points<<<nblk(m.nleaf, 256), 256>>>(m, lpts); ++g_launches; }
  k_scan<long long, long long><<<1, 1024>>>(lpts, m.leaf_pt, (int)m.nleaf); ++g_launches;
  CK(cudaMemcpy(&h->pts_adp, m.leaf_pt + m.nleaf, sizeof(long long), cudaMemcpyDeviceToHost));
  m.nleaf_pts = h->pts_adp;
  m.leaf_geo = nullptr;
  const size_t geo_budget = (size_t)8 << 30;
  if (m.nleaf_pts > 0 && (size_t)m.nleaf_pts * 14 * sizeof(double) <= geo_budget) {
    if ((rc = dalloc(h, (void**)&m.leaf_geo, (size_t)m.nleaf_pts * 14 * sizeof(double)))) return rc;
    k_leaf_geo<<<nblk(m.nleaf_pts, 128), 128>>>(m); ++g_launches;
  }
  // the df64 copy of the hoisted geometry is rebuilt by the next mixed sweep
  if (h->geo_f.p) cudaFree(h->geo_f.p);
  h->geo_f.p = nullptr;
  h->geo_f.bytes = 0;
  h->geo_f.dev = -1;
  CK(cudaGetLastError());
  CK(cudaDeviceSynchronize());
  if (n_learned && w) {
    std::vector<int> c(m.nadp);
    CK(cudaMemcpy(c.data(), choice, sizeof(int) * m.nadp, cudaMemcpyDeviceToHost));
    int k = 0;
    for (int v : c) k += v >= 0;
    *n_learned = k;
  }
  h->stats.adaptive_leaves = (int)m.nleaf;
  h->stats.points_adaptive = h->pts_adp;
  return 0;
}
