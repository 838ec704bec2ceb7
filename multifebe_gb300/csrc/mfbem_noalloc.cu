// mfbem_solve_c_static: the complex FP64 dense solve of mfbem_solve_c (LU with
// partial pivoting + triangular solves) for callers that cannot allocate device
// memory. Its whole device working set lives in one file-scope __device__
// array; the call performs no cudaMalloc / cudaFree and uses no allocating
// library (the trailing update is a kernel of this file).
//
// Limits: n <= MFBEM_STATIC_MAX_N, n_rhs <= MFBEM_STATIC_MAX_RHS. The array
// (about 16 MiB) is held by every GPU that loads the library until the process
// exits. All calls share it and it keeps the previous call's contents; calls
// that overlap on the GPU (several host threads at once) race on it.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "../../include/mfbem.h"
#include "mfbem_host.h"
#include "mfbem_lu.cuh"

namespace {

constexpr size_t kMaxN = MFBEM_STATIC_MAX_N;
constexpr size_t kMaxRhs = MFBEM_STATIC_MAX_RHS;
constexpr size_t kOffA = 0;
constexpr size_t kOffB = kOffA + kMaxN * kMaxN * sizeof(double2);
constexpr size_t kOffPiv = kOffB + kMaxN * kMaxRhs * sizeof(double2);
constexpr size_t kOffInfo = kOffPiv + kMaxN * sizeof(int);
constexpr size_t kBytes = kOffInfo + 256;

// the working set: factors, right-hand sides, pivots, info
static __device__ __align__(256) unsigned char g_static_scratch[kBytes];

// device address of g_static_scratch per device ordinal, resolved once per
// device with that device current (the array's host-side name is only a
// stand-in, not a device address)
constexpr int kMaxDevices = 64;
static void* g_scratch_ptr[kMaxDevices] = {nullptr};
static std::mutex g_setup_mutex;

int scratch_for_current_device(unsigned char** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return mfb::fail(MFBEM_ECUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return mfb::fail(MFBEM_ECUDA, "device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_static_scratch);
    if (e != cudaSuccess || !p)
      return mfb::fail(MFBEM_ECUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    g_scratch_ptr[dev] = p;
  }
  *out = static_cast<unsigned char*>(g_scratch_ptr[dev]);
  return 0;
}

// C(m x n) -= A(m x k) B(k x n), complex, column-major, k <= 32
__global__ void k_update_c(double2* C, const double2* A, const double2* B, int lda, int m, int n, int k) {
  __shared__ double2 As[16][33];
  __shared__ double2 Bs[32][17];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int i = blockIdx.x * 16 + tx, j = blockIdx.y * 16 + ty;
  for (int t = ty; t < k; t += 16)
    As[tx][t] = (i < m) ? A[(size_t)t * lda + i] : make_double2(0.0, 0.0);
  for (int t = tx; t < k; t += 16)
    Bs[t][ty] = (j < n) ? B[(size_t)j * lda + t] : make_double2(0.0, 0.0);
  __syncthreads();
  if (i >= m || j >= n) return;
  double2 acc = make_double2(0.0, 0.0);
  for (int t = 0; t < k; ++t) {
    double2 a = As[tx][t], b = Bs[t][ty];
    acc.x += a.x * b.x - a.y * b.y;
    acc.y += a.x * b.y + a.y * b.x;
  }
  double2 c = C[(size_t)j * lda + i];
  C[(size_t)j * lda + i] = make_double2(c.x - acc.x, c.y - acc.y);
}

inline unsigned nb_(long long n, int t) { return (unsigned)((n + t - 1) / t); }

#define CKS(call)                                                                                            \
  do {                                                                                                       \
    cudaError_t e_ = (call);                                                                                 \
    if (e_ != cudaSuccess) return mfb::fail(MFBEM_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

}  // namespace

using namespace mfb;

extern "C" int mfbem_solve_c_static(int32_t n, double* A, int32_t* ipiv, int32_t n_rhs, double* b,
                                    int32_t factorize) {
  mfb::set_error("");
  if (n <= 0 || !A || !ipiv || (n_rhs > 0 && !b) || n_rhs < 0)
    return mfb::fail(MFBEM_EARG, "invalid argument");
  if ((size_t)n > kMaxN || (size_t)n_rhs > kMaxRhs)
    return mfb::fail(MFBEM_EARG, "mfbem_solve_c_static: n must be <= " + std::to_string(kMaxN) + " and n_rhs <= " +
                                     std::to_string(kMaxRhs) + " (fixed no-allocation working set)");
  if (!factorize) {
    // pivots handed back must be getrf's (1-based, ipiv(j) in [j, n]): the
    // row interchanges of the solve index the vectors with them
    for (int32_t j = 0; j < n; ++j)
      if (ipiv[j] < j + 1 || ipiv[j] > n)
        return mfb::fail(MFBEM_EARG, "ipiv(" + std::to_string(j + 1) + ") = " + std::to_string(ipiv[j]) +
                                         " is not a pivot of getrf (must lie in [" + std::to_string(j + 1) + ", n])");
  }
  unsigned char* base = nullptr;
  int rc = scratch_for_current_device(&base);
  if (rc) return rc;
  double2* dA = reinterpret_cast<double2*>(base + kOffA);
  double2* dB = reinterpret_cast<double2*>(base + kOffB);
  int* dP = reinterpret_cast<int*>(base + kOffPiv);
  int* dI = reinterpret_cast<int*>(base + kOffInfo);
  const cudaStream_t st = 0;
  const size_t bytesA = (size_t)n * n * sizeof(double2);
  CKS(cudaMemcpyAsync(dA, A, bytesA, cudaMemcpyHostToDevice, st));
  if (factorize) {
    CKS(cudaMemsetAsync(dI, 0, sizeof(int), st));  // the array keeps the previous call's info
    const int nbk = 32;
    for (int k = 0; k < n; k += nbk) {
      const int kb = (n - k < nbk) ? n - k : nbk;
      for (int j = k; j < k + kb; ++j) {
        k_pcol_pivot<double2, 256><<<1, 256, 0, st>>>(dA, 0, n, n, k, kb, j, dP, dI);
        int g = (n - j - 1 + 255) / 256;
        if (g < 1) g = 1;
        if (g > 64) g = 64;
        k_pcol_update<double2, 256><<<dim3(g, 1), 256, 0, st>>>(dA, 0, n, n, k, kb, j);
      }
      if (n - kb > 0) k_laswp<double2><<<dim3(nb_(n - kb, 128), 1), 128, 0, st>>>(dA, 0, n, n, k, kb, dP);
      if (k + kb < n) {
        const int nc = n - k - kb;
        k_trsm_llu<double2><<<dim3(nb_(nc, 64), 1), 64, kb * kb * sizeof(double2), st>>>(dA, 0, n, n, k, kb);
        k_update_c<<<dim3(nb_(nc, 16), nb_(nc, 16)), dim3(16, 16), 0, st>>>(
            dA + (k + kb) + (size_t)(k + kb) * n, dA + (k + kb) + (size_t)k * n, dA + k + (size_t)(k + kb) * n, n, nc,
            nc, kb);
      }
    }
    CKS(cudaGetLastError());
    int info = 0;
    CKS(cudaMemcpyAsync(A, dA, bytesA, cudaMemcpyDeviceToHost, st));
    CKS(cudaMemcpyAsync(ipiv, dP, sizeof(int) * n, cudaMemcpyDeviceToHost, st));
    CKS(cudaMemcpyAsync(&info, dI, sizeof(int), cudaMemcpyDeviceToHost, st));
    CKS(cudaStreamSynchronize(st));
    if (info > 0) return mfb::fail(info, "singular matrix: zero pivot U(info,info)");
  } else {
    CKS(cudaMemcpyAsync(dP, ipiv, sizeof(int) * n, cudaMemcpyHostToDevice, st));
  }
  if (n_rhs > 0) {
    CKS(cudaMemcpyAsync(dB, b, (size_t)n * n_rhs * sizeof(double2), cudaMemcpyHostToDevice, st));
    for (int r = 0; r < n_rhs; ++r) {
      double2* x = dB + (size_t)r * n;
      k_rhs_swap<double2><<<1, 1, 0, st>>>(x, 0, n, dP, 1);
      const int TB = 128;
      for (int r0 = 0; r0 < n; r0 += TB) {
        int w = (n - r0 < TB) ? n - r0 : TB;
        k_trsv_diag<double2, true><<<1, TB, 0, st>>>(dA, 0, n, x, 0, r0, w);
        if (r0 + w < n) k_trsv_update<double2><<<dim3(nb_(n - r0 - w, 256), 1), 256, 0, st>>>(dA, 0, n, x, 0, r0, w, r0 + w, n);
      }
      for (int r0 = ((n - 1) / TB) * TB; r0 >= 0; r0 -= TB) {
        int w = (n - r0 < TB) ? n - r0 : TB;
        k_trsv_diag<double2, false><<<1, TB, 0, st>>>(dA, 0, n, x, 0, r0, w);
        if (r0 > 0) k_trsv_update<double2><<<dim3(nb_(r0, 256), 1), 256, 0, st>>>(dA, 0, n, x, 0, r0, w, 0, r0);
      }
    }
    CKS(cudaGetLastError());
    CKS(cudaMemcpyAsync(b, dB, (size_t)n * n_rhs * sizeof(double2), cudaMemcpyDeviceToHost, st));
  }
  CKS(cudaStreamSynchronize(st));
  return 0;
}
