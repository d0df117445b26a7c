// noalloc.cu -- jmm_plain_full_energy_noalloc: the plain form's full FP64
// pair sum (the nine totals that fad and ECheck form, src/jmmMCState.cpp:
// 853-1003 and :1965-2095) for caller-owned positions, without allocating.
//
// Who needs it: code that may not call cudaMalloc/cudaFree or any allocating
// library routine -- a caller capturing a stream into a CUDA graph (an
// allocation is not a capturable stream operation), a real-time or embedded
// host that pre-reserves all device memory at start-up and treats a later
// allocation as a failure, or a tight per-step loop (the reference's driver
// calls ECheck inside its step loop) that cannot afford allocation latency.
//
// The pair terms of one sum are staged in one file-scope device array of
// fixed size, g_pair_terms below: 9 doubles per pair for at most
// kNoallocMaxN = 256 particles (32,640 pairs, 2.35 MB).  Every GPU that loads
// libjmmgpu.so holds that array until the process exits.  Host code cannot
// use the array's name as a device address (in host code it names a
// host-side stand-in): the address is obtained once per device with
// cudaGetSymbolAddress, with that device current, on the entry point's first
// call on the device; make that first call before any stream capture.
// All calls share the one array and it keeps the last call's contents:
// every term a call reads is written by the same call first, and two calls
// whose kernels overlap on the GPU race on the array.
#include <math.h>
#include <string.h>

#include <mutex>

#include "common.cuh"

namespace {

constexpr uint64_t kNoallocMaxN = 256;
constexpr uint64_t kNoallocMaxPairs = kNoallocMaxN * (kNoallocMaxN - 1) / 2;
constexpr int kThreads = 1024;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_pair_terms[9 * kNoallocMaxPairs];

std::mutex g_setup_mu;
double *g_terms_addr[kMaxDevices] = {};

// phiLJcut / phiLJinfcutoff / phiHarmoniccut (src/pot.cpp:19-141) with the
// virial terms on, the reference's operand order, no fused multiply-add.
__device__ void phi(int potential, double cutoff, double d, double l, double *out) {
#pragma unroll
  for (int k = 0; k < 9; ++k) out[k] = 0.0;
  if (potential == JMM_POT_HARMONIC) {
    if (d <= 0) {
      out[0] = 10E10;
      out[1] = 10E10;
    } else if (d < cutoff) {
      const double rijm = __dsub_rn(d, 1.0);
      out[0] = __dmul_rn(rijm, rijm);
      out[1] = __dmul_rn(__dmul_rn(__ddiv_rn(2.0, l), d), rijm);
    }
    return;
  }
  const double cut = potential == JMM_POT_LJ ? (double)INFINITY : cutoff;
  const double d3 = __dmul_rn(__dmul_rn(d, d), d);
  const double r6 = __ddiv_rn(1.0, __dmul_rn(d3, d3));
  const double r12 = __dmul_rn(r6, r6);
  if (d <= cut) {
    const double phi6 = __dmul_rn(4.0, r6), phi12 = __dmul_rn(4.0, r12);
    const double vir6 = __dmul_rn(24.0, r6), vir12 = __dmul_rn(48.0, r12);
    const double hv6 = __dmul_rn(144.0, r6), hv12 = __dmul_rn(576.0, r12);
    out[0] = __dsub_rn(phi12, phi6);
    out[1] = __dsub_rn(vir12, vir6);
    out[2] = phi12;
    out[3] = vir12;
    out[4] = phi6;
    out[5] = vir6;
    out[6] = __dsub_rn(hv12, hv6);
    out[7] = hv12;
    out[8] = hv6;
  }
}

// One block: the pair terms into the staging array in parallel, then nine
// lanes form the nine sums in the reference's pair order.
__global__ void __launch_bounds__(kThreads, 1)
    full_energy_noalloc_kernel(int potential, double cutoff, int nbn, const double *r, uint64_t n,
                               double l, double *terms, double *out) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
  for (uint64_t i = warp; i < n; i += nwarps) {
    // pair (i, j), i < j, is number i(N-1) - i(i+1)/2 + j - 1 in row-major order
    const uint64_t row = i * (n - 1) - (i * (i + 1)) / 2 + i;
    for (uint64_t j = i + 1 + lane; j < n; j += 32) {
      double t[9];
      if (nbn >= 0 && (j - i) > (uint64_t)nbn) {
#pragma unroll
        for (int k = 0; k < 9; ++k) t[k] = 0.0;
      } else {
        phi(potential, cutoff, __dsub_rn(r[j], r[i]), l, t);
      }
      double *dst = terms + (row + (j - i - 1)) * 9;
#pragma unroll
      for (int k = 0; k < 9; ++k) dst[k] = t[k];
    }
  }
  __syncthreads();
  if (threadIdx.x < 9) {
    const uint64_t npairs = n * (n - 1) / 2;
    double s = 0.0;
    for (uint64_t p = 0; p < npairs; ++p) s = __dadd_rn(s, terms[p * 9 + threadIdx.x]);
    out[threadIdx.x] = s;
  }
}

// The staging array's device address on the current device (looked up once).
int terms_address(double **addr) {
  int dev = 0;
  JMM_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices)
    return jmm::fail(JMM_ERR_INVALID, "jmm_plain_full_energy_noalloc: device %d beyond %d", dev,
                     kMaxDevices);
  std::lock_guard<std::mutex> lock(g_setup_mu);
  if (!g_terms_addr[dev]) {
    void *p = nullptr;
    JMM_CUDA(cudaGetSymbolAddress(&p, g_pair_terms));
    g_terms_addr[dev] = static_cast<double *>(p);
  }
  *addr = g_terms_addr[dev];
  return JMM_OK;
}

}  // namespace

extern "C" int jmm_plain_full_energy_noalloc(const jmm_params *params, const double *r,
                                             uint64_t n, double l, double *out, void *stream) {
  jmm::clear_error();
  JMM_CHECK_ARG(params && r && out, "null argument");
  JMM_CHECK_ARG(n >= 2, "N must be at least 2");
  if (n > kNoallocMaxN)
    return jmm::fail(JMM_ERR_INVALID,
                     "jmm_plain_full_energy_noalloc: N = %llu exceeds the fixed staging size "
                     "(N <= %llu); use the plain chain's energy check instead",
                     (unsigned long long)n, (unsigned long long)kNoallocMaxN);
  JMM_CHECK_ARG(params->potential == JMM_POT_LJCUT || params->potential == JMM_POT_LJ ||
                    params->potential == JMM_POT_HARMONIC,
                "potential must be LJcut, LJ or HARMONIC");
  JMM_CHECK_ARG(isfinite(l) && l > 0.0, "the box length must be finite and positive");
  // r and out must be device (or managed) memory of the current device: a
  // host or another device's pointer is refused here rather than faulting in
  // the kernel (querying attributes allocates nothing)
  int dev = 0;
  JMM_CUDA(cudaGetDevice(&dev));
  for (const void *ptr : {(const void *)r, (const void *)out}) {
    cudaPointerAttributes at;
    const cudaError_t e = cudaPointerGetAttributes(&at, ptr);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return jmm::fail(JMM_ERR_INVALID, "jmm_plain_full_energy_noalloc: %p is not device memory",
                       ptr);
    }
    const bool ok = (at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged) &&
                    at.device == dev;
    if (!ok)
      return jmm::fail(JMM_ERR_INVALID,
                       "jmm_plain_full_energy_noalloc: %p is not device memory of device %d", ptr,
                       dev);
  }
  double *terms = nullptr;
  int rc = terms_address(&terms);
  if (rc) return rc;
  const double cutoff = params->potential == JMM_POT_LJ ? INFINITY : params->cutoff;
  full_energy_noalloc_kernel<<<1, kThreads, 0, (cudaStream_t)stream>>>(
      params->potential, cutoff, params->nbn, r, n, l, terms, out);
  JMM_CUDA(cudaGetLastError());
  return JMM_OK;
}
