// sc_kmeans_step_noalloc: one Lloyd iteration of the FP64 form on
// caller-owned device memory that allocates nothing.
//
// The iteration is the body of the loop in KMeans::fit
// (src/cluster/kmeans.rs:294-310): assign every point to its nearest
// centroid (kmeans.rs:296 through BBDTree::clustering, whose labels equal the
// brute-force FP64 argmin), sum each cluster's points, divide by the sizes
// (kmeans.rs:297-303, an empty cluster keeps its centroid), and the
// distortion of the assignment.  It runs the same kernels as the handle API
// (exact.cu, update.cu); only the home of their scratch differs.
//
// Scratch: one file-scope __device__ byte array per device (static storage
// of this module, zero at module load), carved into
//   acc   k*d 128-bit fixed-point cluster sums   (<= kMaxKD entries)
//   cnt   k   point counts                       (<= kMaxK entries)
//   part  one distortion partial per 128 points  (<= kMaxParts entries)
//   st    the loop state and max |x|
// acc, cnt and st must be zero when a step starts.  Each call clears them
// itself (cudaMemsetAsync) before its first kernel; the finalize kernel also
// leaves acc and cnt at zero.  part is written in full before it is read.
#include <float.h>
#include <math.h>
#include <string.h>

#include <mutex>

#include <cuda.h>

#include "common.cuh"

namespace sc {
namespace {

constexpr int64_t kMaxKD = 65536;     // k * d
constexpr int64_t kMaxK = 4096;       // clusters
constexpr int64_t kMaxParts = 65536;  // assignment blocks of 128 points: n <= 8,388,608

constexpr size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }
constexpr size_t kOffAcc = 0;
constexpr size_t kOffCnt = align256(kOffAcc + kMaxKD * sizeof(Acc128));
constexpr size_t kOffPart = align256(kOffCnt + kMaxK * sizeof(unsigned long long));
constexpr size_t kOffSt = align256(kOffPart + kMaxParts * sizeof(double));
constexpr size_t kOffBits = align256(kOffSt + sizeof(LloydState));
constexpr size_t kScratchBytes = align256(kOffBits + sizeof(unsigned long long));  // 1,606,144 B

static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mutex;  // serialises calls: the scratch is shared
// Device address of g_scratch, looked up once per device and CUDA context: a
// __device__ symbol's address belongs to the context that loaded the module,
// so a new context on the same device (after cudaDeviceReset, or a caller's
// own driver-API context) gets its own lookup.
struct ScratchAddr {
  CUcontext ctx = nullptr;
  unsigned char *addr = nullptr;
};
ScratchAddr g_addr[kMaxDevices];

// cuCtxGetCurrent through the runtime's driver entry point (the library does
// not link the driver library itself).
CUresult current_context(CUcontext *ctx) {
  using Fn = CUresult (*)(CUcontext *);
  static Fn fn = nullptr;
  if (!fn) {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPoint("cuCtxGetCurrent", &p, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !p)
      return CUDA_ERROR_NOT_FOUND;
    fn = (Fn)p;
  }
  return fn(ctx);
}

// Waits for the call's work on the stream before the lock is released, on
// every return path: a call that fails after its first launch must not leave
// kernels writing the shared scratch while the next call clears it.
struct DrainOnExit {
  cudaStream_t s;
  bool armed = false;
  ~DrainOnExit() {
    if (armed) cudaStreamSynchronize(s);
  }
};

}  // namespace
}  // namespace sc

using namespace sc;

extern "C" sc_status sc_kmeans_step_noalloc(const void *x, int32_t dtype, int64_t n, int64_t d,
                                            double *centroids, int64_t k, int32_t *labels,
                                            int64_t *sizes, double *distortion, void *stream) {
  // Argument checks touch no GPU state.
  if (dtype != SC_F32 && dtype != SC_F64) { set_error("unsupported dtype %d", dtype); return SC_ERR_INVALID; }
  if (n < 1 || d < 1 || d > (1 << 16)) { set_error("invalid shape (%lld, %lld)", (long long)n, (long long)d); return SC_ERR_INVALID; }
  if (k < 1) { set_error("invalid number of clusters: %lld", (long long)k); return SC_ERR_INVALID; }
  if (k > kMaxK || k * d > kMaxKD) {
    set_error("k=%lld, d=%lld exceeds the no-allocation scratch (k <= %lld and k*d <= %lld)",
              (long long)k, (long long)d, (long long)kMaxK, (long long)kMaxKD);
    return SC_ERR_INVALID;
  }
  if ((n + 127) / 128 > kMaxParts) {
    set_error("n=%lld exceeds the no-allocation scratch (n <= %lld)", (long long)n, (long long)(kMaxParts * 128));
    return SC_ERR_INVALID;
  }
  if (!x || !centroids || !labels) { set_error("null device pointer"); return SC_ERR_INVALID; }
  const int nparts = assign_block_count(n);  // one partial per 128 points

  std::lock_guard<std::mutex> lock(g_mutex);
  int dev = 0, num_sms = 0;
  SC_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) { set_error("device ordinal %d is not supported", dev); return SC_ERR_INVALID; }
  SC_CUDA(cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, dev));
  CUcontext ctx = nullptr;
  if (current_context(&ctx) != CUDA_SUCCESS) ctx = nullptr;
  if (!ctx || g_addr[dev].ctx != ctx || !g_addr[dev].addr) {
    // Set-up for this device and context.  The lookup also makes the
    // device's primary context current when no context is.
    void *p = nullptr;
    SC_CUDA(cudaGetSymbolAddress(&p, g_scratch));
    if (current_context(&ctx) != CUDA_SUCCESS || !ctx) { set_error("no current CUDA context"); return SC_ERR_CUDA; }
    g_addr[dev].ctx = ctx;
    g_addr[dev].addr = (unsigned char *)p;
  }
  unsigned char *base = g_addr[dev].addr;
  Acc128 *acc = (Acc128 *)(base + kOffAcc);
  unsigned long long *cnt = (unsigned long long *)(base + kOffCnt);
  double *part = (double *)(base + kOffPart);
  LloydState *st = (LloydState *)(base + kOffSt);
  unsigned long long *bits = (unsigned long long *)(base + kOffBits);
  cudaStream_t s = (cudaStream_t)stream;
  DrainOnExit drain{s};
  drain.armed = true;

  SC_CUDA(cudaMemsetAsync(acc, 0, (size_t)(k * d) * sizeof(Acc128), s));
  SC_CUDA(cudaMemsetAsync(cnt, 0, (size_t)k * sizeof(unsigned long long), s));
  SC_CUDA(cudaMemsetAsync(st, 0, sizeof(LloydState), s));

  // Fixed-point scale of the 128-bit sums: the scale the handle API picks for
  // the same (n, d, k) and max |x|, so every value rounds to the same integer
  // and the centroids equal the handle's bit for bit.
  SC_TRY(launch_absmax(dtype, x, n * d, bits, s));
  unsigned long long hb = 0;
  SC_CUDA(cudaMemcpyAsync(&hb, bits, sizeof hb, cudaMemcpyDeviceToHost, s));
  SC_CUDA(cudaStreamSynchronize(s));
  double amax;
  memcpy(&amax, &hb, sizeof amax);
  if (!(amax <= DBL_MAX)) { set_error("x contains NaN or infinity; the GPU path requires finite input"); return SC_ERR_INVALID; }
  const int scale = update_plan(dtype, n, (int)d, (int)k, amax, num_sms).scale;

  SC_TRY(launch_assign_fp64(dtype, x, n, (int)d, centroids, (int)k, labels, part, st, s));
  SC_TRY(launch_update_fixed(dtype, x, n, (int)d, labels, acc, cnt, scale, st, s));
  SC_TRY(launch_finalize_centroids(acc, cnt, centroids, sizes, (int)k, (int)d, scale, nullptr, 0, st, s));
  SC_TRY(launch_finalize_scalar(part, nparts, nullptr, k, nullptr, st, s));
  if (distortion) SC_CUDA(cudaMemcpyAsync(distortion, &st->last_dist, sizeof(double), cudaMemcpyDeviceToHost, s));
  SC_CUDA(cudaStreamSynchronize(s));
  drain.armed = false;
  return SC_OK;
}
