// extern "C" entry points of libsmartcore_gb300 (declared in
// include/smartcore_gb300.h): argument checks with the reference's messages,
// device buffers owned by handles, and the launch sequences of the Lloyd
// loop, k-means++ and kNN.
#include <float.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <mutex>
#include <thread>
#include <vector>

#include "common.cuh"
#include "split.cuh"

namespace sc {

static thread_local char g_err[512];
static std::atomic<long long> g_launches{0};

void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

void set_error(const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof g_err, fmt, ap);
  va_end(ap);
}

sc_status cuda_fail(cudaError_t e, const char *what) {
  set_error("CUDA error %s (%s) in %s", cudaGetErrorName(e), cudaGetErrorString(e), what);
  if (e == cudaErrorMemoryAllocation) {
    cudaGetLastError();  // allocation failures are not sticky
    return SC_ERR_OOM;
  }
  return SC_ERR_CUDA;
}

std::mutex g_pool_mutex;
bool g_pool_ready[64] = {};
// Testing hooks: allocations left before injected failures (-1: none), and
// the number of live device allocations made through dev_alloc.
std::atomic<long long> g_fail_after{-1};
std::atomic<long long> g_live_allocs{0};

sc_status dev_alloc(void **p, size_t bytes, cudaStream_t s) {
  *p = nullptr;
  if (g_fail_after.load() >= 0 && g_fail_after.fetch_sub(1) <= 0) {
    g_fail_after.store(0);
    set_error("device allocation of %zu bytes failed (injected)", bytes);
    return SC_ERR_OOM;
  }
  int dev = 0;
  SC_CUDA(cudaGetDevice(&dev));
  if (dev >= 0 && dev < 64) {
    std::lock_guard<std::mutex> lock(g_pool_mutex);
    if (!g_pool_ready[dev]) {
      cudaMemPool_t pool;
      SC_CUDA(cudaDeviceGetDefaultMemPool(&pool, dev));
      uint64_t keep = UINT64_MAX;
      SC_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
      g_pool_ready[dev] = true;
    }
  }
  SC_CUDA(cudaMallocAsync(p, bytes ? bytes : 1, s));
  g_live_allocs.fetch_add(1);
  return SC_OK;
}

void dev_free(void *p, cudaStream_t s) {
  if (p) {
    cudaFreeAsync(p, s);
    g_live_allocs.fetch_sub(1);
  }
}

// Pinned host staging buffer for results copied into caller memory (grows,
// never shrinks; callers hold g_stage_mutex while they use it).  A device
// copy into pageable memory that the caller has just allocated pays for the
// first touch of every page inside the CUDA copy; a copy into pinned
// memory and a CPU memcpy do not.
std::mutex g_stage_mutex;
void *g_stage = nullptr;
size_t g_stage_bytes = 0;

sc_status host_stage(size_t bytes, void **out) {
  if (bytes > g_stage_bytes) {
    if (g_stage) cudaFreeHost(g_stage);
    g_stage = nullptr;
    g_stage_bytes = 0;
    SC_CUDA(cudaHostAlloc(&g_stage, bytes, cudaHostAllocDefault));
    g_stage_bytes = bytes;
  }
  *out = g_stage;
  return SC_OK;
}

// memcpy of a large result out of the staging buffer, split over host
// threads: the caller's freshly allocated pages are first touched (and
// faulted in) by several cores at once.
void stage_copy_out(void *dst, const void *src, size_t bytes) {
  constexpr size_t kPerThread = 2u << 20;
  const int nth = (int)std::min<size_t>({(size_t)std::max(1u, std::thread::hardware_concurrency()), 8,
                                         bytes / kPerThread + 1});
  if (nth <= 1) {
    memcpy(dst, src, bytes);
    return;
  }
  const size_t part = (bytes / nth + 63) & ~(size_t)63;
  auto piece = [&](int t) {
    const size_t a = std::min(bytes, (size_t)t * part), b = std::min(bytes, a + part);
    if (b > a) memcpy((char *)dst + a, (const char *)src + a, b - a);
  };
  std::vector<std::thread> pool;
  int started = 1;
  try {
    for (; started < nth; ++started) pool.emplace_back(piece, started);
  } catch (...) {  // no more threads: the rest on this one
    for (int t = started; t < nth; ++t) piece(t);
  }
  piece(0);
  for (auto &th : pool) th.join();
}

namespace {

size_t esize(int dtype) { return dtype == SC_F32 ? 4 : 8; }

sc_status check_matrix(const void *x, int32_t dtype, int32_t layout, int32_t mem,
                       int64_t n, int64_t d, int64_t ld) {
  if (dtype != SC_F32 && dtype != SC_F64) { set_error("unsupported dtype %d", dtype); return SC_ERR_INVALID; }
  if (layout != SC_ROW_MAJOR && layout != SC_COL_MAJOR) { set_error("unsupported layout %d", layout); return SC_ERR_INVALID; }
  if (mem != SC_MEM_HOST && mem != SC_MEM_DEVICE) { set_error("unsupported memory kind %d", mem); return SC_ERR_INVALID; }
  if (n < 0 || d < 1 || d > (1 << 16)) { set_error("invalid shape (%lld, %lld)", (long long)n, (long long)d); return SC_ERR_INVALID; }
  if (layout == SC_ROW_MAJOR && ld < d) { set_error("leading dimension %lld < number of columns %lld", (long long)ld, (long long)d); return SC_ERR_INVALID; }
  if (layout == SC_COL_MAJOR && ld < n) { set_error("leading dimension %lld < number of rows %lld", (long long)ld, (long long)n); return SC_ERR_INVALID; }
  if (n > 0 && !x) { set_error("null matrix pointer"); return SC_ERR_INVALID; }
  return SC_OK;
}

// Copies an n x d matrix (host or device, either layout) into a contiguous
// row-major device buffer dst.
sc_status upload_matrix(const void *x, int32_t dtype, int32_t layout, int32_t mem,
                        int64_t n, int64_t d, int64_t ld, void *dst, cudaStream_t s) {
  if (n == 0) return SC_OK;
  const size_t es = esize(dtype);
  const cudaMemcpyKind kind = mem == SC_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
  if (layout == SC_ROW_MAJOR) {
    if (ld == d) SC_CUDA(cudaMemcpyAsync(dst, x, (size_t)(n * d) * es, kind, s));
    else SC_CUDA(cudaMemcpy2DAsync(dst, (size_t)d * es, x, (size_t)ld * es, (size_t)d * es, (size_t)n, kind, s));
    return SC_OK;
  }
  void *tmp = nullptr;
  const size_t span = (size_t)((d - 1) * ld + n);
  const void *src = x;
  if (mem == SC_MEM_HOST) {
    SC_TRY(dev_alloc(&tmp, span * es, s));
    if (cudaMemcpyAsync(tmp, x, span * es, cudaMemcpyHostToDevice, s) != cudaSuccess) {
      dev_free(tmp, s);
      return cuda_fail(cudaGetLastError(), "upload");
    }
    src = tmp;
  }
  sc_status r = launch_to_row_major(dtype, src, n, d, ld, dst, s);
  dev_free(tmp, s);
  return r;
}


}  // namespace
}  // namespace sc

using namespace sc;

// ---------------------------------------------------------------------------
// KMeans handle
// ---------------------------------------------------------------------------
struct sc_kmeans {
  int dtype = SC_F32, form = SC_FORM_FP64;
  int64_t n = 0, d = 0, k = 0;
  cudaStream_t stream = nullptr;
  void *x = nullptr;  // row-major n x d
  double absmax = 0.0;          // max |x|, sets the fixed-point scales
  int num_sms = 0;
  UpdateBuf upd;                // centroid-sum buffers (per k)
  double *cent = nullptr;       // k x d
  int32_t *labels = nullptr;    // n
  double *dd = nullptr;         // n, k-means++ distances
  float *dd32 = nullptr;        // n, k-means++ distances rounded up to f32
  double *part = nullptr;       // block partials
  int64_t *sizes = nullptr;     // k
  double *cterms = nullptr;     // k
  double *uniforms = nullptr;   // k - 1
  void *seed_x = nullptr;       // k x d, k-means++ seed rows (element type)
  float *seed_cc = nullptr;     // k, k-means++ seed-to-seed distance bounds
  double *xnorm_total = nullptr;
  LloydState *st = nullptr;
  unsigned long long *bits = nullptr;
  SplitState split;             // split-BF16 form buffers
  int64_t k_alloc = 0;
  int profile = 0;                   // record events around each assignment kernel
  std::vector<cudaEvent_t> events;   // begin/end pairs
  size_t events_used = 0;
};

// Next begin/end event pair for timing one assignment kernel (nullptr when
// profiling is off).
static cudaEvent_t *next_timing(sc_kmeans *h) {
  if (!h->profile) return nullptr;
  if (h->events_used + 2 > h->events.size()) {
    for (int i = 0; i < 64; ++i) {
      cudaEvent_t e;
      if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
      h->events.push_back(e);
    }
  }
  cudaEvent_t *ev = &h->events[h->events_used];
  h->events_used += 2;
  return ev;
}

static sc_status kmeans_alloc_k(sc_kmeans *h, int64_t k) {
  if (k == h->k_alloc) { h->k = k; return SC_OK; }
  // until every buffer of the new k exists the handle has no centroids
  h->k_alloc = 0;
  h->k = 0;
  cudaStream_t hs = h->stream;
  dfree(h->cent, hs); dfree(h->sizes, hs); dfree(h->cterms, hs); dfree(h->uniforms, hs);
  dfree(h->seed_x, hs); dfree(h->seed_cc, hs);
  SC_TRY(dalloc(&h->cent, (size_t)(k * h->d), h->stream));
  SC_TRY(dalloc(&h->sizes, (size_t)k, h->stream));
  SC_TRY(dalloc(&h->cterms, (size_t)(k * h->d), h->stream));
  SC_TRY(dalloc(&h->uniforms, (size_t)k, h->stream));
  SC_TRY(dalloc((char **)&h->seed_x, (size_t)(k * h->d) * esize(h->dtype), h->stream));
  SC_TRY(dalloc(&h->seed_cc, (size_t)k, h->stream));
  SC_CUDA(cudaStreamSynchronize(h->stream));
  SC_TRY(update_alloc(&h->upd, h->dtype, h->n, (int)h->d, (int)k, h->absmax, h->num_sms, h->stream));
  if (h->dtype == SC_F32) SC_TRY(update_pack(&h->upd, (const float *)h->x, h->n, (int)h->d, h->stream));
  h->k_alloc = k;
  h->k = k;
  return SC_OK;
}

static sc_status reset_state(sc_kmeans *h) {
  LloydState s;
  memset(&s, 0, sizeof s);
  s.distortion = DBL_MAX;
  s.stop = 1;
  SC_CUDA(cudaMemcpyAsync(h->st, &s, sizeof s, cudaMemcpyHostToDevice, h->stream));
  return SC_OK;
}

extern "C" {

const char *sc_last_error(void) { return g_err; }
int32_t sc_abi_version(void) { return 100; }

int32_t sc_device_ok(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n < 1) { cudaGetLastError(); return 0; }
  int dev = 0, major = 0, minor = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
  cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
  return (major == 10 && minor == 3) ? 1 : 0;
}

void sc_kmeans_destroy(sc_kmeans *h) {
  if (!h) return;
  if (h->stream) cudaStreamSynchronize(h->stream);
  cudaStream_t hs = h->stream;  // frees in stream order: no device-wide synchronisation
  dfree(h->x, hs); dfree(h->cent, hs); dfree(h->labels, hs); dfree(h->dd, hs); dfree(h->dd32, hs);
  dfree(h->part, hs); dfree(h->sizes, hs); dfree(h->cterms, hs); dfree(h->uniforms, hs);
  dfree(h->seed_x, hs); dfree(h->seed_cc, hs);
  update_free(&h->upd, hs);
  dfree(h->xnorm_total, hs); dfree(h->st, hs); dfree(h->bits, hs);
  split_free(&h->split, hs);
  for (cudaEvent_t e : h->events) cudaEventDestroy(e);
  // the frees complete before the stream goes away, so the pool hands the
  // blocks to the next handle's stream without waiting on a dead one
  if (h->stream) {
    cudaStreamSynchronize(h->stream);
    cudaStreamDestroy(h->stream);
  }
  delete h;
}

sc_status sc_kmeans_create(const void *x, int32_t dtype, int32_t layout, int32_t mem,
                           int64_t n, int64_t d, int64_t ld, int32_t form,
                           sc_kmeans **out) {
  if (!out) { set_error("null output handle"); return SC_ERR_INVALID; }
  *out = nullptr;
  SC_TRY(check_matrix(x, dtype, layout, mem, n, d, ld));
  if (form != SC_FORM_FP64 && form != SC_FORM_SPLIT_BF16) { set_error("unknown form %d", form); return SC_ERR_INVALID; }
  if (n > ((int64_t)1 << 40)) { set_error("n=%lld is too large", (long long)n); return SC_ERR_INVALID; }
  // the split-BF16 k-means kernels serve rows of up to 128 features; wider
  // data runs the FP64 form, whose results are the same
  if (form == SC_FORM_SPLIT_BF16 && d > kSplitKMeansMaxD) form = SC_FORM_FP64;
  sc_kmeans *h = new sc_kmeans();
  h->dtype = dtype; h->form = form; h->n = n; h->d = d;
  sc_status r = SC_OK;
  do {
    if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) {
      r = cuda_fail(cudaGetLastError(), "cudaStreamCreate");
      h->stream = nullptr;
      break;
    }
    const int nparts = std::max(assign_block_count(n), pp_block_count(n));
    if ((r = dalloc((char **)&h->x, (size_t)(n * d) * esize(dtype), h->stream)) != SC_OK) break;
    if ((r = dalloc(&h->labels, (size_t)n, h->stream)) != SC_OK) break;
    if ((r = dalloc(&h->dd, (size_t)n, h->stream)) != SC_OK) break;
    if ((r = dalloc(&h->dd32, (size_t)n, h->stream)) != SC_OK) break;
    if ((r = dalloc(&h->part, (size_t)nparts, h->stream)) != SC_OK) break;
    if ((r = dalloc(&h->st, 1, h->stream)) != SC_OK) break;
    if ((r = dalloc(&h->bits, 1, h->stream)) != SC_OK) break;
    if ((r = dalloc(&h->xnorm_total, 1, h->stream)) != SC_OK) break;
    if ((r = upload_matrix(x, dtype, layout, mem, n, d, ld, h->x, h->stream)) != SC_OK) break;
    if ((r = launch_absmax(dtype, h->x, n * d, h->bits, h->stream)) != SC_OK) break;
    unsigned long long bits = 0;
    if (cudaMemcpyAsync(&bits, h->bits, sizeof bits, cudaMemcpyDeviceToHost, h->stream) != cudaSuccess ||
        cudaStreamSynchronize(h->stream) != cudaSuccess) {
      r = cuda_fail(cudaGetLastError(), "absmax");
      break;
    }
    double amax;
    memcpy(&amax, &bits, sizeof amax);
    if (!(amax <= DBL_MAX)) {
      set_error("x contains NaN or infinity; the GPU path requires finite input");
      r = SC_ERR_INVALID;
      break;
    }
    h->absmax = amax;
    {
      int dev = 0;
      if (cudaGetDevice(&dev) != cudaSuccess ||
          cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
        r = cuda_fail(cudaGetLastError(), "device attributes");
        break;
      }
    }
    if ((r = reset_state(h)) != SC_OK) break;
    if (form == SC_FORM_SPLIT_BF16 &&
        (r = split_prepare(&h->split, dtype, h->x, n, (int)d, h->xnorm_total, h->stream)) != SC_OK)
      break;
  } while (0);
  if (r != SC_OK) { sc_kmeans_destroy(h); return r; }
  *out = h;
  return SC_OK;
}

void *sc_kmeans_stream(sc_kmeans *h) { return h ? (void *)h->stream : nullptr; }

static sc_status seed_impl(sc_kmeans *h, int64_t k, int64_t first_index, const double *uniforms) {
  SC_TRY(kmeans_alloc_k(h, k));
  SC_TRY(reset_state(h));
  cudaStream_t s = h->stream;
  if (k > 1) SC_CUDA(cudaMemcpyAsync(h->uniforms, uniforms, (size_t)(k - 1) * sizeof(double), cudaMemcpyHostToDevice, s));
  SC_CUDA(cudaMemcpyAsync(&h->st->pp_chosen, &first_index, sizeof(int64_t), cudaMemcpyHostToDevice, s));
  const size_t row_bytes = (size_t)h->d * esize(h->dtype);
  SC_CUDA(cudaMemcpyAsync(h->seed_x, (const char *)h->x + (size_t)first_index * row_bytes, row_bytes,
                          cudaMemcpyDeviceToDevice, s));
  const int nb = pp_block_count(h->n);
  // the split form's BF16 rows serve the update's first bound
  const __nv_bfloat16 *xh = h->form == SC_FORM_SPLIT_BF16 && h->split.ready ? h->split.xh : nullptr;
  for (int64_t j = 1; j < k; ++j) {  // kmeans.rs:367-397
    SC_TRY(launch_pp_update(h->dtype, h->x, h->n, (int)h->d, h->st, (int32_t)(j - 1), h->dd, h->dd32, h->labels,
                            h->part, j == 1, h->seed_cc, xh, h->split.d_pad, h->split.xnrm, s));
    SC_TRY(launch_pp_select(h->dtype, h->x, (int)h->d, h->dd, h->part, h->n, nb, h->uniforms + (j - 1), h->st,
                            h->seed_x, h->seed_cc, (int)j, s));
  }
  SC_TRY(launch_pp_update(h->dtype, h->x, h->n, (int)h->d, h->st, (int32_t)(k - 1), h->dd, h->dd32, h->labels,
                          nullptr, k == 1, h->seed_cc, xh, h->split.d_pad, h->split.xnrm, s));  // :399-410
  // initial centroids: means of the seeding partition (kmeans.rs:275-292)
  SC_TRY(launch_update(&h->upd, h->dtype, h->x, h->n, (int)h->d, h->labels, (int)k, nullptr, s));
  SC_TRY(launch_finalize(&h->upd, h->cent, h->sizes, (int)k, (int)h->d, nullptr, 1, nullptr, s));
  SC_TRY(update_mark_sums(&h->upd, h->labels, h->n, h->st, s));  // the first step may move rows alone
  if (h->form == SC_FORM_SPLIT_BF16) SC_TRY(split_centroids_changed(&h->split, h->cent, (int)k, s));
  SC_CUDA(cudaStreamSynchronize(s));
  return SC_OK;
}

sc_status sc_kmeans_seed(sc_kmeans *h, int64_t k, int64_t first_index, const double *uniforms) {
  if (!h) { set_error("null handle"); return SC_ERR_INVALID; }
  if (k < 1) { set_error("invalid number of clusters: %lld", (long long)k); return SC_ERR_INVALID; }
  if (h->n < 1) { set_error("cannot seed an empty dataset"); return SC_ERR_INVALID; }
  if (first_index < 0 || first_index >= h->n) { set_error("first seed index %lld out of range", (long long)first_index); return SC_ERR_INVALID; }
  if (k > 1 && !uniforms) { set_error("null uniforms"); return SC_ERR_INVALID; }
  if (k > (1 << 20)) { set_error("k=%lld is too large", (long long)k); return SC_ERR_INVALID; }
  sc_status r = seed_impl(h, k, first_index, uniforms);
  if (r != SC_OK) h->k = 0;  // the handle has no usable centroids after a failed seeding
  return r;
}

static sc_status set_centroids_impl(sc_kmeans *h, int64_t k, const double *centroids) {
  SC_TRY(kmeans_alloc_k(h, k));
  SC_TRY(reset_state(h));
  SC_CUDA(cudaMemcpyAsync(h->cent, centroids, (size_t)(k * h->d) * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  if (h->form == SC_FORM_SPLIT_BF16) SC_TRY(split_centroids_changed(&h->split, h->cent, (int)k, h->stream));
  SC_CUDA(cudaStreamSynchronize(h->stream));
  return SC_OK;
}

sc_status sc_kmeans_set_centroids(sc_kmeans *h, int64_t k, const double *centroids) {
  if (!h) { set_error("null handle"); return SC_ERR_INVALID; }
  if (k < 1 || !centroids) { set_error("invalid number of clusters: %lld", (long long)k); return SC_ERR_INVALID; }
  sc_status r = set_centroids_impl(h, k, centroids);
  if (r != SC_OK) h->k = 0;  // no usable centroids after a failed update
  return r;
}

// One Lloyd iteration: assignment, sums, new centroids, distortion + break.
static sc_status lloyd_step(sc_kmeans *h) {
  cudaStream_t s = h->stream;
  const int k = (int)h->k, d = (int)h->d;
  if (h->form == SC_FORM_FP64) {
    cudaEvent_t *ev = next_timing(h);
    if (ev) SC_CUDA(cudaEventRecord(ev[0], s));
    SC_TRY(launch_assign_fp64(h->dtype, h->x, h->n, d, h->cent, k, h->labels, h->part, h->st, s));
    if (ev) SC_CUDA(cudaEventRecord(ev[1], s));
    SC_TRY(launch_update(&h->upd, h->dtype, h->x, h->n, d, h->labels, k, h->st, s));
    SC_TRY(launch_finalize(&h->upd, h->cent, h->sizes, k, d, h->cterms, 0, h->st, s));
    SC_TRY(launch_finalize_scalar(h->part, assign_block_count(h->n), nullptr, k, nullptr, h->st, s));
  } else {
    SC_TRY(split_assign(&h->split, h->dtype, h->x, h->n, d, h->cent, k, h->labels, h->st, s, next_timing(h)));
    SC_TRY(launch_update(&h->upd, h->dtype, h->x, h->n, d, h->labels, k, h->st, s));
    SC_TRY(launch_finalize(&h->upd, h->cent, h->sizes, k, d, h->cterms, 0, h->st, s));
    SC_TRY(launch_finalize_scalar(nullptr, 0, h->cterms, update_nterms(&h->upd, k, d), h->xnorm_total, h->st, s));
    SC_TRY(split_centroids_changed(&h->split, h->cent, k, s));
  }
  return SC_OK;
}

// One Lloyd step captured as a CUDA graph (its kernels recorded, not run):
// the later steps of an iterate call replay it, one launch instead of the
// step's nine.  Every buffer exists after the call's first step and the
// step's kernels take the same arguments each time (their state lives on the
// device), so the replay runs exactly what lloyd_step would launch.
// *kernels gets the step's kernel count; the capture itself launches nothing.
static sc_status capture_step(sc_kmeans *h, cudaGraphExec_t *exec, int64_t *kernels) {
  *exec = nullptr;
  cudaStream_t s = h->stream;
  const long long l0 = g_launches.load();
  if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
    cudaGetLastError();
    return SC_ERR_CUDA;
  }
  const sc_status r = lloyd_step(h);
  cudaGraph_t g = nullptr;
  const cudaError_t e = cudaStreamEndCapture(s, &g);
  *kernels = g_launches.load() - l0;
  g_launches.fetch_sub(*kernels);
  if (r != SC_OK || e != cudaSuccess || !g || cudaGraphInstantiate(exec, g, 0) != cudaSuccess) {
    *exec = nullptr;
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    return SC_ERR_CUDA;
  }
  cudaGraphDestroy(g);
  return SC_OK;
}

namespace {
struct GraphExecGuard {
  cudaGraphExec_t exec = nullptr;
  ~GraphExecGuard() {
    if (exec) cudaGraphExecDestroy(exec);
  }
};
}  // namespace

sc_status sc_kmeans_iterate(sc_kmeans *h, int64_t max_iter, int32_t stop_on_converge, int64_t *iters_done) {
  if (!h) { set_error("null handle"); return SC_ERR_INVALID; }
  if (h->k < 1) { set_error("centroids are not set"); return SC_ERR_INVALID; }
  if (max_iter < 0) { set_error("invalid maximum number of iterations: %lld", (long long)max_iter); return SC_ERR_INVALID; }
  cudaStream_t s = h->stream;
  const int32_t flags[2] = {0, stop_on_converge ? 1 : 0};  // done, stop
  SC_CUDA(cudaMemcpyAsync(&h->st->done, flags, sizeof flags, cudaMemcpyHostToDevice, s));
  const int64_t zero = 0;
  SC_CUDA(cudaMemcpyAsync(&h->st->iters, &zero, sizeof zero, cudaMemcpyHostToDevice, s));
  SC_CUDA(cudaMemcpyAsync(&h->st->rescored, &zero, sizeof zero, cudaMemcpyHostToDevice, s));
  SC_CUDA(cudaMemcpyAsync(&h->st->incremental_steps, &zero, sizeof zero, cudaMemcpyHostToDevice, s));
  GraphExecGuard graph;
  int64_t per_step = 0;
  for (int64_t t = 0; t < max_iter; ++t) {
    if (graph.exec) {
      SC_CUDA(cudaGraphLaunch(graph.exec, s));
      g_launches.fetch_add(per_step, std::memory_order_relaxed);
      continue;
    }
    SC_TRY(lloyd_step(h));
    // per-step timing events stay outside graphs, and a stream the caller is
    // capturing into its own graph keeps plain launches; a failed capture
    // leaves them too
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (t == 0 && max_iter > 2 && !h->profile && cudaStreamIsCapturing(s, &cs) == cudaSuccess &&
        cs == cudaStreamCaptureStatusNone && capture_step(h, &graph.exec, &per_step) != SC_OK)
      graph.exec = nullptr;
  }
  if (iters_done) {
    SC_CUDA(cudaMemcpyAsync(iters_done, &h->st->iters, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    SC_CUDA(cudaStreamSynchronize(s));
    int32_t err = 0;
    SC_CUDA(cudaMemcpyAsync(&err, &h->st->err, sizeof err, cudaMemcpyDeviceToHost, s));
    SC_CUDA(cudaStreamSynchronize(s));
    if (err) { set_error("device-side check failed (code %d)", err); return err == 4 ? SC_ERR_TIMEOUT : SC_ERR_INTERNAL; }
  }
  return SC_OK;
}

sc_status sc_kmeans_get(sc_kmeans *h, double *centroids, int64_t *sizes, int64_t *labels,
                        double *distortion, int64_t *iters) {
  if (!h) { set_error("null handle"); return SC_ERR_INVALID; }
  cudaStream_t s = h->stream;
  if (centroids)
    SC_CUDA(cudaMemcpyAsync(centroids, h->cent, (size_t)(h->k * h->d) * sizeof(double), cudaMemcpyDeviceToHost, s));
  if (sizes) SC_CUDA(cudaMemcpyAsync(sizes, h->sizes, (size_t)h->k * sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  int64_t *wide = nullptr;
  std::unique_lock<std::mutex> stage_lock(g_stage_mutex, std::defer_lock);
  void *stage = nullptr;
  const size_t label_bytes = (size_t)h->n * sizeof(int64_t);
  if (labels && h->n > 0) {  // widened on the device, copied through the pinned staging buffer
    SC_TRY(dalloc(&wide, (size_t)h->n, s));
    SC_TRY(launch_widen_labels(h->labels, wide, h->n, s));
    stage_lock.lock();
    SC_TRY(host_stage(label_bytes, &stage));
    SC_CUDA(cudaMemcpyAsync(stage, wide, label_bytes, cudaMemcpyDeviceToHost, s));
    dfree(wide, s);
  }
  LloydState st;
  SC_CUDA(cudaMemcpyAsync(&st, h->st, sizeof st, cudaMemcpyDeviceToHost, s));
  SC_CUDA(cudaStreamSynchronize(s));
  if (stage) stage_copy_out(labels, stage, label_bytes);
  if (distortion) *distortion = st.distortion;
  if (iters) *iters = st.iters;
  return SC_OK;
}

sc_status sc_kmeans_stats(sc_kmeans *h, int64_t *rescored, int64_t *pp_replays) {
  if (!h) { set_error("null handle"); return SC_ERR_INVALID; }
  LloydState st;
  SC_CUDA(cudaMemcpyAsync(&st, h->st, sizeof st, cudaMemcpyDeviceToHost, h->stream));
  SC_CUDA(cudaStreamSynchronize(h->stream));
  if (rescored) *rescored = st.rescored;
  if (pp_replays) *pp_replays = st.pp_replays;
  return SC_OK;
}

sc_status sc_kmeans_sum_stats(sc_kmeans *h, int64_t *incremental_steps) {
  if (!h) { set_error("null handle"); return SC_ERR_INVALID; }
  LloydState st;
  SC_CUDA(cudaMemcpyAsync(&st, h->st, sizeof st, cudaMemcpyDeviceToHost, h->stream));
  SC_CUDA(cudaStreamSynchronize(h->stream));
  if (incremental_steps) *incremental_steps = st.incremental_steps;
  return SC_OK;
}

sc_status sc_kmeans_profile(sc_kmeans *h, int32_t enable) {
  if (!h) { set_error("null handle"); return SC_ERR_INVALID; }
  h->profile = enable ? 1 : 0;
  h->events_used = 0;
  return SC_OK;
}

sc_status sc_kmeans_profile_read(sc_kmeans *h, double *total_ms, int64_t *launches) {
  if (!h) { set_error("null handle"); return SC_ERR_INVALID; }
  SC_CUDA(cudaStreamSynchronize(h->stream));
  double tot = 0.0;
  for (size_t i = 0; i + 1 < h->events_used; i += 2) {
    float ms = 0.f;
    SC_CUDA(cudaEventElapsedTime(&ms, h->events[i], h->events[i + 1]));
    tot += ms;
  }
  if (total_ms) *total_ms = tot;
  if (launches) *launches = (int64_t)(h->events_used / 2);
  h->events_used = 0;
  return SC_OK;
}

int64_t sc_kernel_launches(void) { return (int64_t)g_launches.load(); }

sc_status sc_kmeans_set_wait_limit(sc_kmeans *h, int64_t ns) {
  if (!h) { set_error("null handle"); return SC_ERR_INVALID; }
  if (ns < 0) { set_error("invalid wait limit %lld", (long long)ns); return SC_ERR_INVALID; }
  h->split.wait_ns = (uint64_t)ns;
  return SC_OK;
}

sc_status sc_debug_fail_alloc_after(int64_t after) {
  g_fail_after.store(after < 0 ? -1 : after);
  return SC_OK;
}

int64_t sc_debug_live_allocations(void) { return (int64_t)g_live_allocs.load(); }

sc_status sc_debug_knn_candidate_cap(int64_t cap) {
  split_knn_set_candidate_cap(cap);
  return SC_OK;
}

sc_status sc_debug_knn_chunk_queries(int64_t q) {
  split_knn_set_chunk_queries(q);
  return SC_OK;
}

sc_status sc_kmeans_sync(sc_kmeans *h) {
  if (!h) { set_error("null handle"); return SC_ERR_INVALID; }
  SC_CUDA(cudaStreamSynchronize(h->stream));
  return SC_OK;
}

sc_status sc_kmeans_fit(const void *x, int32_t dtype, int32_t layout, int64_t n, int64_t d,
                        int64_t ld, int64_t k, int64_t max_iter, int64_t first_index,
                        const double *uniforms, int32_t form, double *centroids_out,
                        int64_t *sizes_out, int64_t *labels_out, double *distortion_out,
                        int64_t *iters_out) {
  // validation order and messages of KMeans::fit (kmeans.rs:257-269)
  if (k < 2) { set_error("invalid number of clusters: %lld", (long long)k); return SC_ERR_INVALID; }
  if (max_iter == 0) { set_error("invalid maximum number of iterations: %lld", (long long)max_iter); return SC_ERR_INVALID; }
  sc_kmeans *h = nullptr;
  SC_TRY(sc_kmeans_create(x, dtype, layout, SC_MEM_HOST, n, d, ld, form, &h));
  sc_status r = sc_kmeans_seed(h, k, first_index, uniforms);
  if (r == SC_OK) r = sc_kmeans_iterate(h, max_iter, 1, nullptr);
  if (r == SC_OK) r = sc_kmeans_get(h, centroids_out, sizes_out, labels_out, distortion_out, iters_out);
  sc_kmeans_destroy(h);
  return r;
}

sc_status sc_kmeans_predict(const void *x, int32_t dtype, int32_t layout, int64_t n, int64_t d,
                            int64_t ld, const double *centroids, int64_t k, int32_t form,
                            int64_t *labels_out) {
  if (k < 1 || !centroids) { set_error("invalid number of clusters: %lld", (long long)k); return SC_ERR_INVALID; }
  sc_kmeans *h = nullptr;
  SC_TRY(sc_kmeans_create(x, dtype, layout, SC_MEM_HOST, n, d, ld, form, &h));
  sc_status r = sc_kmeans_set_centroids(h, k, centroids);
  if (r == SC_OK) {
    if (h->form == SC_FORM_FP64)
      r = launch_assign_fp64(h->dtype, h->x, h->n, (int)h->d, h->cent, (int)k, h->labels, nullptr, nullptr, h->stream);
    else
      r = split_assign(&h->split, h->dtype, h->x, h->n, (int)h->d, h->cent, (int)k, h->labels, h->st, h->stream);
  }
  if (r == SC_OK) r = sc_kmeans_get(h, nullptr, nullptr, labels_out, nullptr, nullptr);
  sc_kmeans_destroy(h);
  return r;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// kNN handle
// ---------------------------------------------------------------------------
struct sc_knn {
  int dtype = SC_F32;
  int64_t n = 0, d = 0;
  cudaStream_t stream = nullptr;
  void *train = nullptr;  // row-major n x d
  void *q = nullptr;      // queries, row-major
  int64_t q_cap = 0;
  int64_t *idx = nullptr;
  double *dist = nullptr;
  int64_t res_cap = 0;
  int64_t *aux_i = nullptr;  // class indices / outputs
  double *aux_d = nullptr;
  int64_t aux_cap = 0;
  int64_t rescored = 0;
  SplitKnnState split;
  int64_t *lists = nullptr;  // pinned host: the last radius lists' row indices
  size_t lists_cap = 0;
};

static sc_status knn_reserve(sc_knn *h, int64_t m, int64_t k) {
  if (m > h->q_cap) {
    h->q_cap = 0;  // a failed allocation leaves no stale capacity
    dfree(h->q, h->stream);
    SC_TRY(dalloc((char **)&h->q, (size_t)(m * h->d) * esize(h->dtype), h->stream));
    h->q_cap = m;
  }
  if (m * k > h->res_cap) {
    h->res_cap = 0;
    dfree(h->idx, h->stream); dfree(h->dist, h->stream);
    SC_TRY(dalloc(&h->idx, (size_t)(m * k), h->stream));
    SC_TRY(dalloc(&h->dist, (size_t)(m * k), h->stream));
    h->res_cap = m * k;
  }
  return SC_OK;
}

static sc_status knn_run(sc_knn *h, const void *queries, int32_t layout, int32_t mem, int64_t m,
                         int64_t ld, int64_t k, int32_t form) {
  SC_TRY(check_matrix(queries, h->dtype, layout, mem, m, h->d, ld));
  if (k < 1 || k > h->n) {  // linear_search.rs:53-58
    set_error("k should be >= 1 and <= length(data)");
    return SC_ERR_INVALID;
  }
  if (k > (1 << 24)) { set_error("k=%lld is too large", (long long)k); return SC_ERR_INVALID; }
  if (form != SC_FORM_FP64 && form != SC_FORM_SPLIT_BF16) { set_error("unknown form %d", form); return SC_ERR_INVALID; }
  // beyond the split kernel's heaps and tiles the FP64 kernel serves the call (same results)
  if (form == SC_FORM_SPLIT_BF16 && !split_knn_serves((int)h->d, (int)k, h->dtype, false)) form = SC_FORM_FP64;
  SC_TRY(knn_reserve(h, m, k));
  SC_TRY(upload_matrix(queries, h->dtype, layout, mem, m, h->d, ld, h->q, h->stream));
  if (form == SC_FORM_FP64)
    return launch_knn_fp64(h->dtype, h->train, h->n, (int)h->d, h->q, m, (int)k, h->idx, h->dist, h->stream);
  return split_knn(&h->split, h->dtype, h->train, h->n, (int)h->d, h->q, m, (int)k, h->idx, h->dist,
                   &h->rescored, h->stream);
}

extern "C" {

void sc_knn_destroy(sc_knn *h) {
  if (!h) return;
  if (h->stream) cudaStreamSynchronize(h->stream);
  cudaStream_t hs = h->stream;
  dfree(h->train, hs); dfree(h->q, hs); dfree(h->idx, hs); dfree(h->dist, hs);
  dfree(h->aux_i, hs); dfree(h->aux_d, hs);
  split_knn_free(&h->split, hs);
  if (h->stream) {
    cudaStreamSynchronize(h->stream);
    cudaStreamDestroy(h->stream);
  }
  if (h->lists) cudaFreeHost(h->lists);
  delete h;
}

sc_status sc_knn_create(const void *train, int32_t dtype, int32_t layout, int32_t mem, int64_t n,
                        int64_t d, int64_t ld, sc_knn **out) {
  if (!out) { set_error("null output handle"); return SC_ERR_INVALID; }
  *out = nullptr;
  SC_TRY(check_matrix(train, dtype, layout, mem, n, d, ld));
  if (n >= ((int64_t)1 << 31)) { set_error("n=%lld exceeds 2^31-1 training rows", (long long)n); return SC_ERR_INVALID; }
  sc_knn *h = new sc_knn();
  h->dtype = dtype; h->n = n; h->d = d;
  sc_status r = SC_OK;
  do {
    if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) {
      r = cuda_fail(cudaGetLastError(), "cudaStreamCreate");
      h->stream = nullptr;
      break;
    }
    if ((r = dalloc((char **)&h->train, (size_t)(n * d) * esize(dtype), h->stream)) != SC_OK) break;
    if ((r = upload_matrix(train, dtype, layout, mem, n, d, ld, h->train, h->stream)) != SC_OK) break;
    if (cudaStreamSynchronize(h->stream) != cudaSuccess) { r = cuda_fail(cudaGetLastError(), "upload"); break; }
  } while (0);
  if (r != SC_OK) { sc_knn_destroy(h); return r; }
  *out = h;
  return SC_OK;
}

void *sc_knn_stream(sc_knn *h) { return h ? (void *)h->stream : nullptr; }

sc_status sc_knn_stats(sc_knn *h, int64_t *rescored) {
  if (!h) { set_error("null handle"); return SC_ERR_INVALID; }
  if (rescored) *rescored = h->rescored;
  return SC_OK;
}

sc_status sc_knn_find(sc_knn *h, const void *queries, int32_t layout, int32_t mem, int64_t m,
                      int64_t ld, int64_t k, int32_t form, int32_t out_mem, int64_t *idx_out,
                      double *dist_out) {
  if (!h) { set_error("null handle"); return SC_ERR_INVALID; }
  SC_TRY(knn_run(h, queries, layout, mem, m, ld, k, form));
  const cudaMemcpyKind kind = out_mem == SC_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  if (m > 0) {
    if (idx_out) SC_CUDA(cudaMemcpyAsync(idx_out, h->idx, (size_t)(m * k) * sizeof(int64_t), kind, h->stream));
    if (dist_out) SC_CUDA(cudaMemcpyAsync(dist_out, h->dist, (size_t)(m * k) * sizeof(double), kind, h->stream));
  }
  SC_CUDA(cudaStreamSynchronize(h->stream));
  return SC_OK;
}

}  // extern "C"

// Pinned host room for `count` row indices in the handle (grows, kept until
// the handle goes): device copies into it run at the link's speed.
static sc_status lists_room(sc_knn *h, int64_t count) {
  if ((size_t)count > h->lists_cap) {
    if (h->lists) cudaFreeHost(h->lists);
    h->lists = nullptr;
    h->lists_cap = 0;
    SC_CUDA(cudaHostAlloc((void **)&h->lists, (size_t)count * sizeof(int64_t), cudaHostAllocDefault));
    h->lists_cap = (size_t)count;
  }
  return SC_OK;
}

// Rows of the handle's training set within `radius` of each of m device
// query rows (row-major), in index order: CSR lists off (m + 1) and *idx,
// which points into the handle's pinned buffer until its next radius search.
static sc_status radius_lists(sc_knn *h, const void *q_dev, int64_t m, double radius, int32_t form,
                              std::vector<int64_t> &off, const int64_t **idx_out) {
  if (form == SC_FORM_SPLIT_BF16 && !split_knn_serves((int)h->d, 1, h->dtype, true)) form = SC_FORM_FP64;
  off.assign((size_t)m + 1, 0);
  *idx_out = nullptr;
  if (m == 0) return SC_OK;
  int64_t *dcnt = nullptr, *doff = nullptr, *didx = nullptr;
  double *ddist = nullptr;
  if (form == SC_FORM_SPLIT_BF16) {  // usually one pass
    sc_status r = split_knn_radius_lists(&h->split, h->dtype, h->train, h->n, (int)h->d, q_dev, m, radius, off,
                                         &didx, &ddist, h->stream);
    if (r == SC_OK) {
      const int64_t total = off[(size_t)m];
      if (total > 0 && (r = lists_room(h, total)) == SC_OK) {
        if (cudaMemcpyAsync(h->lists, didx, (size_t)total * sizeof(int64_t), cudaMemcpyDeviceToHost, h->stream) !=
                cudaSuccess ||
            cudaStreamSynchronize(h->stream) != cudaSuccess)
          r = cuda_fail(cudaGetLastError(), "radius lists");
        *idx_out = h->lists;
      }
      cudaStreamSynchronize(h->stream);
      dfree(didx, h->stream);
      dfree(ddist, h->stream);
      return r;
    }
    if (r != SC_ERR_INVALID) return r;
    off.assign((size_t)m + 1, 0);  // too many queries for the slots: count, then fill
  }
  sc_status r = SC_OK;
  do {
    if ((r = dalloc(&dcnt, (size_t)m, h->stream)) != SC_OK || (r = dalloc(&doff, (size_t)m, h->stream)) != SC_OK) break;
    r = form == SC_FORM_FP64
            ? launch_knn_radius_fp64(h->dtype, h->train, h->n, (int)h->d, q_dev, m, radius, dcnt, nullptr, nullptr,
                                     nullptr, h->stream)
            : split_knn_radius(&h->split, h->dtype, h->train, h->n, (int)h->d, q_dev, m, radius, dcnt, nullptr,
                               nullptr, nullptr, h->stream);
    if (r != SC_OK) break;
    if (cudaMemcpyAsync(off.data() + 1, dcnt, (size_t)m * sizeof(int64_t), cudaMemcpyDeviceToHost, h->stream) !=
            cudaSuccess ||
        cudaStreamSynchronize(h->stream) != cudaSuccess) {
      r = cuda_fail(cudaGetLastError(), "radius counts");
      break;
    }
    for (int64_t q = 0; q < m; ++q) off[(size_t)q + 1] += off[(size_t)q];
    const int64_t total = off[(size_t)m];
    if (total == 0) break;
    if ((r = lists_room(h, total)) != SC_OK) break;
    if ((r = dalloc(&didx, (size_t)total, h->stream)) != SC_OK || (r = dalloc(&ddist, (size_t)total, h->stream)) != SC_OK) break;
    if (cudaMemcpyAsync(doff, off.data(), (size_t)m * sizeof(int64_t), cudaMemcpyHostToDevice, h->stream) !=
        cudaSuccess) {
      r = cuda_fail(cudaGetLastError(), "radius offsets");
      break;
    }
    r = form == SC_FORM_FP64
            ? launch_knn_radius_fp64(h->dtype, h->train, h->n, (int)h->d, q_dev, m, radius, nullptr, doff, didx,
                                     ddist, h->stream)
            : split_knn_radius(&h->split, h->dtype, h->train, h->n, (int)h->d, q_dev, m, radius, nullptr, doff,
                               didx, ddist, h->stream);
    if (r != SC_OK) break;
    if (cudaMemcpyAsync(h->lists, didx, (size_t)total * sizeof(int64_t), cudaMemcpyDeviceToHost, h->stream) !=
            cudaSuccess ||
        cudaStreamSynchronize(h->stream) != cudaSuccess) {
      r = cuda_fail(cudaGetLastError(), "radius lists");
      break;
    }
    *idx_out = h->lists;
  } while (0);
  cudaStreamSynchronize(h->stream);
  dfree(dcnt, h->stream); dfree(doff, h->stream); dfree(didx, h->stream); dfree(ddist, h->stream);
  return r;
}

// The expansion loop of DBSCAN::fit (src/cluster/dbscan.rs:299-360) over
// precomputed neighbourhoods (each find_radius result is fixed by its query
// row, so computing all of them first changes nothing): the same marks
// (undefined -3, queued -2, outlier -1), the same LIFO stack of neighbours and
// the same order of visits.  Returns the number of clusters.
static int64_t dbscan_expand(int64_t n, const std::vector<int64_t> &off, const int64_t *idx,
                             int64_t min_samples, int64_t *y) {
  const int64_t queued = -2, outlier = -1, undefined = -3;
  for (int64_t i = 0; i < n; ++i) y[i] = undefined;
  int64_t k = 0;
  std::vector<int64_t> stack;
  for (int64_t i = 0; i < n; ++i) {
    if (y[i] != undefined) continue;
    const int64_t *nb = idx + off[(size_t)i];
    const int64_t nn = off[(size_t)i + 1] - off[(size_t)i];
    if (nn < min_samples) {
      y[i] = outlier;
      continue;
    }
    y[i] = k;
    for (int64_t j = 0; j < nn; ++j)
      if (y[nb[j]] == undefined) y[nb[j]] = queued;
    stack.assign(nb, nb + nn);
    while (!stack.empty()) {
      const int64_t index = stack.back();
      stack.pop_back();
      if (y[index] == outlier) y[index] = k;
      if (y[index] == undefined || y[index] == queued) {
        y[index] = k;
        const int64_t *sec = idx + off[(size_t)index];
        const int64_t ns = off[(size_t)index + 1] - off[(size_t)index];
        if (ns >= min_samples) {
          for (int64_t j = 0; j < ns; ++j) {
            const int64_t label = y[sec[j]];
            if (label == undefined) y[sec[j]] = queued;
            if (label == undefined || label == outlier) stack.push_back(sec[j]);
          }
        }
      }
    }
    ++k;
  }
  return k;
}

extern "C" {

sc_status sc_dbscan_fit(sc_knn *h, double eps, int64_t min_samples, int32_t form, int64_t *labels_out,
                        int64_t *n_clusters_out) {
  if (!h) { set_error("null handle"); return SC_ERR_INVALID; }
  if (min_samples < 1) { set_error("Invalid minPts"); return SC_ERR_INVALID; }  // dbscan.rs:278-280
  if (!(eps > 0.0)) { set_error("Invalid radius: "); return SC_ERR_INVALID; }   // dbscan.rs:282-284
  if (form != SC_FORM_FP64 && form != SC_FORM_SPLIT_BF16) { set_error("unknown form %d", form); return SC_ERR_INVALID; }
  if (!labels_out && h->n > 0) { set_error("null labels"); return SC_ERR_INVALID; }
  std::vector<int64_t> off;
  const int64_t *idx = nullptr;
  SC_TRY(radius_lists(h, h->train, h->n, eps, form, off, &idx));  // every row's neighbourhood
  const int64_t k = dbscan_expand(h->n, off, idx, min_samples, labels_out);
  if (n_clusters_out) *n_clusters_out = k;
  return SC_OK;
}

sc_status sc_dbscan_predict(sc_knn *h, const void *queries, int32_t layout, int32_t mem, int64_t m, int64_t ld,
                            double eps, int32_t form, const int64_t *train_labels, int64_t n_clusters,
                            int64_t *out) {
  if (!h) { set_error("null handle"); return SC_ERR_INVALID; }
  if (!(eps > 0.0)) { set_error("radius should be > 0"); return SC_ERR_INVALID; }  // linear_search.rs:90-95
  SC_TRY(check_matrix(queries, h->dtype, layout, mem, m, h->d, ld));
  if (form != SC_FORM_FP64 && form != SC_FORM_SPLIT_BF16) { set_error("unknown form %d", form); return SC_ERR_INVALID; }
  if (n_clusters < 0 || (!train_labels && h->n > 0) || (!out && m > 0)) { set_error("invalid labels"); return SC_ERR_INVALID; }
  if (m == 0) return SC_OK;
  SC_TRY(knn_reserve(h, m, 1));
  SC_TRY(upload_matrix(queries, h->dtype, layout, mem, m, h->d, ld, h->q, h->stream));
  std::vector<int64_t> off;
  const int64_t *idx = nullptr;
  SC_TRY(radius_lists(h, h->q, m, eps, form, off, &idx));
  // dbscan.rs:378-397: votes per cluster, noise counted last; the first
  // maximum wins (which_max, src/tree/decision_tree_classifier.rs:490-502)
  std::vector<int64_t> votes((size_t)n_clusters + 1);
  for (int64_t q = 0; q < m; ++q) {
    std::fill(votes.begin(), votes.end(), 0);
    for (int64_t e = off[(size_t)q]; e < off[(size_t)q + 1]; ++e) {
      const int64_t yi = train_labels[idx[e]];
      ++votes[yi < 0 ? (size_t)n_clusters : (size_t)yi];
    }
    size_t which = 0;
    for (size_t c = 1; c < votes.size(); ++c)
      if (votes[c] > votes[which]) which = c;
    out[q] = which != (size_t)n_clusters ? (int64_t)which + 1 : 0;
  }
  return SC_OK;
}

sc_status sc_fastpair(sc_knn *h, int64_t *neighbour_out, double *distance_out, int64_t *closest_out,
                      double *closest_distance_out) {
  if (!h) { set_error("null handle"); return SC_ERR_INVALID; }
  if (h->n < 3) { set_error("min number of rows should be 3"); return SC_ERR_INVALID; }  // fastpair.rs:60-65
  const int64_t n = h->n;
  std::vector<int64_t> nb((size_t)n);
  std::vector<double> dist((size_t)n);
  int64_t *dnb = nullptr;
  double *ddist = nullptr;
  sc_status r = SC_OK;
  do {
    if ((r = dalloc(&dnb, (size_t)n, h->stream)) != SC_OK || (r = dalloc(&ddist, (size_t)n, h->stream)) != SC_OK) break;
    if ((r = launch_fastpair(h->dtype, h->train, n, (int)h->d, dnb, ddist, h->stream)) != SC_OK) break;
    if (cudaMemcpyAsync(nb.data(), dnb, (size_t)n * sizeof(int64_t), cudaMemcpyDeviceToHost, h->stream) !=
            cudaSuccess ||
        cudaMemcpyAsync(dist.data(), ddist, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost, h->stream) !=
            cudaSuccess ||
        cudaStreamSynchronize(h->stream) != cudaSuccess) {
      r = cuda_fail(cudaGetLastError(), "fastpair");
      break;
    }
  } while (0);
  cudaStreamSynchronize(h->stream);
  dfree(dnb, h->stream); dfree(ddist, h->stream);
  if (r != SC_OK) return r;
  if (neighbour_out) memcpy(neighbour_out, nb.data(), (size_t)n * sizeof(int64_t));
  if (distance_out) memcpy(distance_out, dist.data(), (size_t)n * sizeof(double));
  // closest_pair (fastpair.rs:165-182): the first smallest distance along the
  // neighbours list 0, 1, ..., n - 1
  int64_t a = 0;
  for (int64_t p = 0; p < n; ++p)
    if (dist[(size_t)p] < dist[(size_t)a]) a = p;
  if (closest_out) { closest_out[0] = a; closest_out[1] = nb[(size_t)a]; }
  if (closest_distance_out) *closest_distance_out = dist[(size_t)a];
  return SC_OK;
}

sc_status sc_knn_find_radius(sc_knn *h, const void *queries, int32_t layout, int32_t mem, int64_t m,
                             int64_t ld, double radius, int32_t form, int64_t *counts_out, int64_t capacity,
                             int64_t *idx_out, double *dist_out, int64_t *total_out) {
  if (!h) { set_error("null handle"); return SC_ERR_INVALID; }
  if (!(radius > 0.0)) { set_error("radius should be > 0"); return SC_ERR_INVALID; }  // linear_search.rs:90-95
  SC_TRY(check_matrix(queries, h->dtype, layout, mem, m, h->d, ld));
  if (form != SC_FORM_FP64 && form != SC_FORM_SPLIT_BF16) { set_error("unknown form %d", form); return SC_ERR_INVALID; }
  if (form == SC_FORM_SPLIT_BF16 && !split_knn_serves((int)h->d, 1, h->dtype, true)) form = SC_FORM_FP64;
  if (total_out) *total_out = 0;
  if (m == 0) return SC_OK;
  SC_TRY(knn_reserve(h, m, 1));
  SC_TRY(upload_matrix(queries, h->dtype, layout, mem, m, h->d, ld, h->q, h->stream));
  int64_t *dcnt = nullptr, *doff = nullptr, *didx = nullptr;
  double *ddist = nullptr;
  sc_status r = SC_OK;
  std::vector<int64_t> cnt((size_t)m);
  int64_t total = 0;
  if (form == SC_FORM_SPLIT_BF16 && (idx_out || dist_out)) {  // usually one pass: counts and rows together
    std::vector<int64_t> off;
    r = split_knn_radius_lists(&h->split, h->dtype, h->train, h->n, (int)h->d, h->q, m, radius, off, &didx, &ddist,
                               h->stream);
    if (r == SC_OK) {
      total = off[(size_t)m];
      for (int64_t q = 0; q < m; ++q) cnt[(size_t)q] = off[(size_t)q + 1] - off[(size_t)q];
      if (counts_out) memcpy(counts_out, cnt.data(), (size_t)m * sizeof(int64_t));
      if (total_out) *total_out = total;
      if (capacity < total) {
        set_error("capacity %lld is smaller than the %lld neighbours found", (long long)capacity, (long long)total);
        r = SC_ERR_INVALID;
      } else if (total > 0 &&
                 ((idx_out && cudaMemcpyAsync(idx_out, didx, (size_t)total * sizeof(int64_t), cudaMemcpyDeviceToHost,
                                              h->stream) != cudaSuccess) ||
                  (dist_out && cudaMemcpyAsync(dist_out, ddist, (size_t)total * sizeof(double),
                                               cudaMemcpyDeviceToHost, h->stream) != cudaSuccess) ||
                  cudaStreamSynchronize(h->stream) != cudaSuccess)) {
        r = cuda_fail(cudaGetLastError(), "find_radius results");
      }
      cudaStreamSynchronize(h->stream);
      dfree(didx, h->stream);
      dfree(ddist, h->stream);
      return r;
    }
    if (r != SC_ERR_INVALID) return r;
    r = SC_OK;  // too many queries for the slots: count, then fill
    didx = nullptr;
    ddist = nullptr;
  }
  do {
    if ((r = dalloc(&dcnt, (size_t)m, h->stream)) != SC_OK || (r = dalloc(&doff, (size_t)m, h->stream)) != SC_OK) break;
    // counting pass
    r = form == SC_FORM_FP64
            ? launch_knn_radius_fp64(h->dtype, h->train, h->n, (int)h->d, h->q, m, radius, dcnt, nullptr, nullptr,
                                     nullptr, h->stream)
            : split_knn_radius(&h->split, h->dtype, h->train, h->n, (int)h->d, h->q, m, radius, dcnt, nullptr,
                               nullptr, nullptr, h->stream);
    if (r != SC_OK) break;
    if (cudaMemcpyAsync(cnt.data(), dcnt, (size_t)m * sizeof(int64_t), cudaMemcpyDeviceToHost, h->stream) !=
            cudaSuccess ||
        cudaStreamSynchronize(h->stream) != cudaSuccess) {
      r = cuda_fail(cudaGetLastError(), "find_radius counts");
      break;
    }
    std::vector<int64_t> off((size_t)m);
    for (int64_t q = 0; q < m; ++q) { off[(size_t)q] = total; total += cnt[(size_t)q]; }
    if (counts_out) memcpy(counts_out, cnt.data(), (size_t)m * sizeof(int64_t));
    if (total_out) *total_out = total;
    if (!idx_out && !dist_out) break;  // counts only
    if (capacity < total) {
      set_error("capacity %lld is smaller than the %lld neighbours found", (long long)capacity, (long long)total);
      r = SC_ERR_INVALID;
      break;
    }
    if (total == 0) break;
    if ((r = dalloc(&didx, (size_t)total, h->stream)) != SC_OK || (r = dalloc(&ddist, (size_t)total, h->stream)) != SC_OK) break;
    if (cudaMemcpyAsync(doff, off.data(), (size_t)m * sizeof(int64_t), cudaMemcpyHostToDevice, h->stream) !=
        cudaSuccess) {
      r = cuda_fail(cudaGetLastError(), "find_radius offsets");
      break;
    }
    // filling pass
    r = form == SC_FORM_FP64
            ? launch_knn_radius_fp64(h->dtype, h->train, h->n, (int)h->d, h->q, m, radius, nullptr, doff, didx,
                                     ddist, h->stream)
            : split_knn_radius(&h->split, h->dtype, h->train, h->n, (int)h->d, h->q, m, radius, nullptr, doff,
                               didx, ddist, h->stream);
    if (r != SC_OK) break;
    if ((idx_out && cudaMemcpyAsync(idx_out, didx, (size_t)total * sizeof(int64_t), cudaMemcpyDeviceToHost,
                                    h->stream) != cudaSuccess) ||
        (dist_out && cudaMemcpyAsync(dist_out, ddist, (size_t)total * sizeof(double), cudaMemcpyDeviceToHost,
                                     h->stream) != cudaSuccess) ||
        cudaStreamSynchronize(h->stream) != cudaSuccess) {
      r = cuda_fail(cudaGetLastError(), "find_radius results");
      break;
    }
  } while (0);
  cudaStreamSynchronize(h->stream);
  dfree(dcnt, h->stream); dfree(doff, h->stream); dfree(didx, h->stream); dfree(ddist, h->stream);
  return r;
}

sc_status sc_knn_classify(sc_knn *h, const void *queries, int32_t layout, int32_t mem, int64_t m,
                          int64_t ld, int64_t k, int32_t form, int32_t weight,
                          const int64_t *y_class, int64_t n_classes, int64_t *classes_out) {
  if (!h) { set_error("null handle"); return SC_ERR_INVALID; }
  if (!y_class || n_classes < 1) { set_error("invalid class labels"); return SC_ERR_INVALID; }
  SC_TRY(knn_run(h, queries, layout, mem, m, ld, k, form));
  if (h->aux_cap < std::max(h->n, m)) {
    h->aux_cap = 0;
    dfree(h->aux_i, h->stream); dfree(h->aux_d, h->stream);
    SC_TRY(dalloc(&h->aux_i, (size_t)(h->n + m), h->stream));
    SC_TRY(dalloc(&h->aux_d, (size_t)(h->n + m), h->stream));
    h->aux_cap = std::max(h->n, m);
  }
  SC_CUDA(cudaMemcpyAsync(h->aux_i, y_class, (size_t)h->n * sizeof(int64_t), cudaMemcpyHostToDevice, h->stream));
  SC_TRY(launch_knn_vote(h->idx, h->dist, m, (int)k, weight, h->aux_i, h->aux_i + h->n, h->stream));
  if (m > 0) SC_CUDA(cudaMemcpyAsync(classes_out, h->aux_i + h->n, (size_t)m * sizeof(int64_t), cudaMemcpyDeviceToHost, h->stream));
  SC_CUDA(cudaStreamSynchronize(h->stream));
  return SC_OK;
}

sc_status sc_knn_regress(sc_knn *h, const void *queries, int32_t layout, int32_t mem, int64_t m,
                         int64_t ld, int64_t k, int32_t form, int32_t weight, const double *y,
                         double *out) {
  if (!h) { set_error("null handle"); return SC_ERR_INVALID; }
  if (!y) { set_error("null targets"); return SC_ERR_INVALID; }
  SC_TRY(knn_run(h, queries, layout, mem, m, ld, k, form));
  if (h->aux_cap < std::max(h->n, m)) {
    h->aux_cap = 0;
    dfree(h->aux_i, h->stream); dfree(h->aux_d, h->stream);
    SC_TRY(dalloc(&h->aux_i, (size_t)(h->n + m), h->stream));
    SC_TRY(dalloc(&h->aux_d, (size_t)(h->n + m), h->stream));
    h->aux_cap = std::max(h->n, m);
  }
  SC_CUDA(cudaMemcpyAsync(h->aux_d, y, (size_t)h->n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  SC_TRY(launch_knn_regress(h->idx, h->dist, m, (int)k, weight, h->aux_d, h->aux_d + h->n, h->stream));
  if (m > 0) SC_CUDA(cudaMemcpyAsync(out, h->aux_d + h->n, (size_t)m * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  SC_CUDA(cudaStreamSynchronize(h->stream));
  return SC_OK;
}

}  // extern "C"
