// FP64 kernels that keep smartcore's own operation order, so every distance
// they produce is bit-identical to the reference CPU value.
//
// This translation unit is compiled with -fmad=false, and every arithmetic
// step is also spelled with an explicit round-to-nearest intrinsic: no
// multiply-add is ever fused (rustc never fuses either).
#include <float.h>

#include "common.cuh"
#include "exactsum.cuh"

namespace sc {

// One term of Euclidian::squared_distance (src/metrics/distance/
// euclidian.rs:56-62): r = a - b and r * r in the element type, then to_f64.
__device__ __forceinline__ double sq_term(float a, float b) {
  float r = __fsub_rn(a, b);
  return (double)__fmul_rn(r, r);
}
__device__ __forceinline__ double sq_term(double a, double b) {
  double r = __dsub_rn(a, b);
  return __dmul_rn(r, r);
}

// Fixed-order block sum (warp shuffle tree, then warps in index order).
// Every thread passes a value; thread 0 returns the total.
template <int kThreads>
__device__ __forceinline__ double block_sum_fixed(double v) {
  __shared__ double ws[kThreads / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = __dadd_rn(v, __shfl_down_sync(0xffffffffu, v, o));
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) ws[w] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < kThreads / 32; ++i) t = __dadd_rn(t, ws[i]);
  return t;
}

// ---------------------------------------------------------------------------
// K1: assignment in FP64 — KMeans::predict (src/cluster/kmeans.rs:327-352)
// and the per-point outcome of BBDTree::clustering (src/algorithm/neighbour/
// bbd_tree.rs:101-111 at the leaves): argmin over centroids of
// sum_j (f64(x_j) - c_j)^2, strict <, lowest index wins ties; min starts at
// f64::MAX.  Also writes the block's fixed-order sum of the winning distances
// (the distortion of this step) to part[blockIdx.x].
// ---------------------------------------------------------------------------
constexpr int kAssignThreads = 128;

template <typename T>
__global__ void __launch_bounds__(kAssignThreads)
assign_fp64_kernel(const T *__restrict__ x, int64_t n, int d,
                   const double *__restrict__ cent, int k, int ktile,
                   int32_t *__restrict__ labels, double *__restrict__ part,
                   const LloydState *st) {
  if (st && st->done) return;
  extern __shared__ double cs[];  // ktile x d centroid tile
  const int64_t i = (int64_t)blockIdx.x * kAssignThreads + threadIdx.x;
  const bool live = i < n;
  const T *xr = x + (live ? i : 0) * (int64_t)d;
  double best = DBL_MAX;
  int bi = 0;
  for (int c0 = 0; c0 < k; c0 += ktile) {
    const int kt = min(ktile, k - c0);
    __syncthreads();
    for (int t = threadIdx.x; t < kt * d; t += kAssignThreads) cs[t] = cent[(int64_t)c0 * d + t];
    __syncthreads();
    if (!live) continue;
    int c = 0;
    for (; c + 4 <= kt; c += 4) {
      const double *p = cs + c * d;
      double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
      for (int j = 0; j < d; ++j) {
        const double xj = (double)xr[j];
        a0 = __dadd_rn(a0, sq_term(xj, p[j]));
        a1 = __dadd_rn(a1, sq_term(xj, p[d + j]));
        a2 = __dadd_rn(a2, sq_term(xj, p[2 * d + j]));
        a3 = __dadd_rn(a3, sq_term(xj, p[3 * d + j]));
      }
      if (a0 < best) { best = a0; bi = c0 + c; }
      if (a1 < best) { best = a1; bi = c0 + c + 1; }
      if (a2 < best) { best = a2; bi = c0 + c + 2; }
      if (a3 < best) { best = a3; bi = c0 + c + 3; }
    }
    for (; c < kt; ++c) {
      const double *p = cs + c * d;
      double a = 0.0;
      for (int j = 0; j < d; ++j) a = __dadd_rn(a, sq_term((double)xr[j], p[j]));
      if (a < best) { best = a; bi = c0 + c; }
    }
  }
  if (live) labels[i] = bi;
  const double tot = block_sum_fixed<kAssignThreads>(live ? best : 0.0);
  if (threadIdx.x == 0 && part) part[blockIdx.x] = tot;
}

int assign_block_count(int64_t n) { return (int)((n + kAssignThreads - 1) / kAssignThreads); }

sc_status launch_assign_fp64(int dtype, const void *x, int64_t n, int d,
                             const double *cent, int k, int32_t *labels,
                             double *part, const LloydState *st,
                             cudaStream_t s) {
  if (n == 0) return SC_OK;
  const int max_smem = 96 * 1024;
  int ktile = max_smem / (d * (int)sizeof(double));
  if (ktile < 1) {
    set_error("d=%d is too large for the FP64 assignment kernel", d);
    return SC_ERR_INVALID;
  }
  if (ktile > k) ktile = k;
  const size_t smem = (size_t)ktile * d * sizeof(double);
  const int grid = assign_block_count(n);
  if (dtype == SC_F32) {
    auto kern = assign_fp64_kernel<float>;
    SC_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    kern<<<grid, kAssignThreads, smem, s>>>((const float *)x, n, d, cent, k, ktile, labels, part, st);
  } else {
    auto kern = assign_fp64_kernel<double>;
    SC_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    kern<<<grid, kAssignThreads, smem, s>>>((const double *)x, n, d, cent, k, ktile, labels, part, st);
  }
  SC_LAUNCHED();
  return SC_OK;
}

// ---------------------------------------------------------------------------
// K3: k-means++ D^2 update — KMeans::kmeans_plus_plus (src/cluster/
// kmeans.rs:367-379 and :399-410).  The seed row is st->pp_chosen; the
// distance uses the element type's arithmetic (a - b and its square in T,
// summed in f64).  first_pass initialises d = f64::MAX and y = 0 (:357, :364).
// ---------------------------------------------------------------------------
constexpr int kPPThreads = 256;

int pp_block_count(int64_t n) { return (int)((n + kPPThreads - 1) / kPPThreads); }

template <typename T>
__global__ void __launch_bounds__(kPPThreads)
pp_update_kernel(const T *__restrict__ x, int64_t n, int d, const LloydState *st,
                 int32_t label_of_seed, double *__restrict__ dd,
                 int32_t *__restrict__ labels, double *__restrict__ part,
                 int first_pass, int lg_d) {
  extern __shared__ unsigned char smraw[];
  T *cen = reinterpret_cast<T *>(smraw);
  const int64_t ci = st->pp_chosen;
  for (int t = threadIdx.x; t < d; t += kPPThreads) cen[t] = x[ci * d + t];
  __syncthreads();
  const int64_t i = (int64_t)blockIdx.x * kPPThreads + threadIdx.x;
  double v = 0.0;
  if (i < n) {
    const T *xr = x + i * (int64_t)d;
    double s = 0.0;
    bool exact = false;
    // f32 rows: the same value from the integer reproduction of the sequential sum
    if constexpr (sizeof(T) == 4) exact = sqd_seq_f32(xr, cen, d, lg_d, s);
    if (!exact) {
      s = 0.0;
      for (int j = 0; j < d; ++j) s = __dadd_rn(s, sq_term(xr[j], cen[j]));
    }
    double cur = first_pass ? DBL_MAX : dd[i];
    int32_t lab = first_pass ? 0 : labels[i];
    if (s < cur) { cur = s; lab = label_of_seed; }
    dd[i] = cur;
    labels[i] = lab;
    v = cur;
  }
  const double tot = block_sum_fixed<kPPThreads>(v);
  if (threadIdx.x == 0 && part) part[blockIdx.x] = tot;
}

// f32 rows, d <= 128: the same update with each warp's 32 rows staged in
// shared memory by coalesced loads (row stride d + 1: conflict-free when each
// lane then walks its own row).  Thread t still handles row 256 b + t, so the
// block partials are the same.
__global__ void __launch_bounds__(kPPThreads)
pp_update_staged_kernel(const float *__restrict__ x, int64_t n, int d, const LloydState *st,
                        int32_t label_of_seed, double *__restrict__ dd, int32_t *__restrict__ labels,
                        double *__restrict__ part, int first_pass, int lg_d) {
  extern __shared__ float smf[];
  float *cen = smf;                                                // d
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  float *tile = smf + ((d + 3) & ~3) + (size_t)w * 32 * (d + 1);  // 32 rows x (d + 1)
  const int64_t ci = st->pp_chosen;
  for (int t = threadIdx.x; t < d; t += kPPThreads) cen[t] = x[ci * d + t];
  const int64_t r0 = (int64_t)blockIdx.x * kPPThreads + w * 32;
  // asynchronous 4-byte copies: every row of the warp in flight at once
  for (int rr = 0; rr < 32; ++rr) {
    const int64_t i = r0 + rr;
    if (i < n)
      for (int c = lane; c < d; c += 32) {
        const uint32_t dst = (uint32_t)__cvta_generic_to_shared(tile + rr * (d + 1) + c);
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(dst), "l"(x + i * d + c) : "memory");
      }
  }
  asm volatile("cp.async.wait_all;" ::: "memory");
  __syncthreads();
  __shared__ int s_q[kPPThreads];  // block rows that need the exact distance
  __shared__ double s_v[kPPThreads];
  __shared__ int s_qn;
  if (threadIdx.x == 0) s_qn = 0;
  __syncthreads();
  const int64_t i = r0 + lane;
  double cur = DBL_MAX;
  if (i < n) {
    const float *xr = tile + lane * (d + 1);
    cur = first_pass ? DBL_MAX : dd[i];
    // The reference's terms q_t = fl32((x_t - c_t)^2) summed in f32 bound its
    // f64 sum from below by s32 (1 - 1.05 d 2^-24): when that exceeds the
    // current distance, the row keeps it and the exact sum is not needed.
    float s32 = 0.f;
    for (int j = 0; j < d; ++j) {
      const float r = __fsub_rn(xr[j], cen[j]);
      s32 = __fadd_rn(s32, __fmul_rn(r, r));
    }
    const bool keep = !first_pass && __fmul_rd(s32, 1.f - 1.05f * d * 0x1p-24f) > __double2float_ru(cur);
    if (!keep) s_q[atomicAdd(&s_qn, 1)] = threadIdx.x;
  }
  s_v[threadIdx.x] = i < n ? cur : 0.0;
  __syncthreads();
  // the rows that need it, on contiguous threads (full warps)
  const int qn = s_qn;
  for (int qi = threadIdx.x; qi < qn; qi += kPPThreads) {
    const int t = s_q[qi];
    const int64_t row = (int64_t)blockIdx.x * kPPThreads + t;
    const float *xr = smf + ((d + 3) & ~3) + (size_t)(t >> 5) * 32 * (d + 1) + (t & 31) * (d + 1);
    double sq = 0.0;
    if (!sqd_seq_f32(xr, cen, d, lg_d, sq)) {
      sq = 0.0;
      for (int j = 0; j < d; ++j) sq = __dadd_rn(sq, sq_term(xr[j], cen[j]));
    }
    double c = s_v[t];
    int32_t lab = first_pass ? 0 : labels[row];
    if (sq < c) { c = sq; lab = label_of_seed; }
    dd[row] = c;
    labels[row] = lab;
    s_v[t] = c;
  }
  __syncthreads();
  const double v = s_v[threadIdx.x];
  const double tot = block_sum_fixed<kPPThreads>(v);
  if (threadIdx.x == 0 && part) part[blockIdx.x] = tot;
}

sc_status launch_pp_update(int dtype, const void *x, int64_t n, int d,
                           const LloydState *st, int32_t label_of_seed,
                           double *dd, int32_t *labels, double *part,
                           int first_pass, cudaStream_t s) {
  const int grid = pp_block_count(n);
  const size_t smem = (size_t)d * (dtype == SC_F32 ? 4 : 8);
  if (smem > 48 * 1024) {
    set_error("d=%d is too large for the k-means++ kernel", d);
    return SC_ERR_INVALID;
  }
  int lg_d = 0;
  while ((1 << lg_d) < d) ++lg_d;
  if (dtype == SC_F32 && d <= 128) {
    const size_t ssm = ((size_t)((d + 3) & ~3) + (size_t)kPPThreads * (d + 1)) * sizeof(float);
    SC_CUDA(cudaFuncSetAttribute(pp_update_staged_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ssm));
    pp_update_staged_kernel<<<grid, kPPThreads, ssm, s>>>((const float *)x, n, d, st, label_of_seed, dd, labels,
                                                          part, first_pass, lg_d);
  } else if (dtype == SC_F32)
    pp_update_kernel<float><<<grid, kPPThreads, smem, s>>>((const float *)x, n, d, st, label_of_seed, dd, labels, part, first_pass, lg_d);
  else
    pp_update_kernel<double><<<grid, kPPThreads, smem, s>>>((const double *)x, n, d, st, label_of_seed, dd, labels, part, first_pass, lg_d);
  SC_LAUNCHED();
  return SC_OK;
}

// ---------------------------------------------------------------------------
// k-means++ seed selection (kmeans.rs:381-396): sum = sequential f64 sum of
// d, cutoff = u * sum, index = first i whose sequential prefix >= cutoff.
//
// The sequential prefix S_i is inherently serial.  Here a parallel prefix
// Q_i (block partials, then a chunked scan) locates the candidate, and the
// choice is certified with a rigorous bound: all d_i >= 0, so
// |S_i - P_i| <= gamma_i P_i (Higham) for the exact prefix P_i, and Q_i obeys
// the same bound with the depth of its own summation tree.  Only when the
// cutoff falls inside the uncertainty band of the crossing is the draw
// resolved by pp_replay_kernel, which recomputes S exactly as the reference
// does, on one thread.
// ---------------------------------------------------------------------------
constexpr int kSelThreads = 1024;

__device__ __forceinline__ double pp_tol(double q, double depth) {
  // (depth) * 2^-53 * q, inflated by 1% to absorb the rounding of this bound
  return depth * 1.1102230246251565e-16 * 1.01 * q;
}

__global__ void __launch_bounds__(kSelThreads)
pp_select_kernel(const double *__restrict__ dd, const double *__restrict__ part,
                 int64_t n, int nb, const double *__restrict__ uniform,
                 LloydState *st) {
  __shared__ double scan[kSelThreads];
  __shared__ int s_chunk;
  const int t = threadIdx.x;
  const int chunk = (nb + kSelThreads - 1) / kSelThreads;
  const int b0 = min(nb, t * chunk), b1 = min(nb, b0 + chunk);
  double loc = 0.0;
  for (int b = b0; b < b1; ++b) loc = __dadd_rn(loc, part[b]);
  scan[t] = loc;
  if (t == 0) s_chunk = kSelThreads;
  __syncthreads();
  for (int o = 1; o < kSelThreads; o <<= 1) {  // inclusive Hillis-Steele scan
    double add = t >= o ? scan[t - o] : 0.0;
    __syncthreads();
    scan[t] = __dadd_rn(scan[t], add);
    __syncthreads();
  }
  const double total = scan[kSelThreads - 1];
  const double u = *uniform;
  const double cutoff = __dmul_rn(u, total);
  const double depth_q = (double)chunk + 2.0 * kSelThreads + 2.0 * kPPThreads + 64.0;
  const double excl = t > 0 ? scan[t - 1] : 0.0;
  if (b1 > b0 && scan[t] >= cutoff && !(excl >= cutoff)) atomicMin(&s_chunk, t);
  __syncthreads();
  if (t != 0) return;
  const bool finite = isfinite(total) && total < DBL_MAX;
  const double tol_tot = pp_tol(total, (double)n + depth_q);
  const double cut_lo = __dmul_rn(u, __dsub_rn(total, tol_tot));
  const double cut_hi = __dmul_rn(u, __dadd_rn(total, tol_tot));
  int64_t pick = -1;
  if (finite && s_chunk < kSelThreads) {
    const int c = s_chunk;
    const int cb0 = c * chunk, cb1 = min(nb, cb0 + chunk);
    double base = c > 0 ? scan[c - 1] : 0.0;
    int b = cb0;
    for (; b < cb1; ++b) {
      const double nxt = __dadd_rn(base, part[b]);
      if (nxt >= cutoff) break;
      base = nxt;
    }
    if (b < cb1) {
      const int64_t i0 = (int64_t)b * kPPThreads, i1 = min(n, i0 + kPPThreads);
      double q = base, qprev = base;
      int64_t i = i0;
      for (; i < i1; ++i) {
        qprev = q;
        q = __dadd_rn(q, dd[i]);
        if (q >= cutoff) break;
      }
      if (i < i1) {
        const bool above = __dsub_rn(q, pp_tol(q, (double)i + depth_q)) >= cut_hi;
        const bool below = i == 0 ? (0.0 < cut_lo)
                                  : (__dadd_rn(qprev, pp_tol(qprev, (double)i + depth_q)) < cut_lo);
        if (above && below) pick = i;
      }
    }
  }
  if (pick >= 0) {
    st->pp_chosen = pick;
    st->pp_flag = 0;
  } else {
    st->pp_flag = 1;
  }
}

// The exact serial computation of kmeans.rs:381-396, used only when the
// certified parallel selection could not decide.
__global__ void pp_replay_kernel(const double *__restrict__ dd, int64_t n,
                                 const double *__restrict__ uniform,
                                 LloydState *st) {
  if (!st->pp_flag) return;
  double sum = 0.0;
  for (int64_t i = 0; i < n; ++i) sum = __dadd_rn(sum, dd[i]);
  const double cutoff = __dmul_rn(*uniform, sum);
  double cost = 0.0;
  int64_t index = 0;
  while (index < n) {
    cost = __dadd_rn(cost, dd[index]);
    if (cost >= cutoff) break;
    ++index;
  }
  st->pp_chosen = index < n ? index : n - 1;
  st->pp_flag = 0;
  st->pp_replays += 1;
}

sc_status launch_pp_select(const double *dd, const double *part, int64_t n,
                           int nb, const double *uniform, LloydState *st,
                           cudaStream_t s) {
  pp_select_kernel<<<1, kSelThreads, 0, s>>>(dd, part, n, nb, uniform, st);
  SC_LAUNCHED();
  pp_replay_kernel<<<1, 1, 0, s>>>(dd, n, uniform, st);
  SC_LAUNCHED();
  return SC_OK;
}

// ---------------------------------------------------------------------------
// K4: LinearKNNSearch::find (src/algorithm/neighbour/linear_search.rs:52-84)
// in FP64, one query per thread.  The training rows stream through shared
// memory in index order; each thread keeps the reference's k-slot heap and
// replays it exactly: a row enters iff its distance is strictly below
// heap[0], which it replaces, followed by a full heapify
// (src/algorithm/sort/heap_select.rs:42-50, :71-86).
// ---------------------------------------------------------------------------
constexpr int kKnnTile = 32;  // training rows per shared-memory tile

__device__ __forceinline__ void heap_sift_down(double *hd, int32_t *hi, int kk,
                                               int nn, int stride) {
  while (2 * kk <= nn) {
    int j = 2 * kk;
    if (j < nn && hd[j * stride] < hd[(j + 1) * stride]) ++j;
    const double a = hd[kk * stride], b = hd[j * stride];
    if (a == b || a > b) break;
    if (j == kk) break;  // only reachable with a NaN root
    hd[kk * stride] = b;
    hd[j * stride] = a;
    const int32_t ti = hi[kk * stride];
    hi[kk * stride] = hi[j * stride];
    hi[j * stride] = ti;
    kk = j;
  }
}

__device__ __forceinline__ void heap_heapify(double *hd, int32_t *hi, int k, int stride) {
  if (k <= 1) return;
  for (int s = k / 2 - 1; s >= 0; --s) heap_sift_down(hd, hi, s, k - 1, stride);
}

template <typename T>
__global__ void knn_fp64_kernel(const T *__restrict__ train, int64_t n, int d,
                                const T *__restrict__ queries, int64_t m, int k,
                                int64_t *__restrict__ idx_out,
                                double *__restrict__ dist_out) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int nt = blockDim.x;
  double *hd = reinterpret_cast<double *>(smraw);                // k x nt
  int32_t *hi = reinterpret_cast<int32_t *>(hd + (size_t)k * nt);  // k x nt
  T *qs = reinterpret_cast<T *>(hi + (size_t)k * nt + ((k * nt) & 1));  // d x nt
  T *ts = qs + (size_t)d * nt;                                   // kKnnTile x d
  const int tid = threadIdx.x;
  const int64_t q = (int64_t)blockIdx.x * nt + tid;
  const bool live = q < m;
  for (int j = 0; j < d; ++j) qs[j * nt + tid] = live ? queries[q * d + j] : T(0);
  for (int s = 0; s < k; ++s) {
    hd[s * nt + tid] = __longlong_as_double(0x7ff0000000000000ll);  // +inf
    hi[s * nt + tid] = -1;
  }
  double *mh = hd + tid;
  int32_t *mi = hi + tid;
  for (int64_t r0 = 0; r0 < n; r0 += kKnnTile) {
    const int rt = (int)min((int64_t)kKnnTile, n - r0);
    __syncthreads();
    for (int t = tid; t < rt * d; t += nt) ts[t] = train[r0 * d + t];
    __syncthreads();
    if (!live) continue;
    for (int r = 0; r < rt; ++r) {
      const T *tr = ts + r * d;
      double s = 0.0;
      for (int j = 0; j < d; ++j) s = __dadd_rn(s, sq_term(qs[j * nt + tid], tr[j]));
      const double dist = __dsqrt_rn(s);
      if (dist < mh[0]) {
        mh[0] = dist;
        mi[0] = (int32_t)(r0 + r);
        heap_heapify(mh, mi, k, nt);
      }
    }
  }
  if (!live) return;
  for (int s = 0; s < k; ++s) {
    idx_out[q * k + s] = mi[s * nt];
    dist_out[q * k + s] = mh[s * nt];
  }
}

sc_status launch_knn_fp64(int dtype, const void *train, int64_t n, int d,
                          const void *queries, int64_t m, int k, int64_t *idx,
                          double *dist, cudaStream_t s) {
  if (m == 0) return SC_OK;
  const int es = dtype == SC_F32 ? 4 : 8;
  int nt = 128;
  size_t smem = 0;
  for (; nt >= 32; nt >>= 1) {
    smem = (size_t)k * nt * 12 + 8 + (size_t)d * nt * es + (size_t)kKnnTile * d * es + 16;
    if (smem <= 200 * 1024) break;
  }
  if (nt < 32) {
    set_error("d=%d, k=%d exceed the FP64 kNN kernel's shared memory", d, k);
    return SC_ERR_INVALID;
  }
  const int grid = (int)((m + nt - 1) / nt);
  if (dtype == SC_F32) {
    auto kern = knn_fp64_kernel<float>;
    SC_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    kern<<<grid, nt, smem, s>>>((const float *)train, n, d, (const float *)queries, m, k, idx, dist);
  } else {
    auto kern = knn_fp64_kernel<double>;
    SC_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    kern<<<grid, nt, smem, s>>>((const double *)train, n, d, (const double *)queries, m, k, idx, dist);
  }
  SC_LAUNCHED();
  return SC_OK;
}

// ---------------------------------------------------------------------------
// LinearKNNSearch::find_radius (src/algorithm/neighbour/linear_search.rs:89-
// 108) in FP64, one query per thread: every training row i in index order
// with d = sqrt(D) <= radius.  Pass 1 (out == nullptr) counts per query; pass
// 2 writes each query's rows from offsets[q] on.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void knn_radius_fp64_kernel(const T *__restrict__ train, int64_t n, int d,
                                       const T *__restrict__ queries, int64_t m, double radius,
                                       int64_t *__restrict__ counts, const int64_t *__restrict__ offsets,
                                       int64_t *__restrict__ idx_out, double *__restrict__ dist_out) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int nt = blockDim.x;
  T *qs = reinterpret_cast<T *>(smraw);  // d x nt
  T *ts = qs + (size_t)d * nt;           // kKnnTile x d
  const int tid = threadIdx.x;
  const int64_t q = (int64_t)blockIdx.x * nt + tid;
  const bool live = q < m;
  for (int j = 0; j < d; ++j) qs[j * nt + tid] = live ? queries[q * d + j] : T(0);
  int64_t c = 0, pos = live && idx_out ? offsets[q] : 0;
  for (int64_t r0 = 0; r0 < n; r0 += kKnnTile) {
    const int rt = (int)min((int64_t)kKnnTile, n - r0);
    __syncthreads();
    for (int t = tid; t < rt * d; t += nt) ts[t] = train[r0 * d + t];
    __syncthreads();
    if (!live) continue;
    for (int r = 0; r < rt; ++r) {
      const T *tr = ts + r * d;
      double sq = 0.0;
      for (int j = 0; j < d; ++j) sq = __dadd_rn(sq, sq_term(qs[j * nt + tid], tr[j]));
      const double dist = __dsqrt_rn(sq);
      if (dist <= radius) {
        if (idx_out) {
          idx_out[pos] = r0 + r;
          dist_out[pos] = dist;
          ++pos;
        }
        ++c;
      }
    }
  }
  if (live && !idx_out) counts[q] = c;
}

sc_status launch_knn_radius_fp64(int dtype, const void *train, int64_t n, int d, const void *queries, int64_t m,
                                 double radius, int64_t *counts, const int64_t *offsets, int64_t *idx,
                                 double *dist, cudaStream_t s) {
  if (m == 0) return SC_OK;
  const int es = dtype == SC_F32 ? 4 : 8;
  int nt = 128;
  size_t smem = 0;
  for (; nt >= 32; nt >>= 1) {
    smem = (size_t)d * nt * es + (size_t)kKnnTile * d * es + 16;
    if (smem <= 200 * 1024) break;
  }
  if (nt < 32) {
    set_error("d=%d exceeds the FP64 radius kernel's shared memory", d);
    return SC_ERR_INVALID;
  }
  const int grid = (int)((m + nt - 1) / nt);
  if (dtype == SC_F32) {
    auto kern = knn_radius_fp64_kernel<float>;
    SC_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    kern<<<grid, nt, smem, s>>>((const float *)train, n, d, (const float *)queries, m, radius, counts, offsets,
                                idx, dist);
  } else {
    auto kern = knn_radius_fp64_kernel<double>;
    SC_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    kern<<<grid, nt, smem, s>>>((const double *)train, n, d, (const double *)queries, m, radius, counts, offsets,
                                idx, dist);
  }
  SC_LAUNCHED();
  return SC_OK;
}

// ---------------------------------------------------------------------------
// KNNWeightFunction::calc_weights (src/neighbors/mod.rs:62-78) and the
// classifier vote (src/neighbors/knn_classifier.rs:279-299): weights in heap
// order over the entries whose index is Some, w_sum summed in that order,
// c[y] += w / w_sum, argmax by strict > scanned in heap order.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int knn_weights(const int64_t *qi, const double *qd,
                                           int k, int weight, double *w,
                                           int *pos) {
  int c = 0;
  bool any_zero = false;
  for (int s = 0; s < k; ++s)
    if (qi[s] >= 0) {
      pos[c++] = s;
      any_zero |= qd[s] == 0.0;
    }
  for (int t = 0; t < c; ++t) {
    const double e = qd[pos[t]];
    w[t] = weight == SC_KNN_UNIFORM ? 1.0 : (any_zero ? (e == 0.0 ? 1.0 : 0.0) : __ddiv_rn(1.0, e));
  }
  return c;
}

__global__ void knn_vote_kernel(const int64_t *__restrict__ idx,
                                const double *__restrict__ dist, int64_t m,
                                int k, int weight,
                                const int64_t *__restrict__ y_class,
                                int64_t *__restrict__ out) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= m) return;
  double w[kMaxKnnK], cv[kMaxKnnK];
  int pos[kMaxKnnK];
  int64_t cls[kMaxKnnK];
  const int c = knn_weights(idx + q * k, dist + q * k, k, weight, w, pos);
  double w_sum = 0.0;
  for (int t = 0; t < c; ++t) w_sum = __dadd_rn(w_sum, w[t]);
  int ncls = 0;
  double max_c = 0.0;
  int64_t max_i = 0;
  for (int t = 0; t < c; ++t) {
    const int64_t y = y_class[idx[q * k + pos[t]]];
    int slot = 0;
    while (slot < ncls && cls[slot] != y) ++slot;
    if (slot == ncls) { cls[ncls] = y; cv[ncls] = 0.0; ++ncls; }
    cv[slot] = __dadd_rn(cv[slot], __ddiv_rn(w[t], w_sum));
    if (cv[slot] > max_c) { max_c = cv[slot]; max_i = y; }
  }
  out[q] = max_i;
}

// KNNRegressor::predict_for_row (src/neighbors/knn_regressor.rs:268-282).
__global__ void knn_regress_kernel(const int64_t *__restrict__ idx,
                                   const double *__restrict__ dist, int64_t m,
                                   int k, int weight,
                                   const double *__restrict__ y,
                                   double *__restrict__ out) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= m) return;
  double w[kMaxKnnK];
  int pos[kMaxKnnK];
  const int c = knn_weights(idx + q * k, dist + q * k, k, weight, w, pos);
  double w_sum = 0.0;
  for (int t = 0; t < c; ++t) w_sum = __dadd_rn(w_sum, w[t]);
  double r = 0.0;
  for (int t = 0; t < c; ++t)
    r = __dadd_rn(r, __dmul_rn(y[idx[q * k + pos[t]]], __ddiv_rn(w[t], w_sum)));
  out[q] = r;
}

sc_status launch_knn_vote(const int64_t *idx, const double *dist, int64_t m,
                          int k, int weight, const int64_t *y_class,
                          int64_t *out, cudaStream_t s) {
  if (m == 0) return SC_OK;
  knn_vote_kernel<<<(unsigned)((m + 127) / 128), 128, 0, s>>>(idx, dist, m, k, weight, y_class, out);
  SC_LAUNCHED();
  return SC_OK;
}

sc_status launch_knn_regress(const int64_t *idx, const double *dist,
                             int64_t m, int k, int weight, const double *y,
                             double *out, cudaStream_t s) {
  if (m == 0) return SC_OK;
  knn_regress_kernel<<<(unsigned)((m + 127) / 128), 128, 0, s>>>(idx, dist, m, k, weight, y, out);
  SC_LAUNCHED();
  return SC_OK;
}

}  // namespace sc
