// autograd.cu -- backward kernels for differentiable jagged operations.
//
// awkward has no CUDA backward kernels (its differentiation goes through JAX,
// src/awkward/_connect/jax/reducers.py:51-200); these entry points back the
// torch.autograd.Function classes of awkward_gb300/autograd.py:
//   segmented sum      d x_j = g_{list(j)}                      (broadcast by offsets)
//   segmented max      d x_{argmax(l)} = g_l, 0 elsewhere        (argmax-routed scatter)
//   jagged softmax     y_j = exp(x_j - m_l) / sum_k exp(x_k - m_l)
//                      d x_j = y_j (g_j - sum_k g_k y_k)         (fused Jacobian product)
// The forward sum and max use the segmented reducers of this library.
//
// Layout: a CTA owns a tile of kSoftLists consecutive lists, one statistics
// thread per list, and twice as many threads for the memory passes.  It stages
// the tile's offsets and, when the tile's elements fit
// (kSoftBytes per array), the element arrays it reads more than once in
// shared memory by asynchronous copies (cp.async, issued from the tile's two
// end offsets so they are in flight with the offsets loads), plus an
// element -> list map (one byte per element).  Per-list statistics (max, sums) are computed by one thread
// per list in element order, from shared memory; then the tile's elements are
// visited with consecutive threads on consecutive elements, so every global
// read and write is coalesced.  A tile whose elements do not fit reads them
// from global memory and finds each element's list by binary search.
#include <math.h>

#include "list_tile.cuh"

using namespace gb;

namespace {

template <class T>
__device__ __forceinline__ T exp_t(T v);
template <>
__device__ __forceinline__ float exp_t<float>(float v) { return __expf(v); }
template <>
__device__ __forceinline__ double exp_t<double>(double v) { return exp(v); }

template <class T>
__device__ __forceinline__ T max_t(T a, T b) { return a > b ? a : b; }

constexpr int kSoftLists = 64;        // lists per CTA (one statistics thread each)
constexpr int kSoftThreads = 128;     // threads per CTA (staging and element passes)
constexpr int kSoftBytes = 8192;      // staging per element array
constexpr int kSoftElems = 2048;      // element -> list map entries (>= kSoftBytes / 4)

struct SoftTile {
  long long loc[kSoftLists + 1];  // offsets of the tile's lists, relative to its first element
  unsigned char owner[kSoftElems];
  long long base;                 // first element of the tile
  int count;                      // lists in this tile
  int mapped;                     // owner[] holds every element's list
};

// One element global -> shared memory without a register round trip
// (cp.async, completed by cp_async_wait_all).
template <class T>
__device__ __forceinline__ void cp_async_elem(T* dst, const T* src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], %2;" ::"r"(d), "l"(src), "n"(sizeof(T))
               : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_all;" ::: "memory");
}

// Stage a tile: offsets[l0 .. l0+count] and, if the tile has at most `cap`
// elements, its elements of src0 (and src1 when given) into dst0 (dst1) and
// the element -> list map (all threads; ends with __syncthreads).  The
// element copies are issued first, from the tile's two end offsets alone, so
// they are in flight together with the offsets loads.
template <class T>
__device__ __forceinline__ void stage_soft_tile(SoftTile& t, const int64_t* __restrict__ offsets,
                                                long long l0, long long nlists, int cap,
                                                T* dst0, const T* __restrict__ src0, T* dst1,
                                                const T* __restrict__ src1) {
  const long long rem = nlists - l0;
  const int count = (int)(rem < kSoftLists ? rem : kSoftLists);
  const long long base = __ldg(offsets + l0);
  const long long total = __ldg(offsets + l0 + count) - base;
  const bool mapped = total <= cap;
  if (mapped) {
    for (long long q = threadIdx.x; q < total; q += blockDim.x) {
      cp_async_elem(dst0 + q, src0 + base + q);
      if (src1) cp_async_elem(dst1 + q, src1 + base + q);
    }
  }
  for (int i = threadIdx.x; i <= kSoftLists; i += blockDim.x) {
    const int k = i < count ? i : count;
    t.loc[i] = __ldg(offsets + l0 + k) - base;
  }
  if (threadIdx.x == 0) {
    t.base = base;
    t.count = count;
    t.mapped = mapped ? 1 : 0;
  }
  __syncthreads();
  if (mapped && (int)threadIdx.x < count) {
    const int a = (int)t.loc[threadIdx.x], b = (int)t.loc[threadIdx.x + 1];
    for (int q = a; q < b; q++) t.owner[q] = (unsigned char)threadIdx.x;
  }
  cp_async_wait_all();
  __syncthreads();
}

// List of tile element q: the map, or the last r with loc[r] <= q.
__device__ __forceinline__ int soft_list(const SoftTile& t, long long q) {
  if (t.mapped) return t.owner[q];
  int lo = 0, hi = t.count;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (t.loc[mid] <= q) lo = mid;
    else hi = mid;
  }
  return lo;
}

inline unsigned soft_tiles(long long nlists) {
  return (unsigned)((nlists + kSoftLists - 1) / kSoftLists);
}

// ---------------------------------------------------------------- sum backward
// Warp rounds of 32 lists (one lane per list, list ends loaded coalesced,
// starts from the lane below): each lane writes its list's gradient value
// over its elements in a per-warp stage in shared memory, then the warp copies
// the round's span out with consecutive lanes on consecutive elements
// (coalesced stores).  A round whose span exceeds the stage (long lists)
// writes straight from its lanes.  No block barriers: warps run independently.
constexpr int kBcastStage = 1024;  // elements staged per warp and round

template <class T>
__global__ void __launch_bounds__(256)
    sum_backward_rounds_kernel(T* __restrict__ gx, const T* __restrict__ gout,
                               const int64_t* __restrict__ offsets, long long nlists) {
  __shared__ T stage[256 / 32][kBcastStage];
  T* sw = stage[threadIdx.x >> 5];
  const int lane = threadIdx.x & 31;
  const long long nrounds = (nlists + 31) / 32;
  const long long stride = (long long)gridDim.x * (blockDim.x >> 5);
  for (long long r = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5; r < nrounds;
       r += stride) {
    const long long base = r * 32, li = base + lane;
    const bool act = li < nlists;
    const long long en = __ldg(offsets + (act ? li : nlists - 1) + 1);
    long long st = __shfl_up_sync(0xffffffffu, en, 1);
    if (lane == 0) st = __ldg(offsets + base);
    const unsigned acts = __ballot_sync(0xffffffffu, act);
    const long long lo = __shfl_sync(0xffffffffu, st, 0);
    const long long hi = __shfl_sync(0xffffffffu, en, 31 - __clz(acts));
    const T g = act ? __ldg(gout + li) : T(0);
    const bool sorted = __all_sync(0xffffffffu, !act || st <= en);
    if (sorted && hi - lo <= kBcastStage) {
      if (act)
        for (long long j = st; j < en; j++) sw[j - lo] = g;
      __syncwarp();
      const int span = (int)(hi - lo);
      for (int j = lane; j < span; j += 32) gx[lo + j] = sw[j];
      __syncwarp();
    } else if (act) {
      for (long long j = st; j < en; j++) gx[j] = g;
    }
  }
}

// ---------------------------------------------------------------- max backward
// argmax holds global element indices (-1 for an empty list); indices outside
// [0, nelements) are ignored.
template <class T>
__global__ void max_backward_kernel(T* __restrict__ gx, const T* __restrict__ gout,
                                    const int64_t* __restrict__ argmax, long long nelements,
                                    long long nlists) {
  for (long long l = blockIdx.x * (long long)blockDim.x + threadIdx.x; l < nlists;
       l += (long long)gridDim.x * blockDim.x) {
    const long long j = argmax[l];
    if (j >= 0 && j < nelements) gx[j] = gout[l];
  }
}

// ---------------------------------------------------------------- softmax
template <class T>
__global__ void __launch_bounds__(kSoftThreads)
    softmax_forward_kernel(T* __restrict__ y, const T* __restrict__ x,
                           const int64_t* __restrict__ offsets, long long nlists) {
  constexpr int cap = kSoftBytes / (int)sizeof(T);
  __shared__ SoftTile t;
  __shared__ T sx[cap];
  __shared__ T s_max[kSoftLists];
  __shared__ T s_sum[kSoftLists];
  const long long l0 = (long long)blockIdx.x * kSoftLists;
  stage_soft_tile(t, offsets, l0, nlists, cap, sx, x, (T*)nullptr, (const T*)nullptr);
  const long long total = t.loc[t.count];
  const T* xs = t.mapped ? sx : x + t.base;
  const int r = threadIdx.x;
  if (r < t.count) {  // per-list max and sum of exp(x - max)
    const long long a = t.loc[r], b = t.loc[r + 1];
    T m = -INFINITY;
    for (long long q = a; q < b; q++) m = max_t(m, xs[q]);
    T sum = 0;
    for (long long q = a; q < b; q++) sum += exp_t(xs[q] - m);
    s_max[r] = m;
    s_sum[r] = T(1) / sum;  // one division per list; elements multiply by it
  }
  __syncthreads();
  for (long long q = threadIdx.x; q < total; q += blockDim.x) {
    const int l = soft_list(t, q);
    y[t.base + q] = exp_t(xs[q] - s_max[l]) * s_sum[l];
  }
}

// d x_j = y_j (g_j - sum_k g_k y_k); y from `ysaved` when given, else
// recomputed from x (max and normaliser recomputed per list).
template <class T>
__global__ void __launch_bounds__(kSoftThreads)
    softmax_backward_kernel(T* __restrict__ gx, const T* __restrict__ gy,
                            const T* __restrict__ x, const T* __restrict__ ysaved,
                            const int64_t* __restrict__ offsets, long long nlists) {
  constexpr int cap = kSoftBytes / (int)sizeof(T);
  __shared__ SoftTile t;
  __shared__ T sa[cap];  // x, or the saved y
  __shared__ T sg[cap];  // gy
  __shared__ T s_max[kSoftLists];
  __shared__ T s_sum[kSoftLists];
  __shared__ T s_dot[kSoftLists];
  const long long l0 = (long long)blockIdx.x * kSoftLists;
  const T* src = ysaved ? ysaved : x;
  stage_soft_tile(t, offsets, l0, nlists, cap, sa, src, sg, gy);
  const long long total = t.loc[t.count];
  const T* as = t.mapped ? sa : src + t.base;
  const T* gs = t.mapped ? sg : gy + t.base;
  const int r = threadIdx.x;
  if (ysaved) {
    if (r < t.count) {
      const long long a = t.loc[r], b = t.loc[r + 1];
      T d = 0;
      for (long long q = a; q < b; q++) d += gs[q] * as[q];
      s_dot[r] = d;
    }
    __syncthreads();
    for (long long q = threadIdx.x; q < total; q += blockDim.x) {
      const int l = soft_list(t, q);
      gx[t.base + q] = as[q] * (gs[q] - s_dot[l]);
    }
    return;
  }
  if (r < t.count) {
    const long long a = t.loc[r], b = t.loc[r + 1];
    T m = -INFINITY;
    for (long long q = a; q < b; q++) m = max_t(m, as[q]);
    T sum = 0, gsum = 0;
    for (long long q = a; q < b; q++) {
      const T e = exp_t(as[q] - m);
      sum += e;
      gsum += gs[q] * e;
    }
    s_max[r] = m;
    const T inv = T(1) / sum;  // one division per list; elements multiply by it
    s_sum[r] = inv;
    s_dot[r] = gsum * inv;
  }
  __syncthreads();
  for (long long q = threadIdx.x; q < total; q += blockDim.x) {
    const int l = soft_list(t, q);
    const T yj = exp_t(as[q] - s_max[l]) * s_sum[l];
    gx[t.base + q] = yj * (gs[q] - s_dot[l]);
  }
}

// Zero a[j] for j outside [offsets[0], offsets[nlists]) within [0, nvalues):
// the elements no list covers, which the kernels above never write.  Only
// those elements are touched (none when the offsets span the whole array),
// so the callers need not clear the whole output first.
template <class T>
__global__ void zero_outside_kernel(T* __restrict__ a, const int64_t* __restrict__ offsets,
                                    long long nlists, long long nvalues) {
  long long lo = __ldg(offsets), hi = __ldg(offsets + nlists);
  lo = lo < 0 ? 0 : (lo > nvalues ? nvalues : lo);
  hi = hi < lo ? lo : (hi > nvalues ? nvalues : hi);
  const long long stride = (long long)gridDim.x * blockDim.x;
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  for (long long j = t; j < lo; j += stride) a[j] = T(0);
  for (long long j = hi + t; j < nvalues; j += stride) a[j] = T(0);
}

template <class T>
cudaError_t zero_outside(T* a, const int64_t* offsets, long long nlists, long long nvalues,
                         cudaStream_t s) {
  if (nvalues <= 0) return cudaSuccess;
  zero_outside_kernel<T><<<device_sm_count() * 4, 256, 0, s>>>(a, offsets, nlists, nvalues);
  return cudaGetLastError();
}

}  // namespace

// ================================================================== entry points
#define GB_AUTOGRAD(SUFFIX, T)                                                                  \
  GB_EXPORT int awkward_gb300_segment_sum_backward_##SUFFIX(                                    \
      T* grad_x, const T* grad_out, const int64_t* offsets, int64_t nlists, int64_t nvalues,   \
      void* stream) {                                                                           \
    cudaStream_t s = (cudaStream_t)stream;                                                      \
    if (nlists <= 0) return (int)(nvalues > 0 ? cudaMemsetAsync(grad_x, 0, sizeof(T) * (size_t)nvalues, s) : cudaSuccess); \
    sum_backward_rounds_kernel<T><<<device_sm_count() * 8, 256, 0, s>>>(grad_x, grad_out,    \
                                                                       offsets, nlists);        \
    cudaError_t e = cudaGetLastError();                                                         \
    return (int)(e != cudaSuccess ? e : zero_outside(grad_x, offsets, nlists, nvalues, s));     \
  }                                                                                             \
  GB_EXPORT int awkward_gb300_segment_max_backward_##SUFFIX(                                    \
      T* grad_x, const T* grad_out, const int64_t* argmax, int64_t nelements, int64_t nlists,  \
      void* stream) {                                                                           \
    cudaStream_t s = (cudaStream_t)stream;                                                      \
    if (nelements > 0) {                                                                        \
      cudaError_t e = cudaMemsetAsync(grad_x, 0, sizeof(T) * (size_t)nelements, s);             \
      if (e != cudaSuccess) return (int)e;                                                      \
    }                                                                                           \
    if (nlists <= 0) return 0;                                                                  \
    long long g = (nlists + 255) / 256;                                                         \
    const long long cap = (long long)device_sm_count() * 16;                                    \
    max_backward_kernel<T><<<(unsigned)(g < cap ? g : cap), 256, 0, s>>>(                      \
        grad_x, grad_out, argmax, nelements, nlists);                                           \
    return (int)cudaGetLastError();                                                             \
  }                                                                                             \
  GB_EXPORT int awkward_gb300_jagged_softmax_forward_##SUFFIX(                                  \
      T* y, const T* x, const int64_t* offsets, int64_t nlists, int64_t nvalues, void* stream) { \
    cudaStream_t s = (cudaStream_t)stream;                                                      \
    if (nlists <= 0) return (int)(nvalues > 0 ? cudaMemsetAsync(y, 0, sizeof(T) * (size_t)nvalues, s) : cudaSuccess); \
    softmax_forward_kernel<T><<<soft_tiles(nlists), kSoftThreads, 0, s>>>(y, x, offsets, nlists); \
    cudaError_t e = cudaGetLastError();                                                         \
    return (int)(e != cudaSuccess ? e : zero_outside(y, offsets, nlists, nvalues, s));          \
  }                                                                                             \
  GB_EXPORT int awkward_gb300_jagged_softmax_backward_##SUFFIX(                                 \
      T* grad_x, const T* grad_y, const T* x, const T* y_saved, const int64_t* offsets,        \
      int64_t nlists, int64_t nvalues, void* stream) {                                          \
    cudaStream_t s = (cudaStream_t)stream;                                                      \
    if (nlists <= 0) return (int)(nvalues > 0 ? cudaMemsetAsync(grad_x, 0, sizeof(T) * (size_t)nvalues, s) : cudaSuccess); \
    softmax_backward_kernel<T><<<soft_tiles(nlists), kSoftThreads, 0, s>>>(                    \
        grad_x, grad_y, x, y_saved, offsets, nlists);                                           \
    cudaError_t e = cudaGetLastError();                                                         \
    return (int)(e != cudaSuccess ? e : zero_outside(grad_x, offsets, nlists, nvalues, s));     \
  }

GB_AUTOGRAD(float32, float)
GB_AUTOGRAD(float64, double)
