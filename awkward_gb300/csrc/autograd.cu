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
// Layout: a CTA owns a tile of kTileLists consecutive lists.  It stages the
// tile's offsets in shared memory, computes per-list statistics (max, sums)
// with one thread per list where a pass needs them, and then visits the
// tile's elements in order -- consecutive threads on consecutive elements,
// each finding its list by a short forward walk over the staged offsets -- so
// every element-sized read and write is coalesced.
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

struct TileLists {
  long long loc[kTileLists + 1];  // offsets of the tile's lists, relative to its first element
  long long base;                 // first element of the tile
  int count;                      // lists in this tile
};

// Stage offsets[l0 .. l0+count] (all threads; ends with __syncthreads).
__device__ __forceinline__ void stage_tile(TileLists& t, const int64_t* __restrict__ offsets,
                                           long long l0, long long nlists) {
  const long long rem = nlists - l0;
  const int count = (int)(rem < kTileLists ? rem : kTileLists);
  const long long base = __ldg(offsets + l0);
  for (int i = threadIdx.x; i <= kTileLists; i += blockDim.x) {
    const int k = i < count ? i : count;
    t.loc[i] = __ldg(offsets + l0 + k) - base;
  }
  if (threadIdx.x == 0) {
    t.base = base;
    t.count = count;
  }
  __syncthreads();
}

// Visit every element of the tile in order: fn(element index, local list).
// Each warp takes a contiguous share, 32 consecutive elements per step.
template <class F>
__device__ __forceinline__ void for_tile_elements(const TileLists& t, F fn) {
  constexpr int kWarps = kTileBlock / 32;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long total = t.loc[t.count];
  const long long qa = total * warp / kWarps, qb = total * (warp + 1) / kWarps;
  if (qa >= qb) return;
  int lo = 0, hi = t.count;  // last r with loc[r] <= qa
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (t.loc[mid] <= qa) lo = mid;
    else hi = mid;
  }
  int r = lo;
  for (long long g = qa; g < qb; g += 32) {
    while (t.loc[r + 1] <= g) r++;
    const long long q = g + lane;
    if (q >= qb) continue;
    int rl = r;
    while (t.loc[rl + 1] <= q) rl++;
    fn(t.base + q, rl);
  }
}

// ---------------------------------------------------------------- sum backward
template <class T>
__global__ void __launch_bounds__(kTileBlock)
    sum_backward_kernel(T* __restrict__ gx, const T* __restrict__ gout,
                        const int64_t* __restrict__ offsets, long long nlists) {
  __shared__ TileLists t;
  const long long l0 = (long long)blockIdx.x * kTileLists;
  stage_tile(t, offsets, l0, nlists);
  for_tile_elements(t, [&](long long j, int r) { gx[j] = __ldg(gout + l0 + r); });
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
// Per-list max and sum of exp(x - max) by one thread per list.
template <class T>
__device__ __forceinline__ void list_stats(const T* __restrict__ x, const TileLists& t,
                                           T* s_max, T* s_sum) {
  for (int r = threadIdx.x; r < t.count; r += blockDim.x) {
    const T* p = x + t.base + t.loc[r];
    const long long n = t.loc[r + 1] - t.loc[r];
    T m = -INFINITY;
    for (long long i = 0; i < n; i++) m = max_t(m, p[i]);
    T s = 0;
    for (long long i = 0; i < n; i++) s += exp_t(p[i] - m);
    s_max[r] = m;
    s_sum[r] = s;
  }
}

template <class T>
__global__ void __launch_bounds__(kTileBlock)
    softmax_forward_kernel(T* __restrict__ y, const T* __restrict__ x,
                           const int64_t* __restrict__ offsets, long long nlists) {
  __shared__ TileLists t;
  __shared__ T s_max[kTileLists];
  __shared__ T s_sum[kTileLists];
  const long long l0 = (long long)blockIdx.x * kTileLists;
  stage_tile(t, offsets, l0, nlists);
  list_stats(x, t, s_max, s_sum);
  __syncthreads();
  for_tile_elements(t, [&](long long j, int r) { y[j] = exp_t(x[j] - s_max[r]) / s_sum[r]; });
}

// d x_j = y_j (g_j - sum_k g_k y_k); y from `ysaved` when given, else
// recomputed from x (max and normaliser recomputed per list).
template <class T>
__global__ void __launch_bounds__(kTileBlock)
    softmax_backward_kernel(T* __restrict__ gx, const T* __restrict__ gy,
                            const T* __restrict__ x, const T* __restrict__ ysaved,
                            const int64_t* __restrict__ offsets, long long nlists) {
  __shared__ TileLists t;
  __shared__ T s_max[kTileLists];
  __shared__ T s_sum[kTileLists];
  __shared__ T s_dot[kTileLists];
  const long long l0 = (long long)blockIdx.x * kTileLists;
  stage_tile(t, offsets, l0, nlists);
  if (ysaved) {
    for (int r = threadIdx.x; r < t.count; r += blockDim.x) {
      const long long a = t.base + t.loc[r], b = t.base + t.loc[r + 1];
      T d = 0;
      for (long long j = a; j < b; j++) d += gy[j] * ysaved[j];
      s_dot[r] = d;
    }
    __syncthreads();
    for_tile_elements(t, [&](long long j, int r) { gx[j] = ysaved[j] * (gy[j] - s_dot[r]); });
    return;
  }
  for (int r = threadIdx.x; r < t.count; r += blockDim.x) {
    const long long a = t.base + t.loc[r], b = t.base + t.loc[r + 1];
    T m = -INFINITY;
    for (long long j = a; j < b; j++) m = max_t(m, x[j]);
    T s = 0, gs = 0;
    for (long long j = a; j < b; j++) {
      const T e = exp_t(x[j] - m);
      s += e;
      gs += gy[j] * e;
    }
    s_max[r] = m;
    s_sum[r] = s;
    s_dot[r] = gs / s;
  }
  __syncthreads();
  for_tile_elements(t, [&](long long j, int r) {
    const T yj = exp_t(x[j] - s_max[r]) / s_sum[r];
    gx[j] = yj * (gy[j] - s_dot[r]);
  });
}

inline unsigned tiles_of(long long nlists) { return (unsigned)tile_count(nlists); }

}  // namespace

// ================================================================== entry points
#define GB_AUTOGRAD(SUFFIX, T)                                                                  \
  GB_EXPORT int awkward_gb300_segment_sum_backward_##SUFFIX(                                    \
      T* grad_x, const T* grad_out, const int64_t* offsets, int64_t nlists, void* stream) {    \
    if (nlists <= 0) return 0;                                                                  \
    sum_backward_kernel<T><<<tiles_of(nlists), kTileBlock, 0, (cudaStream_t)stream>>>(         \
        grad_x, grad_out, offsets, nlists);                                                     \
    return (int)cudaGetLastError();                                                             \
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
      T* y, const T* x, const int64_t* offsets, int64_t nlists, void* stream) {                \
    if (nlists <= 0) return 0;                                                                  \
    softmax_forward_kernel<T><<<tiles_of(nlists), kTileBlock, 0, (cudaStream_t)stream>>>(      \
        y, x, offsets, nlists);                                                                 \
    return (int)cudaGetLastError();                                                             \
  }                                                                                             \
  GB_EXPORT int awkward_gb300_jagged_softmax_backward_##SUFFIX(                                 \
      T* grad_x, const T* grad_y, const T* x, const T* y_saved, const int64_t* offsets,        \
      int64_t nlists, void* stream) {                                                           \
    if (nlists <= 0) return 0;                                                                  \
    softmax_backward_kernel<T><<<tiles_of(nlists), kTileBlock, 0, (cudaStream_t)stream>>>(     \
        grad_x, grad_y, x, y_saved, offsets, nlists);                                           \
    return (int)cudaGetLastError();                                                             \
  }

GB_AUTOGRAD(float32, float)
GB_AUTOGRAD(float64, double)
