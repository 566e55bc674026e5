// sort.cu -- segmented sort and argsort.
//
//   awkward_argsort  awkward_argsort.cpp:62-108
//   awkward_sort     awkward_sort.cpp:62-117
//
// Every element becomes a 64-bit order key whose ascending order is the
// requested order (descending keys are complemented), with awkward's
// comparator rules: integers and bool compare directly; floating point puts
// NaN before every number in both directions, and -0.0 equals +0.0.  Pairs
// (key, global index) are sorted ascending -- the index breaks ties, so the
// result is the stable order (std::stable_sort's; it is also a valid answer
// when `stable` is false).  Segments by length:
//   <= 32        one warp, bitonic network across the lanes (registers);
//   <= 2048      one CTA, bitonic network in shared memory;
//   longer       runs of 2048 sorted in shared memory, then merged pass by
//                pass (one CTA per segment, merge-path split per thread)
//                between two index buffers from the library's pool.
// The long segments are listed on the device; their count and total size are
// read back once to size the buffers (only when there are any).
#include <limits.h>

#include <type_traits>

#include "gb_common.cuh"

using namespace gb;

namespace {

constexpr int kSortBlock = 256;
constexpr int kSortTile = 2048;  // elements sorted in shared memory by one CTA
constexpr unsigned long long kPadKey = ~0ull;
constexpr long long kPadIdx = LLONG_MAX;

template <class T>
__device__ __forceinline__ unsigned long long sort_key(T v, bool asc) {
  unsigned long long k;
  if constexpr (std::is_floating_point<T>::value) {
    const double d = (double)v;
    if (d != d) return 0ull;  // NaN: first in both directions
    long long b = __double_as_longlong(d);
    if ((b << 1) == 0) b = 0;  // -0.0 == +0.0
    k = b >= 0 ? ((unsigned long long)b | 0x8000000000000000ull) : ~(unsigned long long)b;
  } else if constexpr (std::is_signed<T>::value) {
    k = (unsigned long long)(long long)v ^ 0x8000000000000000ull;
  } else {
    k = (unsigned long long)v;
  }
  return asc ? k : ~k;
}

__device__ __forceinline__ bool pair_less(unsigned long long ka, long long ia, unsigned long long kb,
                                          long long ib) {
  return ka < kb || (ka == kb && ia < ib);
}

// Bitonic sort of one (key, index) per lane across the warp, ascending.
__device__ __forceinline__ void warp_bitonic(unsigned long long& key, long long& idx) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int k = 2; k <= 32; k <<= 1) {
#pragma unroll
    for (int j = k >> 1; j > 0; j >>= 1) {
      const unsigned long long ok = __shfl_xor_sync(0xffffffffu, key, j);
      const long long oi = __shfl_xor_sync(0xffffffffu, idx, j);
      const bool up = (lane & k) == 0;
      const bool lower = (lane & j) == 0;
      const bool partner_less = pair_less(ok, oi, key, idx);
      const bool take = (lower == up) ? partner_less : !partner_less && (ok != key || oi != idx);
      if (take) {
        key = ok;
        idx = oi;
      }
    }
  }
}

// Bitonic sort of P (power of two, <= kSortTile) pairs in shared memory.
__device__ __forceinline__ void block_bitonic(unsigned long long* key, long long* idx, int P) {
  for (int k = 2; k <= P; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = threadIdx.x; i < P; i += blockDim.x) {
        const int p = i ^ j;
        if (p > i) {
          const bool up = (i & k) == 0;
          const bool swap = up ? pair_less(key[p], idx[p], key[i], idx[i])
                               : pair_less(key[i], idx[i], key[p], idx[p]);
          if (swap) {
            const unsigned long long tk = key[i];
            key[i] = key[p];
            key[p] = tk;
            const long long ti = idx[i];
            idx[i] = idx[p];
            idx[p] = ti;
          }
        }
      }
      __syncthreads();
    }
  }
}

// Segment bounds clamped to [0, length] (the CPU clamps against `length`;
// a negative offset, undefined there, stays inside the buffers here).
template <class U>
__device__ __forceinline__ void seg_bounds(const U* offsets, long long i, long long length,
                                           long long* st, long long* sp) {
  long long a = (long long)offsets[i], b = (long long)offsets[i + 1];
  if (a > length) a = length;
  if (b > length) b = length;
  if (a < 0) a = 0;
  if (b < 0) b = 0;
  *st = a;
  *sp = b;
}

// Deliver the sorted global index `j` of position p of segment [st, ...);
// sort writes only the first `limit` = min(offsets[last], length) values.
template <class T, bool ARG>
__device__ __forceinline__ void emit(void* out, const T* x, long long p, long long st,
                                     long long j, long long limit) {
  if (ARG) static_cast<int64_t*>(out)[p] = j - st;
  else if (p < limit) static_cast<T*>(out)[p] = x[j];
}

// Positions outside every segment: argsort keeps the iota, sort copies through.
template <class T, bool ARG>
__global__ void sort_init_kernel(void* out, const T* __restrict__ x, long long length,
                                 long long limit) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < length;
       i += (long long)gridDim.x * blockDim.x) {
    if (ARG) static_cast<int64_t*>(out)[i] = i;
    else if (i < limit) static_cast<T*>(out)[i] = x[i];
  }
}

template <class T, class U, bool ARG>
__global__ void __launch_bounds__(kSortBlock)
    sort_small_kernel(void* out, const T* __restrict__ x, long long length,
                      const U* __restrict__ offsets, long long nseg, long long limit, bool asc) {
  const long long w = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  const int lane = threadIdx.x & 31;
  for (long long s = w; s < nseg; s += nw) {
    long long st, sp;
    seg_bounds(offsets, s, length, &st, &sp);
    const long long L = sp - st;
    if (L < 1 || L > 32) continue;  // warp-uniform (one element still becomes local 0)
    unsigned long long key = kPadKey;
    long long idx = kPadIdx;
    if (lane < L) {
      idx = st + lane;
      key = sort_key(x[idx], asc);
    }
    warp_bitonic(key, idx);
    if (lane < L) emit<T, ARG>(out, x, st + lane, st, idx, limit);
  }
}

template <class T, class U, bool ARG>
__global__ void __launch_bounds__(kSortBlock)
    sort_medium_kernel(void* out, const T* __restrict__ x, long long length,
                       const U* __restrict__ offsets, long long nseg, long long limit, bool asc) {
  __shared__ unsigned long long s_key[kSortTile];
  __shared__ long long s_idx[kSortTile];
  for (long long s = blockIdx.x; s < nseg; s += gridDim.x) {
    long long st, sp;
    seg_bounds(offsets, s, length, &st, &sp);
    const long long L = sp - st;
    if (L <= 32 || L > kSortTile) continue;  // block-uniform
    int P = 64;
    while (P < L) P <<= 1;
    for (int i = threadIdx.x; i < P; i += blockDim.x) {
      if (i < L) {
        s_key[i] = sort_key(x[st + i], asc);
        s_idx[i] = st + i;
      } else {
        s_key[i] = kPadKey;
        s_idx[i] = kPadIdx;
      }
    }
    __syncthreads();
    block_bitonic(s_key, s_idx, P);
    for (int i = threadIdx.x; i < L; i += blockDim.x) emit<T, ARG>(out, x, st + i, st, s_idx[i], limit);
    __syncthreads();
  }
}

// List the segments longer than kSortTile: ids[k], the slot bases[k] of
// its index runs in the merge buffers, and (counters) their count and total.
template <class U>
__global__ void sort_classify_kernel(const U* __restrict__ offsets, long long nseg,
                                     long long length, long long* __restrict__ ids,
                                     long long* __restrict__ bases,
                                     unsigned long long* counters) {
  for (long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x; s < nseg;
       s += (long long)gridDim.x * blockDim.x) {
    long long st, sp;
    seg_bounds(offsets, s, length, &st, &sp);
    if (sp - st > kSortTile) {
      const unsigned long long k = atomicAdd(counters, 1ull);
      ids[k] = s;
      bases[k] = (long long)atomicAdd(counters + 1, (unsigned long long)(sp - st));
    }
  }
}

// Key of the element an index buffer holds at position p.
template <class T>
__device__ __forceinline__ unsigned long long key_at(const T* x, const long long* buf, long long p,
                                                     bool asc) {
  return sort_key(x[buf[p]], asc);
}

// One CTA per long segment: runs of kSortTile sorted in shared memory into
// `a` (positions relative to the segment's slot `base` in the buffers), then
// pairs of runs merged between `a` and `b` until one run remains.
template <class T, class U, bool ARG>
__global__ void __launch_bounds__(kSortBlock)
    sort_long_kernel(void* out, const T* __restrict__ x, long long length,
                     const U* __restrict__ offsets, const long long* __restrict__ ids,
                     const long long* __restrict__ bases, long long* __restrict__ a,
                     long long* __restrict__ b, long long limit, bool asc) {
  __shared__ unsigned long long s_key[kSortTile];
  __shared__ long long s_idx[kSortTile];
  const long long s = ids[blockIdx.x];
  long long st, sp;
  seg_bounds(offsets, s, length, &st, &sp);
  const long long L = sp - st;
  long long* src = a + bases[blockIdx.x];
  long long* dst = b + bases[blockIdx.x];
  for (long long r0 = 0; r0 < L; r0 += kSortTile) {
    const int n = (int)(L - r0 < kSortTile ? L - r0 : kSortTile);
    for (int i = threadIdx.x; i < kSortTile; i += blockDim.x) {
      if (i < n) {
        s_key[i] = sort_key(x[st + r0 + i], asc);
        s_idx[i] = st + r0 + i;
      } else {
        s_key[i] = kPadKey;
        s_idx[i] = kPadIdx;
      }
    }
    __syncthreads();
    block_bitonic(s_key, s_idx, kSortTile);
    for (int i = threadIdx.x; i < n; i += blockDim.x) src[r0 + i] = s_idx[i];
    __syncthreads();
  }
  constexpr int kPer = 8;  // outputs merged by one thread per step
  for (long long w = kSortTile; w < L; w <<= 1) {
    for (long long lo = 0; lo < L; lo += 2 * w) {
      const long long mid = lo + w < L ? lo + w : L, hi = lo + 2 * w < L ? lo + 2 * w : L;
      const long long na = mid - lo, nb = hi - mid, total = hi - lo;
      for (long long o0 = (long long)threadIdx.x * kPer; o0 < total; o0 += (long long)blockDim.x * kPer) {
        // merge path: i elements from the first run, o0 - i from the second
        long long ilo = o0 - nb > 0 ? o0 - nb : 0, ihi = o0 < na ? o0 : na;
        while (ilo < ihi) {
          const long long i = (ilo + ihi) >> 1;
          const long long j = o0 - i - 1;
          // first run's element i goes before second run's element j?
          const bool before = pair_less(key_at(x, src, lo + i, asc), src[lo + i],
                                        key_at(x, src, mid + j, asc), src[mid + j]);
          if (before) ilo = i + 1;
          else ihi = i;
        }
        long long i = ilo, j = o0 - ilo;
        const long long oend = o0 + kPer < total ? o0 + kPer : total;
        for (long long o = o0; o < oend; o++) {
          bool take_a;
          if (i >= na) take_a = false;
          else if (j >= nb) take_a = true;
          else
            take_a = pair_less(key_at(x, src, lo + i, asc), src[lo + i],
                               key_at(x, src, mid + j, asc), src[mid + j]);
          dst[lo + o] = take_a ? src[lo + i++] : src[mid + j++];
        }
      }
    }
    __syncthreads();
    long long* t = src;
    src = dst;
    dst = t;
  }
  for (long long i = threadIdx.x; i < L; i += blockDim.x) emit<T, ARG>(out, x, st + i, st, src[i], limit);
}

template <class T, class U, bool ARG>
cudaError_t launch_sort(void* toptr, const T* fromptr, long long length, const U* offsets,
                        long long offsetslength, bool ascending, cudaStream_t s) {
  if (length <= 0) return cudaSuccess;
  const long long nseg = offsetslength - 1;
  long long limit = length;
  if (!ARG) {
    // the CPU gathers min(offsets[last], length) values; read offsets[last]
    limit = 0;
    if (offsetslength > 0) {
      U last = 0;
      cudaError_t e = cudaMemcpyAsync(&last, offsets + (offsetslength - 1), sizeof(U),
                                      cudaMemcpyDeviceToHost, s);
      if (e == cudaSuccess) e = cudaStreamSynchronize(s);
      if (e != cudaSuccess) return e;
      limit = (long long)last < length ? (long long)last : length;
    }
  }
  const long long cap = (long long)device_sm_count() * 16;
  auto grid = [cap](long long want) { return (unsigned)(want < 1 ? 1 : want < cap ? want : cap); };
  sort_init_kernel<T, ARG><<<grid((length + 255) / 256), 256, 0, s>>>(toptr, fromptr, length,
                                                                      limit);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess || nseg <= 0) return e;
  // 8 warps per CTA, one segment per warp at a time
  sort_small_kernel<T, U, ARG><<<grid((nseg + 7) / 8), kSortBlock, 0, s>>>(
      toptr, fromptr, length, offsets, nseg, limit, ascending);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  sort_medium_kernel<T, U, ARG><<<grid(nseg), kSortBlock, 0, s>>>(toptr, fromptr, length, offsets,
                                                                 nseg, limit, ascending);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  // long segments: list them, read their count and total size back
  void* scratch = nullptr;
  e = scratch_alloc(&scratch, sizeof(long long) * (size_t)(2 * nseg + 2), s);
  if (e != cudaSuccess) return e;
  unsigned long long* counters = static_cast<unsigned long long*>(scratch);
  long long* ids = reinterpret_cast<long long*>(counters + 2);
  long long* bases = ids + nseg;
  e = cudaMemsetAsync(counters, 0, 2 * sizeof(unsigned long long), s);
  if (e == cudaSuccess) {
    sort_classify_kernel<U><<<grid((nseg + 255) / 256), 256, 0, s>>>(offsets, nseg, length, ids,
                                                                     bases, counters);
    e = cudaGetLastError();
  }
  unsigned long long host_counters[2] = {0, 0};
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(host_counters, counters, sizeof(host_counters), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e == cudaSuccess && host_counters[0] > 0) {
    const long long nlong = (long long)host_counters[0], elems = (long long)host_counters[1];
    void* bufs = nullptr;
    e = scratch_alloc(&bufs, sizeof(long long) * (size_t)(2 * elems), s);
    if (e == cudaSuccess) {
      long long* a = static_cast<long long*>(bufs);
      sort_long_kernel<T, U, ARG><<<(unsigned)nlong, kSortBlock, 0, s>>>(
          toptr, fromptr, length, offsets, ids, bases, a, a + elems, limit, ascending);
      e = cudaGetLastError();
      cudaError_t f = scratch_free(bufs, s);
      if (e == cudaSuccess) e = f;
    }
  }
  cudaError_t f = scratch_free(scratch, s);
  return e != cudaSuccess ? e : f;
}

}  // namespace

#define GB_ARGSORT(SUF, T, USUF, U)                                                            \
  GB_EXPORT int awkward_argsort_##SUF##_##USUF(int64_t* toptr, const T* fromptr, int64_t length, \
                                               const U* offsets, int64_t offsetslength,       \
                                               bool ascending, bool stable,                   \
                                               uint64_t invocation_index, uint64_t* err_code, \
                                               void* stream) {                                \
    (void)stable;                                                                             \
    (void)invocation_index;                                                                   \
    (void)err_code;                                                                           \
    return (int)launch_sort<T, U, true>(toptr, fromptr, length, offsets, offsetslength,        \
                                        ascending, (cudaStream_t)stream);                     \
  }
#define GB_ARGSORT_ALL(SUF, T)                                                                 \
  GB_ARGSORT(SUF, T, int32, int32_t)                                                           \
  GB_ARGSORT(SUF, T, uint32, uint32_t)                                                         \
  GB_ARGSORT(SUF, T, uint64, uint64_t)                                                         \
  GB_ARGSORT(SUF, T, int64, int64_t)
GB_ARGSORT_ALL(bool, bool)
GB_ARGSORT_ALL(int8, int8_t)
GB_ARGSORT_ALL(uint8, uint8_t)
GB_ARGSORT_ALL(int16, int16_t)
GB_ARGSORT_ALL(uint16, uint16_t)
GB_ARGSORT_ALL(int32, int32_t)
GB_ARGSORT_ALL(uint32, uint32_t)
GB_ARGSORT_ALL(int64, int64_t)
GB_ARGSORT_ALL(uint64, uint64_t)
GB_ARGSORT_ALL(float32, float)
GB_ARGSORT_ALL(float64, double)

#define GB_SORT(SUF, T)                                                                        \
  GB_EXPORT int awkward_sort_##SUF(T* toptr, const T* fromptr, int64_t length,                 \
                                   const int64_t* offsets, int64_t offsetslength,             \
                                   bool ascending, bool stable, uint64_t invocation_index,    \
                                   uint64_t* err_code, void* stream) {                        \
    (void)stable;                                                                             \
    (void)invocation_index;                                                                   \
    (void)err_code;                                                                           \
    return (int)launch_sort<T, int64_t, false>(toptr, fromptr, length, offsets, offsetslength, \
                                               ascending, (cudaStream_t)stream);              \
  }
GB_SORT(bool, bool)
GB_SORT(int8, int8_t)
GB_SORT(uint8, uint8_t)
GB_SORT(int16, int16_t)
GB_SORT(uint16, uint16_t)
GB_SORT(int32, int32_t)
GB_SORT(uint32, uint32_t)
GB_SORT(int64, int64_t)
GB_SORT(uint64, uint64_t)
GB_SORT(float32, float)
GB_SORT(float64, double)
