// sort_impl.cuh -- segmented sort and argsort (the entry points are in
// sort_argsort_narrow.cu, sort_argsort_wide.cu and sort_values.cu, split
// only to compile in parallel).
//
//   awkward_argsort  awkward_argsort.cpp:62-108
//   awkward_sort     awkward_sort.cpp:62-117
//
// Every element becomes a 64-bit order key whose ascending order is the
// requested order (descending keys are complemented), with awkward's
// comparator rules: integers and bool compare directly; floating point puts
// NaN before every number in both directions, and -0.0 equals +0.0.  Pairs
// (key, index) are sorted ascending -- the index breaks ties, so the result
// is the stable order (std::stable_sort's; it is also a valid answer when
// `stable` is false).  Segments by length:
//   <= 16        a tile of 256 segments: keys staged in shared memory, each
//                element's rank (= output position) counted by one thread;
//   <= 256       one warp: bitonic network in the warp's shared memory;
//   <= 2048      one CTA: merge sort in shared memory (8 pairs per thread
//                sorted in registers, then merge-path rounds);
//   longer       runs of 2048 sorted by many CTAs (as above), then merged
//                pass by pass:
//                each CTA merges 2048 outputs of one pair of runs, staging
//                the inputs they need (found by a merge-path search) in shared
//                memory; (key, index) pairs travel together between two
//                buffers from the library's pool.
// One pass over the segments sorts the short ones and puts the others on
// per-class lists (device counters, read by the later kernels); the long
// class's count, total and longest length are read back once, and only when
// `length` admits a long segment.  Offsets are taken to be non-decreasing, as
// awkward builds them.
#pragma once

#include <limits.h>

#include <type_traits>

#include "gb_common.cuh"
#include "radix_sort.cuh"

using namespace gb;

namespace {

constexpr int kSortBlock = 256;
constexpr int kThreadMax = 16;    // longest segment sorted by ranking its elements
constexpr int kWarpMax = 256;     // ... by one warp
constexpr int kSortTile = 2048;   // ... by one CTA; the run length of long segments
constexpr int kMergePer = kSortTile / kSortBlock;  // outputs merged per thread
constexpr unsigned long long kPadKey = ~0ull;
constexpr long long kPadIdx = LLONG_MAX;

// Counter words (device, zeroed per call).
enum { kCntWarp = 0, kCntCta = 1, kCntLong = 2, kCntLongTotal = 3, kCntLongMax = 4, kCntWords = 5 };

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

template <class I>
__device__ __forceinline__ bool pair_less(unsigned long long ka, I ia, unsigned long long kb, I ib) {
  return ka < kb || (ka == kb && ia < ib);
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

// Position p = st + j of a segment receives its j-th element in order, the
// segment-local index `local`: argsort writes it, sort gathers its value
// (only the first `limit` = min(offsets[last], length) positions).
template <class T, bool ARG>
__device__ __forceinline__ void emit(void* out, const T* x, long long st, long long j,
                                     long long local, long long limit) {
  if (ARG) static_cast<int64_t*>(out)[st + j] = local;
  else if (st + j < limit) static_cast<T*>(out)[st + j] = x[st + local];
}

// The CPU's sort copies min(offsets[last], length) values (argsort: all of
// them); every kernel reads it from the offsets itself, so the host needs no
// copy of it.
template <class U, bool ARG>
__device__ __forceinline__ long long sort_limit(const U* offsets, long long olen,
                                                long long length) {
  if (ARG) return length;
  if (olen <= 0) return 0;
  const long long last = (long long)offsets[olen - 1];
  return last < length ? last : length;
}

// Positions outside [offsets[0], offsets[last]): argsort keeps the iota, sort
// copies through (below `limit`).
template <class T, class U, bool ARG>
__global__ void __launch_bounds__(kSortBlock)
    sort_gaps_kernel(void* out, const T* __restrict__ x, long long length, const U* offsets,
                     long long nseg) {
  const long long limit = sort_limit<U, ARG>(offsets, nseg + 1, length);
  long long first = 0, last = 0;
  if (nseg >= 0) {
    first = (long long)offsets[0];
    last = (long long)offsets[nseg];
    first = first < 0 ? 0 : first > length ? length : first;
    last = last < first ? first : last > length ? length : last;
  }
  const long long gap = first + (length - last);
  for (long long g = blockIdx.x * (long long)kSortBlock + threadIdx.x; g < gap;
       g += (long long)gridDim.x * kSortBlock) {
    const long long i = g < first ? g : last + (g - first);
    if (ARG) static_cast<int64_t*>(out)[i] = i;
    else if (i < limit) static_cast<T*>(out)[i] = x[i];
  }
}

// ------------------------------------------------------------ one thread
template <int N, class I>
__device__ __forceinline__ void reg_bitonic(unsigned long long (&k)[N], I (&ix)[N]) {
#pragma unroll
  for (int size = 2; size <= N; size <<= 1) {
#pragma unroll
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
#pragma unroll
      for (int a = 0; a < N; a++) {
        const int b = a ^ stride;
        if (b > a) {
          const bool up = (a & size) == 0;
          const bool b_first = pair_less(k[b], ix[b], k[a], ix[a]);
          if (b_first == up) {
            const unsigned long long tk = k[a];
            k[a] = k[b];
            k[b] = tk;
            const I ti = ix[a];
            ix[a] = ix[b];
            ix[b] = ti;
          }
        }
      }
    }
  }
}


// Sort the segments of <= 16 elements; list the others by class.  A CTA
// takes 256 consecutive segments: the order keys of the short ones are staged
// in shared memory (coalesced loads), then every element counts the keys of
// its segment that precede it (smaller key, or equal key at a lower position)
// -- its rank is its output position.  One thread per element: the work of a
// segment is spread over its elements and no lane runs a network sized for
// the longest segment of its warp.
constexpr int kRankSegs = kSortBlock;              // segments per tile
constexpr int kRankElems = kRankSegs * kThreadMax;  // staged keys per tile

template <class T, class U, bool ARG>
__global__ void __launch_bounds__(kSortBlock)
    sort_small_kernel(void* out, const T* __restrict__ x, long long length,
                      const U* __restrict__ offsets, long long nseg, bool asc,
                      long long* __restrict__ lists, unsigned long long* counters,
                      long long* __restrict__ long_ids, long long* __restrict__ long_base,
                      long long long_cap) {
  const long long limit = sort_limit<U, ARG>(offsets, nseg + 1, length);
  __shared__ unsigned long long s_key[kRankElems];
  __shared__ unsigned char s_seg[kRankElems];  // tile segment of each staged key
  __shared__ int s_loc[kRankSegs + 1];
  __shared__ long long s_st[kRankSegs];
  __shared__ int s_scan[kSortBlock / 32 + 1];
  const int lane = threadIdx.x & 31;
  const long long ntiles = (nseg + kRankSegs - 1) / kRankSegs;
  for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const long long s = tile * kRankSegs + threadIdx.x;
    long long st = 0, sp = 0;
    if (s < nseg) seg_bounds(offsets, s, length, &st, &sp);
    const long long L = sp - st;
    const int cls = L <= 0 ? -1 : L <= kThreadMax ? 0 : L <= kWarpMax ? 1 : L <= kSortTile ? 2 : 3;
    // class lists: warps from the front of `lists`, CTAs from the back
#pragma unroll
    for (int c = 1; c <= 2; c++) {
      const unsigned m = __ballot_sync(0xffffffffu, cls == c);
      if (m == 0) continue;
      unsigned long long b0 = 0;
      if (lane == __ffs(m) - 1)
        b0 = atomicAdd(counters + (c == 1 ? kCntWarp : kCntCta), (unsigned long long)__popc(m));
      b0 = __shfl_sync(0xffffffffu, b0, __ffs(m) - 1);
      if (cls == c) {
        const long long r = (long long)b0 + __popc(m & ((1u << lane) - 1u));
        lists[c == 1 ? r : nseg - 1 - r] = s;
      }
    }
    if (cls == 3) {
      const unsigned long long k = atomicAdd(counters + kCntLong, 1ull);
      if ((long long)k < long_cap) {  // beyond it only with overlapping segments
        long_ids[k] = s;
        long_base[k] = (long long)atomicAdd(counters + kCntLongTotal, (unsigned long long)L);
        atomicMax(counters + kCntLongMax, (unsigned long long)L);
      }
    }
    // the short segments' local offsets
    int total;
    auto add = [](int a, int b) { return a + b; };
    const int loc = block_exclusive_scan<kSortBlock>(cls == 0 ? (int)L : 0, add, 0, s_scan, &total);
    s_loc[threadIdx.x] = loc;
    s_st[threadIdx.x] = st;
    if (threadIdx.x == 0) s_loc[kRankSegs] = total;
    if (cls == 0)
      for (int p = 0; p < (int)L; p++) s_seg[loc + p] = (unsigned char)threadIdx.x;
    __syncthreads();
    for (int q = threadIdx.x; q < total; q += kSortBlock) {
      const int r = s_seg[q];
      s_key[q] = sort_key(x[s_st[r] + (q - s_loc[r])], asc);
    }
    __syncthreads();
    for (int q = threadIdx.x; q < total; q += kSortBlock) {
      const int r = s_seg[q];
      const int b = s_loc[r], n = s_loc[r + 1] - b, p = q - b;
      const unsigned long long k = s_key[q];
      int rank = 0;
      for (int j = 0; j < n; j++) {
        const unsigned long long kj = s_key[b + j];
        rank += (kj < k) | ((kj == k) & (j < p));
      }
      emit<T, ARG>(out, x, s_st[r], rank, p, limit);
    }
    __syncthreads();
  }
}

// ------------------------------------------------------------ one warp
template <class T, class U, bool ARG>
__global__ void __launch_bounds__(kSortBlock)
    sort_warp_kernel(void* out, const T* __restrict__ x, long long length,
                     const U* __restrict__ offsets, long long nseg, bool asc,
                     const long long* __restrict__ lists, const unsigned long long* counters) {
  const long long limit = sort_limit<U, ARG>(offsets, nseg + 1, length);
  __shared__ unsigned long long s_key[kSortBlock / 32][kWarpMax];
  __shared__ int s_idx[kSortBlock / 32][kWarpMax];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  unsigned long long* key = s_key[w];
  int* idx = s_idx[w];
  const long long n = (long long)counters[kCntWarp];
  for (long long e = (blockIdx.x * (long long)kSortBlock + threadIdx.x) >> 5; e < n;
       e += ((long long)gridDim.x * kSortBlock) >> 5) {
    const long long s = lists[e];
    long long st, sp;
    seg_bounds(offsets, s, length, &st, &sp);
    const int L = (int)(sp - st);
    int P = 32;
    while (P < L) P <<= 1;
    for (int i = lane; i < P; i += 32) {
      key[i] = i < L ? sort_key(x[st + i], asc) : kPadKey;
      idx[i] = i;
    }
    __syncwarp();
    for (int k = 2; k <= P; k <<= 1) {
      for (int j = k >> 1; j > 0; j >>= 1) {
        for (int i = lane; i < P; i += 32) {
          const int p = i ^ j;
          if (p > i) {
            const bool up = (i & k) == 0;
            if (pair_less(key[p], idx[p], key[i], idx[i]) == up) {
              const unsigned long long tk = key[i];
              key[i] = key[p];
              key[p] = tk;
              const int ti = idx[i];
              idx[i] = idx[p];
              idx[p] = ti;
            }
          }
        }
        __syncwarp();
      }
    }
    for (int i = lane; i < L; i += 32) emit<T, ARG>(out, x, st, i, idx[i], limit);
    __syncwarp();
  }
}

// ------------------------------------------------------------ one CTA
// Shared-memory tiles hold pair p at slot p + p/16: with 8 consecutive pairs
// per thread (and merges reading about 4 apart), unpadded 64-bit slots would
// put the lanes of a warp on a few banks.
constexpr int kPadTile = kSortTile + kSortTile / 16;
__device__ __forceinline__ int pslot(int p) { return p + (p >> 4); }

// Number of elements taken from run a (slots a0.., length na) among the first
// d outputs of merging it with run b (slots b0.., length nb); ties go to a.
template <class I>
__device__ __forceinline__ int merge_split_s(const unsigned long long* sk, const I* si, int a0,
                                             int na, int b0, int nb, int d) {
  int lo = d - nb > 0 ? d - nb : 0, hi = d < na ? d : na;
  while (lo < hi) {
    const int i = (lo + hi) >> 1;
    const int pa = pslot(a0 + i), pb = pslot(b0 + d - i - 1);
    if (pair_less(sk[pa], si[pa], sk[pb], si[pb])) lo = i + 1;
    else hi = i;
  }
  return lo;
}

// Merge kMergePer outputs starting at output d of runs a and b into registers.
template <class I>
__device__ __forceinline__ void merge_into(const unsigned long long* sk, const I* si, int a0,
                                           int na, int b0, int nb, int d,
                                           unsigned long long (&k)[kMergePer], I (&ix)[kMergePer]) {
  int i = merge_split_s(sk, si, a0, na, b0, nb, d);
  int j = d - i;
#pragma unroll
  for (int o = 0; o < kMergePer; o++) {
    // clamped to a real slot of the other run once one is used up (b0 = a0 + na
    // and na + nb >= 1 in every caller), so both reads stay in the tile
    const int pa = pslot(a0 + (i < na ? i : (na > 0 ? na - 1 : 0)));
    const int pb = pslot(b0 + (j < nb ? j : (nb > 0 ? nb - 1 : -1)));
    const bool take_a = i < na && (j >= nb || !pair_less(sk[pb], si[pb], sk[pa], si[pa]));
    k[o] = take_a ? sk[pa] : sk[pb];
    ix[o] = take_a ? si[pa] : si[pb];
    i += take_a;
    j += !take_a;
  }
}

// Sort the kSortTile pairs of a padded shared-memory tile: kMergePer
// consecutive pairs per thread sorted in registers, then rounds that merge
// runs of doubling width, each thread producing kMergePer consecutive outputs
// from a merge-path split.
template <class I>
__device__ __forceinline__ void block_merge_sort(unsigned long long* s_key, I* s_idx) {
  unsigned long long k[kMergePer];
  I ix[kMergePer];
  const int t0 = threadIdx.x * kMergePer;
#pragma unroll
  for (int i = 0; i < kMergePer; i++) {
    k[i] = s_key[pslot(t0 + i)];
    ix[i] = s_idx[pslot(t0 + i)];
  }
  reg_bitonic<kMergePer, I>(k, ix);
  for (int width = kMergePer; width < kSortTile; width <<= 1) {
    __syncthreads();
#pragma unroll
    for (int i = 0; i < kMergePer; i++) {
      s_key[pslot(t0 + i)] = k[i];
      s_idx[pslot(t0 + i)] = ix[i];
    }
    __syncthreads();
    const int start = t0 & ~(2 * width - 1);
    merge_into(s_key, s_idx, start, width, start + width, width, t0 - start, k, ix);
  }
  __syncthreads();
#pragma unroll
  for (int i = 0; i < kMergePer; i++) {
    s_key[pslot(t0 + i)] = k[i];
    s_idx[pslot(t0 + i)] = ix[i];
  }
  __syncthreads();
}

template <class T, class U, bool ARG>
__global__ void __launch_bounds__(kSortBlock)
    sort_cta_kernel(void* out, const T* __restrict__ x, long long length,
                    const U* __restrict__ offsets, long long nseg, bool asc,
                    const long long* __restrict__ lists, const unsigned long long* counters) {
  const long long limit = sort_limit<U, ARG>(offsets, nseg + 1, length);
  __shared__ unsigned long long s_key[kPadTile];
  __shared__ int s_idx[kPadTile];
  const long long n = (long long)counters[kCntCta];
  for (long long e = blockIdx.x; e < n; e += gridDim.x) {
    const long long s = lists[nseg - 1 - e];
    long long st, sp;
    seg_bounds(offsets, s, length, &st, &sp);
    const int L = (int)(sp - st);
    for (int i = threadIdx.x; i < kSortTile; i += kSortBlock) {
      s_key[pslot(i)] = i < L ? sort_key(x[st + i], asc) : kPadKey;
      s_idx[pslot(i)] = i;
    }
    __syncthreads();
    block_merge_sort(s_key, s_idx);
    for (int i = threadIdx.x; i < L; i += kSortBlock)
      emit<T, ARG>(out, x, st, i, s_idx[pslot(i)], limit);
    __syncthreads();
  }
}

// ------------------------------------------------------------ long segments
// Runs of kSortTile sorted in shared memory into (key, global index) pairs at
// the segment's slot `base` of buffer A.
template <class T, class U>
__global__ void __launch_bounds__(kSortBlock)
    sort_runs_kernel(const T* __restrict__ x, long long length, const U* __restrict__ offsets,
                     const long long* __restrict__ long_ids, const long long* __restrict__ long_base,
                     long long nlong, bool asc, unsigned long long* __restrict__ akey,
                     long long* __restrict__ aidx) {
  __shared__ unsigned long long s_key[kPadTile];
  __shared__ long long s_idx[kPadTile];
  for (long long k = blockIdx.y; k < nlong; k += gridDim.y) {
    long long st, stop;
    seg_bounds(offsets, long_ids[k], length, &st, &stop);
    const long long L = stop - st, base = long_base[k];
    for (long long r0 = (long long)blockIdx.x * kSortTile; r0 < L;
         r0 += (long long)gridDim.x * kSortTile) {
      const int n = (int)(L - r0 < kSortTile ? L - r0 : kSortTile);
      for (int i = threadIdx.x; i < kSortTile; i += kSortBlock) {
        s_key[pslot(i)] = i < n ? sort_key(x[st + r0 + i], asc) : kPadKey;
        s_idx[pslot(i)] = i < n ? st + r0 + i : kPadIdx;
      }
      __syncthreads();
      block_merge_sort(s_key, s_idx);
      for (int i = threadIdx.x; i < n; i += kSortBlock) {
        akey[base + r0 + i] = s_key[pslot(i)];
        aidx[base + r0 + i] = s_idx[pslot(i)];
      }
      __syncthreads();
    }
  }
}

__device__ __forceinline__ long long merge_split_g(const unsigned long long* ak, const long long* ai,
                                                   long long na, const unsigned long long* bk,
                                                   const long long* bi, long long nb, long long d) {
  long long lo = d - nb > 0 ? d - nb : 0, hi = d < na ? d : na;
  while (lo < hi) {
    const long long i = (lo + hi) >> 1;
    const long long j = d - i - 1;
    if (pair_less(ak[i], ai[i], bk[j], bi[j])) lo = i + 1;
    else hi = i;
  }
  return lo;
}

// Merge-path splits of every chunk start of the merge pass at width w: the
// number of pairs run a contributes to the outputs before the chunk (relative
// to the chunk's pair of runs).  One thread per chunk, all in flight at once.
__global__ void __launch_bounds__(kSortBlock)
    sort_partition_kernel(const long long* __restrict__ long_lengths,
                          const long long* __restrict__ long_base,
                          const long long* __restrict__ cbase, long long nlong, long long w,
                          const unsigned long long* __restrict__ skey,
                          const long long* __restrict__ sidx, long long* __restrict__ splits) {
  for (long long k = blockIdx.y; k < nlong; k += gridDim.y) {
    const long long L = long_lengths[k], base = long_base[k];
    if (L <= w) continue;
    const long long nchunks = (L + kSortTile - 1) / kSortTile;
    for (long long c = blockIdx.x * (long long)kSortBlock + threadIdx.x; c < nchunks;
         c += (long long)gridDim.x * kSortBlock) {
      const long long o0 = c * kSortTile;
      const long long lo = o0 / (2 * w) * (2 * w);
      const long long mid = lo + w < L ? lo + w : L, hi = lo + 2 * w < L ? lo + 2 * w : L;
      splits[cbase[k] + c] = merge_split_g(skey + base + lo, sidx + base + lo, mid - lo,
                                           skey + base + mid, sidx + base + mid, hi - mid, o0 - lo);
    }
  }
}

__global__ void long_chunks_kernel(const long long* __restrict__ lens, long long nlong,
                                   long long* __restrict__ chunks) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < nlong;
       k += (long long)gridDim.x * blockDim.x)
    chunks[k] = (lens[k] + kSortTile - 1) / kSortTile;
}

// One merge pass at run width w: runs [lo, lo+w) and [lo+w, lo+2w) of each
// segment longer than w merge into 2w.  A CTA produces kSortTile consecutive
// outputs of one pair (pairs are multiples of kSortTile long).
__global__ void __launch_bounds__(kSortBlock)
    sort_merge_kernel(const long long* __restrict__ long_lengths,
                      const long long* __restrict__ long_base, const long long* __restrict__ cbase,
                      long long nlong, long long w, const long long* __restrict__ splits,
                      const unsigned long long* __restrict__ skey, const long long* __restrict__ sidx,
                      unsigned long long* __restrict__ dkey, long long* __restrict__ didx) {
  __shared__ unsigned long long s_key[kPadTile];
  __shared__ long long s_idx[kPadTile];
  for (long long k = blockIdx.y; k < nlong; k += gridDim.y) {
    const long long L = long_lengths[k], base = long_base[k];
    if (L <= w) continue;  // already one run: its pairs stay where its last pass put them
    for (long long o0 = (long long)blockIdx.x * kSortTile; o0 < L;
         o0 += (long long)gridDim.x * kSortTile) {
      const long long lo = o0 / (2 * w) * (2 * w);
      const long long mid = lo + w < L ? lo + w : L, hi = lo + 2 * w < L ? lo + 2 * w : L;
      const long long na = mid - lo;
      const long long o1 = o0 + kSortTile < hi ? o0 + kSortTile : hi;
      const unsigned long long* ak = skey + base + lo;
      const long long* ai = sidx + base + lo;
      const unsigned long long* bk = skey + base + mid;
      const long long* bi = sidx + base + mid;
      // the chunk's bounding splits, found by the partition kernel (the next
      // chunk's start when it lies in the same pair of runs)
      const long long ci = cbase[k] + o0 / kSortTile;
      const long long a0 = splits[ci];
      const long long a1 = o1 == hi ? na : splits[ci + 1];
      const long long b0 = (o0 - lo) - a0, b1 = (o1 - lo) - a1;
      const int ca = (int)(a1 - a0), cb = (int)(b1 - b0);
      // stage this chunk's inputs: ca from run a, then cb from run b
      for (int i = threadIdx.x; i < ca + cb; i += kSortBlock) {
        if (i < ca) {
          s_key[pslot(i)] = ak[a0 + i];
          s_idx[pslot(i)] = ai[a0 + i];
        } else {
          s_key[pslot(i)] = bk[b0 + (i - ca)];
          s_idx[pslot(i)] = bi[b0 + (i - ca)];
        }
      }
      __syncthreads();
      const int d = threadIdx.x * kMergePer;
      const int cnt = ca + cb;
      unsigned long long ok[kMergePer];
      long long oi[kMergePer];
      if (d < cnt) merge_into(s_key, s_idx, 0, ca, ca, cb, d, ok, oi);
      __syncthreads();
      // outputs through shared memory, then coalesced stores
#pragma unroll
      for (int o = 0; o < kMergePer; o++) {
        if (d + o < cnt) {
          s_key[pslot(d + o)] = ok[o];
          s_idx[pslot(d + o)] = oi[o];
        }
      }
      __syncthreads();
      for (int i = threadIdx.x; i < cnt; i += kSortBlock) {
        dkey[base + o0 + i] = s_key[pslot(i)];
        didx[base + o0 + i] = s_idx[pslot(i)];
      }
      __syncthreads();
    }
  }
}

// Long segments' final pairs to the output (in A or B by their pass count).
template <class T, class U, bool ARG>
__global__ void __launch_bounds__(kSortBlock)
    sort_long_emit_kernel(void* out, const T* __restrict__ x, long long length,
                          const U* __restrict__ offsets, const long long* __restrict__ long_ids,
                          const long long* __restrict__ long_base, long long nlong,
                          const long long* __restrict__ aidx, const long long* __restrict__ bidx,
                          long long nseg) {
  const long long limit = sort_limit<U, ARG>(offsets, nseg + 1, length);
  for (long long k = blockIdx.y; k < nlong; k += gridDim.y) {
    long long st, sp;
    seg_bounds(offsets, long_ids[k], length, &st, &sp);
    const long long L = sp - st, base = long_base[k];
    int passes = 0;
    for (long long w = kSortTile; w < L; w <<= 1) passes++;
    const long long* src = (passes & 1) ? bidx : aidx;
    for (long long i = blockIdx.x * (long long)kSortBlock + threadIdx.x; i < L;
         i += (long long)gridDim.x * kSortBlock)
      emit<T, ARG>(out, x, st, i, src[base + i] - st, limit);
  }
}

template <class U>
__global__ void long_lengths_kernel(const U* __restrict__ offsets, long long length,
                                    const long long* __restrict__ long_ids, long long nlong,
                                    long long* __restrict__ lens) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < nlong;
       k += (long long)gridDim.x * blockDim.x) {
    long long st, sp;
    seg_bounds(offsets, long_ids[k], length, &st, &sp);
    lens[k] = sp - st;
  }
}

template <class T, class U, bool ARG>
cudaError_t launch_sort(void* toptr, const T* fromptr, long long length, const U* offsets,
                        long long offsetslength, bool ascending, uint64_t inv, uint64_t* err,
                        cudaStream_t s) {
  if (length <= 0) return cudaSuccess;
  const long long nseg = offsetslength - 1;
  const long long cap = (long long)device_sm_count() * 16;
  auto grid = [cap](long long want) { return (unsigned)(want < 1 ? 1 : want < cap ? want : cap); };
  sort_gaps_kernel<T, U, ARG><<<grid((length + kSortBlock - 1) / kSortBlock), kSortBlock, 0, s>>>(
      toptr, fromptr, length, offsets, nseg < 0 ? -1 : nseg);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess || nseg <= 0) return e;
  // class lists and counters
  const long long long_cap_n = length / (kSortTile + 1) + 1;
  const long long long_cap = long_cap_n < nseg ? long_cap_n : nseg;
  void* scratch = nullptr;
  e = scratch_alloc(&scratch, sizeof(long long) * (size_t)(kCntWords + nseg + 3 * long_cap), s);
  if (e != cudaSuccess) return e;
  unsigned long long* counters = static_cast<unsigned long long*>(scratch);
  long long* lists = reinterpret_cast<long long*>(counters + kCntWords);
  long long* long_ids = lists + nseg;
  long long* long_base = long_ids + long_cap;
  long long* long_len = long_base + long_cap;
  e = cudaMemsetAsync(counters, 0, sizeof(unsigned long long) * kCntWords, s);
  if (e == cudaSuccess) {
    sort_small_kernel<T, U, ARG><<<grid((nseg + kSortBlock - 1) / kSortBlock), kSortBlock, 0, s>>>(
        toptr, fromptr, length, offsets, nseg, ascending, lists, counters, long_ids,
        long_base, long_cap);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) {
    sort_warp_kernel<T, U, ARG><<<(unsigned)cap, kSortBlock, 0, s>>>(
        toptr, fromptr, length, offsets, nseg, ascending, lists, counters);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) {
    sort_cta_kernel<T, U, ARG><<<(unsigned)cap, kSortBlock, 0, s>>>(
        toptr, fromptr, length, offsets, nseg, ascending, lists, counters);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess && length > kSortTile) {
    unsigned long long hc[kCntWords];
    e = cudaMemcpyAsync(hc, counters, sizeof(hc), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    const long long nlong = (long long)hc[kCntLong] < long_cap ? (long long)hc[kCntLong] : long_cap;
    const long long total = (long long)hc[kCntLongTotal];
    const long long maxl = (long long)hc[kCntLongMax];
    if (e == cudaSuccess && nlong > 0) {
      void* bufs = nullptr;
      // pair buffers A and B, then per long segment its chunk count and first
      // chunk, then one split per chunk
      const long long nsplit = total / kSortTile + nlong + 1;
      e = scratch_alloc(&bufs, 32 * (size_t)total + 8 * (size_t)(2 * nlong + nsplit), s);
      if (e == cudaSuccess) {
        unsigned long long* akey = static_cast<unsigned long long*>(bufs);
        long long* aidx = reinterpret_cast<long long*>(akey + total);
        unsigned long long* bkey = reinterpret_cast<unsigned long long*>(aidx + total);
        long long* bidx = reinterpret_cast<long long*>(bkey + total);
        long long* chunks_n = bidx + total;
        long long* cbase = chunks_n + nlong;
        long long* splits = cbase + nlong;
        const unsigned gy = (unsigned)(nlong < 65535 ? nlong : 65535);
        const long long chunks = (maxl + kSortTile - 1) / kSortTile;
        const unsigned gx = (unsigned)(chunks < 65535 ? chunks : 65535);
        const long long pchunks = (chunks + kSortBlock - 1) / kSortBlock;
        const unsigned pgx = (unsigned)(pchunks < 65535 ? pchunks : 65535);
        long_lengths_kernel<U><<<grid((nlong + 255) / 256), 256, 0, s>>>(offsets, length, long_ids,
                                                                        nlong, long_len);
        long_chunks_kernel<<<grid((nlong + 255) / 256), 256, 0, s>>>(long_len, nlong, chunks_n);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = exclusive_scan_i64(chunks_n, cbase, nlong, nullptr, inv, err, s);
        if (e == cudaSuccess) {
          sort_runs_kernel<T, U><<<dim3(gx, gy), kSortBlock, 0, s>>>(
              fromptr, length, offsets, long_ids, long_base, nlong, ascending, akey, aidx);
          e = cudaGetLastError();
        }
        int pass = 0;
        for (long long w = kSortTile; w < maxl && e == cudaSuccess; w <<= 1, pass++) {
          const bool even = (pass & 1) == 0;
          sort_partition_kernel<<<dim3(pgx, gy), kSortBlock, 0, s>>>(
              long_len, long_base, cbase, nlong, w, even ? akey : bkey, even ? aidx : bidx, splits);
          sort_merge_kernel<<<dim3(gx, gy), kSortBlock, 0, s>>>(
              long_len, long_base, cbase, nlong, w, splits, even ? akey : bkey, even ? aidx : bidx,
              even ? bkey : akey, even ? bidx : aidx);
          e = cudaGetLastError();
        }
        if (e == cudaSuccess) {
          const long long egx = (maxl + kSortBlock - 1) / kSortBlock;
          sort_long_emit_kernel<T, U, ARG>
              <<<dim3((unsigned)(egx < 65535 ? egx : 65535), gy), kSortBlock, 0, s>>>(
                  toptr, fromptr, length, offsets, long_ids, long_base, nlong, aidx, bidx, nseg);
          e = cudaGetLastError();
        }
        cudaError_t f = scratch_free(bufs, s);
        if (e == cudaSuccess) e = f;
      }
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
    return (int)launch_sort<T, U, true>(toptr, fromptr, length, offsets, offsetslength,        \
                                        ascending, invocation_index, err_code,                \
                                        (cudaStream_t)stream);                                \
  }
#define GB_ARGSORT_ALL(SUF, T)                                                                 \
  GB_ARGSORT(SUF, T, int32, int32_t)                                                           \
  GB_ARGSORT(SUF, T, uint32, uint32_t)                                                         \
  GB_ARGSORT(SUF, T, uint64, uint64_t)                                                         \
  GB_ARGSORT(SUF, T, int64, int64_t)
#define GB_SORT(SUF, T)                                                                        \
  GB_EXPORT int awkward_sort_##SUF(T* toptr, const T* fromptr, int64_t length,                 \
                                   const int64_t* offsets, int64_t offsetslength,             \
                                   bool ascending, bool stable, uint64_t invocation_index,    \
                                   uint64_t* err_code, void* stream) {                        \
    (void)stable;                                                                             \
    return (int)launch_sort<T, int64_t, false>(toptr, fromptr, length, offsets, offsetslength, \
                                               ascending, invocation_index, err_code,         \
                                               (cudaStream_t)stream);                         \
  }
