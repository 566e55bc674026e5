// combinations.cu -- n-tuples of the elements of each list.
//
//   awkward_ListArray_combinations_length  awkward_ListArray_combinations_length.cpp:8-45
//   awkward_ListArray_combinations         awkward_ListArray_combinations.cpp:9-33 with the
//                                          enumeration of kernel-utils.cpp:41-80
//
// The CPU enumerates each list's tuples depth-first in lexicographic order.
// Here every output slot is produced independently: a list tile scans the
// per-list tuple counts (decoupled look-back), then each warp fills a
// contiguous share of the tile's slots, 32 consecutive slots per step; the
// lanes find their lists from the list of the step's first slot, and each
// unranks the slot's lexicographic rank into the tuple (combinatorial
// number system: closed forms for n = 1, 2, 3; for larger n each position by
// bisection over "tuples whose next element is below v" = C(s-lo, rem) -
// C(s-v, rem)).  With replacement the non-decreasing tuple over s elements is
// the strictly increasing tuple over s+n-1 elements with position p shifted
// down by p.  All n output arrays are written coalesced.
#include "list_tile.cuh"

using namespace gb;

namespace {

constexpr int kMaxPtrs = 32;

// The CPU's per-list count, including its arithmetic (no overflow check).
__device__ __forceinline__ long long combinations_count(long long size, long long n,
                                                        bool replacement) {
  if (replacement) size += n - 1;
  if (n == 2 && size < (1ll << 31)) return size < 2 ? 0 : size * (size - 1) / 2;  // same value
  long long thisn = n;
  if (thisn > size) return 0;
  if (thisn == size) return 1;
  if (thisn * 2 > size) thisn = size - thisn;
  long long len = size;
  for (long long j = 2; j <= thisn; j++) {
    len *= (size - j + 1);
    len /= j;
  }
  return len;
}

// C(m, k) by the exact multiplicative recurrence; 0 outside 0 <= k <= m.
__device__ __forceinline__ long long binom(long long m, long long k) {
  if (k < 0 || m < 0 || k > m) return 0;
  if (k > m - k) k = m - k;
  if (k == 0) return 1;
  if (k == 1) return m;
  if (k == 2) return m * (m - 1) / 2;
  long long r = 1;
  for (long long j = 1; j <= k; j++) r = r * (m - k + j) / j;
  return r;
}

template <class C>
__global__ void __launch_bounds__(kTileBlock)
    combinations_length_kernel(int64_t* __restrict__ totallen, int64_t* __restrict__ tooffsets,
                               long long n, bool replacement, const C* __restrict__ starts,
                               const C* __restrict__ stops, long long length, long long ntiles,
                               ScanTiles st, uint64_t inv, uint64_t* err) {
  __shared__ TileSmem sm;
  const long long tile = tile_claim(sm, st);
  const long long l0 = tile * kTileLists;
  long long cnt[kTileLPT];
#pragma unroll
  for (int r = 0; r < kTileLPT; r++) {
    const long long i = l0 + threadIdx.x * kTileLPT + r;
    cnt[r] = i < length ? combinations_count((long long)(stops[i] - starts[i]), n, replacement) : 0;
  }
  const long long prefix = tile_scan(sm, st, tile, cnt, inv, err);
  for (int li = threadIdx.x; li < kTileLists; li += kTileBlock) {
    const long long i = l0 + li;
    if (i < length) tooffsets[i + 1] = prefix + sm.loc[li + 1];
  }
  if (tile == 0 && threadIdx.x == 0) tooffsets[0] = 0;
  if (tile == ntiles - 1 && threadIdx.x == 0) totallen[0] = prefix + sm.total;
}

// Pairs before first element i in a list of s: T(i) = i * (2s - i - 1) / 2.
__device__ __forceinline__ long long pairs_before(long long s, long long i) {
  return i * (2 * s - i - 1) / 2;
}

// Rank -> (i, j), i < j < s, in lexicographic order.  The first element is
// estimated from the closed form of T(i) <= rank in float32 and corrected
// exactly with 64-bit integers (a few steps at most for s < 2^20; a bisection
// above that).
__device__ __forceinline__ void unrank2(long long s, long long rank, long long* i, long long* j) {
  long long a;
  if (s < (1ll << 20)) {
    const float d = (float)(2 * s - 1);
    const float disc = fmaxf(d * d - 8.0f * (float)rank, 0.0f);
    a = (long long)floorf((d - sqrtf(disc)) * 0.5f);
    a = a < 0 ? 0 : (a > s - 2 ? s - 2 : a);
    while (a > 0 && pairs_before(s, a) > rank) a--;
    while (a < s - 2 && pairs_before(s, a + 1) <= rank) a++;
  } else {
    long long lo = 0, hi = s - 2;
    while (lo < hi) {
      const long long mid = (lo + hi + 1) >> 1;
      if (pairs_before(s, mid) <= rank) lo = mid;
      else hi = mid - 1;
    }
    a = lo;
  }
  *i = a;
  *j = a + 1 + (rank - pairs_before(s, a));
}

// The same for lists shorter than 2^15 in 32-bit arithmetic (every product
// stays below 2^31): float estimate from 1/sqrt, then exact correction.
__device__ __forceinline__ void unrank2_small(int s, int rank, int* i, int* j) {
  const float d = (float)(2 * s - 1);
  const float disc = fmaxf(d * d - 8.0f * (float)rank, 1.0f);
  int a = (int)((d - disc * rsqrtf(disc)) * 0.5f);
  a = a < 0 ? 0 : (a > s - 2 ? s - 2 : a);
  const int two_s1 = 2 * s - 1;
  while (a > 0 && ((a * (two_s1 - a)) >> 1) > rank) a--;
  while (a < s - 2 && (((a + 1) * (two_s1 - a - 1)) >> 1) <= rank) a++;
  *i = a;
  *j = a + 1 + (rank - ((a * (two_s1 - a)) >> 1));
}

// C(m, 3) without division in the loop (valid for m < 2^21).
__device__ __forceinline__ long long binom3(long long m) {
  return m < 3 ? 0 : m * (m - 1) * (m - 2) / 6;
}

// Pairs (N = 2) or triples (N = 3) of one warp's share [qa, qb) of a tile's
// output slots, tile-local positions in 32 bits (the tile has fewer than
// 2^31 - 64 tuples).  Each step covers 256 consecutive slots: lane l owns
// slots g + 8l .. g + 8l + 7, finds the list of its first slot by binary
// search over the tile's offsets, unranks that slot (closed forms, as the
// per-slot path) and steps through the next seven by the lexicographic
// successor -- (i, j) -> (i, j + 1), or (i + 1, i + 2) after the row's last
// pair; triples likewise -- moving to the next non-empty list where one
// ends.  The tuples pass through the warp's padded stage `sw` in shared
// memory (kSuccStage words, one output array at a time) so that the stores to
// global memory are coalesced.
constexpr int kSuccStep = 256, kSuccPer = 8;  // slots per warp step, per lane
constexpr int kSuccStage = kSuccStep + kSuccStep / kSuccPer;  // padded: slot j at j + j/8

template <int N>
__device__ __forceinline__ void fill_successors(long long* __restrict__ sw,
                                                const TileSmem& sm, const int* __restrict__ loc32,
                                                const long long* __restrict__ s_start,
                                                const long long* __restrict__ s_size,
                                                int64_t* const* s_ptr, long long prefix, int qa,
                                                int qb, bool replacement) {
  constexpr int kStep = kSuccStep, kPer = kSuccPer;
  const int lane = threadIdx.x & 31;
  const int shift = replacement ? 1 : 0;
  int r = tile_find(sm, qa);
  for (int g = qa; g < qb; g += kStep) {
    const int q0 = g + kPer * lane;
    long long v[N][kPer];
    int rl = r;
    if (q0 < qb) {
      int hi = kTileLists - 1;  // largest rl with loc32[rl] <= q0: the list of slot q0
      while (rl < hi) {
        const int mid = (rl + hi + 1) >> 1;
        if (loc32[mid] <= q0) rl = mid;
        else hi = mid - 1;
      }
      int s = (int)s_size[rl];
      long long base = s_start[rl];
      int cend = loc32[rl + 1];
      const int rank = q0 - loc32[rl];
      int a, b, c = 0;
      if constexpr (N == 2) {
        if (s < (1 << 15)) {
          unrank2_small(s, rank, &a, &b);
        } else {
          long long A, B;
          unrank2(s, rank, &A, &B);
          a = (int)A;
          b = (int)B;
        }
      } else {
        // first element: largest v with C(s,3) - C(s-v,3) <= rank; C(s,3) < 2^31
        auto c3 = [](long long m) { return m < 3 ? 0ll : m * (m - 1) * (m - 2) / 6; };
        const long long tot = c3(s);
        int lo = 0, hi2 = s - 3;
        while (lo < hi2) {
          const int mid = (lo + hi2 + 1) >> 1;
          if (tot - c3(s - mid) <= rank) lo = mid;
          else hi2 = mid - 1;
        }
        int a2, b2;
        unrank2_small(s - lo - 1, (int)(rank - (tot - c3(s - lo))), &a2, &b2);
        a = lo;
        b = lo + 1 + a2;
        c = lo + 1 + b2;
      }
#pragma unroll
      for (int k = 0; k < kPer; k++) {
        const int q = q0 + k;
        v[0][k] = base + a;
        v[1][k] = base + b - shift;
        if constexpr (N == 3) v[2][k] = base + c - 2 * shift;
        if (k + 1 < kPer && q + 1 < qb) {
          if (q + 1 == cend) {  // the next non-empty list
            do {
              rl++;
            } while (loc32[rl + 1] <= q + 1);
            s = (int)s_size[rl];
            base = s_start[rl];
            cend = loc32[rl + 1];
            a = 0;
            b = 1;
            c = 2;
          } else if constexpr (N == 2) {
            if (++b == s) {
              ++a;
              b = a + 1;
            }
          } else {
            if (++c == s) {
              if (++b == s - 1) {
                ++a;
                b = a + 1;
              }
              c = b + 1;
            }
          }
        }
      }
    }
#pragma unroll
    for (int o = 0; o < N; o++) {
      __syncwarp();
      if (q0 < qb) {
#pragma unroll
        for (int k = 0; k < kPer; k++) sw[(kPer + 1) * lane + k] = v[o][k];
      }
      __syncwarp();
      int64_t* __restrict__ outp = s_ptr[o] + prefix;
#pragma unroll
      for (int m = 0; m < kStep / 32; m++) {
        const int j = 32 * m + lane;
        if (g + j < qb) outp[g + j] = sw[j + (j >> 3)];
      }
    }
    r = __shfl_sync(0xffffffffu, rl, 31);  // lists only increase
  }
}

template <class C>
__global__ void __launch_bounds__(kTileBlock, 4)  // 64 registers: 32 warps per SM
    combinations_kernel(int64_t** __restrict__ tocarry, int64_t* __restrict__ toindex,
                        long long n, bool replacement, const C* __restrict__ starts,
                        const C* __restrict__ stops, long long length, long long ntiles,
                        ScanTiles st, uint64_t inv, uint64_t* err) {
  __shared__ TileSmem sm;
  __shared__ long long s_start[kTileLists];
  __shared__ long long s_size[kTileLists];
  __shared__ int64_t* s_ptr[kMaxPtrs];
  const long long tile = tile_claim(sm, st);
  const long long l0 = tile * kTileLists;
  if (threadIdx.x < kMaxPtrs && threadIdx.x < n) s_ptr[threadIdx.x] = tocarry[threadIdx.x];
  long long cnt[kTileLPT];
#pragma unroll
  for (int r = 0; r < kTileLPT; r++) {
    const int li = threadIdx.x * kTileLPT + r;
    const long long i = l0 + li;
    long long c = 0;
    if (i < length) {
      const long long s0 = (long long)starts[i];
      const long long size = (long long)(stops[i] - starts[i]);
      c = combinations_count(size, n, replacement);
      s_start[li] = s0;
      s_size[li] = replacement ? size + n - 1 : size;
    }
    cnt[r] = c;
  }
  const long long prefix = tile_scan(sm, st, tile, cnt, inv, err);
  const long long total = sm.total;
  if (tile == ntiles - 1 && threadIdx.x < n)
    for (long long p = threadIdx.x; p < n; p += kTileBlock) toindex[p] = prefix + total;
  if (n <= 0) return;
  // Each warp fills a contiguous share of the tile's tuples, 32 consecutive
  // output slots per step (coalesced stores); the lanes find their lists
  // from the list of the step's first slot (warp_step_lists).
  constexpr int kWarps = kTileBlock / 32;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if ((n == 2 || n == 3) && total < (1ll << 31) - 64) {
    // pairs or triples of a tile with fewer than 2^31 - 64 of them: tile-local
    // positions in 32 bits (the step positions g + 32 and g + lane stay
    // below 2^31)
    __shared__ int loc32[kTileLists + 1];
    for (int i = threadIdx.x; i <= kTileLists; i += kTileBlock) loc32[i] = (int)sm.loc[i];
    __syncthreads();
    const int t32 = (int)total;
    const int qa = (int)((long long)t32 * warp / kWarps), qb = (int)((long long)t32 * (warp + 1) / kWarps);
    if (qa >= qb) return;
    __shared__ long long stage[kWarps][kSuccStage];  // the warp's output stage
    if (n == 2)
      fill_successors<2>(stage[warp], sm, loc32, s_start, s_size, s_ptr, prefix, qa, qb, replacement);
    else
      fill_successors<3>(stage[warp], sm, loc32, s_start, s_size, s_ptr, prefix, qa, qb, replacement);
    return;
  }
  const long long qa = total * warp / kWarps, qb = total * (warp + 1) / kWarps;
  if (qa >= qb) return;
  int r = tile_find(sm, qa);
  for (long long g = qa; g < qb; g += 32) {
    while (sm.loc[r + 1] <= g) r++;
    const long long q = g + lane;
    int rnext;
    int rl = warp_step_lists(sm.loc, r, g, lane, &rnext);
    if (rl < 0) {
      rl = r;
      if (q < qb)
        while (sm.loc[rl + 1] <= q) rl++;
      rnext = r;
    }
    r = rnext;
    if (q >= qb) continue;
    long long rank = q - sm.loc[rl];
    const long long s = s_size[rl];
    const long long base = s_start[rl];
    const long long out = prefix + q;
    if (n == 1) {
      s_ptr[0][out] = base + rank;
    } else if (n == 2 && s < (1ll << 15)) {
      int a, b;
      unrank2_small((int)s, (int)rank, &a, &b);
      s_ptr[0][out] = base + a;
      s_ptr[1][out] = base + (replacement ? b - 1 : b);
    } else if (n == 2) {
      long long a, b;
      unrank2(s, rank, &a, &b);
      s_ptr[0][out] = base + a;
      s_ptr[1][out] = base + (replacement ? b - 1 : b);
    } else if (n == 3 && s < (1ll << 21)) {
      // first element: largest v with C(s,3) - C(s-v,3) <= rank
      const long long tot = binom3(s);
      long long lo = 0, hi = s - 3;
      while (lo < hi) {
        const long long mid = (lo + hi + 1) >> 1;
        if (tot - binom3(s - mid) <= rank) lo = mid;
        else hi = mid - 1;
      }
      rank -= tot - binom3(s - lo);
      long long a, b;
      unrank2(s - lo - 1, rank, &a, &b);
      const long long p1 = lo + 1 + a, p2 = lo + 1 + b;
      s_ptr[0][out] = base + lo;
      s_ptr[1][out] = base + (replacement ? p1 - 1 : p1);
      s_ptr[2][out] = base + (replacement ? p2 - 2 : p2);
    } else {
      long long lo = 0;
      for (long long p = 0; p < n; p++) {
        const long long rem = n - p;
        const long long here = binom(s - lo, rem);
        long long vlo = lo, vhi = s - rem;
        while (vlo < vhi) {
          long long mid = (vlo + vhi + 1) >> 1;
          if (here - binom(s - mid, rem) <= rank) vlo = mid;
          else vhi = mid - 1;
        }
        rank -= here - binom(s - vlo, rem);
        int64_t* dst = p < kMaxPtrs ? s_ptr[p] : tocarry[p];
        dst[out] = base + (replacement ? vlo - p : vlo);
        lo = vlo + 1;
      }
    }
  }
}

// RegularArray combinations: list i is [size*i, size*i + size), every list
// has the same tuple count c, so slot q belongs to list q / c with rank q % c.
__global__ void regular_combinations_kernel(int64_t** __restrict__ tocarry, long long n,
                                            bool replacement, long long size, long long length,
                                            long long per_list) {
  __shared__ int64_t* s_ptr[kMaxPtrs];
  if (threadIdx.x < kMaxPtrs && threadIdx.x < n) s_ptr[threadIdx.x] = tocarry[threadIdx.x];
  __syncthreads();
  const long long s = replacement ? size + n - 1 : size;
  const long long total = per_list * length;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total;
       q += (long long)gridDim.x * blockDim.x) {
    const long long i = q / per_list;
    long long rank = q - i * per_list;
    const long long base = size * i;
    if (n == 1) {
      s_ptr[0][q] = base + rank;
    } else if (n == 2) {
      long long a, b;
      unrank2(s, rank, &a, &b);
      s_ptr[0][q] = base + a;
      s_ptr[1][q] = base + (replacement ? b - 1 : b);
    } else {
      long long lo = 0;
      for (long long p = 0; p < n; p++) {
        const long long rem = n - p;
        const long long here = binom(s - lo, rem);
        long long vlo = lo, vhi = s - rem;
        while (vlo < vhi) {
          const long long mid = (vlo + vhi + 1) >> 1;
          if (here - binom(s - mid, rem) <= rank) vlo = mid;
          else vhi = mid - 1;
        }
        rank -= here - binom(s - vlo, rem);
        int64_t* dst = p < kMaxPtrs ? s_ptr[p] : tocarry[p];
        dst[q] = base + (replacement ? vlo - p : vlo);
        lo = vlo + 1;
      }
    }
  }
}

__global__ void fill_kernel(int64_t* __restrict__ dst, long long n, long long value) {
  for (long long i = threadIdx.x; i < n; i += blockDim.x) dst[i] = value;
}

long long combinations_count_host(long long size, long long n, bool replacement) {
  if (replacement) size += n - 1;
  long long thisn = n;
  if (thisn > size) return 0;
  if (thisn == size) return 1;
  if (thisn * 2 > size) thisn = size - thisn;
  long long len = size;
  for (long long j = 2; j <= thisn; j++) {
    len *= (size - j + 1);
    len /= j;
  }
  return len;
}

}  // namespace

// awkward_RegularArray_combinations_64.cpp:8-29.  toindex[k] receives the
// total (the CPU's final counters); fromindex is the CPU's scratch cursor.
GB_EXPORT int awkward_RegularArray_combinations_64(int64_t** tocarry, int64_t* toindex,
                                                   int64_t* fromindex, int64_t n, bool replacement,
                                                   int64_t size, int64_t length,
                                                   uint64_t invocation_index, uint64_t* err_code,
                                                   void* stream) {
  (void)fromindex;
  (void)invocation_index;
  (void)err_code;
  cudaStream_t s = (cudaStream_t)stream;
  if (n <= 0) return 0;
  const long long per_list = length > 0 ? combinations_count_host(size, n, replacement) : 0;
  const long long total = per_list * (length > 0 ? length : 0);
  fill_kernel<<<1, 32, 0, s>>>(toindex, n, total);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess || total <= 0) return (int)e;
  long long g = (total + 255) / 256;
  const long long cap = (long long)device_sm_count() * 32;
  regular_combinations_kernel<<<(unsigned)(g < cap ? g : cap), 256, 0, s>>>(
      tocarry, n, replacement, size, length, per_list);
  return (int)cudaGetLastError();
}

#define GB_COMB_LENGTH(NAME, C)                                                                 \
  GB_EXPORT int NAME(int64_t* totallen, int64_t* tooffsets, int64_t n, bool replacement,       \
                     const C* starts, const C* stops, int64_t length, uint64_t invocation_index, \
                     uint64_t* err_code, void* stream) {                                        \
    cudaStream_t s = (cudaStream_t)stream;                                                      \
    if (length <= 0) {                                                                          \
      cudaError_t e = cudaMemsetAsync(tooffsets, 0, sizeof(int64_t), s);                        \
      if (e != cudaSuccess) return (int)e;                                                      \
      return (int)cudaMemsetAsync(totallen, 0, sizeof(int64_t), s);                             \
    }                                                                                           \
    const long long nt = tile_count(length);                                                    \
    ScanTiles st;                                                                               \
    void* base = nullptr;                                                                       \
    cudaError_t e = scan_tiles_alloc(&st, &base, nt, s);                                        \
    if (e != cudaSuccess) return (int)e;                                                        \
    combinations_length_kernel<C><<<(unsigned)nt, kTileBlock, 0, s>>>(                          \
        totallen, tooffsets, n, replacement, starts, stops, length, nt, st, invocation_index,   \
        err_code);                                                                              \
    e = cudaGetLastError();                                                                     \
    cudaError_t f = scratch_free(base, s);                                                      \
    return (int)(e != cudaSuccess ? e : f);                                                     \
  }
GB_COMB_LENGTH(awkward_ListArray32_combinations_length_64, int32_t)
GB_COMB_LENGTH(awkward_ListArrayU32_combinations_length_64, uint32_t)
GB_COMB_LENGTH(awkward_ListArray64_combinations_length_64, int64_t)

// toindex must hold n entries; it receives the total number of tuples per
// position (the CPU's final counters).  fromindex is the CPU's scratch
// cursor and is not used.
#define GB_COMB(NAME, C)                                                                       \
  GB_EXPORT int NAME(int64_t** tocarry, int64_t* toindex, int64_t* fromindex, int64_t n,       \
                     bool replacement, const C* starts, const C* stops, int64_t length,        \
                     uint64_t invocation_index, uint64_t* err_code, void* stream) {            \
    (void)fromindex;                                                                           \
    cudaStream_t s = (cudaStream_t)stream;                                                     \
    if (n <= 0) return 0;                                                                      \
    if (length <= 0) return (int)cudaMemsetAsync(toindex, 0, sizeof(int64_t) * n, s);          \
    const long long nt = tile_count(length);                                                   \
    ScanTiles st;                                                                              \
    void* base = nullptr;                                                                      \
    cudaError_t e = scan_tiles_alloc(&st, &base, nt, s);                                       \
    if (e != cudaSuccess) return (int)e;                                                       \
    combinations_kernel<C><<<(unsigned)nt, kTileBlock, 0, s>>>(tocarry, toindex, n,            \
                                                               replacement, starts, stops,     \
                                                               length, nt, st,                 \
                                                               invocation_index, err_code);    \
    e = cudaGetLastError();                                                                    \
    cudaError_t f = scratch_free(base, s);                                                     \
    return (int)(e != cudaSuccess ? e : f);                                                    \
  }
GB_COMB(awkward_ListArray32_combinations_64, int32_t)
GB_COMB(awkward_ListArrayU32_combinations_64, uint32_t)
GB_COMB(awkward_ListArray64_combinations_64, int64_t)
