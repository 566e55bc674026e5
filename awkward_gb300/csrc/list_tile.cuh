// list_tile.cuh -- "length-scan then fill" over tiles of consecutive lists.
//
// The jagged getitem, range-slice and combinations kernels all compute a
// per-list output length, an exclusive scan of those lengths (the output
// offsets) and then fill one output slot per (list, position) pair.  Here a
// CTA owns a tile of TL = BLOCK*LPT consecutive lists (tile index from a
// ticket counter, so every predecessor tile is already running): it scans
// its lengths in shared memory, obtains the tile's global prefix with a
// decoupled look-back (single pass, bounded spins), writes its offsets, and
// then fills its outputs in output order -- each warp a contiguous share of
// the tile's slots, consecutive lanes on consecutive slots, the lanes of a
// step finding their lists together from the tile's local offsets.  The fill
// is therefore coalesced and balanced inside the tile regardless of list
// lengths.
#pragma once

#include "gb_common.cuh"

namespace gb {

constexpr int kTileBlock = 256;
constexpr int kTileLPT = 4;
constexpr int kTileLists = kTileBlock * kTileLPT;

// Shared state of one list tile.
struct TileSmem {
  long long loc[kTileLists + 1];  // local exclusive offsets of the tile's lists
  long long scan[kTileBlock / 32 + 1];
  long long tile;
  long long prefix;
  long long total;
};

// Ticket: claim the next tile (all threads; returns it).
__device__ __forceinline__ long long tile_claim(TileSmem& sm, const ScanTiles& st) {
  if (threadIdx.x == 0) sm.tile = (long long)atomicAdd(st.ticket, 1ull);
  __syncthreads();
  return sm.tile;
}

// Scan the per-thread list lengths cnt[0..LPT) (thread t owns lists
// t*LPT .. t*LPT+LPT-1 of the tile), fill sm.loc, and publish / look back.
// Returns the tile's global exclusive prefix; sm.total = tile total.
__device__ __forceinline__ long long tile_scan(TileSmem& sm, const ScanTiles& st,
                                               long long tile, const long long (&cnt)[kTileLPT],
                                               uint64_t inv, uint64_t* err) {
  long long s = 0;
#pragma unroll
  for (int r = 0; r < kTileLPT; r++) s += cnt[r];
  long long total;
  auto add = [](long long a, long long b) { return a + b; };
  long long excl = block_exclusive_scan<kTileBlock>(s, add, 0ll, sm.scan, &total);
  long long run = excl;
#pragma unroll
  for (int r = 0; r < kTileLPT; r++) {
    sm.loc[threadIdx.x * kTileLPT + r] = run;
    run += cnt[r];
  }
  if (threadIdx.x == 0) sm.loc[kTileLists] = total;
  if (threadIdx.x < 32) {
    long long p = lookback_exclusive(st, tile, total, inv, err, GB_MSG_TIMEOUT);
    if (threadIdx.x == 0) {
      sm.prefix = p;
      sm.total = total;
    }
  }
  __syncthreads();
  return sm.prefix;
}

// Local list r (0 <= r < kTileLists) with loc[r] <= q < loc[r+1].
__device__ __forceinline__ int tile_find(const TileSmem& sm, long long q) {
  int lo = 0, hi = kTileLists;  // last r with loc[r] <= q
  while (hi - lo > 1) {
    int mid = (lo + hi) >> 1;
    if (sm.loc[mid] <= q) lo = mid;
    else hi = mid;
  }
  return lo;
}

// Lists of the 32 slots g .. g+31 of one warp step (all lanes call it).  r is
// the list of slot g (the last list with loc[r] <= g).  Lane j gets the list
// of slot g + j, and *rnext the list of slot g + 32.  The ends of lists
// r .. r+31 are loaded one per lane; slot g + j lies in list
// r + #{k : loc[r+1+k] <= g + j}.  Without empty lists among them the ends
// in the step are distinct and that count is a popcount of their bitmask;
// with empty ones a 5-step shuffle search over the sorted ends gives it.
// Returns -1 on every lane when all 32 loaded lists end within the step.
template <class T>
__device__ __forceinline__ int warp_step_lists(const T* loc, int r, T g, int lane, int* rnext) {
  constexpr unsigned kFull = 0xffffffffu;
  const int k = r + 1 + lane;
  int d = 33;  // distance of list r+lane's end from g (1..32 inside the step)
  if (k <= kTileLists) {
    const T diff = loc[k] - g;
    if (diff <= 32) d = (int)diff;
  }
  const unsigned in = __ballot_sync(kFull, d <= 32);
  if (in == kFull) return -1;
  *rnext = r + __popc(in);
  const unsigned ends = __reduce_or_sync(kFull, d <= 32 ? 1u << (d - 1) : 0u);
  const int dn = __shfl_down_sync(kFull, d, 1);
  if (!__any_sync(kFull, lane < 31 && d <= 32 && dn == d))
    return r + __popc(ends & ((1u << lane) - 1u));
  int c = 0;  // largest c with d[c-1] <= lane (d sorted; c <= 31 as in != kFull)
#pragma unroll
  for (int s = 16; s >= 1; s >>= 1) {
    const int dv = __shfl_sync(kFull, d, c + s - 1);
    if (dv <= lane) c += s;
  }
  return r + c;
}

// Visit every output slot q (0 <= q < total) of the tile with its list r.
// With at least 1.5 slots per list on average each warp takes a contiguous
// share, 32 consecutive slots per step (coalesced stores), and the lanes find
// their lists from the list of the step's first slot (warp_step_lists; a
// forward walk when more than 31 lists end inside one step); with fewer a
// 32-slot step often spans more than 32 lists, and a binary search per slot
// is shorter.
template <class F>
__device__ __forceinline__ void tile_for_each_slot(const TileSmem& sm, long long total, F fn) {
  if (total < (long long)(kTileLists + kTileLists / 2)) {
    for (long long q = threadIdx.x; q < total; q += kTileBlock) fn(q, tile_find(sm, q));
    return;
  }
  constexpr int kWarps = kTileBlock / 32;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
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
    if (q < qb) fn(q, rl);
    r = rnext;
  }
}

// Stage the tile of lists [l0, l0 + kTileLists) (those below n): sm.loc holds
// the local exclusive offsets of their (non-negative) counts; returns the
// tile's total count.  All threads call it.
template <class CountFn>
__device__ __forceinline__ long long stage_lists(TileSmem& sm, long long l0, long long n,
                                                 CountFn count) {
  long long c[kTileLPT];
  long long sum = 0;
#pragma unroll
  for (int r = 0; r < kTileLPT; r++) {
    const long long l = l0 + threadIdx.x * kTileLPT + r;
    c[r] = l < n ? count(l) : 0;
    if (c[r] < 0) c[r] = 0;
    sum += c[r];
  }
  long long total;
  auto add = [](long long a, long long b) { return a + b; };
  long long run = block_exclusive_scan<kTileBlock>(sum, add, 0ll, sm.scan, &total);
#pragma unroll
  for (int r = 0; r < kTileLPT; r++) {
    sm.loc[threadIdx.x * kTileLPT + r] = run;
    run += c[r];
  }
  if (threadIdx.x == 0) sm.loc[kTileLists] = total;
  __syncthreads();
  return total;
}

inline long long tile_count(long long n) { return (n + kTileLists - 1) / kTileLists; }

}  // namespace gb
