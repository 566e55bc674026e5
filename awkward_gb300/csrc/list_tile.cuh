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
// the tile's slots, consecutive lanes on consecutive slots, each slot finding
// its list by a forward walk over the tile's local offsets.  The fill is
// therefore coalesced and balanced inside the tile regardless of list lengths.
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

// Visit every output slot q (0 <= q < total) of the tile with its list r.
// With at least 4 slots per list on average each warp takes a contiguous
// share, 32 consecutive slots per step (coalesced stores), and a lane finds
// its list by walking forward from the list of the step's first slot; with
// fewer a 32-slot step spans many lists, and a binary search per slot is
// shorter than the walk.
template <class F>
__device__ __forceinline__ void tile_for_each_slot(const TileSmem& sm, long long total, F fn) {
  if (total < 4ll * kTileLists) {
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
    if (q < qb) {
      int rl = r;
      while (sm.loc[rl + 1] <= q) rl++;
      fn(q, rl);
    }
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
