// seg_reduce.cuh -- merge-path segmented reduction over ListOffsetArray offsets.
//
// Replaces the per-bin loops of awkward-cpp's reducers
// (awkward-cpp/src/cpu-kernels/awkward_reduce_*.cpp) for the cupy backend.
//
// Work decomposition.  The reduction is a merge of two sorted streams: the
// list ends A[i] = offsets[i+1] (i < nlists) and the element indices
// j in [offsets[0], offsets[nlists]).  Consuming an element accumulates it
// into the current list; consuming a list end emits that list's result.  The
// merged sequence has D = nlists + E items.  A persistent grid of G CTAs
// splits D into equal diagonal ranges (perfect balance for any length
// distribution: empty lists, Poisson, heavy tails, one giant list); each CTA
// locates its two ends with a warp-wide 32-ary merge-path search in global
// memory.
//
// Inside a CTA, one producer warp streams the CTA's slices of `offsets` and
// of the content into two shared-memory rings of fixed-size stages with 1-D
// TMA bulk copies (cp.async.bulk of the 16-byte aligned interior; ragged
// head and tail by plain loads), guarded by full/empty mbarrier pairs, so
// loads run several chunks ahead of the reduction.  Eight consumer warps
// reduce chunks of IPC = 256*IPT merge items: they convert the chunk's list
// ends into a linear int32 window (relative to the chunk's first element),
// every thread locates its IPT items by binary search in that window and
// walks them, a block-wide segmented scan stitches lists that cross
// threads, and finished stages are handed back to the producer.  HBM
// traffic is one pass over offsets and content.  Lists that cross CTAs leave
// one head and one tail record per CTA; a one-block fix-up kernel combines
// them with a segmented scan in CTA order.  No CTA ever waits on another.
//
// Combination order is always earlier-then-later, so order-sensitive
// reducers (max/min/argmax/argmin tie and NaN rules) are bit-exact with the
// sequential CPU loops; floating-point sums differ from the CPU only by
// rounding (a tree instead of a left-to-right sum).
#pragma once

#include <type_traits>

#include "gb_common.cuh"

namespace gb {

// Storage type of a content element (bool is read as a byte).
template <class T>
using store_t = typename std::conditional<std::is_same<T, bool>::value, uint8_t, T>::type;

template <class Acc>
struct SegVal {
  Acc acc;
  uint32_t flag;  // a segment (list) starts inside this range
  uint32_t pad;
};

template <class Acc>
struct CtaRecord {
  long long head_list;  // list that started before this CTA and ends in it, or -1
  long long tail_list;  // list open at the end of this CTA (nlists: none)
  Acc head_acc;
  Acc tail_acc;
  int tail_fresh;  // tail list has no elements before this CTA
  int pad;
};

constexpr int kConsumers = 256;  // consumer threads (8 warps)
constexpr int kProducerWarp = kConsumers / 32;
constexpr int kSegThreads = kConsumers + 32;
constexpr int kSegIPT = 16;
constexpr int kSegIPC = kConsumers * kSegIPT;  // merge items per chunk (at most)
constexpr int kEStage = 1024;                  // elements per content stage
constexpr int kEStages = 6;                    // content ring: 6144 elements
constexpr int kOStage = 256;                   // offsets per offsets stage
constexpr int kOStages = 6;                    // offsets ring: 1536 entries
constexpr int kOWin = 1024;                    // list ends visible to one chunk
constexpr int kLendBig = 0x7fffffff;
static_assert(kEStages * kEStage >= kSegIPC + kEStage, "content ring too small");
static_assert(kOStages * kOStage >= kOWin + 1 + kOStage, "offsets ring too small");
static_assert((kEStage & (kEStage - 1)) == 0 && (kOStage & (kOStage - 1)) == 0,
              "stage sizes are powers of two");

template <class Store, class Acc>
struct SegSmem {
  int64_t oring[kOStages * kOStage];
  Store ering[kEStages * kEStage];
  int lend[kOWin + 1];  // chunk-local list ends (element position relative to cj)
  SegVal<Acc> scan[kConsumers / 32 + 1];
  SegVal<Acc> carry;
  uint64_t full_e[kEStages], empty_e[kEStages];
  uint64_t full_o[kOStages], empty_o[kOStages];
  long long coords[4];
  long long lstart0;  // start of list ci relative to cj
  int kend;
  int len;
  int head_pending;
};

__device__ __forceinline__ void consumer_sync() {
  asm volatile("bar.sync 1, %0;" ::"n"(kConsumers) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_test(uint64_t* bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n"
      ".reg .pred p;\n"
      "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      "selp.u32 %0, 1, 0, p;\n"
      "}\n"
      : "=r"(done)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return done != 0;
}

// Merge-path split of diagonal d in global memory (one warp).  Returns the
// number of list ends consumed among the first d merged items.
__device__ __forceinline__ long long mp_search_global(const int64_t* __restrict__ offsets,
                                                      long long nlists, long long e0,
                                                      long long E, long long d) {
  const int lane = threadIdx.x & 31;
  long long lo = d - E > 0 ? d - E : 0;
  long long hi = d < nlists ? d : nlists;  // answer in [lo, hi]
  while (hi - lo > 32) {
    const long long step = (hi - lo) / 32;
    const long long k = lo + (long long)lane * step;
    const bool p = (k + (offsets[k + 1] - e0)) < d;
    const unsigned msk = __ballot_sync(0xffffffffu, p);
    const int cnt = __popc(msk);
    const long long nlo = cnt > 0 ? lo + (long long)(cnt - 1) * step + 1 : lo;
    const long long nhi = cnt < 32 ? lo + (long long)cnt * step : hi;
    lo = nlo;
    hi = nhi;
  }
  const long long k = lo + lane;
  const bool p = (k < hi) && ((k + (offsets[k + 1] - e0)) < d);
  const unsigned msk = __ballot_sync(0xffffffffu, p);
  return lo + __popc(msk);
}

// Producer warp: copy global [lo, hi) of `src` into ring slot `slot` (the
// slot holds global [stage_lo, stage_lo + STAGE)), completing barrier
// `full`.  With TMA the 16-byte aligned interior is one bulk copy and the
// ragged head and tail (each shorter than 16 bytes) are plain loads issued
// before the arrive, which releases them.
template <class T, int STAGE>
__device__ __forceinline__ void produce_stage(T* ring, const T* src, long long stage_lo,
                                              long long lo, long long hi, int slot,
                                              uint64_t* full, bool use_tma) {
  T* slot_base = ring + (size_t)slot * STAGE;
  const int lane = threadIdx.x & 31;
  if (use_tma) {
    constexpr int A = 16 / (int)sizeof(T);
    long long a16 = (lo + A - 1) / A * A;
    long long b16 = hi / A * A;
    if (a16 >= b16) a16 = b16 = hi;
    if (lane == 0) {
      const uint32_t bytes = (uint32_t)((b16 - a16) * (long long)sizeof(T));
      for (long long g = lo; g < a16; g++) slot_base[g - stage_lo] = src[g];
      for (long long g = b16; g < hi; g++) slot_base[g - stage_lo] = src[g];
      mbar_arrive_expect_tx(full, bytes);
      if (bytes) bulk_g2s(slot_base + (a16 - stage_lo), src + a16, bytes, full);
    }
  } else {
    for (long long g = lo + lane; g < hi; g += 32) slot_base[g - stage_lo] = src[g];
    __syncwarp();
    if (lane == 0) mbar_arrive(full);
  }
}

template <class Op>
__global__ void __launch_bounds__(kSegThreads)
    seg_reduce_kernel(Op op, const store_t<typename Op::In>* __restrict__ x,
                      const int64_t* __restrict__ offsets, long long nlists,
                      typename Op::Out* __restrict__ out, CtaRecord<typename Op::Acc>* records,
                      int G, int use_tma_i, uint64_t inv, uint64_t* err) {
  using Acc = typename Op::Acc;
  using Store = store_t<typename Op::In>;
  using V = SegVal<Acc>;
  using Sm = SegSmem<Store, Acc>;
  constexpr int IPC = kSegIPC, IPT = kSegIPT;
  constexpr int RE = kEStages * kEStage;
  constexpr int RO = kOStages * kOStage;
  static_assert(kEStage == 1024 && kOStage == 256, "stage shifts below assume these sizes");

  extern __shared__ __align__(128) unsigned char smem_raw[];
  Sm& sm = *reinterpret_cast<Sm*>(smem_raw);
  const bool use_tma = use_tma_i != 0;

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const long long e0 = offsets[0];
  const long long eN = offsets[nlists];
  const long long E = eN > e0 ? eN - e0 : 0;
  const long long D = nlists + E;
  const int Geff = (int)((D + IPC - 1) / IPC < G ? (D + IPC - 1) / IPC : G);
  const int b = blockIdx.x;
  if (b >= Geff) return;
  const long long d_begin = D * b / Geff, d_end = D * (b + 1) / Geff;

  if (warp < 2) {
    const long long d = warp == 0 ? d_begin : d_end;
    const long long i = mp_search_global(offsets, nlists, e0, E, d);
    if (lane == 0) {
      sm.coords[warp * 2] = i;
      sm.coords[warp * 2 + 1] = e0 + (d - i);
    }
  }
  if (tid == 0) {
    for (int s = 0; s < kEStages; s++) {
      mbar_init(&sm.full_e[s], 1);
      mbar_init(&sm.empty_e[s], 1);
    }
    for (int s = 0; s < kOStages; s++) {
      mbar_init(&sm.full_o[s], 1);
      mbar_init(&sm.empty_o[s], 1);
    }
    fence_barrier_init();
    records[b].head_list = -1;
  }
  __syncthreads();
  const long long I0 = sm.coords[0], J0 = sm.coords[1], I1 = sm.coords[2], J1 = sm.coords[3];
  // Stage grids: content stage s holds [EB + s*kEStage, ...) and offsets stage
  // t holds [OB + t*kOStage, ...); both bases are multiples of the stage size.
  const long long EB = J0 / kEStage * kEStage;
  const long long OB = I0 / kOStage * kOStage;
  const long long ne_st = J1 > J0 ? (J1 - EB + kEStage - 1) / kEStage : 0;
  const long long no_st = (I1 + 1 - OB + kOStage - 1) / kOStage;

  if (warp == kProducerWarp) {
    // ------------------------------------------------------------ producer
    long long se = 0, so = 0;
    uint32_t spins = 0;
    while (se < ne_st || so < no_st) {
      bool progressed = false;
      if (se < ne_st) {
        const int slot = (int)(se % kEStages);
        const long long round = se / kEStages;
        int ok = round == 0;
        if (!ok && lane == 0) ok = mbar_test(&sm.empty_e[slot], (uint32_t)((round - 1) & 1));
        if (__shfl_sync(0xffffffffu, ok, 0)) {
          const long long st = EB + se * kEStage;
          const long long lo = st > J0 ? st : J0;  // never read before the CTA's first element
          const long long hi = st + kEStage < J1 ? st + kEStage : J1;
          produce_stage<Store, kEStage>(sm.ering, x, st, lo, hi, slot, &sm.full_e[slot],
                                        use_tma);
          se++;
          progressed = true;
        }
      }
      if (so < no_st) {
        const int slot = (int)(so % kOStages);
        const long long round = so / kOStages;
        int ok = round == 0;
        if (!ok && lane == 0) ok = mbar_test(&sm.empty_o[slot], (uint32_t)((round - 1) & 1));
        if (__shfl_sync(0xffffffffu, ok, 0)) {
          const long long st = OB + so * kOStage;
          const long long hi = st + kOStage < I1 + 1 ? st + kOStage : I1 + 1;
          produce_stage<int64_t, kOStage>(sm.oring, offsets, st, st, hi, slot, &sm.full_o[slot],
                                          use_tma);
          so++;
          progressed = true;
        }
      }
      if (progressed) {
        spins = 0;
      } else {
        if (++spins > kSpinLimit) {
          if (lane == 0) raise_error(err, inv, GB_MSG_TIMEOUT);
          break;
        }
        __nanosleep(64);
      }
    }
    return;
  }

  // -------------------------------------------------------------- consumers
  if (tid == 0) {
    sm.carry.acc = op.identity();
    sm.carry.flag = 0;
    sm.carry.pad = 0;
    sm.head_pending = offsets[I0] < J0 ? 1 : 0;  // list I0 has elements in earlier CTAs
  }
  long long ci = I0, cj = J0, cd = d_begin;
  int opos = (int)(I0 - OB);  // ring slot of offsets[ci]
  int xpos = (int)(J0 - EB);  // ring slot of content[cj]
  // stage bookkeeping (32-bit, incremental): next stage to wait for / release
  int we = 0, wo = 0, re_ = 0, ro = 0;
  const int ne = (int)ne_st, no = (int)no_st;
  long long rel_e_end = EB + kEStage, rel_o_end = OB + kOStage;
  bool timed_out = false;

  auto wait_full = [&](uint64_t* bars, int nst, int stage) {
    if (timed_out) return;  // after one expired wait, never wait again
    const int round = stage / nst;
    if (!mbar_wait(&bars[stage - round * nst], (uint32_t)(round & 1), 1u << 22)) timed_out = true;
  };
  auto seg = [&](const V& a, const V& bb) -> V {
    V r;
    r.flag = a.flag | bb.flag;
    r.acc = bb.flag ? bb.acc : op.combine(a.acc, bb.acc);
    r.pad = 0;
    return r;
  };
  V ident;
  ident.acc = op.identity();
  ident.flag = 0;
  ident.pad = 0;

  while (cd < d_end) {
    // windows (clamped at 0 so inconsistent offsets cannot index outside)
    const long long Lrem = I1 - ci;
    const int La = (int)(Lrem < 0 ? 0 : (Lrem < kOWin ? Lrem : kOWin));
    const long long Erem = J1 - cj;
    const int Ew = (int)(Erem < 0 ? 0 : (Erem < IPC ? Erem : IPC));
    // wait for the stages holding offsets[ci .. ci+La] and content[cj .. cj+Ew)
    {
      const int need_o = (int)((ci + La - OB) >> 8);  // kOStage = 256
      while (wo <= need_o && wo < no) wait_full(sm.full_o, kOStages, wo++);
      if (Ew > 0) {
        const int need_e = (int)((cj + Ew - 1 - EB) >> 10);  // kEStage = 1024
        while (we <= need_e && we < ne) wait_full(sm.full_e, kEStages, we++);
      }
    }
    // linear chunk-local list ends with a sentinel after the window
    for (int kk = tid; kk <= La; kk += kConsumers) {
      int v = kLendBig;
      if (kk < La) {
        int s = opos + 1 + kk;
        if (s >= RO) s -= RO;
        const long long rel = sm.oring[s] - cj;
        v = rel < kLendBig ? (int)rel : kLendBig;
      }
      sm.lend[kk] = v;
    }
    if (tid == 0) sm.lstart0 = sm.oring[opos] - cj;
    consumer_sync();
    // chunk length: at most IPC items, and never past the last visible list end
    int len = (int)(d_end - cd < IPC ? d_end - cd : IPC);
    if (La < Lrem && La > 0) {
      const long long lim = (long long)La + sm.lend[La - 1];
      if (lim < len) len = (int)(lim > 0 ? lim : 1);
    }
    const long long lstart0 = sm.lstart0;

    // this thread's items: local diagonal [dt, dt + nitems)
    const int dt = tid * IPT;
    const int nitems = dt < len ? (len - dt < IPT ? len - dt : IPT) : 0;
    int k = 0;
    if (nitems) {
      int lo = dt - Ew > 0 ? dt - Ew : 0;
      int hi = dt < La ? dt : La;
      while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (mid + sm.lend[mid] < dt) lo = mid + 1;
        else hi = mid;
      }
      k = lo < La ? lo : La;
    }
    int m = dt - k;
    Acc acc = op.identity();
    Acc head_acc = op.identity();
    bool has_end = false;
    int head_k = -1;
    for (int s = 0; s < nitems; s++) {
      if (sm.lend[k] <= m) {
        if (!has_end) {
          has_end = true;
          head_k = k;
          head_acc = acc;
        } else {
          out[ci + k] = op.finalize(acc, ci + k);
        }
        acc = op.identity();
        k++;
      } else {
        int xi = xpos + m;
        if (xi >= RE) xi -= RE;
        const Store v = sm.ering[xi];
        bool first = false;
        if (Op::kNeedsFirst) first = ((long long)m == (k == 0 ? lstart0 : (long long)sm.lend[k - 1]));
        acc = op.combine(acc, op.lift(v, cj + m, first, ci + k));
        m++;
      }
    }
    if (nitems && dt + nitems == len) sm.kend = k;  // state after the chunk's last item

    // block segmented scan of the thread tails (consumer warps only)
    V mine;
    mine.acc = acc;
    mine.flag = has_end ? 1u : 0u;
    mine.pad = 0;
    V incl = warp_inclusive_scan(mine, seg, ident);
    if (lane == 31) sm.scan[warp] = incl;
    consumer_sync();
    if (warp == 0) {
      V w = lane < kConsumers / 32 ? sm.scan[lane] : ident;
      V wi = warp_inclusive_scan(w, seg, ident);
      if (lane < kConsumers / 32) sm.scan[lane] = wi;
    }
    consumer_sync();
    V excl = shfl_up(incl, 1);
    if (lane == 0) excl = ident;
    if (warp > 0) excl = seg(sm.scan[warp - 1], excl);
    const V total = sm.scan[kConsumers / 32 - 1];
    const V carry = sm.carry;
    const V cin = seg(carry, excl);
    if (has_end) {
      const Acc whole = op.combine(cin.acc, head_acc);
      const long long list = ci + head_k;
      if (list == I0 && sm.head_pending) {
        records[b].head_list = I0;  // began in an earlier CTA: left to the fix-up
        records[b].head_acc = whole;
      } else {
        out[list] = op.finalize(whole, list);
      }
    }
    consumer_sync();
    const int kend = sm.kend;
    if (tid == 0) {
      sm.carry = seg(carry, total);
      if (total.flag) sm.head_pending = 0;
    }
    ci += kend;
    cj += len - kend;
    cd += len;
    opos += kend;
    if (opos >= RO) opos -= RO;
    xpos += len - kend;
    if (xpos >= RE) xpos -= RE;
    // hand fully consumed stages back to the producer
    while (re_ < we && rel_e_end <= cj) {
      if (tid == 0) mbar_arrive(&sm.empty_e[re_ % kEStages]);
      re_++;
      rel_e_end += kEStage;
    }
    while (ro < wo && rel_o_end <= ci) {
      if (tid == 0) mbar_arrive(&sm.empty_o[ro % kOStages]);
      ro++;
      rel_o_end += kOStage;
    }
    consumer_sync();
  }
  if (tid == 0) {
    records[b].tail_list = I1;
    records[b].tail_acc = sm.carry.acc;
    records[b].tail_fresh = (I1 < nlists) ? (offsets[I1] >= J0 ? 1 : 0) : 1;
  }
  // every issued stage completes before the CTA exits
  while (wo < no) wait_full(sm.full_o, kOStages, wo++);
  while (we < ne) wait_full(sm.full_e, kEStages, we++);
  if (timed_out && tid == 0) raise_error(err, inv, GB_MSG_TIMEOUT);
}

// One block: resolve lists that cross CTA boundaries, in CTA order.
template <class Op, int BLOCK>
__global__ void __launch_bounds__(BLOCK)
    seg_reduce_fixup_kernel(Op op, const int64_t* __restrict__ offsets, long long nlists,
                            typename Op::Out* __restrict__ out,
                            const CtaRecord<typename Op::Acc>* __restrict__ records, int G,
                            int ipc) {
  using V = SegVal<typename Op::Acc>;
  constexpr int NW = BLOCK / 32;
  __shared__ V scan_smem[NW + 1];
  __shared__ V running;
  const long long e0 = offsets[0];
  const long long eN = offsets[nlists];
  const long long E = eN > e0 ? eN - e0 : 0;
  const long long D = nlists + E;
  const int Geff = (int)((D + ipc - 1) / ipc < G ? (D + ipc - 1) / ipc : G);
  auto seg = [&](const V& a, const V& bb) -> V {
    V r;
    r.flag = a.flag | bb.flag;
    r.acc = bb.flag ? bb.acc : op.combine(a.acc, bb.acc);
    r.pad = 0;
    return r;
  };
  V ident;
  ident.acc = op.identity();
  ident.flag = 0;
  ident.pad = 0;
  if (threadIdx.x == 0) running = ident;
  __syncthreads();
  for (int base = 0; base < Geff; base += BLOCK) {
    const int c = base + threadIdx.x;
    V mine = ident;
    if (c < Geff) {
      const long long tl = records[c].tail_list;
      mine.acc = records[c].tail_acc;
      mine.flag = (c == 0 || records[c].tail_fresh || records[c - 1].tail_list != tl) ? 1u : 0u;
    }
    V total;
    V excl = block_exclusive_scan<BLOCK>(mine, seg, ident, scan_smem, &total);
    V before = seg(running, excl);  // scan through CTA c-1
    if (c < Geff && c > 0) {
      const long long hl = records[c].head_list;
      if (hl >= 0 && hl < nlists)
        out[hl] = op.finalize(op.combine(before.acc, records[c].head_acc), hl);
    }
    __syncthreads();
    if (threadIdx.x == 0) running = seg(running, total);
    __syncthreads();
  }
}

}  // namespace gb
