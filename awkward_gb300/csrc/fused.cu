// fused.cu -- an elementwise map fused into the float64 segmented reduction.
//
// awkward evaluates ak.sum(x * y, axis=-1) as two kernels: the product is
// materialised in device memory by an elementwise kernel, then the segmented
// reducer reads it back (and its lazy backend fuses the chain into
// cuda.compute iterators, src/awkward/_connect/lazy/_fusion.py:493).  Here the
// map is applied inside the reducer's load path, so x and y are each read once
// and nothing is written but the per-list results.
//
// Maps: x, x*y, x*x, |x| (products rounded once, as an elementwise kernel
// rounds them).  Reductions: sum (the fixed-point sum of the reducers), max,
// min (identity -inf / +inf), argmax, argmin (global element indices, -1 for
// empty lists) -- each equal to materialising the mapped values and calling
// awkward_reduce_* on them: bit for bit for max/min/argmax/argmin, and within
// the reducers' bound for sums.
//
// Layout: a warp walks its merge-path range 32 lists per round (as
// seg_reduce_kernel).  When a round's lists are whole, short (<= 32
// elements) and their span fits the warp's stage, the 32 lanes compute the
// mapped values of the whole span together -- coalesced loads, and every
// float64 multiply on a converged warp (GB300's float64 unit is narrow) --
// into the stage in shared memory, and each lane then reduces its list from
// the stage with the reducers' short-run arithmetic.  Other rounds (long
// lists, the lists crossing the range ends) map on the fly: short lists by
// their lane, long ones by the whole warp, the giant list crossing a range
// end into the range records that seg_reduce_fixup_kernel combines.
#include "reduce_ops.cuh"

using namespace gb;

namespace {

constexpr int kFuseBlock = 256;
constexpr int kFuseStage = 512;  // mapped values staged per warp and round

enum : int { kMapX = 0, kMapXY = 1, kMapXX = 2, kMapAbs = 3 };

template <int MAP>
__device__ __forceinline__ double map_at(const double* __restrict__ x,
                                         const double* __restrict__ y, long long j) {
  const double a = __ldg(x + j);
  if constexpr (MAP == kMapXY) return __dmul_rn(a, __ldg(y + j));
  else if constexpr (MAP == kMapXX) return __dmul_rn(a, a);
  else if constexpr (MAP == kMapAbs) return __longlong_as_double(__double_as_longlong(a) & 0x7fffffffffffffffLL);
  else return a;
}

template <class Op, int MAP>
__global__ void __launch_bounds__(kFuseBlock)
    fused_reduce_kernel(Op op, const double* __restrict__ x, const double* __restrict__ y,
                        const int64_t* __restrict__ offsets, long long nlists,
                        typename Op::Out* __restrict__ out, RangeRecord<typename Op::Acc>* records,
                        int W) {
  using Acc = typename Op::Acc;
  __shared__ double stage[kFuseBlock / 32][kFuseStage];
  double* sw = stage[threadIdx.x >> 5];
  const int lane = threadIdx.x & 31;
  const int w = (int)((blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5);
  const long long e0 = __ldg(offsets);
  const long long eN = __ldg(offsets + nlists);
  const long long E = eN > e0 ? eN - e0 : 0;
  const long long D = nlists + E;
  const int Weff = seg_ranges(nlists, E, W);
  if (w >= Weff) return;
  const long long d0 = D * w / Weff, d1 = D * (w + 1) / Weff;
  RangeRecord<Acc>& rec = records[w];
  const bool upper = lane >= 16;
  const long long split = mp_search_half(offsets, nlists, e0, E, upper ? d1 : d0,
                                         upper ? 0xffff0000u : 0x0000ffffu);
  const long long I0 = __shfl_sync(0xffffffffu, split, 0);
  const long long I1 = __shfl_sync(0xffffffffu, split, 16);
  const long long J0 = e0 + (d0 - I0), J1 = e0 + (d1 - I1);
  const long long last_list = I1 < nlists ? I1 : I1 - 1;  // I1 itself is the tail, if any
  long long carry = __ldg(offsets + I0);
  for (long long base = I0; base <= last_list; base += 32) {
    const long long li = base + lane;
    const bool act = li <= last_list;
    const long long en = __ldg(offsets + (act ? li : last_list) + 1);
    long long st = __shfl_up_sync(0xffffffffu, en, 1);
    if (lane == 0) st = carry;
    carry = __shfl_sync(0xffffffffu, en, 31);
    const long long n = en - st;
    const bool plain = li != I1 && (unsigned long long)n <= (unsigned long long)kShortList;
    const unsigned acts = __ballot_sync(0xffffffffu, act);
    const long long lo = __shfl_sync(0xffffffffu, st, 0);
    const long long hi = __shfl_sync(0xffffffffu, en, 31 - __clz(acts));
    if (__all_sync(0xffffffffu, !act || plain) && hi - lo <= kFuseStage && hi >= lo) {
      const int span = (int)(hi - lo);
      for (int j = lane; j < span; j += 32) sw[j] = map_at<MAP>(x, y, lo + j);
      __syncwarp();
      if (act) {
        const int m = (int)n;
        out[li] = op.finalize(run_short(op, sw + (st - lo), m, st, st, li, LdShared{}), li);
      }
      __syncwarp();
      continue;
    }
    // general round: map on the fly
    long long s0 = 0, e = 0;
    bool skip = false;
    if (act) {
      const bool small = n <= kAbsorb;  // reduced whole by the range where it ends
      s0 = (st < J0 && !small) ? J0 : st;
      e = li == I1 ? J1 : en;
      skip = li == I1 && small;
      if (e < s0) e = s0;
    }
    const bool run = act && !skip;
    Acc acc = op.identity();
    if (run && e - s0 <= kShortList)
      for (long long j = s0; j < e; j++) acc = op.step(acc, map_at<MAP>(x, y, j), j, j == st, li);
    unsigned longl = __ballot_sync(0xffffffffu, run && e - s0 > kShortList);
    while (longl) {  // the whole warp on one long list, strided (coalesced)
      const int src = __ffs(longl) - 1;
      longl &= longl - 1;
      const long long s2 = __shfl_sync(0xffffffffu, s0, src);
      const long long e2 = __shfl_sync(0xffffffffu, e, src);
      const long long st2 = __shfl_sync(0xffffffffu, st, src);
      const long long l2 = base + src;
      Acc a2 = op.identity();
      for (long long j = s2 + lane; j < e2; j += 32) a2 = op.step(a2, map_at<MAP>(x, y, j), j, j == st2, l2);
      a2 = group_allreduce<32>(op, a2);
      if (lane == src) acc = a2;
    }
    if (run) {
      if (li == I1) rec.tail_acc = acc;         // a giant list continues in the next range
      else if (s0 > st) rec.head_acc = acc;     // the end of a giant list that began earlier
      else out[li] = op.finalize(acc, li);
    }
  }
  if (lane == 0) seg_range_records(op, offsets, nlists, I0, I1, J0, rec);
}

template <class Op, int MAP>
cudaError_t launch_fused(const Op& op, const double* x, const double* y, const int64_t* offsets,
                         long long nlists, typename Op::Out* out, cudaStream_t stream) {
  using Rec = RangeRecord<typename Op::Acc>;
  int bps = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
      &bps, fused_reduce_kernel<Op, MAP>, kFuseBlock, 0);
  if (e != cudaSuccess) return e;
  if (bps < 1) bps = 1;
  const int blocks = device_sm_count() * bps;
  const int W = blocks * (kFuseBlock / 32);
  void* rec = nullptr;
  e = scratch_alloc(&rec, (size_t)W * sizeof(Rec), stream);
  if (e != cudaSuccess) return e;
  fused_reduce_kernel<Op, MAP><<<blocks, kFuseBlock, 0, stream>>>(
      op, x, y, offsets, nlists, out, reinterpret_cast<Rec*>(rec), W);
  e = cudaGetLastError();
  if (e == cudaSuccess) {
    seg_reduce_fixup_kernel<Op><<<(W + 255) / 256, 256, 0, stream>>>(
        op, offsets, nlists, out, reinterpret_cast<const Rec*>(rec), W);
    e = cudaGetLastError();
  }
  cudaError_t f = scratch_free(rec, stream);
  return e != cudaSuccess ? e : f;
}

template <class Op>
cudaError_t fused_by_map(const Op& op, int map, const double* x, const double* y,
                         const int64_t* offsets, long long nlists, typename Op::Out* out,
                         cudaStream_t s) {
  switch (map) {
    case kMapX: return launch_fused<Op, kMapX>(op, x, y, offsets, nlists, out, s);
    case kMapXY: return launch_fused<Op, kMapXY>(op, x, y, offsets, nlists, out, s);
    case kMapXX: return launch_fused<Op, kMapXX>(op, x, y, offsets, nlists, out, s);
    default: return launch_fused<Op, kMapAbs>(op, x, y, offsets, nlists, out, s);
  }
}

}  // namespace

GB_EXPORT int awkward_gb300_fused_reduce_float64(void* out, const double* x, const double* y,
                                                 const int64_t* offsets, int64_t nlists,
                                                 int64_t map, int64_t reduce,
                                                 uint64_t invocation_index, uint64_t* err_code,
                                                 void* stream) {
  (void)invocation_index;
  (void)err_code;
  if (map < kMapX || map > kMapAbs || reduce < 0 || reduce > 4) return (int)cudaErrorInvalidValue;
  if (map == kMapXY && y == nullptr) return (int)cudaErrorInvalidValue;
  if (nlists <= 0) return (int)cudaSuccess;
  cudaStream_t s = (cudaStream_t)stream;
  const int m = (int)map;
  switch (reduce) {
    case 0:
      return (int)fused_by_map(FixedSumOp<double>{}, m, x, y, offsets, nlists,
                               static_cast<double*>(out), s);
    case 1: {
      ExtremumOp<double, true> op;
      op.ident = -__builtin_inf();
      return (int)fused_by_map(op, m, x, y, offsets, nlists, static_cast<double*>(out), s);
    }
    case 2: {
      ExtremumOp<double, false> op;
      op.ident = __builtin_inf();
      return (int)fused_by_map(op, m, x, y, offsets, nlists, static_cast<double*>(out), s);
    }
    case 3:
      return (int)fused_by_map(ArgExtremumOp<double, true>{}, m, x, y, offsets, nlists,
                               static_cast<int64_t*>(out), s);
    default:
      return (int)fused_by_map(ArgExtremumOp<double, false>{}, m, x, y, offsets, nlists,
                               static_cast<int64_t*>(out), s);
  }
}
