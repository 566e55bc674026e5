// reduce_ops.cuh -- reducer policies for seg_reduce_kernel and the launcher.
//
// A policy states one awkward-cpp reducer as (identity, lift, combine,
// finalize) with an ORDERED combine(earlier, later), so the parallel
// reduction reproduces the CPU loop's result:
//   sum/prod        awkward_reduce_sum.cpp:12-25, awkward_reduce_prod.cpp:12-25
//   sum_bool (any)  awkward_reduce_sum_bool.cpp:18-31
//   prod_bool (all) awkward_reduce_prod_bool.cpp:10-23
//   countnonzero    awkward_reduce_countnonzero.cpp:14-36
//   max/min         awkward_reduce_max.cpp:9-26, awkward_reduce_min.cpp:26-43
//   argmax/argmin   awkward_reduce_argmax.cpp:9-33, awkward_reduce_argmin.cpp:25-49
//   sumofsquares    awkward_reduce_sumofsquares.cpp:12-25
//   sumofpowers     awkward_reduce_sumofpowers.cpp:14-60
//   centered        awkward_reduce_centered_sumofsquares.cpp:15-29
#pragma once

#include <math.h>

#include <mutex>

#include "seg_reduce.cuh"

namespace gb {

template <class T>
__device__ __forceinline__ bool is_nan(T v) {
  if constexpr (std::is_floating_point<T>::value) return v != v;
  return false;
}

// Accumulator wider than 4 bytes for sub-word outputs (shuffles move 32-bit words).
template <class T>
using acc_word_t = typename std::conditional<
    (sizeof(T) >= 4), T,
    typename std::conditional<std::is_signed<T>::value, int32_t, uint32_t>::type>::type;

// acc = OUT{}; acc += (OUT)x   (integers wrap like the CPU loop)
template <class OUT, class IN>
struct SumOp {
  using In = IN;
  using Out = OUT;
  using Acc = OUT;
  static constexpr bool kNeedsFirst = false;
  __device__ Acc identity() const { return Acc(0); }
  __device__ Acc lift(store_t<IN> v, long long, bool, long long) const {
    if constexpr (std::is_same<IN, bool>::value) return Acc(v != 0 ? 1 : 0);
    else return static_cast<OUT>(v);
  }
  __device__ Acc combine(Acc a, Acc b) const { return a + b; }
  __device__ Out finalize(Acc a, long long) const { return a; }
};

// acc = (OUT)1; acc *= (OUT)x
template <class OUT, class IN>
struct ProdOp {
  using In = IN;
  using Out = OUT;
  using Acc = OUT;
  static constexpr bool kNeedsFirst = false;
  __device__ Acc identity() const { return Acc(1); }
  __device__ Acc lift(store_t<IN> v, long long, bool, long long) const {
    return static_cast<OUT>(v);
  }
  __device__ Acc combine(Acc a, Acc b) const { return a * b; }
  __device__ Out finalize(Acc a, long long) const { return a; }
};

// any(x != 0) / all(x != 0) into bool
template <class IN, bool ALL>
struct AnyAllOp {
  using In = IN;
  using Out = bool;
  using Acc = uint32_t;
  static constexpr bool kNeedsFirst = false;
  __device__ Acc identity() const { return ALL ? 1u : 0u; }
  __device__ Acc lift(store_t<IN> v, long long, bool, long long) const {
    return v != 0 ? 1u : 0u;
  }
  __device__ Acc combine(Acc a, Acc b) const { return ALL ? (a & b) : (a | b); }
  __device__ Out finalize(Acc a, long long) const { return a != 0; }
};

// count of x != 0 into int64
template <class IN>
struct CountNonzeroOp {
  using In = IN;
  using Out = int64_t;
  using Acc = int64_t;
  static constexpr bool kNeedsFirst = false;
  __device__ Acc identity() const { return 0; }
  __device__ Acc lift(store_t<IN> v, long long, bool, long long) const { return v != 0 ? 1 : 0; }
  __device__ Acc combine(Acc a, Acc b) const { return a + b; }
  __device__ Out finalize(Acc a, long long) const { return a; }
};

// best = identity; best = (v > best) ? v : best   (or <).  The partial of a
// range is its earliest extremal non-NaN element; ties keep the earlier one
// (this preserves the sign of zero); the identity precedes every element.
template <class T, bool MAX>
struct ExtremumOp {
  using In = T;
  using Out = T;
  struct Acc {
    acc_word_t<T> v;
    uint32_t valid;
  };
  static constexpr bool kNeedsFirst = false;
  T ident;
  __device__ static bool better(T b, T a) { return MAX ? (b > a) : (b < a); }
  __device__ Acc identity() const { return Acc{acc_word_t<T>(0), 0u}; }
  __device__ Acc lift(T v, long long, bool, long long) const {
    return Acc{static_cast<acc_word_t<T>>(v), is_nan(v) ? 0u : 1u};
  }
  __device__ Acc combine(Acc a, Acc b) const {
    if (b.valid && (!a.valid || better(static_cast<T>(b.v), static_cast<T>(a.v)))) return b;
    return a;
  }
  __device__ Out finalize(Acc a, long long) const {
    return (a.valid && better(static_cast<T>(a.v), ident)) ? static_cast<T>(a.v) : ident;
  }
};

// Global index of the first extremum; -1 if empty.  The list's first
// element is always a candidate (a leading NaN wins, as in the CPU loop that
// seeds best = start); later NaNs never win.
template <class T, bool MAX>
struct ArgExtremumOp {
  using In = T;
  using Out = int64_t;
  struct Acc {
    acc_word_t<T> v;
    uint32_t pad;
    long long idx;
  };
  static constexpr bool kNeedsFirst = true;
  __device__ static bool better(T b, T a) { return MAX ? (b > a) : (b < a); }
  __device__ Acc identity() const { return Acc{acc_word_t<T>(0), 0u, -1}; }
  __device__ Acc lift(T v, long long j, bool first, long long) const {
    if (!first && is_nan(v)) return identity();
    return Acc{static_cast<acc_word_t<T>>(v), 0u, j};
  }
  __device__ Acc combine(Acc a, Acc b) const {
    if (a.idx < 0) return b;
    if (b.idx < 0) return a;
    if (is_nan(static_cast<T>(a.v))) return a;
    return better(static_cast<T>(b.v), static_cast<T>(a.v)) ? b : a;
  }
  __device__ Out finalize(Acc a, long long) const { return a.idx; }
};

template <class IN>
struct SumSqOp {
  using In = IN;
  using Out = double;
  using Acc = double;
  static constexpr bool kNeedsFirst = false;
  __device__ Acc identity() const { return 0.0; }
  __device__ Acc lift(store_t<IN> v, long long, bool, long long) const {
    double d = static_cast<double>(v);
    return d * d;
  }
  __device__ Acc combine(Acc a, Acc b) const { return a + b; }
  __device__ Out finalize(Acc a, long long) const { return a; }
};

// Integer power by binary exponentiation (exponent bits low to high, as the
// CPU loop does); pow() for negative exponents.
__device__ __forceinline__ double ipow_binary(double base, long long n) {
  if (n < 0) return pow(base, static_cast<double>(n));
  double result = 1.0, b = base;
  long long e = n;
  while (e > 0) {
    if (e & 1) result *= b;
    e >>= 1;
    if (e > 0) b *= b;
  }
  return result;
}

template <class IN>
struct SumPowOp {
  using In = IN;
  using Out = double;
  using Acc = double;
  static constexpr bool kNeedsFirst = false;
  long long n;
  __device__ Acc identity() const { return 0.0; }
  __device__ Acc lift(store_t<IN> v, long long, bool, long long) const {
    return ipow_binary(static_cast<double>(v), n);
  }
  __device__ Acc combine(Acc a, Acc b) const { return a + b; }
  __device__ Out finalize(Acc a, long long) const { return a; }
};

template <class IN>
struct CenteredSumSqOp {
  using In = IN;
  using Out = double;
  using Acc = double;
  static constexpr bool kNeedsFirst = false;
  const double* means;
  __device__ Acc identity() const { return 0.0; }
  __device__ Acc lift(store_t<IN> v, long long, bool, long long list) const {
    double d = static_cast<double>(v) - means[list];
    return d * d;
  }
  __device__ Acc combine(Acc a, Acc b) const { return a + b; }
  __device__ Out finalize(Acc a, long long) const { return a; }
};

// ---------------------------------------------------------------- launcher
constexpr int kFixupBlock = 1024;

template <class Op>
struct SegReduceConfig {
  using Sm = SegSmem<store_t<typename Op::In>, typename Op::Acc>;
  static int blocks_per_sm() {
    static std::once_flag once;
    static int bps = 1;
    std::call_once(once, [] {
      auto k = seg_reduce_kernel<Op>;
      cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(Sm));
      int n = 0;
      if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, kSegThreads, sizeof(Sm)) !=
              cudaSuccess ||
          n < 1)
        n = 1;
      bps = n;
    });
    return bps;
  }
};

// Launch the segmented reduction of `nlists` lists on `stream`: the
// persistent merge-path kernel, then the one-block cross-CTA fix-up.
// Returns the launch status; data never travel to the host.
template <class Op>
cudaError_t launch_seg_reduce(const Op& op, const store_t<typename Op::In>* x,
                              const int64_t* offsets, long long nlists, typename Op::Out* out,
                              uint64_t inv, uint64_t* err, cudaStream_t stream,
                              int grid_override = 0) {
  if (nlists <= 0) return cudaSuccess;
  using Rec = CtaRecord<typename Op::Acc>;
  using Sm = typename SegReduceConfig<Op>::Sm;
  const int G = grid_override > 0 ? grid_override
                                  : device_sm_count() * SegReduceConfig<Op>::blocks_per_sm();
  void* rec = nullptr;
  cudaError_t e = scratch_alloc(&rec, (size_t)G * sizeof(Rec), stream);
  if (e != cudaSuccess) return e;
  const int use_tma = ((reinterpret_cast<uintptr_t>(x) | reinterpret_cast<uintptr_t>(offsets)) &
                       15) == 0;
  seg_reduce_kernel<Op><<<G, kSegThreads, sizeof(Sm), stream>>>(
      op, x, offsets, nlists, out, reinterpret_cast<Rec*>(rec), G, use_tma, inv, err);
  e = cudaGetLastError();
  if (e == cudaSuccess) {
    seg_reduce_fixup_kernel<Op, kFixupBlock><<<1, kFixupBlock, 0, stream>>>(
        op, offsets, nlists, out, reinterpret_cast<const Rec*>(rec), G, kSegIPC);
    e = cudaGetLastError();
  }
  cudaError_t f = scratch_free(rec, stream);
  return e != cudaSuccess ? e : f;
}

}  // namespace gb
