// reduce_ops.cuh -- reducer policies for seg_reduce_kernel and the launcher.
//
// A policy states one awkward-cpp reducer as (identity, lift, combine,
// finalize).  Every combine is commutative and associative (extremum
// reducers carry the element index and resolve ties to the lowest index),
// so any reduction order reproduces the CPU loop's result exactly, except
// for floating-point rounding of sums and products:
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

// This GPU executes float64 arithmetic AND comparisons on a narrow pipe
// (about 1/64 of float32), so the float64 reducers below keep most per-element
// work off it: comparisons go through an integer total-order key, and sums
// split each short run between the float64 unit (even positions, one add
// each) and a fixed-point accumulator on the integer pipe (odd positions;
// addend bits below the anchor's unit truncated, the total rounded once:
// within n*eps*sum|x| of the exact sum).
template <class T>
__device__ __forceinline__ bool is_nan(T v) {
  if constexpr (std::is_same<T, double>::value) {
    return (__double_as_longlong(v) & 0x7fffffffffffffffLL) > 0x7ff0000000000000LL;
  } else if constexpr (std::is_floating_point<T>::value) {
    return v != v;
  }
  return false;
}

// Integer key with the numeric order of non-NaN doubles; -0.0 and +0.0 share
// key 0 (they compare equal, as in C).
__device__ __forceinline__ long long f64_key(double v) {
  const long long b = __double_as_longlong(v);
  if ((b & 0x7fffffffffffffffLL) == 0) return 0;
  return b >= 0 ? b : (b ^ 0x7fffffffffffffffLL);
}

// b > a (MAX) or b < a (MIN) with C semantics: false if either is NaN.
template <class T, bool MAX>
__device__ __forceinline__ bool num_better(T b, T a) {
  if constexpr (std::is_same<T, double>::value) {
    if (is_nan(a) || is_nan(b)) return false;
    const long long kb = f64_key(b), ka = f64_key(a);
    return MAX ? (kb > ka) : (kb < ka);
  } else {
    return MAX ? (b > a) : (b < a);
  }
}

// ---------------------------------------------------------------- fixed-point sum
// Fixed-point accumulator for float64 sums on the integer pipe: the value is
// acc * 2^(anchor - 1075); every addend's 53-bit significand is aligned to the
// anchor (the largest exponent seen; bits below the anchor's unit are
// truncated, < 1 unit each) and |acc| is kept below 2^62 by raising the anchor.
// A float64 partial `dp` (the even positions of short runs, added on the
// FP64 unit) rides along and is added once, in float64, at the end.
// finalize() rounds the fixed-point total to nearest-even once, then adds dp.
// Infinities and NaNs are tracked in `flags` with IEEE semantics (NaN
// absorbs; +inf + -inf = NaN), and in dp by the float64 addition itself.
struct FxAcc {
  long long acc;
  int anchor;  // >= 1 (1 is the subnormal scale)
  int flags;   // 1 NaN, 2 +inf, 4 -inf
  double dp;   // float64 partial, added last
};

__device__ __forceinline__ FxAcc fx_norm(FxAcc a) {
  if ((a.acc ^ (a.acc >> 63)) >= (1LL << 62)) {
    a.acc >>= 1;
    a.anchor += 1;
  }
  return a;
}

// add (-1)^neg * m * 2^(ee - 1075), m < 2^53, ee >= 1
__device__ __forceinline__ FxAcc fx_add(FxAcc a, bool neg, long long m, int ee) {
  if (ee > a.anchor) {
    const int sh = ee - a.anchor;
    a.acc = sh >= 63 ? (a.acc >> 63) : (a.acc >> sh);
    a.anchor = ee;
  }
  const int d = a.anchor - ee;
  const long long t = d >= 63 ? 0 : (m >> d);
  a.acc += neg ? -t : t;
  return fx_norm(a);
}

__device__ __forceinline__ FxAcc fx_add_f64(FxAcc a, double v) {
  const long long b = __double_as_longlong(v);
  const int e = (int)((b >> 52) & 0x7ff);
  if (e == 0x7ff) {
    a.flags |= (b & 0xfffffffffffffLL) ? 1 : (b < 0 ? 4 : 2);
    return a;
  }
  const long long m = (b & 0xfffffffffffffLL) | (e ? (1LL << 52) : 0);
  return fx_add(a, b < 0, m, e ? e : 1);
}

__device__ __forceinline__ FxAcc fx_add_f32(FxAcc a, float v) {
  const int b = __float_as_int(v);
  const int e = (b >> 23) & 0xff;
  if (e == 0xff) {
    a.flags |= (b & 0x7fffff) ? 1 : (b < 0 ? 4 : 2);
    return a;
  }
  const long long m = (long long)((b & 0x7fffff) | (e ? (1 << 23) : 0)) << 29;
  return fx_add(a, b < 0, m, (e ? e : 1) + 896);  // float exponent -> double anchor scale
}

__device__ __forceinline__ FxAcc fx_combine(FxAcc a, FxAcc b) {
  if (a.anchor < b.anchor) {
    FxAcc t = a;
    a = b;
    b = t;
  }
  const int sh = a.anchor - b.anchor;
  a.acc += sh >= 63 ? (b.acc >> 63) : (b.acc >> sh);
  a.flags |= b.flags;
  a.dp += b.dp;
  return fx_norm(a);
}

// The fixed-point part acc * 2^(anchor - 1075) rounded to nearest-even.
__device__ __forceinline__ double fx_fixed_value(FxAcc a) {
  if ((a.flags & 1) || (a.flags & 6) == 6) return __longlong_as_double(0x7ff8000000000000LL);
  if (a.flags & 2) return __longlong_as_double(0x7ff0000000000000LL);
  if (a.flags & 4) return __longlong_as_double((long long)0xfff0000000000000ULL);
  if (a.acc == 0) return 0.0;
  if (a.anchor >= 53 && a.anchor <= 1970) {
    // |acc| >= 1 and < 2^63: the scaled value is a normal double, so the
    // integer's correctly rounded conversion scaled by adding to its exponent
    // field is the rounded value (the same bits as the general path below)
    const long long c = __double_as_longlong(__ll2double_rn(a.acc));
    return __longlong_as_double(c + ((long long)(a.anchor - 1075) << 52));
  }
  const unsigned long long sign = a.acc < 0 ? 0x8000000000000000ULL : 0ULL;
  unsigned long long mag = a.acc < 0 ? (unsigned long long)(-a.acc) : (unsigned long long)a.acc;
  const int p = 63 - __clzll((long long)mag);  // leading bit of mag
  long long biased = (long long)p + a.anchor - 52;
  unsigned long long q;
  if (p > 52) {
    const int sh = p - 52;
    q = mag >> sh;
    const unsigned long long rem = mag & ((1ULL << sh) - 1), half = 1ULL << (sh - 1);
    if (rem > half || (rem == half && (q & 1))) q++;
    if (q == (1ULL << 53)) {
      q >>= 1;
      biased++;
    }
  } else {
    q = mag << (52 - p);
  }
  if (biased >= 2047) return __longlong_as_double((long long)(sign | 0x7ff0000000000000ULL));
  if (biased <= 0) {
    // subnormal: the value is mag * 2^(anchor-1075) with anchor small enough
    // that mag << (anchor - 1) is the exact subnormal significand
    return __longlong_as_double((long long)(sign | (mag << (a.anchor - 1))));
  }
  return __longlong_as_double(
      (long long)(sign | ((unsigned long long)biased << 52) | (q & 0xfffffffffffffULL)));
}

__device__ __forceinline__ double fx_finalize(FxAcc a) { return fx_fixed_value(a) + a.dp; }

// Sum of float64 (or float32) into float64 on the integer pipe in fixed
// point, rounded once at the end (runs of at most 32 elements also add half
// their elements in float64, see run_short); within n*eps*sum|x| of the exact
// sum, like the CPU loop that rounds after every addition.
template <class IN>
struct FixedSumOp {
  using In = IN;
  using Out = double;
  using Acc = FxAcc;
  static constexpr bool kNeedsFirst = false;
  __device__ Acc identity() const { return FxAcc{0, 1, 0}; }
  __device__ Acc lift(IN v, long long, bool, long long) const { return step(identity(), v, 0, false, 0); }
  __device__ Acc combine(Acc a, Acc b) const { return fx_combine(a, b); }
  __device__ Acc step(Acc a, IN v, long long, bool, long long) const {
    if constexpr (std::is_same<IN, double>::value) return fx_add_f64(a, v);
    else return fx_add_f32(a, v);
  }
  __device__ Out finalize(Acc a, long long) const { return fx_finalize(a); }
};

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
  __device__ Acc step(Acc a, store_t<IN> v, long long j, bool f, long long) const {
    return a + lift(v, j, f, 0);
  }
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
  __device__ Acc step(Acc a, store_t<IN> v, long long, bool, long long) const {
    return a * static_cast<OUT>(v);
  }
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
  __device__ Acc step(Acc a, store_t<IN> v, long long, bool, long long) const {
    return ALL ? (a & (v != 0 ? 1u : 0u)) : (a | (v != 0 ? 1u : 0u));
  }
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
  __device__ Acc step(Acc a, store_t<IN> v, long long, bool, long long) const { return a + (v != 0 ? 1 : 0); }
  __device__ Out finalize(Acc a, long long) const { return a; }
};

// best = identity; best = (v > best) ? v : best   (or <).  The partial of a
// range is its extremal non-NaN element, ties resolved to the lowest index
// (this keeps the CPU's first occurrence, e.g. the sign of a zero), so the
// combine is commutative and any reduction order gives the CPU's answer;
// the identity precedes every element.
template <class T, bool MAX>
struct ExtremumOp {
  using In = T;
  using Out = T;
  struct Acc {
    acc_word_t<T> v;
    long long idx;  // -1: no candidate yet
  };
  static constexpr bool kNeedsFirst = false;
  T ident;
  __device__ static bool better(T b, T a) { return num_better<T, MAX>(b, a); }
  __device__ Acc identity() const { return Acc{acc_word_t<T>(0), -1}; }
  __device__ Acc lift(T v, long long j, bool, long long) const {
    return Acc{static_cast<acc_word_t<T>>(v), is_nan(v) ? -1 : j};
  }
  __device__ Acc combine(Acc a, Acc b) const {
    if (b.idx < 0) return a;
    if (a.idx < 0) return b;
    const T av = static_cast<T>(a.v), bv = static_cast<T>(b.v);
    if (better(bv, av)) return b;
    if (better(av, bv)) return a;
    return b.idx < a.idx ? b : a;
  }
  // one element after all earlier ones (the CPU loop's update; NaN never wins)
  __device__ Acc step(Acc a, T v, long long j, bool, long long) const {
    if (!is_nan(v) && (a.idx < 0 || better(v, static_cast<T>(a.v))))
      a = Acc{static_cast<acc_word_t<T>>(v), j};
    return a;
  }
  __device__ Out finalize(Acc a, long long) const {
    return (a.idx >= 0 && better(static_cast<T>(a.v), ident)) ? static_cast<T>(a.v) : ident;
  }
};

// Global index of the first extremum; -1 if empty.  The list's first
// element is always a candidate and wins when it is NaN (the CPU loop seeds
// best = start and NaN never compares greater); later NaNs never win; ties
// go to the lowest index.  Commutative, like ExtremumOp.
template <class T, bool MAX>
struct ArgExtremumOp {
  using In = T;
  using Out = int64_t;
  struct Acc {
    acc_word_t<T> v;
    long long idx;  // -1: empty
  };
  static constexpr bool kNeedsFirst = true;
  __device__ static bool better(T b, T a) { return num_better<T, MAX>(b, a); }
  __device__ Acc identity() const { return Acc{acc_word_t<T>(0), -1}; }
  __device__ Acc lift(T v, long long j, bool first, long long) const {
    if (!first && is_nan(v)) return identity();
    return Acc{static_cast<acc_word_t<T>>(v), j};
  }
  __device__ Acc combine(Acc a, Acc b) const {
    if (a.idx < 0) return b;
    if (b.idx < 0) return a;
    const T av = static_cast<T>(a.v), bv = static_cast<T>(b.v);
    if (is_nan(av)) return a;  // only a list's leading element can be a NaN candidate
    if (is_nan(bv)) return b;
    if (better(bv, av)) return b;
    if (better(av, bv)) return a;
    return b.idx < a.idx ? b : a;
  }
  // one element after all earlier ones: the CPU loop's update
  __device__ Acc step(Acc a, T v, long long j, bool first, long long) const {
    if (a.idx < 0) {
      if (first || !is_nan(v)) a = Acc{static_cast<acc_word_t<T>>(v), j};
    } else if (better(v, static_cast<T>(a.v))) {
      a = Acc{static_cast<acc_word_t<T>>(v), j};
    }
    return a;
  }
  __device__ Out finalize(Acc a, long long) const { return a.idx; }
};

// ---------------------------------------------------------------- float64 keys
// Float64 extremum reducers on the integer pipe.  k(v) is the order key of
// f64_key, reversed (~) for MIN so both directions maximise; NaN gets the
// lowest key (never selected), except a list's leading element in the
// arg-reducers, which gets the highest (it stays selected, as in the CPU loop).
template <bool MAX>
__device__ __forceinline__ long long f64_dir_key(double v) {
  const long long k = f64_key(v);
  return MAX ? k : ~k;
}
constexpr long long kKeyLow = (long long)0x8000000000000000ULL;
constexpr long long kKeyHigh = 0x7fffffffffffffffLL;

template <bool MAX>
struct ExtremumOp<double, MAX> {
  using In = double;
  using Out = double;
  struct Acc {
    long long key;
    long long bits;
    long long idx;  // -1: no candidate yet
  };
  static constexpr bool kNeedsFirst = false;
  double ident;
  __device__ Acc identity() const { return Acc{kKeyLow, 0, -1}; }
  __device__ Acc lift(double v, long long j, bool, long long) const {
    if (is_nan(v)) return identity();
    return Acc{f64_dir_key<MAX>(v), __double_as_longlong(v), j};
  }
  __device__ Acc combine(Acc a, Acc b) const {
    if (b.idx < 0) return a;
    if (a.idx < 0) return b;
    if (b.key != a.key) return b.key > a.key ? b : a;
    return b.idx < a.idx ? b : a;
  }
  __device__ Acc step(Acc a, double v, long long j, bool, long long) const {
    if (!is_nan(v)) {
      const long long k = f64_dir_key<MAX>(v);
      if (a.idx < 0 || k > a.key) a = Acc{k, __double_as_longlong(v), j};
    }
    return a;
  }
  __device__ Out finalize(Acc a, long long) const {
    if (a.idx < 0 || is_nan(ident)) return ident;
    return a.key > f64_dir_key<MAX>(ident) ? __longlong_as_double(a.bits) : ident;
  }
};

template <bool MAX>
struct ArgExtremumOp<double, MAX> {
  using In = double;
  using Out = int64_t;
  struct Acc {
    long long key;
    long long idx;  // -1: empty
  };
  static constexpr bool kNeedsFirst = true;
  __device__ Acc identity() const { return Acc{kKeyLow, -1}; }
  __device__ static long long k_of(double v, bool first) {
    return is_nan(v) ? (first ? kKeyHigh : kKeyLow) : f64_dir_key<MAX>(v);
  }
  __device__ Acc lift(double v, long long j, bool first, long long) const {
    const long long k = k_of(v, first);
    return k == kKeyLow ? identity() : Acc{k, j};
  }
  __device__ Acc combine(Acc a, Acc b) const {
    if (b.idx < 0) return a;
    if (a.idx < 0) return b;
    if (b.key != a.key) return b.key > a.key ? b : a;
    return b.idx < a.idx ? b : a;
  }
  __device__ Acc step(Acc a, double v, long long j, bool first, long long) const {
    const long long k = k_of(v, first);
    if (k > a.key) a = Acc{k, j};
    return a;
  }
  __device__ Out finalize(Acc a, long long) const { return a.idx; }
};

// Put the later cache sectors of a short run in flight before its loop walks
// them (loads whose results are never read: nothing waits for them, so the
// misses overlap instead of following one another).
#pragma nv_diag_suppress 550  // the touch loads' destination is never read, by design
__device__ __forceinline__ void touch_run(const void* p, int n, int esize) {
  const char* c = reinterpret_cast<const char*>(p);
  long long d;
  if (n > 4) asm volatile("ld.global.nc.b64 %0, [%1];" : "=l"(d) : "l"(c + 4 * esize));
  if (n > 8) asm volatile("ld.global.nc.b64 %0, [%1];" : "=l"(d) : "l"(c + 8 * esize));
  if (n > 12) asm volatile("ld.global.nc.b64 %0, [%1];" : "=l"(d) : "l"(c + 12 * esize));
}
#pragma nv_diag_default 550

// ---------------------------------------------------------------- short runs
// Element loaders of the short-run reducers: global memory through the
// read-only path (with "touch" loads that put a run's later sectors in
// flight), or a run staged in shared memory.  Both give the same arithmetic.
struct LdGlobal {
  static constexpr bool kTouch = true;
  template <class T>
  __device__ __forceinline__ T operator()(const T* p) const {
    return __ldg(p);
  }
};
struct LdShared {
  static constexpr bool kTouch = false;
  template <class T>
  __device__ __forceinline__ T operator()(const T* p) const {
    return *p;
  }
};

// Reduce n consecutive elements p[0..n) (global indices j0..j0+n) of one
// list into a fresh accumulator, elements read by `ld`.  The default steps
// element by element.
template <class Op, class Ld = LdGlobal>
__device__ __forceinline__ typename Op::Acc run_short(const Op& op,
                                                      const store_t<typename Op::In>* p, int n,
                                                      long long j0, long long st, long long li,
                                                      Ld ld = Ld{}) {
  typename Op::Acc a = op.identity();
  for (int i = 0; i < n; i++) a = op.step(a, ld(p + i), j0 + i, j0 + i == st, li);
  return a;
}

// Float64 max/min of a short run, fast path: the raw key b ^ ((b >> 63) &
// 0x7ff..f) orders all non-NaN doubles except that it puts -0.0 below +0.0,
// and it puts positive NaNs above +inf (negative NaNs below -inf).  The loop
// uses it unconditioned; if the winner is a zero or a NaN (rare) the run is
// redone with the exact step, which resolves ties to the first occurrence and
// never selects a NaN.
__device__ __forceinline__ long long f64_raw_key(long long b) {
  return b ^ ((long long)((unsigned long long)b >> 63) * 0x7fffffffffffffffLL);
}
__device__ __forceinline__ bool raw_key_exact(long long k) {
  // not a zero (raw keys 0 and -1) and not a NaN (beyond the infinities)
  return k != 0 && k != -1 && k <= 0x7ff0000000000000LL && k >= (long long)0x800fffffffffffffULL;
}

template <bool MAX, class Ld = LdGlobal>
__device__ __forceinline__ typename ExtremumOp<double, MAX>::Acc run_short(
    const ExtremumOp<double, MAX>& op, const double* p, int n, long long j0, long long st,
    long long li, Ld ld = Ld{}) {
  if constexpr (Ld::kTouch) touch_run(p, n, 8);
  const long long* q = reinterpret_cast<const long long*>(p);
  long long best = 0;
  int at = -1;
  for (int i = 0; i < n; i++) {
    const long long k = MAX ? f64_raw_key(ld(q + i)) : ~f64_raw_key(ld(q + i));
    if (at < 0 || k > best) {
      best = k;
      at = i;
    }
  }
  typename ExtremumOp<double, MAX>::Acc a = op.identity();
  if (at < 0) return a;
  const long long bits = ld(q + at);
  if (raw_key_exact(f64_raw_key(bits))) return {f64_dir_key<MAX>(__longlong_as_double(bits)), bits, j0 + at};
  for (int i = 0; i < n; i++) a = op.step(a, ld(p + i), j0 + i, j0 + i == st, li);
  return a;
}

template <bool MAX, class Ld = LdGlobal>
__device__ __forceinline__ typename ArgExtremumOp<double, MAX>::Acc run_short(
    const ArgExtremumOp<double, MAX>& op, const double* p, int n, long long j0, long long st,
    long long li, Ld ld = Ld{}) {
  const long long* q = reinterpret_cast<const long long*>(p);
  long long best = 0;
  int at = -1;
  for (int i = 0; i < n; i++) {
    const long long k = MAX ? f64_raw_key(ld(q + i)) : ~f64_raw_key(ld(q + i));
    if (at < 0 || k > best) {
      best = k;
      at = i;
    }
  }
  typename ArgExtremumOp<double, MAX>::Acc a = op.identity();
  if (at < 0) return a;
  const long long bits = ld(q + at);
  // exact unless the winner is a zero or a NaN, or the run starts with a NaN
  if (raw_key_exact(f64_raw_key(bits)) && !(j0 == st && is_nan(ld(p))))
    return {f64_dir_key<MAX>(__longlong_as_double(bits)), j0 + at};
  for (int i = 0; i < n; i++) a = op.step(a, ld(p + i), j0 + i, j0 + i == st, li);
  return a;
}

// Exact float64 sum of at most 32 elements, branch-free: pass 1 finds the
// largest exponent (and any inf/NaN), pass 2 adds the significands aligned to
// it (|sum| < 2^58, no renormalisation needed).
template <class IN, class Ld = LdGlobal>
__device__ __forceinline__ FxAcc run_short(const FixedSumOp<IN>& op, const IN* p, int n,
                                           long long, long long, long long, Ld ld = Ld{}) {
  if constexpr (!std::is_same<IN, double>::value) {
    FxAcc a = op.identity();
    for (int i = 0; i < n; i++) a = op.step(a, ld(p + i), 0, false, 0);
    return a;
  } else {
    // Even positions are added in float64 (one DADD per pair, on the FP64
    // unit) while odd positions go through the fixed point on the integer
    // pipes; the float64 partial rides in FxAcc::dp and is added to the
    // rounded fixed-point part at the end (IEEE inf/NaN included).  The
    // result stays within n*eps*sum|x| of the exact sum.
    if constexpr (Ld::kTouch) touch_run(p, n, 8);
    const long long* q = reinterpret_cast<const long long*>(p);
    const int* qh = reinterpret_cast<const int*>(p) + 1;
    double dsum = 0.0;
    int ebmax = 0, ebmin = 0x7ff00000;
    int i = 0;
    for (; i + 1 < n; i += 2) {
      dsum += ld(p + i);
      const int eb = ld(qh + 2 * (i + 1)) & 0x7ff00000;
      ebmax = eb > ebmax ? eb : ebmax;
      ebmin = eb < ebmin ? eb : ebmin;
    }
    if (i < n) dsum += ld(p + i);
    const int half = n >> 1;  // odd positions 1, 3, ..., 2*half-1
    if (half == 0) return FxAcc{0, 1, 0, dsum};
    const int emax_f = ebmax >> 20, emin_f = ebmin >> 20;
    long long acc = 0;
    int anchor;
    if (emax_f != 0x7ff && emin_f != 0 && emax_f - emin_f < 32) {
      // every odd element normal and within 32 binades: two funnel shifts
      // each.  The shifts take d mod 32 (wrap), and (hi >> 20) differs from
      // the exponent only in bit 11 (the sign), so d needs no mask; a
      // negative addend is added as its one's complement and the count of
      // negatives added back once.
      long long xs = 0;
      int negs = 0;
      for (int k = 1; k < n; k += 2) {
        const long long b = ld(q + k);
        const unsigned hi = (unsigned)((unsigned long long)b >> 32);
        const unsigned d = (unsigned)emax_f - (hi >> 20);
        const unsigned mh = (hi & 0xfffffu) | 0x100000u;
        const unsigned tl = __funnelshift_r((unsigned)b, mh, d);
        const unsigned th = __funnelshift_r(mh, 0u, d);
        const long long t = (long long)(((unsigned long long)th << 32) | tl);
        const int sg = (int)hi >> 31;  // 0 or -1
        xs += t ^ (long long)sg;
        negs -= sg;
      }
      acc = xs + negs;
      anchor = emax_f;
    } else if (emax_f == 0x7ff) {  // inf / NaN among them: the general accumulator
      FxAcc a = op.identity();
      for (int k = 1; k < n; k += 2) a = fx_add_f64(a, __longlong_as_double(ld(q + k)));
      a.dp = dsum;
      return a;
    } else {  // zeros, subnormals or a wide exponent spread
      anchor = emax_f > 1 ? emax_f : 1;
      for (int k = 1; k < n; k += 2) {
        const long long b = ld(q + k);
        const int e = (int)((unsigned long long)b >> 52) & 0x7ff;
        const long long m = (b & 0xfffffffffffffLL) | ((long long)(e != 0) << 52);
        const int d = anchor - (e ? e : 1);
        const long long t = m >> (d < 63 ? d : 63);
        const long long sg = b >> 63;  // 0 or -1
        acc += (t ^ sg) - sg;
      }
    }
    return FxAcc{acc, anchor, 0, dsum};
  }
}

// ---------------------------------------------------------------- whole short lists
// The output of a whole list of n <= kShortList float64 elements at p
// (global index st) for the lane-per-list rounds of seg_reduce_kernel: the
// largest raw key in one pass, with nothing but the key kept per element.
// The raw key is a bijection, so the winner's bits are the key mapped back,
// and the output equals finalize(run_short(...)) bit for bit whenever *fast
// stays true -- that is, unless the winner is a zero or a NaN (or, for the
// arg-reducers, the list starts with a NaN), where the caller reruns
// run_short's exact path.
template <bool MAX>
struct LaneFinal<ExtremumOp<double, MAX>> : std::true_type {};
template <bool MAX>
struct LaneFinal<ArgExtremumOp<double, MAX>> : std::true_type {};

// 0 < |b| <= inf: the winner is neither a zero nor a NaN
__device__ __forceinline__ bool raw_winner_exact(long long b) {
  return (unsigned long long)((b & 0x7fffffffffffffffLL) - 1) < 0x7ff0000000000000ULL;
}

template <bool MAX>
__device__ __forceinline__ double lane_final(const ExtremumOp<double, MAX>& op, const double* p,
                                             int n, long long, bool& fast) {
  if (n <= 0) return op.ident;
  const long long* q = reinterpret_cast<const long long*>(p);
  long long best = kKeyLow;  // the first element is always taken
  for (int i = 0; i < n; i++) {
    const long long k = MAX ? f64_raw_key(__ldg(q + i)) : ~f64_raw_key(__ldg(q + i));
    best = k > best ? k : best;
  }
  const long long bits = f64_raw_key(MAX ? best : ~best);  // the raw key is an involution
  fast = raw_winner_exact(bits);
  // identity -inf (max) / +inf (min): every non-NaN winner is the output
  // (an infinite winner equal to the identity has the identity's bits)
  if (__double_as_longlong(op.ident) == (MAX ? (long long)0xfff0000000000000ULL : 0x7ff0000000000000LL))
    return __longlong_as_double(bits);
  return op.finalize({f64_dir_key<MAX>(__longlong_as_double(bits)), bits, 0}, 0);
}

template <bool MAX>
__device__ __forceinline__ int64_t lane_final(const ArgExtremumOp<double, MAX>&, const double* p,
                                              int n, long long st, bool& fast) {
  if (n <= 0) return -1;
  const long long* q = reinterpret_cast<const long long*>(p);
  long long best = kKeyLow;
  int at = 0;
  for (int i = 0; i < n; i++) {
    const long long k = MAX ? f64_raw_key(__ldg(q + i)) : ~f64_raw_key(__ldg(q + i));
    if (k > best) {
      best = k;
      at = i;
    }
  }
  const long long bits = f64_raw_key(MAX ? best : ~best);
  fast = raw_winner_exact(bits) && !is_nan(__longlong_as_double(__ldg(q)));
  return st + at;
}

// ---------------------------------------------------------------- warp runs
// Reduce elements [s, e) of list `li` (first element st) with a group of G
// lanes (G = 32: the whole warp; G = 8: four groups, four lists at once),
// lanes strided within the group; every lane of the group returns the
// result.  All lanes of the warp call together (every group with its own
// list); any fallback to the exact path is taken by the whole warp.

// Combine across the G lanes of a group.
template <int G, class Op>
__device__ __forceinline__ typename Op::Acc group_allreduce(const Op& op, typename Op::Acc a) {
#pragma unroll
  for (int d = G / 2; d > 0; d >>= 1) {
    constexpr int W = sizeof(typename Op::Acc) / 4;
    union U { typename Op::Acc v; uint32_t w[W]; } u;
    u.v = a;
#pragma unroll
    for (int i = 0; i < W; i++) u.w[i] = __shfl_xor_sync(0xffffffffu, u.w[i], d);
    a = op.combine(a, u.v);
  }
  return a;
}

template <int G, class Op>
__device__ __forceinline__ typename Op::Acc run_coop_exact(const Op& op,
                                                           const store_t<typename Op::In>* x,
                                                           long long s, long long e, long long st,
                                                           long long li) {
  const int sub = threadIdx.x & (G - 1);
  typename Op::Acc a = op.identity();
  for (long long j = s + sub; j < e; j += G) a = op.step(a, __ldg(x + j), j, j == st, li);
  return group_allreduce<G>(op, a);
}

template <int G, class Op>
__device__ typename Op::Acc run_coop(const Op& op, const store_t<typename Op::In>* x, long long s,
                                     long long e, long long st, long long li) {
  return run_coop_exact<G>(op, x, s, e, st, li);
}

// Float64 sum: a group-wide largest exponent, then every lane adds its
// elements aligned to it (one anchor: no renormalisation inside the run, the
// same truncation whatever the lane order) and the lanes' fixed-point
// partials are combined.  Runs with an infinity or NaN, or with more than 256
// elements per lane (a lane partial could exceed 2^62), take the general
// accumulator.
template <int G, class IN>
__device__ __forceinline__ FxAcc run_coop_sum(const FixedSumOp<IN>& op, const IN* x, long long s,
                                              long long e, long long st, long long li) {
  if constexpr (!std::is_same<IN, double>::value) {
    return run_coop_exact<G>(op, x, s, e, st, li);
  } else {
    const int sub = threadIdx.x & (G - 1);
    const int* xh = reinterpret_cast<const int*>(x) + 1;
    int eb = 0;
    const bool too_long = e - s > 256ll * G;
    if (!too_long)
      for (long long j = s + sub; j < e; j += G) {
        const int v = __ldg(xh + 2 * j) & 0x7ff00000;
        eb = v > eb ? v : eb;
      }
#pragma unroll
    for (int d = G / 2; d > 0; d >>= 1) {
      const int o = __shfl_xor_sync(0xffffffffu, eb, d);
      eb = o > eb ? o : eb;
    }
    const int emax_f = eb >> 20;
    if (__any_sync(0xffffffffu, too_long || emax_f == 0x7ff))
      return run_coop_exact<G>(op, x, s, e, st, li);
    const int anchor = emax_f > 1 ? emax_f : 1;
    const long long* q = reinterpret_cast<const long long*>(x);
    long long acc = 0;
    for (long long j = s + sub; j < e; j += G) {
      const long long b = __ldg(q + j);
      const int ex = (int)((unsigned long long)b >> 52) & 0x7ff;
      const long long m = (b & 0xfffffffffffffLL) | ((long long)(ex != 0) << 52);
      const int d = anchor - (ex ? ex : 1);
      const long long t = m >> (d < 63 ? d : 63);
      const long long sg = b >> 63;
      acc += (t ^ sg) - sg;
    }
    return group_allreduce<G>(op, FxAcc{acc, anchor, 0});
  }
}
template <int G, class IN>
__device__ __forceinline__ FxAcc run_coop(const FixedSumOp<IN>& op, const IN* x, long long s,
                                          long long e, long long st, long long li) {
  return run_coop_sum<G>(op, x, s, e, st, li);
}

// Float64 extrema: lanes reduce raw order keys (first occurrence kept by the
// strict comparison, ties across lanes to the lower index); the result is the
// exact op's unless the winner is a zero or a NaN, or (argmax/argmin) the run
// starts the list with a NaN -- then the run is redone exactly.  Positions
// are kept as 32-bit offsets from s (runs shorter than 2^30).
template <int G, bool MAX>
__device__ __forceinline__ void raw_group_best(const double* x, long long s, long long e,
                                               long long* rk, long long* idx) {
  const int sub = threadIdx.x & (G - 1);
  const long long* q = reinterpret_cast<const long long*>(x + s);
  const int n = (int)(e - s);
  long long best = kKeyLow;
  int at = -1;
  for (int j = sub; j < n; j += G) {
    const long long k = MAX ? f64_raw_key(__ldg(q + j)) : ~f64_raw_key(__ldg(q + j));
    if (at < 0 || k > best) {
      best = k;
      at = j;
    }
  }
#pragma unroll
  for (int d = G / 2; d > 0; d >>= 1) {
    const long long ob = __shfl_xor_sync(0xffffffffu, best, d);
    const int oa = __shfl_xor_sync(0xffffffffu, at, d);
    const bool take = oa >= 0 && (at < 0 || ob > best || (ob == best && oa < at));
    best = take ? ob : best;
    at = take ? oa : at;
  }
  *rk = best;
  *idx = at < 0 ? -1 : s + at;
}

template <int G, bool MAX>
__device__ __forceinline__ typename ExtremumOp<double, MAX>::Acc run_coop(
    const ExtremumOp<double, MAX>& op, const double* x, long long s, long long e, long long st,
    long long li) {
  const bool too_long = e - s >= (1ll << 30);
  long long rk = kKeyLow, at = -1;
  if (!__any_sync(0xffffffffu, too_long)) raw_group_best<G, MAX>(x, s, e, &rk, &at);
  long long bits = 0;
  bool exact = !too_long;
  if (exact && at >= 0) {
    bits = __ldg(reinterpret_cast<const long long*>(x) + at);
    exact = raw_key_exact(f64_raw_key(bits));
  }
  if (__any_sync(0xffffffffu, !exact)) return run_coop_exact<G>(op, x, s, e, st, li);
  if (at < 0) return op.identity();
  return {f64_dir_key<MAX>(__longlong_as_double(bits)), bits, at};
}

template <int G, bool MAX>
__device__ __forceinline__ typename ArgExtremumOp<double, MAX>::Acc run_coop(
    const ArgExtremumOp<double, MAX>& op, const double* x, long long s, long long e, long long st,
    long long li) {
  const bool too_long = e - s >= (1ll << 30);
  long long rk = kKeyLow, at = -1;
  if (!__any_sync(0xffffffffu, too_long)) raw_group_best<G, MAX>(x, s, e, &rk, &at);
  long long bits = 0;
  bool exact = !too_long && !(st >= s && st < e && is_nan(__ldg(x + st)));
  if (exact && at >= 0) {
    bits = __ldg(reinterpret_cast<const long long*>(x) + at);
    exact = raw_key_exact(f64_raw_key(bits));
  }
  if (__any_sync(0xffffffffu, !exact)) return run_coop_exact<G>(op, x, s, e, st, li);
  if (at < 0) return op.identity();
  return {f64_dir_key<MAX>(__longlong_as_double(bits)), at};
}

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
  __device__ Acc step(Acc a, store_t<IN> v, long long j, bool f, long long l) const { return a + lift(v, j, f, l); }
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
  __device__ Acc step(Acc a, store_t<IN> v, long long j, bool f, long long l) const { return a + lift(v, j, f, l); }
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
  __device__ Acc step(Acc a, store_t<IN> v, long long j, bool f, long long l) const { return a + lift(v, j, f, l); }
  __device__ Out finalize(Acc a, long long) const { return a; }
};

// ---------------------------------------------------------------- launcher
template <class Op>
struct SegReduceConfig {
  static int blocks_per_sm() {
    static std::once_flag once;
    static int bps = 1;
    std::call_once(once, [] {
      int n = 0;
      if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, seg_reduce_kernel<Op>, kSegBlock, 0) !=
              cudaSuccess ||
          n < 1)
        n = 1;
      bps = n;
    });
    return bps;
  }
};

// Launch the segmented reduction of `nlists` lists on `stream`: the
// warp-balanced kernel over a persistent grid, then the fix-up of lists
// longer than kAbsorb elements that cross warp ranges.  Returns the launch status; data never
// travel to the host.
template <class Op>
cudaError_t launch_seg_reduce(const Op& op, const store_t<typename Op::In>* x,
                              const int64_t* offsets, long long nlists, typename Op::Out* out,
                              uint64_t inv, uint64_t* err, cudaStream_t stream) {
  if (nlists <= 0) return cudaSuccess;
  using Rec = RangeRecord<typename Op::Acc>;
  const int blocks = device_sm_count() * SegReduceConfig<Op>::blocks_per_sm();
  const int W = blocks * (kSegBlock / 32);
  void* rec = nullptr;
  cudaError_t e = scratch_alloc(&rec, (size_t)W * sizeof(Rec), stream);
  if (e != cudaSuccess) return e;
  seg_reduce_kernel<Op><<<blocks, kSegBlock, 0, stream>>>(op, x, offsets, nlists, out,
                                                          reinterpret_cast<Rec*>(rec), W, inv,
                                                          err);
  e = cudaGetLastError();
  if (e == cudaSuccess) {
    const int fix_blocks = (W + 255) / 256;  // one warp per 32 records
    seg_reduce_fixup_kernel<Op><<<fix_blocks, 256, 0, stream>>>(
        op, offsets, nlists, out, reinterpret_cast<const Rec*>(rec), W);
    e = cudaGetLastError();
  }
  cudaError_t f = scratch_free(rec, stream);
  return e != cudaSuccess ? e : f;
}

}  // namespace gb
