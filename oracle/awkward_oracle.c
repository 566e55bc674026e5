/* awkward_oracle.c -- CPU oracle for the GB300 jagged hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file restates, in plain C, the awkward-cpp
 * CPU kernels that libawkward_gb300 replaces, so that the CUDA results can be
 * checked against the reference algorithm on the same inputs.  Only the test
 * suite, the smoke check and the CPU-baseline leg of bench.py load it; the
 * product path never calls it.
 *
 * Every function has the exact name and C signature of the awkward-cpp
 * specialization it restates (kernel-specification.yml) and returns the same
 * `struct Error` (awkward-cpp/include/awkward/common.h:39-77): str == NULL on
 * success, else the message, the failing outer index (identity) and the
 * offending value (attempt, kSliceNone when none).
 *
 * Parity is pinned two ways (tests/test_oracle_golden.py):
 *   - awkward's kernel-test-data.json unit tests for every family here that
 *     has them (fixtures in tests/golden/kernel_test_data_subset.json);
 *   - outputs of awkward-cpp's own CPU kernels, compiled from the reference
 *     sources by oracle/build.py, on seeded random inputs
 *     (tests/golden/ref_random.npz).
 *
 * A pthread driver at the end (oracle_parallel_reduce) splits a reduction
 * over list ranges for the multi-core CPU baseline.
 */
#include <math.h>
#include <pthread.h>
#include <stdbool.h>
#include <stddef.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

struct Error {
  const char* str;
  const char* filename;
  int64_t identity;
  int64_t attempt;
};

#define kSliceNone ((int64_t)9223372036854775807LL)

static struct Error success(void) {
  struct Error e = {NULL, NULL, kSliceNone, kSliceNone};
  return e;
}
static struct Error failure(const char* s, int64_t identity, int64_t attempt) {
  struct Error e = {s, "oracle/awkward_oracle.c", identity, attempt};
  return e;
}

/* ======================================================================
 * Segmented reducers over offsets (awkward-cpp/src/cpu-kernels/awkward_reduce_*.cpp)
 * Every reducer visits bin b's elements fromptr[offsets[b] .. offsets[b+1])
 * in order, left to right, accumulating in the output type.
 * ====================================================================== */

/* awkward_reduce_sum.cpp:12-25 -- acc = OUT{}; acc += (OUT)x */
#define ORACLE_SUM(NAME, OUT, IN)                                              \
  struct Error NAME(OUT* toptr, const IN* fromptr, const int64_t* offsets,     \
                    int64_t outlength) {                                       \
    for (int64_t b = 0; b < outlength; b++) {                                  \
      OUT acc = (OUT)0;                                                        \
      for (int64_t i = offsets[b]; i < offsets[b + 1]; i++) acc += (OUT)fromptr[i]; \
      toptr[b] = acc;                                                          \
    }                                                                          \
    return success();                                                          \
  }
ORACLE_SUM(awkward_reduce_sum_int64_int8_64, int64_t, int8_t)
ORACLE_SUM(awkward_reduce_sum_uint64_uint8_64, uint64_t, uint8_t)
ORACLE_SUM(awkward_reduce_sum_int64_int16_64, int64_t, int16_t)
ORACLE_SUM(awkward_reduce_sum_uint64_uint16_64, uint64_t, uint16_t)
ORACLE_SUM(awkward_reduce_sum_int64_int32_64, int64_t, int32_t)
ORACLE_SUM(awkward_reduce_sum_uint64_uint32_64, uint64_t, uint32_t)
ORACLE_SUM(awkward_reduce_sum_int64_int64_64, int64_t, int64_t)
ORACLE_SUM(awkward_reduce_sum_uint64_uint64_64, uint64_t, uint64_t)
ORACLE_SUM(awkward_reduce_sum_float32_float32_64, float, float)
ORACLE_SUM(awkward_reduce_sum_float64_float64_64, double, double)
ORACLE_SUM(awkward_reduce_sum_int32_int8_64, int32_t, int8_t)
ORACLE_SUM(awkward_reduce_sum_uint32_uint8_64, uint32_t, uint8_t)
ORACLE_SUM(awkward_reduce_sum_int32_int16_64, int32_t, int16_t)
ORACLE_SUM(awkward_reduce_sum_uint32_uint16_64, uint32_t, uint16_t)
ORACLE_SUM(awkward_reduce_sum_int32_int32_64, int32_t, int32_t)
ORACLE_SUM(awkward_reduce_sum_uint32_uint32_64, uint32_t, uint32_t)
ORACLE_SUM(awkward_reduce_sum_float64_int8_64, double, int8_t)
ORACLE_SUM(awkward_reduce_sum_float64_uint8_64, double, uint8_t)
ORACLE_SUM(awkward_reduce_sum_float64_int16_64, double, int16_t)
ORACLE_SUM(awkward_reduce_sum_float64_uint16_64, double, uint16_t)
ORACLE_SUM(awkward_reduce_sum_float64_int32_64, double, int32_t)
ORACLE_SUM(awkward_reduce_sum_float64_uint32_64, double, uint32_t)
ORACLE_SUM(awkward_reduce_sum_float64_int64_64, double, int64_t)
ORACLE_SUM(awkward_reduce_sum_float64_uint64_64, double, uint64_t)
ORACLE_SUM(awkward_reduce_sum_float64_float32_64, double, float)

/* awkward_reduce_sum_int32_bool_64.cpp:7-19, awkward_reduce_sum_int64_bool_64.cpp:7-19 */
#define ORACLE_SUM_OF_BOOL(NAME, OUT)                                          \
  struct Error NAME(OUT* toptr, const bool* fromptr, const int64_t* offsets,   \
                    int64_t outlength) {                                       \
    for (int64_t b = 0; b < outlength; b++) {                                  \
      OUT acc = 0;                                                             \
      for (int64_t i = offsets[b]; i < offsets[b + 1]; i++) if (fromptr[i]) acc++; \
      toptr[b] = acc;                                                          \
    }                                                                          \
    return success();                                                          \
  }
ORACLE_SUM_OF_BOOL(awkward_reduce_sum_int32_bool_64, int32_t)
ORACLE_SUM_OF_BOOL(awkward_reduce_sum_int64_bool_64, int64_t)

/* awkward_reduce_sum_bool.cpp:18-31 (any nonzero) and
 * awkward_reduce_prod_bool.cpp:10-23 (all nonzero); NaN != 0 is true. */
#define ORACLE_ANY(NAME, IN)                                                   \
  struct Error NAME(bool* toptr, const IN* fromptr, const int64_t* offsets,    \
                    int64_t outlength) {                                       \
    for (int64_t b = 0; b < outlength; b++) {                                  \
      bool found = false;                                                      \
      for (int64_t i = offsets[b]; i < offsets[b + 1]; i++)                    \
        if (fromptr[i] != 0) { found = true; break; }                          \
      toptr[b] = found;                                                        \
    }                                                                          \
    return success();                                                          \
  }
#define ORACLE_ALL(NAME, IN)                                                   \
  struct Error NAME(bool* toptr, const IN* fromptr, const int64_t* offsets,    \
                    int64_t outlength) {                                       \
    for (int64_t b = 0; b < outlength; b++) {                                  \
      bool all = true;                                                         \
      for (int64_t i = offsets[b]; i < offsets[b + 1]; i++)                    \
        if (fromptr[i] == 0) { all = false; break; }                           \
      toptr[b] = all;                                                          \
    }                                                                          \
    return success();                                                          \
  }
#define ORACLE_FOR_ALL_IN(M, PREFIX)                                           \
  M(PREFIX##bool_64, bool) M(PREFIX##int8_64, int8_t) M(PREFIX##uint8_64, uint8_t) \
  M(PREFIX##int16_64, int16_t) M(PREFIX##uint16_64, uint16_t)                  \
  M(PREFIX##int32_64, int32_t) M(PREFIX##uint32_64, uint32_t)                  \
  M(PREFIX##int64_64, int64_t) M(PREFIX##uint64_64, uint64_t)                  \
  M(PREFIX##float32_64, float) M(PREFIX##float64_64, double)
ORACLE_FOR_ALL_IN(ORACLE_ANY, awkward_reduce_sum_bool_)
ORACLE_FOR_ALL_IN(ORACLE_ALL, awkward_reduce_prod_bool_)

/* awkward_reduce_prod.cpp:12-25 -- acc = (OUT)1; acc *= (OUT)x */
#define ORACLE_PROD(NAME, OUT, IN)                                             \
  struct Error NAME(OUT* toptr, const IN* fromptr, const int64_t* offsets,     \
                    int64_t outlength) {                                       \
    for (int64_t b = 0; b < outlength; b++) {                                  \
      OUT acc = (OUT)1;                                                        \
      for (int64_t i = offsets[b]; i < offsets[b + 1]; i++) acc *= (OUT)fromptr[i]; \
      toptr[b] = acc;                                                          \
    }                                                                          \
    return success();                                                          \
  }
ORACLE_PROD(awkward_reduce_prod_int64_int8_64, int64_t, int8_t)
ORACLE_PROD(awkward_reduce_prod_uint64_uint8_64, uint64_t, uint8_t)
ORACLE_PROD(awkward_reduce_prod_int64_int16_64, int64_t, int16_t)
ORACLE_PROD(awkward_reduce_prod_uint64_uint16_64, uint64_t, uint16_t)
ORACLE_PROD(awkward_reduce_prod_int64_int32_64, int64_t, int32_t)
ORACLE_PROD(awkward_reduce_prod_uint64_uint32_64, uint64_t, uint32_t)
ORACLE_PROD(awkward_reduce_prod_int64_int64_64, int64_t, int64_t)
ORACLE_PROD(awkward_reduce_prod_uint64_uint64_64, uint64_t, uint64_t)
ORACLE_PROD(awkward_reduce_prod_float32_float32_64, float, float)
ORACLE_PROD(awkward_reduce_prod_float64_float64_64, double, double)
ORACLE_PROD(awkward_reduce_prod_int32_int8_64, int32_t, int8_t)
ORACLE_PROD(awkward_reduce_prod_uint32_uint8_64, uint32_t, uint8_t)
ORACLE_PROD(awkward_reduce_prod_int32_int16_64, int32_t, int16_t)
ORACLE_PROD(awkward_reduce_prod_uint32_uint16_64, uint32_t, uint16_t)
ORACLE_PROD(awkward_reduce_prod_int32_int32_64, int32_t, int32_t)
ORACLE_PROD(awkward_reduce_prod_uint32_uint32_64, uint32_t, uint32_t)

/* awkward_reduce_max.cpp:9-26 / awkward_reduce_min.cpp:26-43 --
 * best = identity; best = (v > best) ? v : best.  NaN never replaces best;
 * among equal values (e.g. -0.0 and +0.0) the earliest, identity first, stays. */
#define ORACLE_EXTREMUM(NAME, T, CMP)                                          \
  struct Error NAME(T* toptr, const T* fromptr, const int64_t* offsets,        \
                    int64_t outlength, T identity) {                           \
    for (int64_t b = 0; b < outlength; b++) {                                  \
      T best = identity;                                                       \
      for (int64_t i = offsets[b]; i < offsets[b + 1]; i++) {                  \
        T v = fromptr[i];                                                      \
        best = (v CMP best) ? v : best;                                        \
      }                                                                        \
      toptr[b] = best;                                                         \
    }                                                                          \
    return success();                                                          \
  }
#define ORACLE_FOR_NUMERIC_SAME(M, PREFIX, CMP)                                \
  M(PREFIX##int8_int8_64, int8_t, CMP) M(PREFIX##uint8_uint8_64, uint8_t, CMP) \
  M(PREFIX##int16_int16_64, int16_t, CMP) M(PREFIX##uint16_uint16_64, uint16_t, CMP) \
  M(PREFIX##int32_int32_64, int32_t, CMP) M(PREFIX##uint32_uint32_64, uint32_t, CMP) \
  M(PREFIX##int64_int64_64, int64_t, CMP) M(PREFIX##uint64_uint64_64, uint64_t, CMP) \
  M(PREFIX##float32_float32_64, float, CMP) M(PREFIX##float64_float64_64, double, CMP)
ORACLE_FOR_NUMERIC_SAME(ORACLE_EXTREMUM, awkward_reduce_max_, >)
ORACLE_FOR_NUMERIC_SAME(ORACLE_EXTREMUM, awkward_reduce_min_, <)

/* awkward_reduce_argmax.cpp:9-33 / awkward_reduce_argmin.cpp:25-49 --
 * global index of the first extremum; -1 for an empty bin.  The first
 * element is taken unconditionally, so a leading NaN wins; later NaNs never
 * win.  `starts` is unused. */
#define ORACLE_ARG(NAME, IN, CMP)                                              \
  struct Error NAME(int64_t* toptr, const IN* fromptr, const int64_t* offsets, \
                    const int64_t* starts, int64_t outlength) {                \
    (void)starts;                                                              \
    for (int64_t b = 0; b < outlength; b++) {                                  \
      int64_t start = offsets[b], stop = offsets[b + 1], best = -1;            \
      if (start < stop) {                                                      \
        best = start;                                                          \
        IN bv = fromptr[start];                                                \
        for (int64_t i = start + 1; i < stop; i++)                             \
          if (fromptr[i] CMP bv) { bv = fromptr[i]; best = i; }                \
      }                                                                        \
      toptr[b] = best;                                                         \
    }                                                                          \
    return success();                                                          \
  }
#define ORACLE_FOR_NUMERIC_IN(M, PREFIX, CMP)                                  \
  M(PREFIX##int8_64, int8_t, CMP) M(PREFIX##uint8_64, uint8_t, CMP)            \
  M(PREFIX##int16_64, int16_t, CMP) M(PREFIX##uint16_64, uint16_t, CMP)        \
  M(PREFIX##int32_64, int32_t, CMP) M(PREFIX##uint32_64, uint32_t, CMP)        \
  M(PREFIX##int64_64, int64_t, CMP) M(PREFIX##uint64_64, uint64_t, CMP)        \
  M(PREFIX##float32_64, float, CMP) M(PREFIX##float64_64, double, CMP)
ORACLE_FOR_NUMERIC_IN(ORACLE_ARG, awkward_reduce_argmax_, >)
ORACLE_FOR_NUMERIC_IN(ORACLE_ARG, awkward_reduce_argmin_, <)

/* awkward_reduce_count_64.cpp:7-15 */
struct Error awkward_reduce_count_64(int64_t* toptr, const int64_t* offsets,
                                     int64_t outlength) {
  for (int64_t b = 0; b < outlength; b++) toptr[b] = offsets[b + 1] - offsets[b];
  return success();
}

/* awkward_reduce_countnonzero.cpp:14-36 */
#define ORACLE_COUNTNONZERO(NAME, IN)                                          \
  struct Error NAME(int64_t* toptr, const IN* fromptr, const int64_t* offsets, \
                    int64_t outlength) {                                       \
    for (int64_t b = 0; b < outlength; b++) {                                  \
      int64_t c = 0;                                                           \
      for (int64_t i = offsets[b]; i < offsets[b + 1]; i++) c += (fromptr[i] != 0); \
      toptr[b] = c;                                                            \
    }                                                                          \
    return success();                                                          \
  }
ORACLE_FOR_ALL_IN(ORACLE_COUNTNONZERO, awkward_reduce_countnonzero_)

/* awkward_reduce_sumofsquares.cpp:12-25: acc += v*v with v = (double)x */
#define ORACLE_SUMSQ(NAME, IN)                                                 \
  struct Error NAME(double* toptr, const IN* fromptr, const int64_t* offsets,  \
                    int64_t outlength) {                                       \
    for (int64_t b = 0; b < outlength; b++) {                                  \
      double acc = 0.0;                                                        \
      for (int64_t i = offsets[b]; i < offsets[b + 1]; i++) {                  \
        double v = (double)fromptr[i];                                         \
        acc += v * v;                                                          \
      }                                                                        \
      toptr[b] = acc;                                                          \
    }                                                                          \
    return success();                                                          \
  }
#define ORACLE_FOR_F64_OUT(M, PREFIX)                                          \
  M(PREFIX##float64_int8_64, int8_t) M(PREFIX##float64_uint8_64, uint8_t)      \
  M(PREFIX##float64_int16_64, int16_t) M(PREFIX##float64_uint16_64, uint16_t)  \
  M(PREFIX##float64_int32_64, int32_t) M(PREFIX##float64_uint32_64, uint32_t)  \
  M(PREFIX##float64_int64_64, int64_t) M(PREFIX##float64_uint64_64, uint64_t)  \
  M(PREFIX##float64_bool_64, bool) M(PREFIX##float64_float32_64, float)        \
  M(PREFIX##float64_float64_64, double)
ORACLE_FOR_F64_OUT(ORACLE_SUMSQ, awkward_reduce_sumofsquares_)

/* awkward_reduce_sumofpowers.cpp:14-60: integer powers by repeated
 * squaring (exponent bits low to high), std::pow for n < 0. */
static double oracle_ipow(double base, int64_t n) {
  if (n < 0) return pow(base, (double)n);
  double result = 1.0, b = base;
  int64_t e = n;
  while (e > 0) {
    if (e & 1) result *= b;
    e >>= 1;
    if (e > 0) b *= b;
  }
  return result;
}
#define ORACLE_SUMPOW(NAME, IN)                                                \
  struct Error NAME(double* toptr, const IN* fromptr, const int64_t* offsets,  \
                    int64_t outlength, int64_t n) {                            \
    for (int64_t b = 0; b < outlength; b++) {                                  \
      double acc = 0.0;                                                        \
      for (int64_t i = offsets[b]; i < offsets[b + 1]; i++)                    \
        acc += oracle_ipow((double)fromptr[i], n);                             \
      toptr[b] = acc;                                                          \
    }                                                                          \
    return success();                                                          \
  }
ORACLE_FOR_F64_OUT(ORACLE_SUMPOW, awkward_reduce_sumofpowers_)

/* awkward_reduce_centered_sumofsquares.cpp:15-29: d = (double)x - means[b] */
#define ORACLE_CSUMSQ(NAME, IN)                                                \
  struct Error NAME(double* toptr, const IN* fromptr, const int64_t* offsets,  \
                    int64_t outlength, const double* means) {                  \
    for (int64_t b = 0; b < outlength; b++) {                                  \
      double acc = 0.0, m = means[b];                                          \
      for (int64_t i = offsets[b]; i < offsets[b + 1]; i++) {                  \
        double d = (double)fromptr[i] - m;                                     \
        acc += d * d;                                                          \
      }                                                                        \
      toptr[b] = acc;                                                          \
    }                                                                          \
    return success();                                                          \
  }
ORACLE_FOR_F64_OUT(ORACLE_CSUMSQ, awkward_reduce_centered_sumofsquares_)

/* awkward_NumpyArray_reduce_adjust_starts_64.cpp:7-25 */
struct Error awkward_NumpyArray_reduce_adjust_starts_64(int64_t* toptr, int64_t outlength,
                                                        const int64_t* offsets,
                                                        const int64_t* starts) {
  (void)offsets;
  for (int64_t k = 0; k < outlength; k++)
    if (toptr[k] >= 0) toptr[k] -= starts[k];
  return success();
}

/* awkward_NumpyArray_reduce_mask_ByteMaskedArray_64.cpp:7-20 */
struct Error awkward_NumpyArray_reduce_mask_ByteMaskedArray_64(int8_t* toptr,
                                                               const int64_t* offsets,
                                                               int64_t outlength) {
  for (int64_t i = 0; i < outlength; i++) toptr[i] = (offsets[i + 1] - offsets[i] > 0) ? 0 : 1;
  return success();
}

/* ======================================================================
 * Jagged getitem (awkward-cpp/src/cpu-kernels/awkward_ListArray_getitem_jagged_*.cpp)
 * ====================================================================== */

/* awkward_ListArray_getitem_jagged_apply.cpp:8-56 */
#define ORACLE_JAGGED_APPLY(NAME, C)                                           \
  struct Error NAME(int64_t* tooffsets, int64_t* tocarry, const int64_t* slicestarts, \
                    const int64_t* slicestops, int64_t sliceouterlen,          \
                    const int64_t* sliceindex, int64_t sliceinnerlen,          \
                    const C* fromstarts, const C* fromstops, int64_t contentlen) { \
    int64_t k = 0;                                                             \
    for (int64_t i = 0; i < sliceouterlen; i++) {                              \
      int64_t ss = slicestarts[i], se = slicestops[i];                         \
      tooffsets[i] = k;                                                        \
      if (ss == se) continue;                                                  \
      if (se < ss) return failure("jagged slice's stops[i] < starts[i]", i, kSliceNone); \
      if (se > sliceinnerlen)                                                  \
        return failure("jagged slice's offsets extend beyond its content", i, se); \
      int64_t start = (int64_t)fromstarts[i], stop = (int64_t)fromstops[i];    \
      if (stop < start) return failure("stops[i] < starts[i]", i, kSliceNone); \
      if (start != stop && stop > contentlen)                                  \
        return failure("stops[i] > len(content)", i, kSliceNone);              \
      int64_t count = stop - start;                                            \
      for (int64_t j = ss; j < se; j++) {                                      \
        int64_t index = sliceindex[j];                                         \
        if (index < -count || index >= count)                                  \
          return failure("index out of range", i, index);                      \
        if (index < 0) index += count;                                         \
        tocarry[k++] = start + index;                                          \
      }                                                                        \
    }                                                                          \
    tooffsets[sliceouterlen] = k;                                              \
    return success();                                                          \
  }
ORACLE_JAGGED_APPLY(awkward_ListArray32_getitem_jagged_apply_64, int32_t)
ORACLE_JAGGED_APPLY(awkward_ListArrayU32_getitem_jagged_apply_64, uint32_t)
ORACLE_JAGGED_APPLY(awkward_ListArray64_getitem_jagged_apply_64, int64_t)

/* awkward_ListArray_getitem_jagged_carrylen.cpp:8-18 */
struct Error awkward_ListArray_getitem_jagged_carrylen_64(int64_t* carrylen,
                                                         const int64_t* slicestarts,
                                                         const int64_t* slicestops,
                                                         int64_t sliceouterlen) {
  int64_t total = 0;
  for (int64_t i = 0; i < sliceouterlen; i++) total += slicestops[i] - slicestarts[i];
  *carrylen = total;
  return success();
}

/* awkward_ListArray_getitem_jagged_descend.cpp:8-31 */
#define ORACLE_JAGGED_DESCEND(NAME, C)                                         \
  struct Error NAME(int64_t* tooffsets, const int64_t* slicestarts,            \
                    const int64_t* slicestops, int64_t sliceouterlen,          \
                    const C* fromstarts, const C* fromstops) {                 \
    tooffsets[0] = sliceouterlen == 0 ? 0 : slicestarts[0];                    \
    for (int64_t i = 0; i < sliceouterlen; i++) {                              \
      int64_t slicecount = slicestops[i] - slicestarts[i];                     \
      int64_t count = (int64_t)(fromstops[i] - fromstarts[i]);                 \
      if (slicecount != count)                                                 \
        return failure("jagged slice inner length differs from array inner length", i, kSliceNone); \
      tooffsets[i + 1] = tooffsets[i] + count;                                 \
    }                                                                          \
    return success();                                                          \
  }
ORACLE_JAGGED_DESCEND(awkward_ListArray32_getitem_jagged_descend_64, int32_t)
ORACLE_JAGGED_DESCEND(awkward_ListArrayU32_getitem_jagged_descend_64, uint32_t)
ORACLE_JAGGED_DESCEND(awkward_ListArray64_getitem_jagged_descend_64, int64_t)

/* awkward_ListArray_getitem_jagged_expand.cpp:8-32 */
#define ORACLE_JAGGED_EXPAND(NAME, C)                                          \
  struct Error NAME(int64_t* multistarts, int64_t* multistops,                 \
                    const int64_t* singleoffsets, int64_t* tocarry,            \
                    const C* fromstarts, const C* fromstops, int64_t jaggedsize, \
                    int64_t length) {                                          \
    for (int64_t i = 0; i < length; i++) {                                     \
      C start = fromstarts[i], stop = fromstops[i];                            \
      if (stop < start) return failure("stops[i] < starts[i]", i, kSliceNone); \
      if ((int64_t)(stop - start) != jaggedsize)                               \
        return failure("cannot fit jagged slice into nested list", i, kSliceNone); \
      for (int64_t j = 0; j < jaggedsize; j++) {                               \
        multistarts[i * jaggedsize + j] = singleoffsets[j];                    \
        multistops[i * jaggedsize + j] = singleoffsets[j + 1];                 \
        tocarry[i * jaggedsize + j] = (int64_t)start + j;                      \
      }                                                                        \
    }                                                                          \
    return success();                                                          \
  }
ORACLE_JAGGED_EXPAND(awkward_ListArray32_getitem_jagged_expand_64, int32_t)
ORACLE_JAGGED_EXPAND(awkward_ListArrayU32_getitem_jagged_expand_64, uint32_t)
ORACLE_JAGGED_EXPAND(awkward_ListArray64_getitem_jagged_expand_64, int64_t)

/* awkward_ListArray_getitem_jagged_numvalid.cpp:8-30 */
struct Error awkward_ListArray_getitem_jagged_numvalid_64(int64_t* numvalid,
                                                         const int64_t* slicestarts,
                                                         const int64_t* slicestops,
                                                         int64_t length,
                                                         const int64_t* missing,
                                                         int64_t missinglength) {
  int64_t total = 0;
  *numvalid = 0;
  for (int64_t i = 0; i < length; i++) {
    int64_t ss = slicestarts[i], se = slicestops[i];
    if (ss == se) continue;
    if (se < ss) return failure("jagged slice's stops[i] < starts[i]", i, kSliceNone);
    if (se > missinglength)
      return failure("jagged slice's offsets extend beyond its content", i, se);
    for (int64_t j = ss; j < se; j++) total += missing[j] >= 0 ? 1 : 0;
    *numvalid = total;
  }
  *numvalid = total;
  return success();
}

/* awkward_ListArray_getitem_jagged_shrink.cpp:8-46 */
struct Error awkward_ListArray_getitem_jagged_shrink_64(int64_t* tocarry, int64_t* tosmalloffsets,
                                                       int64_t* tolargeoffsets,
                                                       const int64_t* slicestarts,
                                                       const int64_t* slicestops, int64_t length,
                                                       const int64_t* missing) {
  int64_t k = 0;
  tosmalloffsets[0] = length == 0 ? 0 : slicestarts[0];
  tolargeoffsets[0] = length == 0 ? 0 : slicestarts[0];
  for (int64_t i = 0; i < length; i++) {
    int64_t ss = slicestarts[i], se = slicestops[i];
    if (ss != se) {
      int64_t small = 0;
      for (int64_t j = ss; j < se; j++)
        if (missing[j] >= 0) { tocarry[k++] = j; small++; }
      tosmalloffsets[i + 1] = tosmalloffsets[i] + small;
    } else {
      tosmalloffsets[i + 1] = tosmalloffsets[i];
    }
    tolargeoffsets[i + 1] = tolargeoffsets[i] + (se - ss);
  }
  return success();
}

/* awkward_RegularArray_getitem_jagged_expand.cpp:8-20 */
struct Error awkward_RegularArray_getitem_jagged_expand_64(int64_t* multistarts, int64_t* multistops,
                                                          const int64_t* singleoffsets,
                                                          int64_t regularsize,
                                                          int64_t regularlength) {
  for (int64_t i = 0; i < regularlength; i++)
    for (int64_t j = 0; j < regularsize; j++) {
      multistarts[i * regularsize + j] = singleoffsets[j];
      multistops[i * regularsize + j] = singleoffsets[j + 1];
    }
  return success();
}

/* awkward_ListArray_localindex.cpp:8-19 */
#define ORACLE_LOCALINDEX(NAME, C)                                             \
  struct Error NAME(int64_t* toindex, const C* offsets, int64_t length) {      \
    for (int64_t i = 0; i < length; i++) {                                     \
      int64_t start = (int64_t)offsets[i], stop = (int64_t)offsets[i + 1];     \
      for (int64_t j = start; j < stop; j++) toindex[j] = j - start;           \
    }                                                                          \
    return success();                                                          \
  }
ORACLE_LOCALINDEX(awkward_ListArray32_localindex_64, int32_t)
ORACLE_LOCALINDEX(awkward_ListArrayU32_localindex_64, uint32_t)
ORACLE_LOCALINDEX(awkward_ListArray64_localindex_64, int64_t)

/* ======================================================================
 * Range slices (awkward_ListArray_getitem_next_range*.cpp, kernel-utils.cpp)
 * ====================================================================== */

/* kernel-utils.cpp:7-39: clip a Python slice against one list's length */
static void oracle_regularize_rangeslice(int64_t* start, int64_t* stop, bool posstep,
                                         bool hasstart, bool hasstop, int64_t length) {
  if (posstep) {
    if (!hasstart) *start = 0;
    else if (*start < 0) *start += length;
    if (*start < 0) *start = 0;
    if (*start > length) *start = length;
    if (!hasstop) *stop = length;
    else if (*stop < 0) *stop += length;
    if (*stop < 0) *stop = 0;
    if (*stop > length) *stop = length;
    if (*stop < *start) *stop = *start;
  } else {
    if (!hasstart) *start = length - 1;
    else if (*start < 0) *start += length;
    if (*start < -1) *start = -1;
    if (*start > length - 1) *start = length - 1;
    if (!hasstop) *stop = -1;
    else if (*stop < 0) *stop += length;
    if (*stop < -1) *stop = -1;
    if (*stop > length - 1) *stop = length - 1;
    if (*stop > *start) *stop = *start;
  }
}

/* awkward_ListArray_getitem_next_range.cpp:9-41 */
#define ORACLE_NEXT_RANGE(NAME, C)                                             \
  struct Error NAME(C* tooffsets, int64_t* tocarry, const C* fromstarts,       \
                    const C* fromstops, int64_t lenstarts, int64_t start,      \
                    int64_t stop, int64_t step) {                              \
    int64_t k = 0;                                                             \
    tooffsets[0] = 0;                                                          \
    for (int64_t i = 0; i < lenstarts; i++) {                                  \
      int64_t length = (int64_t)fromstops[i] - (int64_t)fromstarts[i];         \
      int64_t rs = start, re = stop;                                           \
      oracle_regularize_rangeslice(&rs, &re, step > 0, start != kSliceNone,    \
                                   stop != kSliceNone, length);                \
      if (step > 0) {                                                          \
        for (int64_t j = rs; j < re; j += step) tocarry[k++] = (int64_t)fromstarts[i] + j; \
      } else {                                                                 \
        for (int64_t j = rs; j > re; j += step) tocarry[k++] = (int64_t)fromstarts[i] + j; \
      }                                                                        \
      tooffsets[i + 1] = (C)k;                                                 \
    }                                                                          \
    return success();                                                          \
  }
ORACLE_NEXT_RANGE(awkward_ListArray32_getitem_next_range_64, int32_t)
ORACLE_NEXT_RANGE(awkward_ListArrayU32_getitem_next_range_64, uint32_t)
ORACLE_NEXT_RANGE(awkward_ListArray64_getitem_next_range_64, int64_t)

/* awkward_ListArray_getitem_next_range_carrylength.cpp:9-35 */
#define ORACLE_NEXT_RANGE_CARRYLENGTH(NAME, C)                                 \
  struct Error NAME(int64_t* carrylength, const C* fromstarts, const C* fromstops, \
                    int64_t lenstarts, int64_t start, int64_t stop, int64_t step) { \
    int64_t total = 0;                                                         \
    for (int64_t i = 0; i < lenstarts; i++) {                                  \
      int64_t length = (int64_t)fromstops[i] - (int64_t)fromstarts[i];         \
      int64_t rs = start, re = stop;                                           \
      oracle_regularize_rangeslice(&rs, &re, step > 0, start != kSliceNone,    \
                                   stop != kSliceNone, length);                \
      if (step > 0) { for (int64_t j = rs; j < re; j += step) total++; }       \
      else { for (int64_t j = rs; j > re; j += step) total++; }                \
    }                                                                          \
    *carrylength = total;                                                      \
    return success();                                                          \
  }
ORACLE_NEXT_RANGE_CARRYLENGTH(awkward_ListArray32_getitem_next_range_carrylength, int32_t)
ORACLE_NEXT_RANGE_CARRYLENGTH(awkward_ListArrayU32_getitem_next_range_carrylength, uint32_t)
ORACLE_NEXT_RANGE_CARRYLENGTH(awkward_ListArray64_getitem_next_range_carrylength, int64_t)

/* awkward_RegularArray_getitem_next_range.cpp:8-19 */
struct Error awkward_RegularArray_getitem_next_range_64(int64_t* tocarry, int64_t regular_start,
                                                       int64_t step, int64_t length,
                                                       int64_t size, int64_t nextsize) {
  for (int64_t i = 0; i < length; i++)
    for (int64_t j = 0; j < nextsize; j++)
      tocarry[i * nextsize + j] = i * size + regular_start + j * step;
  return success();
}

/* ======================================================================
 * Combinations (awkward_ListArray_combinations*.cpp, kernel-utils.cpp:41-98)
 * ====================================================================== */

/* awkward_ListArray_combinations_length.cpp:8-45: C(size, n) by the
 * multiplicative loop (size += n-1 with replacement); no overflow check. */
#define ORACLE_COMBINATIONS_LENGTH(NAME, C)                                    \
  struct Error NAME(int64_t* totallen, int64_t* tooffsets, int64_t n,          \
                    bool replacement, const C* starts, const C* stops,         \
                    int64_t length) {                                          \
    int64_t total = 0;                                                         \
    tooffsets[0] = 0;                                                          \
    for (int64_t i = 0; i < length; i++) {                                     \
      int64_t size = (int64_t)(stops[i] - starts[i]);                          \
      if (replacement) size += n - 1;                                          \
      int64_t thisn = n, len;                                                  \
      if (thisn > size) len = 0;                                               \
      else if (thisn == size) len = 1;                                         \
      else {                                                                   \
        if (thisn * 2 > size) thisn = size - thisn;                            \
        len = size;                                                            \
        for (int64_t j = 2; j <= thisn; j++) { len *= (size - j + 1); len /= j; } \
      }                                                                        \
      total += len;                                                            \
      tooffsets[i + 1] = tooffsets[i] + len;                                   \
    }                                                                          \
    *totallen = total;                                                         \
    return success();                                                          \
  }
ORACLE_COMBINATIONS_LENGTH(awkward_ListArray32_combinations_length_64, int32_t)
ORACLE_COMBINATIONS_LENGTH(awkward_ListArrayU32_combinations_length_64, uint32_t)
ORACLE_COMBINATIONS_LENGTH(awkward_ListArray64_combinations_length_64, int64_t)

/* kernel-utils.cpp:41-80: depth-first lexicographic enumeration of the
 * n-tuples of one list; fromindex[0..n) is the running tuple. */
static void oracle_combinations_step(int64_t** tocarry, int64_t* toindex, int64_t* fromindex,
                                     int64_t j, int64_t stop, int64_t n, bool replacement) {
  while (fromindex[j] < stop) {
    for (int64_t k = j + 1; k < n; k++)
      fromindex[k] = replacement ? fromindex[j] : fromindex[j] + (k - j);
    if (j + 1 == n) {
      for (int64_t k = 0; k < n; k++) tocarry[k][toindex[k]++] = fromindex[k];
    } else {
      oracle_combinations_step(tocarry, toindex, fromindex, j + 1, stop, n, replacement);
    }
    fromindex[j]++;
  }
}

/* awkward_ListArray_combinations.cpp:9-33 */
#define ORACLE_COMBINATIONS(NAME, C)                                           \
  struct Error NAME(int64_t** tocarry, int64_t* toindex, int64_t* fromindex,   \
                    int64_t n, bool replacement, const C* starts, const C* stops, \
                    int64_t length) {                                          \
    for (int64_t j = 0; j < n; j++) toindex[j] = 0;                            \
    for (int64_t i = 0; i < length; i++) {                                     \
      fromindex[0] = (int64_t)starts[i];                                       \
      oracle_combinations_step(tocarry, toindex, fromindex, 0, (int64_t)stops[i], n, \
                               replacement);                                   \
    }                                                                          \
    return success();                                                          \
  }
ORACLE_COMBINATIONS(awkward_ListArray32_combinations_64, int32_t)
ORACLE_COMBINATIONS(awkward_ListArrayU32_combinations_64, uint32_t)
ORACLE_COMBINATIONS(awkward_ListArray64_combinations_64, int64_t)

/* awkward_RegularArray_combinations_64.cpp:8-29: every list is [size*i, size*i + size) */
struct Error awkward_RegularArray_combinations_64(int64_t** tocarry, int64_t* toindex,
                                                  int64_t* fromindex, int64_t n, bool replacement,
                                                  int64_t size, int64_t length) {
  for (int64_t j = 0; j < n; j++) toindex[j] = 0;
  for (int64_t i = 0; i < length; i++) {
    int64_t start = size * i;
    fromindex[0] = start;
    oracle_combinations_step(tocarry, toindex, fromindex, 0, start + size, n, replacement);
  }
  return success();
}

/* ======================================================================
 * Broadcast of a ListArray to given offsets
 * (awkward_ListArray_broadcast_tooffsets.cpp:8-33)
 * ====================================================================== */
#define ORACLE_BROADCAST_TOOFFSETS(NAME, C)                                    \
  struct Error NAME(int64_t* tocarry, const int64_t* fromoffsets,              \
                    int64_t offsetslength, const C* fromstarts,                \
                    const C* fromstops, int64_t lencontent) {                  \
    int64_t k = 0;                                                             \
    for (int64_t i = 0; i < offsetslength - 1; i++) {                          \
      int64_t start = (int64_t)fromstarts[i], stop = (int64_t)fromstops[i];    \
      if (start != stop && stop > lencontent)                                  \
        return failure("stops[i] > len(content)", i, stop);                    \
      int64_t count = fromoffsets[i + 1] - fromoffsets[i];                     \
      if (count < 0)                                                           \
        return failure("broadcast's offsets must be monotonically increasing", \
                       i, kSliceNone);                                         \
      if (stop - start != count)                                               \
        return failure("cannot broadcast nested list", i, kSliceNone);         \
      for (int64_t j = start; j < stop; j++) tocarry[k++] = j;                 \
    }                                                                          \
    return success();                                                          \
  }
ORACLE_BROADCAST_TOOFFSETS(awkward_ListArray32_broadcast_tooffsets_64, int32_t)
ORACLE_BROADCAST_TOOFFSETS(awkward_ListArrayU32_broadcast_tooffsets_64, uint32_t)
ORACLE_BROADCAST_TOOFFSETS(awkward_ListArray64_broadcast_tooffsets_64, int64_t)

/* ======================================================================
 * Segmented sort (awkward_argsort.cpp:62-108, awkward_sort.cpp:62-117)
 * ====================================================================== */

/* The comparators of awkward_argsort.cpp:23-59 / awkward_sort.cpp:23-59:
 * integers and bool compare directly; floating point puts NaN before every
 * number in both directions. */
typedef int (*oracle_less_fn)(const void* x, int64_t a, int64_t b, int asc);
#define ORACLE_LESS_INT(NAME, T)                                               \
  static int NAME(const void* x, int64_t a, int64_t b, int asc) {              \
    T l = ((const T*)x)[a], r = ((const T*)x)[b];                              \
    return asc ? (l < r) : (l > r);                                            \
  }
#define ORACLE_LESS_FLT(NAME, T)                                               \
  static int NAME(const void* x, int64_t a, int64_t b, int asc) {              \
    T l = ((const T*)x)[a], r = ((const T*)x)[b];                              \
    return !isnan(r) && (isnan(l) || (asc ? l < r : l > r));                   \
  }
ORACLE_LESS_INT(oracle_less_bool, bool)
ORACLE_LESS_INT(oracle_less_int8, int8_t)
ORACLE_LESS_INT(oracle_less_uint8, uint8_t)
ORACLE_LESS_INT(oracle_less_int16, int16_t)
ORACLE_LESS_INT(oracle_less_uint16, uint16_t)
ORACLE_LESS_INT(oracle_less_int32, int32_t)
ORACLE_LESS_INT(oracle_less_uint32, uint32_t)
ORACLE_LESS_INT(oracle_less_int64, int64_t)
ORACLE_LESS_INT(oracle_less_uint64, uint64_t)
ORACLE_LESS_FLT(oracle_less_float32, float)
ORACLE_LESS_FLT(oracle_less_float64, double)

/* Stable sort of idx[0..n) by x[idx[.]] (std::stable_sort's contract):
 * bottom-up merge, taking from the right run only when strictly less. */
static void oracle_stable_sort(int64_t* idx, int64_t n, const void* x, oracle_less_fn less,
                               int asc) {
  if (n < 2) return;
  int64_t* tmp = (int64_t*)malloc((size_t)n * sizeof(int64_t));
  int64_t* a = idx;
  int64_t* b = tmp;
  for (int64_t w = 1; w < n; w *= 2) {
    for (int64_t lo = 0; lo < n; lo += 2 * w) {
      int64_t mid = lo + w < n ? lo + w : n, hi = lo + 2 * w < n ? lo + 2 * w : n;
      int64_t i = lo, j = mid, k = lo;
      while (i < mid && j < hi) b[k++] = less(x, a[j], a[i], asc) ? a[j++] : a[i++];
      while (i < mid) b[k++] = a[i++];
      while (j < hi) b[k++] = a[j++];
    }
    int64_t* t = a;
    a = b;
    b = t;
  }
  if (a != idx) memcpy(idx, a, (size_t)n * sizeof(int64_t));
  free(tmp);
}

/* argsort: iota, each clamped segment sorted (stable), then made local. */
#define ORACLE_ARGSORT(NAME, T, U, LESS)                                       \
  struct Error NAME(int64_t* toptr, const T* fromptr, int64_t length,          \
                    const U* offsets, int64_t offsetslength, bool ascending,   \
                    bool stable) {                                             \
    (void)stable;                                                              \
    for (int64_t i = 0; i < length; i++) toptr[i] = i;                         \
    for (int64_t i = 0; i < offsetslength - 1; i++) {                          \
      int64_t st = (int64_t)offsets[i], sp = (int64_t)offsets[i + 1];          \
      if (st > length) st = length;                                            \
      if (sp > length) sp = length;                                            \
      if (st >= sp) continue;                                                  \
      oracle_stable_sort(toptr + st, sp - st, fromptr, LESS, ascending);      \
      for (int64_t j = st; j < sp; j++) toptr[j] -= st;                        \
    }                                                                          \
    return success();                                                          \
  }
#define ORACLE_ARGSORT_ALL(T, SUF, LESS)                                       \
  ORACLE_ARGSORT(awkward_argsort_##SUF##_int32, T, int32_t, LESS)              \
  ORACLE_ARGSORT(awkward_argsort_##SUF##_uint32, T, uint32_t, LESS)            \
  ORACLE_ARGSORT(awkward_argsort_##SUF##_uint64, T, uint64_t, LESS)            \
  ORACLE_ARGSORT(awkward_argsort_##SUF##_int64, T, int64_t, LESS)
ORACLE_ARGSORT_ALL(bool, bool, oracle_less_bool)
ORACLE_ARGSORT_ALL(int8_t, int8, oracle_less_int8)
ORACLE_ARGSORT_ALL(uint8_t, uint8, oracle_less_uint8)
ORACLE_ARGSORT_ALL(int16_t, int16, oracle_less_int16)
ORACLE_ARGSORT_ALL(uint16_t, uint16, oracle_less_uint16)
ORACLE_ARGSORT_ALL(int32_t, int32, oracle_less_int32)
ORACLE_ARGSORT_ALL(uint32_t, uint32, oracle_less_uint32)
ORACLE_ARGSORT_ALL(int64_t, int64, oracle_less_int64)
ORACLE_ARGSORT_ALL(uint64_t, uint64, oracle_less_uint64)
ORACLE_ARGSORT_ALL(float, float32, oracle_less_float32)
ORACLE_ARGSORT_ALL(double, float64, oracle_less_float64)

/* sort: the same on an index, then the first min(offsets[last], length)
 * values gathered through it. */
#define ORACLE_SORT(NAME, T, LESS)                                             \
  struct Error NAME(T* toptr, const T* fromptr, int64_t length,                \
                    const int64_t* offsets, int64_t offsetslength,             \
                    bool ascending, bool stable) {                             \
    (void)stable;                                                              \
    int64_t* index = (int64_t*)malloc((size_t)(length > 0 ? length : 1) * sizeof(int64_t)); \
    for (int64_t i = 0; i < length; i++) index[i] = i;                         \
    for (int64_t i = 0; i < offsetslength - 1; i++) {                          \
      int64_t st = offsets[i], sp = offsets[i + 1];                            \
      if (st > length) st = length;                                            \
      if (sp > length) sp = length;                                            \
      if (st >= sp) continue;                                                  \
      oracle_stable_sort(index + st, sp - st, fromptr, LESS, ascending);      \
    }                                                                          \
    int64_t total = offsetslength > 0 ? offsets[offsetslength - 1] : 0;        \
    int64_t copy = total < length ? total : length;                            \
    for (int64_t i = 0; i < copy; i++) toptr[i] = fromptr[index[i]];           \
    free(index);                                                               \
    return success();                                                          \
  }
ORACLE_SORT(awkward_sort_bool, bool, oracle_less_bool)
ORACLE_SORT(awkward_sort_int8, int8_t, oracle_less_int8)
ORACLE_SORT(awkward_sort_uint8, uint8_t, oracle_less_uint8)
ORACLE_SORT(awkward_sort_int16, int16_t, oracle_less_int16)
ORACLE_SORT(awkward_sort_uint16, uint16_t, oracle_less_uint16)
ORACLE_SORT(awkward_sort_int32, int32_t, oracle_less_int32)
ORACLE_SORT(awkward_sort_uint32, uint32_t, oracle_less_uint32)
ORACLE_SORT(awkward_sort_int64, int64_t, oracle_less_int64)
ORACLE_SORT(awkward_sort_uint64, uint64_t, oracle_less_uint64)
ORACLE_SORT(awkward_sort_float32, float, oracle_less_float32)
ORACLE_SORT(awkward_sort_float64, double, oracle_less_float64)

/* ======================================================================
 * Reductions above the innermost axis and through option types
 * (awkward_ListOffsetArray_reduce_*, awkward_RegularArray_reduce_*,
 *  awkward_IndexedArray_reduce_next*, awkward_ByteMaskedArray_reduce_next*)
 * ====================================================================== */

/* awkward_ListOffsetArray_reduce_nonlocal_maxcount_offsetscopy_64.cpp:7-21 */
struct Error awkward_ListOffsetArray_reduce_nonlocal_maxcount_offsetscopy_64(
    int64_t* maxcount, int64_t* offsetscopy, const int64_t* offsets, int64_t length) {
  int64_t best = 0;
  offsetscopy[0] = offsets[0];
  for (int64_t i = 0; i < length; i++) {
    if (offsets[i + 1] - offsets[i] > best) best = offsets[i + 1] - offsets[i];
    offsetscopy[i + 1] = offsets[i + 1];
  }
  *maxcount = best;
  return success();
}

/* awkward_ListOffsetArray_reduce_nonlocal_preparenext_64.cpp:7-57: the
 * elements of the rows of each outer bin, column by column (bin-major), so
 * next bin b*maxcount + col holds column `col` of every row of bin b that
 * reaches it, rows in order. */
struct Error awkward_ListOffsetArray_reduce_nonlocal_preparenext_64(
    int64_t* nextcarry, int64_t* nextoffsets, int64_t nextlen, int64_t* maxnextparents,
    int64_t* distincts, int64_t distinctslen, int64_t* offsetscopy, const int64_t* offsets,
    int64_t length, const int64_t* outer_offsets, int64_t outlength, int64_t maxcount) {
  (void)nextlen;
  (void)offsetscopy;
  (void)length;
  *maxnextparents = -1;
  for (int64_t i = 0; i < distinctslen; i++) distincts[i] = -1;
  int64_t k = 0;
  nextoffsets[0] = 0;
  for (int64_t b = 0; b < outlength; b++) {
    for (int64_t col = 0; col < maxcount; col++) {
      const int64_t bin = b * maxcount + col;
      const int64_t k0 = k;
      for (int64_t row = outer_offsets[b]; row < outer_offsets[b + 1]; row++)
        if (col < offsets[row + 1] - offsets[row]) nextcarry[k++] = offsets[row] + col;
      nextoffsets[bin + 1] = k;
      if (k > k0) {
        if (bin < distinctslen) distincts[bin] = bin;
        if (bin > *maxnextparents) *maxnextparents = bin;
      }
    }
  }
  return success();
}

/* awkward_ListOffsetArray_reduce_nonlocal_outstartsstops_64.cpp:10-44:
 * sublist k of `distincts` is [k*maxcount, (k+1)*maxcount); it ends after
 * its last entry that is not -1. */
struct Error awkward_ListOffsetArray_reduce_nonlocal_outstartsstops_64(
    int64_t* outstarts, int64_t* outstops, const int64_t* distincts, int64_t lendistincts,
    int64_t outlength) {
  if (outlength > 0 && lendistincts > 0) {
    const int64_t maxcount = lendistincts / outlength;
    int64_t k = 0, next = 0;
    for (int64_t i = 0; i < lendistincts; i++) {
      if (i == next) {
        next += maxcount;
        outstarts[k] = i;
        outstops[k] = i;
        k++;
      }
      if (distincts[i] != -1) outstops[k - 1] = i + 1;
    }
  } else {
    for (int64_t k = 0; k < outlength; k++) outstarts[k] = outstops[k] = 0;
  }
  return success();
}

/* awkward_ListOffsetArray_reduce_nonlocal_nextshifts_64.cpp:7-43:
 * missing[element (row, j)] = rows of the same outer bin up to `row` that
 * end at or before column j; nextshifts gathers it through nextcarry. */
struct Error awkward_ListOffsetArray_reduce_nonlocal_nextshifts_64(
    int64_t* nummissing, int64_t* missing, int64_t* nextshifts, const int64_t* offsets,
    int64_t length, const int64_t* starts, const int64_t* outer_offsets, int64_t outlength,
    int64_t maxcount, int64_t nextlen, const int64_t* nextcarry) {
  (void)length;
  (void)starts;
  for (int64_t b = 0; b < outlength; b++) {
    for (int64_t c = 0; c < maxcount; c++) nummissing[c] = 0;
    for (int64_t row = outer_offsets[b]; row < outer_offsets[b + 1]; row++) {
      const int64_t start = offsets[row], count = offsets[row + 1] - offsets[row];
      for (int64_t c = count; c < maxcount; c++) nummissing[c]++;
      for (int64_t j = 0; j < count; j++) missing[start + j] = nummissing[j];
    }
  }
  for (int64_t j = 0; j < nextlen; j++) nextshifts[j] = missing[nextcarry[j]];
  return success();
}

/* awkward_ListOffsetArray_reduce_local_nextparents_64.cpp:14-27 */
#define ORACLE_LOCAL_NEXTPARENTS(NAME, C)                                      \
  struct Error NAME(C* nextparents, const C* offsets, int64_t length,          \
                    int64_t nextparents_length) {                              \
    const int64_t base = (int64_t)offsets[0];                                  \
    for (int64_t i = 0; i < length; i++)                                       \
      for (int64_t j = (int64_t)offsets[i] - base;                             \
           j < (int64_t)offsets[i + 1] - base && j < nextparents_length; j++)  \
        nextparents[j] = (C)i;                                                 \
    return success();                                                          \
  }
ORACLE_LOCAL_NEXTPARENTS(awkward_ListOffsetArray32_reduce_local_nextparents_64, int32_t)
ORACLE_LOCAL_NEXTPARENTS(awkward_ListOffsetArrayU32_reduce_local_nextparents_64, uint32_t)
ORACLE_LOCAL_NEXTPARENTS(awkward_ListOffsetArray64_reduce_local_nextparents_64, int64_t)

/* awkward_ListOffsetArray_local_preparenext_64.cpp:11-26: the permutation
 * that orders `fromindex` (ties, which the CPU leaves in std::sort's order,
 * are kept in index order here). */
struct Error awkward_ListOffsetArray_local_preparenext_64(int64_t* tocarry,
                                                          const int64_t* fromindex,
                                                          int64_t length) {
  for (int64_t i = 0; i < length; i++) tocarry[i] = i;
  oracle_stable_sort(tocarry, length, fromindex, oracle_less_int64, 1);
  return success();
}

/* awkward_RegularArray_reduce_local_nextparents_64.cpp:14-26 */
struct Error awkward_RegularArray_reduce_local_nextparents_64(int64_t* nextparents, int64_t size,
                                                              int64_t length) {
  int64_t k = 0;
  for (int64_t i = 0; i < length; i++)
    for (int64_t j = 0; j < size; j++) nextparents[k++] = i;
  return success();
}

/* awkward_RegularArray_reduce_nonlocal_preparenext_64.cpp:7-36 */
struct Error awkward_RegularArray_reduce_nonlocal_preparenext_64(
    int64_t* nextcarry, int64_t* nextoffsets, const int64_t* offsets, int64_t size,
    int64_t length, int64_t outlength) {
  (void)length;
  int64_t k = 0;
  nextoffsets[0] = 0;
  for (int64_t b = 0; b < outlength; b++) {
    for (int64_t j = 0; j < size; j++) {
      for (int64_t i = offsets[b]; i < offsets[b + 1]; i++) nextcarry[k++] = i * size + j;
      nextoffsets[b * size + j + 1] = k;
    }
  }
  return success();
}

/* awkward_IndexedArray_reduce_next_64.cpp:7-30: compact the non-missing
 * entries of each bin. */
#define ORACLE_INDEXED_REDUCE_NEXT(NAME, T)                                    \
  struct Error NAME(int64_t* nextcarry, int64_t* nextoffsets, int64_t* outindex, \
                    const T* index, const int64_t* offsets, int64_t outlength) { \
    int64_t k = 0;                                                             \
    nextoffsets[0] = 0;                                                        \
    for (int64_t b = 0; b < outlength; b++) {                                  \
      for (int64_t i = offsets[b]; i < offsets[b + 1]; i++) {                  \
        if ((int64_t)index[i] >= 0) {                                          \
          nextcarry[k] = (int64_t)index[i];                                    \
          outindex[i] = k++;                                                   \
        } else {                                                               \
          outindex[i] = -1;                                                    \
        }                                                                      \
      }                                                                        \
      nextoffsets[b + 1] = k;                                                  \
    }                                                                          \
    return success();                                                          \
  }
ORACLE_INDEXED_REDUCE_NEXT(awkward_IndexedArray32_reduce_next_64, int32_t)
ORACLE_INDEXED_REDUCE_NEXT(awkward_IndexedArrayU32_reduce_next_64, uint32_t)
ORACLE_INDEXED_REDUCE_NEXT(awkward_IndexedArray64_reduce_next_64, int64_t)

/* awkward_IndexedArray_reduce_next_fix_offsets_64.cpp:7-17 */
struct Error awkward_IndexedArray_reduce_next_fix_offsets_64(int64_t* outoffsets,
                                                             const int64_t* starts,
                                                             int64_t startslength,
                                                             int64_t outindexlength) {
  for (int64_t i = 0; i < startslength; i++) outoffsets[i] = starts[i];
  outoffsets[startslength] = outindexlength;
  return success();
}

/* awkward_IndexedArray_reduce_next_nonlocal_nextshifts_64.cpp:7-24 and
 * ..._fromshifts_64.cpp:7-25: for the k-th non-missing entry i, the number
 * of missing entries before it (plus shifts[i]). */
#define ORACLE_INDEXED_NEXTSHIFTS(NAME, T)                                     \
  struct Error NAME(int64_t* nextshifts, const T* index, int64_t length) {     \
    int64_t k = 0;                                                             \
    for (int64_t i = 0; i < length; i++)                                       \
      if ((int64_t)index[i] >= 0) {                                            \
        nextshifts[k] = i - k;                                                 \
        k++;                                                                   \
      }                                                                        \
    return success();                                                          \
  }
#define ORACLE_INDEXED_NEXTSHIFTS_FROM(NAME, T)                                \
  struct Error NAME(int64_t* nextshifts, const T* index, int64_t length,       \
                    const int64_t* shifts) {                                   \
    int64_t k = 0;                                                             \
    for (int64_t i = 0; i < length; i++)                                       \
      if ((int64_t)index[i] >= 0) {                                            \
        nextshifts[k] = shifts[i] + (i - k);                                   \
        k++;                                                                   \
      }                                                                        \
    return success();                                                          \
  }
ORACLE_INDEXED_NEXTSHIFTS(awkward_IndexedArray32_reduce_next_nonlocal_nextshifts_64, int32_t)
ORACLE_INDEXED_NEXTSHIFTS(awkward_IndexedArrayU32_reduce_next_nonlocal_nextshifts_64, uint32_t)
ORACLE_INDEXED_NEXTSHIFTS(awkward_IndexedArray64_reduce_next_nonlocal_nextshifts_64, int64_t)
ORACLE_INDEXED_NEXTSHIFTS_FROM(awkward_IndexedArray32_reduce_next_nonlocal_nextshifts_fromshifts_64, int32_t)
ORACLE_INDEXED_NEXTSHIFTS_FROM(awkward_IndexedArrayU32_reduce_next_nonlocal_nextshifts_fromshifts_64, uint32_t)
ORACLE_INDEXED_NEXTSHIFTS_FROM(awkward_IndexedArray64_reduce_next_nonlocal_nextshifts_fromshifts_64, int64_t)

/* awkward_IndexedArray_local_preparenext_64.cpp:7-31 */
struct Error awkward_IndexedArray_local_preparenext_64(int64_t* tocarry, const int64_t* starts,
                                                       const int64_t* offsets,
                                                       const int64_t* nextoffsets,
                                                       int64_t outlength) {
  (void)starts;
  for (int64_t b = 0; b < outlength; b++) {
    int64_t k = nextoffsets[b];
    for (int64_t i = offsets[b]; i < offsets[b + 1]; i++)
      tocarry[i] = k < nextoffsets[b + 1] ? k++ : -1;
  }
  return success();
}

/* awkward_ByteMaskedArray_reduce_next_64.cpp:7-32 */
struct Error awkward_ByteMaskedArray_reduce_next_64(int64_t* nextcarry, int64_t* nextoffsets,
                                                    int64_t* outindex, const int8_t* mask,
                                                    const int64_t* offsets, int64_t outlength,
                                                    bool validwhen) {
  int64_t k = 0;
  nextoffsets[0] = 0;
  for (int64_t b = 0; b < outlength; b++) {
    for (int64_t i = offsets[b]; i < offsets[b + 1]; i++) {
      if ((mask[i] != 0) == validwhen) {
        nextcarry[k] = i;
        outindex[i] = k++;
      } else {
        outindex[i] = -1;
      }
    }
    nextoffsets[b + 1] = k;
  }
  return success();
}

/* awkward_ByteMaskedArray_reduce_next_nonlocal_nextshifts_64.cpp:7-25 and
 * ..._fromshifts_64.cpp:7-26 */
struct Error awkward_ByteMaskedArray_reduce_next_nonlocal_nextshifts_64(int64_t* nextshifts,
                                                                        const int8_t* mask,
                                                                        int64_t length,
                                                                        bool valid_when) {
  int64_t k = 0;
  for (int64_t i = 0; i < length; i++)
    if ((mask[i] != 0) == valid_when) {
      nextshifts[k] = i - k;
      k++;
    }
  return success();
}
struct Error awkward_ByteMaskedArray_reduce_next_nonlocal_nextshifts_fromshifts_64(
    int64_t* nextshifts, const int8_t* mask, int64_t length, bool valid_when,
    const int64_t* shifts) {
  int64_t k = 0;
  for (int64_t i = 0; i < length; i++)
    if ((mask[i] != 0) == valid_when) {
      nextshifts[k] = shifts[i] + (i - k);
      k++;
    }
  return success();
}

/* ======================================================================
 * Complex reducers (interleaved re, im): awkward_reduce_*_complex.cpp
 * ====================================================================== */

/* awkward_reduce_sum_complex.cpp:7-24 */
#define ORACLE_SUM_COMPLEX(NAME, T)                                            \
  struct Error NAME(T* toptr, const T* fromptr, const int64_t* offsets,        \
                    int64_t outlength) {                                       \
    for (int64_t b = 0; b < outlength; b++) {                                  \
      T re = 0, im = 0;                                                        \
      for (int64_t i = offsets[b]; i < offsets[b + 1]; i++) {                  \
        re += fromptr[2 * i];                                                  \
        im += fromptr[2 * i + 1];                                              \
      }                                                                        \
      toptr[2 * b] = re;                                                       \
      toptr[2 * b + 1] = im;                                                   \
    }                                                                          \
    return success();                                                          \
  }
ORACLE_SUM_COMPLEX(awkward_reduce_sum_complex64_complex64_64, float)
ORACLE_SUM_COMPLEX(awkward_reduce_sum_complex128_complex128_64, double)

/* awkward_reduce_prod_complex.cpp:9-31 */
#define ORACLE_PROD_COMPLEX(NAME, T)                                           \
  struct Error NAME(T* toptr, const T* fromptr, const int64_t* offsets,        \
                    int64_t outlength) {                                       \
    for (int64_t b = 0; b < outlength; b++) {                                  \
      T a = 1, bb = 0;                                                         \
      for (int64_t i = offsets[b]; i < offsets[b + 1]; i++) {                  \
        const T c = fromptr[2 * i], d = fromptr[2 * i + 1];                    \
        const T na = a * c - bb * d, nb = a * d + bb * c;                      \
        a = na;                                                                \
        bb = nb;                                                               \
      }                                                                        \
      toptr[2 * b] = a;                                                        \
      toptr[2 * b + 1] = bb;                                                   \
    }                                                                          \
    return success();                                                          \
  }
ORACLE_PROD_COMPLEX(awkward_reduce_prod_complex64_complex64_64, float)
ORACLE_PROD_COMPLEX(awkward_reduce_prod_complex128_complex128_64, double)

/* awkward_reduce_max_complex.cpp:7-33 / awkward_reduce_min_complex.cpp:7-33:
 * the first element seeds; a later one replaces the best when it is
 * lexicographically greater (smaller) by (re, im). */
#define ORACLE_EXT_COMPLEX(NAME, T, OP)                                        \
  struct Error NAME(T* toptr, const T* fromptr, const int64_t* offsets,        \
                    int64_t outlength, T identity) {                           \
    for (int64_t b = 0; b < outlength; b++) {                                  \
      T bre = identity, bim = 0;                                               \
      int seen = 0;                                                            \
      for (int64_t i = offsets[b]; i < offsets[b + 1]; i++) {                  \
        const T x = fromptr[2 * i], y = fromptr[2 * i + 1];                    \
        if (!seen || x OP bre || (x == bre && y OP bim)) {                     \
          bre = x;                                                             \
          bim = y;                                                             \
          seen = 1;                                                            \
        }                                                                      \
      }                                                                        \
      toptr[2 * b] = bre;                                                      \
      toptr[2 * b + 1] = bim;                                                  \
    }                                                                          \
    return success();                                                          \
  }
ORACLE_EXT_COMPLEX(awkward_reduce_max_complex64_complex64_64, float, >)
ORACLE_EXT_COMPLEX(awkward_reduce_max_complex128_complex128_64, double, >)
ORACLE_EXT_COMPLEX(awkward_reduce_min_complex64_complex64_64, float, <)
ORACLE_EXT_COMPLEX(awkward_reduce_min_complex128_complex128_64, double, <)

/* awkward_reduce_argmax_complex.cpp:7-33 / argmin: the global index of that element. */
#define ORACLE_ARG_COMPLEX(NAME, T, OP)                                        \
  struct Error NAME(int64_t* toptr, const T* fromptr, const int64_t* offsets,  \
                    int64_t outlength) {                                       \
    for (int64_t b = 0; b < outlength; b++) {                                  \
      int64_t best = -1;                                                       \
      for (int64_t i = offsets[b]; i < offsets[b + 1]; i++) {                  \
        if (best == -1) {                                                      \
          best = i;                                                            \
        } else {                                                               \
          const T x = fromptr[2 * i], y = fromptr[2 * i + 1];                  \
          const T bx = fromptr[2 * best], by = fromptr[2 * best + 1];          \
          if (x OP bx || (x == bx && y OP by)) best = i;                       \
        }                                                                      \
      }                                                                        \
      toptr[b] = best;                                                         \
    }                                                                          \
    return success();                                                          \
  }
ORACLE_ARG_COMPLEX(awkward_reduce_argmax_complex64_64, float, >)
ORACLE_ARG_COMPLEX(awkward_reduce_argmax_complex128_64, double, >)
ORACLE_ARG_COMPLEX(awkward_reduce_argmin_complex64_64, float, <)
ORACLE_ARG_COMPLEX(awkward_reduce_argmin_complex128_64, double, <)

/* awkward_reduce_countnonzero_complex.cpp:7-21, _sum_bool_complex (any element
 * nonzero), _prod_bool_complex (every element nonzero). */
#define ORACLE_NONZERO_COMPLEX(NAME, OUT, T, MODE)                             \
  struct Error NAME(OUT* toptr, const T* fromptr, const int64_t* offsets,      \
                    int64_t outlength) {                                       \
    for (int64_t b = 0; b < outlength; b++) {                                  \
      int64_t nz = 0, n = offsets[b + 1] - offsets[b];                         \
      for (int64_t i = offsets[b]; i < offsets[b + 1]; i++)                    \
        nz += (fromptr[2 * i] != 0 || fromptr[2 * i + 1] != 0);                \
      toptr[b] = MODE == 0 ? (OUT)nz : MODE == 1 ? (OUT)(nz > 0) : (OUT)(nz == n || n <= 0); \
    }                                                                          \
    return success();                                                          \
  }
ORACLE_NONZERO_COMPLEX(awkward_reduce_countnonzero_complex64_64, int64_t, float, 0)
ORACLE_NONZERO_COMPLEX(awkward_reduce_countnonzero_complex128_64, int64_t, double, 0)
ORACLE_NONZERO_COMPLEX(awkward_reduce_sum_bool_complex64_64, bool, float, 1)
ORACLE_NONZERO_COMPLEX(awkward_reduce_sum_bool_complex128_64, bool, double, 1)
ORACLE_NONZERO_COMPLEX(awkward_reduce_prod_bool_complex64_64, bool, float, 2)
ORACLE_NONZERO_COMPLEX(awkward_reduce_prod_bool_complex128_64, bool, double, 2)

/* ======================================================================
 * List-layout conversions (ListArray -> offsets, regular carries)
 * ====================================================================== */

/* awkward_ListArray_compact_offsets.cpp:7-23 */
#define ORACLE_COMPACT_OFFSETS(NAME, C)                                        \
  struct Error NAME(int64_t* tooffsets, const C* fromstarts, const C* fromstops, \
                    int64_t length) {                                          \
    tooffsets[0] = 0;                                                          \
    for (int64_t i = 0; i < length; i++) {                                     \
      if (fromstops[i] < fromstarts[i])                                        \
        return failure("stops[i] < starts[i]", i, kSliceNone);                 \
      tooffsets[i + 1] = tooffsets[i] + (int64_t)(fromstops[i] - fromstarts[i]); \
    }                                                                          \
    return success();                                                          \
  }
ORACLE_COMPACT_OFFSETS(awkward_ListArray32_compact_offsets_64, int32_t)
ORACLE_COMPACT_OFFSETS(awkward_ListArrayU32_compact_offsets_64, uint32_t)
ORACLE_COMPACT_OFFSETS(awkward_ListArray64_compact_offsets_64, int64_t)

/* awkward_RegularArray_getitem_carry.cpp:7-19 */
struct Error awkward_RegularArray_getitem_carry_64(int64_t* tocarry, const int64_t* fromcarry,
                                                   int64_t lencarry, int64_t size) {
  for (int64_t i = 0; i < lencarry; i++)
    for (int64_t j = 0; j < size; j++) tocarry[i * size + j] = fromcarry[i] * size + j;
  return success();
}

/* awkward_RegularArray_localindex.cpp:7-18 */
struct Error awkward_RegularArray_localindex_64(int64_t* toindex, int64_t size, int64_t length) {
  for (int64_t i = 0; i < length; i++)
    for (int64_t j = 0; j < size; j++) toindex[i * size + j] = j;
  return success();
}

/* ======================================================================
 * Small siblings on the same driver paths
 * ====================================================================== */

/* awkward_NumpyArray_reduce_adjust_starts_shifts_64.cpp:7-23 */
struct Error awkward_NumpyArray_reduce_adjust_starts_shifts_64(int64_t* toptr, int64_t outlength,
                                                               const int64_t* offsets,
                                                               const int64_t* starts,
                                                               const int64_t* shifts) {
  (void)offsets;
  for (int64_t k = 0; k < outlength; k++) {
    const int64_t i = toptr[k];
    if (i >= 0) toptr[k] += shifts[i] - starts[k];
  }
  return success();
}

/* awkward_localindex.cpp:8-14 */
struct Error awkward_localindex_64(int64_t* toindex, int64_t length) {
  for (int64_t i = 0; i < length; i++) toindex[i] = i;
  return success();
}

/* awkward_ListArray_getitem_next_range_counts.cpp:7-18 */
#define ORACLE_RANGE_COUNTS(NAME, C)                                           \
  struct Error NAME(int64_t* total, const C* fromoffsets, int64_t lenstarts) { \
    *total = 0;                                                                \
    for (int64_t i = 0; i < lenstarts; i++)                                    \
      *total = *total + fromoffsets[i + 1] - fromoffsets[i];                   \
    return success();                                                          \
  }
ORACLE_RANGE_COUNTS(awkward_ListArray32_getitem_next_range_counts_64, int32_t)
ORACLE_RANGE_COUNTS(awkward_ListArrayU32_getitem_next_range_counts_64, uint32_t)
ORACLE_RANGE_COUNTS(awkward_ListArray64_getitem_next_range_counts_64, int64_t)

/* awkward_ListArray_getitem_next_range_spreadadvanced.cpp:7-21 */
#define ORACLE_RANGE_SPREAD(NAME, C)                                           \
  struct Error NAME(int64_t* toadvanced, const int64_t* fromadvanced,          \
                    const C* fromoffsets, int64_t lenstarts) {                 \
    for (int64_t i = 0; i < lenstarts; i++) {                                  \
      const C count = fromoffsets[i + 1] - fromoffsets[i];                     \
      for (int64_t j = 0; j < (int64_t)count; j++)                             \
        toadvanced[fromoffsets[i] + j] = fromadvanced[i];                      \
    }                                                                          \
    return success();                                                          \
  }
ORACLE_RANGE_SPREAD(awkward_ListArray32_getitem_next_range_spreadadvanced_64, int32_t)
ORACLE_RANGE_SPREAD(awkward_ListArrayU32_getitem_next_range_spreadadvanced_64, uint32_t)
ORACLE_RANGE_SPREAD(awkward_ListArray64_getitem_next_range_spreadadvanced_64, int64_t)

/* awkward_RegularArray_getitem_next_range_spreadadvanced.cpp:7-19 */
struct Error awkward_RegularArray_getitem_next_range_spreadadvanced_64(int64_t* toadvanced,
                                                                       const int64_t* fromadvanced,
                                                                       int64_t length,
                                                                       int64_t nextsize) {
  for (int64_t i = 0; i < length; i++)
    for (int64_t j = 0; j < nextsize; j++) toadvanced[i * nextsize + j] = fromadvanced[i];
  return success();
}

/* awkward_Content_getitem_next_missing_jagged_getmaskstartstop.cpp:7-28 */
struct Error awkward_Content_getitem_next_missing_jagged_getmaskstartstop(
    int64_t* index_in, int64_t* offsets_in, int64_t* mask_out, int64_t* starts_out,
    int64_t* stops_out, int64_t length) {
  int64_t k = 0;
  for (int64_t i = 0; i < length; i++) {
    starts_out[i] = offsets_in[k];
    if (index_in[i] < 0) {
      mask_out[i] = -1;
    } else {
      mask_out[i] = i;
      k++;
    }
    stops_out[i] = offsets_in[k];
  }
  return success();
}

/* awkward_MaskedArray_getitem_next_jagged_project.cpp:7-25 */
#define ORACLE_JAGGED_PROJECT(NAME, T)                                         \
  struct Error NAME(T* index, int64_t* starts_in, int64_t* stops_in,           \
                    int64_t* starts_out, int64_t* stops_out, int64_t length) { \
    int64_t k = 0;                                                             \
    for (int64_t i = 0; i < length; i++)                                       \
      if ((int64_t)index[i] >= 0) {                                            \
        starts_out[k] = starts_in[i];                                          \
        stops_out[k] = stops_in[i];                                            \
        k++;                                                                   \
      }                                                                        \
    return success();                                                          \
  }
ORACLE_JAGGED_PROJECT(awkward_MaskedArray32_getitem_next_jagged_project, int32_t)
ORACLE_JAGGED_PROJECT(awkward_MaskedArrayU32_getitem_next_jagged_project, uint32_t)
ORACLE_JAGGED_PROJECT(awkward_MaskedArray64_getitem_next_jagged_project, int64_t)

/* ======================================================================
 * FP64 compensated per-list sums: the accuracy reference for float sums.
 * awkward-cpp's sum (awkward_reduce_sum.cpp:17-23) adds left to right and
 * rounds after every addition, so it carries up to (n-1)*u*sum|x| of error
 * (u = 2^-53); the GPU sums in a different order.  Both are judged against
 * this double-double accumulation instead: every addition is made
 * error-free with Knuth's TwoSum (s + x = s' + e exactly, in round-to-
 * nearest double arithmetic, no fused operations) and the errors are
 * accumulated in a second double, so the result is within u*|S| +
 * n*u^2*sum|x| of the exact sum S.  Lists holding an infinity or a NaN take
 * the plain left-to-right sum (IEEE: inf + -inf = NaN).
 *
 * out[2b] = the compensated sum of list b, out[2b+1] = sum|x| over it (the
 * scale of the error bound).  The signature matches the reducers above, so
 * oracle_parallel_reduce can split it over threads (output size 16 bytes).
 * ====================================================================== */
#define ORACLE_SUM_COMPENSATED(NAME, IN)                                       \
  struct Error NAME(double* out, const IN* fromptr, const int64_t* offsets,    \
                    int64_t outlength) {                                       \
    for (int64_t b = 0; b < outlength; b++) {                                  \
      double s = 0.0, c = 0.0, plain = 0.0, a = 0.0;                           \
      for (int64_t i = offsets[b]; i < offsets[b + 1]; i++) {                  \
        const double x = (double)fromptr[i];                                   \
        const double t = s + x;                                                \
        const double bp = t - s;                                               \
        const double e = (s - (t - bp)) + (x - bp);                            \
        s = t;                                                                 \
        c += e;                                                                \
        plain += x;                                                            \
        a += fabs(x);                                                          \
      }                                                                        \
      out[2 * b] = isfinite(plain) ? s + c : plain;                            \
      out[2 * b + 1] = a;                                                      \
    }                                                                          \
    return success();                                                          \
  }
ORACLE_SUM_COMPENSATED(oracle_sum_compensated_float64, double)
ORACLE_SUM_COMPENSATED(oracle_sum_compensated_float32, float)

/* ======================================================================
 * Multi-core runner for the CPU baseline: run one reducer (any of the
 * (toptr, fromptr, offsets, outlength) family above, or argmax/argmin with
 * `starts`) over `nthreads` contiguous list ranges.  Each thread calls the
 * single-threaded restatement on its own range; ranges never share an output.
 * ====================================================================== */
typedef struct Error (*oracle_reduce4_fn)(void*, const void*, const int64_t*, int64_t);
typedef struct Error (*oracle_reduce5_fn)(void*, const void*, const int64_t*, const int64_t*, int64_t);
typedef struct Error (*oracle_reduce_ident_fn)(void*, const void*, const int64_t*, int64_t, double);

typedef struct {
  void* fn;
  int kind; /* 4 = (to, from, offsets, n); 5 = argmax form (to, from, offsets, starts, n);
               6 = float64 max/min form (to, from, offsets, n, identity) */
  double identity;
  char* toptr;
  const void* fromptr;
  const int64_t* offsets;
  int64_t lo, hi;
  size_t outsize;
} oracle_job;

static void* oracle_job_run(void* p) {
  oracle_job* j = (oracle_job*)p;
  if (j->kind == 4)
    ((oracle_reduce4_fn)j->fn)(j->toptr + j->lo * j->outsize, j->fromptr, j->offsets + j->lo,
                               j->hi - j->lo);
  else if (j->kind == 6)
    ((oracle_reduce_ident_fn)j->fn)(j->toptr + j->lo * j->outsize, j->fromptr, j->offsets + j->lo,
                                    j->hi - j->lo, j->identity);
  else
    ((oracle_reduce5_fn)j->fn)(j->toptr + j->lo * j->outsize, j->fromptr, j->offsets + j->lo,
                               NULL, j->hi - j->lo);
  return NULL;
}

int oracle_parallel_reduce_ident(void* fn, int kind, void* toptr, size_t outsize,
                                 const void* fromptr, const int64_t* offsets, int64_t outlength,
                                 int nthreads, double identity);
int oracle_parallel_reduce(void* fn, int kind, void* toptr, size_t outsize, const void* fromptr,
                           const int64_t* offsets, int64_t outlength, int nthreads) {
  return oracle_parallel_reduce_ident(fn, kind, toptr, outsize, fromptr, offsets, outlength,
                                      nthreads, 0.0);
}

int oracle_parallel_reduce_ident(void* fn, int kind, void* toptr, size_t outsize,
                                 const void* fromptr, const int64_t* offsets, int64_t outlength,
                                 int nthreads, double identity) {
  if (nthreads < 1) nthreads = 1;
  if (nthreads > 256) nthreads = 256;
  pthread_t th[256];
  oracle_job jobs[256];
  for (int t = 0; t < nthreads; t++) {
    jobs[t].fn = fn;
    jobs[t].kind = kind;
    jobs[t].toptr = (char*)toptr;
    jobs[t].fromptr = fromptr;
    jobs[t].offsets = offsets;
    jobs[t].lo = outlength * t / nthreads;
    jobs[t].hi = outlength * (t + 1) / nthreads;
    jobs[t].outsize = outsize;
    jobs[t].identity = identity;
    if (pthread_create(&th[t], NULL, oracle_job_run, &jobs[t]) != 0) return -1;
  }
  for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
  return 0;
}
