// Entry points of awkward_reduce_sum (kernel-specification.yml:5035) and
// awkward_reduce_sum_int32_bool_64 / _int64_bool_64 (:5581, :5599).
#include "reduce_ops.cuh"

using namespace gb;

#define GB_SUM(NAME, OUT, IN)                                                                  \
  GB_EXPORT int NAME(OUT* toptr, const IN* fromptr, const int64_t* offsets, int64_t outlength, \
                     uint64_t invocation_index, uint64_t* err_code, void* stream) {            \
    return (int)launch_seg_reduce(SumOp<OUT, IN>{},                                            \
                                  reinterpret_cast<const store_t<IN>*>(fromptr), offsets,      \
                                  outlength, toptr, invocation_index, err_code,                \
                                  (cudaStream_t)stream);                                       \
  }

// float64 results of floating inputs: exact fixed-point accumulation (no
// per-element float64 arithmetic)
#define GB_FSUM(NAME, IN)                                                                      \
  GB_EXPORT int NAME(double* toptr, const IN* fromptr, const int64_t* offsets, int64_t outlength, \
                     uint64_t invocation_index, uint64_t* err_code, void* stream) {            \
    return (int)launch_seg_reduce(FixedSumOp<IN>{}, fromptr, offsets, outlength, toptr,        \
                                  invocation_index, err_code, (cudaStream_t)stream);           \
  }

GB_SUM(awkward_reduce_sum_int64_int8_64, int64_t, int8_t)
GB_SUM(awkward_reduce_sum_uint64_uint8_64, uint64_t, uint8_t)
GB_SUM(awkward_reduce_sum_int64_int16_64, int64_t, int16_t)
GB_SUM(awkward_reduce_sum_uint64_uint16_64, uint64_t, uint16_t)
GB_SUM(awkward_reduce_sum_int64_int32_64, int64_t, int32_t)
GB_SUM(awkward_reduce_sum_uint64_uint32_64, uint64_t, uint32_t)
GB_SUM(awkward_reduce_sum_int64_int64_64, int64_t, int64_t)
GB_SUM(awkward_reduce_sum_uint64_uint64_64, uint64_t, uint64_t)
GB_SUM(awkward_reduce_sum_float32_float32_64, float, float)
GB_FSUM(awkward_reduce_sum_float64_float64_64, double)
GB_SUM(awkward_reduce_sum_int32_int8_64, int32_t, int8_t)
GB_SUM(awkward_reduce_sum_uint32_uint8_64, uint32_t, uint8_t)
GB_SUM(awkward_reduce_sum_int32_int16_64, int32_t, int16_t)
GB_SUM(awkward_reduce_sum_uint32_uint16_64, uint32_t, uint16_t)
GB_SUM(awkward_reduce_sum_int32_int32_64, int32_t, int32_t)
GB_SUM(awkward_reduce_sum_uint32_uint32_64, uint32_t, uint32_t)
GB_SUM(awkward_reduce_sum_float64_int8_64, double, int8_t)
GB_SUM(awkward_reduce_sum_float64_uint8_64, double, uint8_t)
GB_SUM(awkward_reduce_sum_float64_int16_64, double, int16_t)
GB_SUM(awkward_reduce_sum_float64_uint16_64, double, uint16_t)
GB_SUM(awkward_reduce_sum_float64_int32_64, double, int32_t)
GB_SUM(awkward_reduce_sum_float64_uint32_64, double, uint32_t)
GB_SUM(awkward_reduce_sum_float64_int64_64, double, int64_t)
GB_SUM(awkward_reduce_sum_float64_uint64_64, double, uint64_t)
GB_FSUM(awkward_reduce_sum_float64_float32_64, float)
GB_SUM(awkward_reduce_sum_int32_bool_64, int32_t, bool)
GB_SUM(awkward_reduce_sum_int64_bool_64, int64_t, bool)
