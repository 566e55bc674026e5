// sort_argsort_narrow.cu -- awkward_argsort for bool and the 8/16/32-bit
// signed integer value types (segmented sort kernels: sort_impl.cuh).
#include "sort_impl.cuh"

GB_ARGSORT_ALL(bool, bool)
GB_ARGSORT_ALL(int8, int8_t)
GB_ARGSORT_ALL(uint8, uint8_t)
GB_ARGSORT_ALL(int16, int16_t)
GB_ARGSORT_ALL(uint16, uint16_t)
GB_ARGSORT_ALL(int32, int32_t)
