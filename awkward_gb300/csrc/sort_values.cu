// sort_values.cu -- awkward_sort for every value type (segmented sort
// kernels: sort_impl.cuh).
#include "sort_impl.cuh"

GB_SORT(bool, bool)
GB_SORT(int8, int8_t)
GB_SORT(uint8, uint8_t)
GB_SORT(int16, int16_t)
GB_SORT(uint16, uint16_t)
GB_SORT(int32, int32_t)
GB_SORT(uint32, uint32_t)
GB_SORT(int64, int64_t)
GB_SORT(uint64, uint64_t)
GB_SORT(float32, float)
GB_SORT(float64, double)
