/* libawkward_gb300: GB300 (sm_103a) kernels for awkward's jagged hot path.
 *
 * Generated by awkward_gb300/gen_signatures.py from awkward's
 * kernel-specification.yml; do not edit by hand.
 *
 * Every entry point keeps the name and the argument list of one
 * specialization of kernel-specification.yml (cited per declaration as
 * kernel-specification.yml:<line>, with the awkward-cpp CPU template it
 * replaces), so a ctypes adapter can install it into awkward's cupy
 * kernel table keyed by (family, *dtypes).  Differences from the spec:
 *   - every pointer is a DEVICE pointer; List[List[T]] is a device array
 *     of device pointers;
 *   - three trailing arguments follow the spec's arguments:
 *       uint64_t  invocation_index  index of this call in the caller's
 *                                   pending-invocation list;
 *       uint64_t* err_code          device word; a failing kernel does
 *                                   atomicMin(err_code,
 *                                     invocation_index*256 + message)
 *                                   (awkward's RawModule protocol) and
 *                                   kernels skip work when it is set;
 *       void*     stream            cudaStream_t to launch on (0 = legacy).
 *   - the return value is the cudaError_t of the launch (0 = success);
 *     data errors are reported only through err_code.
 * Outputs are preallocated by the caller.  Temporary buffers (tile
 * states of the single-pass scans) come from a stream-ordered pool owned
 * by the library and are released in stream order.
 */
#ifndef AWKWARD_GB300_H_
#define AWKWARD_GB300_H_

#include <stdint.h>
#include <stdbool.h>

#ifdef __cplusplus
extern "C" {
#endif

#define AWKWARD_GB300_ERROR_BITS 8
#define AWKWARD_GB300_NO_ERROR 0xffffffffffffffffULL

/* ---- awkward_ByteMaskedArray_reduce_next_64: replaces awkward-cpp/src/cpu-kernels/awkward_ByteMaskedArray_reduce_next_64.cpp:7 */
/* kernel-specification.yml:233 */
int awkward_ByteMaskedArray_reduce_next_64(int64_t* nextcarry, int64_t* nextoffsets, int64_t* outindex, const int8_t* mask, const int64_t* offsets, int64_t outlength, bool validwhen, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* ---- awkward_ByteMaskedArray_reduce_next_nonlocal_nextshifts_64: replaces awkward-cpp/src/cpu-kernels/awkward_ByteMaskedArray_reduce_next_nonlocal_nextshifts_64.cpp:7 */
/* kernel-specification.yml:261 */
int awkward_ByteMaskedArray_reduce_next_nonlocal_nextshifts_64(int64_t* nextshifts, const int8_t* mask, int64_t length, bool valid_when, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* ---- awkward_ByteMaskedArray_reduce_next_nonlocal_nextshifts_fromshifts_64: replaces awkward-cpp/src/cpu-kernels/awkward_ByteMaskedArray_reduce_next_nonlocal_nextshifts_fromshifts_64.cpp:7 */
/* kernel-specification.yml:284 */
int awkward_ByteMaskedArray_reduce_next_nonlocal_nextshifts_fromshifts_64(int64_t* nextshifts, const int8_t* mask, int64_t length, bool valid_when, const int64_t* shifts, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* ---- awkward_Content_getitem_next_missing_jagged_getmaskstartstop: replaces awkward-cpp/src/cpu-kernels/awkward_Content_getitem_next_missing_jagged_getmaskstartstop.cpp:7 */
/* kernel-specification.yml:323 */
int awkward_Content_getitem_next_missing_jagged_getmaskstartstop(int64_t* index_in, int64_t* offsets_in, int64_t* mask_out, int64_t* starts_out, int64_t* stops_out, int64_t length, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* ---- awkward_IndexedArray_local_preparenext_64: replaces awkward-cpp/src/cpu-kernels/awkward_IndexedArray_local_preparenext_64.cpp:7 */
/* kernel-specification.yml:549 */
int awkward_IndexedArray_local_preparenext_64(int64_t* tocarry, const int64_t* starts, const int64_t* offsets, const int64_t* nextoffsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* ---- awkward_IndexedArray_reduce_next_64: replaces awkward-cpp/src/cpu-kernels/awkward_IndexedArray_reduce_next_64.cpp:7 */
/* kernel-specification.yml:707 */
int awkward_IndexedArray32_reduce_next_64(int64_t* nextcarry, int64_t* nextoffsets, int64_t* outindex, const int32_t* index, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:715 */
int awkward_IndexedArray64_reduce_next_64(int64_t* nextcarry, int64_t* nextoffsets, int64_t* outindex, const int64_t* index, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:723 */
int awkward_IndexedArrayU32_reduce_next_64(int64_t* nextcarry, int64_t* nextoffsets, int64_t* outindex, const uint32_t* index, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* ---- awkward_IndexedArray_reduce_next_fix_offsets_64: replaces awkward-cpp/src/cpu-kernels/awkward_IndexedArray_reduce_next_fix_offsets_64.cpp:7 */
/* kernel-specification.yml:750 */
int awkward_IndexedArray_reduce_next_fix_offsets_64(int64_t* outoffsets, const int64_t* starts, int64_t startslength, int64_t outindexlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* ---- awkward_IndexedArray_reduce_next_nonlocal_nextshifts_64: replaces awkward-cpp/src/cpu-kernels/awkward_IndexedArray_reduce_next_nonlocal_nextshifts_64.cpp:7 */
/* kernel-specification.yml:799 */
int awkward_IndexedArray32_reduce_next_nonlocal_nextshifts_64(int64_t* nextshifts, const int32_t* index, int64_t length, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:804 */
int awkward_IndexedArray64_reduce_next_nonlocal_nextshifts_64(int64_t* nextshifts, const int64_t* index, int64_t length, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:809 */
int awkward_IndexedArrayU32_reduce_next_nonlocal_nextshifts_64(int64_t* nextshifts, const uint32_t* index, int64_t length, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* ---- awkward_IndexedArray_reduce_next_nonlocal_nextshifts_fromshifts_64: replaces awkward-cpp/src/cpu-kernels/awkward_IndexedArray_reduce_next_nonlocal_nextshifts_fromshifts_64.cpp:7 */
/* kernel-specification.yml:829 */
int awkward_IndexedArray32_reduce_next_nonlocal_nextshifts_fromshifts_64(int64_t* nextshifts, const int32_t* index, int64_t length, const int64_t* shifts, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:835 */
int awkward_IndexedArray64_reduce_next_nonlocal_nextshifts_fromshifts_64(int64_t* nextshifts, const int64_t* index, int64_t length, const int64_t* shifts, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:841 */
int awkward_IndexedArrayU32_reduce_next_nonlocal_nextshifts_fromshifts_64(int64_t* nextshifts, const uint32_t* index, int64_t length, const int64_t* shifts, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* ---- awkward_ListArray_broadcast_tooffsets: replaces awkward-cpp/src/cpu-kernels/awkward_ListArray_broadcast_tooffsets.cpp:8 */
/* kernel-specification.yml:1080 */
int awkward_ListArray32_broadcast_tooffsets_64(int64_t* tocarry, const int64_t* fromoffsets, int64_t offsetslength, const int32_t* fromstarts, const int32_t* fromstops, int64_t lencontent, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:1088 */
int awkward_ListArray64_broadcast_tooffsets_64(int64_t* tocarry, const int64_t* fromoffsets, int64_t offsetslength, const int64_t* fromstarts, const int64_t* fromstops, int64_t lencontent, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:1096 */
int awkward_ListArrayU32_broadcast_tooffsets_64(int64_t* tocarry, const int64_t* fromoffsets, int64_t offsetslength, const uint32_t* fromstarts, const uint32_t* fromstops, int64_t lencontent, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* ---- awkward_ListArray_combinations: replaces awkward-cpp/src/cpu-kernels/awkward_ListArray_combinations.cpp:9 */
/* kernel-specification.yml:1127 */
int awkward_ListArray32_combinations_64(int64_t** tocarry, int64_t* toindex, int64_t* fromindex, int64_t n, bool replacement, const int32_t* starts, const int32_t* stops, int64_t length, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:1137 */
int awkward_ListArray64_combinations_64(int64_t** tocarry, int64_t* toindex, int64_t* fromindex, int64_t n, bool replacement, const int64_t* starts, const int64_t* stops, int64_t length, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:1147 */
int awkward_ListArrayU32_combinations_64(int64_t** tocarry, int64_t* toindex, int64_t* fromindex, int64_t n, bool replacement, const uint32_t* starts, const uint32_t* stops, int64_t length, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* ---- awkward_ListArray_combinations_length: replaces awkward-cpp/src/cpu-kernels/awkward_ListArray_combinations_length.cpp:8 */
/* kernel-specification.yml:1177 */
int awkward_ListArray32_combinations_length_64(int64_t* totallen, int64_t* tooffsets, int64_t n, bool replacement, const int32_t* starts, const int32_t* stops, int64_t length, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:1186 */
int awkward_ListArray64_combinations_length_64(int64_t* totallen, int64_t* tooffsets, int64_t n, bool replacement, const int64_t* starts, const int64_t* stops, int64_t length, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:1195 */
int awkward_ListArrayU32_combinations_length_64(int64_t* totallen, int64_t* tooffsets, int64_t n, bool replacement, const uint32_t* starts, const uint32_t* stops, int64_t length, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* ---- awkward_ListArray_compact_offsets: replaces awkward-cpp/src/cpu-kernels/awkward_ListArray_compact_offsets.cpp:7 */
/* kernel-specification.yml:1237 */
int awkward_ListArray32_compact_offsets_64(int64_t* tooffsets, const int32_t* fromstarts, const int32_t* fromstops, int64_t length, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:1243 */
int awkward_ListArray64_compact_offsets_64(int64_t* tooffsets, const int64_t* fromstarts, const int64_t* fromstops, int64_t length, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:1249 */
int awkward_ListArrayU32_compact_offsets_64(int64_t* tooffsets, const uint32_t* fromstarts, const uint32_t* fromstops, int64_t length, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* ---- awkward_ListArray_getitem_jagged_apply: replaces awkward-cpp/src/cpu-kernels/awkward_ListArray_getitem_jagged_apply.cpp:8 */
/* kernel-specification.yml:1318 */
int awkward_ListArray32_getitem_jagged_apply_64(int64_t* tooffsets, int64_t* tocarry, const int64_t* slicestarts, const int64_t* slicestops, int64_t sliceouterlen, const int64_t* sliceindex, int64_t sliceinnerlen, const int32_t* fromstarts, const int32_t* fromstops, int64_t contentlen, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:1330 */
int awkward_ListArray64_getitem_jagged_apply_64(int64_t* tooffsets, int64_t* tocarry, const int64_t* slicestarts, const int64_t* slicestops, int64_t sliceouterlen, const int64_t* sliceindex, int64_t sliceinnerlen, const int64_t* fromstarts, const int64_t* fromstops, int64_t contentlen, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:1342 */
int awkward_ListArrayU32_getitem_jagged_apply_64(int64_t* tooffsets, int64_t* tocarry, const int64_t* slicestarts, const int64_t* slicestops, int64_t sliceouterlen, const int64_t* sliceindex, int64_t sliceinnerlen, const uint32_t* fromstarts, const uint32_t* fromstops, int64_t contentlen, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* ---- awkward_ListArray_getitem_jagged_carrylen: replaces awkward-cpp/src/cpu-kernels/awkward_ListArray_getitem_jagged_carrylen.cpp:8 */
/* kernel-specification.yml:1398 */
int awkward_ListArray_getitem_jagged_carrylen_64(int64_t* carrylen, const int64_t* slicestarts, const int64_t* slicestops, int64_t sliceouterlen, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* ---- awkward_ListArray_getitem_jagged_descend: replaces awkward-cpp/src/cpu-kernels/awkward_ListArray_getitem_jagged_descend.cpp:8 */
/* kernel-specification.yml:1416 */
int awkward_ListArray32_getitem_jagged_descend_64(int64_t* tooffsets, const int64_t* slicestarts, const int64_t* slicestops, int64_t sliceouterlen, const int32_t* fromstarts, const int32_t* fromstops, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:1424 */
int awkward_ListArray64_getitem_jagged_descend_64(int64_t* tooffsets, const int64_t* slicestarts, const int64_t* slicestops, int64_t sliceouterlen, const int64_t* fromstarts, const int64_t* fromstops, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:1432 */
int awkward_ListArrayU32_getitem_jagged_descend_64(int64_t* tooffsets, const int64_t* slicestarts, const int64_t* slicestops, int64_t sliceouterlen, const uint32_t* fromstarts, const uint32_t* fromstops, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* ---- awkward_ListArray_getitem_jagged_expand: replaces awkward-cpp/src/cpu-kernels/awkward_ListArray_getitem_jagged_expand.cpp:8 */
/* kernel-specification.yml:1461 */
int awkward_ListArray32_getitem_jagged_expand_64(int64_t* multistarts, int64_t* multistops, const int64_t* singleoffsets, int64_t* tocarry, const int32_t* fromstarts, const int32_t* fromstops, int64_t jaggedsize, int64_t length, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:1471 */
int awkward_ListArray64_getitem_jagged_expand_64(int64_t* multistarts, int64_t* multistops, const int64_t* singleoffsets, int64_t* tocarry, const int64_t* fromstarts, const int64_t* fromstops, int64_t jaggedsize, int64_t length, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:1481 */
int awkward_ListArrayU32_getitem_jagged_expand_64(int64_t* multistarts, int64_t* multistops, const int64_t* singleoffsets, int64_t* tocarry, const uint32_t* fromstarts, const uint32_t* fromstops, int64_t jaggedsize, int64_t length, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* ---- awkward_ListArray_getitem_jagged_numvalid: replaces awkward-cpp/src/cpu-kernels/awkward_ListArray_getitem_jagged_numvalid.cpp:8 */
/* kernel-specification.yml:1518 */
int awkward_ListArray_getitem_jagged_numvalid_64(int64_t* numvalid, const int64_t* slicestarts, const int64_t* slicestops, int64_t length, const int64_t* missing, int64_t missinglength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* ---- awkward_ListArray_getitem_jagged_shrink: replaces awkward-cpp/src/cpu-kernels/awkward_ListArray_getitem_jagged_shrink.cpp:8 */
/* kernel-specification.yml:1547 */
int awkward_ListArray_getitem_jagged_shrink_64(int64_t* tocarry, int64_t* tosmalloffsets, int64_t* tolargeoffsets, const int64_t* slicestarts, const int64_t* slicestops, int64_t length, const int64_t* missing, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* ---- awkward_ListArray_getitem_next_range: replaces awkward-cpp/src/cpu-kernels/awkward_ListArray_getitem_next_range.cpp:9 */
/* kernel-specification.yml:1741 */
int awkward_ListArray32_getitem_next_range_64(int32_t* tooffsets, int64_t* tocarry, const int32_t* fromstarts, const int32_t* fromstops, int64_t lenstarts, int64_t start, int64_t stop, int64_t step, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:1751 */
int awkward_ListArray64_getitem_next_range_64(int64_t* tooffsets, int64_t* tocarry, const int64_t* fromstarts, const int64_t* fromstops, int64_t lenstarts, int64_t start, int64_t stop, int64_t step, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:1761 */
int awkward_ListArrayU32_getitem_next_range_64(uint32_t* tooffsets, int64_t* tocarry, const uint32_t* fromstarts, const uint32_t* fromstops, int64_t lenstarts, int64_t start, int64_t stop, int64_t step, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* ---- awkward_ListArray_getitem_next_range_carrylength: replaces awkward-cpp/src/cpu-kernels/awkward_ListArray_getitem_next_range_carrylength.cpp:9 */
/* kernel-specification.yml:1806 */
int awkward_ListArray32_getitem_next_range_carrylength(int64_t* carrylength, const int32_t* fromstarts, const int32_t* fromstops, int64_t lenstarts, int64_t start, int64_t stop, int64_t step, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:1815 */
int awkward_ListArray64_getitem_next_range_carrylength(int64_t* carrylength, const int64_t* fromstarts, const int64_t* fromstops, int64_t lenstarts, int64_t start, int64_t stop, int64_t step, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:1824 */
int awkward_ListArrayU32_getitem_next_range_carrylength(int64_t* carrylength, const uint32_t* fromstarts, const uint32_t* fromstops, int64_t lenstarts, int64_t start, int64_t stop, int64_t step, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* ---- awkward_ListArray_getitem_next_range_counts: replaces awkward-cpp/src/cpu-kernels/awkward_ListArray_getitem_next_range_counts.cpp:7 */
/* kernel-specification.yml:1865 */
int awkward_ListArray32_getitem_next_range_counts_64(int64_t* total, const int32_t* fromoffsets, int64_t lenstarts, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:1870 */
int awkward_ListArray64_getitem_next_range_counts_64(int64_t* total, const int64_t* fromoffsets, int64_t lenstarts, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:1875 */
int awkward_ListArrayU32_getitem_next_range_counts_64(int64_t* total, const uint32_t* fromoffsets, int64_t lenstarts, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* ---- awkward_ListArray_getitem_next_range_spreadadvanced: replaces awkward-cpp/src/cpu-kernels/awkward_ListArray_getitem_next_range_spreadadvanced.cpp:7 */
/* kernel-specification.yml:1890 */
int awkward_ListArray32_getitem_next_range_spreadadvanced_64(int64_t* toadvanced, const int64_t* fromadvanced, const int32_t* fromoffsets, int64_t lenstarts, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:1896 */
int awkward_ListArray64_getitem_next_range_spreadadvanced_64(int64_t* toadvanced, const int64_t* fromadvanced, const int64_t* fromoffsets, int64_t lenstarts, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:1902 */
int awkward_ListArrayU32_getitem_next_range_spreadadvanced_64(int64_t* toadvanced, const int64_t* fromadvanced, const uint32_t* fromoffsets, int64_t lenstarts, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* ---- awkward_ListArray_localindex: replaces awkward-cpp/src/cpu-kernels/awkward_ListArray_localindex.cpp:8 */
/* kernel-specification.yml:1921 */
int awkward_ListArray32_localindex_64(int64_t* toindex, const int32_t* offsets, int64_t length, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:1926 */
int awkward_ListArray64_localindex_64(int64_t* toindex, const int64_t* offsets, int64_t length, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:1931 */
int awkward_ListArrayU32_localindex_64(int64_t* toindex, const uint32_t* offsets, int64_t length, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* ---- awkward_ListOffsetArray_local_preparenext_64: replaces awkward-cpp/src/cpu-kernels/awkward_ListOffsetArray_local_preparenext_64.cpp:11 */
/* kernel-specification.yml:2153 */
int awkward_ListOffsetArray_local_preparenext_64(int64_t* tocarry, const int64_t* fromindex, int64_t length, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* ---- awkward_ListOffsetArray_reduce_local_nextparents_64: replaces awkward-cpp/src/cpu-kernels/awkward_ListOffsetArray_reduce_local_nextparents_64.cpp:14 */
/* kernel-specification.yml:2168 */
int awkward_ListOffsetArray32_reduce_local_nextparents_64(int32_t* nextparents, const int32_t* offsets, int64_t length, int64_t nextparents_length, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:2174 */
int awkward_ListOffsetArray64_reduce_local_nextparents_64(int64_t* nextparents, const int64_t* offsets, int64_t length, int64_t nextparents_length, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:2180 */
int awkward_ListOffsetArrayU32_reduce_local_nextparents_64(uint32_t* nextparents, const uint32_t* offsets, int64_t length, int64_t nextparents_length, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* ---- awkward_ListOffsetArray_reduce_nonlocal_maxcount_offsetscopy_64: replaces awkward-cpp/src/cpu-kernels/awkward_ListOffsetArray_reduce_nonlocal_maxcount_offsetscopy_64.cpp:7 */
/* kernel-specification.yml:2199 */
int awkward_ListOffsetArray_reduce_nonlocal_maxcount_offsetscopy_64(int64_t* maxcount, int64_t* offsetscopy, const int64_t* offsets, int64_t length, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* ---- awkward_ListOffsetArray_reduce_nonlocal_nextshifts_64: replaces awkward-cpp/src/cpu-kernels/awkward_ListOffsetArray_reduce_nonlocal_nextshifts_64.cpp:7 */
/* kernel-specification.yml:2221 */
int awkward_ListOffsetArray_reduce_nonlocal_nextshifts_64(int64_t* nummissing, int64_t* missing, int64_t* nextshifts, const int64_t* offsets, int64_t length, const int64_t* starts, const int64_t* outer_offsets, int64_t outlength, int64_t maxcount, int64_t nextlen, const int64_t* nextcarry, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* ---- awkward_ListOffsetArray_reduce_nonlocal_outstartsstops_64: replaces awkward-cpp/src/cpu-kernels/awkward_ListOffsetArray_reduce_nonlocal_outstartsstops_64.cpp:10 */
/* kernel-specification.yml:2258 */
int awkward_ListOffsetArray_reduce_nonlocal_outstartsstops_64(int64_t* outstarts, int64_t* outstops, const int64_t* distincts, int64_t lendistincts, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* ---- awkward_ListOffsetArray_reduce_nonlocal_preparenext_64: replaces awkward-cpp/src/cpu-kernels/awkward_ListOffsetArray_reduce_nonlocal_preparenext_64.cpp:7 */
/* kernel-specification.yml:2298 */
int awkward_ListOffsetArray_reduce_nonlocal_preparenext_64(int64_t* nextcarry, int64_t* nextoffsets, int64_t nextlen, int64_t* maxnextparents, int64_t* distincts, int64_t distinctslen, int64_t* offsetscopy, const int64_t* offsets, int64_t length, const int64_t* outer_offsets, int64_t outlength, int64_t maxcount, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* ---- awkward_MaskedArray_getitem_next_jagged_project: replaces awkward-cpp/src/cpu-kernels/awkward_MaskedArray_getitem_next_jagged_project.cpp:7 */
/* kernel-specification.yml:2486 */
int awkward_MaskedArray32_getitem_next_jagged_project(int32_t* index, int64_t* starts_in, int64_t* stops_in, int64_t* starts_out, int64_t* stops_out, int64_t length, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:2494 */
int awkward_MaskedArray64_getitem_next_jagged_project(int64_t* index, int64_t* starts_in, int64_t* stops_in, int64_t* starts_out, int64_t* stops_out, int64_t length, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:2502 */
int awkward_MaskedArrayU32_getitem_next_jagged_project(uint32_t* index, int64_t* starts_in, int64_t* stops_in, int64_t* starts_out, int64_t* stops_out, int64_t length, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* ---- awkward_NumpyArray_reduce_adjust_starts_64: replaces awkward-cpp/src/cpu-kernels/awkward_NumpyArray_reduce_adjust_starts_64.cpp:7 */
/* kernel-specification.yml:2552 */
int awkward_NumpyArray_reduce_adjust_starts_64(int64_t* toptr, int64_t outlength, const int64_t* offsets, const int64_t* starts, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* ---- awkward_NumpyArray_reduce_adjust_starts_shifts_64: replaces awkward-cpp/src/cpu-kernels/awkward_NumpyArray_reduce_adjust_starts_shifts_64.cpp:7 */
/* kernel-specification.yml:2568 */
int awkward_NumpyArray_reduce_adjust_starts_shifts_64(int64_t* toptr, int64_t outlength, const int64_t* offsets, const int64_t* starts, const int64_t* shifts, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* ---- awkward_NumpyArray_reduce_mask_ByteMaskedArray_64: replaces awkward-cpp/src/cpu-kernels/awkward_NumpyArray_reduce_mask_ByteMaskedArray_64.cpp:7 */
/* kernel-specification.yml:2587 */
int awkward_NumpyArray_reduce_mask_ByteMaskedArray_64(int8_t* toptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* ---- awkward_RegularArray_combinations_64: replaces awkward-cpp/src/cpu-kernels/awkward_RegularArray_combinations_64.cpp:8 */
/* kernel-specification.yml:2868 */
int awkward_RegularArray_combinations_64(int64_t** tocarry, int64_t* toindex, int64_t* fromindex, int64_t n, bool replacement, int64_t size, int64_t length, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* ---- awkward_RegularArray_getitem_carry: replaces awkward-cpp/src/cpu-kernels/awkward_RegularArray_getitem_carry.cpp:7 */
/* kernel-specification.yml:2896 */
int awkward_RegularArray_getitem_carry_64(int64_t* tocarry, const int64_t* fromcarry, int64_t lencarry, int64_t size, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* ---- awkward_RegularArray_getitem_jagged_expand: replaces awkward-cpp/src/cpu-kernels/awkward_RegularArray_getitem_jagged_expand.cpp:8 */
/* kernel-specification.yml:2912 */
int awkward_RegularArray_getitem_jagged_expand_64(int64_t* multistarts, int64_t* multistops, const int64_t* singleoffsets, int64_t regularsize, int64_t regularlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* ---- awkward_RegularArray_getitem_next_range: replaces awkward-cpp/src/cpu-kernels/awkward_RegularArray_getitem_next_range.cpp:8 */
/* kernel-specification.yml:3014 */
int awkward_RegularArray_getitem_next_range_64(int64_t* tocarry, int64_t regular_start, int64_t step, int64_t length, int64_t size, int64_t nextsize, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* ---- awkward_RegularArray_getitem_next_range_spreadadvanced: replaces awkward-cpp/src/cpu-kernels/awkward_RegularArray_getitem_next_range_spreadadvanced.cpp:7 */
/* kernel-specification.yml:3034 */
int awkward_RegularArray_getitem_next_range_spreadadvanced_64(int64_t* toadvanced, const int64_t* fromadvanced, int64_t length, int64_t nextsize, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* ---- awkward_RegularArray_localindex: replaces awkward-cpp/src/cpu-kernels/awkward_RegularArray_localindex.cpp:7 */
/* kernel-specification.yml:3052 */
int awkward_RegularArray_localindex_64(int64_t* toindex, int64_t size, int64_t length, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* ---- awkward_RegularArray_reduce_local_nextparents_64: replaces awkward-cpp/src/cpu-kernels/awkward_RegularArray_reduce_local_nextparents_64.cpp:14 */
/* kernel-specification.yml:3067 */
int awkward_RegularArray_reduce_local_nextparents_64(int64_t* nextparents, int64_t size, int64_t length, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* ---- awkward_RegularArray_reduce_nonlocal_preparenext_64: replaces awkward-cpp/src/cpu-kernels/awkward_RegularArray_reduce_nonlocal_preparenext_64.cpp:7 */
/* kernel-specification.yml:3085 */
int awkward_RegularArray_reduce_nonlocal_preparenext_64(int64_t* nextcarry, int64_t* nextoffsets, const int64_t* offsets, int64_t size, int64_t length, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* ---- awkward_argsort: replaces awkward-cpp/src/cpu-kernels/awkward_argsort.cpp:62 */
/* kernel-specification.yml:3724 */
int awkward_argsort_bool_int32(int64_t* toptr, const bool* fromptr, int64_t length, const int32_t* offsets, int64_t offsetslength, bool ascending, bool stable, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:3733 */
int awkward_argsort_bool_uint32(int64_t* toptr, const bool* fromptr, int64_t length, const uint32_t* offsets, int64_t offsetslength, bool ascending, bool stable, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:3742 */
int awkward_argsort_bool_uint64(int64_t* toptr, const bool* fromptr, int64_t length, const uint64_t* offsets, int64_t offsetslength, bool ascending, bool stable, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:3751 */
int awkward_argsort_bool_int64(int64_t* toptr, const bool* fromptr, int64_t length, const int64_t* offsets, int64_t offsetslength, bool ascending, bool stable, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:3760 */
int awkward_argsort_int8_int32(int64_t* toptr, const int8_t* fromptr, int64_t length, const int32_t* offsets, int64_t offsetslength, bool ascending, bool stable, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:3769 */
int awkward_argsort_int8_uint32(int64_t* toptr, const int8_t* fromptr, int64_t length, const uint32_t* offsets, int64_t offsetslength, bool ascending, bool stable, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:3778 */
int awkward_argsort_int8_uint64(int64_t* toptr, const int8_t* fromptr, int64_t length, const uint64_t* offsets, int64_t offsetslength, bool ascending, bool stable, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:3787 */
int awkward_argsort_int8_int64(int64_t* toptr, const int8_t* fromptr, int64_t length, const int64_t* offsets, int64_t offsetslength, bool ascending, bool stable, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:3796 */
int awkward_argsort_int16_int32(int64_t* toptr, const int16_t* fromptr, int64_t length, const int32_t* offsets, int64_t offsetslength, bool ascending, bool stable, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:3805 */
int awkward_argsort_int16_uint32(int64_t* toptr, const int16_t* fromptr, int64_t length, const uint32_t* offsets, int64_t offsetslength, bool ascending, bool stable, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:3814 */
int awkward_argsort_int16_uint64(int64_t* toptr, const int16_t* fromptr, int64_t length, const uint64_t* offsets, int64_t offsetslength, bool ascending, bool stable, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:3823 */
int awkward_argsort_int16_int64(int64_t* toptr, const int16_t* fromptr, int64_t length, const int64_t* offsets, int64_t offsetslength, bool ascending, bool stable, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:3832 */
int awkward_argsort_int32_int32(int64_t* toptr, const int32_t* fromptr, int64_t length, const int32_t* offsets, int64_t offsetslength, bool ascending, bool stable, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:3841 */
int awkward_argsort_int32_uint32(int64_t* toptr, const int32_t* fromptr, int64_t length, const uint32_t* offsets, int64_t offsetslength, bool ascending, bool stable, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:3850 */
int awkward_argsort_int32_uint64(int64_t* toptr, const int32_t* fromptr, int64_t length, const uint64_t* offsets, int64_t offsetslength, bool ascending, bool stable, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:3859 */
int awkward_argsort_int32_int64(int64_t* toptr, const int32_t* fromptr, int64_t length, const int64_t* offsets, int64_t offsetslength, bool ascending, bool stable, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:3868 */
int awkward_argsort_int64_int32(int64_t* toptr, const int64_t* fromptr, int64_t length, const int32_t* offsets, int64_t offsetslength, bool ascending, bool stable, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:3877 */
int awkward_argsort_int64_uint32(int64_t* toptr, const int64_t* fromptr, int64_t length, const uint32_t* offsets, int64_t offsetslength, bool ascending, bool stable, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:3886 */
int awkward_argsort_int64_uint64(int64_t* toptr, const int64_t* fromptr, int64_t length, const uint64_t* offsets, int64_t offsetslength, bool ascending, bool stable, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:3895 */
int awkward_argsort_int64_int64(int64_t* toptr, const int64_t* fromptr, int64_t length, const int64_t* offsets, int64_t offsetslength, bool ascending, bool stable, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:3904 */
int awkward_argsort_uint8_int32(int64_t* toptr, const uint8_t* fromptr, int64_t length, const int32_t* offsets, int64_t offsetslength, bool ascending, bool stable, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:3913 */
int awkward_argsort_uint8_uint32(int64_t* toptr, const uint8_t* fromptr, int64_t length, const uint32_t* offsets, int64_t offsetslength, bool ascending, bool stable, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:3922 */
int awkward_argsort_uint8_uint64(int64_t* toptr, const uint8_t* fromptr, int64_t length, const uint64_t* offsets, int64_t offsetslength, bool ascending, bool stable, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:3931 */
int awkward_argsort_uint8_int64(int64_t* toptr, const uint8_t* fromptr, int64_t length, const int64_t* offsets, int64_t offsetslength, bool ascending, bool stable, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:3940 */
int awkward_argsort_uint16_int32(int64_t* toptr, const uint16_t* fromptr, int64_t length, const int32_t* offsets, int64_t offsetslength, bool ascending, bool stable, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:3949 */
int awkward_argsort_uint16_uint32(int64_t* toptr, const uint16_t* fromptr, int64_t length, const uint32_t* offsets, int64_t offsetslength, bool ascending, bool stable, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:3958 */
int awkward_argsort_uint16_uint64(int64_t* toptr, const uint16_t* fromptr, int64_t length, const uint64_t* offsets, int64_t offsetslength, bool ascending, bool stable, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:3967 */
int awkward_argsort_uint16_int64(int64_t* toptr, const uint16_t* fromptr, int64_t length, const int64_t* offsets, int64_t offsetslength, bool ascending, bool stable, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:3976 */
int awkward_argsort_uint32_int32(int64_t* toptr, const uint32_t* fromptr, int64_t length, const int32_t* offsets, int64_t offsetslength, bool ascending, bool stable, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:3985 */
int awkward_argsort_uint32_uint32(int64_t* toptr, const uint32_t* fromptr, int64_t length, const uint32_t* offsets, int64_t offsetslength, bool ascending, bool stable, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:3994 */
int awkward_argsort_uint32_uint64(int64_t* toptr, const uint32_t* fromptr, int64_t length, const uint64_t* offsets, int64_t offsetslength, bool ascending, bool stable, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4003 */
int awkward_argsort_uint32_int64(int64_t* toptr, const uint32_t* fromptr, int64_t length, const int64_t* offsets, int64_t offsetslength, bool ascending, bool stable, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4012 */
int awkward_argsort_uint64_int32(int64_t* toptr, const uint64_t* fromptr, int64_t length, const int32_t* offsets, int64_t offsetslength, bool ascending, bool stable, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4021 */
int awkward_argsort_uint64_uint32(int64_t* toptr, const uint64_t* fromptr, int64_t length, const uint32_t* offsets, int64_t offsetslength, bool ascending, bool stable, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4030 */
int awkward_argsort_uint64_uint64(int64_t* toptr, const uint64_t* fromptr, int64_t length, const uint64_t* offsets, int64_t offsetslength, bool ascending, bool stable, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4039 */
int awkward_argsort_uint64_int64(int64_t* toptr, const uint64_t* fromptr, int64_t length, const int64_t* offsets, int64_t offsetslength, bool ascending, bool stable, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4048 */
int awkward_argsort_float32_int32(int64_t* toptr, const float* fromptr, int64_t length, const int32_t* offsets, int64_t offsetslength, bool ascending, bool stable, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4057 */
int awkward_argsort_float32_uint32(int64_t* toptr, const float* fromptr, int64_t length, const uint32_t* offsets, int64_t offsetslength, bool ascending, bool stable, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4066 */
int awkward_argsort_float32_uint64(int64_t* toptr, const float* fromptr, int64_t length, const uint64_t* offsets, int64_t offsetslength, bool ascending, bool stable, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4075 */
int awkward_argsort_float32_int64(int64_t* toptr, const float* fromptr, int64_t length, const int64_t* offsets, int64_t offsetslength, bool ascending, bool stable, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4084 */
int awkward_argsort_float64_int32(int64_t* toptr, const double* fromptr, int64_t length, const int32_t* offsets, int64_t offsetslength, bool ascending, bool stable, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4093 */
int awkward_argsort_float64_uint32(int64_t* toptr, const double* fromptr, int64_t length, const uint32_t* offsets, int64_t offsetslength, bool ascending, bool stable, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4102 */
int awkward_argsort_float64_uint64(int64_t* toptr, const double* fromptr, int64_t length, const uint64_t* offsets, int64_t offsetslength, bool ascending, bool stable, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4111 */
int awkward_argsort_float64_int64(int64_t* toptr, const double* fromptr, int64_t length, const int64_t* offsets, int64_t offsetslength, bool ascending, bool stable, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* ---- awkward_localindex: replaces awkward-cpp/src/cpu-kernels/awkward_localindex.cpp:8 */
/* kernel-specification.yml:4196 */
int awkward_localindex_64(int64_t* toindex, int64_t length, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* ---- awkward_reduce_argmax: replaces awkward-cpp/src/cpu-kernels/awkward_reduce_argmax.cpp:9 */
/* kernel-specification.yml:4227 */
int awkward_reduce_argmax_int8_64(int64_t* toptr, const int8_t* fromptr, const int64_t* offsets, const int64_t* starts, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4234 */
int awkward_reduce_argmax_uint8_64(int64_t* toptr, const uint8_t* fromptr, const int64_t* offsets, const int64_t* starts, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4241 */
int awkward_reduce_argmax_int16_64(int64_t* toptr, const int16_t* fromptr, const int64_t* offsets, const int64_t* starts, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4248 */
int awkward_reduce_argmax_uint16_64(int64_t* toptr, const uint16_t* fromptr, const int64_t* offsets, const int64_t* starts, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4255 */
int awkward_reduce_argmax_int32_64(int64_t* toptr, const int32_t* fromptr, const int64_t* offsets, const int64_t* starts, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4262 */
int awkward_reduce_argmax_uint32_64(int64_t* toptr, const uint32_t* fromptr, const int64_t* offsets, const int64_t* starts, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4269 */
int awkward_reduce_argmax_int64_64(int64_t* toptr, const int64_t* fromptr, const int64_t* offsets, const int64_t* starts, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4276 */
int awkward_reduce_argmax_uint64_64(int64_t* toptr, const uint64_t* fromptr, const int64_t* offsets, const int64_t* starts, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4283 */
int awkward_reduce_argmax_float32_64(int64_t* toptr, const float* fromptr, const int64_t* offsets, const int64_t* starts, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4290 */
int awkward_reduce_argmax_float64_64(int64_t* toptr, const double* fromptr, const int64_t* offsets, const int64_t* starts, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* ---- awkward_reduce_argmax_complex: replaces awkward-cpp/src/cpu-kernels/awkward_reduce_argmax_complex.cpp:7 */
/* kernel-specification.yml:4309 */
int awkward_reduce_argmax_complex64_64(int64_t* toptr, const float* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4315 */
int awkward_reduce_argmax_complex128_64(int64_t* toptr, const double* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* ---- awkward_reduce_argmin: replaces awkward-cpp/src/cpu-kernels/awkward_reduce_argmin.cpp:25 */
/* kernel-specification.yml:4338 */
int awkward_reduce_argmin_int8_64(int64_t* toptr, const int8_t* fromptr, const int64_t* offsets, const int64_t* starts, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4345 */
int awkward_reduce_argmin_uint8_64(int64_t* toptr, const uint8_t* fromptr, const int64_t* offsets, const int64_t* starts, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4352 */
int awkward_reduce_argmin_int16_64(int64_t* toptr, const int16_t* fromptr, const int64_t* offsets, const int64_t* starts, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4359 */
int awkward_reduce_argmin_uint16_64(int64_t* toptr, const uint16_t* fromptr, const int64_t* offsets, const int64_t* starts, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4366 */
int awkward_reduce_argmin_int32_64(int64_t* toptr, const int32_t* fromptr, const int64_t* offsets, const int64_t* starts, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4373 */
int awkward_reduce_argmin_uint32_64(int64_t* toptr, const uint32_t* fromptr, const int64_t* offsets, const int64_t* starts, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4380 */
int awkward_reduce_argmin_int64_64(int64_t* toptr, const int64_t* fromptr, const int64_t* offsets, const int64_t* starts, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4387 */
int awkward_reduce_argmin_uint64_64(int64_t* toptr, const uint64_t* fromptr, const int64_t* offsets, const int64_t* starts, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4394 */
int awkward_reduce_argmin_float32_64(int64_t* toptr, const float* fromptr, const int64_t* offsets, const int64_t* starts, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4401 */
int awkward_reduce_argmin_float64_64(int64_t* toptr, const double* fromptr, const int64_t* offsets, const int64_t* starts, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* ---- awkward_reduce_argmin_complex: replaces awkward-cpp/src/cpu-kernels/awkward_reduce_argmin_complex.cpp:7 */
/* kernel-specification.yml:4420 */
int awkward_reduce_argmin_complex64_64(int64_t* toptr, const float* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4426 */
int awkward_reduce_argmin_complex128_64(int64_t* toptr, const double* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* ---- awkward_reduce_count_64: replaces awkward-cpp/src/cpu-kernels/awkward_reduce_count_64.cpp:7 */
/* kernel-specification.yml:4449 */
int awkward_reduce_count_64(int64_t* toptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* ---- awkward_reduce_countnonzero: replaces awkward-cpp/src/cpu-kernels/awkward_reduce_countnonzero.cpp:14 */
/* kernel-specification.yml:4462 */
int awkward_reduce_countnonzero_bool_64(int64_t* toptr, const bool* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4468 */
int awkward_reduce_countnonzero_int8_64(int64_t* toptr, const int8_t* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4474 */
int awkward_reduce_countnonzero_uint8_64(int64_t* toptr, const uint8_t* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4480 */
int awkward_reduce_countnonzero_int16_64(int64_t* toptr, const int16_t* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4486 */
int awkward_reduce_countnonzero_uint16_64(int64_t* toptr, const uint16_t* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4492 */
int awkward_reduce_countnonzero_int32_64(int64_t* toptr, const int32_t* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4498 */
int awkward_reduce_countnonzero_uint32_64(int64_t* toptr, const uint32_t* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4504 */
int awkward_reduce_countnonzero_int64_64(int64_t* toptr, const int64_t* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4510 */
int awkward_reduce_countnonzero_uint64_64(int64_t* toptr, const uint64_t* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4516 */
int awkward_reduce_countnonzero_float32_64(int64_t* toptr, const float* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4522 */
int awkward_reduce_countnonzero_float64_64(int64_t* toptr, const double* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* ---- awkward_reduce_countnonzero_complex: replaces awkward-cpp/src/cpu-kernels/awkward_reduce_countnonzero_complex.cpp:7 */
/* kernel-specification.yml:4540 */
int awkward_reduce_countnonzero_complex64_64(int64_t* toptr, const float* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4546 */
int awkward_reduce_countnonzero_complex128_64(int64_t* toptr, const double* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* ---- awkward_reduce_max: replaces awkward-cpp/src/cpu-kernels/awkward_reduce_max.cpp:9 */
/* kernel-specification.yml:4564 */
int awkward_reduce_max_int8_int8_64(int8_t* toptr, const int8_t* fromptr, const int64_t* offsets, int64_t outlength, int8_t identity, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4571 */
int awkward_reduce_max_uint8_uint8_64(uint8_t* toptr, const uint8_t* fromptr, const int64_t* offsets, int64_t outlength, uint8_t identity, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4578 */
int awkward_reduce_max_int16_int16_64(int16_t* toptr, const int16_t* fromptr, const int64_t* offsets, int64_t outlength, int16_t identity, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4585 */
int awkward_reduce_max_uint16_uint16_64(uint16_t* toptr, const uint16_t* fromptr, const int64_t* offsets, int64_t outlength, uint16_t identity, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4592 */
int awkward_reduce_max_int32_int32_64(int32_t* toptr, const int32_t* fromptr, const int64_t* offsets, int64_t outlength, int32_t identity, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4599 */
int awkward_reduce_max_uint32_uint32_64(uint32_t* toptr, const uint32_t* fromptr, const int64_t* offsets, int64_t outlength, uint32_t identity, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4606 */
int awkward_reduce_max_int64_int64_64(int64_t* toptr, const int64_t* fromptr, const int64_t* offsets, int64_t outlength, int64_t identity, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4613 */
int awkward_reduce_max_uint64_uint64_64(uint64_t* toptr, const uint64_t* fromptr, const int64_t* offsets, int64_t outlength, uint64_t identity, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4620 */
int awkward_reduce_max_float32_float32_64(float* toptr, const float* fromptr, const int64_t* offsets, int64_t outlength, float identity, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4627 */
int awkward_reduce_max_float64_float64_64(double* toptr, const double* fromptr, const int64_t* offsets, int64_t outlength, double identity, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* ---- awkward_reduce_max_complex: replaces awkward-cpp/src/cpu-kernels/awkward_reduce_max_complex.cpp:7 */
/* kernel-specification.yml:4647 */
int awkward_reduce_max_complex64_complex64_64(float* toptr, const float* fromptr, const int64_t* offsets, int64_t outlength, float identity, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4654 */
int awkward_reduce_max_complex128_complex128_64(double* toptr, const double* fromptr, const int64_t* offsets, int64_t outlength, double identity, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* ---- awkward_reduce_min: replaces awkward-cpp/src/cpu-kernels/awkward_reduce_min.cpp:26 */
/* kernel-specification.yml:4680 */
int awkward_reduce_min_int8_int8_64(int8_t* toptr, const int8_t* fromptr, const int64_t* offsets, int64_t outlength, int8_t identity, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4687 */
int awkward_reduce_min_uint8_uint8_64(uint8_t* toptr, const uint8_t* fromptr, const int64_t* offsets, int64_t outlength, uint8_t identity, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4694 */
int awkward_reduce_min_int16_int16_64(int16_t* toptr, const int16_t* fromptr, const int64_t* offsets, int64_t outlength, int16_t identity, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4701 */
int awkward_reduce_min_uint16_uint16_64(uint16_t* toptr, const uint16_t* fromptr, const int64_t* offsets, int64_t outlength, uint16_t identity, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4708 */
int awkward_reduce_min_int32_int32_64(int32_t* toptr, const int32_t* fromptr, const int64_t* offsets, int64_t outlength, int32_t identity, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4715 */
int awkward_reduce_min_uint32_uint32_64(uint32_t* toptr, const uint32_t* fromptr, const int64_t* offsets, int64_t outlength, uint32_t identity, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4722 */
int awkward_reduce_min_int64_int64_64(int64_t* toptr, const int64_t* fromptr, const int64_t* offsets, int64_t outlength, int64_t identity, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4729 */
int awkward_reduce_min_uint64_uint64_64(uint64_t* toptr, const uint64_t* fromptr, const int64_t* offsets, int64_t outlength, uint64_t identity, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4736 */
int awkward_reduce_min_float32_float32_64(float* toptr, const float* fromptr, const int64_t* offsets, int64_t outlength, float identity, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4743 */
int awkward_reduce_min_float64_float64_64(double* toptr, const double* fromptr, const int64_t* offsets, int64_t outlength, double identity, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* ---- awkward_reduce_min_complex: replaces awkward-cpp/src/cpu-kernels/awkward_reduce_min_complex.cpp:7 */
/* kernel-specification.yml:4763 */
int awkward_reduce_min_complex64_complex64_64(float* toptr, const float* fromptr, const int64_t* offsets, int64_t outlength, float identity, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4770 */
int awkward_reduce_min_complex128_complex128_64(double* toptr, const double* fromptr, const int64_t* offsets, int64_t outlength, double identity, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* ---- awkward_reduce_prod: replaces awkward-cpp/src/cpu-kernels/awkward_reduce_prod.cpp:12 */
/* kernel-specification.yml:4796 */
int awkward_reduce_prod_int64_int8_64(int64_t* toptr, const int8_t* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4802 */
int awkward_reduce_prod_uint64_uint8_64(uint64_t* toptr, const uint8_t* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4808 */
int awkward_reduce_prod_int64_int16_64(int64_t* toptr, const int16_t* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4814 */
int awkward_reduce_prod_uint64_uint16_64(uint64_t* toptr, const uint16_t* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4820 */
int awkward_reduce_prod_int64_int32_64(int64_t* toptr, const int32_t* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4826 */
int awkward_reduce_prod_uint64_uint32_64(uint64_t* toptr, const uint32_t* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4832 */
int awkward_reduce_prod_int64_int64_64(int64_t* toptr, const int64_t* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4838 */
int awkward_reduce_prod_uint64_uint64_64(uint64_t* toptr, const uint64_t* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4844 */
int awkward_reduce_prod_float32_float32_64(float* toptr, const float* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4850 */
int awkward_reduce_prod_float64_float64_64(double* toptr, const double* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4856 */
int awkward_reduce_prod_int32_int8_64(int32_t* toptr, const int8_t* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4862 */
int awkward_reduce_prod_uint32_uint8_64(uint32_t* toptr, const uint8_t* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4868 */
int awkward_reduce_prod_int32_int16_64(int32_t* toptr, const int16_t* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4874 */
int awkward_reduce_prod_uint32_uint16_64(uint32_t* toptr, const uint16_t* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4880 */
int awkward_reduce_prod_int32_int32_64(int32_t* toptr, const int32_t* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4886 */
int awkward_reduce_prod_uint32_uint32_64(uint32_t* toptr, const uint32_t* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* ---- awkward_reduce_prod_complex: replaces awkward-cpp/src/cpu-kernels/awkward_reduce_prod_complex.cpp:9 */
/* kernel-specification.yml:4903 */
int awkward_reduce_prod_complex64_complex64_64(float* toptr, const float* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4909 */
int awkward_reduce_prod_complex128_complex128_64(double* toptr, const double* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* ---- awkward_reduce_prod_bool: replaces awkward-cpp/src/cpu-kernels/awkward_reduce_prod_bool.cpp:10 */
/* kernel-specification.yml:4933 */
int awkward_reduce_prod_bool_bool_64(bool* toptr, const bool* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4939 */
int awkward_reduce_prod_bool_int8_64(bool* toptr, const int8_t* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4945 */
int awkward_reduce_prod_bool_uint8_64(bool* toptr, const uint8_t* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4951 */
int awkward_reduce_prod_bool_int16_64(bool* toptr, const int16_t* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4957 */
int awkward_reduce_prod_bool_uint16_64(bool* toptr, const uint16_t* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4963 */
int awkward_reduce_prod_bool_int32_64(bool* toptr, const int32_t* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4969 */
int awkward_reduce_prod_bool_uint32_64(bool* toptr, const uint32_t* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4975 */
int awkward_reduce_prod_bool_int64_64(bool* toptr, const int64_t* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4981 */
int awkward_reduce_prod_bool_uint64_64(bool* toptr, const uint64_t* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4987 */
int awkward_reduce_prod_bool_float32_64(bool* toptr, const float* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:4993 */
int awkward_reduce_prod_bool_float64_64(bool* toptr, const double* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* ---- awkward_reduce_prod_bool_complex: replaces awkward-cpp/src/cpu-kernels/awkward_reduce_prod_bool_complex.cpp:7 */
/* kernel-specification.yml:5012 */
int awkward_reduce_prod_bool_complex64_64(bool* toptr, const float* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5018 */
int awkward_reduce_prod_bool_complex128_64(bool* toptr, const double* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* ---- awkward_reduce_sum: replaces awkward-cpp/src/cpu-kernels/awkward_reduce_sum.cpp:12 */
/* kernel-specification.yml:5037 */
int awkward_reduce_sum_int64_int8_64(int64_t* toptr, const int8_t* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5043 */
int awkward_reduce_sum_uint64_uint8_64(uint64_t* toptr, const uint8_t* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5049 */
int awkward_reduce_sum_int64_int16_64(int64_t* toptr, const int16_t* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5055 */
int awkward_reduce_sum_uint64_uint16_64(uint64_t* toptr, const uint16_t* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5061 */
int awkward_reduce_sum_int64_int32_64(int64_t* toptr, const int32_t* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5067 */
int awkward_reduce_sum_uint64_uint32_64(uint64_t* toptr, const uint32_t* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5073 */
int awkward_reduce_sum_int64_int64_64(int64_t* toptr, const int64_t* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5079 */
int awkward_reduce_sum_uint64_uint64_64(uint64_t* toptr, const uint64_t* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5085 */
int awkward_reduce_sum_float32_float32_64(float* toptr, const float* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5091 */
int awkward_reduce_sum_float64_float64_64(double* toptr, const double* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5097 */
int awkward_reduce_sum_int32_int8_64(int32_t* toptr, const int8_t* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5103 */
int awkward_reduce_sum_uint32_uint8_64(uint32_t* toptr, const uint8_t* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5109 */
int awkward_reduce_sum_int32_int16_64(int32_t* toptr, const int16_t* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5115 */
int awkward_reduce_sum_uint32_uint16_64(uint32_t* toptr, const uint16_t* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5121 */
int awkward_reduce_sum_int32_int32_64(int32_t* toptr, const int32_t* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5127 */
int awkward_reduce_sum_uint32_uint32_64(uint32_t* toptr, const uint32_t* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5133 */
int awkward_reduce_sum_float64_int8_64(double* toptr, const int8_t* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5139 */
int awkward_reduce_sum_float64_uint8_64(double* toptr, const uint8_t* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5145 */
int awkward_reduce_sum_float64_int16_64(double* toptr, const int16_t* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5151 */
int awkward_reduce_sum_float64_uint16_64(double* toptr, const uint16_t* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5157 */
int awkward_reduce_sum_float64_int32_64(double* toptr, const int32_t* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5163 */
int awkward_reduce_sum_float64_uint32_64(double* toptr, const uint32_t* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5169 */
int awkward_reduce_sum_float64_int64_64(double* toptr, const int64_t* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5175 */
int awkward_reduce_sum_float64_uint64_64(double* toptr, const uint64_t* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5181 */
int awkward_reduce_sum_float64_float32_64(double* toptr, const float* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* ---- awkward_reduce_sumofsquares: replaces awkward-cpp/src/cpu-kernels/awkward_reduce_sumofsquares.cpp:12 */
/* kernel-specification.yml:5198 */
int awkward_reduce_sumofsquares_float64_int8_64(double* toptr, const int8_t* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5204 */
int awkward_reduce_sumofsquares_float64_uint8_64(double* toptr, const uint8_t* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5210 */
int awkward_reduce_sumofsquares_float64_int16_64(double* toptr, const int16_t* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5216 */
int awkward_reduce_sumofsquares_float64_uint16_64(double* toptr, const uint16_t* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5222 */
int awkward_reduce_sumofsquares_float64_int32_64(double* toptr, const int32_t* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5228 */
int awkward_reduce_sumofsquares_float64_uint32_64(double* toptr, const uint32_t* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5234 */
int awkward_reduce_sumofsquares_float64_int64_64(double* toptr, const int64_t* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5240 */
int awkward_reduce_sumofsquares_float64_uint64_64(double* toptr, const uint64_t* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5246 */
int awkward_reduce_sumofsquares_float64_bool_64(double* toptr, const bool* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5252 */
int awkward_reduce_sumofsquares_float64_float32_64(double* toptr, const float* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5258 */
int awkward_reduce_sumofsquares_float64_float64_64(double* toptr, const double* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* ---- awkward_reduce_sumofpowers: replaces awkward-cpp/src/cpu-kernels/awkward_reduce_sumofpowers.cpp:39 */
/* kernel-specification.yml:5275 */
int awkward_reduce_sumofpowers_float64_int8_64(double* toptr, const int8_t* fromptr, const int64_t* offsets, int64_t outlength, int64_t n, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5282 */
int awkward_reduce_sumofpowers_float64_uint8_64(double* toptr, const uint8_t* fromptr, const int64_t* offsets, int64_t outlength, int64_t n, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5289 */
int awkward_reduce_sumofpowers_float64_int16_64(double* toptr, const int16_t* fromptr, const int64_t* offsets, int64_t outlength, int64_t n, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5296 */
int awkward_reduce_sumofpowers_float64_uint16_64(double* toptr, const uint16_t* fromptr, const int64_t* offsets, int64_t outlength, int64_t n, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5303 */
int awkward_reduce_sumofpowers_float64_int32_64(double* toptr, const int32_t* fromptr, const int64_t* offsets, int64_t outlength, int64_t n, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5310 */
int awkward_reduce_sumofpowers_float64_uint32_64(double* toptr, const uint32_t* fromptr, const int64_t* offsets, int64_t outlength, int64_t n, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5317 */
int awkward_reduce_sumofpowers_float64_int64_64(double* toptr, const int64_t* fromptr, const int64_t* offsets, int64_t outlength, int64_t n, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5324 */
int awkward_reduce_sumofpowers_float64_uint64_64(double* toptr, const uint64_t* fromptr, const int64_t* offsets, int64_t outlength, int64_t n, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5331 */
int awkward_reduce_sumofpowers_float64_bool_64(double* toptr, const bool* fromptr, const int64_t* offsets, int64_t outlength, int64_t n, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5338 */
int awkward_reduce_sumofpowers_float64_float32_64(double* toptr, const float* fromptr, const int64_t* offsets, int64_t outlength, int64_t n, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5345 */
int awkward_reduce_sumofpowers_float64_float64_64(double* toptr, const double* fromptr, const int64_t* offsets, int64_t outlength, int64_t n, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* ---- awkward_reduce_centered_sumofsquares: replaces awkward-cpp/src/cpu-kernels/awkward_reduce_centered_sumofsquares.cpp:15 */
/* kernel-specification.yml:5363 */
int awkward_reduce_centered_sumofsquares_float64_int8_64(double* toptr, const int8_t* fromptr, const int64_t* offsets, int64_t outlength, const double* means, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5370 */
int awkward_reduce_centered_sumofsquares_float64_uint8_64(double* toptr, const uint8_t* fromptr, const int64_t* offsets, int64_t outlength, const double* means, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5377 */
int awkward_reduce_centered_sumofsquares_float64_int16_64(double* toptr, const int16_t* fromptr, const int64_t* offsets, int64_t outlength, const double* means, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5384 */
int awkward_reduce_centered_sumofsquares_float64_uint16_64(double* toptr, const uint16_t* fromptr, const int64_t* offsets, int64_t outlength, const double* means, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5391 */
int awkward_reduce_centered_sumofsquares_float64_int32_64(double* toptr, const int32_t* fromptr, const int64_t* offsets, int64_t outlength, const double* means, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5398 */
int awkward_reduce_centered_sumofsquares_float64_uint32_64(double* toptr, const uint32_t* fromptr, const int64_t* offsets, int64_t outlength, const double* means, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5405 */
int awkward_reduce_centered_sumofsquares_float64_int64_64(double* toptr, const int64_t* fromptr, const int64_t* offsets, int64_t outlength, const double* means, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5412 */
int awkward_reduce_centered_sumofsquares_float64_uint64_64(double* toptr, const uint64_t* fromptr, const int64_t* offsets, int64_t outlength, const double* means, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5419 */
int awkward_reduce_centered_sumofsquares_float64_bool_64(double* toptr, const bool* fromptr, const int64_t* offsets, int64_t outlength, const double* means, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5426 */
int awkward_reduce_centered_sumofsquares_float64_float32_64(double* toptr, const float* fromptr, const int64_t* offsets, int64_t outlength, const double* means, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5433 */
int awkward_reduce_centered_sumofsquares_float64_float64_64(double* toptr, const double* fromptr, const int64_t* offsets, int64_t outlength, const double* means, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* ---- awkward_reduce_sum_complex: replaces awkward-cpp/src/cpu-kernels/awkward_reduce_sum_complex.cpp:7 */
/* kernel-specification.yml:5453 */
int awkward_reduce_sum_complex64_complex64_64(float* toptr, const float* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5459 */
int awkward_reduce_sum_complex128_complex128_64(double* toptr, const double* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* ---- awkward_reduce_sum_bool: replaces awkward-cpp/src/cpu-kernels/awkward_reduce_sum_bool.cpp:18 */
/* kernel-specification.yml:5479 */
int awkward_reduce_sum_bool_bool_64(bool* toptr, const bool* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5485 */
int awkward_reduce_sum_bool_int8_64(bool* toptr, const int8_t* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5491 */
int awkward_reduce_sum_bool_uint8_64(bool* toptr, const uint8_t* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5497 */
int awkward_reduce_sum_bool_int16_64(bool* toptr, const int16_t* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5503 */
int awkward_reduce_sum_bool_uint16_64(bool* toptr, const uint16_t* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5509 */
int awkward_reduce_sum_bool_int32_64(bool* toptr, const int32_t* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5515 */
int awkward_reduce_sum_bool_uint32_64(bool* toptr, const uint32_t* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5521 */
int awkward_reduce_sum_bool_int64_64(bool* toptr, const int64_t* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5527 */
int awkward_reduce_sum_bool_uint64_64(bool* toptr, const uint64_t* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5533 */
int awkward_reduce_sum_bool_float32_64(bool* toptr, const float* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5539 */
int awkward_reduce_sum_bool_float64_64(bool* toptr, const double* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* ---- awkward_reduce_sum_bool_complex: replaces awkward-cpp/src/cpu-kernels/awkward_reduce_sum_bool_complex.cpp:7 */
/* kernel-specification.yml:5558 */
int awkward_reduce_sum_bool_complex64_64(bool* toptr, const float* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5564 */
int awkward_reduce_sum_bool_complex128_64(bool* toptr, const double* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* ---- awkward_reduce_sum_int32_bool_64: replaces awkward-cpp/src/cpu-kernels/awkward_reduce_sum_int32_bool_64.cpp:7 */
/* kernel-specification.yml:5583 */
int awkward_reduce_sum_int32_bool_64(int32_t* toptr, const bool* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* ---- awkward_reduce_sum_int64_bool_64: replaces awkward-cpp/src/cpu-kernels/awkward_reduce_sum_int64_bool_64.cpp:7 */
/* kernel-specification.yml:5601 */
int awkward_reduce_sum_int64_bool_64(int64_t* toptr, const bool* fromptr, const int64_t* offsets, int64_t outlength, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* ---- awkward_sort: replaces awkward-cpp/src/cpu-kernels/awkward_sort.cpp:62 */
/* kernel-specification.yml:5619 */
int awkward_sort_bool(bool* toptr, const bool* fromptr, int64_t length, const int64_t* offsets, int64_t offsetslength, bool ascending, bool stable, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5628 */
int awkward_sort_int8(int8_t* toptr, const int8_t* fromptr, int64_t length, const int64_t* offsets, int64_t offsetslength, bool ascending, bool stable, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5637 */
int awkward_sort_int16(int16_t* toptr, const int16_t* fromptr, int64_t length, const int64_t* offsets, int64_t offsetslength, bool ascending, bool stable, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5646 */
int awkward_sort_int32(int32_t* toptr, const int32_t* fromptr, int64_t length, const int64_t* offsets, int64_t offsetslength, bool ascending, bool stable, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5655 */
int awkward_sort_int64(int64_t* toptr, const int64_t* fromptr, int64_t length, const int64_t* offsets, int64_t offsetslength, bool ascending, bool stable, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5664 */
int awkward_sort_uint8(uint8_t* toptr, const uint8_t* fromptr, int64_t length, const int64_t* offsets, int64_t offsetslength, bool ascending, bool stable, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5673 */
int awkward_sort_uint16(uint16_t* toptr, const uint16_t* fromptr, int64_t length, const int64_t* offsets, int64_t offsetslength, bool ascending, bool stable, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5682 */
int awkward_sort_uint32(uint32_t* toptr, const uint32_t* fromptr, int64_t length, const int64_t* offsets, int64_t offsetslength, bool ascending, bool stable, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5691 */
int awkward_sort_uint64(uint64_t* toptr, const uint64_t* fromptr, int64_t length, const int64_t* offsets, int64_t offsetslength, bool ascending, bool stable, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5700 */
int awkward_sort_float32(float* toptr, const float* fromptr, int64_t length, const int64_t* offsets, int64_t offsetslength, bool ascending, bool stable, uint64_t invocation_index, uint64_t* err_code, void* stream);
/* kernel-specification.yml:5709 */
int awkward_sort_float64(double* toptr, const double* fromptr, int64_t length, const int64_t* offsets, int64_t offsetslength, bool ascending, bool stable, uint64_t invocation_index, uint64_t* err_code, void* stream);

/* ---- no-alloc variant.  No counterpart in awkward: an extra entry point
 * of this library for callers that may not allocate device memory while
 * they run, e.g. code embedded in a process whose GPU memory is owned by
 * another framework's pooling allocator (cudaMalloc then fails or goes
 * around the pool, and the caller has no handle to the pool).
 * Same arguments and results as awkward_ListArray64_getitem_jagged_apply_64;
 * its tile-state scratch is a fixed 512 KiB device array inside the
 * library (held on every GPU that loads it until exit) instead of a
 * pool allocation.  sliceouterlen above AWKWARD_GB300_NOALLOC_MAX_LISTS
 * returns cudaErrorInvalidValue (1) and launches nothing.  All calls
 * share the array: calls that overlap on the GPU (other streams or
 * threads) race and must be ordered by the caller.  The first call in
 * each CUDA context looks up the array's device address (cached per
 * device and context), so make it before any stream capture there. */
#define AWKWARD_GB300_NOALLOC_MAX_LISTS 67108864LL
int awkward_ListArray64_getitem_jagged_apply_64_noalloc(int64_t* tooffsets, int64_t* tocarry, const int64_t* slicestarts, const int64_t* slicestops, int64_t sliceouterlen, const int64_t* sliceindex, int64_t sliceinnerlen, const int64_t* fromstarts, const int64_t* fromstops, int64_t contentlen, uint64_t invocation_index, uint64_t* err_code, void* stream);

/* ---- jagged getitem steps that awkward performs with cupy array operations
 * instead of kernels of its specification (no counterpart in
 * kernel-specification.yml):
 *   jagged_mask_to_index: jagged boolean mask (uint8, one byte per element,
 *     indexed globally over offsets[0]..offsets[nlists]) -> new offsets
 *     [nlists + 1] and, for each true entry in order, its position within its
 *     list (src/awkward/_slicing.py:476-530: localindex + compaction + cumsum);
 *   jagged_mask_select: array[mask] in one pass -- the new offsets, the
 *     selected content (itemsize 1, 2, 4 or 8) and optionally the carry
 *     (NULL to skip), without the local index of the chain;
 *   jagged_index_select: array[index] with a jagged int64 index in one pass
 *     -- jagged_apply with the content gathered at each carry (itemsize 1, 2,
 *     4 or 8; tocarry NULL to skip), errors as jagged_apply's;
 *   take: out[i] = content[carry[i]] for itemsize 1, 2, 4 or 8 bytes
 *     (NumpyArray._carry); a carry outside [0, contentlen) sets err_code to
 *     invocation_index*256 + 0 ("index out of range"). */
int awkward_gb300_jagged_mask_to_index(int64_t* tooffsets, int64_t* toindex, const uint8_t* mask, const int64_t* offsets, int64_t nlists, uint64_t* err_code, void* stream);
int awkward_gb300_jagged_mask_select(int64_t* tooffsets, void* tocontent, int64_t* tocarry, const uint8_t* mask, const int64_t* offsets, const void* content, int64_t itemsize, int64_t nlists, uint64_t* err_code, void* stream);
int awkward_gb300_jagged_index_select(int64_t* tooffsets, void* tocontent, int64_t* tocarry, const int64_t* index_offsets, const int64_t* index, int64_t indexlen, const int64_t* offsets, const void* content, int64_t itemsize, int64_t contentlen, int64_t nlists, uint64_t* err_code, void* stream);
int awkward_gb300_take(void* out, const void* content, int64_t itemsize, const int64_t* carry, int64_t n, int64_t contentlen, uint64_t invocation_index, uint64_t* err_code, void* stream);

/* ---- backward kernels of differentiable jagged operations (torch.autograd
 * in awkward_gb300/autograd.py).  No counterpart in awkward, which has no
 * CUDA backward kernels.  Pointers are device pointers; offsets are int64
 * [nlists + 1] (need not start at 0); element arrays are indexed globally;
 * nvalues is the length of the element arrays: elements no list covers are
 * set to 0, the others written by the kernels (no prior clearing needed).
 *   segment_sum_backward:   grad_x[j] = grad_out[list of j]
 *   segment_max_backward:   grad_x = 0; grad_x[argmax[l]] = grad_out[l] for
 *                           argmax[l] in [0, nelements) (global indices, -1 empty)
 *   jagged_softmax_forward: y = exp(x - max) / sum(exp(x - max)) per list
 *   jagged_softmax_backward: grad_x = y * (grad_y - sum(grad_y * y)) per list,
 *                           y from y_saved, or recomputed from x when NULL */
int awkward_gb300_segment_sum_backward_float32(float* grad_x, const float* grad_out, const int64_t* offsets, int64_t nlists, int64_t nvalues, void* stream);
int awkward_gb300_segment_max_backward_float32(float* grad_x, const float* grad_out, const int64_t* argmax, int64_t nelements, int64_t nlists, void* stream);
int awkward_gb300_jagged_softmax_forward_float32(float* y, const float* x, const int64_t* offsets, int64_t nlists, int64_t nvalues, void* stream);
int awkward_gb300_jagged_softmax_backward_float32(float* grad_x, const float* grad_y, const float* x, const float* y_saved, const int64_t* offsets, int64_t nlists, int64_t nvalues, void* stream);
int awkward_gb300_segment_sum_backward_float64(double* grad_x, const double* grad_out, const int64_t* offsets, int64_t nlists, int64_t nvalues, void* stream);
int awkward_gb300_segment_max_backward_float64(double* grad_x, const double* grad_out, const int64_t* argmax, int64_t nelements, int64_t nlists, void* stream);
int awkward_gb300_jagged_softmax_forward_float64(double* y, const double* x, const int64_t* offsets, int64_t nlists, int64_t nvalues, void* stream);
int awkward_gb300_jagged_softmax_backward_float64(double* grad_x, const double* grad_y, const double* x, const double* y_saved, const int64_t* offsets, int64_t nlists, int64_t nvalues, void* stream);

/* ---- batched execution (no counterpart in awkward): sum, max, argmax and
 * count (axis=-1) and array[mask] of many float64 ListOffsetArrays in one
 * launch per operation.  plan_create (set-up: allocates and uploads the
 * work-queue tables, synchronous) takes host arrays of narrays entries:
 * list counts, element counts (offsets[n] - offsets[0]) and the device
 * pointers of each array's content, offsets, uint8 mask and outputs
 * (out_sum/out_max [n] float64, out_argmax/out_count [n] int64,
 * sel_offsets [n + 1] int64, sel_content [elements] float64).  Tuning
 * knobs: order_mode (0 array order, 1 largest ranges first),
 * occupancy_div (persistent CTAs per SM = occupancy / div), range_min
 * (items per range of arrays with no list above 4096 elements, >= 512),
 * block (threads per reducer CTA, 128 or 256).  Reducer results are
 * bit-identical to the per-array entry points.  plan_run only
 * launches (capturable in a CUDA graph); plan_destroy frees the plan. */
int awkward_gb300_batch_plan_create(void** plan, int64_t narrays, const int64_t* nlists, const int64_t* nelements, const int64_t* maxlen, const double* const* x, const int64_t* const* offsets, const uint8_t* const* mask, double* const* out_sum, double* const* out_max, int64_t* const* out_argmax, int64_t* const* out_count, int64_t* const* sel_offsets, double* const* sel_content, int64_t order_mode, int64_t occupancy_div, int64_t range_min, int64_t block, uint64_t* err_code);
int awkward_gb300_batch_plan_run(void* plan, void* stream);
int awkward_gb300_batch_plan_destroy(void* plan);

/* ---- host-buffer reduction with overlapped transfers (no counterpart in
 * awkward): segmented sum, max (identity -inf) and argmax of a float64
 * ListOffsetArray in pinned host memory.  Lists are cut into `chunks`
 * (1..64) at list boundaries; copies in of chunk c+1, the reductions of
 * chunk c and copies back of chunk c-1 overlap.  Device workspace: d_x
 * (element j at d_x[j]), d_offsets [nlists + 1], three outputs [nlists].
 * Returns after enqueueing; `stream` waits for the last copy back. */
int awkward_gb300_reduce_sum_max_argmax_host_float64(double* h_sum, double* h_max, int64_t* h_argmax, const double* h_x, const int64_t* h_offsets, int64_t nlists, double* d_x, int64_t* d_offsets, double* d_sum, double* d_max, int64_t* d_argmax, int64_t chunks, void* stream);

/* ---- elementwise map fused into the segmented reduction (no counterpart in
 * kernel-specification.yml; awkward evaluates such chains as an elementwise
 * kernel followed by a reducer, or through its lazy fusion backend).
 * float64 content x (and y), int64 offsets [nlists + 1] (need not start at
 * 0), indexed globally.  map: 0 x, 1 x*y, 2 x*x, 3 |x| (y may be NULL unless
 * map is 1).  reduce: 0 sum, 1 max (identity -inf), 2 min (identity +inf)
 * into double out[nlists]; 3 argmax, 4 argmin into int64 out[nlists]
 * (global indices, -1 for empty lists).  Equal to awkward_reduce_* on the
 * materialised mapped values (sums within the reducers' bound).  Other
 * map or reduce values, or map 1 without y, return cudaErrorInvalidValue. */
int awkward_gb300_fused_reduce_float64(void* out, const double* x, const double* y, const int64_t* offsets, int64_t nlists, int64_t map, int64_t reduce, uint64_t invocation_index, uint64_t* err_code, void* stream);

/* ---- self-test of the failure report (no counterpart in awkward): one warp
 * runs the decoupled look-back of the scan kernels on tile 1 of a fresh
 * scan whose tile 0 never publishes, with a spin limit of `spin_limit`
 * polls (clamped to 1..2^22; each poll sleeps at most 256 ns).  The wait
 * runs out and the kernel sets err_code to invocation_index*256 + 32, the
 * library's "bounded wait gave up" code, then returns; the GPU stays
 * usable.  It is how the tests check that a stalled look-back ends with an
 * error the host can read instead of a hang. */
int awkward_gb300_selftest_lookback_timeout(uint32_t spin_limit, uint64_t invocation_index, uint64_t* err_code, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* AWKWARD_GB300_H_ */
