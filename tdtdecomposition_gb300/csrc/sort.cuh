// Device-wide scan and radix sort primitives (sort.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>

namespace tdt {

size_t scan_scratch_bytes(int64_t n);
template <class TI, class TO>
int exclusive_scan(const TI* in, TO* out, int64_t n, TO* total_out, void* scratch, cudaStream_t st);

size_t radix_sort_scratch_bytes(int64_t n);
template <class K>
int radix_sort_pairs(K* keys, uint32_t* vals, K* keys_alt, uint32_t* vals_alt, int64_t n, int begin_bit,
                     int end_bit, void* scratch, bool* result_in_alt, cudaStream_t st);

}  // namespace tdt
