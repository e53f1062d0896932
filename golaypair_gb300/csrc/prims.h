// prims.h -- scan / compaction / radix sort building blocks (prims.cu).
#pragma once
#include <cstddef>
#include <cstdint>

#include <cuda_runtime.h>

namespace gp {

size_t scan_tmp_bytes(int64_t n);
cudaError_t exclusive_scan_u32(const uint32_t* in, uint32_t* out, int64_t n, uint32_t* tmp, cudaStream_t st);
// dst[pos] = src ? src[i] : i for every i with flags[i] != 0, in order;
// *d_count = number kept.  pos_tmp: n words; scan_tmp: scan_tmp_bytes(n).
cudaError_t compact_flags(const uint32_t* flags, const uint32_t* src, uint32_t* dst, int64_t n, uint32_t* pos_tmp,
                          uint32_t* scan_tmp, uint32_t* d_count, cudaStream_t st);
// flags[i] = 1 where key[idx[i]] differs from key[idx[i-1]] in its first
// cmp_words words (flags[0] = 1).
cudaError_t mark_unique(const uint32_t* keys, int W, const uint32_t* idx, int64_t n, int cmp_words, uint32_t* flags,
                        cudaStream_t st);
cudaError_t iota_u32(uint32_t* p, int64_t n, cudaStream_t st);
size_t radix_sort_tmp_bytes(int64_t n);
cudaError_t radix_sort_keys(const uint32_t* keys, int W, int sort_words, uint32_t* idx, int64_t n, void* tmp,
                            cudaStream_t st, int radix_bits = 8);

}  // namespace gp
