// prims.cu -- device building blocks of the sort/match stages: exclusive scan,
// stable compaction, and a stable LSD radix sort of fixed-width keys.
//
// Keys are rows of W 32-bit words, word 0 most significant.  The sort
// permutes a uint32 index array (keys stay in place and are gathered per
// pass), 4 or 8 bits per pass (the sort's tuner picks); a pass whose digit
// is the same for every key is skipped (its histogram has a single non-empty
// bucket).
#include <cstdio>
#include <vector>

#include "prims.h"

namespace gp {

namespace {

constexpr int kScanBlock = 1024;

__global__ void scan_block_kernel(const uint32_t* in, uint32_t* out, uint32_t* block_sums, int64_t n) {
    __shared__ uint32_t warp_tot[32];
    const int64_t i = (int64_t)blockIdx.x * kScanBlock + threadIdx.x;
    uint32_t v = i < n ? in[i] : 0u;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t t = warp_tot[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xFFFFFFFFu, t, o);
            if (lane >= o) t += y;
        }
        warp_tot[lane] = t;
    }
    __syncthreads();
    const uint32_t before = warp ? warp_tot[warp - 1] : 0u;
    if (i < n) out[i] = before + x - v;  // exclusive
    if (threadIdx.x == kScanBlock - 1 && block_sums) block_sums[blockIdx.x] = before + x;
}

__global__ void scan_add_kernel(uint32_t* out, const uint32_t* block_off, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * kScanBlock + threadIdx.x;
    if (i < n) out[i] += block_off[blockIdx.x];
}

__global__ void compact_kernel(const uint32_t* flags, const uint32_t* pos, const uint32_t* src, uint32_t* dst,
                               int64_t n, uint32_t* count) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        if (flags[i]) dst[pos[i]] = src ? src[i] : (uint32_t)i;
        if (i == n - 1) *count = pos[i] + (flags[i] ? 1u : 0u);
    }
}

// ------------------------------------------------------------ radix sort
constexpr int kSortThreads = 256;
constexpr int kSortItems = 8;
constexpr int kSortTile = kSortThreads * kSortItems;

template <int RB>
__device__ __forceinline__ uint32_t key_digit(const uint32_t* keys, int W, uint32_t idx, int word, int shift) {
    return (keys[(int64_t)idx * W + word] >> shift) & ((1u << RB) - 1u);
}

// RB bits per pass: 2^RB buckets (RB <= 8, so one thread per bucket).
template <int RB>
__global__ void __launch_bounds__(kSortThreads) radix_hist_kernel(const uint32_t* keys, int W, const uint32_t* idx,
                                                                   int64_t n, int word, int shift, uint32_t* counts,
                                                                   int64_t nblocks, uint32_t* total) {
    constexpr int NB = 1 << RB;
    __shared__ uint32_t h[NB];
    if (threadIdx.x < NB) h[threadIdx.x] = 0;
    __syncthreads();
    const int64_t base = (int64_t)blockIdx.x * kSortTile;
    for (int k = 0; k < kSortItems; ++k) {
        const int64_t i = base + (int64_t)k * kSortThreads + threadIdx.x;
        if (i < n) atomicAdd(&h[key_digit<RB>(keys, W, idx[i], word, shift)], 1u);
    }
    __syncthreads();
    if (threadIdx.x < NB) {
        const uint32_t c = h[threadIdx.x];
        counts[(int64_t)threadIdx.x * nblocks + blockIdx.x] = c;
        if (c) atomicAdd(&total[threadIdx.x], c);
    }
}

template <int RB>
__global__ void __launch_bounds__(kSortThreads) radix_scatter_kernel(const uint32_t* keys, int W, const uint32_t* idx_in,
                                                                      uint32_t* idx_out, int64_t n, int word, int shift,
                                                                      const uint32_t* offsets, int64_t nblocks) {
    constexpr int NB = 1 << RB;
    __shared__ uint32_t base[NB];
    __shared__ uint32_t wh[kSortThreads / 32][NB];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x < NB) base[threadIdx.x] = offsets[(int64_t)threadIdx.x * nblocks + blockIdx.x];
    const int64_t tile0 = (int64_t)blockIdx.x * kSortTile;
    for (int k = 0; k < kSortItems; ++k) {
        if (threadIdx.x < NB)
            for (int w = 0; w < kSortThreads / 32; ++w) wh[w][threadIdx.x] = 0;
        __syncthreads();
        const int64_t i = tile0 + (int64_t)k * kSortThreads + threadIdx.x;
        const bool valid = i < n;
        uint32_t my_idx = 0, d = 0x100u + (uint32_t)lane;  // invalid lanes: unique sentinel
        if (valid) {
            my_idx = idx_in[i];
            d = key_digit<RB>(keys, W, my_idx, word, shift);
        }
        const uint32_t peers = __match_any_sync(0xFFFFFFFFu, d);
        const uint32_t rank = __popc(peers & ((1u << lane) - 1u));
        if (valid && rank == 0) wh[warp][d] = __popc(peers);
        __syncthreads();
        if (threadIdx.x < NB) {
            uint32_t run = base[threadIdx.x];
            for (int w = 0; w < kSortThreads / 32; ++w) {
                const uint32_t c = wh[w][threadIdx.x];
                wh[w][threadIdx.x] = run;
                run += c;
            }
            base[threadIdx.x] = run;
        }
        __syncthreads();
        if (valid) idx_out[wh[warp][d] + rank] = my_idx;
        __syncthreads();
    }
}

__global__ void iota_kernel(uint32_t* p, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        p[i] = (uint32_t)i;
}

__global__ void adjacent_diff_kernel(const uint32_t* keys, int W, const uint32_t* idx, int64_t n, int cmp_words,
                                     uint32_t* flags) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        uint32_t f = 1;
        if (i > 0) {
            const uint32_t* a = keys + (int64_t)idx[i] * W;
            const uint32_t* b = keys + (int64_t)idx[i - 1] * W;
            f = 0;
            for (int w = 0; w < cmp_words; ++w)
                if (a[w] != b[w]) {
                    f = 1;
                    break;
                }
        }
        flags[i] = f;
    }
}

unsigned grid_for(int64_t n, int block) {
    int64_t g = (n + block - 1) / block;
    if (g > 65535 * 16) g = 65535 * 16;
    return (unsigned)(g < 1 ? 1 : g);
}

}  // namespace

size_t scan_tmp_bytes(int64_t n) {
    size_t total = 0;
    while (n > kScanBlock) {
        n = (n + kScanBlock - 1) / kScanBlock;
        total += (size_t)n * 4 * 2;
    }
    return total + 256;
}

cudaError_t exclusive_scan_u32(const uint32_t* in, uint32_t* out, int64_t n, uint32_t* tmp, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    const int64_t nb = (n + kScanBlock - 1) / kScanBlock;
    if (nb == 1) {
        scan_block_kernel<<<1, kScanBlock, 0, st>>>(in, out, nullptr, n);
        return cudaGetLastError();
    }
    uint32_t* sums = tmp;
    uint32_t* sums_scan = tmp + nb;
    scan_block_kernel<<<(unsigned)nb, kScanBlock, 0, st>>>(in, out, sums, n);
    cudaError_t e = exclusive_scan_u32(sums, sums_scan, nb, tmp + 2 * nb, st);
    if (e != cudaSuccess) return e;
    scan_add_kernel<<<(unsigned)nb, kScanBlock, 0, st>>>(out, sums_scan, n);
    return cudaGetLastError();
}

cudaError_t compact_flags(const uint32_t* flags, const uint32_t* src, uint32_t* dst, int64_t n, uint32_t* pos_tmp,
                          uint32_t* scan_tmp, uint32_t* d_count, cudaStream_t st) {
    if (n <= 0) return cudaMemsetAsync(d_count, 0, 4, st);
    cudaError_t e = exclusive_scan_u32(flags, pos_tmp, n, scan_tmp, st);
    if (e != cudaSuccess) return e;
    compact_kernel<<<grid_for(n, 256), 256, 0, st>>>(flags, pos_tmp, src, dst, n, d_count);
    return cudaGetLastError();
}

cudaError_t mark_unique(const uint32_t* keys, int W, const uint32_t* idx, int64_t n, int cmp_words, uint32_t* flags,
                        cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    adjacent_diff_kernel<<<grid_for(n, 256), 256, 0, st>>>(keys, W, idx, n, cmp_words, flags);
    return cudaGetLastError();
}

cudaError_t iota_u32(uint32_t* p, int64_t n, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    iota_kernel<<<grid_for(n, 256), 256, 0, st>>>(p, n);
    return cudaGetLastError();
}

size_t radix_sort_tmp_bytes(int64_t n) {
    const int64_t nb = (n + kSortTile - 1) / kSortTile;
    return (size_t)n * 4                      // ping-pong index
           + (size_t)nb * 256 * 4 * 2         // counts + offsets
           + scan_tmp_bytes(nb * 256) + 256 * 4 + 1024;
}

// Sorts idx (a permutation of row numbers) by the keys' first `sort_words`
// words (of W).  Stable.  tmp: radix_sort_tmp_bytes(n) bytes of device memory.
// radix_bits: 4 or 8 bits per pass.
cudaError_t radix_sort_keys(const uint32_t* keys, int W, int sort_words, uint32_t* idx, int64_t n, void* tmp,
                            cudaStream_t st, int radix_bits) {
    if (n <= 1) return cudaSuccess;
    if (radix_bits != 4 && radix_bits != 8) return cudaErrorInvalidValue;
    const int NB = 1 << radix_bits;
    const int per_word = 32 / radix_bits;
    const int64_t nb = (n + kSortTile - 1) / kSortTile;
    uint8_t* t = static_cast<uint8_t*>(tmp);
    uint32_t* alt = reinterpret_cast<uint32_t*>(t);
    t += (size_t)n * 4;
    uint32_t* counts = reinterpret_cast<uint32_t*>(t);
    t += (size_t)nb * 256 * 4;
    uint32_t* offs = reinterpret_cast<uint32_t*>(t);
    t += (size_t)nb * 256 * 4;
    uint32_t* total = reinterpret_cast<uint32_t*>(t);
    t += 256 * 4;
    t = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(t) + 255) & ~uintptr_t(255));
    uint32_t* stmp = reinterpret_cast<uint32_t*>(t);
    uint32_t* cur = idx;
    uint32_t* nxt = alt;
    std::vector<uint32_t> htotal(NB);
    for (int bi = 0; bi < per_word * sort_words; ++bi) {
        const int word = sort_words - 1 - bi / per_word;
        const int shift = radix_bits * (bi % per_word);
        cudaError_t e = cudaMemsetAsync(total, 0, NB * 4, st);
        if (e != cudaSuccess) return e;
        if (radix_bits == 8)
            radix_hist_kernel<8><<<(unsigned)nb, kSortThreads, 0, st>>>(keys, W, cur, n, word, shift, counts, nb, total);
        else
            radix_hist_kernel<4><<<(unsigned)nb, kSortThreads, 0, st>>>(keys, W, cur, n, word, shift, counts, nb, total);
        e = cudaMemcpyAsync(htotal.data(), total, NB * 4, cudaMemcpyDeviceToHost, st);
        if (e != cudaSuccess) return e;
        e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return e;
        int nonempty = 0;
        for (uint32_t c : htotal) nonempty += c != 0;
        if (nonempty <= 1) continue;  // every key has the same digit here
        e = exclusive_scan_u32(counts, offs, nb * NB, stmp, st);
        if (e != cudaSuccess) return e;
        if (radix_bits == 8)
            radix_scatter_kernel<8><<<(unsigned)nb, kSortThreads, 0, st>>>(keys, W, cur, nxt, n, word, shift, offs, nb);
        else
            radix_scatter_kernel<4><<<(unsigned)nb, kSortThreads, 0, st>>>(keys, W, cur, nxt, n, word, shift, offs, nb);
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        uint32_t* sw = cur;
        cur = nxt;
        nxt = sw;
    }
    if (cur != idx) return cudaMemcpyAsync(idx, cur, (size_t)n * 4, cudaMemcpyDeviceToDevice, st);
    return cudaSuccess;
}

}  // namespace gp
