// finalize.cu -- exact per-survivor work after the tensor-core filter.
//
// For every candidate whose mask bit survived the guarded filter, one warp:
//   * computes all L PSD bins in FP64 (src/utils/fourier.cpp:25-43) and
//     re-applies the exact filter (fourier.cpp:45-52);
//   * for each role (A / B) of the candidate, optionally checks that the
//     sequence is the lexicographic minimum of its orbit, as isCanonical
//     (src/utils/orderly_equivalence.cpp:53-68) with the generator sets of
//     constructGenerators(0|1, L) (:17-51): for A the affine maps
//     i -> u*i + t (u a unit mod L), for B the dihedral maps i -> +-i + t;
//   * writes a record: the word, the role and the signature
//     rint(psd[k]) (or bound - rint(psd[k]) for inverted roles), k = 1..L-1
//     (src/utils/io.cpp:14-36).
#include "gp_device.cuh"
#include "finalize.h"
#include "rows.cuh"

namespace gp {

namespace {

constexpr int kWarps = 8;

__device__ __forceinline__ void list_bits(const uint32_t* mask, int64_t n, const unsigned long long* n_dev,
                                          uint32_t* out, unsigned long long* count, int64_t cap, int* status) {
    const int lane = threadIdx.x & 31;
    if (n_dev && (int64_t)*n_dev < n) n = (int64_t)*n_dev;
    const int64_t nwords = (n + 31) / 32;
    for (int64_t wi = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; wi < nwords;
         wi += ((int64_t)gridDim.x * blockDim.x) >> 5) {
        const uint32_t m = mask[wi];
        const bool bit = (m >> lane) & 1u;
        const uint32_t bal = __ballot_sync(0xFFFFFFFFu, bit);
        if (!bal) continue;
        unsigned long long base = 0;
        if (lane == 0) base = atomicAdd(count, (unsigned long long)__popc(bal));
        base = __shfl_sync(0xFFFFFFFFu, base, 0);
        if (bit) {
            const unsigned long long pos = base + __popc(bal & ((1u << lane) - 1u));
            if ((int64_t)pos < cap)
                out[pos] = (uint32_t)(wi * 32 + lane);
            else
                atomicCAS(status, 0, GP_KSTATUS_OVERFLOW);
        }
    }
}

__global__ void mask_to_list_kernel(const uint32_t* mask, int64_t n, const unsigned long long* n_dev, uint32_t* out,
                                    unsigned long long* count, int64_t cap, int* status) {
    list_bits(mask, n, n_dev, out, count, cap, status);
}

// every job's mask in one launch: grid row y serves job y
__global__ void mask_to_list_multi_kernel(ListMultiArgs a) {
    const ListJob& j = a.job[blockIdx.y];
    list_bits(j.mask, j.n, j.n_dev, j.out, j.count, j.cap, a.status);
}

__device__ __forceinline__ void finalize_rows(const FinalizeArgs& a, double2* sh_tw) {
    const int L = a.src.L;
    double* psd_all = reinterpret_cast<double*>(sh_tw + L);
    int8_t* xs_all = reinterpret_cast<int8_t*>(psd_all + kWarps * L);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    double* psd = psd_all + warp * L;
    int8_t* xs = xs_all + warp * kMaxLen;
    for (int m = threadIdx.x; m < L; m += blockDim.x) sh_tw[m] = make_double2(a.tw[2 * m], a.tw[2 * m + 1]);
    __syncthreads();
    int64_t cnt = (int64_t)*a.n_idx;
    if (cnt > a.idx_cap) cnt = a.idx_cap;
    const int H = L / 2;
    for (int64_t i = (int64_t)blockIdx.x * kWarps + warp; i < cnt; i += (int64_t)gridDim.x * kWarps) {
        const uint32_t row = a.idx[i];
        if (lane == 0) decode_row(a.src, row, xs);
        __syncwarp();
        bool fail = false;
        for (int k = lane; k < L; k += 32) {
            double re = 0.0, im = 0.0;
            int m = 0;
            for (int j = 0; j < L; ++j) {
                const double v = (double)xs[j];
                const double2 w = sh_tw[m];
                re = fma(v, w.x, re);
                im = fma(-v, w.y, im);
                m += k;
                if (m >= L) m -= L;
            }
            const double p = re * re + im * im;
            psd[k] = p;
            if (k >= 1 && k <= H && p > a.thr) fail = true;
        }
        fail = __any_sync(0xFFFFFFFFu, fail);
        __syncwarp();
        if (fail) continue;
        if (lane == 0) atomicAdd(a.psd_pass, 1ull);
        if (a.prune_tab) {
            // p(L/2) is the square of the alternating sum and p(L/3) the norm
            // of an Eisenstein integer: both exact integers here
            bool keep = true;
            if (L % 2 == 0) {
                const int m = a.bound - __double2int_rn(psd[L / 2]);
                keep = m >= 0 && m <= a.bound && (a.prune_tab[m] & 1);
            }
            if (keep && L % 3 == 0) {
                const int m = a.bound - __double2int_rn(psd[L / 3]);
                keep = m >= 0 && m <= a.bound && (a.prune_tab[m] & 2);
            }
            if (!keep) continue;
        }
        const uint8_t roles = a.roles ? a.roles[row] : a.fixed_role;
        for (int r = 0; r < 2; ++r) {
            if (!((roles >> r) & 1)) continue;
            bool canonical = true;
            if (a.check_canonical) {
                // r = 0: affine maps (constructGenerators(0, L)); r = 1: dihedral
                const int nmul = r == 0 ? a.n_units : (L > 2 ? 2 : 1);
                const int64_t G = (int64_t)nmul * L;
                bool less = false;
                for (int64_t g = lane; g < G && !less; g += 32) {
                    const int mi = (int)(g / L);
                    const int u = r == 0 ? a.units[mi] : (mi == 0 ? 1 : L - 1);
                    const int t = (int)(g % L);
                    int idx = t;
                    for (int q = 0; q < L; ++q) {
                        const int v = xs[idx], x = xs[q];
                        if (v != x) {
                            less = v < x;
                            break;
                        }
                        idx += u;
                        if (idx >= L) idx -= L;
                    }
                }
                canonical = !__any_sync(0xFFFFFFFFu, less);
            }
            if (!canonical) continue;
            unsigned long long pos = 0;
            if (lane == 0) pos = atomicAdd(a.rec_count, 1ull);
            pos = __shfl_sync(0xFFFFFFFFu, pos, 0);
            if ((int64_t)pos >= a.rec_cap) {
                if (lane == 0) atomicCAS(a.status, 0, GP_KSTATUS_OVERFLOW);
                continue;
            }
            const bool inv = (a.invert_roles >> r) & 1;
            for (int k = 1 + lane; k < L; k += 32) {
                const int s = __double2int_rn(psd[k]);
                a.rec_sig[pos * (L - 1) + (k - 1)] = (uint16_t)(inv ? a.bound - s : s);
            }
            if (lane == 0) {
                a.rec_words[pos] = a.src.words ? a.src.words[row] : make_uint4(row, 0, 0, 0);
                if (a.rec_role) a.rec_role[pos] = (uint8_t)(1 << r);
                if (a.rec_src) a.rec_src[pos] = row;
            }
        }
        __syncwarp();
    }
}

__global__ void __launch_bounds__(kWarps * 32) finalize_kernel(FinalizeArgs a) {
    extern __shared__ double2 sh_tw[];
    finalize_rows(a, sh_tw);
}

// every job's survivors in one launch: grid row y serves job y
__global__ void __launch_bounds__(kWarps * 32) finalize_multi_kernel(FinalizeMultiArgs m) {
    extern __shared__ double2 sh_tw[];
    finalize_rows(m.job[blockIdx.y], sh_tw);
}

size_t finalize_smem(int L) {
    return sizeof(double2) * L + sizeof(double) * kWarps * L + (size_t)kWarps * kMaxLen;
}

}  // namespace

cudaError_t launch_mask_to_list(const uint32_t* mask, int64_t n, uint32_t* out, unsigned long long* count,
                                int64_t cap, int* status, int num_sms, cudaStream_t st,
                                const unsigned long long* n_dev) {
    if (n <= 0) return cudaSuccess;
    int64_t blocks = ((n + 31) / 32 + 7) / 8;
    if (blocks > (int64_t)num_sms * 16) blocks = (int64_t)num_sms * 16;
    mask_to_list_kernel<<<(unsigned)blocks, 256, 0, st>>>(mask, n, n_dev, out, count, cap, status);
    return cudaGetLastError();
}

cudaError_t launch_finalize(const FinalizeArgs& a, int64_t max_rows, int num_sms, cudaStream_t st) {
    if (max_rows <= 0) return cudaSuccess;
    int64_t blocks = (max_rows + kWarps - 1) / kWarps;
    if (blocks > (int64_t)num_sms * 16) blocks = (int64_t)num_sms * 16;
    const size_t smem = finalize_smem(a.src.L);
    cudaError_t e = cudaFuncSetAttribute(finalize_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    finalize_kernel<<<(unsigned)blocks, kWarps * 32, smem, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_mask_to_list_multi(const ListMultiArgs& a, int num_sms, cudaStream_t st) {
    if (a.njobs <= 0 || a.njobs > kMaxMultiJobs) return a.njobs == 0 ? cudaSuccess : cudaErrorInvalidValue;
    int64_t maxn = 0;
    for (int j = 0; j < a.njobs; ++j) maxn = a.job[j].n > maxn ? a.job[j].n : maxn;
    if (maxn <= 0) return cudaSuccess;
    int64_t blocks = ((maxn + 31) / 32 + 7) / 8;
    // per job as many blocks as its own launch would take: blocks of a job
    // with fewer rows end at once
    if (blocks > (int64_t)num_sms * 16) blocks = (int64_t)num_sms * 16;
    mask_to_list_multi_kernel<<<dim3((unsigned)blocks, (unsigned)a.njobs), 256, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_finalize_multi(const FinalizeMultiArgs& a, const int64_t* max_rows, int num_sms,
                                  cudaStream_t st) {
    if (a.njobs <= 0 || a.njobs > kMaxMultiJobs) return a.njobs == 0 ? cudaSuccess : cudaErrorInvalidValue;
    int64_t rows = 0;
    int maxL = 1;
    for (int j = 0; j < a.njobs; ++j) {
        rows = max_rows[j] > rows ? max_rows[j] : rows;
        maxL = a.job[j].src.L > maxL ? a.job[j].src.L : maxL;
    }
    if (rows <= 0) return cudaSuccess;
    int64_t blocks = (rows + kWarps - 1) / kWarps;
    // per job as many blocks as its own launch would take: blocks of a job
    // with fewer rows end at once
    if (blocks > (int64_t)num_sms * 16) blocks = (int64_t)num_sms * 16;
    const size_t smem = finalize_smem(maxL);
    cudaError_t e =
        cudaFuncSetAttribute(finalize_multi_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    finalize_multi_kernel<<<dim3((unsigned)blocks, (unsigned)a.njobs), kWarps * 32, smem, st>>>(a);
    return cudaGetLastError();
}

}  // namespace gp
