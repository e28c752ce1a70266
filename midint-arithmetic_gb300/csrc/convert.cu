// convert.cu -- batched conversion between the library's limb layout and the
// word formats of GMP's mpz_import / mpz_export.
//
// The reference moves every operand through mpz_import / mpz_export with
// order -1 and 4-byte native words (cuda/helper.h:116, 146-170); callers that
// hold their integers in another GMP word format (most significant word
// first, big-endian bytes, 1- to 8-byte words) convert on the device here
// instead of on the host.  A field is `words` words of `size` bytes per
// instance; order 1 = most significant word first, -1 = least significant
// first; endian 1 = big-endian bytes in a word, -1 or 0 = little-endian.
// Both directions are one pass over HBM: every thread assembles (import) one
// u64 limb from the 8/size words that hold its bytes, or extracts (export) one
// word from the limb that holds it, with a byte swap for big-endian words.
// Export also reports mpz_export's count of significant words per instance.
#include <cstdio>

#include "common.cuh"
#include "kernels.h"

namespace mi {
namespace {

template <int SIZE>
struct Word;
template <>
struct Word<1> {
    using T = uint8_t;
    __device__ static T swap(T x) { return x; }
};
template <>
struct Word<2> {
    using T = uint16_t;
    __device__ static T swap(T x) { return T((x >> 8) | (x << 8)); }
};
template <>
struct Word<4> {
    using T = uint32_t;
    __device__ static T swap(T x) { return __byte_perm(x, 0, 0x0123); }
};
template <>
struct Word<8> {
    using T = uint64_t;
    __device__ static T swap(T x) {
        const uint32_t lo = uint32_t(x), hi = uint32_t(x >> 32);
        return (uint64_t(__byte_perm(lo, 0, 0x0123)) << 32) | __byte_perm(hi, 0, 0x0123);
    }
};

template <int SIZE>
__global__ void k_import(const typename Word<SIZE>::T* __restrict__ src, uint64_t* __restrict__ dst, uint64_t total,
                         uint32_t words, uint32_t limbs, int most_first, int big) {
    using W = Word<SIZE>;
    constexpr uint32_t PER = 8 / SIZE;  // words per limb
    pdl_wait();  // launched with launch_pdl
    pdl_trigger();
    for (uint64_t idx = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; idx < total;
         idx += uint64_t(gridDim.x) * blockDim.x) {
        const uint64_t i = idx / limbs;
        const uint32_t j = uint32_t(idx % limbs);
        const typename W::T* row = src + i * words;
        uint64_t v = 0;
#pragma unroll
        for (uint32_t q = 0; q < PER; ++q) {
            const uint64_t w = uint64_t(j) * PER + q;
            if (w < words) {
                typename W::T x = __ldcs(row + (most_first ? words - 1 - w : w));
                if (big) x = W::swap(x);
                v |= uint64_t(x) << (q * SIZE * 8);
            }
        }
        __stcs(reinterpret_cast<unsigned long long*>(dst + idx), (unsigned long long)v);
    }
}

template <int SIZE>
__global__ void k_export(const uint64_t* __restrict__ src, typename Word<SIZE>::T* __restrict__ dst, uint64_t total,
                         uint32_t limbs, uint32_t words, int most_first, int big) {
    using W = Word<SIZE>;
    constexpr uint32_t PER = 8 / SIZE;
    pdl_wait();  // launched with launch_pdl
    pdl_trigger();
    for (uint64_t idx = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; idx < total;
         idx += uint64_t(gridDim.x) * blockDim.x) {
        const uint64_t i = idx / words;
        const uint32_t w = uint32_t(idx % words);
        const uint32_t j = w / PER;
        const uint64_t limb = j < limbs ? __ldg(src + i * limbs + j) : 0ull;
        typename W::T x = typename W::T(limb >> ((w % PER) * SIZE * 8));
        if (big) x = W::swap(x);
        dst[i * words + (most_first ? words - 1 - w : w)] = x;
    }
}

// counts[i] = mpz_export's count of significant `size`-byte words (0 for
// zero): one warp per instance scans its limbs from the top.
__global__ void k_count_words(const uint64_t* __restrict__ src, uint32_t* __restrict__ counts, uint32_t n,
                              uint32_t limbs, uint32_t size) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint64_t warps = uint64_t(gridDim.x) * (blockDim.x / 32);
    pdl_wait();  // launched with launch_pdl
    pdl_trigger();
    for (uint64_t i = (uint64_t(blockIdx.x) * blockDim.x + threadIdx.x) / 32; i < n; i += warps) {
        const uint64_t* row = src + i * limbs;
        uint32_t count = 0;
        for (int64_t top = int64_t(limbs) - 1; top >= 0; top -= 32) {
            const int64_t j = top - lane;
            const uint64_t v = j >= 0 ? row[j] : 0ull;
            const uint32_t nz = __ballot_sync(MI_FULL_MASK, v != 0);
            if (nz) {
                const uint32_t src_lane = __ffs(nz) - 1;  // the highest nonzero limb
                const uint64_t hv = __shfl_sync(MI_FULL_MASK, v, src_lane);
                const uint64_t jt = uint64_t(top) - src_lane;
                const uint32_t top_byte = uint32_t(63 - __clzll(hv)) / 8;
                count = uint32_t((jt * 8 + top_byte) / size + 1);
                break;
            }
        }
        if (lane == 0) counts[i] = count;
    }
}

uint32_t grid_for(uint64_t total) {
    const uint64_t blocks = (total + 255) / 256;
    const uint64_t cap = uint64_t(sm_count()) * 16;
    return uint32_t(blocks < cap ? (blocks ? blocks : 1) : cap);
}

}  // namespace

mi_status launch_import(const void* src, uint64_t* dst, uint32_t n, uint32_t words, uint32_t size, int order,
                        int endian, uint32_t limbs, cudaStream_t st) {
    const uint64_t total = uint64_t(n) * limbs;
    const int mf = order > 0, big = endian > 0;
    const uint32_t g = grid_for(total);
    cudaError_t e = cudaSuccess;
    switch (size) {
        case 1: e = launch_pdl(k_import<1>, g, 256, 0, st, static_cast<const uint8_t*>(src), dst, total, words, limbs, mf, big); break;
        case 2: e = launch_pdl(k_import<2>, g, 256, 0, st, static_cast<const uint16_t*>(src), dst, total, words, limbs, mf, big); break;
        case 4: e = launch_pdl(k_import<4>, g, 256, 0, st, static_cast<const uint32_t*>(src), dst, total, words, limbs, mf, big); break;
        case 8: e = launch_pdl(k_import<8>, g, 256, 0, st, static_cast<const uint64_t*>(src), dst, total, words, limbs, mf, big); break;
        default: return set_error(MI_EINVAL, "import: word size %u not 1, 2, 4 or 8", size);
    }
    MI_CUDA_TRY(e);
    return MI_OK;
}

mi_status launch_export(const uint64_t* src, void* dst, uint32_t n, uint32_t limbs, uint32_t words, uint32_t size,
                        int order, int endian, uint32_t* counts, cudaStream_t st) {
    const uint64_t total = uint64_t(n) * words;
    const int mf = order > 0, big = endian > 0;
    const uint32_t g = grid_for(total);
    cudaError_t e = cudaSuccess;
    switch (size) {
        case 1: e = launch_pdl(k_export<1>, g, 256, 0, st, src, static_cast<uint8_t*>(dst), total, limbs, words, mf, big); break;
        case 2: e = launch_pdl(k_export<2>, g, 256, 0, st, src, static_cast<uint16_t*>(dst), total, limbs, words, mf, big); break;
        case 4: e = launch_pdl(k_export<4>, g, 256, 0, st, src, static_cast<uint32_t*>(dst), total, limbs, words, mf, big); break;
        case 8: e = launch_pdl(k_export<8>, g, 256, 0, st, src, static_cast<uint64_t*>(dst), total, limbs, words, mf, big); break;
        default: return set_error(MI_EINVAL, "export: word size %u not 1, 2, 4 or 8", size);
    }
    MI_CUDA_TRY(e);
    if (counts != nullptr) {
        MI_CUDA_TRY(launch_pdl(k_count_words, grid_for(uint64_t(n) * 32), 256, 0, st, src, counts, n, limbs, size));
    }
    return MI_OK;
}

}  // namespace mi
