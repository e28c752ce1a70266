// mul.cu -- batched classical (quadratic) multiplication on 32-bit limbs.
//
// Counterpart of the reference's bmulKerQ (cuda/ker-classic-mul.cu.h:468-498),
// which returns the low half of the product of two m-limb operands.  Each
// instance is one square product of mul_core.cuh, computed by a group of
// NT = pow2ceil(n32/8) threads.  Groups of 16 or 32 threads run in blocks of
// one warp, launched as one block per warp's worth of instances: the blocks
// of an SM then start and finish at different times, so one warp's carry
// resolution overlaps the others' tile loops, and the last wave spreads
// evenly over the SMs (persistent blocks striding over the batch stay in phase
// and measured 8-10 % slower; eight instances per 256-thread block 3 %
// slower).  Other sizes, and launches capped at a few resident blocks per SM
// (the zero-copy host path, whose cap was tuned on them), use blocks of
// max(256, NT) threads that stride over the batch.  `full` selects the 2*n32-limb product or its low n32 limbs (the
// reference's semantics); low halves of more than one block of limbs go to the
// half-work kernel of mul_lo.cu.
#include <cstdio>

#include "common.cuh"
#include "kernels.h"
#include "mul_core.cuh"

namespace mi {
namespace {

using classic::T;

template <int NT, bool WB = false>
struct MulShape {
    static constexpr bool WARP = WB && (NT == 16 || NT == 32);  // one-warp blocks
    static constexpr int BLOCK = WARP ? 32 : (NT > 256 ? NT : 256);
    // one-warp blocks: 16 per SM for 32-thread groups (up to 128 registers:
    // 0.1376 -> 0.1362 ms on the 8192-bit batch against 24 at 80; 20, 14 and
    // 12 measured 0.1367, 0.1368 and 0.1428 ms), 24 for 16-thread groups;
    // 256-thread blocks of 16- or 32-thread groups serve only the capped
    // zero-copy launches (two resident blocks per SM there), whose groups keep
    // the next instance's operands in registers
    static constexpr int MIN_BLOCKS = WARP ? (NT == 32 ? 16 : 24)
                                           : (NT >= 512 ? 1 : (NT == 2 || NT == 16 || NT == 32 ? 2 : 3));
    static constexpr int IPB = BLOCK / NT;   // instances per block
    static constexpr int WPAD = NT * T;      // padded limbs per operand
    // operands (2 x IPB x WPAD words) + per-thread snapshot/combine words; the
    // per-warp words of wide groups' carry resolution reuse the operand area.
    static constexpr size_t SMEM = size_t(2 * IPB * WPAD + BLOCK * classic::PER_T) * 4;
};

template <int NT, bool VEC, bool WB>
__global__ void __launch_bounds__(MulShape<NT, WB>::BLOCK, MulShape<NT, WB>::MIN_BLOCKS)
    k_mul(const uint32_t* __restrict__ a, const uint32_t* __restrict__ b, uint32_t* __restrict__ r, uint32_t n,
          uint32_t n32, bool full) {
    using S = MulShape<NT, WB>;
    extern __shared__ __align__(16) uint32_t smem[];
    uint32_t* sA = smem;
    uint32_t* sB = sA + S::IPB * S::WPAD;
    uint32_t* sT = sB + S::IPB * S::WPAD;

    const uint32_t grp = threadIdx.x / NT;
    const uint32_t t = threadIdx.x % NT;
    uint32_t* gA = sA + grp * S::WPAD;
    uint4* gB4 = reinterpret_cast<uint4*>(sB + grp * S::WPAD);
    uint2* slots = reinterpret_cast<uint2*>(sT) + grp * NT * classic::PAIRS;
    uint32_t* scr = sA;  // only used after the tile loop, by groups wider than a warp
    const uint32_t rlen = full ? 2 * n32 : n32;
    const uint32_t nb = (n32 + T - 1) / T;  // blocks holding limbs; the rest of the NT are zero padding
    const uint64_t stride = uint64_t(gridDim.x) * S::IPB;
    pdl_wait();  // launched with launch_pdl
    pdl_trigger();

    if constexpr ((NT == 16 || NT == 32) && !S::WARP && VEC) {
        if (full && n32 == NT * T) {
            // The capped launches of the zero-copy host path, whose rows are
            // host-mapped: each group reads the operands of its next instance
            // into registers while it multiplies this one, and its product
            // leaves through the group's operand areas as stores of whole
            // 16-byte slots in order (one contiguous 16*NT-byte run per warp
            // instruction rather than every other slot).  0.250 -> 0.242 ms for
            // the 8192-bit batch of 16384 products over the host link.
            uint4 qa[T / 4], qb[T / 4];
            uint64_t inst = uint64_t(blockIdx.x) * S::IPB + grp;
            classic::fetch_ab<NT, true>(qa, qb, a + inst * n32, b + inst * n32, n32, inst < n, t);
            uint4* gA4 = reinterpret_cast<uint4*>(gA);
            for (uint64_t base = uint64_t(blockIdx.x) * S::IPB; base < n; base += stride, inst += stride) {
                classic::put_ab<NT>(gA, gB4, qa, qb, t);
                group_sync<NT>();
                const uint64_t next = inst + stride;  // past the batch: nothing is read (valid = false)
                classic::fetch_ab<NT, true>(qa, qb, a + next * n32, b + next * n32, n32, next < n, t);
                uint32_t ulo[T], uhi[T];
                classic::square_product<NT, 1, NT, false>(gA, gB4, slots, scr, t, ulo, uhi, NT);
                if (inst < n) {
                    group_sync<NT>();  // the group's operand reads are done
                    gA4[2 * t] = make_uint4(ulo[0], ulo[1], ulo[2], ulo[3]);
                    gA4[2 * t + 1] = make_uint4(ulo[4], ulo[5], ulo[6], ulo[7]);
                    gB4[2 * t] = make_uint4(uhi[0], uhi[1], uhi[2], uhi[3]);
                    gB4[2 * t + 1] = make_uint4(uhi[4], uhi[5], uhi[6], uhi[7]);
                    group_sync<NT>();
                    uint4* r4 = reinterpret_cast<uint4*>(r + inst * rlen);  // 4*NT slots
                    __stcs(r4 + t, gA4[t]);
                    __stcs(r4 + NT + t, gA4[NT + t]);
                    __stcs(r4 + 2 * NT + t, gB4[t]);
                    __stcs(r4 + 3 * NT + t, gB4[NT + t]);
                }
                group_sync<NT>();  // shared memory is reused by the next instance
            }
            return;
        }
    }

    // Every group of a block runs the same trip count (wide groups synchronise
    // the whole block).
    for (uint64_t base = uint64_t(blockIdx.x) * S::IPB; base < n; base += stride) {
        const uint64_t inst = base + grp;
        const bool valid = inst < n;
        const uint64_t off = valid ? inst * n32 : 0;
        classic::stage_ab<NT, VEC>(gA, gB4, a + off, b + off, n32, valid, t);
        group_sync<NT>();
        uint32_t ulo[T], uhi[T];
        if (nb == NT)  // no padding: a compile-time trip count, unrolled in full for 8..32 steps; the
                       // 32-thread groups in one-warp blocks prefetch each step's operands (the other
                       // shapes would spill)
            classic::square_product<NT, 1, (NT >= 8 && NT <= 32) ? NT : (NT >= 16 ? 8 : 2), NT == 32 && S::WARP>(
                gA, gB4, slots, scr, t, ulo, uhi, NT);
        else
            classic::square_product<NT>(gA, gB4, slots, scr, t, ulo, uhi, nb);
        if (valid) {
            uint32_t* rr = r + inst * rlen;
            classic::store_block<VEC>(rr, t * T, rlen, ulo);
            if (full) classic::store_block<VEC>(rr, (t + NT) * T, rlen, uhi);
        }
        group_sync<NT>();  // shared memory is reused by the next instance
    }
}

// Dynamic shared memory that leaves room for at most max_per_sm blocks of a
// kernel per SM (at least `smem`, at most the per-block maximum).
mi_status capped_smem(size_t smem, uint32_t max_per_sm, size_t* out) {
    *out = smem;
    if (max_per_sm == 0) return MI_OK;
    int dev = 0, per_sm = 0, reserved = 0, per_block = 0;
    MI_CUDA_TRY(cudaGetDevice(&dev));
    MI_CUDA_TRY(cudaDeviceGetAttribute(&per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev));
    MI_CUDA_TRY(cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev));
    MI_CUDA_TRY(cudaDeviceGetAttribute(&per_block, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    // max_per_sm + 1 blocks of `need` bytes (plus the reservation) overflow the SM
    const size_t need = size_t(per_sm) / (max_per_sm + 1) + 1024 - size_t(reserved);
    if (need > *out) *out = need < size_t(per_block) ? need : size_t(per_block);
    return MI_OK;
}

template <int NT, bool VEC, bool WB>
mi_status launch_shape(const uint32_t* a, const uint32_t* b, uint32_t* r, uint32_t n, uint32_t n32, bool full,
                       cudaStream_t st, uint32_t max_per_sm) {
    using S = MulShape<NT, WB>;
    auto kern = k_mul<NT, VEC, WB>;
    size_t smem = S::SMEM;
    MI_TRY(capped_smem(S::SMEM, max_per_sm, &smem));
    MI_TRY(ensure_dyn_smem(kern, smem));
    uint64_t blocks = (uint64_t(n) + S::IPB - 1) / S::IPB;
    // one block per unit of work for one-warp blocks (see above); the others
    // stride over the batch from a grid of a few waves
    const uint64_t cap = S::WARP ? (uint64_t(1) << 24) : uint64_t(sm_count()) * 32;
    if (blocks > cap) blocks = cap;
    MI_CUDA_TRY(launch_pdl(kern, dim3(uint32_t(blocks)), dim3(S::BLOCK), smem, st, a, b, r, n, n32, full));
    return MI_OK;
}

template <int NT, bool VEC>
mi_status launch_nt(const uint32_t* a, const uint32_t* b, uint32_t* r, uint32_t n, uint32_t n32, bool full,
                    cudaStream_t st, uint32_t max_per_sm) {
    if constexpr (NT == 16 || NT == 32)
        if (max_per_sm == 0) return launch_shape<NT, VEC, true>(a, b, r, n, n32, full, st, 0);
    return launch_shape<NT, VEC, false>(a, b, r, n, n32, full, st, max_per_sm);
}

template <bool VEC>
mi_status dispatch(const uint32_t* a, const uint32_t* b, uint32_t* r, uint32_t n, uint32_t n32, bool full,
                   cudaStream_t st, uint32_t cap) {
    const uint32_t nt = pow2ceil((n32 + T - 1) / T);
    switch (nt) {
        case 1: return launch_nt<1, VEC>(a, b, r, n, n32, full, st, cap);
        case 2: return launch_nt<2, VEC>(a, b, r, n, n32, full, st, cap);
        case 4: return launch_nt<4, VEC>(a, b, r, n, n32, full, st, cap);
        case 8: return launch_nt<8, VEC>(a, b, r, n, n32, full, st, cap);
        case 16: return launch_nt<16, VEC>(a, b, r, n, n32, full, st, cap);
        case 32: return launch_nt<32, VEC>(a, b, r, n, n32, full, st, cap);
        case 64: return launch_nt<64, VEC>(a, b, r, n, n32, full, st, cap);
        case 128: return launch_nt<128, VEC>(a, b, r, n, n32, full, st, cap);
        case 256: return launch_nt<256, VEC>(a, b, r, n, n32, full, st, cap);
        case 512: return launch_nt<512, VEC>(a, b, r, n, n32, full, st, cap);
        default: return set_error(MI_EINVAL, "mul: %u u32 limbs exceeds the classical maximum", n32);
    }
}

}  // namespace

mi_status launch_mul_classic(const uint32_t* a, const uint32_t* b, uint32_t* r, uint32_t n, uint32_t n32, bool full,
                             cudaStream_t st, uint32_t max_per_sm) {
    const bool vec = aligned16(a) && aligned16(b) && aligned16(r) && (n32 % 4 == 0);
    if (!full && n32 > T)  // low halves: half the partial products of a full product
        return launch_mul_lo(a, b, r, n, n32, st);
    return vec ? dispatch<true>(a, b, r, n, n32, full, st, max_per_sm)
               : dispatch<false>(a, b, r, n, n32, full, st, max_per_sm);
}

}  // namespace mi
