// mul_lo.cu -- batched low-half classical products.
//
// The reference's bmulKerQ (cuda/ker-classic-mul.cu.h:468-498) returns the low
// m limbs of m-limb products.  Only the anti-diagonals below the middle of the
// partial-product grid reach those limbs, so this kernel uses
// classic::low_product (half the partial products of a full product).
#include <cstdio>

#include "mul_lo.cuh"

namespace mi {
namespace {

using classic::T;

// The low n32 limbs of a*b (the reference's bmulKerQ semantics) with half the
// partial products of a full product: classic::low_product per instance.
template <int NH, bool VEC>
__global__ void __launch_bounds__(NH > 256 ? NH : 256, 3)
    k_mul_lo(const uint32_t* __restrict__ a, const uint32_t* __restrict__ b, uint32_t* __restrict__ r, uint32_t n,
             uint32_t n32) {
    using S = LoShape<NH>;
    extern __shared__ __align__(16) uint32_t smem[];
    uint32_t* sA = smem;
    uint32_t* sB = sA + S::IPB * S::WPAD;
    uint32_t* sT = sB + S::IPB * S::WPAD;
    const uint32_t grp = threadIdx.x / NH;
    const uint32_t t = threadIdx.x % NH;
    uint4* gA4 = reinterpret_cast<uint4*>(sA + grp * S::WPAD);
    uint4* gB4 = reinterpret_cast<uint4*>(sB + grp * S::WPAD);
    uint2* slots = reinterpret_cast<uint2*>(sT) + grp * NH * classic::PAIRS;
    uint32_t* scr = sA;  // only used after the tile loop, by groups wider than a warp
    const uint32_t nb = (n32 + T - 1) / T;  // blocks holding limbs; the rest of the NB are zero padding
    const uint64_t stride = uint64_t(gridDim.x) * S::IPB;
    pdl_wait();  // launched with launch_pdl
    pdl_trigger();
    for (uint64_t base = uint64_t(blockIdx.x) * S::IPB; base < n; base += stride) {
        const uint64_t inst = base + grp;
        const bool valid = inst < n;
        const uint64_t off = valid ? inst * n32 : 0;
        classic::stage_planes<S::NB, NH, VEC>(gA4, a + off, n32, valid, t);
        classic::stage_planes<S::NB, NH, VEC>(gB4, b + off, n32, valid, t);
        group_sync<NH>();
        uint32_t ulo[T], uhi[T];
        if (nb == S::NB)  // no padding: a compile-time trip count, unrolled in full for 9..65 steps
            // each step's operands read one step ahead for 16- and 32-thread groups
            // on aligned rows (8192-bit batch 0.0776 -> 0.0757 ms; the other shapes
            // would spill more)
            classic::low_product<NH, (NH >= 4 && NH <= 32) ? 2 * NH + 1 : (NH >= 16 ? 8 : 2),
                                 VEC && (NH == 16 || NH == 32)>(gA4, gB4, slots, scr, t, ulo, uhi, S::NB);
        else
            classic::low_product<NH>(gA4, gB4, slots, scr, t, ulo, uhi, nb);
        if (valid) {
            uint32_t* rr = r + inst * n32;
            classic::store_block<VEC>(rr, t * T, n32, ulo);
            classic::store_block<VEC>(rr, (NH + t) * T, n32, uhi);
        }
        group_sync<NH>();
    }
}

template <bool VEC>
mi_status dispatch(const uint32_t* a, const uint32_t* b, uint32_t* r, uint32_t n, uint32_t n32, cudaStream_t st) {
    switch (lo_threads(n32)) {
#define MI_LO_CASE(NH) \
    case NH: return launch_lo<NH>(k_mul_lo<NH, VEC>, a, b, r, n, n32, st);
        MI_LO_CASE(1) MI_LO_CASE(2) MI_LO_CASE(4) MI_LO_CASE(8) MI_LO_CASE(16) MI_LO_CASE(32) MI_LO_CASE(64)
        MI_LO_CASE(128) MI_LO_CASE(256)
#undef MI_LO_CASE
        default: return set_error(MI_EINVAL, "mul: %u u32 limbs exceeds the classical maximum", n32);
    }
}

}  // namespace

mi_status launch_mul_lo(const uint32_t* a, const uint32_t* b, uint32_t* r, uint32_t n, uint32_t n32,
                        cudaStream_t st) {
    const bool vec = aligned16(a) && aligned16(b) && aligned16(r) && (n32 % 4 == 0);
    return vec ? dispatch<true>(a, b, r, n, n32, st) : dispatch<false>(a, b, r, n, n32, st);
}

}  // namespace mi
