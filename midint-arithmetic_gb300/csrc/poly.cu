// poly.cu -- the fused polynomial composite ((a^2 + b)(b^2 + b) + ab) mod
// 2^(32*n32), the reference's polyKerQ (cuda/ker-classic-mul.cu.h:500-575), as
// four low-half products (classic::low_product) and three sums in one kernel.
#include <cstdio>

#include "mul_lo.cuh"

namespace mi {
namespace {

using classic::T;

// Block q (limbs qT..qT+T-1) of an n32-limb row, zero beyond n32.
template <bool VEC>
__device__ __forceinline__ void load_block(uint32_t (&x)[T], const uint32_t* __restrict__ row, uint32_t q,
                                           uint32_t n32, bool valid) {
    const uint32_t o = q * T;
    if (VEC && valid && o + T <= n32) {
#pragma unroll
        for (int h = 0; h < T / 4; ++h) {
            const uint4 v = __ldcs(reinterpret_cast<const uint4*>(row + o) + h);
            x[4 * h] = v.x, x[4 * h + 1] = v.y, x[4 * h + 2] = v.z, x[4 * h + 3] = v.w;
        }
    } else {
#pragma unroll
        for (int w = 0; w < T; ++w) x[w] = (valid && o + w < n32) ? __ldcs(row + o + w) : 0u;
    }
}

// A thread's two blocks (q and NH+q) of an operand held in registers.
struct Pair {
    uint32_t lo[T], hi[T];
};

// Zeroes the limbs at or beyond n32 (everything is mod 2^(32*n32)).
template <int NH>
__device__ __forceinline__ void mask_pair(Pair& x, uint32_t q, uint32_t n32) {
#pragma unroll
    for (int w = 0; w < T; ++w) {
        if (q * T + w >= n32) x.lo[w] = 0;
        if ((NH + q) * T + w >= n32) x.hi[w] = 0;
    }
}

// Stages register operands x (as A) and y (as B) in the plane layout.
template <int NH>
__device__ __forceinline__ void stage_pair(uint4* g4, uint32_t q, const Pair& x) {
    constexpr int NB = 2 * NH;
    g4[q] = make_uint4(x.lo[0], x.lo[1], x.lo[2], x.lo[3]);
    g4[NB + q] = make_uint4(x.lo[4], x.lo[5], x.lo[6], x.lo[7]);
    g4[NH + q] = make_uint4(x.hi[0], x.hi[1], x.hi[2], x.hi[3]);
    g4[NB + NH + q] = make_uint4(x.hi[4], x.hi[5], x.hi[6], x.hi[7]);
}

// (x + y) mod 2^(32*T*NB) over the group's blocks.
template <int NH>
__device__ __forceinline__ void add_pair(const Pair& x, const Pair& y, Pair& r, uint32_t* scr) {
    bool g0, p0, g1, p1;
    uint32_t c0, c1;
    chunk_add<uint32_t, T>(x.lo, y.lo, r.lo, g0, p0);
    chunk_add<uint32_t, T>(x.hi, y.hi, r.hi, g1, p1);
    const uint32_t cl = group_carry<NH>(g0, p0, 0u, &c0, scr);
    const uint32_t ch = group_carry<NH>(g1, p1, c0, &c1, scr);
    chunk_inc<uint32_t, T>(r.lo, cl);
    chunk_inc<uint32_t, T>(r.hi, ch);
}

// r = ((a^2 + b)(b^2 + b) + ab) mod 2^(32*n32): the composite of the
// reference's polyKerQ (cuda/ker-classic-mul.cu.h:500-575) in one kernel, as
// four low-half products.  The group keeps its blocks of a, b and the partial
// results in registers and restages the operands of each product in shared
// memory; ab is formed first so that a is dead after a^2.
template <int NH, bool VEC>
__global__ void __launch_bounds__(NH > 256 ? NH : 256, 2)
    k_poly(const uint32_t* __restrict__ a, const uint32_t* __restrict__ b, uint32_t* __restrict__ r, uint32_t n,
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
    // per-warp carry words of wide groups: the operand area, which is free
    // whenever a carry is resolved (after a product's tile loop, and between a
    // product and the next staging)
    uint32_t* scr = sA;
    const uint32_t nb = (n32 + T - 1) / T;
    const uint64_t stride = uint64_t(gridDim.x) * S::IPB;
    pdl_wait();  // launched with launch_pdl
    pdl_trigger();
    for (uint64_t base = uint64_t(blockIdx.x) * S::IPB; base < n; base += stride) {
        const uint64_t inst = base + grp;
        const bool valid = inst < n;
        Pair xa, xb, t6, u, v;
        {
            const uint32_t* ra = a + (valid ? inst * n32 : 0);
            const uint32_t* rb = b + (valid ? inst * n32 : 0);
            load_block<VEC>(xa.lo, ra, t, n32, valid);
            load_block<VEC>(xa.hi, ra, NH + t, n32, valid);
            load_block<VEC>(xb.lo, rb, t, n32, valid);
            load_block<VEC>(xb.hi, rb, NH + t, n32, valid);
        }
        stage_pair<NH>(gA4, t, xa);  // t6 = a*b
        stage_pair<NH>(gB4, t, xb);
        group_sync<NH>();
        classic::low_product<NH>(gA4, gB4, slots, scr, t, t6.lo, t6.hi, nb);
        mask_pair<NH>(t6, t, n32);
        group_sync<NH>();
        stage_pair<NH>(gA4, t, xa);  // t1 = a*a
        stage_pair<NH>(gB4, t, xa);
        group_sync<NH>();
        classic::low_product<NH>(gA4, gB4, slots, scr, t, u.lo, u.hi, nb);
        mask_pair<NH>(u, t, n32);
        group_sync<NH>();
        add_pair<NH>(u, xb, xa, scr);  // t2 = t1 + b (into xa)
        mask_pair<NH>(xa, t, n32);
        stage_pair<NH>(gA4, t, xb);  // t3 = b*b
        stage_pair<NH>(gB4, t, xb);
        group_sync<NH>();
        classic::low_product<NH>(gA4, gB4, slots, scr, t, u.lo, u.hi, nb);
        mask_pair<NH>(u, t, n32);
        group_sync<NH>();
        add_pair<NH>(u, xb, v, scr);  // t4 = t3 + b
        mask_pair<NH>(v, t, n32);
        stage_pair<NH>(gA4, t, xa);  // t5 = t2*t4
        stage_pair<NH>(gB4, t, v);
        group_sync<NH>();
        classic::low_product<NH>(gA4, gB4, slots, scr, t, u.lo, u.hi, nb);
        mask_pair<NH>(u, t, n32);
        group_sync<NH>();
        add_pair<NH>(u, t6, v, scr);  // r = t5 + t6
        if (valid) {
            uint32_t* rr = r + inst * n32;
            classic::store_block<VEC>(rr, t * T, n32, v.lo);
            classic::store_block<VEC>(rr, (NH + t) * T, n32, v.hi);
        }
        group_sync<NH>();
    }
}

template <bool VEC>
mi_status dispatch(const uint32_t* a, const uint32_t* b, uint32_t* r, uint32_t n, uint32_t n32, cudaStream_t st) {
    switch (lo_threads(n32)) {
#define MI_LO_CASE(NH) \
    case NH: return launch_lo<NH>(k_poly<NH, VEC>, a, b, r, n, n32, st);
        MI_LO_CASE(1) MI_LO_CASE(2) MI_LO_CASE(4) MI_LO_CASE(8) MI_LO_CASE(16) MI_LO_CASE(32) MI_LO_CASE(64)
        MI_LO_CASE(128) MI_LO_CASE(256)
#undef MI_LO_CASE
        default: return set_error(MI_EINVAL, "poly: %u u32 limbs exceeds the classical maximum", n32);
    }
}

}  // namespace

mi_status launch_poly(const uint32_t* a, const uint32_t* b, uint32_t* r, uint32_t n, uint32_t n32, cudaStream_t st) {
    const bool vec = aligned16(a) && aligned16(b) && aligned16(r) && (n32 % 4 == 0);
    return vec ? dispatch<true>(a, b, r, n, n32, st) : dispatch<false>(a, b, r, n, n32, st);
}

}  // namespace mi
