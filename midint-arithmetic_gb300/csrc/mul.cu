// mul.cu -- batched classical (quadratic) multiplication on 32-bit limbs.
//
// Counterpart of the reference's bmulKerQ (cuda/ker-classic-mul.cu.h:468-498),
// which returns the low half of the product of two m-limb operands.  Each
// instance is one square product of mul_core.cuh, computed by a group of
// NT = pow2ceil(n32/8) threads; a block of max(256, NT) threads holds 256/NT
// groups and strides over the batch.  `full` selects the 2*n32-limb product or
// its low n32 limbs (the reference's semantics).
#include <cstdio>

#include "common.cuh"
#include "kernels.h"
#include "mul_core.cuh"

namespace mi {
namespace {

using classic::T;

template <int NT>
struct MulShape {
    static constexpr int BLOCK = NT > 256 ? NT : 256;
    static constexpr int IPB = BLOCK / NT;   // instances per block
    static constexpr int WPAD = NT * T;      // padded limbs per operand
    // operands (2 x IPB x WPAD words) + per-thread snapshot/combine words; the
    // per-warp words of wide groups' carry resolution reuse the operand area.
    static constexpr size_t SMEM = size_t(2 * IPB * WPAD + BLOCK * classic::PER_T) * 4;
};

template <int NT, bool VEC>
__global__ void __launch_bounds__(NT > 256 ? NT : 256)
    k_mul(const uint32_t* __restrict__ a, const uint32_t* __restrict__ b, uint32_t* __restrict__ r, uint32_t n,
          uint32_t n32, bool full) {
    using S = MulShape<NT>;
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
    const uint64_t stride = uint64_t(gridDim.x) * S::IPB;

    // Every group of a block runs the same trip count (wide groups synchronise
    // the whole block).
    for (uint64_t base = uint64_t(blockIdx.x) * S::IPB; base < n; base += stride) {
        const uint64_t inst = base + grp;
        const bool valid = inst < n;
        const uint64_t off = valid ? inst * n32 : 0;
        classic::stage_a<NT, VEC>(gA, a + off, n32, valid, t);
        classic::stage_b<NT, VEC>(gB4, b + off, n32, valid, t);
        group_sync<NT>();
        uint32_t ulo[T], uhi[T];
        classic::square_product<NT>(gA, gB4, slots, scr, t, ulo, uhi);
        if (valid) {
            uint32_t* rr = r + inst * rlen;
            classic::store_block<VEC>(rr, t * T, rlen, ulo);
            if (full) classic::store_block<VEC>(rr, (t + NT) * T, rlen, uhi);
        }
        group_sync<NT>();  // shared memory is reused by the next instance
    }
}

// Stages the thread's block t of two register operands as the group's A and
// B (plane layout) operands.
template <int NT>
__device__ __forceinline__ void stage_regs(uint32_t* gA, uint4* gB4, uint32_t t, const uint32_t (&x)[T],
                                           const uint32_t (&y)[T]) {
    reinterpret_cast<uint4*>(gA + t * T)[0] = make_uint4(x[0], x[1], x[2], x[3]);
    reinterpret_cast<uint4*>(gA + t * T)[1] = make_uint4(x[4], x[5], x[6], x[7]);
    gB4[t] = make_uint4(y[0], y[1], y[2], y[3]);
    gB4[NT + t] = make_uint4(y[4], y[5], y[6], y[7]);
}

// Block t (limbs tT..tT+T-1) of an n32-limb row, zero beyond n32.
template <bool VEC>
__device__ __forceinline__ void load_block(uint32_t (&x)[T], const uint32_t* __restrict__ row, uint32_t t,
                                           uint32_t n32, bool valid) {
    const uint32_t o = t * T;
    if (VEC && valid && o + T <= n32) {
#pragma unroll
        for (int q = 0; q < T / 4; ++q) {
            const uint4 v = __ldcs(reinterpret_cast<const uint4*>(row + o) + q);
            x[4 * q] = v.x, x[4 * q + 1] = v.y, x[4 * q + 2] = v.z, x[4 * q + 3] = v.w;
        }
    } else {
#pragma unroll
        for (int w = 0; w < T; ++w) x[w] = (valid && o + w < n32) ? __ldcs(row + o + w) : 0u;
    }
}

// Zeroes the limbs of block t at or beyond n32 (everything is mod 2^(32*n32)).
__device__ __forceinline__ void mask_block(uint32_t (&x)[T], uint32_t t, uint32_t n32) {
#pragma unroll
    for (int w = 0; w < T; ++w)
        if (t * T + w >= n32) x[w] = 0;
}

// (x + y) mod 2^(32*NT*T) over the group's low blocks.
template <int NT>
__device__ __forceinline__ void add_low(const uint32_t (&x)[T], const uint32_t (&y)[T], uint32_t (&r)[T],
                                        uint32_t* scr) {
    bool g, p;
    uint32_t gc;
    chunk_add<uint32_t, T>(x, y, r, g, p);
    chunk_inc<uint32_t, T>(r, group_carry<NT>(g, p, 0u, &gc, scr));
}

// r = ((a^2 + b)(b^2 + b) + ab) mod 2^(32*n32): the composite of the
// reference's polyKerQ (cuda/ker-classic-mul.cu.h:500-575) in one kernel; the
// group keeps its blocks of a and b in registers and restages the operands of
// each of the four products in shared memory.
template <int NT, bool VEC>
__global__ void __launch_bounds__(NT > 256 ? NT : 256)
    k_poly(const uint32_t* __restrict__ a, const uint32_t* __restrict__ b, uint32_t* __restrict__ r, uint32_t n,
           uint32_t n32) {
    using S = MulShape<NT>;
    extern __shared__ __align__(16) uint32_t smem[];
    uint32_t* sA = smem;
    uint32_t* sB = sA + S::IPB * S::WPAD;
    uint32_t* sT = sB + S::IPB * S::WPAD;
    const uint32_t grp = threadIdx.x / NT;
    const uint32_t t = threadIdx.x % NT;
    uint32_t* gA = sA + grp * S::WPAD;
    uint4* gB4 = reinterpret_cast<uint4*>(sB + grp * S::WPAD);
    uint2* slots = reinterpret_cast<uint2*>(sT) + grp * NT * classic::PAIRS;
    // per-warp carry words of wide groups: the operand area, which is free
    // whenever a carry is resolved (after a product's tile loop, and between a
    // product and the next staging)
    uint32_t* scr = sA;
    const uint64_t stride = uint64_t(gridDim.x) * S::IPB;
    for (uint64_t base = uint64_t(blockIdx.x) * S::IPB; base < n; base += stride) {
        const uint64_t inst = base + grp;
        const bool valid = inst < n;
        uint32_t xa[T], xb[T];
        load_block<VEC>(xa, a + (valid ? inst * n32 : 0), t, n32, valid);
        load_block<VEC>(xb, b + (valid ? inst * n32 : 0), t, n32, valid);
        uint32_t lo[T], hi[T], t2[T], t4[T], t5[T];
        stage_regs<NT>(gA, gB4, t, xa, xa);  // t1 = a*a
        group_sync<NT>();
        classic::square_product<NT>(gA, gB4, slots, scr, t, lo, hi);
        mask_block(lo, t, n32);
        group_sync<NT>();
        add_low<NT>(lo, xb, t2, scr);  // t2 = t1 + b
        mask_block(t2, t, n32);
        stage_regs<NT>(gA, gB4, t, xb, xb);  // t3 = b*b
        group_sync<NT>();
        classic::square_product<NT>(gA, gB4, slots, scr, t, lo, hi);
        mask_block(lo, t, n32);
        group_sync<NT>();
        add_low<NT>(lo, xb, t4, scr);  // t4 = t3 + b
        mask_block(t4, t, n32);
        stage_regs<NT>(gA, gB4, t, t2, t4);  // t5 = t2*t4
        group_sync<NT>();
        classic::square_product<NT>(gA, gB4, slots, scr, t, t5, hi);
        mask_block(t5, t, n32);
        group_sync<NT>();
        stage_regs<NT>(gA, gB4, t, xa, xb);  // t6 = a*b
        group_sync<NT>();
        classic::square_product<NT>(gA, gB4, slots, scr, t, lo, hi);
        mask_block(lo, t, n32);
        group_sync<NT>();
        uint32_t res[T];
        add_low<NT>(t5, lo, res, scr);  // r = t5 + t6
        if (valid) classic::store_block<VEC>(r + inst * n32, t * T, n32, res);
        group_sync<NT>();
    }
}

template <int NT, bool VEC>
mi_status launch_nt(const uint32_t* a, const uint32_t* b, uint32_t* r, uint32_t n, uint32_t n32, bool full,
                    cudaStream_t st) {
    using S = MulShape<NT>;
    auto kern = k_mul<NT, VEC>;
    static bool attr_done[64] = {};
    int dev = 0;
    MI_CUDA_TRY(cudaGetDevice(&dev));
    if (dev >= 0 && dev < 64 && !attr_done[dev]) {
        MI_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(S::SMEM)));
        attr_done[dev] = true;
    }
    uint64_t blocks = (uint64_t(n) + S::IPB - 1) / S::IPB;
    const uint64_t cap = uint64_t(sm_count()) * 32;
    if (blocks > cap) blocks = cap;
    kern<<<dim3(uint32_t(blocks)), dim3(S::BLOCK), S::SMEM, st>>>(a, b, r, n, n32, full);
    MI_CUDA_TRY(cudaGetLastError());
    return MI_OK;
}

template <bool VEC>
mi_status dispatch(const uint32_t* a, const uint32_t* b, uint32_t* r, uint32_t n, uint32_t n32, bool full,
                   cudaStream_t st) {
    const uint32_t nt = pow2ceil((n32 + T - 1) / T);
    switch (nt) {
        case 1: return launch_nt<1, VEC>(a, b, r, n, n32, full, st);
        case 2: return launch_nt<2, VEC>(a, b, r, n, n32, full, st);
        case 4: return launch_nt<4, VEC>(a, b, r, n, n32, full, st);
        case 8: return launch_nt<8, VEC>(a, b, r, n, n32, full, st);
        case 16: return launch_nt<16, VEC>(a, b, r, n, n32, full, st);
        case 32: return launch_nt<32, VEC>(a, b, r, n, n32, full, st);
        case 64: return launch_nt<64, VEC>(a, b, r, n, n32, full, st);
        case 128: return launch_nt<128, VEC>(a, b, r, n, n32, full, st);
        case 256: return launch_nt<256, VEC>(a, b, r, n, n32, full, st);
        default: return set_error(MI_EINVAL, "mul: %u u32 limbs exceeds the classical maximum", n32);
    }
}

template <int NT, bool VEC>
mi_status launch_poly_nt(const uint32_t* a, const uint32_t* b, uint32_t* r, uint32_t n, uint32_t n32,
                         cudaStream_t st) {
    using S = MulShape<NT>;
    auto kern = k_poly<NT, VEC>;
    static bool attr_done[64] = {};
    int dev = 0;
    MI_CUDA_TRY(cudaGetDevice(&dev));
    if (dev >= 0 && dev < 64 && !attr_done[dev]) {
        MI_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(S::SMEM)));
        attr_done[dev] = true;
    }
    uint64_t blocks = (uint64_t(n) + S::IPB - 1) / S::IPB;
    const uint64_t cap = uint64_t(sm_count()) * 32;
    if (blocks > cap) blocks = cap;
    kern<<<dim3(uint32_t(blocks)), dim3(S::BLOCK), S::SMEM, st>>>(a, b, r, n, n32);
    MI_CUDA_TRY(cudaGetLastError());
    return MI_OK;
}

template <bool VEC>
mi_status dispatch_poly(const uint32_t* a, const uint32_t* b, uint32_t* r, uint32_t n, uint32_t n32,
                        cudaStream_t st) {
    switch (pow2ceil((n32 + T - 1) / T)) {
        case 1: return launch_poly_nt<1, VEC>(a, b, r, n, n32, st);
        case 2: return launch_poly_nt<2, VEC>(a, b, r, n, n32, st);
        case 4: return launch_poly_nt<4, VEC>(a, b, r, n, n32, st);
        case 8: return launch_poly_nt<8, VEC>(a, b, r, n, n32, st);
        case 16: return launch_poly_nt<16, VEC>(a, b, r, n, n32, st);
        case 32: return launch_poly_nt<32, VEC>(a, b, r, n, n32, st);
        case 64: return launch_poly_nt<64, VEC>(a, b, r, n, n32, st);
        case 128: return launch_poly_nt<128, VEC>(a, b, r, n, n32, st);
        case 256: return launch_poly_nt<256, VEC>(a, b, r, n, n32, st);
        default: return set_error(MI_EINVAL, "poly: %u u32 limbs exceeds the classical maximum", n32);
    }
}

}  // namespace

mi_status launch_poly(const uint32_t* a, const uint32_t* b, uint32_t* r, uint32_t n, uint32_t n32, cudaStream_t st) {
    const bool vec = aligned16(a) && aligned16(b) && aligned16(r) && (n32 % 4 == 0);
    return vec ? dispatch_poly<true>(a, b, r, n, n32, st) : dispatch_poly<false>(a, b, r, n, n32, st);
}

mi_status launch_mul_classic(const uint32_t* a, const uint32_t* b, uint32_t* r, uint32_t n, uint32_t n32, bool full,
                             cudaStream_t st) {
    const bool vec = aligned16(a) && aligned16(b) && aligned16(r) && (n32 % 4 == 0);
    return vec ? dispatch<true>(a, b, r, n, n32, full, st) : dispatch<false>(a, b, r, n, n32, full, st);
}

}  // namespace mi
