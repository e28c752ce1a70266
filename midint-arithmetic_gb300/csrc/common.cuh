// common.cuh -- shared device primitives and host plumbing of the library.
//
// Limb layout (all kernels): instance i of an operand with m limbs occupies
// limbs [i*m, (i+1)*m), limb 0 least significant -- the layout of the
// reference's drivers and of its GMP oracle (cuda/helper.h:116, GMP_ORDER -1).
// A u64 limb is the little-endian pair of two u32 limbs, so a u64 buffer with m
// limbs is the same bytes as a u32 buffer with 2m limbs; the kernels use this
// to run u32 and u64 entry points on one code path.
#pragma once

#include <cstdint>
#include <cstddef>
#include <cuda_runtime.h>

#include "../../include/midint.h"

#define MI_FULL_MASK 0xffffffffu

namespace mi {

// ---------------------------------------------------------------------------
// Error plumbing (host).  Every entry point records a detail string in a
// thread-local buffer and returns a status; nothing aborts.
// ---------------------------------------------------------------------------
mi_status set_error(mi_status st, const char* fmt, ...);
mi_status cuda_error(cudaError_t e, const char* what);

#define MI_CUDA_TRY(expr)                                         \
    do {                                                          \
        cudaError_t _e = (expr);                                  \
        if (_e != cudaSuccess) return ::mi::cuda_error(_e, #expr); \
    } while (0)

#define MI_TRY(expr)                          \
    do {                                      \
        mi_status _s = (expr);                \
        if (_s != MI_OK) return _s;           \
    } while (0)

// Number of SMs of the current device (cached per device).
int sm_count();

// Raises the dynamic shared-memory limit of kernel `kern` on the current
// device to at least `bytes`, never lowering it; safe from several host
// threads (one lock, a per-kernel-and-device record of the limit set).
mi_status ensure_dyn_smem(const void* kern, size_t bytes);
template <typename K>
inline mi_status ensure_dyn_smem(K* kern, size_t bytes) {
    return ensure_dyn_smem(reinterpret_cast<const void*>(kern), bytes);
}

inline bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }
inline bool aligned8(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 7u) == 0; }

inline uint32_t pow2ceil(uint32_t x) {
    uint32_t p = 1;
    while (p < x) p <<= 1;
    return p;
}

// True when [p, p+bytes) and [q, q+bytes2) overlap without being identical.
inline bool partial_overlap(const void* p, size_t bytes, const void* q, size_t bytes2) {
    auto a0 = reinterpret_cast<uintptr_t>(p), b0 = reinterpret_cast<uintptr_t>(q);
    if (a0 == b0) return false;
    return a0 < b0 + bytes2 && b0 < a0 + bytes;
}
inline bool any_overlap(const void* p, size_t bytes, const void* q, size_t bytes2) {
    auto a0 = reinterpret_cast<uintptr_t>(p), b0 = reinterpret_cast<uintptr_t>(q);
    return a0 < b0 + bytes2 && b0 < a0 + bytes;
}

// Programmatic dependent launch.  A kernel launched with launch_pdl may have
// its blocks made resident while the previous kernel of the stream is still
// finishing; it must call pdl_wait() before its first global-memory access,
// which returns once that kernel has completed and its writes are visible.
// pdl_trigger() lets the next kernel's blocks start the same way once every
// block of this grid has called it.  The launch latency between back-to-back
// kernels then overlaps the previous kernel's tail.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                              Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kern, static_cast<KArgs>(args)...);
}

// ---------------------------------------------------------------------------
// Device primitives: 32-bit carry chains in PTX.  Each wrapper is one PTX
// instruction in its own `asm volatile`, so the compiler keeps them in program
// order and ptxas sees an unbroken condition-code chain.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void mad_lo_cc(uint32_t& d, uint32_t a, uint32_t b) {
    asm volatile("mad.lo.cc.u32 %0, %1, %2, %0;" : "+r"(d) : "r"(a), "r"(b));
}
__device__ __forceinline__ void madc_lo_cc(uint32_t& d, uint32_t a, uint32_t b) {
    asm volatile("madc.lo.cc.u32 %0, %1, %2, %0;" : "+r"(d) : "r"(a), "r"(b));
}
__device__ __forceinline__ void madc_hi_cc(uint32_t& d, uint32_t a, uint32_t b) {
    asm volatile("madc.hi.cc.u32 %0, %1, %2, %0;" : "+r"(d) : "r"(a), "r"(b));
}
__device__ __forceinline__ void add_cc(uint32_t& d, uint32_t a) {
    asm volatile("add.cc.u32 %0, %0, %1;" : "+r"(d) : "r"(a));
}
__device__ __forceinline__ void addc_cc(uint32_t& d, uint32_t a) {
    asm volatile("addc.cc.u32 %0, %0, %1;" : "+r"(d) : "r"(a));
}
__device__ __forceinline__ void addc(uint32_t& d, uint32_t a) {
    asm volatile("addc.u32 %0, %0, %1;" : "+r"(d) : "r"(a));
}
__device__ __forceinline__ void sub_cc(uint32_t& d, uint32_t a) {
    asm volatile("sub.cc.u32 %0, %0, %1;" : "+r"(d) : "r"(a));
}
__device__ __forceinline__ void subc_cc(uint32_t& d, uint32_t a) {
    asm volatile("subc.cc.u32 %0, %0, %1;" : "+r"(d) : "r"(a));
}
__device__ __forceinline__ void subc(uint32_t& d, uint32_t a) {
    asm volatile("subc.u32 %0, %0, %1;" : "+r"(d) : "r"(a));
}

// ---------------------------------------------------------------------------
// Carry resolution over a group of GS consecutive threads (GS a power of two).
//
// Each thread holds a chunk of a big number and knows its chunk's generate bit
// g (carry-out with carry-in 0) and propagate bit p (chunk is all ones, so a
// carry-in passes through).  The carry into every chunk is the carry-lookahead
// recurrence c[i+1] = g[i] | (p[i] & c[i]), which is exactly the carry of the
// integer sum x + y with x = g|p, y = g (bit i of x+y+c0 equals x^y^carry-in).
// One ballot per bit-plane and one 64-bit add resolve a whole warp; groups of
// more than 32 threads resolve per warp and then once more over the warps'
// aggregates.  This replaces the reference's Hillis-Steele scan of the
// CarrySegBop monoid over volatile shared memory (cuda/ker-addition.cu.h:
// 50-134), whose segment-start bit becomes the group boundary here.
//
// cin0: carry into the group's first chunk.  Returns the carry into this
// thread's chunk; *gcarry receives the carry out of the whole group.  For
// GS > 32 every thread of the block must call this (it synchronises the
// block) and `scratch` must hold (blockDim.x/32) words.
// ---------------------------------------------------------------------------
// Lanes of the calling thread's group of GS <= 32 lanes (all 32 for GS = 32).
template <int GS>
__device__ __forceinline__ uint32_t group_lanes() {
    static_assert(GS <= 32, "sub-warp groups only");
    if constexpr (GS == 32) {
        return MI_FULL_MASK;
    } else {
        const uint32_t lane = threadIdx.x & 31u;
        return ((1u << GS) - 1u) << (lane & ~uint32_t(GS - 1));
    }
}

// Barrier over the group: its own lanes for groups within a warp (so groups
// of one warp may run different loops), the whole block otherwise.
template <int GS>
__device__ __forceinline__ void group_sync() {
    if constexpr (GS <= 32)
        __syncwarp(group_lanes<GS>());
    else
        __syncthreads();
}

template <int GS>
__device__ __forceinline__ uint32_t group_carry(bool g, bool p, uint32_t cin0, uint32_t* gcarry,
                                                uint32_t* scratch) {
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t vote = MI_FULL_MASK;
    if constexpr (GS <= 32) vote = group_lanes<GS>();
    const uint32_t G = __ballot_sync(vote, g);
    const uint32_t P = __ballot_sync(vote, p);
    if constexpr (GS <= 32) {
        const uint32_t base = lane & ~uint32_t(GS - 1);
        const uint64_t mask = (GS == 32) ? 0xffffffffull : ((1ull << GS) - 1ull);
        const uint64_t x = (uint64_t((G | P) >> base)) & mask;
        const uint64_t y = (uint64_t(G >> base)) & mask;
        const uint64_t s = x + y + cin0;
        const uint64_t c = s ^ x ^ y;
        *gcarry = uint32_t(s >> GS) & 1u;
        return uint32_t(c >> (lane - base)) & 1u;
    } else {
        constexpr int W = GS / 32;
        static_assert(W <= 32, "group too large");
        const uint32_t warp = threadIdx.x >> 5;
        const uint32_t wig = warp & (W - 1);        // warp index within group
        const uint32_t gbase = warp & ~uint32_t(W - 1);
        const uint64_t x = uint64_t(G | P), y = uint64_t(G);
        const uint64_t s0 = x + y;
        if (lane == 0) scratch[warp] = uint32_t((s0 >> 32) & 1u) | ((P == MI_FULL_MASK) ? 2u : 0u);
        __syncthreads();
        const uint32_t f = (lane < (uint32_t)W) ? scratch[gbase + lane] : 0u;
        const uint32_t WG = __ballot_sync(MI_FULL_MASK, f & 1u);
        const uint32_t WP = __ballot_sync(MI_FULL_MASK, (f & 2u) != 0);
        const uint64_t X = uint64_t(WG | WP), Y = uint64_t(WG);
        const uint64_t S = X + Y + cin0;
        const uint64_t C = S ^ X ^ Y;
        *gcarry = uint32_t(S >> W) & 1u;
        const uint32_t cinw = uint32_t(C >> wig) & 1u;
        const uint64_t s1 = x + y + cinw;
        const uint64_t c1 = s1 ^ x ^ y;
        __syncthreads();
        return uint32_t(c1 >> lane) & 1u;
    }
}

// Adds the Q-limb chunks x + y into r with an internal carry chain and carry-in
// 0; returns generate (carry-out) and propagate (r is all ones).
template <typename L, int Q>
__device__ __forceinline__ void chunk_add(const L (&x)[Q], const L (&y)[Q], L (&r)[Q], bool& g, bool& p) {
    L c = 0;
    bool ones = true;
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        const L s = x[q] + y[q];
        const L c1 = s < x[q];
        const L s2 = s + c;
        const L c2 = s2 < s;
        r[q] = s2;
        c = c1 | c2;
        ones = ones && (s2 == ~L(0));
    }
    g = c != 0;
    p = ones;
}

// r += cin (0 or 1) with carry through the chunk; the carry out of the chunk
// is g | (p & cin), already known to the caller.
template <typename L, int Q>
__device__ __forceinline__ void chunk_inc(L (&r)[Q], uint32_t cin) {
    L c = L(cin);
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        r[q] += c;
        c = (r[q] < c) ? L(1) : L(0);
    }
}

}  // namespace mi
