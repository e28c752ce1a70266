// add.cu -- batched big-integer addition by carry-lookahead over thread groups.
//
// Counterpart of the reference's baddKer / a6pb10Ker (cuda/ker-addition.cu.h:
// 227-328).  The reference stages each operand global -> shared -> registers
// with 8-byte loads (cpGlb2Reg, cuda/ker-helpers.cu.h:121-144) and resolves the
// carries with a Hillis-Steele scan over volatile shared memory plus four block
// barriers (cuda/ker-addition.cu.h:88-134).  Here every thread loads its Q
// limbs straight into registers with 128-bit streaming loads, and the carries
// of a whole warp are resolved by two ballots and one 64-bit add
// (mi::group_carry); only integers wider than one warp touch shared memory, one
// word per warp.
//
// Mapping: a group of GS threads (power of two) owns one instance, thread t of
// the group owns limbs [t*Q, t*Q+Q).  GS*Q >= limbs; limbs beyond the instance
// are zero and never stored.  A block of max(256, GS) threads holds 256/GS
// groups and strides over the batch.
#include <cstdio>

#include "common.cuh"
#include "kernels.h"

namespace mi {
namespace {

template <typename L>
struct Lim;
template <>
struct Lim<uint64_t> {
    using dev_t = unsigned long long;
};
template <>
struct Lim<uint32_t> {
    using dev_t = unsigned int;
};

// Streaming (evict-first) scalar load/store; every input limb is read once.
template <typename L>
__device__ __forceinline__ L ld_stream(const L* p) {
    using D = typename Lim<L>::dev_t;
    return (L)__ldcs(reinterpret_cast<const D*>(p));
}
template <typename L>
__device__ __forceinline__ void st_stream(L* p, L v) {
    using D = typename Lim<L>::dev_t;
    __stcs(reinterpret_cast<D*>(p), (D)v);
}

template <typename L, int Q>
__device__ __forceinline__ void unpack16(const uint4& t, L* v) {
    if constexpr (sizeof(L) == 8) {
        v[0] = (uint64_t(t.y) << 32) | t.x;
        v[1] = (uint64_t(t.w) << 32) | t.z;
    } else {
        v[0] = t.x;
        v[1] = t.y;
        v[2] = t.z;
        v[3] = t.w;
    }
}
template <typename L, int Q>
__device__ __forceinline__ uint4 pack16(const L* v) {
    uint4 t;
    if constexpr (sizeof(L) == 8) {
        t.x = uint32_t(v[0]);
        t.y = uint32_t(v[0] >> 32);
        t.z = uint32_t(v[1]);
        t.w = uint32_t(v[1] >> 32);
    } else {
        t.x = v[0];
        t.y = v[1];
        t.z = v[2];
        t.w = v[3];
    }
    return t;
}

// Loads the chunk [start, start+Q) of one instance row, zero beyond m.
template <typename L, int Q, bool VEC>
__device__ __forceinline__ void load_chunk(const L* __restrict__ row, uint32_t start, uint32_t m, bool valid,
                                           L (&v)[Q]) {
    constexpr int PER = 16 / sizeof(L);
    if constexpr (VEC) {
        if (valid && start + Q <= m) {
            const uint4* p = reinterpret_cast<const uint4*>(row + start);
#pragma unroll
            for (int k = 0; k < Q / PER; ++k) {
                const uint4 t = __ldcs(p + k);
                unpack16<L, Q>(t, &v[k * PER]);
            }
            return;
        }
    }
#pragma unroll
    for (int q = 0; q < Q; ++q) v[q] = (valid && start + q < m) ? ld_stream(row + start + q) : L(0);
}

template <typename L, int Q, bool VEC>
__device__ __forceinline__ void store_chunk(L* __restrict__ row, uint32_t start, uint32_t m, bool valid,
                                            const L (&v)[Q]) {
    constexpr int PER = 16 / sizeof(L);
    if (!valid) return;
    if constexpr (VEC) {
        if (start + Q <= m) {
            uint4* p = reinterpret_cast<uint4*>(row + start);
#pragma unroll
            for (int k = 0; k < Q / PER; ++k) __stcs(p + k, pack16<L, Q>(&v[k * PER]));
            return;
        }
    }
#pragma unroll
    for (int q = 0; q < Q; ++q)
        if (start + q < m) st_stream(row + start + q, v[q]);
}

// x + y over the group, result in r; returns the group's carry-out.
template <typename L, int Q, int GS>
__device__ __forceinline__ uint32_t group_add(const L (&x)[Q], const L (&y)[Q], L (&r)[Q], uint32_t* scratch) {
    bool g, p;
    chunk_add<L, Q>(x, y, r, g, p);
    uint32_t gc;
    const uint32_t cin = group_carry<GS>(g, p, 0u, &gc, scratch);
    chunk_inc<L, Q>(r, cin);
    return gc;
}

// The value v of thread t-1 of the group (0 for t == 0).  Groups wider than a
// warp pass the last lane's value through one shared word per warp.
template <int GS>
__device__ __forceinline__ uint64_t group_shift_up(uint64_t v, uint32_t t, uint64_t* xs) {
    if constexpr (GS <= 32) {
        const uint64_t u = __shfl_up_sync(group_lanes<GS>(), v, 1, GS);
        return t == 0 ? 0ull : u;
    } else {
        const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
        const uint64_t u = __shfl_up_sync(MI_FULL_MASK, v, 1);
        if (lane == 31) xs[warp] = v;
        __syncthreads();
        const uint64_t w = (lane == 0) ? ((t == 0) ? 0ull : xs[warp - 1]) : u;
        __syncthreads();
        return w;
    }
}

template <typename L, int Q, int GS, bool VEC, int OP>
__global__ void __launch_bounds__(GS > 256 ? GS : 256)
    k_add(const L* __restrict__ a, const L* __restrict__ b, L* __restrict__ r, uint8_t* __restrict__ carry,
          uint32_t n, uint32_t m) {
    constexpr int BLOCK = GS > 256 ? GS : 256;
    constexpr int IPB = BLOCK / GS;
    __shared__ uint32_t scratch[BLOCK / 32];
    __shared__ uint64_t shift[OP == ADD_PLAIN ? 1 : BLOCK / 32];
    const uint32_t grp = threadIdx.x / GS;
    const uint32_t t = threadIdx.x % GS;
    const uint32_t start = t * Q;
    const uint64_t stride = uint64_t(gridDim.x) * IPB;
    pdl_wait();  // launched with launch_pdl
    pdl_trigger();
    // Uniform trip count per block: group_carry synchronises the block for GS > 32.
    for (uint64_t base = uint64_t(blockIdx.x) * IPB; base < n; base += stride) {
        const uint64_t inst = base + grp;
        const bool valid = inst < n;
        const uint64_t off = valid ? inst * m : 0;
        L x[Q], y[Q], s[Q];
        load_chunk<L, Q, VEC>(a + off, start, m, valid, x);
        load_chunk<L, Q, VEC>(b + off, start, m, valid, y);
        uint32_t gc;
        if constexpr (OP == ADD_PLAIN) {
            gc = group_add<L, Q, GS>(x, y, s, scratch);
        } else {
            // 6a + 10b mod 2^(64m), the value of a6pb10Ker's chain of six
            // additions (cuda/ker-addition.cu.h:304-324) with one carry pass:
            // per limb 6a_i + 10b_i = lo_i + hi_i*2^64 with hi_i <= 15, and
            // the result is lo + (hi shifted up one limb), whose limb sums
            // carry at most 1.
            static_assert(sizeof(L) == 8, "6a + 10b is defined on u64 limbs");
            L lo[Q], hi[Q];
#pragma unroll
            for (int q = 0; q < Q; ++q) {
                const L pa = x[q] * 6u, pb = y[q] * 10u;
                lo[q] = pa + pb;
                hi[q] = __umul64hi(x[q], 6u) + __umul64hi(y[q], 10u) + L(lo[q] < pa);
            }
            L sh[Q];
            sh[0] = group_shift_up<GS>(hi[Q - 1], t, shift);
#pragma unroll
            for (int q = 1; q < Q; ++q) sh[q] = hi[q - 1];
            gc = group_add<L, Q, GS>(lo, sh, s, scratch);
        }
        store_chunk<L, Q, VEC>(r + off, start, m, valid, s);
        if (OP == ADD_PLAIN && carry != nullptr && valid) {
            // The carry-out is the value left at limb position m (a padding
            // limb of zeros plus the carry), or the group's carry-out when the
            // instance fills the group exactly.
            if (m < uint32_t(GS * Q)) {
#pragma unroll
                for (int q = 0; q < Q; ++q)
                    if (start + q == m) carry[inst] = uint8_t(s[q]);
            } else if (t == GS - 1) {
                carry[inst] = uint8_t(gc);
            }
        }
    }
}

// --- instances wider than one block: decoupled look-back -------------------
//
// A tile is one 256-thread block over 64 bytes of each operand per thread
// (2048 u64 limbs).  Tiles take their index from an atomic counter in launch
// order, so every tile a tile waits for has already started and will finish
// (no dependence on the scheduler).  A plain addition first reads the 32 limbs
// below its tile: the nearest one whose sum is not all ones gives the
// carry-in directly, which settles almost every tile of random data without
// waiting (the tile then only publishes its inclusive status).  Otherwise, and
// for 6a + 10b, each tile adds its limbs with carry-in 0,
// publishes its status word -- inclusive (its true carry-out) when it does not
// propagate a carry or is the first tile of its instance, otherwise an
// aggregate that says "passes the carry-in through" -- then it walks back
// over aggregates to the nearest inclusive status, bounded by spin_limit polls
// of an unpublished word (then the error word is set and the tile carries on
// with carry-in 0, so the kernel always completes), publishes its own
// inclusive status, and the block redoes the carry pass with that carry-in.
// The walk back is done by a warp, 32 predecessors per step.
// Status word: bits 0-1 state (1 aggregate, 2 inclusive), bit 2 carry value,
// bits 3-31 the launch's epoch (a word of another epoch is unpublished).

constexpr uint32_t ST_AGG = 1u, ST_INC = 2u;

__device__ __forceinline__ void st_release(uint32_t* p, uint32_t v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ uint32_t ld_acquire(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

template <typename L, bool VEC, int OP>
__global__ void __launch_bounds__(256)
    k_add_wide(const L* __restrict__ a, const L* __restrict__ b, L* __restrict__ r, uint8_t* __restrict__ carry,
               uint32_t m, uint32_t tiles_per, uint32_t n_tiles, uint32_t* status, uint32_t spin_limit,
               uint32_t withhold, uint64_t base, uint32_t epoch) {
    constexpr int Q = 64 / int(sizeof(L));
    constexpr uint32_t W = 256u * Q;  // limbs per tile
    __shared__ uint32_t scratch[8];
    __shared__ uint64_t shift[8];
    __shared__ uint32_t s_tile, s_cin;
    // a monotonic tile counter (this launch's tiles are base .. base+n_tiles-1)
    // and tile words tagged with the launch's epoch: nothing is cleared
    // between launches; a word of an older epoch reads as unpublished
    unsigned long long* counter = reinterpret_cast<unsigned long long*>(status + kWideTiles);
    uint32_t* err = status + kWideTiles + 2;
    pdl_wait();  // launched with launch_pdl: the previous launch has completed
    if (threadIdx.x == 0) s_tile = uint32_t(atomicAdd(counter, 1ull) - base);
    __syncthreads();
    const uint32_t tile = s_tile;
    if (tile >= n_tiles) return;  // (the grid has exactly n_tiles blocks)
    const uint32_t inst = tile / tiles_per, j = tile % tiles_per;
    const uint32_t t = threadIdx.x;
    const uint64_t off = uint64_t(inst) * m;
    const uint32_t start = j * W + t * Q;
    L x[Q], y[Q], s[Q];
    load_chunk<L, Q, VEC>(a + off, start, m, true, x);
    load_chunk<L, Q, VEC>(b + off, start, m, true, y);
    // Carry-in straight from the 32 limbs below the tile: the nearest limb
    // whose sum is not all ones decides it (generate: 1, kill: 0).  Random
    // limbs almost always settle it here and the tile never waits; only a
    // run of 32 all-ones sums falls back to the look-back.
    uint32_t local_cin = 0;
    bool local_ok = j == 0;
    if (OP == ADD_PLAIN && j > 0 && t < 32) {
        const uint64_t i = uint64_t(j) * W - 1 - t;  // lane 0 is the limb just below the tile
        const L ai = a[off + i], bi = b[off + i];
        const L si = ai + bi;
        const uint32_t settled = __ballot_sync(MI_FULL_MASK, si != L(~L(0)));
        const uint32_t gen = __ballot_sync(MI_FULL_MASK, si < ai);
        if (settled) {
            local_ok = true;
            local_cin = (gen >> (__ffs(settled) - 1)) & 1u;
        }
    }
    if constexpr (OP == ADD_SIX) {
        // 6a + 10b as lo + (hi shifted up one limb), as in k_add; thread 0
        // recomputes the high word of the limb before its tile
        static_assert(sizeof(L) == 8, "6a + 10b is defined on u64 limbs");
        L hi[Q];
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            const L pa = x[q] * 6u, pb = y[q] * 10u;
            const L lo = pa + pb;
            hi[q] = __umul64hi(x[q], 6u) + __umul64hi(y[q], 10u) + L(lo < pa);
            x[q] = lo;
        }
        uint64_t prev = group_shift_up<256>(hi[Q - 1], t, shift);
        if (t == 0 && j > 0) {
            const L xp = a[off + j * W - 1], yp = b[off + j * W - 1];
            const L pa = xp * 6u, pb = yp * 10u;
            prev = __umul64hi(xp, 6u) + __umul64hi(yp, 10u) + L(pa + pb < pa);
        }
        y[0] = prev;
#pragma unroll
        for (int q = 1; q < Q; ++q) y[q] = hi[q - 1];
    }
    bool g, p;
    chunk_add<L, Q>(x, y, s, g, p);
    uint32_t gc0;
    (void)group_carry<256>(g, p, 0u, &gc0, scratch);
    const bool P = __syncthreads_and(p) != 0;  // the tile passes a carry-in through
    if (t < 32) {
        // warp 0 looks back 32 tiles at a time: lane l reads tile k - l; the
        // carry-in is the value of the nearest inclusive tile, valid once
        // every tile between (all propagating aggregates) has published
        uint32_t cin = local_cin;
        if (!local_ok) {
            if (t == 0) st_release(status + tile, (epoch << 3) | (P ? ST_AGG : (ST_INC | (gc0 << 2))));
            const int32_t first = int32_t(tile - j);  // the instance's first tile: always inclusive
            int32_t k = int32_t(tile) - 1;
            uint32_t spins = 0;
            for (;;) {
                const int32_t i = k - int32_t(t);
                const uint32_t raw = i >= first ? ld_acquire(status + i) : ((epoch << 3) | ST_INC);
                const uint32_t sv = (raw >> 3) == epoch ? (raw & 7u) : 0u;
                const uint32_t inc = __ballot_sync(MI_FULL_MASK, (sv & 3u) == ST_INC);
                const uint32_t pending = __ballot_sync(MI_FULL_MASK, (sv & 3u) == 0u);
                const uint32_t nearest = inc ? uint32_t(__ffs(inc) - 1) : 32u;
                const uint32_t nearer = nearest == 32u ? MI_FULL_MASK : ((1u << nearest) - 1u);
                if (pending & nearer) {
                    if (++spins > spin_limit) {
                        if (t == 0) atomicOr(err, 1u);
                        break;
                    }
                    __nanosleep(64);
                    continue;
                }
                if (inc) {
                    cin = (__shfl_sync(MI_FULL_MASK, sv, int(nearest)) >> 2) & 1u;
                    break;
                }
                k -= 32;
            }
        }
        if (t == 0) {
            if (!(withhold && j == 0))
                st_release(status + tile, (epoch << 3) | ST_INC | ((gc0 | (P ? cin : 0u)) << 2));
            s_cin = cin;
        }
    }
    __syncthreads();
    uint32_t gc;
    const uint32_t c = group_carry<256>(g, p, s_cin, &gc, scratch);
    chunk_inc<L, Q>(s, c);
    store_chunk<L, Q, VEC>(r + off, start, m, true, s);
    if (OP == ADD_PLAIN && carry != nullptr && j == tiles_per - 1) {
        // carry-out: the value at limb m (zero padding plus the carry), or
        // the tile's carry-out when the instance ends with the tile
        if (m % W != 0) {
#pragma unroll
            for (int q = 0; q < Q; ++q)
                if (start + q == m) carry[inst] = uint8_t(s[q]);
        } else if (t == 255) {
            carry[inst] = uint8_t(gc);
        }
    }
}

// Rounds of whole instances, at most kWideTiles tiles each; every round is a
// new epoch of the tile words and takes the next n_tiles values of the tile
// counter, so nothing is cleared between launches (the words are cleared
// only when the 29-bit epoch wraps).
template <typename L, bool VEC, int OP>
mi_status launch_wide(const L* a, const L* b, L* r, uint8_t* carry, uint32_t n, uint32_t m, WideState& w,
                      cudaStream_t st) {
    constexpr uint32_t W = 256u * (64 / uint32_t(sizeof(L)));
    const uint32_t tiles_per = (m + W - 1) / W;
    const uint32_t cap = w.round_tiles < kWideTiles ? w.round_tiles : kWideTiles;
    if (tiles_per > cap) return set_error(MI_EINVAL, "add: %u limbs exceeds the multi-block maximum", m);
    const uint32_t per_round = cap / tiles_per;
    for (uint32_t i0 = 0; i0 < n; i0 += per_round) {
        const uint32_t k = (n - i0) < per_round ? (n - i0) : per_round;
        const uint32_t n_tiles = k * tiles_per;
        if (w.epoch >= (1u << 29) - 1) {  // the epoch field wraps: start over from cleared words
            MI_CUDA_TRY(cudaMemsetAsync(w.status, 0, size_t(kWideTiles) * 4, st));
            w.epoch = 0;
        }
        ++w.epoch;
        const uint64_t o = uint64_t(i0) * m;
        MI_CUDA_TRY(launch_pdl(k_add_wide<L, VEC, OP>, dim3(n_tiles), dim3(256), 0, st, a + o, b + o, r + o,
                               carry ? carry + i0 : nullptr, m, tiles_per, n_tiles, w.status, w.spin_limit,
                               w.withhold, w.issued, w.epoch));
        w.issued += n_tiles;  // every block of the launch takes one counter value
    }
    return MI_OK;
}

template <typename L, int Q, int GS, bool VEC, int OP>
mi_status launch_one(const L* a, const L* b, L* r, uint8_t* carry, uint32_t n, uint32_t m, cudaStream_t st) {
    constexpr int BLOCK = GS > 256 ? GS : 256;
    constexpr int IPB = BLOCK / GS;
    uint64_t blocks = (uint64_t(n) + IPB - 1) / IPB;
    // Enough blocks for full residency several times over; the kernel strides.
    const uint64_t cap = uint64_t(sm_count()) * 64;
    if (blocks > cap) blocks = cap;
    MI_CUDA_TRY(launch_pdl(k_add<L, Q, GS, VEC, OP>, dim3(uint32_t(blocks)), dim3(BLOCK), 0, st, a, b, r, carry, n, m));
    return MI_OK;
}

template <typename L, bool VEC, int OP, int Q>
mi_status dispatch_gs(const L* a, const L* b, L* r, uint8_t* carry, uint32_t n, uint32_t m, uint32_t gs,
                      cudaStream_t st) {
    switch (gs) {
        case 1: return launch_one<L, Q, 1, VEC, OP>(a, b, r, carry, n, m, st);
        case 2: return launch_one<L, Q, 2, VEC, OP>(a, b, r, carry, n, m, st);
        case 4: return launch_one<L, Q, 4, VEC, OP>(a, b, r, carry, n, m, st);
        case 8: return launch_one<L, Q, 8, VEC, OP>(a, b, r, carry, n, m, st);
        case 16: return launch_one<L, Q, 16, VEC, OP>(a, b, r, carry, n, m, st);
        case 32: return launch_one<L, Q, 32, VEC, OP>(a, b, r, carry, n, m, st);
        case 64: return launch_one<L, Q, 64, VEC, OP>(a, b, r, carry, n, m, st);
        case 128: return launch_one<L, Q, 128, VEC, OP>(a, b, r, carry, n, m, st);
        case 256: return launch_one<L, Q, 256, VEC, OP>(a, b, r, carry, n, m, st);
        case 512: return launch_one<L, Q, 512, VEC, OP>(a, b, r, carry, n, m, st);
        case 1024: return launch_one<L, Q, 1024, VEC, OP>(a, b, r, carry, n, m, st);
        default: return set_error(MI_EINVAL, "add: %u limbs exceeds the single-group maximum", m);
    }
}

// Q = thread_bytes / sizeof(L) limbs per thread (16, 32 or 64 bytes, raised
// until the group fits 1024 threads), GS = pow2ceil(m / Q) threads per
// instance.  VEC needs 16-byte aligned rows.
template <typename L, bool VEC, int OP>
mi_status dispatch(const L* a, const L* b, L* r, uint8_t* carry, uint32_t n, uint32_t m, uint32_t thread_bytes,
                   cudaStream_t st) {
    constexpr uint32_t QS = 16 / sizeof(L);  // limbs per 128-bit access
    uint32_t q = thread_bytes >= 64 ? 4 * QS : (thread_bytes >= 32 ? 2 * QS : QS);
    while (q < 4 * QS && pow2ceil((m + q - 1) / q) > 1024) q *= 2;
    const uint32_t gs = pow2ceil((m + q - 1) / q);
    if (q == QS) return dispatch_gs<L, VEC, OP, QS>(a, b, r, carry, n, m, gs, st);
    if (q == 2 * QS) return dispatch_gs<L, VEC, OP, 2 * QS>(a, b, r, carry, n, m, gs, st);
    return dispatch_gs<L, VEC, OP, 4 * QS>(a, b, r, carry, n, m, gs, st);
}

}  // namespace

uint32_t add_size_class(uint64_t bytes) {
    const uint64_t limbs = (bytes + 7) / 8;
    uint32_t c = 0;
    while (c < 12 && (uint64_t(1) << c) < limbs) ++c;
    return c;
}

mi_status launch_add_u64(const uint64_t* a, const uint64_t* b, uint64_t* r, uint8_t* carry, uint32_t n,
                         uint32_t limbs, int op, uint32_t thread_bytes, cudaStream_t st, WideState* wide) {
    const bool vec = aligned16(a) && aligned16(b) && aligned16(r) && (limbs % 2 == 0);
    if (limbs > kAddMaxLimbs64) {
        if (wide == nullptr || wide->status == nullptr) return set_error(MI_EINVAL, "add: no multi-block state");
        if (op == ADD_SIX)
            return vec ? launch_wide<uint64_t, true, ADD_SIX>(a, b, r, nullptr, n, limbs, *wide, st)
                       : launch_wide<uint64_t, false, ADD_SIX>(a, b, r, nullptr, n, limbs, *wide, st);
        return vec ? launch_wide<uint64_t, true, ADD_PLAIN>(a, b, r, carry, n, limbs, *wide, st)
                   : launch_wide<uint64_t, false, ADD_PLAIN>(a, b, r, carry, n, limbs, *wide, st);
    }
    if (op == ADD_SIX) {
        return vec ? dispatch<uint64_t, true, ADD_SIX>(a, b, r, nullptr, n, limbs, thread_bytes, st)
                   : dispatch<uint64_t, false, ADD_SIX>(a, b, r, nullptr, n, limbs, thread_bytes, st);
    }
    return vec ? dispatch<uint64_t, true, ADD_PLAIN>(a, b, r, carry, n, limbs, thread_bytes, st)
               : dispatch<uint64_t, false, ADD_PLAIN>(a, b, r, carry, n, limbs, thread_bytes, st);
}

mi_status launch_add_u32(const uint32_t* a, const uint32_t* b, uint32_t* r, uint8_t* carry, uint32_t n,
                         uint32_t limbs, uint32_t thread_bytes, cudaStream_t st, WideState* wide) {
    // An even number of u32 limbs on 8-byte aligned rows is the same bytes as
    // half as many u64 limbs, with the same carry-out.
    if (limbs % 2 == 0 && aligned8(a) && aligned8(b) && aligned8(r))
        return launch_add_u64(reinterpret_cast<const uint64_t*>(a), reinterpret_cast<const uint64_t*>(b),
                              reinterpret_cast<uint64_t*>(r), carry, n, limbs / 2, ADD_PLAIN, thread_bytes, st,
                              wide);
    if (limbs > 2 * kAddMaxLimbs64) {
        if (wide == nullptr || wide->status == nullptr) return set_error(MI_EINVAL, "add: no multi-block state");
        return launch_wide<uint32_t, false, ADD_PLAIN>(a, b, r, carry, n, limbs, *wide, st);
    }
    // Odd limb counts (or 4-byte aligned rows) cannot use 128-bit accesses.
    return dispatch<uint32_t, false, ADD_PLAIN>(a, b, r, carry, n, limbs, thread_bytes, st);
}

}  // namespace mi
