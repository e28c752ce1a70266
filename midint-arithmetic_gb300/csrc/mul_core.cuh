// mul_core.cuh -- the square-product building block of the classical
// multiplication kernels (the plain batched kernel in mul.cu and the chunked
// rectangular products of the ragged kernels in ragged.cu).
//
// Counterpart of the reference's bmulRegsQ and its helpers computeIter64 /
// convolutionQ / combineQ / from4Reg2ShmQ (cuda/ker-classic-mul.cu.h:11-26,
// 299-463).  The reference walks output columns with a 128-bit accumulator and
// a carry counter, reading both operands from shared memory for every 64x64-bit
// product, and balances the low-half triangle by pairing column k with M-k.
//
// Here the grid of 32x32-bit partial products of two operands of NT*T limbs is
// cut into T x T tiles (T = 8).  Thread t of a group of NT threads owns the
// anti-diagonals of tiles s = t and s = t + NT, which together hold exactly NT
// tiles for every t (t+1 below the main anti-diagonal, NT-1-t above), so the
// full product is balanced without mirroring.  At step k every thread
// multiplies A-block k (the same address for the whole group: a broadcast) by
// B-block (t-k) mod NT, stored as two planes of 16-byte halves so that the
// group reads consecutive 16-byte slots (no bank conflicts).
//
// A tile is 2*T*T multiply-adds with the hardware carry flag.  Products with
// i+j even and with i+j odd go to two accumulators split by column parity, so
// every (lo, hi) word pair of a product lands on an even-aligned register pair
// (mad.lo.cc + madc.hi.cc on the same operands then issue as one wide
// multiply-add) and each tile row is two independent carry chains; the single
// carry-out of each chain goes into a per-column counter (one addc).  The
// first anti-diagonal is snapshotted to shared memory at the step where it
// completes (one predicated store sequence per step); the second is the final
// accumulator minus the snapshot.  Every output block of T limbs is then
// L_s + H_(s-1) + O_(s-2) (low, high and overflow words of the anti-diagonal
// values): each block's three-way sum hands its carry of 0..2 to the next
// block, and one carry-lookahead pass over the group (mi::group_carry)
// resolves the one-bit ripple that remains (combine_blocks) -- the
// reference's low/high/carry publish and baddRegs.
#pragma once

#include "common.cuh"

namespace mi {
namespace classic {

constexpr int T = 8;  // tile side, in 32-bit limbs

// Accumulator of one anti-diagonal, split by column parity:
//   a[c]  column c,   products with i+j even (chains start at even columns)
//   b[k]  column k+1, products with i+j odd
//   cc[c] carries out of the chains, at column T+c
struct DiagAcc {
    uint32_t a[2 * T];
    uint32_t b[2 * T - 2];
    uint32_t cc[T + 1];
    static constexpr int WORDS = 2 * T + 2 * T - 2 + T + 1;  // 39
};

constexpr int ACC = 2 * T + 1;  // words of a folded anti-diagonal value
// Shared memory per thread, in 64-bit pairs, laid out [pair][thread of the
// group] so that a thread's own pairs and its neighbours' pairs are read by
// consecutive threads at consecutive 8-byte slots (no bank conflicts).  Holds
// either the snapshot of a DiagAcc (8 + 7 + 5 pairs) or D1, D2 (2 x 17 words).
constexpr int PAIRS = 20;
constexpr int PER_T = 2 * PAIRS;  // words per thread (40)

__device__ __forceinline__ void tile_mac(const uint32_t (&A)[T], const uint32_t (&B)[T], DiagAcc& s) {
#pragma unroll
    for (int i = 0; i < T; ++i) {
        const int j0 = i & 1;  // first j with i+j even: columns i+j0 .. i+j0+T-1
        mad_lo_cc(s.a[i + j0], A[i], B[j0]);
        madc_hi_cc(s.a[i + j0 + 1], A[i], B[j0]);
#pragma unroll
        for (int j = j0 + 2; j < T; j += 2) {
            madc_lo_cc(s.a[i + j], A[i], B[j]);
            madc_hi_cc(s.a[i + j + 1], A[i], B[j]);
        }
        addc(s.cc[i + j0], 0u);
        const int j1 = 1 - j0;  // first j with i+j odd: columns i+j1 .. i+j1+T-1
        mad_lo_cc(s.b[i + j1 - 1], A[i], B[j1]);
        madc_hi_cc(s.b[i + j1], A[i], B[j1]);
#pragma unroll
        for (int j = j1 + 2; j < T; j += 2) {
            madc_lo_cc(s.b[i + j - 1], A[i], B[j]);
            madc_hi_cc(s.b[i + j], A[i], B[j]);
        }
        addc(s.cc[i + j1], 0u);
    }
}

// The (2T+1)-word value a + b*2^32 + cc*2^(32T) of an accumulator; the true
// value of an anti-diagonal of at most 2^31 tiles always fits.
__device__ __forceinline__ void fold(const uint32_t* a, const uint32_t* b, const uint32_t* cc, uint32_t (&f)[ACC]) {
#pragma unroll
    for (int c = 0; c < 2 * T; ++c) f[c] = a[c];
    f[2 * T] = 0;
    add_cc(f[1], b[0]);
#pragma unroll
    for (int k = 1; k < 2 * T - 2; ++k) addc_cc(f[k + 1], b[k]);
    addc_cc(f[2 * T - 1], 0u);
    addc(f[2 * T], 0u);
    add_cc(f[T], cc[0]);
#pragma unroll
    for (int c = 1; c < T; ++c) addc_cc(f[T + c], cc[c]);
    addc(f[2 * T], cc[T]);
}

// r = x + y (+ z when given) + o (o at word 0) as T words; returns the carry
// out, 0..2 (0..3 with z).
__device__ __forceinline__ uint32_t add3_block(const uint32_t (&x)[T], const uint32_t (&y)[T], uint32_t o,
                                               uint32_t (&r)[T], const uint32_t* z = nullptr) {
#pragma unroll
    for (int w = 0; w < T; ++w) r[w] = x[w];
    uint32_t k = 0;
    add_cc(r[0], y[0]);
#pragma unroll
    for (int w = 1; w < T; ++w) addc_cc(r[w], y[w]);
    addc(k, 0u);
    if (z != nullptr) {
        add_cc(r[0], z[0]);
#pragma unroll
        for (int w = 1; w < T; ++w) addc_cc(r[w], z[w]);
        addc(k, 0u);
    }
    add_cc(r[0], o);
#pragma unroll
    for (int w = 1; w < T; ++w) addc_cc(r[w], 0u);
    addc(k, 0u);
    return k;
}

// r += c (a word at word 0) with the carry through the block; returns the
// carry out (0 or 1).
__device__ __forceinline__ uint32_t add_word_block(uint32_t (&r)[T], uint32_t c) {
    uint32_t e = 0;
    add_cc(r[0], c);
#pragma unroll
    for (int w = 1; w < T; ++w) addc_cc(r[w], 0u);
    addc(e, 0u);
    return e;
}

__device__ __forceinline__ bool all_ones(const uint32_t (&r)[T]) {
    uint32_t a = r[0];
#pragma unroll
    for (int w = 1; w < T; ++w) a &= r[w];
    return a == MI_FULL_MASK;
}

// The group's 2NT output blocks in order, block q = t (lo) and q = NT + t
// (hi) of thread t, each L_q + H_(q-1) + O_(q-2), carried through; the carry
// out of the last block is dropped.  One pass: each block's three-way sum
// leaves a carry of 0..2, handed to the next block's thread (a shuffle within
// a warp; pair 18 of the shared slots, free by then, for wider groups) and
// added there; what remains is a one-bit ripple, resolved with one
// carry-lookahead pass per half.  `slots` is the group's pair array as in
// square_product (pair w of thread l at slots[w*NT*G + l]).  `alo`, when
// given, is one more T-word addend of the thread's lo block (the sum of the
// 2NT blocks must fit them: the carry out of the last block is dropped).
template <int NT, int G = 1>
__device__ __forceinline__ void combine_blocks(const uint32_t (&Llo)[T], const uint32_t (&Hlo)[T], uint32_t Olo,
                                               const uint32_t (&Lhi)[T], const uint32_t (&Hhi)[T], uint32_t Ohi,
                                               uint2* slots, uint32_t* scr, uint32_t t, uint32_t (&ulo)[T],
                                               uint32_t (&uhi)[T], const uint32_t* alo = nullptr) {
    const uint32_t clo = add3_block(Llo, Hlo, Olo, ulo, alo);
    const uint32_t chi = add3_block(Lhi, Hhi, Ohi, uhi);
    uint32_t in_lo, in_hi;  // carries of the preceding blocks (lane NT-1's lo block precedes lane 0's hi)
    if constexpr (NT <= 32) {
        const uint32_t mask = group_lanes<NT>();
        const uint32_t plo = __shfl_up_sync(mask, clo, 1, NT);
        const uint32_t phi = __shfl_up_sync(mask, chi, 1, NT);
        const uint32_t top = __shfl_sync(mask, clo, NT - 1, NT);
        in_lo = t ? plo : 0u;
        in_hi = t ? phi : top;
    } else {
        slots[18 * NT * G + t] = make_uint2(clo, chi);
        group_sync<NT>();
        const uint2 prev = slots[18 * NT * G + (t ? t - 1 : NT - 1)];
        in_lo = t ? prev.x : 0u;
        in_hi = t ? prev.y : prev.x;
    }
    const uint32_t elo = add_word_block(ulo, in_lo);
    const uint32_t ehi = add_word_block(uhi, in_hi);
    uint32_t c0, c1;
    const uint32_t rlo = group_carry<NT>(elo != 0, all_ones(ulo), 0u, &c0, scr);
    const uint32_t rhi = group_carry<NT>(ehi != 0, all_ones(uhi), c0, &c1, scr);
    add_word_block(ulo, rlo);
    add_word_block(uhi, rhi);
}

// 16-byte slot v of an operand row of n32 limbs, zero beyond n32 and for an
// invalid instance.  VEC: the row is 16-byte aligned and n32 % 4 == 0.
template <bool VEC>
__device__ __forceinline__ uint4 load_slot(const uint32_t* __restrict__ row, uint32_t v, uint32_t n32, bool valid) {
    uint4 q = make_uint4(0, 0, 0, 0);
    if (VEC && valid && v * 4 + 4 <= n32) {
        q = __ldcs(reinterpret_cast<const uint4*>(row) + v);
    } else if (valid) {
        const uint32_t w = v * 4;
        if (w + 0 < n32) q.x = __ldcs(row + w + 0);
        if (w + 1 < n32) q.y = __ldcs(row + w + 1);
        if (w + 2 < n32) q.z = __ldcs(row + w + 2);
        if (w + 3 < n32) q.w = __ldcs(row + w + 3);
    }
    return q;
}

// Thread t's slots t + i*NT (i < T/4) of both operand rows of its group, read
// into registers: every load of the group is in flight before any is used.
template <int NT, bool VEC>
__device__ __forceinline__ void fetch_ab(uint4 (&qa)[T / 4], uint4 (&qb)[T / 4], const uint32_t* __restrict__ ra,
                                         const uint32_t* __restrict__ rb, uint32_t n32, bool valid, uint32_t t) {
#pragma unroll
    for (int it = 0; it < T / 4; ++it) {
        qa[it] = load_slot<VEC>(ra, t + uint32_t(it) * NT, n32, valid);
        qb[it] = load_slot<VEC>(rb, t + uint32_t(it) * NT, n32, valid);
    }
}

// Writes fetch_ab's slots into the group's shared areas: A as blocks of T
// consecutive limbs, B in the two-plane layout (half h of block j at 16-byte
// slot h*NT + j), both zero padded to NT*T limbs.
template <int NT>
__device__ __forceinline__ void put_ab(uint32_t* gA, uint4* gB4, const uint4 (&qa)[T / 4], const uint4 (&qb)[T / 4],
                                       uint32_t t) {
#pragma unroll
    for (int it = 0; it < T / 4; ++it) {
        const uint32_t v = t + uint32_t(it) * NT;
        reinterpret_cast<uint4*>(gA)[v] = qa[it];
        gB4[(v & 1) * NT + (v >> 1)] = qb[it];
    }
}

// Stages both operand rows of a group.  All loads are issued before the first
// shared-memory store, so the group waits for one round trip to memory, not
// one per operand -- what counts over host-mapped rows: it took the zero-copy
// host step of the 8192-bit batch of 16384 products from 0.264 to 0.250 ms
// (that launch shape now has a loop of its own in k_mul, on the same two
// halves, fetch_ab and put_ab).
template <int NT, bool VEC>
__device__ __forceinline__ void stage_ab(uint32_t* gA, uint4* gB4, const uint32_t* __restrict__ ra,
                                         const uint32_t* __restrict__ rb, uint32_t n32, bool valid, uint32_t t) {
    uint4 qa[T / 4], qb[T / 4];
    fetch_ab<NT, VEC>(qa, qb, ra, rb, n32, valid, t);
    put_ab<NT>(gA, gB4, qa, qb, t);
}

// G > 1: G groups of a warp interleave their operands and slots so that the
// warp's accesses of one step fall on distinct banks: A-block k of group g at
// word (k*G + g)*T, B plane slot (h*G + g)*NT + j, pair w of lane l at
// w*NT*G + g*NT + l (gA, gB4 and slots point at group g's first element).
// The full product of the group's staged A (NT blocks) and B (NT blocks), of
// which only the first nb hold nonzero limbs (1 <= nb <= NT).  Steps k >= nb
// (A-block k zero for the whole group) are not run; anti-diagonal t is then
// complete after step min(t, nb-1).  On return thread t holds output blocks t (lo,
// limbs tT..tT+T-1) and t+NT (hi), fully carried.  `slots` is the group's PAIRS*NT 64-bit shared slots
// (pair w of thread l at slots[w*NT + l]), `scr` per-warp scratch for groups
// wider than a warp.  Starts and ends with the group's shared areas free for
// reuse by the caller after a group_sync.
// Tile-loop unroll: deep for the plain kernels' wide groups (more loads in
// flight per step), shallow where registers are short (small groups, the
// ragged kernel's interleaved groups).
//
// PREFETCH: the operands of steps k+1 and k+2 are read from shared memory
// into registers before the tile of step k is multiplied (32 more registers),
// so a warp's multiply-adds never wait for its own loads (two steps ahead
// against one: 0.1362 -> 0.1355 ms on the 8192-bit batch, 124 registers).
//
// alo: when given, T more words added to the thread's output block t (lo)
// in the same carry pass (the ragged products' pending window).
template <int NT, int G = 1, int UNROLL = (NT >= 16 && G == 1) ? 8 : 2, bool PREFETCH = false>
__device__ __forceinline__ void square_product(const uint32_t* gA, const uint4* gB4, uint2* slots, uint32_t* scr,
                                               uint32_t t, uint32_t (&ulo)[T], uint32_t (&uhi)[T],
                                               uint32_t nb = NT, const uint32_t* alo = nullptr) {
    auto slot = [&](int w, uint32_t lane) -> uint2& { return slots[w * NT * G + lane]; };
    DiagAcc s;
#pragma unroll
    for (int w = 0; w < 2 * T; ++w) s.a[w] = 0;
#pragma unroll
    for (int w = 0; w < 2 * T - 2; ++w) s.b[w] = 0;
#pragma unroll
    for (int w = 0; w < T + 1; ++w) s.cc[w] = 0;
    const uint32_t snap_k = t < nb ? t : nb - 1;
    uint4 na0, na1, nb0, nb1;  // step k+1's operands (PREFETCH)
    uint4 ma0, ma1, mb0, mb1;  // step k+2's (nb >= 2 whenever PREFETCH is used)
    if (PREFETCH) {
        na0 = reinterpret_cast<const uint4*>(gA)[0];
        na1 = reinterpret_cast<const uint4*>(gA)[1];
        nb0 = gB4[t & uint32_t(NT - 1)];
        nb1 = gB4[G * NT + (t & uint32_t(NT - 1))];
        if (nb > 1) {
            const uint32_t jn = (t - 1) & uint32_t(NT - 1);
            ma0 = reinterpret_cast<const uint4*>(gA + G * T)[0];
            ma1 = reinterpret_cast<const uint4*>(gA + G * T)[1];
            mb0 = gB4[jn];
            mb1 = gB4[G * NT + jn];
        }
    }
#pragma unroll UNROLL
    for (uint32_t k = 0; k < nb; ++k) {
        const uint32_t j = (t - k) & uint32_t(NT - 1);
        uint32_t A[T], B[T];
        uint4 a0, a1, b0, b1;
        if (PREFETCH) {
            a0 = na0, a1 = na1, b0 = nb0, b1 = nb1;
            na0 = ma0, na1 = ma1, nb0 = mb0, nb1 = mb1;
            if (k + 2 < nb) {
                const uint32_t jn = (t - k - 2) & uint32_t(NT - 1);
                ma0 = reinterpret_cast<const uint4*>(gA + (k + 2) * G * T)[0];
                ma1 = reinterpret_cast<const uint4*>(gA + (k + 2) * G * T)[1];
                mb0 = gB4[jn];
                mb1 = gB4[G * NT + jn];
            }
        } else {
            a0 = reinterpret_cast<const uint4*>(gA + k * G * T)[0];
            a1 = reinterpret_cast<const uint4*>(gA + k * G * T)[1];
            b0 = gB4[j];
            b1 = gB4[G * NT + j];
        }
        A[0] = a0.x; A[1] = a0.y; A[2] = a0.z; A[3] = a0.w;
        A[4] = a1.x; A[5] = a1.y; A[6] = a1.z; A[7] = a1.w;
        B[0] = b0.x; B[1] = b0.y; B[2] = b0.z; B[3] = b0.w;
        B[4] = b1.x; B[5] = b1.y; B[6] = b1.z; B[7] = b1.w;
        tile_mac(A, B, s);
        if (k == snap_k) {
            // anti-diagonal t is complete: snapshot the accumulator, straight
            // from its register pairs
#pragma unroll
            for (int w = 0; w < T; ++w) slot(w, t) = make_uint2(s.a[2 * w], s.a[2 * w + 1]);
#pragma unroll
            for (int w = 0; w < T - 1; ++w) slot(T + w, t) = make_uint2(s.b[2 * w], s.b[2 * w + 1]);
#pragma unroll
            for (int w = 0; w < T / 2; ++w) slot(2 * T - 1 + w, t) = make_uint2(s.cc[2 * w], s.cc[2 * w + 1]);
            slot(2 * T - 1 + T / 2, t) = make_uint2(s.cc[T], 0u);
        }
    }

    // split into the two anti-diagonal values D1 (s=t) and D2 (s=t+NT)
    uint32_t d1[ACC], d2[ACC];
    {
        uint32_t snap[2 * PAIRS];
#pragma unroll
        for (int w = 0; w < PAIRS; ++w) {
            const uint2 v = slot(w, t);
            snap[2 * w] = v.x;
            snap[2 * w + 1] = v.y;
        }
        fold(snap, snap + 2 * T, snap + 4 * T - 2, d1);
        fold(s.a, s.b, s.cc, d2);
        sub_cc(d2[0], d1[0]);
#pragma unroll
        for (int w = 1; w < ACC - 1; ++w) subc_cc(d2[w], d1[w]);
        subc(d2[ACC - 1], d1[ACC - 1]);
    }

    // output blocks s=t (lo) and s=t+NT (hi): L_s + H_(s-1) + O_(s-2).  The
    // high and overflow words come from thread t-1 (t-2): its D1 for the lo
    // block, its D2 for the hi block, where thread 0 (and 1 for O) wraps to
    // the D1 of threads NT-1 (NT-2)
    uint32_t Hlo[T], Hhi[T], Olo = 0, Ohi = 0;
    if constexpr (NT <= 32) {
        // within a warp: shuffles, each sender offering what its receiver needs
        const uint32_t mask = group_lanes<NT>();
        const uint32_t src1 = (t - 1) & uint32_t(NT - 1), src2 = (t - 2) & uint32_t(NT - 1);
#pragma unroll
        for (int w = 0; w < T; ++w) {
            const uint32_t a = __shfl_sync(mask, d1[T + w], src1, NT);
            const uint32_t b = __shfl_sync(mask, (t == NT - 1) ? d1[T + w] : d2[T + w], src1, NT);
            Hlo[w] = t >= 1 ? a : 0u;
            Hhi[w] = b;
        }
        const uint32_t o1 = __shfl_sync(mask, d1[2 * T], src2, NT);
        const uint32_t o2 = __shfl_sync(mask, (t + 2 >= NT) ? d1[2 * T] : d2[2 * T], src2, NT);
        Olo = t >= 2 ? o1 : 0u;
        if constexpr (NT >= 2) Ohi = o2;
    } else {
        // across warps: D1 words 0..16 in pairs 0..8, D2 words in pairs 9..17
#pragma unroll
        for (int w = 0; w < ACC / 2; ++w) {
            slot(w, t) = make_uint2(d1[2 * w], d1[2 * w + 1]);
            slot(9 + w, t) = make_uint2(d2[2 * w], d2[2 * w + 1]);
        }
        slot(ACC / 2, t) = make_uint2(d1[ACC - 1], 0u);
        slot(9 + ACC / 2, t) = make_uint2(d2[ACC - 1], 0u);
        group_sync<NT>();
        auto peer = [&](uint32_t lane, int which, int w) -> uint32_t {
            const uint2 v = slot(which * 9 + w / 2, lane);
            return (w & 1) ? v.y : v.x;
        };
#pragma unroll
        for (int w = 0; w < T; ++w) {
            Hlo[w] = (t >= 1) ? peer(t - 1, 0, T + w) : 0u;
            Hhi[w] = (t >= 1) ? peer(t - 1, 1, T + w) : peer(NT - 1, 0, T + w);
        }
        if (t >= 2) {
            Olo = peer(t - 2, 0, 2 * T);
            Ohi = peer(t - 2, 1, 2 * T);
        } else {
            Ohi = (t == 1) ? peer(NT - 1, 0, 2 * T) : peer(NT - 2, 0, 2 * T);
        }
    }
    uint32_t Llo[T], Lhi[T];
#pragma unroll
    for (int w = 0; w < T; ++w) {
        Llo[w] = d1[w];
        Lhi[w] = d2[w];
    }
    combine_blocks<NT, G>(Llo, Hlo, Olo, Lhi, Hhi, Ohi, slots, scr, t, ulo, uhi, alo);
}

// Stages `n32` limbs of an operand row in the two-plane layout of NB blocks
// (half h of block j at 16-byte slot h*NB + j), zero padded to NB*T limbs, by
// THREADS threads.
template <int NB, int THREADS, bool VEC>
__device__ __forceinline__ void stage_planes(uint4* g4, const uint32_t* __restrict__ row, uint32_t n32, bool valid,
                                             uint32_t t) {
#pragma unroll
    for (int it = 0; it < 2 * NB / THREADS; ++it) {
        const uint32_t v = t + uint32_t(it) * THREADS;
        uint4 q = make_uint4(0, 0, 0, 0);
        if (VEC && valid && v * 4 + 4 <= n32) {
            q = __ldcs(reinterpret_cast<const uint4*>(row) + v);
        } else if (valid) {
            const uint32_t w = v * 4;
            if (w + 0 < n32) q.x = __ldcs(row + w + 0);
            if (w + 1 < n32) q.y = __ldcs(row + w + 1);
            if (w + 2 < n32) q.z = __ldcs(row + w + 2);
            if (w + 3 < n32) q.w = __ldcs(row + w + 3);
        }
        g4[(v & 1) * NB + (v >> 1)] = q;
    }
}

// The low NB = 2*NH blocks of the product of A and B (NB blocks each, both in
// the two-plane layout), of which only the first nb hold nonzero limbs
// (1 <= nb <= NB).  Only the anti-diagonals s < nb reach the low nb blocks;
// with H = ceil(nb/2), thread t < H owns s = t (t+1 tiles) and its mirror
// s = nb-1-t (nb-t tiles): nb+1 tiles for every thread, the reference's
// column pairing (cuda/ker-classic-mul.cu.h:406-423) at tile granularity.  In
// the first t+1 steps thread t walks anti-diagonal t (A-block k broadcast,
// B-block t-k); then its mirror (A-block k-t-1, B-block nb-k broadcast).
// Threads without a mirror (t >= H, and t = (nb-1)/2 for odd nb) read the
// zero block nb instead, which exists whenever they do.  On return thread t
// holds output blocks t (ulo) and NH+t (uhi), fully carried; the carry out of
// block NB-1 is dropped (the product mod 2^(32*T*NB)).  PREFETCH: each step's
// operands are read one step ahead (16 more registers).
template <int NH, int UNROLL = NH >= 16 ? 8 : 2, bool PREFETCH = false>
__device__ __forceinline__ void low_product(const uint4* gA4, const uint4* gB4, uint2* slots, uint32_t* scr,
                                            uint32_t t, uint32_t (&ulo)[T], uint32_t (&uhi)[T],
                                            uint32_t nb = 2 * NH) {
    constexpr uint32_t NB = 2 * NH;
    auto slot = [&](int w, uint32_t lane) -> uint2& { return slots[w * NH + lane]; };
    DiagAcc s;
#pragma unroll
    for (int w = 0; w < 2 * T; ++w) s.a[w] = 0;
#pragma unroll
    for (int w = 0; w < 2 * T - 2; ++w) s.b[w] = 0;
#pragma unroll
    for (int w = 0; w < T + 1; ++w) s.cc[w] = 0;
    const uint32_t H = (nb + 1) / 2;
    const bool mirror = t < H && t < nb - 1 - t;  // owns a second anti-diagonal
    // the blocks of step k: A-block i, B-block j
    auto blocks = [&](uint32_t k, uint32_t& i, uint32_t& j) {
        const bool first = k <= t;
        i = first ? k : k - t - 1;
        j = first ? t - k : nb - k;
        if (first ? t >= H : !mirror) i = nb;  // a zero block
    };
    uint4 na0, na1, nb0, nb1;  // step k+1's operands (PREFETCH)
    if (PREFETCH) {
        uint32_t i, j;
        blocks(0, i, j);
        na0 = gA4[i], na1 = gA4[NB + i], nb0 = gB4[j], nb1 = gB4[NB + j];
    }
#pragma unroll UNROLL
    for (uint32_t k = 0; k <= nb; ++k) {
        uint32_t A[T], B[T];
        uint4 a0, a1, b0, b1;
        if (PREFETCH) {
            a0 = na0, a1 = na1, b0 = nb0, b1 = nb1;
            if (k < nb) {
                uint32_t i, j;
                blocks(k + 1, i, j);
                na0 = gA4[i], na1 = gA4[NB + i], nb0 = gB4[j], nb1 = gB4[NB + j];
            }
        } else {
            uint32_t i, j;
            blocks(k, i, j);
            a0 = gA4[i], a1 = gA4[NB + i], b0 = gB4[j], b1 = gB4[NB + j];
        }
        A[0] = a0.x; A[1] = a0.y; A[2] = a0.z; A[3] = a0.w;
        A[4] = a1.x; A[5] = a1.y; A[6] = a1.z; A[7] = a1.w;
        B[0] = b0.x; B[1] = b0.y; B[2] = b0.z; B[3] = b0.w;
        B[4] = b1.x; B[5] = b1.y; B[6] = b1.z; B[7] = b1.w;
        tile_mac(A, B, s);
        if (k == t) {
#pragma unroll
            for (int w = 0; w < T; ++w) slot(w, t) = make_uint2(s.a[2 * w], s.a[2 * w + 1]);
#pragma unroll
            for (int w = 0; w < T - 1; ++w) slot(T + w, t) = make_uint2(s.b[2 * w], s.b[2 * w + 1]);
#pragma unroll
            for (int w = 0; w < T / 2; ++w) slot(2 * T - 1 + w, t) = make_uint2(s.cc[2 * w], s.cc[2 * w + 1]);
            slot(2 * T - 1 + T / 2, t) = make_uint2(s.cc[T], 0u);
        }
    }

    // D1 = anti-diagonal t (the snapshot), D2 = anti-diagonal nb-1-t
    {
        uint32_t d1[ACC], d2[ACC];
        uint32_t snap[2 * PAIRS];
#pragma unroll
        for (int w = 0; w < PAIRS; ++w) {
            const uint2 v = slot(w, t);
            snap[2 * w] = v.x;
            snap[2 * w + 1] = v.y;
        }
        fold(snap, snap + 2 * T, snap + 4 * T - 2, d1);
        fold(s.a, s.b, s.cc, d2);
        sub_cc(d2[0], d1[0]);
#pragma unroll
        for (int w = 1; w < ACC - 1; ++w) subc_cc(d2[w], d1[w]);
        subc(d2[ACC - 1], d1[ACC - 1]);
#pragma unroll
        for (int w = 0; w < ACC / 2; ++w) {
            slot(w, t) = make_uint2(d1[2 * w], d1[2 * w + 1]);
            slot(9 + w, t) = make_uint2(d2[2 * w], d2[2 * w + 1]);
        }
        slot(ACC / 2, t) = make_uint2(d1[ACC - 1], 0u);
        slot(9 + ACC / 2, t) = make_uint2(d2[ACC - 1], 0u);
    }
    group_sync<NH>();

    // word w of anti-diagonal value D_s: thread s holds it as D1 for s < H,
    // thread nb-1-s as D2 for H <= s < nb; beyond nb it is not needed (zero)
    auto diag = [&](uint32_t sd, int w) -> uint32_t {
        if (sd >= nb) return 0u;
        const bool low = sd < H;
        const uint2 v = slot((low ? 0 : 9) + w / 2, low ? sd : nb - 1 - sd);
        return (w & 1) ? v.y : v.x;
    };
    // output block q: L_q + H_(q-1) + O_(q-2)
    uint32_t Llo[T], Lhi[T], Hlo[T], Hhi[T];
    const uint32_t qh = NH + t;
#pragma unroll
    for (int w = 0; w < T; ++w) {
        Llo[w] = diag(t, w);
        Lhi[w] = diag(qh, w);
        Hlo[w] = (t >= 1) ? diag(t - 1, T + w) : 0u;
        Hhi[w] = diag(qh - 1, T + w);
    }
    const uint32_t Olo = (t >= 2) ? diag(t - 2, 2 * T) : 0u;
    const uint32_t Ohi = (qh >= 2) ? diag(qh - 2, 2 * T) : 0u;
    combine_blocks<NH>(Llo, Hlo, Olo, Lhi, Hhi, Ohi, slots, scr, t, ulo, uhi);
}

// Stores the T limbs of `v` at limb o of a result row, clipped to rlen.
template <bool VEC>
__device__ __forceinline__ void store_block(uint32_t* rr, uint32_t o, uint32_t rlen, const uint32_t (&v)[T]) {
    if (VEC && o + T <= rlen) {
#pragma unroll
        for (int q = 0; q < T / 4; ++q)
            __stcs(reinterpret_cast<uint4*>(rr + o) + q, make_uint4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]));
    } else {
#pragma unroll
        for (int w = 0; w < T; ++w)
            if (o + w < rlen) __stcs(rr + o + w, v[w]);
    }
}

// The same for rows that are 8-byte aligned, with o and rlen even (u64 limbs
// seen as u32 pairs): one 8-byte store per pair of words.
__device__ __forceinline__ void store_pairs(uint32_t* rr, uint32_t o, uint32_t rlen, const uint32_t (&v)[T]) {
#pragma unroll
    for (int w = 0; w < T; w += 2)
        if (o + w < rlen) __stcs(reinterpret_cast<uint2*>(rr + o + w), make_uint2(v[w], v[w + 1]));
}

}  // namespace classic
}  // namespace mi
