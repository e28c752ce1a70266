// ntt_mul.cuh -- one exact NTT multiplication by a group of L/8 threads
// (shared by the batched kernel in ntt_mul.cu and the ragged kernels).
//
// Three digit modes, each on as many of the five primes p_i < 2^30 as its
// coefficients need (a coefficient of a product is a sum of at most
// min(na, nb) products of two digits, so it is below min(na, nb) * 2^(2d)
// for d-bit digits and CRT over primes whose product exceeds that recovers it
// exactly):
//  * DM64: every u64 limb is one digit, five primes (product 2^149.4 >
//    2048 * 2^128);
//  * DM48: 48-bit digits (three limbs make four digits), the first four
//    primes (2^119.6 > 2731 * 2^96);
//  * DM40: 40-bit digits (five limbs make eight digits), the first three
//    primes (2^89.7): exact while the shorter operand has at most 840 digits
//    (840 (2^40 - 1)^2 < p0 p1 p2), 525 u64 limbs.
// A product runs the mode with the fewest primes whose digits fit the same
// power-of-two length (DM40 when at most 5/8 of it is filled, DM48 at most
// 3/4): fewer primes, the same transforms per prime.  For each prime the
// group converts a and b into the field (a unscaled, b scaled by 2^32 / L:
// the Montgomery pointwise product takes out 2^32 and the inverse transform
// needs no 1/L pass),
// runs the two forward transforms in lockstep (shared twiddle loads and
// barriers), multiplies pointwise in registers and runs the inverse
// transform (ntt32.cuh), leaving the residues in shared memory.  It then
// recombines each coefficient with Garner's mixed-radix formula (Shoup
// products by constant inverses, then a Horner evaluation in 32-bit words),
// sums the coefficients of its 8 digits into its output limbs (8 limbs for
// 64-bit digits, 6 for 48-bit ones, 5 for 40-bit ones), passes the overflow
// words to its right neighbour and resolves the remaining one-bit carries
// with mi::group_carry -- the final carry that the reference does with
// splitFftReg + baddRegMul2Fft (cuda/ker-fft-help.cu.h:3-95).
#pragma once

#include "common.cuh"
#include "ntt32.cuh"
#include "ntt_host.h"

namespace mi {
namespace ntt32 {

// Shared memory of one group, in 32-bit words: exchange buffers of a and b
// (2 Plan::LX) + five residue arrays (5L).
template <int LG>
struct MulSmem {
    static constexpr int L = 1 << LG;
    static constexpr size_t WORDS32 = size_t(2) * Plan<LG>::LX + size_t(5) * L;
};

// x*K mod p in [0, 2p) for a digit x < 2^64: K0 = K mod p, K1 = 2^32 K mod p
// (Shoup pairs).
__device__ __forceinline__ uint32_t convert(uint64_t x, const Field& f, uint2 k0, uint2 k1) {
    return f.add(f.shoup(uint32_t(x), k0), f.shoup(uint32_t(x >> 32), k1));
}

// x mod p in [0, 2p) for a digit x = lo + hi 2^32 < 2^64, c32 the Shoup pair
// of 2^32 mod p: lo is brought below 2p by two conditional subtractions of 2p
// (lo < 2^32 < 6p), hi 2^32 by one Shoup product -- one product instead of
// the two of convert() for the operand that takes no scaling.
__device__ __forceinline__ uint32_t reduce_digit(uint32_t lo, uint32_t hi, const Field& f, uint2 c32) {
    return f.add(f.reduce2(f.reduce2(lo)), f.shoup(hi, c32));
}

// Digit modes (see the top of this file).
enum : int { DM64 = 0, DM48 = 1, DM40 = 2 };
template <int DM>
struct Digits {
    static constexpr int NP = 5 - DM;                              // primes
    static constexpr int BITS = DM == DM64 ? 64 : (DM == DM48 ? 48 : 40);
    static constexpr int OUT = BITS / 8;                           // output limbs per thread (8 digits)
    static constexpr int OVW = DM == DM64 ? 3 : (DM == DM48 ? 2 : 1);  // words overflowing to the next thread
};
// The largest digit count of the shorter operand for which 40-bit digits on
// three primes stay exact: 840 (2^40 - 1)^2 < p0 p1 p2 <= 841 (2^40 - 1)^2.
constexpr uint32_t kD40MaxDigits = 840;

// Digits of an operand of `limbs` u64 limbs in digit mode dm (0: 64-bit,
// 1: 48-bit, 2: 40-bit).
__host__ __device__ constexpr uint32_t ntt_digits(uint32_t limbs, int dm) {
    return dm == DM48 ? (4 * limbs + 2) / 3 : (dm == DM40 ? (8 * limbs + 4) / 5 : limbs);
}

// The digit mode of a product of la and lb limbs on an L-point transform
// with L = max(256, pow2ceil(la + lb)): the one with the fewest primes whose
// digits fit L (and, for 40-bit digits, the exactness bound).
__host__ __device__ constexpr int ntt_mode(uint32_t la, uint32_t lb, uint32_t L) {
    return (ntt_digits(la, DM40) + ntt_digits(lb, DM40) <= L &&
            (la < lb ? ntt_digits(la, DM40) : ntt_digits(lb, DM40)) <= kD40MaxDigits)
               ? DM40
               : (ntt_digits(la, DM48) + ntt_digits(lb, DM48) <= L ? DM48 : DM64);
}

// 48-bit digit i of a row of `words` u32 words (bits [48i, 48i + 48)) as
// its low 32 bits and its high 16; zero past the row.
__device__ __forceinline__ uint2 digit48(const uint32_t* __restrict__ row, uint32_t words, uint32_t i) {
    const uint32_t w = (3 * i) >> 1;  // word holding bit 48i (at bit 0 or 16 of it)
    const uint32_t w0 = w < words ? __ldg(row + w) : 0u;
    const uint32_t w1 = w + 1 < words ? __ldg(row + w + 1) : 0u;
    return (i & 1) ? make_uint2(__funnelshift_r(w0, w1, 16), w1 >> 16) : make_uint2(w0, w1 & 0xffffu);
}

// 40-bit digit i of a row of `words` u32 words (bits [40i, 40i + 40)) as its
// low 32 bits and its high 8; zero past the row.
__device__ __forceinline__ uint2 digit40(const uint32_t* __restrict__ row, uint32_t words, uint32_t i) {
    const uint32_t bit = 40 * i, w = bit >> 5, sh = bit & 31;  // sh in {0, 8, 16, 24}: two words hold it
    const uint32_t w0 = w < words ? __ldg(row + w) : 0u;
    const uint32_t w1 = w + 1 < words ? __ldg(row + w + 1) : 0u;
    return make_uint2(__funnelshift_r(w0, w1, sh), (w1 >> sh) & 0xffu);
}

// Digit i of an operand of `limbs` u64 limbs in digit mode DM, as (low 32
// bits, high bits).
template <int DM>
__device__ __forceinline__ uint2 digit_at(const uint64_t* __restrict__ row, uint32_t limbs, uint32_t i) {
    if constexpr (DM == DM48) return digit48(reinterpret_cast<const uint32_t*>(row), 2 * limbs, i);
    if constexpr (DM == DM40) return digit40(reinterpret_cast<const uint32_t*>(row), 2 * limbs, i);
    const uint64_t v = i < limbs ? __ldg(row + i) : 0ull;
    return make_uint2(uint32_t(v), uint32_t(v >> 32));
}

// s[w..) += (x0, x1, x2) (u64 words, little-endian), carries rippling to s[SW-1].
template <int SW>
__device__ __forceinline__ void add3_at(uint64_t (&s)[SW], int w, uint64_t x0, uint64_t x1, uint64_t x2) {
    unsigned __int128 a = (unsigned __int128)s[w] + x0;
    s[w] = (uint64_t)a;
    a = (unsigned __int128)s[w + 1] + x1 + (uint64_t)(a >> 64);
    s[w + 1] = (uint64_t)a;
    a = (unsigned __int128)s[w + 2] + x2 + (uint64_t)(a >> 64);
    s[w + 2] = (uint64_t)a;
#pragma unroll
    for (int k = w + 3; k < SW; ++k) {
        a = (unsigned __int128)s[k] + (uint64_t)(a >> 64);
        s[k] = (uint64_t)a;
    }
}

// The thread's block of OUT output limbs from its digit sums s (OUT + OVW
// words, the top OVW overflowing into the right neighbour), carried over the
// group, stored to rr[OUT t ..) below rlen.
template <int NT, int OUT, int OVW, int SW>
__device__ __forceinline__ void finish_block(const uint64_t (&s)[SW], uint64_t* ov, uint64_t* __restrict__ rr,
                                             uint32_t rlen, uint32_t t, uint32_t* scr) {
#pragma unroll
    for (int w = 0; w < OVW; ++w) ov[OVW * t + w] = s[OUT + w];
    __syncthreads();
    uint64_t add[OUT];
#pragma unroll
    for (int w = 0; w < OUT; ++w) add[w] = (w < OVW && t > 0) ? ov[OVW * (t - 1) + w] : 0ull;
    uint64_t lo[OUT], blk[OUT];
#pragma unroll
    for (int w = 0; w < OUT; ++w) lo[w] = s[w];
    bool g, p;
    chunk_add<uint64_t, OUT>(lo, add, blk, g, p);
    uint32_t gc;
    const uint32_t cin = group_carry<NT>(g, p, 0u, &gc, scr);
    chunk_inc<uint64_t, OUT>(blk, cin);
    const uint32_t o0 = OUT * t;
    if (rr != nullptr) {
        if (OUT % 2 == 0 && o0 + OUT <= rlen && (reinterpret_cast<uintptr_t>(rr + o0) & 15u) == 0) {
#pragma unroll
            for (int w = 0; w + 1 < OUT; w += 2)
                __stcs(reinterpret_cast<ulonglong2*>(rr + o0 + w), make_ulonglong2(blk[w], blk[w + 1]));
        } else {
#pragma unroll
            for (int w = 0; w < OUT; ++w)
                if (o0 + w < rlen) rr[o0 + w] = blk[w];
        }
    }
}

// r[0..rlen) = a*b for a of la limbs, b of lb limbs, with ntt_digits(la) +
// ntt_digits(lb) <= L in digit mode DM (and, for DM40, the shorter operand
// within kD40MaxDigits digits); every output limb, including the carry out of
// the top coefficient, falls inside the OUT*L/8 limbs the group produces;
// limbs beyond rlen are dropped.  `sm` is the group's MulSmem, `scr` per-warp
// scratch of the block.  Every thread of the block must call this with the
// same LG and DM (the exchanges synchronise the block).  HALF: both operands'
// digits lie below L/2 (balanced products: L = pow2ceil(2m)), so the upper
// half of each transform input is zero and is neither converted nor added
// (a compile-time choice: as a run-time flag in the ragged tasks it cost more
// than it saved).  LOW: only the low half of a balanced product is stored
// (rlen at most m limbs, all of them below digit L/2); the coefficients below
// L/2 alone determine those limbs, so only they are kept and recombined.
template <int LG, int DM, bool HALF = false, bool LOW = false>
__device__ __forceinline__ void mul_one(const uint64_t* __restrict__ ar, uint32_t la, const uint64_t* __restrict__ br,
                                        uint32_t lb, uint64_t* __restrict__ rr, uint32_t rlen, const NttMulParams& P,
                                        uint32_t* sm, uint32_t* scr) {
    using Pl = Plan<LG>;
    using Dg = Digits<DM>;
    constexpr int NP = Dg::NP;
    constexpr int SW = 11;  // digit-sum words: 8 limbs + 3 overflow, 6 + 2 or 5 + 1 (+ headroom)
    uint32_t* sh = sm;                // exchange buffers of a and b (2 LX)
    uint32_t* res = sm + 2 * Pl::LX;  // res[q][slot], q < NP
    const uint32_t t = threadIdx.x % Pl::NT;
#pragma unroll 1
    for (int q = 0; q < NP; ++q) {
        const Field f{P.p[q], 2 * P.p[q], P.pinv[q]};
        // a unscaled; b times 2^32 / L (the Montgomery pointwise product takes
        // out 2^32, and the inverse transform needs no 1/L pass)
        const uint2 c32 = P.kb[q][0];
        const uint2 kb0 = P.ka_by_lg[q][LG - 8][1], kb1 = P.kb_by_lg[q][LG - 8];
        uint32_t x[2][8];  // a and b, transformed in lockstep
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const uint32_t i = t + Pl::NT * j;
            if (HALF && j >= 4) {
                x[0][j] = x[1][j] = 0u;
                continue;
            }
            if constexpr (DM == DM64) {
                const uint64_t da = i < la ? __ldg(ar + i) : 0ull;
                x[0][j] = reduce_digit(uint32_t(da), uint32_t(da >> 32), f, c32);
                x[1][j] = (i < lb) ? convert(__ldg(br + i), f, kb0, kb1) : 0u;
            } else {
                const uint2 da = digit_at<DM>(ar, la, i);
                const uint2 db = digit_at<DM>(br, lb, i);
                x[0][j] = reduce_digit(da.x, da.y, f, c32);
                x[1][j] = f.add(f.shoup(db.x, kb0), f.shoup(db.y, kb1));
            }
        }
        forward<LG, 2, HALF>(x, sh, P.tw[q], f);
#pragma unroll
        for (int j = 0; j < 8; ++j) x[0][j] = f.mont(x[0][j], x[1][j]);
        inverse<LG>(x[0], sh, P.itw[q], f);
#pragma unroll
        for (int j = 0; j < (LOW ? 4 : 8); ++j) res[q * Pl::L + swz(t + Pl::NT * j)] = f.reduce(x[0][j]);
    }
    __syncthreads();

    // Garner: y0 = r0, y_i = (...((r_i - y0) c_0i - y1) c_1i ... - y_(i-1)) c_(i-1)i
    // mod p_i with c_ji = p_j^-1 mod p_i; x = y0 + p0 (y1 + p1 (y2 + ...)),
    // below the product of the NP primes (2^150, 2^120 or 2^90), evaluated in
    // 32-bit words (Horner).
    uint64_t s[SW];
#pragma unroll
    for (int w = 0; w < SW; ++w) s[w] = 0;
#pragma unroll
    for (int j = 0; j < 8; j += 4) {
        if (LOW && 8 * t >= Pl::L / 2) break;  // coefficients that reach no stored limb
        const uint32_t slot = swz(8 * t + j);  // the swizzle keeps the quad slot..slot+3 together
#pragma unroll
        for (int h = 0; h < 4; ++h) {
            uint32_t y[NP];
#pragma unroll
            for (int q = 0; q < NP; ++q) y[q] = res[q * Pl::L + slot + h];
            int c = 0;
#pragma unroll
            for (int i = 1; i < NP; ++i) {
                const Field fi{P.p[i], 2 * P.p[i], 0u};
                uint32_t v = y[i];
#pragma unroll
                for (int k = 0; k < i; ++k) v = fi.shoup(v + fi.p2 - y[k], P.garner[c++]);
                y[i] = fi.reduce(v);
            }
            // Horner in 32-bit words: acc = y_(NP-1); acc = acc * p_i + y_i, i = NP-2..0
            uint32_t acc[kPrimes] = {y[NP - 1], 0u, 0u, 0u, 0u};
#pragma unroll
            for (int i = NP - 2; i >= 0; --i) {
                uint64_t carry = y[i];
#pragma unroll
                for (int w = 0; w < NP - 1 - i; ++w) {
                    const uint64_t tt = uint64_t(acc[w]) * P.p[i] + carry;
                    acc[w] = uint32_t(tt);
                    carry = tt >> 32;
                }
                acc[NP - 1 - i] = uint32_t(carry);
            }
            const uint64_t w0 = uint64_t(acc[0]) | (uint64_t(acc[1]) << 32);
            const uint64_t w1 = uint64_t(acc[2]) | (uint64_t(acc[3]) << 32);
            const int o = j + h;  // the coefficient's digit within the thread's block of 8
            if constexpr (DM == DM64) {
                add3_at<SW>(s, o, w0, w1, uint64_t(acc[4]));
            } else {
                // a value below 2^120 (2^90) at bit BITS*o of the thread's block
                const int bit = Dg::BITS * o, w = bit >> 6, b = bit & 63;
                const uint64_t x0 = w0 << b;
                const uint64_t x1 = b ? (w1 << b) | (w0 >> (64 - b)) : w1;
                const uint64_t x2 = b ? w1 >> (64 - b) : 0ull;
                add3_at<SW>(s, w, x0, x1, x2);
            }
        }
    }
    // the overflow words go to the right neighbour through the exchange buffer
    uint64_t* ov = reinterpret_cast<uint64_t*>(sh);  // 3 x 8 bytes x L/8 threads: fits the 9L bytes of sh
    finish_block<Pl::NT, Dg::OUT, Dg::OVW>(s, ov, rr, rlen, t, scr);
    __syncthreads();  // sh and res are reused by the next call
}

}  // namespace ntt32
}  // namespace mi
