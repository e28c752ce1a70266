// ntt_mul.cuh -- one exact NTT multiplication by a group of L/8 threads
// (shared by the batched kernel in ntt_mul.cu and the ragged kernels).
//
// Two digit modes.  NP = 5: every u64 limb is one digit; the product of an
// la-limb and an lb-limb integer has coefficients below min(la, lb) * 2^128
// <= 2^139 (limbs <= 2048), so five primes p_i < 2^30 (product 2^149.4)
// recover every coefficient exactly by CRT.  NP = 4: 48-bit digits (three
// limbs make four digits), coefficients below min(na, nb) * 2^96 <= 2^107.4
// for up to 2731 digits, so the first four primes (product 2^119.6) suffice;
// a product whose 48-bit digits fit the same power-of-two length as its
// 64-bit ones (at most 3/4 of it filled) runs four transforms' worth of
// primes instead of five.  For each prime the group converts a and b into
// the field (a scaled by 1/L, so the inverse transform needs no scaling pass,
// and b by 2^32, which the Montgomery pointwise product takes out again),
// runs the two forward transforms in lockstep (shared twiddle loads and
// barriers), multiplies pointwise in registers and runs the inverse
// transform (ntt32.cuh), leaving the residues in shared memory.  It then
// recombines each coefficient with Garner's mixed-radix formula (Shoup
// products by constant inverses, then a Horner evaluation in 32-bit words),
// sums the coefficients of its 8 digits into its output limbs (8 limbs for
// 64-bit digits, 6 for 48-bit ones), passes the overflow words to its right
// neighbour and resolves the remaining one-bit carries with mi::group_carry
// -- the final carry that the reference does with splitFftReg +
// baddRegMul2Fft (cuda/ker-fft-help.cu.h:3-95).
#pragma once

#include "common.cuh"
#include "ntt32.cuh"
#include "ntt_host.h"

namespace mi {
namespace ntt32 {

// Shared memory of one group, in 32-bit words: exchange buffers of a and b
// (2L) + five residue arrays (5L).
template <int LG>
struct MulSmem {
    static constexpr int L = 1 << LG;
    static constexpr size_t WORDS32 = size_t(7) * L;
};

// x*K mod p in [0, 2p) for a digit x < 2^64: K0 = K mod p, K1 = 2^32 K mod p
// (Shoup pairs).
__device__ __forceinline__ uint32_t convert(uint64_t x, const Field& f, uint2 k0, uint2 k1) {
    return f.add(f.shoup(uint32_t(x), k0), f.shoup(uint32_t(x >> 32), k1));
}

// Digits of an operand of `limbs` u64 limbs: 64-bit ones, or with d48 48-bit ones.
__host__ __device__ constexpr uint32_t ntt_digits(uint32_t limbs, bool d48) {
    return d48 ? (4 * limbs + 2) / 3 : limbs;
}

// 48-bit digit i of a row of `words` u32 words (bits [48i, 48i + 48)) as
// its low 32 bits and its high 16; zero past the row.
__device__ __forceinline__ uint2 digit48(const uint32_t* __restrict__ row, uint32_t words, uint32_t i) {
    const uint32_t w = (3 * i) >> 1;  // word holding bit 48i (at bit 0 or 16 of it)
    const uint32_t w0 = w < words ? __ldg(row + w) : 0u;
    const uint32_t w1 = w + 1 < words ? __ldg(row + w + 1) : 0u;
    return (i & 1) ? make_uint2(__funnelshift_r(w0, w1, 16), w1 >> 16) : make_uint2(w0, w1 & 0xffffu);
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
        if (o0 + OUT <= rlen && (reinterpret_cast<uintptr_t>(rr + o0) & 15u) == 0) {
#pragma unroll
            for (int w = 0; w < OUT; w += 2)
                __stcs(reinterpret_cast<ulonglong2*>(rr + o0 + w), make_ulonglong2(blk[w], blk[w + 1]));
        } else {
#pragma unroll
            for (int w = 0; w < OUT; ++w)
                if (o0 + w < rlen) rr[o0 + w] = blk[w];
        }
    }
}

// r[0..rlen) = a*b for a of la limbs, b of lb limbs, with ntt_digits(la) +
// ntt_digits(lb) <= L in the chosen digit mode (D48: 48-bit digits on the
// first four primes, else 64-bit digits on five); every output limb,
// including the carry out of the top coefficient, falls inside the limbs the
// group produces (L with 64-bit digits, 3L/4 with 48-bit ones); limbs beyond
// rlen are dropped.  `sm` is the group's MulSmem, `scr` per-warp scratch of
// the block.  Every thread of the block must call this with the same LG and
// D48 (the exchanges synchronise the block).
template <int LG, bool D48>
__device__ __forceinline__ void mul_one(const uint64_t* __restrict__ ar, uint32_t la, const uint64_t* __restrict__ br,
                                        uint32_t lb, uint64_t* __restrict__ rr, uint32_t rlen, const NttMulParams& P,
                                        uint32_t* sm, uint32_t* scr) {
    using Pl = Plan<LG>;
    constexpr bool d48 = D48;
    constexpr int SW = 11;  // digit-sum words: 8 limbs + 3 overflow, or 6 + 2 (+ headroom)
    uint32_t* sh = sm;               // exchange buffers of a and b (2L)
    uint32_t* res = sm + 2 * Pl::L;  // res[q][slot], q < 5
    const uint32_t t = threadIdx.x % Pl::NT;
    const int np = d48 ? 4 : kPrimes;
#pragma unroll 1
    for (int q = 0; q < np; ++q) {
        const Field f{P.p[q], 2 * P.p[q], P.pinv[q]};
        const uint2 ka0 = P.ka_by_lg[q][LG - 8][0], ka1 = P.ka_by_lg[q][LG - 8][1];
        const uint2 kb0 = P.kb[q][0], kb1 = P.kb[q][1];
        uint32_t x[2][8];  // a and b, transformed in lockstep
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const uint32_t i = t + Pl::NT * j;
            if constexpr (d48) {
                const uint2 da = digit48(reinterpret_cast<const uint32_t*>(ar), 2 * la, i);
                const uint2 db = digit48(reinterpret_cast<const uint32_t*>(br), 2 * lb, i);
                x[0][j] = f.add(f.shoup(da.x, ka0), f.shoup(da.y, ka1));
                x[1][j] = f.add(f.shoup(db.x, kb0), f.shoup(db.y, kb1));
            } else {
                x[0][j] = (i < la) ? convert(__ldg(ar + i), f, ka0, ka1) : 0u;
                x[1][j] = (i < lb) ? convert(__ldg(br + i), f, kb0, kb1) : 0u;
            }
        }
        forward<LG, 2>(x, sh, P.tw[q], f);
#pragma unroll
        for (int j = 0; j < 8; ++j) x[0][j] = f.mont(x[0][j], x[1][j]);
        inverse<LG>(x[0], sh, P.itw[q], f);
#pragma unroll
        for (int j = 0; j < 8; ++j) res[q * Pl::L + swz(t + Pl::NT * j)] = f.reduce(x[0][j]);
    }
    __syncthreads();

    // Garner: y0 = r0, y_i = (...((r_i - y0) c_0i - y1) c_1i ... - y_(i-1)) c_(i-1)i
    // mod p_i with c_ji = p_j^-1 mod p_i; x = y0 + p0 (y1 + p1 (y2 + p2 (y3 +
    // p3 y4))) < 2^150, evaluated in 32-bit words.  With four primes y4 = 0
    // and the same evaluation gives y0 + p0 (y1 + p1 (y2 + p2 y3)) < 2^120.
    uint64_t s[SW];
#pragma unroll
    for (int w = 0; w < SW; ++w) s[w] = 0;
#pragma unroll
    for (int j = 0; j < 8; j += 4) {
        const uint32_t slot = swz(8 * t + j);  // the swizzle keeps the quad slot..slot+3 together
#pragma unroll
        for (int h = 0; h < 4; ++h) {
            uint32_t y[kPrimes];
#pragma unroll
            for (int q = 0; q < kPrimes; ++q) y[q] = (q < 4 || !d48) ? res[q * Pl::L + slot + h] : 0u;
            int c = 0;
#pragma unroll
            for (int i = 1; i < kPrimes; ++i) {
                if (d48 && i == kPrimes - 1) break;
                const Field fi{P.p[i], 2 * P.p[i], 0u};
                uint32_t v = y[i];
#pragma unroll
                for (int k = 0; k < i; ++k) v = fi.shoup(v + fi.p2 - y[k], P.garner[c++]);
                y[i] = fi.reduce(v);
            }
            if (d48) y[kPrimes - 1] = 0;
            // Horner in 32-bit words: acc = y4; acc = acc * p_i + y_i, i = 3..0
            uint32_t acc[kPrimes] = {y[kPrimes - 1], 0u, 0u, 0u, 0u};
#pragma unroll
            for (int i = kPrimes - 2; i >= 0; --i) {
                uint64_t carry = y[i];
#pragma unroll
                for (int w = 0; w < kPrimes - 1 - i; ++w) {
                    const uint64_t tt = uint64_t(acc[w]) * P.p[i] + carry;
                    acc[w] = uint32_t(tt);
                    carry = tt >> 32;
                }
                acc[kPrimes - 1 - i] = uint32_t(carry);
            }
            const uint64_t w0 = uint64_t(acc[0]) | (uint64_t(acc[1]) << 32);
            const uint64_t w1 = uint64_t(acc[2]) | (uint64_t(acc[3]) << 32);
            const int o = j + h;  // the coefficient's digit within the thread's block of 8
            if (!d48) {
                add3_at<SW>(s, o, w0, w1, uint64_t(acc[4]));
            } else {
                // a value below 2^120 at bit 48 o of the thread's block
                const int bit = 48 * o, w = bit >> 6, b = bit & 63;
                const uint64_t x0 = w0 << b;
                const uint64_t x1 = b ? (w1 << b) | (w0 >> (64 - b)) : w1;
                const uint64_t x2 = b ? w1 >> (64 - b) : 0ull;
                add3_at<SW>(s, w, x0, x1, x2);
            }
        }
    }
    // the overflow words go to the right neighbour through the exchange buffer
    uint64_t* ov = reinterpret_cast<uint64_t*>(sh);  // 3 x 8 bytes x L/8 threads: fits the 8L bytes of sh
    if (d48)
        finish_block<Pl::NT, 6, 2>(s, ov, rr, rlen, t, scr);
    else
        finish_block<Pl::NT, 8, 3>(s, ov, rr, rlen, t, scr);
    __syncthreads();  // sh and res are reused by the next call
}

}  // namespace ntt32
}  // namespace mi
