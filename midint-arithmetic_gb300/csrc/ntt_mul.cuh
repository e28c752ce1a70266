// ntt_mul.cuh -- one exact NTT multiplication by a group of L/8 threads
// (shared by the batched kernel in ntt_mul.cu and the ragged kernels).
//
// Every u64 limb is one digit; the product of an la-limb and an lb-limb
// integer has coefficients below min(la, lb) * 2^128 <= 2^139 (limbs <= 2048),
// so five primes p_i < 2^30 (product 2^149.4) recover every coefficient
// exactly by CRT.  For each prime the group converts a and b into the field
// (a scaled by 1/L, so the inverse transform needs no scaling pass, and b by
// 2^32, which the Montgomery pointwise product takes out again), runs the two
// forward transforms in lockstep (shared twiddle loads and barriers),
// multiplies pointwise in registers and runs the inverse transform
// (ntt32.cuh), leaving the residues in shared memory.  It then recombines each
// coefficient with Garner's mixed-radix formula (ten Shoup products by
// constant inverses, then a Horner evaluation in 32-bit words), sums the
// three-word coefficients of its 8 output limbs, passes the overflow words to
// its right neighbour and resolves the remaining one-bit carries with
// mi::group_carry -- the final carry that the reference does with
// splitFftReg + baddRegMul2Fft (cuda/ker-fft-help.cu.h:3-95).
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

// x*K mod p in [0, 2p) for a 64-bit digit x: K0 = K mod p, K1 = 2^32 K mod p
// (Shoup pairs).
__device__ __forceinline__ uint32_t convert(uint64_t x, const Field& f, uint2 k0, uint2 k1) {
    return f.add(f.shoup(uint32_t(x), k0), f.shoup(uint32_t(x >> 32), k1));
}

// r[0..rlen) = a*b for a of la limbs, b of lb limbs, la + lb <= L (every
// output limb, including the carry out of the top coefficient, falls inside
// the L limbs the group produces); limbs beyond rlen are dropped.  `sm` is the
// group's MulSmem, `scr` per-warp scratch of the block.  Every thread of the
// block must call this with the same LG (the exchanges synchronise the block).
template <int LG>
__device__ __forceinline__ void mul_one(const uint64_t* __restrict__ ar, uint32_t la, const uint64_t* __restrict__ br,
                                        uint32_t lb, uint64_t* __restrict__ rr, uint32_t rlen, const NttMulParams& P,
                                        uint32_t* sm, uint32_t* scr) {
    using Pl = Plan<LG>;
    uint32_t* sh = sm;               // exchange buffers of a and b (2L)
    uint32_t* res = sm + 2 * Pl::L;  // res[q][slot], q < 5
    const uint32_t t = threadIdx.x % Pl::NT;
#pragma unroll 1
    for (int q = 0; q < kPrimes; ++q) {
        const Field f{P.p[q], 2 * P.p[q], P.pinv[q]};
        const uint2 ka0 = P.ka_by_lg[q][LG - 8][0], ka1 = P.ka_by_lg[q][LG - 8][1];
        const uint2 kb0 = P.kb[q][0], kb1 = P.kb[q][1];
        uint32_t x[2][8];  // a and b, transformed in lockstep
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const uint32_t i = t + Pl::NT * j;
            x[0][j] = (i < la) ? convert(__ldg(ar + i), f, ka0, ka1) : 0u;
            x[1][j] = (i < lb) ? convert(__ldg(br + i), f, kb0, kb1) : 0u;
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
    // p3 y4))) < 2^150, evaluated in 32-bit words.
    uint64_t s[11];
#pragma unroll
    for (int w = 0; w < 11; ++w) s[w] = 0;
#pragma unroll
    for (int j = 0; j < 8; j += 4) {
        const uint32_t slot = swz(8 * t + j);
        uint4 rv[kPrimes];
#pragma unroll
        for (int q = 0; q < kPrimes; ++q) rv[q] = *reinterpret_cast<const uint4*>(res + q * Pl::L + slot);
#pragma unroll
        for (int h = 0; h < 4; ++h) {
            uint32_t y[kPrimes];
#pragma unroll
            for (int q = 0; q < kPrimes; ++q)
                y[q] = h == 0 ? rv[q].x : (h == 1 ? rv[q].y : (h == 2 ? rv[q].z : rv[q].w));
            int c = 0;
#pragma unroll
            for (int i = 1; i < kPrimes; ++i) {
                const Field fi{P.p[i], 2 * P.p[i], 0u};
                uint32_t v = y[i];
#pragma unroll
                for (int k = 0; k < i; ++k) v = fi.shoup(v + fi.p2 - y[k], P.garner[c++]);
                y[i] = fi.reduce(v);
            }
            // Horner in 32-bit words: acc = y4; acc = acc * p_i + y_i, i = 3..0
            uint32_t acc[5] = {y[kPrimes - 1], 0u, 0u, 0u, 0u};
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
            const uint64_t w2 = acc[4];
            // add (w0, w1, w2) at word j+h of the thread's 8-limb block
            const int o = j + h;
            unsigned __int128 a = (unsigned __int128)s[o] + w0;
            s[o] = (uint64_t)a;
            a = (unsigned __int128)s[o + 1] + w1 + (uint64_t)(a >> 64);
            s[o + 1] = (uint64_t)a;
            a = (unsigned __int128)s[o + 2] + w2 + (uint64_t)(a >> 64);
            s[o + 2] = (uint64_t)a;
#pragma unroll
            for (int w = o + 3; w < 11; ++w) {
                a = (unsigned __int128)s[w] + (uint64_t)(a >> 64);
                s[w] = (uint64_t)a;
            }
        }
    }
    // words 8..10 overflow into the right neighbour's block
    uint64_t* ov = reinterpret_cast<uint64_t*>(sh);  // 24 bytes x L/8 threads: fits the 4L bytes of sh
    ov[3 * t + 0] = s[8];
    ov[3 * t + 1] = s[9];
    ov[3 * t + 2] = s[10];
    __syncthreads();
    uint64_t in0 = 0, in1 = 0, in2 = 0;
    if (t > 0) {
        in0 = ov[3 * (t - 1) + 0];
        in1 = ov[3 * (t - 1) + 1];
        in2 = ov[3 * (t - 1) + 2];
    }
    uint64_t lo8[8], blk[8], add[8] = {in0, in1, in2, 0, 0, 0, 0, 0};
#pragma unroll
    for (int w = 0; w < 8; ++w) lo8[w] = s[w];
    bool g, p;
    chunk_add<uint64_t, 8>(lo8, add, blk, g, p);
    uint32_t gc;
    const uint32_t cin = group_carry<Pl::NT>(g, p, 0u, &gc, scr);
    chunk_inc<uint64_t, 8>(blk, cin);
    const uint32_t o0 = 8 * t;
    if (rr != nullptr) {
        if (o0 + 8 <= rlen && (reinterpret_cast<uintptr_t>(rr) & 15u) == 0) {
#pragma unroll
            for (int w = 0; w < 8; w += 2)
                __stcs(reinterpret_cast<ulonglong2*>(rr + o0 + w), make_ulonglong2(blk[w], blk[w + 1]));
        } else {
#pragma unroll
            for (int w = 0; w < 8; ++w)
                if (o0 + w < rlen) rr[o0 + w] = blk[w];
        }
    }
    __syncthreads();  // sh and res are reused by the next call
}

}  // namespace ntt32
}  // namespace mi
