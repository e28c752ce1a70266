// ntt_mul.cuh -- one exact NTT multiplication by a group of L/8 threads
// (shared by the batched kernel in ntt_mul.cu and the ragged kernels).
//
// Every u64 limb is one digit; the product of an la-limb and an lb-limb
// integer has coefficients below min(la, lb) * 2^128 <= 2^139 (limbs <= 2048),
// so three primes q0 < q1 < q2 < 2^62 (product 2^186) recover every coefficient
// exactly by CRT.  For each prime the group converts a and b into the field
// (a scaled by 1/L, so the inverse transform needs no scaling pass), runs two
// forward transforms, multiplies pointwise and runs the inverse transform
// (ntt.cuh), leaving the residues in shared memory.  It then recombines each
// coefficient with Garner's formula, sums the three-word coefficients of its 8
// output limbs, passes the overflow words to its right neighbour and resolves
// the remaining one-bit carries with mi::group_carry -- the final carry that
// the reference does with splitFftReg + baddRegMul2Fft
// (cuda/ker-fft-help.cu.h:3-95).
#pragma once

#include "common.cuh"
#include "ntt.cuh"
#include "ntt_host.h"

namespace mi {
namespace ntt {

// Shared memory of one group: exchange buffer (L) + three residue arrays (3L).
template <int LG>
struct MulSmem {
    static constexpr int L = 1 << LG;
    static constexpr size_t WORDS64 = size_t(4) * L;
};

// r[0..rlen) = a*b for a of la limbs, b of lb limbs, la + lb <= L (every
// output limb, including the carry out of the top coefficient, falls inside
// the L limbs the group produces); limbs beyond rlen are dropped.  `sm` is the group's MulSmem, `scr`
// per-warp scratch of the block.  Every thread of the block must call this
// with the same LG (the exchanges synchronise the block).
template <int LG>
__device__ __forceinline__ void mul_one(const uint64_t* __restrict__ ar, uint32_t la, const uint64_t* __restrict__ br,
                                        uint32_t lb, uint64_t* __restrict__ rr, uint32_t rlen, const NttMulParams& P,
                                        uint64_t* sm, uint32_t* scr) {
    using Pl = Plan<LG>;
    uint64_t* sh = sm;           // exchange buffer
    uint64_t* res = sm + Pl::L;  // res[q][slot], q < 3
    // a's spectrum waits in res[2]'s region: it is read back (by the thread
    // that wrote it) before the inverse transform of the last prime, whose
    // barriers order those reads before res[2] is written.
    uint64_t* spec = res + 2 * Pl::L;
    const uint32_t t = threadIdx.x % Pl::NT;
#pragma unroll 1
    for (int q = 0; q < 3; ++q) {
        const FieldC32 f{P.p[q], 2 * P.p[q], P.c[q]};
        const uint64_t ka = P.ka_by_lg[q][LG];
        uint64_t x[8];
        // a*(R/L)/R = a/L and b*R^2/R = b*R: the pointwise product is then
        // a*b/L in plain form and the inverse needs no scaling.
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const uint32_t i = t + Pl::NT * j;
            x[j] = (i < la) ? f.mul(__ldg(ar + i), ka) : 0;
        }
        forward<LG>(x, sh, P.tw[q], f);
#pragma unroll
        for (int j = 0; j < 8; j += 2)
            *reinterpret_cast<ulonglong2*>(spec + swz(8 * t + j)) = make_ulonglong2(x[j], x[j + 1]);
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const uint32_t i = t + Pl::NT * j;
            x[j] = (i < lb) ? f.mul(__ldg(br + i), P.kb[q]) : 0;
        }
        forward<LG>(x, sh, P.tw[q], f);
#pragma unroll
        for (int j = 0; j < 8; j += 2) {
            const ulonglong2 v = *reinterpret_cast<const ulonglong2*>(spec + swz(8 * t + j));
            x[j] = f.mul(x[j], v.x);
            x[j + 1] = f.mul(x[j + 1], v.y);
        }
        inverse<LG>(x, sh, P.itw[q], f);
#pragma unroll
        for (int j = 0; j < 8; ++j) res[q * Pl::L + swz(t + Pl::NT * j)] = reduce1(x[j], f.p);
    }
    __syncthreads();

    // Garner: x = r0 + q0*y1 + q0*q1*y2, three u64 words (< 2^139).
    const FieldC32 f1{P.p[1], 2 * P.p[1], P.c[1]};
    const FieldC32 f2{P.p[2], 2 * P.p[2], P.c[2]};
    uint64_t s[11];
#pragma unroll
    for (int w = 0; w < 11; ++w) s[w] = 0;
#pragma unroll
    for (int j = 0; j < 8; j += 2) {
        const uint32_t slot = swz(8 * t + j);
        const ulonglong2 r0 = *reinterpret_cast<const ulonglong2*>(res + slot);
        const ulonglong2 r1 = *reinterpret_cast<const ulonglong2*>(res + Pl::L + slot);
        const ulonglong2 r2 = *reinterpret_cast<const ulonglong2*>(res + 2 * Pl::L + slot);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const uint64_t v0 = h ? r0.y : r0.x, v1 = h ? r1.y : r1.x, v2 = h ? r2.y : r2.x;
            const uint64_t y1 = reduce1(f1.mul(v1 + f1.p - v0, P.g01), f1.p);
            const uint64_t u = reduce1(f2.mul(v2 + f2.p - v0, P.g02), f2.p);
            const uint64_t y2 = reduce1(f2.mul(u + f2.p - y1, P.g12), f2.p);
            const unsigned __int128 lo = (unsigned __int128)v0 + (unsigned __int128)P.p[0] * y1 +
                                         (unsigned __int128)P.q01_lo * y2;  // < 2^127
            const unsigned __int128 hi = (unsigned __int128)P.q01_hi * y2 + (uint64_t)(lo >> 64);
            // add (w0, w1, w2) at word j+h of the thread's 8-limb block
            const int o = j + h;
            unsigned __int128 acc = (unsigned __int128)s[o] + (uint64_t)lo;
            s[o] = (uint64_t)acc;
            acc = (unsigned __int128)s[o + 1] + (uint64_t)hi + (uint64_t)(acc >> 64);
            s[o + 1] = (uint64_t)acc;
            acc = (unsigned __int128)s[o + 2] + (uint64_t)(hi >> 64) + (uint64_t)(acc >> 64);
            s[o + 2] = (uint64_t)acc;
#pragma unroll
            for (int w = o + 3; w < 11; ++w) {
                acc = (unsigned __int128)s[w] + (uint64_t)(acc >> 64);
                s[w] = (uint64_t)acc;
            }
        }
    }
    // words 8..10 overflow into the right neighbour's block
    uint64_t* ov = sh;  // 3 words per thread
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

}  // namespace ntt
}  // namespace mi
