// ntt.cuh -- prime fields and the shared-memory NTT used by the NTT
// multiplication kernels.
//
// Fields (Montgomery form, R = 2^64, residues kept lazily in [0, 2p)):
//  * FieldC32: p = c*2^32 + 1 < 2^62.  Since p = 1 mod 2^32, the per-word
//    Montgomery factor is simply m = -t (no multiply), and m*p = m + (m*c)<<32,
//    so one reduction is two 32x32 products plus carries.  The reference's
//    FftPrime64 (cuda/ker-fft-mul.cu.h:44-57: p = 29*2^57+1, g = 21,
//    2-adicity 57) is of this form.
//  * FieldGen: any odd p < 2^62, the textbook word-by-word Montgomery
//    reduction with p' = -p^-1 mod 2^32, e.g. the reference's FftPrime32
//    (p = 3*2^30+1).
// This file serves the single-prime transform of mi_ntt_raw, which checks the
// transform code on the reference's known answers with the reference's own
// primes; the multiplication kernels use the 30-bit fields of ntt32.cuh.
// Both replace zmod_t (cuda/ker-fft-mul.cu.h:76-140), whose multiply is a
// `%` on the double-width product.
//
// Transform: length L = 2^LG held by L/8 threads, 8 residues each, in
// registers.  The forward transform is decimation in frequency (natural order
// in, bit-reversed out) done as radix-8 passes (three butterfly stages in
// registers) at strides L/8, L/64, ... and one final radix-2 or radix-4 pass
// on 8 consecutive residues; the inverse is decimation in time in the reverse
// pass order (bit-reversed in, natural out).  Between passes the residues are
// exchanged through shared memory with an XOR swizzle that keeps every
// pass's access pattern free of bank conflicts.  The reference instead runs
// lg L radix-2 stages in shared memory with a barrier per stage, after a
// bit-reversal permutation with a barrier per element, and reads each twiddle
// from global memory (fft/ifft, cuda/ker-fft-mul.cu.h:304-368).
//
// Twiddles: tw[e] = w^e * R mod p and itw[e] = w^-e * R mod p for e < 2048,
// w a primitive 4096th root of unity (the reference's getOmega convention,
// w = g^(2^(s - lg)), cuda/ker-fft-mul.cu.h:191-199, at lg = 12); a length-L
// transform reads every (4096/L)-th entry.
#pragma once

#include <cstdint>

namespace mi {
namespace ntt {

constexpr int kLgMax = 12;                 // 4096-point transforms at most
constexpr int kTwiddles = (1 << kLgMax) / 2;

struct FieldC32 {
    uint64_t p, p2;
    uint32_t c;
    __device__ __forceinline__ uint64_t mul(uint64_t x, uint64_t y) const {
        const uint32_t x0 = uint32_t(x), x1 = uint32_t(x >> 32), y0 = uint32_t(y), y1 = uint32_t(y >> 32);
        uint32_t t0, t1, t2, t3;
        asm("{\n\t"
            ".reg .u32 m;\n\t"
            "mul.lo.u32 %0, %4, %6;\n\t"
            "mul.hi.u32 %1, %4, %6;\n\t"
            "mul.lo.u32 %2, %5, %7;\n\t"
            "mul.hi.u32 %3, %5, %7;\n\t"
            "mad.lo.cc.u32 %1, %4, %7, %1;\n\t"
            "madc.hi.cc.u32 %2, %4, %7, %2;\n\t"
            "addc.u32 %3, %3, 0;\n\t"
            "mad.lo.cc.u32 %1, %5, %6, %1;\n\t"
            "madc.hi.cc.u32 %2, %5, %6, %2;\n\t"
            "addc.u32 %3, %3, 0;\n\t"
            // reduction word 0: m = -t0, T += m*p
            "sub.u32 m, 0, %0;\n\t"
            "add.cc.u32 %0, %0, m;\n\t"
            "madc.lo.cc.u32 %1, m, %8, %1;\n\t"
            "madc.hi.cc.u32 %2, m, %8, %2;\n\t"
            "addc.u32 %3, %3, 0;\n\t"
            // reduction word 1
            "sub.u32 m, 0, %1;\n\t"
            "add.cc.u32 %1, %1, m;\n\t"
            "madc.lo.cc.u32 %2, m, %8, %2;\n\t"
            "madc.hi.u32 %3, m, %8, %3;\n\t"
            "}"
            : "=&r"(t0), "=&r"(t1), "=&r"(t2), "=&r"(t3)
            : "r"(x0), "r"(x1), "r"(y0), "r"(y1), "r"(c));
        return (uint64_t(t3) << 32) | t2;
    }
};

struct FieldGen {
    uint64_t p, p2;
    uint32_t pinv;  // -p^-1 mod 2^32
    __device__ __forceinline__ uint64_t mul(uint64_t x, uint64_t y) const {
        const uint32_t x0 = uint32_t(x), x1 = uint32_t(x >> 32), y0 = uint32_t(y), y1 = uint32_t(y >> 32);
        const uint32_t p0 = uint32_t(p), p1 = uint32_t(p >> 32);
        uint32_t t0, t1, t2, t3;
        asm("{\n\t"
            ".reg .u32 m;\n\t"
            "mul.lo.u32 %0, %4, %6;\n\t"
            "mul.hi.u32 %1, %4, %6;\n\t"
            "mul.lo.u32 %2, %5, %7;\n\t"
            "mul.hi.u32 %3, %5, %7;\n\t"
            "mad.lo.cc.u32 %1, %4, %7, %1;\n\t"
            "madc.hi.cc.u32 %2, %4, %7, %2;\n\t"
            "addc.u32 %3, %3, 0;\n\t"
            "mad.lo.cc.u32 %1, %5, %6, %1;\n\t"
            "madc.hi.cc.u32 %2, %5, %6, %2;\n\t"
            "addc.u32 %3, %3, 0;\n\t"
            // word 0: m = t0 * p', T += m*p  (low word becomes 0)
            "mul.lo.u32 m, %0, %10;\n\t"
            "mad.lo.cc.u32 %0, m, %8, %0;\n\t"
            "madc.hi.cc.u32 %1, m, %8, %1;\n\t"
            "addc.cc.u32 %2, %2, 0;\n\t"
            "addc.u32 %3, %3, 0;\n\t"
            "mad.lo.cc.u32 %1, m, %9, %1;\n\t"
            "madc.hi.cc.u32 %2, m, %9, %2;\n\t"
            "addc.u32 %3, %3, 0;\n\t"
            // word 1
            "mul.lo.u32 m, %1, %10;\n\t"
            "mad.lo.cc.u32 %1, m, %8, %1;\n\t"
            "madc.hi.cc.u32 %2, m, %8, %2;\n\t"
            "addc.u32 %3, %3, 0;\n\t"
            "mad.lo.cc.u32 %2, m, %9, %2;\n\t"
            "madc.hi.u32 %3, m, %9, %3;\n\t"
            "}"
            : "=&r"(t0), "=&r"(t1), "=&r"(t2), "=&r"(t3)
            : "r"(x0), "r"(x1), "r"(y0), "r"(y1), "r"(p0), "r"(p1), "r"(pinv));
        return (uint64_t(t3) << 32) | t2;
    }
};

__device__ __forceinline__ uint64_t add_lazy(uint64_t u, uint64_t v, uint64_t p2) {
    const uint64_t s = u + v;  // < 4p < 2^64
    return s >= p2 ? s - p2 : s;
}
__device__ __forceinline__ uint64_t reduce1(uint64_t x, uint64_t p) { return x >= p ? x - p : x; }

// Shared-memory slot of residue index i: XOR of bits 2-4 with bits 5-7.  A
// bijection inside every 256-residue block that keeps pairs and quads
// adjacent (so consecutive-layout passes can move two residues per access).
__device__ __forceinline__ uint32_t swz(uint32_t i) { return i ^ (((i >> 5) & 7u) << 2); }

template <int LG>
struct Plan {
    static constexpr int L = 1 << LG;
    static constexpr int NT = L / 8;           // threads per transform
    static constexpr int NF = LG / 3;          // radix-8 passes
    static constexpr int R = LG - 3 * NF;      // stages left for the final pass
    static constexpr int S = (1 << kLgMax) / L;  // twiddle-table stride
    // stride of the thread's 8 residues in pass k (k == NF: final layout)
    __host__ __device__ static constexpr int d(int k) { return k < NF ? (L >> (3 * (k + 1))) : 1; }
    __device__ static __forceinline__ uint32_t idx(int d, uint32_t t, int j) {
        return (t / d) * 8 * d + (t % d) + d * j;
    }
};

// Moves the thread's 8 residues from layout (stride) d_from to d_to through
// shared memory.  Both barriers are needed: the second one protects `sh`
// before anybody writes the next exchange.
template <int LG>
__device__ __forceinline__ void exchange(uint64_t (&x)[8], uint64_t* sh, int d_from, int d_to) {
    using P = Plan<LG>;
    const uint32_t t = threadIdx.x % P::NT;
    if (d_from == 1) {
#pragma unroll
        for (int j = 0; j < 8; j += 2)
            *reinterpret_cast<ulonglong2*>(sh + swz(P::idx(1, t, j))) = make_ulonglong2(x[j], x[j + 1]);
    } else {
#pragma unroll
        for (int j = 0; j < 8; ++j) sh[swz(P::idx(d_from, t, j))] = x[j];
    }
    __syncthreads();
    if (d_to == 1) {
#pragma unroll
        for (int j = 0; j < 8; j += 2) {
            const ulonglong2 v = *reinterpret_cast<const ulonglong2*>(sh + swz(P::idx(1, t, j)));
            x[j] = v.x;
            x[j + 1] = v.y;
        }
    } else {
#pragma unroll
        for (int j = 0; j < 8; ++j) x[j] = sh[swz(P::idx(d_to, t, j))];
    }
    __syncthreads();
}

// Forward transform (DIF).  In: x[j] = residue t + L/8*j (natural order),
// values in [0, 2p).  Out: layout stride 1 (x[j] = slot 8t+j of the
// bit-reversed spectrum), values in [0, 2p).
template <int LG, typename F>
__device__ __forceinline__ void forward(uint64_t (&x)[8], uint64_t* sh, const uint64_t* __restrict__ tw, const F& f) {
    using P = Plan<LG>;
    const uint32_t t = threadIdx.x % P::NT;
    auto bf = [&](int j, int k, uint32_t e) {
        const uint64_t u = x[j], v = x[k];
        x[j] = add_lazy(u, v, f.p2);
        x[k] = f.mul(u + f.p2 - v, __ldg(tw + e));
    };
#pragma unroll
    for (int k = 0; k < P::NF; ++k) {
        const int d = P::d(k);
        if (k > 0) exchange<LG>(x, sh, P::d(k - 1), d);
        const uint32_t off = t % d;
        const uint32_t mult = uint32_t(P::S) << (3 * k);  // (L / 8d) * S
#pragma unroll
        for (int j = 0; j < 4; ++j) bf(j, j + 4, (off + d * j) * mult);
#pragma unroll
        for (int j = 0; j < 8; j += 4) {
            bf(j, j + 2, off * 2 * mult);
            bf(j + 1, j + 3, (off + d) * 2 * mult);
        }
#pragma unroll
        for (int j = 0; j < 8; j += 2) bf(j, j + 1, off * 4 * mult);
    }
    if constexpr (P::R > 0) {
        exchange<LG>(x, sh, P::d(P::NF - 1), 1);
        if constexpr (P::R == 2) {
            const uint32_t e1 = uint32_t(P::L / 4) * P::S;
#pragma unroll
            for (int j = 0; j < 8; j += 4) {
                bf(j, j + 2, 0);
                bf(j + 1, j + 3, e1);
            }
        }
#pragma unroll
        for (int j = 0; j < 8; j += 2) {  // twiddle 1
            const uint64_t u = x[j], v = x[j + 1];
            x[j] = add_lazy(u, v, f.p2);
            x[j + 1] = add_lazy(u + f.p2 - v, 0, f.p2);
        }
    }
}

// Inverse transform without the 1/L scaling (DIT).  In: stride-1 layout of a
// bit-reversed spectrum; out: x[j] = residue t + L/8*j in natural order;
// values in [0, 2p) throughout.
template <int LG, typename F>
__device__ __forceinline__ void inverse(uint64_t (&x)[8], uint64_t* sh, const uint64_t* __restrict__ itw, const F& f) {
    using P = Plan<LG>;
    const uint32_t t = threadIdx.x % P::NT;
    auto bf = [&](int j, int k, uint32_t e) {
        const uint64_t u = x[j], v = f.mul(x[k], __ldg(itw + e));
        x[j] = add_lazy(u, v, f.p2);
        x[k] = add_lazy(u + f.p2 - v, 0, f.p2);
    };
    if constexpr (P::R > 0) {
#pragma unroll
        for (int j = 0; j < 8; j += 2) {  // twiddle 1
            const uint64_t u = x[j], v = x[j + 1];
            x[j] = add_lazy(u, v, f.p2);
            x[j + 1] = add_lazy(u + f.p2 - v, 0, f.p2);
        }
        if constexpr (P::R == 2) {
            const uint32_t e1 = uint32_t(P::L / 4) * P::S;
#pragma unroll
            for (int j = 0; j < 8; j += 4) {
                bf(j, j + 2, 0);
                bf(j + 1, j + 3, e1);
            }
        }
        exchange<LG>(x, sh, 1, P::d(P::NF - 1));
    }
#pragma unroll
    for (int k = P::NF - 1; k >= 0; --k) {
        const int d = P::d(k);
        const uint32_t off = t % d;
        const uint32_t mult = uint32_t(P::S) << (3 * k);
#pragma unroll
        for (int j = 0; j < 8; j += 2) bf(j, j + 1, off * 4 * mult);
#pragma unroll
        for (int j = 0; j < 8; j += 4) {
            bf(j, j + 2, off * 2 * mult);
            bf(j + 1, j + 3, (off + d) * 2 * mult);
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) bf(j, j + 4, (off + d * j) * mult);
        if (k > 0) exchange<LG>(x, sh, d, P::d(k - 1));
    }
}

}  // namespace ntt
}  // namespace mi
