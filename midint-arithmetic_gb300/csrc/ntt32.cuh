// ntt32.cuh -- 30-bit prime fields and the shared-memory NTT of the
// multiplication kernels.
//
// Field: p < 2^30 with 2^21 | p - 1; residues kept lazily in [0, 2p), so every
// sum and difference of two residues fits 32 bits.  Twiddle products use
// Shoup's method with a precomputed companion w' = floor(w * 2^32 / p):
// x*w mod p = x*w - hi(x*w')*p in [0, 2p) for any 32-bit x, three integer
// multiplies.  Products of two variables (the pointwise product of spectra)
// use Montgomery reduction with R = 2^32 (four multiplies), whose 1/R is folded
// into one operand's conversion.  These replace zmod_t
// (cuda/ker-fft-mul.cu.h:76-140), whose multiply is a `%` on the double-width
// product.
//
// Transform: length L = 2^LG held by L/8 threads, 8 residues each, in
// registers.  The forward transform is decimation in frequency (natural order
// in, bit-reversed out) done as radix-8 passes (three butterfly stages in
// registers) at strides L/8, L/64, ... and one final radix-2 or radix-4 pass
// on 8 consecutive residues; the inverse is decimation in time in the reverse
// pass order (bit-reversed in, natural out).  Between passes the residues are
// exchanged through shared memory in a padded layout (residue i at word
// i + 4 floor(i/32)) that keeps the passes free of bank conflicts (one 2-way
// layout at L = 1024) and whose word addresses are a per-thread base plus a
// compile-time offset per residue.
// The reference instead runs lg L radix-2 stages in shared memory with a
// barrier per stage, after a bit-reversal permutation with a barrier per
// element, and reads each twiddle from global memory (fft/ifft,
// cuda/ker-fft-mul.cu.h:304-368).
//
// Twiddles: pairs (w^e, floor(w^e 2^32 / p)) for the forward table and the
// same for w^-e for the inverse, w a primitive 4096th root of unity, stored in
// the order the passes read them (TwLayout): the lanes of a warp read
// consecutive entries, a few cache lines per load instead of one line per
// lane as in a table indexed by exponent.
#pragma once

#include <cstdint>

namespace mi {
namespace ntt32 {

constexpr int kLgMin = 8, kLgMax = 12;         // 256- to 4096-point transforms
constexpr int kTwiddles = (1 << kLgMax) / 2;   // powers w^e, e < 2048, that the passes use
constexpr int kPrimes = 5;

// Twiddle table layout of one prime and direction.  For a length-2^LG
// transform, radix-8 pass k has stride d = L / 8^(k+1) and twiddle step
// m = 4096 / (8d); its butterflies at offset o = t mod d use w^((o + dj) m)
// (stage 1, j < 4), w^(2 (o + dh) m) (stage 2, h < 2) and w^(4 o m) (stage 3).
// The pass's entries are stage 1's 4d powers by o + dj, then stage 2's 2d by
// o + dh, then stage 3's d by o; after the last pass one entry w^1024 (the
// radix-4 step of the final pass).  Sections are rounded up to 16 entries.
struct TwLayout {
    __host__ __device__ static constexpr int nf(int lg) { return lg / 3; }
    __host__ __device__ static constexpr int d(int lg, int k) { return (1 << lg) >> (3 * (k + 1)); }
    // start of pass k inside the section of lg
    __host__ __device__ static constexpr int pass(int lg, int k) {
        int s = 0;
        for (int i = 0; i < k; ++i) s += 7 * d(lg, i);
        return s;
    }
    __host__ __device__ static constexpr int quarter(int lg) { return pass(lg, nf(lg)); }
    __host__ __device__ static constexpr int size(int lg) { return (quarter(lg) + 1 + 15) / 16 * 16; }
    __host__ __device__ static constexpr int base(int lg) {
        int s = 0;
        for (int g = kLgMin; g < lg; ++g) s += size(g);
        return s;
    }
};
constexpr int kTwEntries = TwLayout::base(kLgMax + 1);  // per prime and direction

struct Field {
    uint32_t p, p2, pinv;  // pinv = -p^-1 mod 2^32
    __device__ __forceinline__ uint32_t add(uint32_t u, uint32_t v) const {
        const uint32_t s = u + v;  // < 4p
        return min(s, s - p2);
    }
    // u - v + 2p in (0, 4p), reduced to [0, 2p)
    __device__ __forceinline__ uint32_t sub(uint32_t u, uint32_t v) const {
        const uint32_t s = u + p2 - v;
        return min(s, s - p2);
    }
    __device__ __forceinline__ uint32_t shoup(uint32_t x, uint2 w) const {
        const uint32_t q = __umulhi(x, w.y);
        return x * w.x - q * p;
    }
    // x*y/2^32 mod p in [0, 2p) for x, y < 2p
    __device__ __forceinline__ uint32_t mont(uint32_t x, uint32_t y) const {
        const uint32_t lo = x * y, hi = __umulhi(x, y);
        const uint32_t m = lo * pinv;
        return hi + __umulhi(m, p) + (lo != 0u ? 1u : 0u);
    }
    __device__ __forceinline__ uint32_t reduce(uint32_t x) const { return min(x, x - p); }
    // [0, 4p) -> [0, 2p)
    __device__ __forceinline__ uint32_t reduce2(uint32_t x) const { return min(x, x - p2); }
};

// Shared-memory word of residue index i: XOR of bits 2-4 with bits 5-7.  A
// bijection inside every 256-word block that keeps aligned quads together
// (so the consecutive layout moves four residues per access).
__device__ __forceinline__ uint32_t swz(uint32_t i) { return i ^ (((i >> 5) & 7u) << 2); }

template <int LG>
struct Plan {
    static constexpr int L = 1 << LG;
    static constexpr int NT = L / 8;             // threads per transform
    static constexpr int NF = LG / 3;            // radix-8 passes
    static constexpr int R = LG - 3 * NF;        // stages left for the final pass
    static constexpr int S = (1 << kLgMax) / L;  // twiddle-table stride
    __host__ __device__ static constexpr int d(int k) { return k < NF ? (L >> (3 * (k + 1))) : 1; }
    __device__ static __forceinline__ uint32_t idx(int d, uint32_t t, int j) {
        return (t / d) * 8 * d + (t % d) + d * j;
    }
    // Exchange arrays: residue i at word i + 4 floor(i/32), so L + L/8 words.
    // For the residues idx(d, t, j) of a thread in the layout of stride d the
    // word is xbase(d, t) + xoff(d, j): floor(idx/32) splits into a part of t
    // and a part of j for every power-of-two d.  The 32 lanes of a warp then
    // touch 32 distinct banks for d != 2 (2-way at d = 2), and the quads of
    // the d = 1 layout 8 distinct 16-byte slots per quarter warp.
    static constexpr int LX = L + L / 8;
    __device__ static __forceinline__ uint32_t xbase(int d, uint32_t t) {
        if (d >= 32) return (t / d) * 9 * d + (t % d) + 4 * ((t % d) >> 5);
        if (d == 16) return 144 * (t / 16) + (t % 16);
        if (d == 8) return 72 * (t / 8) + (t % 8);
        if (d == 4) return 36 * (t / 4) + (t % 4);
        if (d == 2) return 16 * (t / 2) + (t % 2) + 4 * (t / 4);
        return 8 * t + 4 * (t / 4);
    }
    __host__ __device__ static constexpr uint32_t xoff(int d, int j) {
        return d >= 32 ? uint32_t(9 * d / 8 * j)
                       : (d == 16 ? uint32_t(16 * j + 4 * (j / 2))
                                  : (d == 8 ? uint32_t(8 * j + 4 * (j / 4)) : uint32_t(d * j)));
    }
};

// Moves the thread's 8 residues of each of NA arrays (each with its own LX
// words of `sh`) from layout (stride) d_from to d_to through shared memory.
// In a layout of stride d <= 32 the residues of a warp are the 256
// consecutive words of its own block, so an exchange between two such
// layouts only synchronises the warp; the others synchronise the block.  The
// first barrier makes every earlier read of the words about to be written
// complete (the transforms start with a block-wide exchange, and between
// transforms `sh` is only read by the thread that wrote it).
template <int LG, int NA>
__device__ __forceinline__ void exchange(uint32_t (&x)[NA][8], uint32_t* sh, int d_from, int d_to) {
    using P = Plan<LG>;
    const uint32_t t = threadIdx.x % P::NT;
    const bool local = P::NT <= 32 || (d_from <= 32 && d_to <= 32);
    if (local) __syncwarp(); else __syncthreads();
#pragma unroll
    for (int q = 0; q < NA; ++q) {
        uint32_t* s = sh + q * P::LX;
        const uint32_t b = P::xbase(d_from, t);
        if (d_from == 1) {
#pragma unroll
            for (int j = 0; j < 8; j += 4)
                *reinterpret_cast<uint4*>(s + b + j) = make_uint4(x[q][j], x[q][j + 1], x[q][j + 2], x[q][j + 3]);
        } else {
#pragma unroll
            for (int j = 0; j < 8; ++j) s[b + P::xoff(d_from, j)] = x[q][j];
        }
    }
    if (local) __syncwarp(); else __syncthreads();
#pragma unroll
    for (int q = 0; q < NA; ++q) {
        const uint32_t* s = sh + q * P::LX;
        const uint32_t b = P::xbase(d_to, t);
        if (d_to == 1) {
#pragma unroll
            for (int j = 0; j < 8; j += 4) {
                const uint4 v = *reinterpret_cast<const uint4*>(s + b + j);
                x[q][j] = v.x;
                x[q][j + 1] = v.y;
                x[q][j + 2] = v.z;
                x[q][j + 3] = v.w;
            }
        } else {
#pragma unroll
            for (int j = 0; j < 8; ++j) x[q][j] = s[b + P::xoff(d_to, j)];
        }
    }
}

// Forward transforms (DIF) of NA arrays in lockstep on one prime (each
// twiddle is loaded once for all of them).  In: x[q][j] = residue t + L/8*j
// (natural order), values in [0, 2p).  Out: layout stride 1 (x[q][j] = slot
// 8t+j of the bit-reversed spectrum), values in [0, 2p).  HALF: residues
// L/2.. are zero (x[q][4..7] are not read), so the first stage of the first
// pass is x[j + 4] = x[j] w with x[j] unchanged.
template <int LG, int NA, bool HALF = false>
__device__ __forceinline__ void forward(uint32_t (&x)[NA][8], uint32_t* sh, const uint2* __restrict__ tw_all,
                                        const Field& f) {
    using P = Plan<LG>;
    const uint32_t t = threadIdx.x % P::NT;
    const uint2* __restrict__ tw = tw_all + TwLayout::base(LG);
    auto bf = [&](int j, int k, uint32_t e) {
        const uint2 w = __ldg(tw + e);
#pragma unroll
        for (int q = 0; q < NA; ++q) {
            const uint32_t u = x[q][j], v = x[q][k];
            x[q][j] = f.add(u, v);
            x[q][k] = f.shoup(u + f.p2 - v, w);
        }
    };
#pragma unroll
    for (int k = 0; k < P::NF; ++k) {
        const int d = P::d(k);
        if (k > 0) exchange<LG, NA>(x, sh, P::d(k - 1), d);
        const uint32_t off = t % d, e0 = TwLayout::pass(LG, k) + off;
        if (HALF && k == 0) {
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const uint2 w = __ldg(tw + e0 + d * j);
#pragma unroll
                for (int q = 0; q < NA; ++q) x[q][j + 4] = f.shoup(x[q][j], w);
            }
        } else {
#pragma unroll
            for (int j = 0; j < 4; ++j) bf(j, j + 4, e0 + d * j);
        }
#pragma unroll
        for (int j = 0; j < 8; j += 4) {
            bf(j, j + 2, e0 + 4 * d);
            bf(j + 1, j + 3, e0 + 5 * d);
        }
#pragma unroll
        for (int j = 0; j < 8; j += 2) bf(j, j + 1, e0 + 6 * d);
    }
    if constexpr (P::R > 0) {
        exchange<LG, NA>(x, sh, P::d(P::NF - 1), 1);
        if constexpr (P::R == 2) {
            const uint2 w1 = __ldg(tw + TwLayout::quarter(LG));
#pragma unroll
            for (int q = 0; q < NA; ++q)
#pragma unroll
                for (int j = 0; j < 8; j += 4) {
                    const uint32_t u0 = x[q][j], v0 = x[q][j + 2], u1 = x[q][j + 1], v1 = x[q][j + 3];
                    x[q][j] = f.add(u0, v0);
                    x[q][j + 2] = f.sub(u0, v0);  // twiddle 1
                    x[q][j + 1] = f.add(u1, v1);
                    x[q][j + 3] = f.shoup(u1 + f.p2 - v1, w1);
                }
        }
#pragma unroll
        for (int q = 0; q < NA; ++q)
#pragma unroll
            for (int j = 0; j < 8; j += 2) {  // twiddle 1
                const uint32_t u = x[q][j], v = x[q][j + 1];
                x[q][j] = f.add(u, v);
                x[q][j + 1] = f.sub(u, v);
            }
    }
}

// Inverse transform without the 1/L scaling (DIT).  In: stride-1 layout of a
// bit-reversed spectrum, values in [0, 2p); out: x[j] = residue t + L/8*j in
// natural order, values in [0, 2p).  In between the values are kept in
// [0, 4p) (Harvey's lazy butterflies): a butterfly brings its unmultiplied
// input to [0, 2p) with one conditional subtraction, the Shoup product of the
// other is in [0, 2p) for any 32-bit input, and both outputs u + v and
// u - v + 2p stay below 4p < 2^32 -- two integer instructions per butterfly
// fewer than reducing both outputs.
template <int LG>
__device__ __forceinline__ void inverse(uint32_t (&x)[8], uint32_t* sh, const uint2* __restrict__ itw_all,
                                        const Field& f) {
    uint32_t(&xs)[1][8] = reinterpret_cast<uint32_t(&)[1][8]>(x);
    using P = Plan<LG>;
    const uint32_t t = threadIdx.x % P::NT;
    const uint2* __restrict__ itw = itw_all + TwLayout::base(LG);
    auto bf = [&](int j, int k, uint32_t e) {
        const uint32_t u = f.reduce2(x[j]), v = f.shoup(x[k], __ldg(itw + e));
        x[j] = u + v;
        x[k] = u + f.p2 - v;
    };
    if constexpr (P::R > 0) {
#pragma unroll
        for (int j = 0; j < 8; j += 2) {  // twiddle 1; inputs in [0, 2p)
            const uint32_t u = x[j], v = x[j + 1];
            x[j] = u + v;
            x[j + 1] = u + f.p2 - v;
        }
        if constexpr (P::R == 2) {
            const uint2 w1 = __ldg(itw + TwLayout::quarter(LG));
#pragma unroll
            for (int j = 0; j < 8; j += 4) {
                const uint32_t u0 = f.reduce2(x[j]), v0 = f.reduce2(x[j + 2]);
                const uint32_t u1 = f.reduce2(x[j + 1]), v1 = f.shoup(x[j + 3], w1);
                x[j] = u0 + v0;
                x[j + 2] = u0 + f.p2 - v0;
                x[j + 1] = u1 + v1;
                x[j + 3] = u1 + f.p2 - v1;
            }
        }
        exchange<LG, 1>(xs, sh, 1, P::d(P::NF - 1));
    }
#pragma unroll
    for (int k = P::NF - 1; k >= 0; --k) {
        const int d = P::d(k);
        const uint32_t off = t % d, e0 = TwLayout::pass(LG, k) + off;
#pragma unroll
        for (int j = 0; j < 8; j += 2) bf(j, j + 1, e0 + 6 * d);
#pragma unroll
        for (int j = 0; j < 8; j += 4) {
            bf(j, j + 2, e0 + 4 * d);
            bf(j + 1, j + 3, e0 + 5 * d);
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) bf(j, j + 4, e0 + d * j);
        if (k > 0) exchange<LG, 1>(xs, sh, d, P::d(k - 1));
    }
#pragma unroll
    for (int j = 0; j < 8; ++j) x[j] = f.reduce2(x[j]);
}

}  // namespace ntt32
}  // namespace mi
