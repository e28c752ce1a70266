// poly_ntt.cu -- the fused polynomial composite ((a^2 + b)(b^2 + b) + ab) mod
// 2^(64m) on number-theoretic transforms, for operands from a few hundred u64
// limbs up, where a transform product is cheaper than the classical one.
//
// Counterpart of the reference's polyFttKer (cuda/ker-fft-mul.cu.h:456-509),
// which runs four FFT products and three additions on 16-bit digits in one
// kernel (and, like its bmulFFT, is exact only for tiny inputs).  The
// classical form of the same composite is poly.cu (polyKerQ).
//
// One CTA of L/8 threads owns an instance (L = pow2ceil(2m), the transform
// length of an m x m product, so the cyclic convolution never wraps into the
// low m coefficients).  The four products all keep only their low m limbs:
//   P3 = ab,  T1 = a^2 + b,  T2 = b^2 + b,  r = T1 T2 + P3   (all mod 2^(64m))
// Each product runs, per prime, the steps of ntt32::mul_one (conversion,
// forward transforms, pointwise product, inverse transform) but stores only
// the residues of its low L/2 coefficients; a square takes one forward
// transform (its pointwise product is X * X * 2^32/L by a Shoup product and a
// Montgomery one).  Garner's recombination and the digit sums then give the
// thread's output limbs, the addend of the step (b or P3) is added into the
// digit sums, and one carry pass over the group leaves the m limbs in shared
// memory (T1, T2, P3) or in the result row (r): the intermediates never leave
// the chip.  Per prime 10 transforms instead of the 12 of four separate
// products; digit modes (64-bit digits on five primes, 48-bit ones on four
// where they fit the same length) as in ntt_mul.cuh.
#include <cstdio>

#include "common.cuh"
#include "kernels.h"
#include "ntt_host.h"
#include "ntt32.cuh"
#include "ntt_mul.cuh"

namespace mi {
namespace {

using ntt32::Field;
using ntt32::Plan;

// Shared memory of one CTA, in 32-bit words: exchange buffers (2 LX), the
// low-half residues of five primes (5 L/2), and the three intermediates T1,
// T2, P3 (m u64 limbs each, at most L/2 limbs: L words each).
template <int LG>
struct PolySmem {
    static constexpr int L = 1 << LG;
    static constexpr int SH = 0, RES = 2 * Plan<LG>::LX, T1 = RES + 5 * L / 2, T2 = T1 + L, P3 = T2 + L;
    static constexpr size_t WORDS32 = size_t(P3 + L);
};

// 48-bit digit i of a row of `words` u32 words read through a generic
// pointer (global or shared), as its low 32 bits and its high 16.
__device__ __forceinline__ uint2 digit48_any(const uint32_t* row, uint32_t words, uint32_t i) {
    const uint32_t w = (3 * i) >> 1;
    const uint32_t w0 = w < words ? row[w] : 0u;
    const uint32_t w1 = w + 1 < words ? row[w + 1] : 0u;
    return (i & 1) ? make_uint2(__funnelshift_r(w0, w1, 16), w1 >> 16) : make_uint2(w0, w1 & 0xffffu);
}

// Residue of digit i of an m-limb operand, times the constant whose Shoup
// pairs are (k0 = K, k1 = 2^32 K).
template <bool D48>
__device__ __forceinline__ uint32_t digit_residue(const uint64_t* x, uint32_t m, uint32_t i, const Field& f, uint2 k0,
                                                  uint2 k1) {
    if constexpr (D48) {
        const uint2 d = digit48_any(reinterpret_cast<const uint32_t*>(x), 2 * m, i);
        return f.add(f.shoup(d.x, k0), f.shoup(d.y, k1));
    } else {
        return i < m ? ntt32::convert(x[i], f, k0, k1) : 0u;
    }
}

// Residue of digit i of an m-limb operand, unscaled (c32: the Shoup pair of
// 2^32 mod p).
template <bool D48>
__device__ __forceinline__ uint32_t digit_plain(const uint64_t* x, uint32_t m, uint32_t i, const Field& f, uint2 c32) {
    if constexpr (D48) {
        const uint2 d = digit48_any(reinterpret_cast<const uint32_t*>(x), 2 * m, i);
        return ntt32::reduce_digit(d.x, d.y, f, c32);
    } else {
        const uint64_t v = i < m ? x[i] : 0ull;
        return ntt32::reduce_digit(uint32_t(v), uint32_t(v >> 32), f, c32);
    }
}

// dst[0..m) = (x * y + addend) mod 2^(64m) (SQ: y is x).  x, y and addend are
// generic pointers to m u64 limbs (global or shared); addend may be null; dst
// is global or shared and may alias neither x nor y.  Every thread of the
// block calls this; it starts and ends with the block's shared areas free.
template <int LG, bool D48, bool SQ>
__device__ __forceinline__ void lo_product(const uint64_t* x, const uint64_t* y, const uint64_t* addend, uint64_t* dst,
                                           uint32_t m, const NttMulParams& P, uint32_t* sm, uint32_t* scr) {
    using Pl = Plan<LG>;
    using S = PolySmem<LG>;
    constexpr int SW = 11;
    constexpr int HALF = Pl::L / 2;
    uint32_t* sh = sm + S::SH;
    uint32_t* res = sm + S::RES;
    const uint32_t t = threadIdx.x % Pl::NT;
    const int np = D48 ? 4 : ntt32::kPrimes;
#pragma unroll 1
    for (int q = 0; q < np; ++q) {
        const Field f{P.p[q], 2 * P.p[q], P.pinv[q]};
        if constexpr (SQ) {
            // X = F(x); pointwise X * (X * 2^32/L) / 2^32 = X^2 / L
            const uint2 c32 = P.kb[q][0], ks = P.ka_by_lg[q][LG - 8][1];
            uint32_t v[1][8];
#pragma unroll
            for (int j = 0; j < 4; ++j) v[0][j] = digit_plain<D48>(x, m, t + Pl::NT * j, f, c32);
            ntt32::forward<LG, 1, true>(v, sh, P.tw[q], f);  // m digits fit L/2: the upper half is zero
#pragma unroll
            for (int j = 0; j < 8; ++j) v[0][j] = f.mont(v[0][j], f.shoup(v[0][j], ks));
            ntt32::inverse<LG>(v[0], sh, P.itw[q], f);
#pragma unroll
            for (int j = 0; j < 4; ++j) res[q * HALF + ntt32::swz(t + Pl::NT * j)] = f.reduce(v[0][j]);
        } else {
            // x unscaled, y times 2^32 / L
            const uint2 c32 = P.kb[q][0];
            const uint2 kb0 = P.ka_by_lg[q][LG - 8][1], kb1 = P.kb_by_lg[q][LG - 8];
            uint32_t v[2][8];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                v[0][j] = digit_plain<D48>(x, m, t + Pl::NT * j, f, c32);
                v[1][j] = digit_residue<D48>(y, m, t + Pl::NT * j, f, kb0, kb1);
            }
            ntt32::forward<LG, 2, true>(v, sh, P.tw[q], f);  // the upper halves are zero
#pragma unroll
            for (int j = 0; j < 8; ++j) v[0][j] = f.mont(v[0][j], v[1][j]);
            ntt32::inverse<LG>(v[0], sh, P.itw[q], f);
#pragma unroll
            for (int j = 0; j < 4; ++j) res[q * HALF + ntt32::swz(t + Pl::NT * j)] = f.reduce(v[0][j]);
        }
    }
    __syncthreads();

    // Garner + digit sums of the thread's 8 coefficients (those of the low
    // half only; the others reach limbs >= m or do not exist)
    uint64_t s[SW];
#pragma unroll
    for (int w = 0; w < SW; ++w) s[w] = 0;
    if (8 * t < HALF) {
#pragma unroll
        for (int j = 0; j < 8; j += 4) {
            const uint32_t slot = ntt32::swz(8 * t + j);
#pragma unroll
            for (int h = 0; h < 4; ++h) {
                uint32_t yv[ntt32::kPrimes];
#pragma unroll
                for (int q = 0; q < ntt32::kPrimes; ++q) yv[q] = (q < 4 || !D48) ? res[q * HALF + slot + h] : 0u;
                int c = 0;
#pragma unroll
                for (int i = 1; i < ntt32::kPrimes; ++i) {
                    if (D48 && i == ntt32::kPrimes - 1) break;
                    const Field fi{P.p[i], 2 * P.p[i], 0u};
                    uint32_t v = yv[i];
#pragma unroll
                    for (int k = 0; k < i; ++k) v = fi.shoup(v + fi.p2 - yv[k], P.garner[c++]);
                    yv[i] = fi.reduce(v);
                }
                if (D48) yv[ntt32::kPrimes - 1] = 0;
                uint32_t acc[ntt32::kPrimes] = {yv[ntt32::kPrimes - 1], 0u, 0u, 0u, 0u};
#pragma unroll
                for (int i = ntt32::kPrimes - 2; i >= 0; --i) {
                    uint64_t carry = yv[i];
#pragma unroll
                    for (int w = 0; w < ntt32::kPrimes - 1 - i; ++w) {
                        const uint64_t tt = uint64_t(acc[w]) * P.p[i] + carry;
                        acc[w] = uint32_t(tt);
                        carry = tt >> 32;
                    }
                    acc[ntt32::kPrimes - 1 - i] = uint32_t(carry);
                }
                const uint64_t w0 = uint64_t(acc[0]) | (uint64_t(acc[1]) << 32);
                const uint64_t w1 = uint64_t(acc[2]) | (uint64_t(acc[3]) << 32);
                const int o = j + h;
                if (!D48) {
                    ntt32::add3_at<SW>(s, o, w0, w1, uint64_t(acc[4]));
                } else {
                    const int bit = 48 * o, w = bit >> 6, b = bit & 63;
                    const uint64_t x0 = w0 << b;
                    const uint64_t x1 = b ? (w1 << b) | (w0 >> (64 - b)) : w1;
                    const uint64_t x2 = b ? w1 >> (64 - b) : 0ull;
                    ntt32::add3_at<SW>(s, w, x0, x1, x2);
                }
            }
        }
    }
    // the addend's limbs of the thread's block enter the digit sums
    constexpr int OUT = D48 ? 6 : 8, OVW = D48 ? 2 : 3;
    const uint32_t o0 = OUT * t;
    if (addend != nullptr) {
        unsigned __int128 acc = 0;
#pragma unroll
        for (int w = 0; w < SW; ++w) {
            acc += s[w];
            if (w < OUT && o0 + w < m) acc += addend[o0 + w];
            s[w] = uint64_t(acc);
            acc >>= 64;
        }
    }
    // overflow words to the right neighbour, one carry pass, limbs below m out
    uint64_t* ov = reinterpret_cast<uint64_t*>(sh);
#pragma unroll
    for (int w = 0; w < OVW; ++w) ov[OVW * t + w] = s[OUT + w];
    __syncthreads();
    uint64_t add[OUT], lo[OUT], blk[OUT];
#pragma unroll
    for (int w = 0; w < OUT; ++w) {
        add[w] = (w < OVW && t > 0) ? ov[OVW * (t - 1) + w] : 0ull;
        lo[w] = s[w];
    }
    bool g, p;
    chunk_add<uint64_t, OUT>(lo, add, blk, g, p);
    uint32_t gc;
    const uint32_t cin = group_carry<Pl::NT>(g, p, 0u, &gc, scr);
    chunk_inc<uint64_t, OUT>(blk, cin);
#pragma unroll
    for (int w = 0; w < OUT; ++w)
        if (o0 + w < m) dst[o0 + w] = blk[w];
    __syncthreads();  // dst complete; sh and res free
}

// 768 threads per SM where shared memory allows (7.5 L words per CTA: three
// 256-thread CTAs for 2048-point transforms, one 512-thread CTA for 4096);
// 512 for the 256-point ones, whose 48-bit digit mode spills at 80 registers
template <int LG, bool D48>
__global__ void __launch_bounds__((1 << LG) / 8, (LG == 8 ? 512 : 768) / ((1 << LG) / 8))
    k_poly_ntt(const uint64_t* __restrict__ a, const uint64_t* __restrict__ b, uint64_t* __restrict__ r, uint32_t n,
               uint32_t m, NttMulParams P) {
    using S = PolySmem<LG>;
    extern __shared__ __align__(16) uint32_t smem32[];
    uint32_t* scr = smem32 + S::WORDS32;
    uint64_t* t1 = reinterpret_cast<uint64_t*>(smem32 + S::T1);
    uint64_t* t2 = reinterpret_cast<uint64_t*>(smem32 + S::T2);
    uint64_t* p3 = reinterpret_cast<uint64_t*>(smem32 + S::P3);
    for (uint64_t inst = blockIdx.x; inst < n; inst += gridDim.x) {
        const uint64_t* ai = a + inst * m;
        const uint64_t* bi = b + inst * m;
        lo_product<LG, D48, false>(ai, bi, nullptr, p3, m, P, smem32, scr);  // P3 = ab
        lo_product<LG, D48, true>(ai, ai, bi, t1, m, P, smem32, scr);        // T1 = a^2 + b
        lo_product<LG, D48, true>(bi, bi, bi, t2, m, P, smem32, scr);        // T2 = b^2 + b
        lo_product<LG, D48, false>(t1, t2, p3, r + inst * m, m, P, smem32, scr);  // r = T1 T2 + P3
    }
}

template <int LG, bool D48>
mi_status launch_lg(const uint64_t* a, const uint64_t* b, uint64_t* r, uint32_t n, uint32_t m, const NttMulParams& P,
                    cudaStream_t st) {
    constexpr int NT = (1 << LG) / 8;
    const size_t smem = PolySmem<LG>::WORDS32 * 4 + size_t(NT / 32 + 1) * 4;
    auto kern = k_poly_ntt<LG, D48>;
    MI_TRY(ensure_dyn_smem(kern, smem));
    int per_sm = 0;
    MI_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, NT, smem));
    uint64_t blocks = uint64_t(sm_count()) * (per_sm > 0 ? per_sm : 1);
    if (blocks > n) blocks = n;
    kern<<<dim3(uint32_t(blocks)), dim3(NT), smem, st>>>(a, b, r, n, m, P);
    MI_CUDA_TRY(cudaGetLastError());
    return MI_OK;
}

}  // namespace

mi_status launch_poly_ntt(const uint64_t* a, const uint64_t* b, uint64_t* r, uint32_t n, uint32_t m,
                          const NttMulParams& P, cudaStream_t st) {
    uint32_t L = pow2ceil(2 * m);
    if (L < 256) L = 256;
    const bool d48 = 2 * ntt32::ntt_digits(m, true) <= L;
    switch (L) {
        case 256: return d48 ? launch_lg<8, true>(a, b, r, n, m, P, st) : launch_lg<8, false>(a, b, r, n, m, P, st);
        case 512: return d48 ? launch_lg<9, true>(a, b, r, n, m, P, st) : launch_lg<9, false>(a, b, r, n, m, P, st);
        case 1024: return d48 ? launch_lg<10, true>(a, b, r, n, m, P, st) : launch_lg<10, false>(a, b, r, n, m, P, st);
        case 2048: return d48 ? launch_lg<11, true>(a, b, r, n, m, P, st) : launch_lg<11, false>(a, b, r, n, m, P, st);
        case 4096: return d48 ? launch_lg<12, true>(a, b, r, n, m, P, st) : launch_lg<12, false>(a, b, r, n, m, P, st);
        default: return set_error(MI_EINVAL, "poly_ntt: %u limbs exceeds the maximum %u", m, kNttMaxLimbs);
    }
}

}  // namespace mi
