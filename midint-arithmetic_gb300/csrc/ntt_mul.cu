// ntt_mul.cu -- exact batched multiplication by number-theoretic transforms.
//
// Counterpart of the reference's bmulFFT / bmulFftReg (cuda/ker-fft-mul.cu.h:
// 375-454, cuda/ker-fft-help.cu.h), which multiplies 16-bit digits with one
// 32-bit prime and is exact only for tiny inputs (its coefficients exceed the
// prime from 16 digits on, and cuda/main.cu:729-739 disables validation).
//
// Here every u64 limb is one digit; the product of two m-limb integers has
// coefficients below m * 2^128 <= 2^138 (m <= 1024), so three primes
// q0 < q1 < q2 < 2^62 (product 2^186) recover every coefficient exactly by
// CRT.  One CTA of L/8 threads owns one instance (L = pow2ceil(2m) >= 256):
// for each prime it converts a and b into the field (a scaled by 1/L, so the
// inverse transform needs no scaling pass), runs two forward transforms,
// multiplies pointwise and runs the inverse transform (ntt.cuh), leaving the
// residues in shared memory.  The same CTA then recombines each coefficient
// with Garner's formula, sums the three-word coefficients of its 8 output
// limbs, passes the overflow words to its right neighbour and resolves the
// remaining one-bit carries with mi::group_carry -- the final carry that the
// reference does with splitFftReg + baddRegMul2Fft.
#include <cstdio>

#include "common.cuh"
#include "kernels.h"
#include "ntt.cuh"
#include "ntt_host.h"

namespace mi {
namespace {

using ntt::FieldC32;
using ntt::FieldGen;
using ntt::Plan;

template <int LG>
struct NttShape {
    static constexpr int L = 1 << LG;
    static constexpr int NT = L / 8;
    // exchange buffer (L) + three residue arrays (3L), u64 each; the carry
    // pass reuses the exchange buffer for the overflow words.
    static constexpr size_t SMEM = size_t(4 * L) * 8 + size_t(NT / 32 + 1) * 4;
};

template <int LG>
__global__ void __launch_bounds__((1 << LG) / 8)
    k_ntt_mul(const uint64_t* __restrict__ a, const uint64_t* __restrict__ b, uint64_t* __restrict__ r, uint32_t n,
              uint32_t m, uint32_t rlen, NttMulParams P) {
    using Pl = Plan<LG>;
    using S = NttShape<LG>;
    extern __shared__ __align__(16) uint64_t smem[];
    uint64_t* sh = smem;
    uint64_t* res = smem + Pl::L;  // res[q][slot], q < 3
    uint32_t* scratch = reinterpret_cast<uint32_t*>(smem + 4 * Pl::L);
    const uint32_t t = threadIdx.x;

    for (uint64_t inst = blockIdx.x; inst < n; inst += gridDim.x) {
        const uint64_t* ar = a + inst * m;
        const uint64_t* br = b + inst * m;
#pragma unroll 1
        for (int q = 0; q < 3; ++q) {
            const FieldC32 f{P.p[q], 2 * P.p[q], P.c[q]};
            uint64_t x[8], y[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const uint32_t i = t + Pl::NT * j;
                // a*(R/L)/R = a/L and b*R^2/R = b*R: the pointwise product is
                // then a*b/L in plain form and the inverse needs no scaling.
                x[j] = (i < m) ? f.mul(__ldg(ar + i), P.ka[q]) : 0;
                y[j] = (i < m) ? f.mul(__ldg(br + i), P.kb[q]) : 0;
            }
            ntt::forward<LG>(x, sh, P.tw[q], f);
            ntt::forward<LG>(y, sh, P.tw[q], f);
#pragma unroll
            for (int j = 0; j < 8; ++j) x[j] = f.mul(x[j], y[j]);
            ntt::inverse<LG>(x, sh, P.itw[q], f);
#pragma unroll
            for (int j = 0; j < 8; ++j) res[q * Pl::L + ntt::swz(t + Pl::NT * j)] = ntt::reduce1(x[j], f.p);
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
            const uint32_t slot = ntt::swz(8 * t + j);
            const ulonglong2 r0 = *reinterpret_cast<const ulonglong2*>(res + slot);
            const ulonglong2 r1 = *reinterpret_cast<const ulonglong2*>(res + Pl::L + slot);
            const ulonglong2 r2 = *reinterpret_cast<const ulonglong2*>(res + 2 * Pl::L + slot);
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const uint64_t v0 = h ? r0.y : r0.x, v1 = h ? r1.y : r1.x, v2 = h ? r2.y : r2.x;
                const uint64_t y1 = ntt::reduce1(f1.mul(v1 + f1.p - v0, P.g01), f1.p);
                const uint64_t u = ntt::reduce1(f2.mul(v2 + f2.p - v0, P.g02), f2.p);
                const uint64_t y2 = ntt::reduce1(f2.mul(u + f2.p - y1, P.g12), f2.p);
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
        const uint32_t cin = group_carry<Pl::NT>(g, p, 0u, &gc, scratch);
        chunk_inc<uint64_t, 8>(blk, cin);
        uint64_t* rr = r + inst * rlen;  // rlen = 2m (full product) or m (low half)
        const uint32_t o0 = 8 * t;
        if (o0 + 8 <= rlen && (rlen & 1) == 0) {
#pragma unroll
            for (int w = 0; w < 8; w += 2)
                __stcs(reinterpret_cast<ulonglong2*>(rr + o0 + w), make_ulonglong2(blk[w], blk[w + 1]));
        } else {
#pragma unroll
            for (int w = 0; w < 8; ++w)
                if (o0 + w < rlen) rr[o0 + w] = blk[w];
        }
        __syncthreads();  // sh and res are reused by the next instance
    }
}

template <int LG>
mi_status launch_lg(const uint64_t* a, const uint64_t* b, uint64_t* r, uint32_t n, uint32_t m, uint32_t rlen,
                    const NttMulParams& P, cudaStream_t st) {
    using S = NttShape<LG>;
    auto kern = k_ntt_mul<LG>;
    static bool attr_done[64] = {};
    int dev = 0;
    MI_CUDA_TRY(cudaGetDevice(&dev));
    if (dev >= 0 && dev < 64 && !attr_done[dev]) {
        MI_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(S::SMEM)));
        attr_done[dev] = true;
    }
    int per_sm = 0;
    MI_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, S::NT, S::SMEM));
    uint64_t blocks = uint64_t(sm_count()) * (per_sm > 0 ? per_sm : 1);
    if (blocks > n) blocks = n;
    kern<<<dim3(uint32_t(blocks)), dim3(S::NT), S::SMEM, st>>>(a, b, r, n, m, rlen, P);
    MI_CUDA_TRY(cudaGetLastError());
    return MI_OK;
}

// --- raw transforms on one prime: the reference's NTT known answers --------

template <int LG, typename F>
__global__ void k_ntt_raw(const uint64_t* __restrict__ a, const uint64_t* __restrict__ b, uint64_t* __restrict__ out,
                          const uint64_t* __restrict__ tw, const uint64_t* __restrict__ itw, F f, uint64_t r2,
                          uint64_t linv_r, int conv) {
    using Pl = Plan<LG>;
    __shared__ __align__(16) uint64_t sh[Pl::L];
    const uint32_t t = threadIdx.x;
    uint64_t x[8], y[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const uint32_t i = t + Pl::NT * j;
        x[j] = f.mul(a[i], r2);  // to Montgomery form
        y[j] = conv ? f.mul(b[i], r2) : 0;
    }
    ntt::forward<LG>(x, sh, tw, f);
    if (!conv) {
        // stride-1 layout holds the bit-reversed spectrum: undo both
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const uint32_t slot = 8 * t + j;
            uint32_t rev = 0;
            for (int k = 0; k < LG; ++k) rev |= ((slot >> k) & 1u) << (LG - 1 - k);
            out[rev] = ntt::reduce1(f.mul(x[j], 1), f.p);
        }
        return;
    }
    ntt::forward<LG>(y, sh, tw, f);
#pragma unroll
    for (int j = 0; j < 8; ++j) x[j] = f.mul(f.mul(x[j], y[j]), linv_r);
    ntt::inverse<LG>(x, sh, itw, f);
#pragma unroll
    for (int j = 0; j < 8; ++j) out[t + Pl::NT * j] = ntt::reduce1(f.mul(x[j], 1), f.p);
}

}  // namespace

mi_status launch_mul_ntt(const uint64_t* a, const uint64_t* b, uint64_t* r, uint32_t n, uint32_t m,
                         const NttMulParams& base, cudaStream_t st, bool low) {
    const uint32_t rlen = low ? m : 2 * m;
    uint32_t L = pow2ceil(2 * m);
    if (L < 256) L = 256;
    NttMulParams P = base;
    for (int q = 0; q < 3; ++q) P.ka[q] = base.ka_by_lg[q][__builtin_ctz(L)];
    switch (L) {
        case 256: return launch_lg<8>(a, b, r, n, m, rlen, P, st);
        case 512: return launch_lg<9>(a, b, r, n, m, rlen, P, st);
        case 1024: return launch_lg<10>(a, b, r, n, m, rlen, P, st);
        case 2048: return launch_lg<11>(a, b, r, n, m, rlen, P, st);
        default: return set_error(MI_EINVAL, "ntt: %u limbs exceeds the maximum %u", m, kNttMaxLimbs);
    }
}

mi_status launch_ntt_raw(const NttRawArgs& A, cudaStream_t st) {
    const uint32_t L = A.len;
    const uint32_t nt = L / 8;
#define RAW_CASE(LGV)                                                                                          \
    case (1u << LGV):                                                                                          \
        if (A.generic)                                                                                         \
            k_ntt_raw<LGV, FieldGen><<<1, nt, 0, st>>>(A.a, A.b, A.out, A.tw, A.itw,                           \
                                                      FieldGen{A.p, 2 * A.p, A.aux}, A.r2, A.linv_r, A.conv); \
        else                                                                                                   \
            k_ntt_raw<LGV, FieldC32><<<1, nt, 0, st>>>(A.a, A.b, A.out, A.tw, A.itw,                           \
                                                      FieldC32{A.p, 2 * A.p, A.aux}, A.r2, A.linv_r, A.conv); \
        break;
    switch (L) {
        RAW_CASE(3)
        RAW_CASE(4)
        RAW_CASE(5)
        RAW_CASE(6)
        RAW_CASE(7)
        RAW_CASE(8)
        RAW_CASE(9)
        RAW_CASE(10)
        RAW_CASE(11)
        default: return set_error(MI_EINVAL, "ntt_raw: length %u not a power of two in [8, 2048]", L);
    }
#undef RAW_CASE
    MI_CUDA_TRY(cudaGetLastError());
    return MI_OK;
}

}  // namespace mi
