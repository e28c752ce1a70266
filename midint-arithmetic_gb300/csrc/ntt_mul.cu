// ntt_mul.cu -- exact batched multiplication by number-theoretic transforms.
//
// Counterpart of the reference's bmulFFT / bmulFftReg (cuda/ker-fft-mul.cu.h:
// 375-454, cuda/ker-fft-help.cu.h), which multiplies 16-bit digits with one
// 32-bit prime and is exact only for tiny inputs (its coefficients exceed the
// prime from 16 digits on, and cuda/main.cu:729-739 disables validation).
//
// Here every u64 limb is one digit; the product of two m-limb integers has
// coefficients below m * 2^128 <= 2^139 (m <= 2048), so five primes
// p_i < 2^30 (product 2^149.4) recover every coefficient exactly by CRT; when
// 40-bit digits fit the same transform length (2 ceil(8m/5) <= L, m <= 525)
// the kernel runs them on three primes instead, else when 48-bit digits fit
// (2 ceil(4m/3) <= L) on four (ntt_mul.cuh).  One CTA of L/8 threads
// owns one instance (L = pow2ceil(2m) >= 256): for each prime it converts a
// and b into the field, runs two forward transforms, multiplies pointwise and
// runs the inverse transform (ntt32.cuh), leaving the residues in shared
// memory.  The same CTA then recombines each
// coefficient with Garner's formula, sums the three-word coefficients of its
// 8 output limbs, passes the overflow words to its right neighbour and
// resolves the remaining one-bit carries with mi::group_carry -- the final
// carry that the reference does with splitFftReg + baddRegMul2Fft.
// (ntt_raw below keeps the 64-bit fields of ntt.cuh, so it can run the
// reference's own primes on its known answers.)
#include <cstdio>

#include "common.cuh"
#include "kernels.h"
#include "ntt.cuh"
#include "ntt_host.h"
#include "ntt32.cuh"
#include "ntt_mul.cuh"

namespace mi {
namespace {

using ntt::FieldC32;
using ntt::FieldGen;
using ntt::Plan;

template <int LG>
struct NttShape {
    static constexpr int L = 1 << LG;
    static constexpr int NT = L / 8;
    static constexpr size_t SMEM = ntt32::MulSmem<LG>::WORDS32 * 4 + size_t(NT / 32 + 1) * 4;
};

// 768 threads per SM: three 256-thread CTAs for 2048-point transforms (one
// 512-thread CTA for 4096-point ones)
template <int LG, int NP, bool LOW>
__global__ void __launch_bounds__((1 << LG) / 8, 768 / ((1 << LG) / 8))
    k_ntt_mul(const uint64_t* __restrict__ a, const uint64_t* __restrict__ b, uint64_t* __restrict__ r, uint32_t n,
              uint32_t m, uint32_t rlen, NttMulParams P) {
    extern __shared__ __align__(16) uint32_t smem32[];
    uint32_t* scratch = smem32 + ntt32::MulSmem<LG>::WORDS32;
    for (uint64_t inst = blockIdx.x; inst < n; inst += gridDim.x)
        ntt32::mul_one<LG, 5 - NP, true, LOW>(a + inst * m, m, b + inst * m, m, r + inst * rlen, rlen, P, smem32,
                                              scratch);  // L = pow2ceil(2m): both operands in the lower half
}

template <int LG, int NP>
mi_status launch_lg(const uint64_t* a, const uint64_t* b, uint64_t* r, uint32_t n, uint32_t m, uint32_t rlen,
                    const NttMulParams& P, cudaStream_t st) {
    using S = NttShape<LG>;
    auto kern = rlen <= m ? k_ntt_mul<LG, NP, true> : k_ntt_mul<LG, NP, false>;  // the low half alone
    MI_TRY(ensure_dyn_smem(kern, S::SMEM));
    int per_sm = 0;
    MI_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, S::NT, S::SMEM));
    uint64_t blocks = uint64_t(sm_count()) * (per_sm > 0 ? per_sm : 1);
    if (blocks > n) blocks = n;
    // A plain launch: the grid is persistent with a fixed stride over the
    // instances, and a programmatic dependent launch, whose blocks become
    // resident one by one during the previous launch's tail, put the blocks
    // with one instance more on the same SMs (measured 0.108 ms against
    // 0.0996 ms per 1024 x 65536-bit batch).
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

// --- raw transforms on one of the five production primes ------------------
// The transform code of the multiplication kernels (ntt32.cuh) on its own,
// one block of L/8 threads: conv = 0 the forward transform of `a` (residues
// < p) written in natural order, conv = 1 the cyclic convolution of a and b
// mod p (a as given, b scaled by 2^32 / L with a Shoup product, both forward
// transforms in lockstep, the Montgomery pointwise product, the unscaled
// inverse) -- exactly the per-prime steps of ntt32::mul_one on residues.
template <int LG>
__global__ void __launch_bounds__((1 << LG) / 8)
    k_ntt32_raw(const uint32_t* __restrict__ a, const uint32_t* __restrict__ b, uint32_t* __restrict__ out,
                NttMulParams P, int q, int conv) {
    using Pl = ntt32::Plan<LG>;
    __shared__ __align__(16) uint32_t sh[2 * Pl::LX];
    const uint32_t t = threadIdx.x;
    const ntt32::Field f{P.p[q], 2 * P.p[q], P.pinv[q]};
    if (!conv) {
        uint32_t x[1][8];
#pragma unroll
        for (int j = 0; j < 8; ++j) x[0][j] = a[t + Pl::NT * j];
        ntt32::forward<LG, 1>(x, sh, P.tw[q], f);
        // stride-1 layout: slot 8t+j holds spectrum entry bitrev(8t+j)
#pragma unroll
        for (int j = 0; j < 8; ++j) out[__brev(8 * t + j) >> (32 - LG)] = f.reduce(x[0][j]);
        return;
    }
    const uint2 kb = P.ka_by_lg[q][LG - 8][1];  // 2^32 / L
    uint32_t x[2][8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        x[0][j] = a[t + Pl::NT * j];  // residues < p
        x[1][j] = f.shoup(b[t + Pl::NT * j], kb);
    }
    ntt32::forward<LG, 2>(x, sh, P.tw[q], f);
#pragma unroll
    for (int j = 0; j < 8; ++j) x[0][j] = f.mont(x[0][j], x[1][j]);
    ntt32::inverse<LG>(x[0], sh, P.itw[q], f);
#pragma unroll
    for (int j = 0; j < 8; ++j) out[t + Pl::NT * j] = f.reduce(x[0][j]);
}

}  // namespace

mi_status launch_mul_ntt(const uint64_t* a, const uint64_t* b, uint64_t* r, uint32_t n, uint32_t m,
                         const NttMulParams& base, cudaStream_t st, bool low) {
    const uint32_t rlen = low ? m : 2 * m;
    uint32_t L = pow2ceil(2 * m);
    if (L < 256) L = 256;
    // the digit mode with the fewest primes that fits the same length
    const int np = 5 - ntt32::ntt_mode(m, m, L);
    const NttMulParams& P = base;
#define NP_CASE(LGV)                                                                                  \
    case (1u << LGV):                                                                                 \
        return np == 3 ? launch_lg<LGV, 3>(a, b, r, n, m, rlen, P, st)                                \
                       : (np == 4 ? launch_lg<LGV, 4>(a, b, r, n, m, rlen, P, st)                     \
                                  : launch_lg<LGV, 5>(a, b, r, n, m, rlen, P, st));
    switch (L) {
        NP_CASE(8)
        NP_CASE(9)
        NP_CASE(10)
        NP_CASE(11)
        NP_CASE(12)
        default: return set_error(MI_EINVAL, "ntt: %u limbs exceeds the maximum %u", m, kNttMaxLimbs);
    }
#undef NP_CASE
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

mi_status launch_ntt32_raw(const uint32_t* a, const uint32_t* b, uint32_t* out, uint32_t len, uint32_t prime,
                           int conv, const NttMulParams& P, cudaStream_t st) {
    const int q = int(prime), c = conv ? 1 : 0;
    switch (len) {
        case 256: k_ntt32_raw<8><<<1, 32, 0, st>>>(a, b, out, P, q, c); break;
        case 512: k_ntt32_raw<9><<<1, 64, 0, st>>>(a, b, out, P, q, c); break;
        case 1024: k_ntt32_raw<10><<<1, 128, 0, st>>>(a, b, out, P, q, c); break;
        case 2048: k_ntt32_raw<11><<<1, 256, 0, st>>>(a, b, out, P, q, c); break;
        case 4096: k_ntt32_raw<12><<<1, 512, 0, st>>>(a, b, out, P, q, c); break;
        default: return set_error(MI_EINVAL, "ntt32_raw: length %u not a power of two in [256, 4096]", len);
    }
    MI_CUDA_TRY(cudaGetLastError());
    return MI_OK;
}

}  // namespace mi
