// mul.cu -- batched classical (quadratic) multiplication on 32-bit limbs.
//
// Counterpart of the reference's bmulKerQ (cuda/ker-classic-mul.cu.h:468-498)
// and its helpers computeIter64 / convolutionQ / combineQ / from4Reg2ShmQ /
// bmulRegsQ (:11-26, :299-463).  The reference walks output columns with a
// 128-bit accumulator plus a carry counter, reading both operands from shared
// memory for every 64x64-bit product, and balances the triangle of the low
// half by pairing column k with its mirror M-k.
//
// Here the n32 x n32 grid of 32x32-bit partial products is cut into T x T
// tiles (T = 8 limbs).  With NT = n32/T tiles per side, thread t of a group
// of NT threads owns the two anti-diagonals of tiles s = t and s = t + NT,
// which together hold exactly NT tiles for every t (t+1 below the main
// anti-diagonal, NT-1-t above), so the full product is balanced without
// mirroring.  At step k every thread multiplies A-block k (the same address
// for the whole group: a shared-memory broadcast) by B-block (t-k) mod NT.
//
// One tile is 2*T*T multiply-add instructions with the hardware carry flag
// (mad.lo.cc / madc.hi.cc): for row i, the products A[i]*B[j] with even j
// tile columns i..i+T-1 without overlap, and those with odd j tile columns
// i+1..i+T, so each is one T-long carry chain whose single carry-out goes into
// a per-column counter (one addc).  The counters are folded in once per
// anti-diagonal.  The first anti-diagonal's value is snapshotted to shared
// memory at the step where it completes (one predicated store per step), the
// second is the final accumulator minus the snapshot.  Finally every output
// block of T limbs is L_s + H_(s-1) + O_(s-2) (low, high and overflow words of
// the anti-diagonal accumulators), added with two carry-lookahead passes over
// the group (mi::group_carry) -- the reference's low/high/carry publish and
// baddRegs (cuda/ker-classic-mul.cu.h:299-350, 425-463).
#include <cstdio>

#include "common.cuh"
#include "kernels.h"

namespace mi {
namespace {

constexpr int kT = 8;  // tile side, in 32-bit limbs

// Accumulator of one anti-diagonal of T x T tiles, split by column parity so
// that every (lo, hi) word pair of a partial product lands on an even-aligned
// register pair (which lets the compiler issue mad.lo.cc + madc.hi.cc as one
// wide multiply-add) and each tile row is two independent carry chains:
//   a[c]   column c,   products with i+j even (chains start at even columns)
//   b[k]   column k+1, products with i+j odd
//   cc[c]  carries out of the chains, at column T+c
template <int T>
struct DiagAcc {
    uint32_t a[2 * T];
    uint32_t b[2 * T - 2];
    uint32_t cc[T + 1];
    static constexpr int WORDS = 2 * T + 2 * T - 2 + T + 1;
};

template <int T>
__device__ __forceinline__ void tile_mac(const uint32_t (&A)[T], const uint32_t (&B)[T], DiagAcc<T>& s) {
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
template <int T>
__device__ __forceinline__ void fold(const uint32_t* a, const uint32_t* b, const uint32_t* cc,
                                     uint32_t (&f)[2 * T + 1]) {
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

template <int T, int NT>
struct MulShape {
    static constexpr int BLOCK = NT > 256 ? NT : 256;
    static constexpr int IPB = BLOCK / NT;            // instances per block
    static constexpr int WPAD = NT * T;               // padded limbs per operand
    static constexpr int ACC = 2 * T + 1;             // folded accumulator words
    static constexpr int SNAP = 4 * ((DiagAcc<T>::WORDS + 3) / 4);
    static constexpr int COMB = 2 * ACC;
    static constexpr int PER_T = COMB > SNAP ? COMB : SNAP;
    // operands (2 x IPB x WPAD) + per-thread snapshot/combine slots; the
    // carry resolution's per-warp words reuse the operand area.
    static constexpr size_t SMEM = size_t(2 * IPB * WPAD + BLOCK * PER_T) * 4;
    static_assert(PER_T % 4 == 0, "16-byte slots");
};

template <int T, int NT, bool VEC>
__global__ void __launch_bounds__(NT > 256 ? NT : 256)
    k_mul(const uint32_t* __restrict__ a, const uint32_t* __restrict__ b, uint32_t* __restrict__ r, uint32_t n,
          uint32_t n32, bool full) {
    using S = MulShape<T, NT>;
    constexpr int ACC = S::ACC;
    static_assert(T == 8, "staging and plane layout assume 8-limb tiles");
    extern __shared__ __align__(16) uint32_t smem[];
    uint32_t* sA = smem;
    uint32_t* sB = sA + S::IPB * S::WPAD;
    uint32_t* sT = sB + S::IPB * S::WPAD;
    uint32_t* sScr = sA;  // free once the tile loop is done

    const uint32_t grp = threadIdx.x / NT;
    const uint32_t t = threadIdx.x % NT;
    uint32_t* gA = sA + grp * S::WPAD;
    // B blocks in two planes of 16-byte halves: half q of block j is slot
    // q*NT + j, so a group reading blocks (t-k) mod NT hits consecutive slots.
    uint4* gB4 = reinterpret_cast<uint4*>(sB + grp * S::WPAD);
    uint32_t* mine = sT + threadIdx.x * S::PER_T;
    const uint32_t* gT = sT + grp * NT * S::PER_T;
    const uint32_t rlen = full ? 2 * n32 : n32;
    const uint64_t stride = uint64_t(gridDim.x) * S::IPB;

    for (uint64_t base = uint64_t(blockIdx.x) * S::IPB; base < n; base += stride) {
        const uint64_t inst = base + grp;
        const bool valid = inst < n;
        // 1. stage both operands in shared memory, zero padded to NT*T limbs
        {
            const uint32_t* ra = a + (valid ? inst * n32 : 0);
            const uint32_t* rb = b + (valid ? inst * n32 : 0);
#pragma unroll
            for (int it = 0; it < T / 4; ++it) {
                const uint32_t v = t + uint32_t(it) * NT;  // 16-byte slot of the operand
                uint4 qa = make_uint4(0, 0, 0, 0), qb = qa;
                if (VEC && valid && v * 4 + 4 <= n32) {
                    qa = __ldcs(reinterpret_cast<const uint4*>(ra) + v);
                    qb = __ldcs(reinterpret_cast<const uint4*>(rb) + v);
                } else if (valid) {
                    const uint32_t w = v * 4;
                    if (w + 0 < n32) { qa.x = __ldcs(ra + w + 0); qb.x = __ldcs(rb + w + 0); }
                    if (w + 1 < n32) { qa.y = __ldcs(ra + w + 1); qb.y = __ldcs(rb + w + 1); }
                    if (w + 2 < n32) { qa.z = __ldcs(ra + w + 2); qb.z = __ldcs(rb + w + 2); }
                    if (w + 3 < n32) { qa.w = __ldcs(ra + w + 3); qb.w = __ldcs(rb + w + 3); }
                }
                reinterpret_cast<uint4*>(gA)[v] = qa;
                gB4[(v & 1) * NT + (v >> 1)] = qb;
            }
        }
        __syncthreads();

        // 2. NT tiles per thread: A-block k times B-block (t-k) mod NT
        DiagAcc<T> s;
#pragma unroll
        for (int w = 0; w < 2 * T; ++w) s.a[w] = 0;
#pragma unroll
        for (int w = 0; w < 2 * T - 2; ++w) s.b[w] = 0;
#pragma unroll
        for (int w = 0; w < T + 1; ++w) s.cc[w] = 0;
#pragma unroll 2
        for (uint32_t k = 0; k < uint32_t(NT); ++k) {
            const uint32_t j = (t - k) & uint32_t(NT - 1);
            uint32_t A[T], B[T];
            const uint4 a0 = reinterpret_cast<const uint4*>(gA + k * T)[0];
            const uint4 a1 = reinterpret_cast<const uint4*>(gA + k * T)[1];
            const uint4 b0 = gB4[j];
            const uint4 b1 = gB4[NT + j];
            A[0] = a0.x; A[1] = a0.y; A[2] = a0.z; A[3] = a0.w;
            A[4] = a1.x; A[5] = a1.y; A[6] = a1.z; A[7] = a1.w;
            B[0] = b0.x; B[1] = b0.y; B[2] = b0.z; B[3] = b0.w;
            B[4] = b1.x; B[5] = b1.y; B[6] = b1.z; B[7] = b1.w;
            tile_mac<T>(A, B, s);
            if (k == t) {
                // anti-diagonal t is complete: snapshot the accumulator
                uint32_t tmp[S::SNAP];
#pragma unroll
                for (int w = 0; w < 2 * T; ++w) tmp[w] = s.a[w];
#pragma unroll
                for (int w = 0; w < 2 * T - 2; ++w) tmp[2 * T + w] = s.b[w];
#pragma unroll
                for (int w = 0; w < T + 1; ++w) tmp[4 * T - 2 + w] = s.cc[w];
#pragma unroll
                for (int w = DiagAcc<T>::WORDS; w < S::SNAP; ++w) tmp[w] = 0;
#pragma unroll
                for (int q = 0; q < S::SNAP / 4; ++q)
                    reinterpret_cast<uint4*>(mine)[q] = make_uint4(tmp[4 * q], tmp[4 * q + 1], tmp[4 * q + 2], tmp[4 * q + 3]);
            }
        }

        // 3. split into the two anti-diagonal values D1 (s=t) and D2 (s=t+NT)
        uint32_t d1[ACC], d2[ACC];
        {
            uint32_t snap[S::SNAP];
#pragma unroll
            for (int q = 0; q < S::SNAP / 4; ++q) {
                const uint4 v = reinterpret_cast<const uint4*>(mine)[q];
                snap[4 * q] = v.x; snap[4 * q + 1] = v.y; snap[4 * q + 2] = v.z; snap[4 * q + 3] = v.w;
            }
            fold<T>(snap, snap + 2 * T, snap + 4 * T - 2, d1);
            fold<T>(s.a, s.b, s.cc, d2);
            sub_cc(d2[0], d1[0]);
#pragma unroll
            for (int w = 1; w < ACC - 1; ++w) subc_cc(d2[w], d1[w]);
            subc(d2[ACC - 1], d1[ACC - 1]);
#pragma unroll
            for (int w = 0; w < ACC; ++w) {
                mine[w] = d1[w];
                mine[ACC + w] = d2[w];
            }
        }
        __syncthreads();

        // 4. output blocks s=t (lo) and s=t+NT (hi): L_s + H_(s-1) + O_(s-2)
        auto peer = [&](uint32_t lane, int which, int w) -> uint32_t {
            return gT[lane * S::PER_T + which * ACC + w];
        };
        uint32_t Hlo[T], Hhi[T], Olo = 0, Ohi = 0;
#pragma unroll
        for (int w = 0; w < T; ++w) {
            Hlo[w] = (t >= 1) ? peer(t - 1, 0, T + w) : 0u;
            Hhi[w] = (t >= 1) ? peer(t - 1, 1, T + w) : peer(NT - 1, 0, T + w);
        }
        if (t >= 2) {
            Olo = peer(t - 2, 0, 2 * T);
            Ohi = peer(t - 2, 1, 2 * T);
        } else if (NT >= 2) {
            Ohi = (t == 1) ? peer(NT - 1, 0, 2 * T) : peer(NT - 2, 0, 2 * T);
        }
        uint32_t Llo[T], Lhi[T];
#pragma unroll
        for (int w = 0; w < T; ++w) {
            Llo[w] = d1[w];
            Lhi[w] = d2[w];
        }
        uint32_t ulo[T], uhi[T];
        {
            bool g0, p0, g1, p1;
            uint32_t c0, c1;
            chunk_add<uint32_t, T>(Llo, Hlo, ulo, g0, p0);
            chunk_add<uint32_t, T>(Lhi, Hhi, uhi, g1, p1);
            const uint32_t cl = group_carry<NT>(g0, p0, 0u, &c0, sScr);
            const uint32_t ch = group_carry<NT>(g1, p1, c0, &c1, sScr);
            chunk_inc<uint32_t, T>(ulo, cl);
            chunk_inc<uint32_t, T>(uhi, ch);
        }
        {
            uint32_t Zlo[T], Zhi[T];
#pragma unroll
            for (int w = 0; w < T; ++w) { Zlo[w] = 0; Zhi[w] = 0; }
            Zlo[0] = Olo;
            Zhi[0] = Ohi;
            uint32_t vlo[T], vhi[T];
            bool g0, p0, g1, p1;
            uint32_t c0, c1;
            chunk_add<uint32_t, T>(ulo, Zlo, vlo, g0, p0);
            chunk_add<uint32_t, T>(uhi, Zhi, vhi, g1, p1);
            const uint32_t cl = group_carry<NT>(g0, p0, 0u, &c0, sScr);
            const uint32_t ch = group_carry<NT>(g1, p1, c0, &c1, sScr);
            chunk_inc<uint32_t, T>(vlo, cl);
            chunk_inc<uint32_t, T>(vhi, ch);
#pragma unroll
            for (int w = 0; w < T; ++w) { ulo[w] = vlo[w]; uhi[w] = vhi[w]; }
        }

        // 5. store (only limbs inside the result row)
        if (valid) {
            uint32_t* rr = r + inst * rlen;
            const uint32_t o0 = t * T;
            if (VEC && o0 + T <= rlen) {
#pragma unroll
                for (int q = 0; q < T / 4; ++q)
                    __stcs(reinterpret_cast<uint4*>(rr + o0) + q,
                           make_uint4(ulo[4 * q], ulo[4 * q + 1], ulo[4 * q + 2], ulo[4 * q + 3]));
            } else {
#pragma unroll
                for (int w = 0; w < T; ++w)
                    if (o0 + w < rlen) __stcs(rr + o0 + w, ulo[w]);
            }
            if (full) {
                const uint32_t o1 = (t + NT) * T;
                if (VEC && o1 + T <= rlen) {
#pragma unroll
                    for (int q = 0; q < T / 4; ++q)
                        __stcs(reinterpret_cast<uint4*>(rr + o1) + q,
                               make_uint4(uhi[4 * q], uhi[4 * q + 1], uhi[4 * q + 2], uhi[4 * q + 3]));
                } else {
#pragma unroll
                    for (int w = 0; w < T; ++w)
                        if (o1 + w < rlen) __stcs(rr + o1 + w, uhi[w]);
                }
            }
        }
        __syncthreads();  // shared memory is reused by the next instance
    }
}

template <int NT, bool VEC>
mi_status launch_nt(const uint32_t* a, const uint32_t* b, uint32_t* r, uint32_t n, uint32_t n32, bool full,
                    cudaStream_t st) {
    using S = MulShape<kT, NT>;
    auto kern = k_mul<kT, NT, VEC>;
    static bool attr_done[64] = {};
    int dev = 0;
    MI_CUDA_TRY(cudaGetDevice(&dev));
    if (dev >= 0 && dev < 64 && !attr_done[dev]) {
        MI_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(S::SMEM)));
        attr_done[dev] = true;
    }
    uint64_t blocks = (uint64_t(n) + S::IPB - 1) / S::IPB;
    const uint64_t cap = uint64_t(sm_count()) * 32;
    if (blocks > cap) blocks = cap;
    kern<<<dim3(uint32_t(blocks)), dim3(S::BLOCK), S::SMEM, st>>>(a, b, r, n, n32, full);
    MI_CUDA_TRY(cudaGetLastError());
    return MI_OK;
}

template <bool VEC>
mi_status dispatch(const uint32_t* a, const uint32_t* b, uint32_t* r, uint32_t n, uint32_t n32, bool full,
                   cudaStream_t st) {
    const uint32_t nt = pow2ceil((n32 + kT - 1) / kT);
    switch (nt) {
        case 1: return launch_nt<1, VEC>(a, b, r, n, n32, full, st);
        case 2: return launch_nt<2, VEC>(a, b, r, n, n32, full, st);
        case 4: return launch_nt<4, VEC>(a, b, r, n, n32, full, st);
        case 8: return launch_nt<8, VEC>(a, b, r, n, n32, full, st);
        case 16: return launch_nt<16, VEC>(a, b, r, n, n32, full, st);
        case 32: return launch_nt<32, VEC>(a, b, r, n, n32, full, st);
        case 64: return launch_nt<64, VEC>(a, b, r, n, n32, full, st);
        case 128: return launch_nt<128, VEC>(a, b, r, n, n32, full, st);
        case 256: return launch_nt<256, VEC>(a, b, r, n, n32, full, st);
        default: return set_error(MI_EINVAL, "mul: %u u32 limbs exceeds the classical maximum", n32);
    }
}

}  // namespace

mi_status launch_mul_classic(const uint32_t* a, const uint32_t* b, uint32_t* r, uint32_t n, uint32_t n32, bool full,
                             cudaStream_t st) {
    const bool vec = aligned16(a) && aligned16(b) && aligned16(r) && (n32 % 4 == 0);
    return vec ? dispatch<true>(a, b, r, n, n32, full, st) : dispatch<false>(a, b, r, n, n32, full, st);
}

}  // namespace mi
