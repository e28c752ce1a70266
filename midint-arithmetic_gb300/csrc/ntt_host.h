// ntt_host.h -- parameters of the NTT kernels and their host-side setup.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/midint.h"

namespace mi {

constexpr uint32_t kNttMaxLimbs = 2048;  // u64 limbs per operand (4096-point transforms)

// The five primes of the multiplication kernels: p < 2^30, 2^21 | p - 1, g a
// primitive root (product 2^149.4 > 2048 * 2^128, the largest coefficient).
struct NttPrime30 {
    uint32_t p;
    uint32_t g;
};
constexpr NttPrime30 kNttPrimes[5] = {
    {1012924417u, 5u}, {1004535809u, 3u}, {998244353u, 3u}, {985661441u, 3u}, {975175681u, 17u},
};

// Kernel parameter block (passed by value).  Constants with a Shoup
// companion are (c, floor(c 2^32 / p)) pairs.
struct NttMulParams {
    uint32_t p[5];
    uint32_t pinv[5];             // -p^-1 mod 2^32
    uint2 ka_by_lg[5][5][2];      // for L = 2^(8+i): (L^-1, 2^32 L^-1) mod p
    uint2 kb[5][2];               // (2^32, 2^64) mod p
    uint2 kb_by_lg[5][5];         // for L = 2^(8+i): 2^64 L^-1 mod p (with ka_by_lg[..][1], b's conversion)
    uint2 garner[10];             // p_k^-1 mod p_i, for i = 1..4, k = 0..i-1
    const uint2* tw[5];           // (w^e, companion), w of order 4096, in ntt32::TwLayout order
    const uint2* itw[5];          // (w^-e, companion), the same layout
};

// Device-resident tables of one context (620 KiB) and the parameter block.
struct NttTables {
    uint2* d_tw = nullptr;
    NttMulParams params{};
};

mi_status ntt_tables_create(NttTables* T);
void ntt_tables_destroy(NttTables* T);

// r = a*b (2m limbs per instance), or its low m limbs when `low`.
mi_status launch_mul_ntt(const uint64_t* a, const uint64_t* b, uint64_t* r, uint32_t n, uint32_t m,
                         const NttMulParams& P, cudaStream_t st, bool low = false);

// One transform or one cyclic convolution on a single prime (device buffers).
struct NttRawArgs {
    const uint64_t* a;
    const uint64_t* b;
    uint64_t* out;
    const uint64_t* tw;
    const uint64_t* itw;
    uint64_t p;
    uint32_t aux;  // c (p = c*2^32+1) or -p^-1 mod 2^32 (generic field)
    uint64_t r2;
    uint64_t linv_r;
    uint32_t len;
    int conv;
    int generic;
};
mi_status launch_ntt_raw(const NttRawArgs& A, cudaStream_t st);

// ((a^2 + b)(b^2 + b) + ab) mod 2^(64m) per instance on the transforms above
// (poly_ntt.cu), m <= kNttMaxLimbs.
mi_status launch_poly_ntt(const uint64_t* a, const uint64_t* b, uint64_t* r, uint32_t n, uint32_t m,
                          const NttMulParams& P, cudaStream_t st);

// One forward transform (conv = 0) or cyclic convolution (conv = 1) of
// length len (256..4096) on production prime `prime` (< 5) by the transform
// code of the multiplication kernels; device buffers of len residues < p.
mi_status launch_ntt32_raw(const uint32_t* a, const uint32_t* b, uint32_t* out, uint32_t len, uint32_t prime,
                           int conv, const NttMulParams& P, cudaStream_t st);

// Host modular arithmetic (exact, 128-bit intermediates).  The raw transform
// path (mi_ntt_raw) keeps 64-bit fields so it can run the reference's own
// primes.
uint64_t host_mulmod(uint64_t a, uint64_t b, uint64_t p);
uint64_t host_powmod(uint64_t a, uint64_t e, uint64_t p);
uint64_t host_invmod(uint64_t a, uint64_t p);  // p prime
// Fills tw/itw (2048 entries each, Montgomery form) for a prime with a
// generator of order 2^s, s >= 12.
void host_twiddles(uint64_t p, uint64_t g, uint32_t s, uint64_t* tw, uint64_t* itw);

}  // namespace mi
