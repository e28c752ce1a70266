// ntt_host.h -- parameters of the NTT kernels and their host-side setup.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/midint.h"

namespace mi {

constexpr uint32_t kNttMaxLimbs = 2048;  // u64 limbs per operand (4096-point transforms)

// One NTT prime: p = c*2^32 + 1 < 2^62, g of multiplicative order exactly 2^s
// (the reference's FftPrime convention, cuda/ker-fft-mul.cu.h:44-72).
struct NttPrime {
    uint64_t p;
    uint64_t g;
    uint32_t s;
};

// q0 < q1 < q2.  q0 is the reference's FftPrime64 (29*2^57+1, g = 21, s = 57).
constexpr NttPrime kNttPrimes[3] = {
    {4179340454199820289ull, 21ull, 57},
    {4611685692009873409ull, 3173265456634446468ull, 34},
    {4611685941117976577ull, 391383840822949112ull, 33},
};

// Kernel parameter block (passed by value).
struct NttMulParams {
    uint64_t p[3];
    uint32_t c[3];
    uint64_t ka[3];            // R/L mod p for the launch's transform length
    uint64_t kb[3];            // R^2 mod p
    uint64_t ka_by_lg[3][13];  // R/2^lg mod p, lg <= 12
    const uint64_t* tw[3];     // w^e R mod p, e < 2048
    const uint64_t* itw[3];    // w^-e R mod p
    uint64_t g01, g02, g12;    // Garner constants q0^-1 mod q1, q0^-1 mod q2, q1^-1 mod q2 (times R)
    uint64_t q01_lo, q01_hi;   // q0*q1
};

// Device-resident tables of one context (96 KiB) and the parameter block.
struct NttTables {
    uint64_t* d_tw = nullptr;
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

// Host modular arithmetic (exact, 128-bit intermediates).
uint64_t host_mulmod(uint64_t a, uint64_t b, uint64_t p);
uint64_t host_powmod(uint64_t a, uint64_t e, uint64_t p);
uint64_t host_invmod(uint64_t a, uint64_t p);  // p prime
// Fills tw/itw (2048 entries each, Montgomery form) for a prime with a
// generator of order 2^s, s >= 12.
void host_twiddles(uint64_t p, uint64_t g, uint32_t s, uint64_t* tw, uint64_t* itw);

}  // namespace mi
