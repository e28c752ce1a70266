// ref_driver.cpp -- C entry points around the reference's own CPU path,
// compiled from its sources where they lie (cuda/helper.h is included from the
// reference tree by oracle/build_ref.py).  Test infrastructure: it validates
// the oracle restatement and generates the committed golden fixtures.
//
//   ref_gmp_add_mul  the reference's gmpAdd / gmpMultiply loops
//                    (cuda/main.cu:165-175, 358-368) over its gmpAddMulOnce<m>
//                    (cuda/helper.h:146-170): output truncated to m u32 words.
//   ref_mk_random    its input generator ourMkRandom<m, nz> (cuda/helper.h:99-114),
//                    glibc rand() after ref_srand(seed).
#include <cuda_runtime_api.h>
#include <stdint.h>
#include "helper.h"

template <uint32_t m>
static void loop(bool is_add, uint32_t n, uint32_t* as, uint32_t* bs, uint32_t* rs) {
    for (uint32_t i = 0; i < n; ++i) gmpAddMulOnce<m>(is_add, as + (size_t)i * m, bs + (size_t)i * m, rs + (size_t)i * m);
}

template <int m>
static void mk(uint32_t nz, uint32_t n, uint32_t* as) {
    if (nz == (uint32_t)m) ourMkRandom<m, m>(n, as);
    else ourMkRandom<m, m / 2>(n, as);
}

#define SIZES(X) X(2) X(4) X(8) X(16) X(32) X(64) X(128) X(256) X(512) X(1024) X(2048) X(4096) X(8192)

extern "C" int ref_gmp_add_mul(int is_add, uint32_t m, uint32_t n, uint32_t* as, uint32_t* bs, uint32_t* rs) {
    switch (m) {
#define CASE(M) case M: loop<M>(is_add != 0, n, as, bs, rs); return 0;
        SIZES(CASE)
#undef CASE
        default: return -1;
    }
}

extern "C" int ref_mk_random(uint32_t m, uint32_t nz, uint32_t n, uint32_t* as) {
    if (nz != m && nz != m / 2) return -2;
    switch (m) {
#define CASE(M) case M: mk<M>(nz, n, as); return 0;
        SIZES(CASE)
#undef CASE
        default: return -1;
    }
}

extern "C" void ref_srand(unsigned seed) { srand(seed); }
