// compat_main.cpp -- the reference's driver calls, unchanged in shape, compiled
// against include/midint_compat.hpp.  Mirrors the test layer of the
// reference's benchmark (testAddition / testNsqMul / testFftMul): it fills
// operands, calls gpuAdd<Base,m>, gpuMultiply<Base,m> and
// gpuMulFFT<FftPrime32,M> and writes inputs and outputs to a binary file that
// the Python test checks against the oracle.
//
// usage: compat_main <out.bin>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "midint_compat.hpp"

using namespace midint_compat;

static uint64_t state = 0x243F6A8885A308D3ull;
static uint64_t next() {  // splitmix64
    uint64_t z = (state += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

template <class T>
static void put(FILE* f, const std::vector<T>& v) {
    const uint64_t n = v.size() * sizeof(T);
    fwrite(&n, 8, 1, f);
    fwrite(v.data(), 1, n, f);
}

int main(int argc, char** argv) {
    if (argc != 2) {
        fprintf(stderr, "usage: %s <out.bin>\n", argv[0]);
        return 2;
    }
    FILE* f = fopen(argv[1], "wb");
    if (!f) return 2;
    const int n = 37;
    int failures = 0;

    {  // gpuAdd<U64bits, 64>: 4096-bit sums
        constexpr uint32_t m = 64;
        std::vector<uint64_t> a(n * m), b(n * m), r(n * m);
        for (auto& x : a) x = next();
        for (auto& x : b) x = next();
        for (uint32_t k = 0; k < m; ++k) { a[k] = ~0ull; b[k] = k == 0; }  // worst-case carry chain
        failures += gpuAdd<U64bits, m>(n, a.data(), b.data(), r.data()) != MI_OK;
        put(f, a); put(f, b); put(f, r);
    }
    {  // gpuAdd<U32bits, 129>
        constexpr uint32_t m = 129;
        std::vector<uint32_t> a(n * m), b(n * m), r(n * m);
        for (auto& x : a) x = uint32_t(next());
        for (auto& x : b) x = uint32_t(next());
        failures += gpuAdd<U32bits, m>(n, a.data(), b.data(), r.data()) != MI_OK;
        put(f, a); put(f, b); put(f, r);
    }
    {  // gpuMultiply<U64bits, 128>: low 128 limbs of 8192-bit products
        constexpr int m = 128;
        std::vector<uint64_t> a(n * m), b(n * m), r(n * m);
        for (auto& x : a) x = next();
        for (auto& x : b) x = next();
        failures += gpuMultiply<U64bits, m>(n, a.data(), b.data(), r.data()) != MI_OK;
        put(f, a); put(f, b); put(f, r);
    }
    {  // gpuMulFFT<FftPrime32, 512>: 512 16-bit digits, low 512 digits of the product
        constexpr uint32_t M = 512;
        std::vector<uint16_t> a(n * M), b(n * M);
        std::vector<uint32_t> r(n * M, 0);
        for (auto& x : a) x = uint16_t(next());
        for (auto& x : b) x = uint16_t(next());
        failures += gpuMulFFT<FftPrime32, M>(n, reinterpret_cast<unsigned short*>(a.data()),
                                             reinterpret_cast<unsigned short*>(b.data()), r.data()) != MI_OK;
        put(f, a); put(f, b); put(f, r);
    }
    fclose(f);
    if (failures) fprintf(stderr, "%d driver call(s) failed: %s\n", failures, mi_last_error());
    return failures ? 1 : 0;
}
