// ntt_host.cu -- host setup of the NTT kernels: constants of the five primes,
// the resident twiddle tables of a context, and the raw single-prime
// transform entry point used to check the transform against the reference's
// known answers.
//
// The reference rebuilds and copies its twiddle tables on every driver call
// (getOmega / mkOmegas, cuda/ker-fft-mul.cu.h:191-211; cuda/main.cu:458-470);
// here they are built once per context and stay in device memory: for each of
// the five 30-bit primes of the multiplication kernels, the powers of w and of
// w^-1 (w = g^((p-1)/4096), the getOmega convention) with their Shoup
// companions, laid out per transform length in the order the passes read
// them (ntt32::TwLayout; 620 KiB per context).
#include <cstring>
#include <vector>

#include "common.cuh"
#include "ctx.h"
#include "kernels.h"
#include "ntt.cuh"
#include "ntt32.cuh"
#include "ntt_host.h"

namespace mi {

using u128 = unsigned __int128;

uint64_t host_mulmod(uint64_t a, uint64_t b, uint64_t p) { return uint64_t((u128)a * b % p); }

uint64_t host_powmod(uint64_t a, uint64_t e, uint64_t p) {
    uint64_t r = 1 % p, x = a % p;
    while (e) {
        if (e & 1) r = host_mulmod(r, x, p);
        x = host_mulmod(x, x, p);
        e >>= 1;
    }
    return r;
}

uint64_t host_invmod(uint64_t a, uint64_t p) { return host_powmod(a, p - 2, p); }

static uint64_t r_mod(uint64_t p) { return uint64_t(((u128)1 << 64) % p); }

void host_twiddles(uint64_t p, uint64_t g, uint32_t s, uint64_t* tw, uint64_t* itw) {
    const uint64_t w = host_powmod(g, uint64_t(1) << (s - ntt::kLgMax), p);  // order 2^kLgMax
    const uint64_t wi = host_invmod(w, p);
    const uint64_t R = r_mod(p);
    uint64_t acc = R, acci = R;  // w^0 * R
    for (int e = 0; e < ntt::kTwiddles; ++e) {
        tw[e] = acc;
        itw[e] = acci;
        acc = host_mulmod(acc, w, p);
        acci = host_mulmod(acci, wi, p);
    }
}

static uint2 shoup_pair(uint64_t c, uint32_t p) {
    c %= p;
    return make_uint2(uint32_t(c), uint32_t((c << 32) / p));
}

mi_status ntt_tables_create(NttTables* T) {
    using ntt32::TwLayout;
    constexpr int E = ntt32::kTwEntries;
    std::vector<uint2> h(size_t(10) * E, make_uint2(0, 0));
    std::vector<uint64_t> pw(ntt32::kTwiddles), ipw(ntt32::kTwiddles);
    NttMulParams& P = T->params;
    std::memset(&P, 0, sizeof(P));
    for (int q = 0; q < 5; ++q) {
        const uint32_t p = kNttPrimes[q].p;
        const uint64_t w = host_powmod(kNttPrimes[q].g, (uint64_t(p) - 1) >> ntt32::kLgMax, p);  // order 4096
        const uint64_t wi = host_invmod(w, p);
        uint64_t acc = 1, acci = 1;
        for (int e = 0; e < ntt32::kTwiddles; ++e) {
            pw[e] = acc;
            ipw[e] = acci;
            acc = host_mulmod(acc, w, p);
            acci = host_mulmod(acci, wi, p);
        }
        // every transform length's sections, in the order its passes read them
        for (int dir = 0; dir < 2; ++dir) {
            uint2* out = h.data() + size_t(2 * q + dir) * E;
            const std::vector<uint64_t>& pows = dir ? ipw : pw;
            for (int lg = ntt32::kLgMin; lg <= ntt32::kLgMax; ++lg) {
                uint2* sec = out + TwLayout::base(lg);
                for (int k = 0; k < TwLayout::nf(lg); ++k) {
                    const int d = TwLayout::d(lg, k), m = (1 << ntt32::kLgMax) / (8 * d);
                    uint2* ps = sec + TwLayout::pass(lg, k);
                    for (int i = 0; i < 4 * d; ++i) ps[i] = shoup_pair(pows[size_t(i) * m], p);
                    for (int i = 0; i < 2 * d; ++i) ps[4 * d + i] = shoup_pair(pows[size_t(2 * i) * m], p);
                    for (int i = 0; i < d; ++i) ps[6 * d + i] = shoup_pair(pows[size_t(4 * i) * m], p);
                }
                sec[TwLayout::quarter(lg)] = shoup_pair(pows[1024], p);
            }
        }
        P.p[q] = p;
        uint32_t inv = 1;  // p^-1 mod 2^32 by Newton iteration
        for (int i = 0; i < 5; ++i) inv *= 2 - p * inv;
        P.pinv[q] = 0u - inv;
        const uint64_t r32 = (uint64_t(1) << 32) % p, r64 = host_mulmod(r32, r32, p);
        for (int lg = 8; lg <= ntt32::kLgMax; ++lg) {
            const uint64_t li = host_invmod(uint64_t(1) << lg, p);
            P.ka_by_lg[q][lg - 8][0] = shoup_pair(li, p);
            P.ka_by_lg[q][lg - 8][1] = shoup_pair(host_mulmod(li, r32, p), p);
            P.kb_by_lg[q][lg - 8] = shoup_pair(host_mulmod(li, r64, p), p);
        }
        P.kb[q][0] = shoup_pair(r32, p);
        P.kb[q][1] = shoup_pair(r64, p);
    }
    int c = 0;
    for (int i = 1; i < 5; ++i)
        for (int k = 0; k < i; ++k)
            P.garner[c++] = shoup_pair(host_invmod(kNttPrimes[k].p % kNttPrimes[i].p, kNttPrimes[i].p), kNttPrimes[i].p);
    MI_CUDA_TRY(cudaMalloc(&T->d_tw, h.size() * sizeof(uint2)));
    MI_CUDA_TRY(cudaMemcpy(T->d_tw, h.data(), h.size() * sizeof(uint2), cudaMemcpyHostToDevice));
    for (int q = 0; q < 5; ++q) {
        P.tw[q] = T->d_tw + size_t(2 * q) * E;
        P.itw[q] = T->d_tw + size_t(2 * q + 1) * E;
    }
    static_assert(ntt32::kTwEntries == 7936, "twiddle sections of 256..4096-point transforms");
    return MI_OK;
}

void ntt_tables_destroy(NttTables* T) {
    if (T->d_tw) cudaFree(T->d_tw);
    T->d_tw = nullptr;
}

}  // namespace mi

using namespace mi;

extern "C" mi_status mi_ntt_raw(uint64_t p, uint64_t g, uint32_t two_adicity, uint32_t len, int conv,
                                const uint64_t* h_a, const uint64_t* h_b, uint64_t* h_out) {
    if (h_a == nullptr || h_out == nullptr || (conv && h_b == nullptr)) return set_error(MI_EINVAL, "ntt_raw: null");
    if (len < 8 || len > 2048 || (len & (len - 1))) return set_error(MI_EINVAL, "ntt_raw: bad length %u", len);
    if ((p & 1) == 0 || p >= (uint64_t(1) << 62) || two_adicity < uint32_t(ntt::kLgMax) || two_adicity > 63)
        return set_error(MI_EINVAL, "ntt_raw: prime must be odd, < 2^62, with 2-adicity >= %d", ntt::kLgMax);
    constexpr int E = ntt::kTwiddles;
    std::vector<uint64_t> tw(2 * E);
    host_twiddles(p, g, two_adicity, tw.data(), tw.data() + E);
    NttRawArgs A{};
    A.p = p;
    A.len = len;
    A.conv = conv;
    A.generic = (p & 0xffffffffull) != 1;
    if (A.generic) {
        uint32_t inv = 1;  // p^-1 mod 2^32 by Newton iteration
        for (int i = 0; i < 5; ++i) inv *= 2 - uint32_t(p) * inv;
        A.aux = uint32_t(0u - inv);
    } else {
        A.aux = uint32_t(p >> 32);
    }
    const uint64_t R = uint64_t(((unsigned __int128)1 << 64) % p);
    A.r2 = host_mulmod(R, R, p);
    A.linv_r = host_mulmod(host_invmod(len, p), R, p);
    uint64_t* d = nullptr;
    MI_CUDA_TRY(cudaMalloc(&d, sizeof(uint64_t) * (2 * E + 3 * size_t(len))));
    mi_status st = MI_OK;
    uint64_t* da = d + 2 * E;
    uint64_t* db = da + len;
    uint64_t* dout = db + len;
    std::vector<uint64_t> ha(len), hb(len, 0);
    for (uint32_t i = 0; i < len; ++i) ha[i] = h_a[i] % p;
    if (conv)
        for (uint32_t i = 0; i < len; ++i) hb[i] = h_b[i] % p;
    cudaError_t e = cudaMemcpy(d, tw.data(), sizeof(uint64_t) * 2 * E, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(da, ha.data(), sizeof(uint64_t) * len, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(db, hb.data(), sizeof(uint64_t) * len, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        st = cuda_error(e, "ntt_raw copy-in");
    } else {
        A.a = da;
        A.b = db;
        A.out = dout;
        A.tw = d;
        A.itw = d + E;
        st = launch_ntt_raw(A, nullptr);
        if (st == MI_OK) {
            e = cudaMemcpy(h_out, dout, sizeof(uint64_t) * len, cudaMemcpyDeviceToHost);
            if (e != cudaSuccess) st = cuda_error(e, "ntt_raw copy-out");
        }
    }
    cudaFree(d);
    return st;
}

extern "C" mi_status mi_ntt32_raw(mi_ctx ctx, uint32_t prime, uint32_t len, int conv, const uint32_t* h_a,
                                  const uint32_t* h_b, uint32_t* h_out) {
    if (ctx == nullptr) return set_error(MI_EINVAL, "ntt32_raw: null context");
    if (h_a == nullptr || h_out == nullptr || (conv && h_b == nullptr)) return set_error(MI_EINVAL, "ntt32_raw: null");
    if (prime >= 5) return set_error(MI_EINVAL, "ntt32_raw: prime index %u not below 5", prime);
    if (len < 256 || len > 4096 || (len & (len - 1)))
        return set_error(MI_EINVAL, "ntt32_raw: length %u not a power of two in [256, 4096]", len);
    int cur = -1;
    MI_CUDA_TRY(cudaGetDevice(&cur));
    if (cur != ctx->device) MI_CUDA_TRY(cudaSetDevice(ctx->device));
    const uint32_t p = kNttPrimes[prime].p;
    std::vector<uint32_t> ha(len), hb(len, 0);
    for (uint32_t i = 0; i < len; ++i) ha[i] = h_a[i] % p;
    if (conv)
        for (uint32_t i = 0; i < len; ++i) hb[i] = h_b[i] % p;
    uint32_t* d = nullptr;
    MI_CUDA_TRY(cudaMalloc(&d, sizeof(uint32_t) * 3 * size_t(len)));
    uint32_t *da = d, *db = d + len, *dout = d + 2 * len;
    mi_status st = MI_OK;
    cudaError_t e = cudaMemcpy(da, ha.data(), sizeof(uint32_t) * len, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(db, hb.data(), sizeof(uint32_t) * len, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        st = cuda_error(e, "ntt32_raw copy-in");
    } else {
        st = launch_ntt32_raw(da, db, dout, len, prime, conv, ctx->ntt.params, nullptr);
        if (st == MI_OK) {
            e = cudaMemcpy(h_out, dout, sizeof(uint32_t) * len, cudaMemcpyDeviceToHost);
            if (e != cudaSuccess) st = cuda_error(e, "ntt32_raw copy-out");
        }
    }
    cudaFree(d);
    return st;
}

extern "C" mi_status mi_ntt32_prime(uint32_t prime, uint32_t* p, uint32_t* g) {
    if (prime >= 5 || p == nullptr || g == nullptr) return set_error(MI_EINVAL, "ntt32_prime: bad argument");
    *p = kNttPrimes[prime].p;
    *g = kNttPrimes[prime].g;
    return MI_OK;
}
