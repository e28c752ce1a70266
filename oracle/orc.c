/*
 * orc.c -- THE ORACLE.  Test infrastructure only: a CPU restatement of the
 * reference's batched big-integer algorithms, used by tests/, by
 * __graft_entry__.smoke() and by bench.py's CPU-baseline leg to check and to
 * time against.  The library never links, loads or calls anything here.
 *
 * Restated (each function cites the reference code it follows):
 *   orc_add_*     carry-monoid scan addition   cuda/ker-addition.cu.h:50-81,141-194
 *   orc_mul_*     column-scanning classical mul cuda/ker-classic-mul.cu.h:11-26,353-404
 *   orc_zmod_*, orc_ntt_*  prime-field NTT      cuda/ker-fft-mul.cu.h:76-140,191-211,304-368
 *   orc_gmp_*     the reference CPU path gmpAddMulOnce over GMP
 *                                               cuda/helper.h:146-170, cuda/main.cu:165-175,358-368
 *   orc_gmp_import / orc_gmp_export  GMP's own mpz_import / mpz_export, the
 *                 word formats the reference's conversions use (cuda/helper.h:116,
 *                 146-170), to pin the import/export restatement in oracle.py
 * Limb layout everywhere: instance i at [i*m, (i+1)*m), limb 0 least
 * significant (cuda/helper.h:116, GMP_ORDER -1).
 *
 * GMP (libgmp.so.10, the 6.x ABI) is opened with dlopen at first use; the
 * declarations below are the public mpz ABI (struct layout and __gmpz_*
 * entry points), written here because the development headers are not
 * installed.  When GMP is absent, orc_gmp_available() returns 0.
 */
#define _GNU_SOURCE
#include <dlfcn.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef unsigned __int128 u128;

/* ------------------------------------------------------------------------
 * Addition: the reference's CarrySegBop monoid (cuda/ker-addition.cu.h:50-81)
 * on carry codes (bit0 = overflow, bit1 = all ones, bit2 = segment start),
 * identity 2, scanned sequentially over one instance; then each limb adds the
 * overflow bit of the scan up to the previous limb (baddRegs, :141-194).
 * ---------------------------------------------------------------------- */
static uint32_t carry_seg_op(uint32_t c1, uint32_t c2) {
    if (c2 & 4) return c2;
    uint32_t res = ((c1 & (c2 >> 1)) | c2) & 1;
    res |= (c1 & c2 & 2);
    res |= ((c1 | c2) & 4);
    return res;
}

#define ORC_ADD_BODY(L, MAXV)                                                   \
    for (uint64_t i = 0; i < n; ++i) {                                          \
        const L* x = a + i * m;                                                 \
        const L* y = b + i * m;                                                 \
        L* z = r + i * m;                                                       \
        uint32_t prefix = 2; /* identity: carry into limb 0 is 0 */             \
        for (uint32_t k = 0; k < m; ++k) {                                      \
            L s = (L)(x[k] + y[k]);                                             \
            uint32_t c = (uint32_t)(s < x[k]) | ((uint32_t)(s == (MAXV)) << 1); \
            if (k == 0) c |= 4;                                                 \
            /* limb k adds the overflow bit of the scan up to limb k-1 */       \
            z[k] = (L)(s + ((k == 0) ? 0 : (prefix & 1)));                      \
            prefix = carry_seg_op(prefix, c);                                   \
        }                                                                       \
        if (carry) carry[i] = (uint8_t)(prefix & 1);                            \
    }

void orc_add_u64(uint64_t n, uint32_t m, const uint64_t* a, const uint64_t* b, uint64_t* r, uint8_t* carry) {
    ORC_ADD_BODY(uint64_t, UINT64_MAX)
}

void orc_add_u32(uint64_t n, uint32_t m, const uint32_t* a, const uint32_t* b, uint32_t* r, uint8_t* carry) {
    ORC_ADD_BODY(uint32_t, UINT32_MAX)
}

/* 6a + 10b mod 2^(64m), the chain of a6pb10Ker (cuda/ker-addition.cu.h:304-324). */
void orc_add6_u64(uint64_t n, uint32_t m, const uint64_t* a, const uint64_t* b, uint64_t* r) {
    uint64_t* t = (uint64_t*)malloc(sizeof(uint64_t) * m * 5);
    for (uint64_t i = 0; i < n; ++i) {
        const uint64_t* x = a + i * m;
        const uint64_t* y = b + i * m;
        uint64_t *t1 = t, *t2 = t + m, *t3 = t + 2 * m, *t4 = t + 3 * m, *t5 = t + 4 * m;
        orc_add_u64(1, m, x, y, t1, NULL);
        orc_add_u64(1, m, t1, t1, t2, NULL);
        orc_add_u64(1, m, t2, y, t3, NULL);
        orc_add_u64(1, m, t3, t3, t4, NULL);
        orc_add_u64(1, m, t4, t3, t5, NULL);
        orc_add_u64(1, m, t5, y, r + i * m, NULL);
    }
    free(t);
}

/* ------------------------------------------------------------------------
 * Classical multiplication: column scanning as computeIter64
 * (cuda/ker-classic-mul.cu.h:11-26): for output column k, a two-word
 * accumulator collects a_i*b_j (i+j = k) and a counter collects the overflow
 * of its high word; the (low, high, carry) triples of all columns are then
 * added at offsets k, k+1, k+2 (combineQ / from4Reg2ShmQ / baddRegs,
 * :299-404, 425-463).  out_limbs = m (the reference's truncated product) or
 * 2m (full product).
 * ---------------------------------------------------------------------- */
static void mul_one_u64(uint32_t m, const uint64_t* x, const uint64_t* y, uint64_t* z, uint32_t out_limbs,
                        uint64_t* tmp /* 2m+2 */) {
    memset(tmp, 0, sizeof(uint64_t) * (2 * (size_t)m + 2));
    const uint32_t cols = out_limbs < 2 * m ? out_limbs : 2 * m - 1;
    for (uint32_t k = 0; k < cols; ++k) {
        u128 acc = 0;
        uint64_t cnt = 0;
        uint32_t i0 = (k >= m) ? k - m + 1 : 0;
        for (uint32_t i = i0; i <= k && i < m; ++i) {
            u128 p = (u128)x[i] * y[k - i];
            uint64_t hi_prev = (uint64_t)(acc >> 64);
            acc += p;
            cnt += ((uint64_t)(acc >> 64) < hi_prev);
        }
        /* add (lo, hi, cnt) at columns k, k+1, k+2 with carry */
        uint64_t w[3] = {(uint64_t)acc, (uint64_t)(acc >> 64), cnt};
        uint64_t c = 0;
        for (uint32_t d = 0; k + d < 2 * m + 2; ++d) {
            u128 s = (u128)tmp[k + d] + (d < 3 ? w[d] : 0) + c;
            tmp[k + d] = (uint64_t)s;
            c = (uint64_t)(s >> 64);
            if (d >= 2 && c == 0) break;
        }
    }
    for (uint32_t k = 0; k < out_limbs; ++k) z[k] = tmp[k];
}

static void mul_one_u32(uint32_t m, const uint32_t* x, const uint32_t* y, uint32_t* z, uint32_t out_limbs,
                        uint32_t* tmp) {
    memset(tmp, 0, sizeof(uint32_t) * (2 * (size_t)m + 2));
    const uint32_t cols = out_limbs < 2 * m ? out_limbs : 2 * m - 1;
    for (uint32_t k = 0; k < cols; ++k) {
        uint64_t acc = 0;
        uint32_t cnt = 0;
        uint32_t i0 = (k >= m) ? k - m + 1 : 0;
        for (uint32_t i = i0; i <= k && i < m; ++i) {
            uint64_t p = (uint64_t)x[i] * y[k - i];
            uint32_t hi_prev = (uint32_t)(acc >> 32);
            acc += p;
            cnt += ((uint32_t)(acc >> 32) < hi_prev);
        }
        uint32_t w[3] = {(uint32_t)acc, (uint32_t)(acc >> 32), cnt};
        uint32_t c = 0;
        for (uint32_t d = 0; k + d < 2 * m + 2; ++d) {
            uint64_t s = (uint64_t)tmp[k + d] + (d < 3 ? w[d] : 0) + c;
            tmp[k + d] = (uint32_t)s;
            c = (uint32_t)(s >> 32);
            if (d >= 2 && c == 0) break;
        }
    }
    for (uint32_t k = 0; k < out_limbs; ++k) z[k] = tmp[k];
}

void orc_mul_u64(uint64_t n, uint32_t m, const uint64_t* a, const uint64_t* b, uint64_t* r, int full) {
    const uint32_t out = full ? 2 * m : m;
    uint64_t* tmp = (uint64_t*)malloc(sizeof(uint64_t) * (2 * (size_t)m + 2));
    for (uint64_t i = 0; i < n; ++i) mul_one_u64(m, a + i * m, b + i * m, r + i * out, out, tmp);
    free(tmp);
}

void orc_mul_u32(uint64_t n, uint32_t m, const uint32_t* a, const uint32_t* b, uint32_t* r, int full) {
    const uint32_t out = full ? 2 * m : m;
    uint32_t* tmp = (uint32_t*)malloc(sizeof(uint32_t) * (2 * (size_t)m + 2));
    for (uint64_t i = 0; i < n; ++i) mul_one_u32(m, a + i * m, b + i * m, r + i * out, out, tmp);
    free(tmp);
}

/* (a^2 + b)(b^2 + b) + ab mod 2^(64m): the composite of polyKerQ
 * (cuda/ker-classic-mul.cu.h:500-575) -- t1 = a*a, t2 = t1 + b, t3 = b*b,
 * t4 = t3 + b, t5 = t2*t4, t6 = a*b, r = t5 + t6, every step mod 2^(64m). */
void orc_poly_u64(uint64_t n, uint32_t m, const uint64_t* a, const uint64_t* b, uint64_t* r) {
    uint64_t* t = (uint64_t*)malloc(sizeof(uint64_t) * m * 6);
    for (uint64_t i = 0; i < n; ++i) {
        const uint64_t* x = a + i * m;
        const uint64_t* y = b + i * m;
        uint64_t *t1 = t, *t2 = t + m, *t3 = t + 2 * m, *t4 = t + 3 * m, *t5 = t + 4 * m, *t6 = t + 5 * m;
        orc_mul_u64(1, m, x, x, t1, 0);
        orc_add_u64(1, m, t1, y, t2, NULL);
        orc_mul_u64(1, m, y, y, t3, 0);
        orc_add_u64(1, m, t3, y, t4, NULL);
        orc_mul_u64(1, m, t2, t4, t5, 0);
        orc_mul_u64(1, m, x, y, t6, 0);
        orc_add_u64(1, m, t5, t6, r + i * m, NULL);
    }
    free(t);
}

/* ------------------------------------------------------------------------
 * Prime-field NTT primitives of the reference (cuda/ker-fft-mul.cu.h):
 * zmod_t add/sub/mul/pow/inv (:76-140) over a prime p < 2^63, getOmega /
 * mkOmegas (:191-211), bit reversal (:9-14), radix-2 DIT transform with the
 * bit-reverse permutation first (fft, :304-348) and the inverse scaled by
 * 1/len (ifft, :350-368).  orc_ntt_conv is the raw cyclic convolution that
 * bmulFFTvalid (:512-554) computes.
 * ---------------------------------------------------------------------- */
uint64_t orc_zmod_mul(uint64_t p, uint64_t x, uint64_t y) { return (uint64_t)(((u128)x * y) % p); }
uint64_t orc_zmod_add(uint64_t p, uint64_t x, uint64_t y) {
    u128 r = (u128)x + y;
    if (r >= p) r -= p;
    return (uint64_t)r;
}
uint64_t orc_zmod_sub(uint64_t p, uint64_t x, uint64_t y) { return (x >= y) ? x - y : x + (p - y); }
uint64_t orc_zmod_pow(uint64_t p, uint64_t x, uint64_t e) {
    uint64_t acc = 1 % p, base = x % p;
    while (e) {
        if (e & 1) acc = orc_zmod_mul(p, acc, base);
        base = orc_zmod_mul(p, base, base);
        e >>= 1;
    }
    return acc;
}
/* extended Euclid as in zmod_t::inv (cuda/ker-fft-mul.cu.h:117-128) */
uint64_t orc_zmod_inv(uint64_t p, uint64_t x) {
    int64_t t = 0, newt = 1;
    uint64_t r = p, newr = x % p;
    while (newr != 0) {
        uint64_t q = r / newr;
        int64_t tt = t - (int64_t)q * newt;
        t = newt;
        newt = tt;
        uint64_t rr = r - q * newr;
        r = newr;
        newr = rr;
    }
    if (t < 0) t += (int64_t)p;
    return (uint64_t)t;
}

static uint32_t ilog2u(uint32_t v) {
    uint32_t l = 0;
    while ((1u << l) < v) ++l;
    return l;
}

/* omega = g^(2^(two_adicity - lg len)), the primitive len-th root (getOmega) */
uint64_t orc_ntt_omega(uint64_t p, uint64_t g, uint32_t two_adicity, uint32_t len) {
    return orc_zmod_pow(p, g, (uint64_t)1 << (two_adicity - ilog2u(len)));
}

static uint32_t bit_reverse(uint32_t j, uint32_t nb) {
    uint32_t r = 0;
    for (; nb--; j >>= 1) r = (r << 1) | (j & 1);
    return r;
}

/* in-place transform with root w, natural order in and out */
static void ntt_inplace(uint64_t p, uint64_t w, uint32_t len, uint64_t* x) {
    const uint32_t lg = ilog2u(len);
    for (uint32_t k = 0; k < len; ++k) {
        uint32_t j = bit_reverse(k, lg);
        if (j > k) {
            uint64_t t = x[k];
            x[k] = x[j];
            x[j] = t;
        }
    }
    uint64_t* om = (uint64_t*)malloc(sizeof(uint64_t) * len);
    uint64_t acc = 1;
    for (uint32_t i = 0; i < len; ++i) {
        om[i] = acc;
        acc = orc_zmod_mul(p, acc, w);
    }
    for (uint32_t q = 1; q <= lg; ++q) {
        const uint32_t L = 1u << q, half = L >> 1, rstep = len >> q;
        for (uint32_t k = 0; k < len; k += L)
            for (uint32_t j = 0; j < half; ++j) {
                uint64_t tau = orc_zmod_mul(p, om[rstep * j], x[k + j + half]);
                uint64_t u = x[k + j];
                x[k + j] = orc_zmod_add(p, u, tau);
                x[k + j + half] = orc_zmod_sub(p, u, tau);
            }
    }
    free(om);
}

void orc_ntt_forward(uint64_t p, uint64_t g, uint32_t two_adicity, uint32_t len, const uint64_t* in, uint64_t* out) {
    for (uint32_t i = 0; i < len; ++i) out[i] = in[i] % p;
    ntt_inplace(p, orc_ntt_omega(p, g, two_adicity, len), len, out);
}

void orc_ntt_inverse(uint64_t p, uint64_t g, uint32_t two_adicity, uint32_t len, const uint64_t* in, uint64_t* out) {
    for (uint32_t i = 0; i < len; ++i) out[i] = in[i] % p;
    uint64_t w = orc_ntt_omega(p, g, two_adicity, len);
    ntt_inplace(p, orc_zmod_inv(p, w), len, out);
    uint64_t inv_len = orc_zmod_inv(p, len);
    for (uint32_t i = 0; i < len; ++i) out[i] = orc_zmod_mul(p, out[i], inv_len);
}

void orc_ntt_conv(uint64_t p, uint64_t g, uint32_t two_adicity, uint32_t len, const uint64_t* a, const uint64_t* b,
                  uint64_t* out) {
    uint64_t* fa = (uint64_t*)malloc(sizeof(uint64_t) * len);
    uint64_t* fb = (uint64_t*)malloc(sizeof(uint64_t) * len);
    orc_ntt_forward(p, g, two_adicity, len, a, fa);
    orc_ntt_forward(p, g, two_adicity, len, b, fb);
    for (uint32_t i = 0; i < len; ++i) fa[i] = orc_zmod_mul(p, fa[i], fb[i]);
    orc_ntt_inverse(p, g, two_adicity, len, fa, out);
    free(fa);
    free(fb);
}

/* ------------------------------------------------------------------------
 * GMP: gmpAddMulOnce (cuda/helper.h:146-170) restated over the mpz ABI.
 * ---------------------------------------------------------------------- */
typedef struct {
    int alloc;
    int size;
    void* d;
} orc_mpz;

typedef void (*fn_init_t)(orc_mpz*);
typedef void (*fn_clear_t)(orc_mpz*);
typedef void (*fn_import_t)(orc_mpz*, size_t, int, size_t, int, size_t, const void*);
typedef void* (*fn_export_t)(void*, size_t*, int, size_t, int, size_t, const orc_mpz*);
typedef void (*fn_bin_t)(orc_mpz*, const orc_mpz*, const orc_mpz*);

static struct {
    int tried, ok;
    fn_init_t init;
    fn_clear_t clear;
    fn_import_t import_;
    fn_export_t export_;
    fn_bin_t add, mul;
} G;
static pthread_mutex_t g_mu = PTHREAD_MUTEX_INITIALIZER;

int orc_gmp_available(void) {
    pthread_mutex_lock(&g_mu);
    if (!G.tried) {
        G.tried = 1;
        void* h = dlopen("libgmp.so.10", RTLD_NOW | RTLD_LOCAL);
        if (!h) h = dlopen("libgmp.so", RTLD_NOW | RTLD_LOCAL);
        if (h) {
            G.init = (fn_init_t)dlsym(h, "__gmpz_init");
            G.clear = (fn_clear_t)dlsym(h, "__gmpz_clear");
            G.import_ = (fn_import_t)dlsym(h, "__gmpz_import");
            G.export_ = (fn_export_t)dlsym(h, "__gmpz_export");
            G.add = (fn_bin_t)dlsym(h, "__gmpz_add");
            G.mul = (fn_bin_t)dlsym(h, "__gmpz_mul");
            G.ok = G.init && G.clear && G.import_ && G.export_ && G.add && G.mul;
        }
    }
    pthread_mutex_unlock(&g_mu);
    return G.ok;
}

#define GMP_ORDER (-1)

/* One instance: import m32 u32 words of a and b (least significant word
 * first), r = a+b or a*b, export, write out_words words (truncating or zero
 * filling) -- gmpAddMulOnce with the output length as a parameter. */
static void gmp_once(int is_add, uint32_t m32, const uint32_t* x, const uint32_t* y, uint32_t* z, uint32_t out_words,
                     uint32_t* buff /* >= 2*m32+2 words */) {
    orc_mpz a, b, r;
    G.init(&a);
    G.init(&b);
    G.init(&r);
    G.import_(&a, m32, GMP_ORDER, sizeof(uint32_t), 0, 0, x);
    G.import_(&b, m32, GMP_ORDER, sizeof(uint32_t), 0, 0, y);
    if (is_add)
        G.add(&r, &a, &b);
    else
        G.mul(&r, &a, &b);
    size_t countp = 0;
    G.export_(buff, &countp, GMP_ORDER, sizeof(uint32_t), 0, 0, &r);
    for (uint32_t j = 0; j < out_words; ++j) z[j] = (j < countp) ? buff[j] : 0;
    G.clear(&a);
    G.clear(&b);
    G.clear(&r);
}

typedef struct {
    int is_add;
    uint32_t m32, out_words;
    const uint32_t *a, *b;
    uint32_t* r;
    uint64_t lo, hi;
} gmp_job;

static void* gmp_worker(void* arg) {
    gmp_job* j = (gmp_job*)arg;
    uint32_t* buff = (uint32_t*)malloc(sizeof(uint32_t) * (2 * (size_t)j->m32 + 4));
    for (uint64_t i = j->lo; i < j->hi; ++i)
        gmp_once(j->is_add, j->m32, j->a + i * j->m32, j->b + i * j->m32, j->r + i * j->out_words, j->out_words, buff);
    free(buff);
    return NULL;
}

/* Batched GMP add/mul over n instances of m32 u32 words, statically
 * partitioned over `threads` POSIX threads.  Returns 0, or -1 without GMP. */
int orc_gmp_batch(int is_add, uint64_t n, uint32_t m32, const uint32_t* a, const uint32_t* b, uint32_t* r,
                  uint32_t out_words, int threads) {
    if (!orc_gmp_available()) return -1;
    if (threads < 1) threads = 1;
    if ((uint64_t)threads > n) threads = (int)(n ? n : 1);
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * threads);
    gmp_job* jobs = (gmp_job*)malloc(sizeof(gmp_job) * threads);
    for (int t = 0; t < threads; ++t) {
        jobs[t] = (gmp_job){is_add, m32, out_words, a, b, r, n * t / threads, n * (t + 1) / threads};
        if (threads == 1)
            gmp_worker(&jobs[t]);
        else
            pthread_create(&th[t], NULL, gmp_worker, &jobs[t]);
    }
    if (threads > 1)
        for (int t = 0; t < threads; ++t) pthread_join(th[t], NULL);
    free(th);
    free(jobs);
    return 0;
}

/* Multi-threaded restatement batch (the fallback CPU baseline when GMP is
 * missing): op 0 = add u64, 1 = full mul u64. */
typedef struct {
    int op;
    uint32_t m;
    const uint64_t *a, *b;
    uint64_t* r;
    uint8_t* carry;
    uint64_t lo, hi;
} orc_job;

static void* orc_worker(void* arg) {
    orc_job* j = (orc_job*)arg;
    const uint64_t cnt = j->hi - j->lo;
    if (j->op == 0)
        orc_add_u64(cnt, j->m, j->a + j->lo * j->m, j->b + j->lo * j->m, j->r + j->lo * j->m,
                    j->carry ? j->carry + j->lo : NULL);
    else
        orc_mul_u64(cnt, j->m, j->a + j->lo * j->m, j->b + j->lo * j->m, j->r + j->lo * 2 * j->m, 1);
    return NULL;
}

void orc_batch_u64(int op, uint64_t n, uint32_t m, const uint64_t* a, const uint64_t* b, uint64_t* r, uint8_t* carry,
                   int threads) {
    if (threads < 1) threads = 1;
    if ((uint64_t)threads > n) threads = (int)(n ? n : 1);
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * threads);
    orc_job* jobs = (orc_job*)malloc(sizeof(orc_job) * threads);
    for (int t = 0; t < threads; ++t) {
        jobs[t] = (orc_job){op, m, a, b, r, carry, n * t / threads, n * (t + 1) / threads};
        if (threads == 1)
            orc_worker(&jobs[t]);
        else
            pthread_create(&th[t], NULL, orc_worker, &jobs[t]);
    }
    if (threads > 1)
        for (int t = 0; t < threads; ++t) pthread_join(th[t], NULL);
    free(th);
    free(jobs);
}

/* ------------------------------------------------------------------------
 * GMP's own word-format conversions (mpz_import / mpz_export with any
 * order, word size and byte order), to pin the restatement in oracle.py.
 * ---------------------------------------------------------------------- */

/* `count` words of `size` bytes at src (GMP's order / endian conventions) ->
 * `nlimbs` u64 limbs, least significant first, zero filled (higher limbs
 * dropped).  Returns the number of significant limbs, or -1 without GMP. */
int orc_gmp_import(const void* src, uint32_t count, int order, uint32_t size, int endian, uint64_t* limbs,
                   uint32_t nlimbs) {
    if (!orc_gmp_available()) return -1;
    orc_mpz z;
    G.init(&z);
    G.import_(&z, count, order, size, endian, 0, src);
    uint64_t* buf = (uint64_t*)calloc((size_t)count * size / 8 + 2, 8);
    size_t cnt = 0;
    G.export_(buf, &cnt, -1, 8, 0, 0, &z);
    for (uint32_t j = 0; j < nlimbs; ++j) limbs[j] = j < cnt ? buf[j] : 0;
    free(buf);
    G.clear(&z);
    return (int)cnt;
}

/* `nlimbs` u64 limbs -> mpz_export with (order, size, endian) into a
 * fixed-width field of `words` words: GMP's `count` significant words, placed
 * at the least significant end of the field (the start for order -1, the end
 * for order 1), the rest zero.  Returns count (count > words: did not fit and
 * nothing is written), or -1 without GMP. */
int orc_gmp_export(const uint64_t* limbs, uint32_t nlimbs, int order, uint32_t size, int endian, void* dst,
                   uint32_t words) {
    if (!orc_gmp_available()) return -1;
    orc_mpz z;
    G.init(&z);
    G.import_(&z, nlimbs, -1, 8, 0, 0, limbs);
    uint8_t* buf = (uint8_t*)calloc((size_t)nlimbs * 8 / size + 2, size);
    size_t cnt = 0;
    G.export_(buf, &cnt, order, size, endian, 0, &z);
    G.clear(&z);
    if (cnt <= words) {
        uint8_t* d = (uint8_t*)dst;
        memset(d, 0, (size_t)words * size);
        if (order < 0)
            memcpy(d, buf, cnt * size);
        else
            memcpy(d + (size_t)(words - cnt) * size, buf, cnt * size);
    }
    free(buf);
    return (int)cnt;
}
