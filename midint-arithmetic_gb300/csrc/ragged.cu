// ragged.cu -- one ragged list of additions and multiplications of uneven
// lengths, binned by size class on the device and consumed by persistent
// kernels, longest work first.  (No reference counterpart: the reference runs
// one kernel per operation and compile-time size, cuda/main.cu:661-746.)
//
// Stages, all asynchronous on one stream (and so capturable in a CUDA graph):
//  1. classify: each op gets a size-class key; blocks count their keys in
//     shared memory and add the counts to the global ones;
//  2. scan (one warp per family): op offsets per key and task offsets per
//     family, with the keys of each family in descending cost order;
//  3. scatter: op indices grouped by key (each block reserves its slots of a
//     key with one atomic);
//  4. one persistent kernel per family, each popping tasks from its atomic
//     queue, chained so that each kernel's blocks start on the SMs the
//     previous kernel's last tasks leave idle (ragged_launch):
//     * NTT products (shorter operand >= the crossover): a task is one CTA of
//       256 threads = 2048/L products with L-point transforms (ntt_mul.cuh),
//       one family with 64-bit digits on five primes, one with 48-bit
//       digits on four for the products whose 48-bit digits fit the same L,
//       and one with 40-bit digits on three for those whose 40-bit digits
//       fit it (and whose shorter operand stays within the 3-prime bound);
//     * classical products with a shorter operand of 9 to 128 limbs whose
//       wider operand exceeds 16 tiles of 8 u32 limbs: one warp per product
//       over rounds of 32 output blocks (rect32_task), the shorter operand
//       broadcast, the longer one in chunks of 32 tiles in two alternating
//       shared-memory buffers, one anti-diagonal per lane per round and a
//       snapshot only in the first (wrap-around) round;
//     * the narrower ones (both operands within 16 tiles): a task per warp
//       of 32/NT square products (mul_core.cuh) whose shorter operand is the
//       broadcast side -- no padding of either operand to a power of two;
//     * comb products, shorter operand of at most 8 limbs, a family and a
//       kernel of their own (each thread multiplies 16 words of the longer
//       operand by all of the shorter one in one parity-split accumulator);
//     * chunked square products for 129..256 limbs in 64-thread groups, each
//       chunk's carry pass adding the pending window of the chunk before;
//     * additions, a task per warp: lanes of one limb for additions of up to
//       32 limbs, rows of 32 limbs per warp above that.
// Within a family the key encodes everything that sets the trip counts of a
// task, so the groups of a task run in lockstep.
#include <algorithm>
#include <cstring>
#include <mutex>
#include <vector>

#include "common.cuh"
#include "ctx.h"
#include "kernels.h"
#include "mul_core.cuh"
#include "ntt32.cuh"
#include "ntt_mul.cuh"

namespace mi {
namespace rg {

constexpr uint32_t kMaxLimbs = 1024;
constexpr int K_NTT = 4;         // transform length 2^8 .. 2^11, 64-bit digits (5 primes)
constexpr int K_N48 = 4;         // the same with 48-bit digits (4 primes)
constexpr int K_N40 = 4;         // the same with 40-bit digits (3 primes)
constexpr int K_CLS = 5;         // NT = 1..16 (one chunk)
constexpr int K_ADD = 11;        // GS = 1..32 lanes of one limb; one warp over 2..32 rows of 32 limbs
constexpr int K_C64 = 4;         // classical, 64-thread groups: chunks = 1..4
constexpr int K_CMB = 7;         // comb, shorter operand <= 8 limbs: groups of 4, 8, 16, 32 x passes 1..4
constexpr int K_R32 = 8;         // classical, 32 threads in rounds: chunks of 32 blocks = 1..8
constexpr int KEY_NTT = 0, KEY_CLS = K_NTT, KEY_ADD = KEY_CLS + K_CLS, KEY_C64 = KEY_ADD + K_ADD,
              KEY_N48 = KEY_C64 + K_C64, KEY_CMB = KEY_N48 + K_N48, KEY_N40 = KEY_CMB + K_CMB,
              KEY_R32 = KEY_N40 + K_N40;
constexpr int K = KEY_R32 + K_R32;
// families: NTT (64-bit digits), classical square products of groups of up
// to 16 threads, additions, classical in 64 threads, NTT with 48-bit digits,
// comb products, NTT with 40-bit digits, classical in 32 threads over rounds
constexpr int NFAM = 8;
constexpr uint32_t KEY_INVALID = 0xffffffffu;
constexpr uint32_t kAddRowOps = 4;  // additions of more than 32 limbs per warp task
constexpr int kAddRowBatch = 4;    // rows of 32 limbs per batch of loads (two batches in flight)
constexpr int CLS_WARP_WORDS = 256 + 256 + 32 * classic::PER_T;  // A, B planes, per-thread slots
constexpr int R32_WARP_WORDS = CLS_WARP_WORDS + 256;  // the same and a second B plane buffer
constexpr int C64_GROUP_WORDS = 512 + 512 + 64 * classic::PER_T;  // the same for one 64-thread group

// Keys of each family in descending cost order (filled once per device).
__constant__ uint16_t c_order[K];

struct Scratch {  // word offsets into the scratch buffer
    static constexpr size_t COUNTS = 0;
    static constexpr size_t CURSORS = COUNTS + K;
    static constexpr size_t OPOFF = CURSORS + K;
    static constexpr size_t TS = OPOFF + K;             // task starts: K + NFAM words (one extra per family)
    static constexpr size_t NTASKS = TS + K + NFAM;     // NFAM words
    static constexpr size_t QUEUE = NTASKS + NFAM;      // NFAM words
    static constexpr size_t INVALID = QUEUE + NFAM;     // 1 word
    static constexpr size_t KEYS = ((INVALID + 1 + 31) / 32) * 32;
    __host__ __device__ static constexpr size_t sorted(uint32_t n) { return KEYS + n; }  // op indices by key
    __host__ __device__ static constexpr size_t words(uint32_t n) { return KEYS + 2 * size_t(n); }
};

struct Params {
    const mi_op* ops;
    uint32_t n_ops;
    const uint64_t* in;
    uint64_t* out;
    uint8_t* carry;
    uint32_t* scr;  // scratch words
    uint32_t ntt_min;    // products whose shorter operand has this many limbs go to the NTT
    uint32_t ntt40_min;  // ... or this many, when their NTT runs on 40-bit digits
    NttMulParams ntt;
};

__device__ __forceinline__ uint32_t ceil_log2(uint32_t x) { return x <= 1 ? 0 : 32 - __clz(x - 1); }

__device__ __forceinline__ uint32_t classify(const mi_op& op, uint32_t ntt_min, uint32_t ntt40_min) {
    const uint32_t la = op.la, lb = op.lb;
    if (la == 0 || lb == 0 || la > kMaxLimbs || lb > kMaxLimbs) return KEY_INVALID;
    if (op.kind == MI_OP_ADD) {
        const uint32_t m = max(la, lb);
        if (m <= 32) return KEY_ADD + ceil_log2(m);       // groups of 1..32 lanes, one limb each
        return KEY_ADD + 5 + ceil_log2((m + 31) / 32);    // a warp over 2, 4, 8, 16, 32 rows
    }
    if (op.kind == MI_OP_MUL) {
        const uint32_t s = min(la, lb), l = max(la, lb);
        if (s >= min(ntt_min, ntt40_min)) {
            // L must hold all la+lb output limbs (the top limb is the carry out
            // of the last of the la+lb-1 coefficients), not only the
            // coefficients; 40-bit digits on three primes or 48-bit ones on
            // four when they fit the same L
            const uint32_t lg = max(8u, ceil_log2(la + lb));
            const int dm = ntt32::ntt_mode(la, lb, 1u << lg);
            if (s >= ntt_min || dm == ntt32::DM40)
                return (dm == ntt32::DM40 ? KEY_N40 : (dm == ntt32::DM48 ? KEY_N48 : KEY_NTT)) + (lg - 8);
        }
        if (s > 128) return KEY_C64 + (2 * l + 511) / 512 - 1;  // 64-thread groups, chunks of 256 limbs
        if (s <= 8) {  // comb: 16 words of the longer operand per thread, 512 per pass of a warp
            const uint32_t na = 2 * l;
            if (na <= 256) return KEY_CMB + (na <= 64 ? 0 : (na <= 128 ? 1 : 2));
            return KEY_CMB + 3 + (na + 511) / 512 - 1;
        }
        // NT threads, NT-block chunks of the longer operand against the
        // shorter one (whose blocks set the steps per chunk): as wide as the
        // longer operand up to one warp, and never narrower than the shorter
        const uint32_t nbs = (2 * s + 7) / 8, nbl = (2 * l + 7) / 8;
        const uint32_t ntl = ceil_log2(max(nbs, min(nbl, 32u)));  // NT = 2^ntl <= 32
        if (ntl < 5) return KEY_CLS + ntl;  // NT >= nbl: one chunk
        return KEY_R32 + (nbl + 31) / 32 - 1;  // NT = 32, nbl <= 256: 1..8 chunks
    }
    return KEY_INVALID;
}

__host__ __device__ __forceinline__ uint32_t ops_per_task(uint32_t key) {
    if (key >= KEY_R32) return 1u;                                    // classical, 32 threads over rounds
    if (key < KEY_CLS) return 2048u >> (8 + key - KEY_NTT);          // NTT: 256 threads / (L/8)
    if (key < KEY_ADD) return 32u >> (key - KEY_CLS);                // classical: one warp of 32/NT groups
    if (key < KEY_C64) {                                              // add: one warp
        const uint32_t k = key - KEY_ADD;
        return k < 6 ? 32u >> k : kAddRowOps;
    }
    if (key < KEY_N48) return 4u;                                     // classical: 256 threads / 64
    if (key < KEY_CMB) return 2048u >> (8 + key - KEY_N48);          // NTT, 48-bit digits
    if (key < KEY_N40) return key - KEY_CMB < 3 ? 8u >> (key - KEY_CMB) : 1u;  // comb: 32 / group
    return 2048u >> (8 + key - KEY_N40);                              // NTT, 40-bit digits
}

// Binning.  Blocks of classify and scatter own the same contiguous ranges of
// kBinRange ops and count their keys in shared memory, so the global counters
// take one atomic per (block, key) instead of one per op.
constexpr uint32_t kBinRange = 1024;
static_assert(K <= 256, "one shared counter per thread");

__global__ void __launch_bounds__(256) k_classify(const mi_op* __restrict__ ops, uint32_t n,
                                                  uint32_t* __restrict__ scr, uint32_t ntt_min, uint32_t ntt40_min) {
    __shared__ uint32_t hist[K + 1];  // the keys, then the invalid ops
    for (int k = threadIdx.x; k <= K; k += blockDim.x) hist[k] = 0;
    __syncthreads();
    uint32_t* keys = scr + Scratch::KEYS;
    const uint32_t lo = blockIdx.x * kBinRange, hi = min(n, lo + kBinRange);
    for (uint32_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
        const uint32_t key = classify(ops[i], ntt_min, ntt40_min);
        keys[i] = key;
        atomicAdd(&hist[key == KEY_INVALID ? K : key], 1u);
    }
    __syncthreads();
    if (threadIdx.x < K && hist[threadIdx.x]) atomicAdd(scr + Scratch::COUNTS + threadIdx.x, hist[threadIdx.x]);
    if (threadIdx.x == K && hist[K]) atomicAdd(scr + Scratch::INVALID, hist[K]);
}

// First key of family f (f = NFAM: the end of the key space).
__host__ __device__ constexpr int fam_base(int f) {
    constexpr int base[NFAM + 1] = {KEY_NTT, KEY_CLS, KEY_ADD, KEY_C64, KEY_N48, KEY_CMB, KEY_N40, KEY_R32, K};
    return base[f];
}
static_assert(fam_base(1) - fam_base(0) <= 32 && fam_base(2) - fam_base(1) <= 32 &&
                  fam_base(3) - fam_base(2) <= 32 && fam_base(4) - fam_base(3) <= 32 &&
                  fam_base(5) - fam_base(4) <= 32 && fam_base(6) - fam_base(5) <= 32 &&
                  fam_base(7) - fam_base(6) <= 32 && fam_base(8) - fam_base(7) <= 32,
              "a family's keys fit one warp");

// One warp per family scans its keys in c_order (shuffle scans): op offsets
// by key (global over the families), task starts by order position with one
// sentinel per family, task counts; the queues restart at 0.
__global__ void __launch_bounds__(32 * NFAM) k_scan(uint32_t* __restrict__ scr) {
    __shared__ uint32_t fam_ops[NFAM];
    const int f = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int base = fam_base(f), nk = fam_base(f + 1) - base;
    uint32_t key = 0, c = 0, tk = 0;
    if (lane < nk) {
        key = c_order[base + lane];
        c = scr[Scratch::COUNTS + key];
        const uint32_t opt = ops_per_task(key);
        tk = (c + opt - 1) / opt;
    }
    uint32_t ci = c, ti = tk;  // inclusive scans
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t u = __shfl_up_sync(MI_FULL_MASK, ci, d), v = __shfl_up_sync(MI_FULL_MASK, ti, d);
        if (lane >= d) {
            ci += u;
            ti += v;
        }
    }
    if (lane == 31) fam_ops[f] = ci;
    __syncthreads();
    uint32_t before = 0;
    for (int g = 0; g < f; ++g) before += fam_ops[g];
    if (lane < nk) {
        scr[Scratch::OPOFF + key] = before + ci - c;
        scr[Scratch::TS + f + base + lane] = ti - tk;
    }
    if (lane == 31) {
        scr[Scratch::TS + f + base + nk] = ti;  // sentinel
        scr[Scratch::NTASKS + f] = ti;
        scr[Scratch::QUEUE + f] = 0;
    }
}

__global__ void __launch_bounds__(256) k_scatter(uint32_t n, uint32_t* __restrict__ scr) {
    __shared__ uint32_t hist[K], base[K];
    for (int k = threadIdx.x; k < K; k += blockDim.x) hist[k] = 0;
    __syncthreads();
    const uint32_t* keys = scr + Scratch::KEYS;
    uint32_t* sorted = scr + Scratch::sorted(n);
    const uint32_t lo = blockIdx.x * kBinRange, hi = min(n, lo + kBinRange);
    for (uint32_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
        const uint32_t key = keys[i];
        if (key != KEY_INVALID) atomicAdd(&hist[key], 1u);
    }
    __syncthreads();
    if (threadIdx.x < K) {  // this block's slots of each key
        const uint32_t k = threadIdx.x;
        if (hist[k]) base[k] = scr[Scratch::OPOFF + k] + atomicAdd(scr + Scratch::CURSORS + k, hist[k]);
        hist[k] = 0;
    }
    __syncthreads();
    for (uint32_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
        const uint32_t key = keys[i];
        if (key != KEY_INVALID) sorted[base[key] + atomicAdd(&hist[key], 1u)] = i;
    }
}

// Task t of a family -> (key, index of its first op in `sorted`, op count).
struct Task {
    uint32_t key, first, count;
};

// A family's decode table in shared memory, loaded once per block from the
// scratch: the task start of every order position of its keys (and the
// sentinel), and each position's key, op offset and op count, so that
// decoding a task is a binary search in shared memory rather than a chain of
// dependent global loads.
struct FamTab {
    uint32_t ts[33];
    uint32_t key[32], first[32], count[32];
};

// By every thread of the block; a __syncthreads must follow before use.
__device__ __forceinline__ void load_tab(FamTab& tab, const uint32_t* scr, int f) {
    const int base = fam_base(f), nk = fam_base(f + 1) - base;
    for (int i = threadIdx.x; i <= nk; i += blockDim.x) {
        tab.ts[i] = scr[Scratch::TS + f + base + i];
        if (i < nk) {
            const uint32_t key = c_order[base + i];
            tab.key[i] = key;
            tab.first[i] = scr[Scratch::OPOFF + key];
            tab.count[i] = scr[Scratch::COUNTS + key];
        }
    }
}

// Task t of family F from its table.
template <int F>
__device__ __forceinline__ Task decode_tab(const FamTab& tab, uint32_t t) {
    constexpr int nk = fam_base(F + 1) - fam_base(F);
    int lo = 0, hi = nk;  // ts[lo] <= t < ts[hi]
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (tab.ts[mid] <= t) lo = mid; else hi = mid;
    }
    const uint32_t key = tab.key[lo];
    const uint32_t opt = ops_per_task(key);
    const uint32_t local = t - tab.ts[lo];
    Task T;
    T.key = key;
    T.first = tab.first[lo] + local * opt;
    T.count = min(opt, tab.count[lo] - local * opt);
    return T;
}

// --- NTT family ----------------------------------------------------------------

template <int LG, int DM>
__device__ __forceinline__ void ntt_task(const Params& P, const Task& tk, uint32_t* sm, uint32_t* scr_warp) {
    constexpr int NT = (1 << LG) / 8;
    const uint32_t g = threadIdx.x / NT;
    const uint32_t* sorted = P.scr + Scratch::sorted(P.n_ops);
    uint32_t* gsm = sm + g * ntt32::MulSmem<LG>::WORDS32;
    // an idle group (g >= count) runs with zero operands, no store and the
    // same barriers: one inlined product for both (two copies spilled)
    const bool busy = g < tk.count;
    mi_op op{};
    if (busy) op = P.ops[sorted[tk.first + g]];
    // 64-bit digits on 2048 points: both operands (at most kMaxLimbs = 1024
    // limbs) lie in the lower half, so the zero upper half is skipped
    ntt32::mul_one<LG, DM, DM == ntt32::DM64 && (1u << LG) >= 2 * kMaxLimbs>(
        P.in + op.a_off, op.la, P.in + op.b_off, op.lb, busy ? P.out + op.r_off : nullptr, op.la + op.lb, P.ntt, gsm,
        scr_warp);
}

// DM: the digit mode of the family (64-bit digits on five primes, 48-bit
// on four, 40-bit on three: a kernel each, so that no digit mode's code
// raises another's registers).  The 64-bit family runs three CTAs per SM at
// up to 80 registers (no spills; NTT band of the 200000-op list 0.786 ->
// 0.777 ms against two), the others two at up to 128: at three they spill
// 200-250 bytes.
template <int DM>
__global__ void __launch_bounds__(256, DM == ntt32::DM64 ? 3 : 2) k_rg_ntt(Params P) {
    constexpr int F = DM == ntt32::DM64 ? 0 : (DM == ntt32::DM48 ? 4 : 6);  // family
    constexpr int KEY0 = DM == ntt32::DM64 ? KEY_NTT : (DM == ntt32::DM48 ? KEY_N48 : KEY_N40);
    extern __shared__ __align__(16) uint32_t smem[];
    uint32_t* scr_warp = smem + ntt32::MulSmem<11>::WORDS32;  // after the groups' shared memory
    __shared__ uint32_t s_task[2];  // this task and the next, fetched while this one runs
    __shared__ FamTab tab;
    const uint32_t ntasks = P.scr[Scratch::NTASKS + F];
    pdl_trigger();  // the next family's kernel may start as this one's blocks finish
    load_tab(tab, P.scr, F);
    if (threadIdx.x == 0) s_task[0] = atomicAdd(P.scr + Scratch::QUEUE + F, 1u);
    __syncthreads();
    for (uint32_t it = 0;; ++it) {
        const uint32_t t = s_task[it & 1];
        if (t >= ntasks) break;
        if (threadIdx.x == 0) s_task[(it + 1) & 1] = atomicAdd(P.scr + Scratch::QUEUE + F, 1u);
        const Task tk = decode_tab<F>(tab, t);
        switch (tk.key - KEY0) {
            case 0: ntt_task<8, DM>(P, tk, smem, scr_warp); break;
            case 1: ntt_task<9, DM>(P, tk, smem, scr_warp); break;
            case 2: ntt_task<10, DM>(P, tk, smem, scr_warp); break;
            default: ntt_task<11, DM>(P, tk, smem, scr_warp); break;
        }
        __syncthreads();  // the next index is visible; this one is read by all
    }
    if (DM != ntt32::DM64) pdl_wait();  // complete only after the task kernel launched before it
}

// --- classical family ----------------------------------------------------------

// Thread t's two 16-byte slots (t and t+NT) of the W = NT*T limbs of x
// starting at limb `start`, zero beyond nx (x rows are 8-byte aligned).
template <int NT>
__device__ __forceinline__ void load_chunk_regs(uint4 (&q)[classic::T / 4], const uint32_t* __restrict__ x,
                                                uint32_t nx, uint32_t start, uint32_t t) {
#pragma unroll
    for (int it = 0; it < classic::T / 4; ++it) {
        const uint32_t w = start + 4 * (t + uint32_t(it) * NT);
        uint2 lo = make_uint2(0, 0), hi = make_uint2(0, 0);
        if (w + 2 <= nx) lo = __ldcs(reinterpret_cast<const uint2*>(x + w));
        if (w + 4 <= nx) hi = __ldcs(reinterpret_cast<const uint2*>(x + w + 2));
        q[it] = make_uint4(lo.x, lo.y, hi.x, hi.y);
    }
}

// One classical task: NT <= 16, 32/NT groups in the caller's warp, one chunk
// (`sm` is the warp's area, the groups interleaved); NT = 64, the four
// 64-thread groups of the block, one or more chunks (`sm` the block's area,
// one C64_GROUP_WORDS region per group; groups without a product run on zeros
// so the block's barriers match, `scr` holds the block's per-warp carry
// words).
template <int NT>
__device__ __forceinline__ void classic_task(const Params& P, const Task& tk, uint32_t* sm, uint32_t* scr) {
    using classic::T;
    constexpr bool WIDE = NT > 32;
    constexpr int G = WIDE ? 1 : 32 / NT;  // groups of the warp, interleaved in shared memory
    const uint32_t lane = WIDE ? threadIdx.x : (threadIdx.x & 31u);
    const uint32_t g = lane / NT, t = lane % NT;
    const bool valid = g < tk.count;
    if (!WIDE && !valid) return;  // warp groups synchronise only among their own lanes
    const uint32_t chunks = WIDE ? tk.key - KEY_C64 + 1 : 1u;
    const uint32_t* sorted = P.scr + Scratch::sorted(P.n_ops);
    mi_op op{};
    if (valid) op = P.ops[sorted[tk.first + g]];
    uint32_t* gA = WIDE ? sm + g * C64_GROUP_WORDS : sm + g * T;
    uint4* gB4 = WIDE ? reinterpret_cast<uint4*>(sm + g * C64_GROUP_WORDS + 512)
                      : reinterpret_cast<uint4*>(sm + 256) + g * NT;
    uint2* slots = WIDE ? reinterpret_cast<uint2*>(sm + g * C64_GROUP_WORDS + 1024)
                        : reinterpret_cast<uint2*>(sm + 512) + g * NT;
    // longer operand x is consumed in chunks of W limbs against the staged shorter y
    const bool a_long = op.la >= op.lb;
    const uint32_t* x = reinterpret_cast<const uint32_t*>(P.in + (a_long ? op.a_off : op.b_off));
    const uint32_t* y = reinterpret_cast<const uint32_t*>(P.in + (a_long ? op.b_off : op.a_off));
    const uint32_t nx = 2 * (a_long ? op.la : op.lb), ny = 2 * (a_long ? op.lb : op.la);
    uint32_t* rr = reinterpret_cast<uint32_t*>(P.out + op.r_off);
    const uint32_t rlen = 2 * (op.la + op.lb);
    constexpr uint32_t W = NT * T;
    // the shorter operand y is the broadcast side (its nby blocks set the
    // steps of every chunk), chunks of x are the two-plane side
    const uint32_t nby = (ny + T - 1) / T;
    uint4 nxt[T / 4];
    load_chunk_regs<NT>(nxt, y, ny, 0, t);
#pragma unroll
    for (int it = 0; it < T / 4; ++it) {  // 16-byte slot v: half v%2 of block v/2
        const uint32_t v = t + it * NT;
        reinterpret_cast<uint4*>(gA)[(v >> 1) * 2 * G + (v & 1)] = nxt[it];
    }
    uint32_t pend[T];
#pragma unroll
    for (int w = 0; w < T; ++w) pend[w] = 0;
    // chunk c+1 of x is loaded into registers while chunk c is multiplied
    load_chunk_regs<NT>(nxt, x, nx, 0, t);
    for (uint32_t c = 0; c < chunks; ++c) {
#pragma unroll
        for (int it = 0; it < T / 4; ++it) {  // half v%2 of block v/2, plane layout
            const uint32_t v = t + it * NT;
            gB4[(v & 1) * G * NT + (v >> 1)] = nxt[it];
        }
        if (c + 1 < chunks) load_chunk_regs<NT>(nxt, x, nx, (c + 1) * W, t);
        group_sync<NT>();
        // the chunk's product plus the pending window, carried in one pass:
        // the low half (limbs [cW, (c+1)W)) is final and the high half becomes
        // the next window (the sum fits the 2W limbs: no carry out)
        uint32_t ulo[T], uhi[T];
        classic::square_product<NT, G>(gA, gB4, slots, scr, t, ulo, uhi, valid ? (nby ? nby : 1u) : 1u, pend);
        if (valid) classic::store_pairs(rr, c * W + t * T, rlen, ulo);
#pragma unroll
        for (int w = 0; w < T; ++w) pend[w] = uhi[w];
        group_sync<NT>();  // gA and the slots are reused by the next chunk
    }
    if (valid) classic::store_pairs(rr, chunks * W + t * T, rlen, pend);
}

// --- 32-thread products over rounds of output blocks --------------------------
//
// A product whose shorter operand y has nby <= 32 blocks (of T words) and
// whose longer operand x has `chunks` chunks of 32 blocks, one warp.  Round c
// gives lane t the whole anti-diagonal of output block 32c + t:
//   D = sum over k < nby of y_k * x_(32c + t - k),
// whose x blocks lie in chunk c (k <= t) or chunk c - 1 (k > t).  Both chunks
// sit in shared memory (two plane buffers, alternating), so a lane's tiles of
// one round all land on one output block: one accumulator, no snapshot, and
// one output block per lane per round.  Only the first round wraps: chunk 0's
// lower anti-diagonals (blocks 0..31) share the lanes with the last chunk's
// upper ones (blocks 32 chunks + t), split by a snapshot as in the square
// product; the upper values wait in shared memory for the last round.  Each
// round resolves its blocks L_t + H_(t-1) + O_(t-2) with the words of the
// previous round's last two anti-diagonals and its carries, so the blocks
// come out final in order.  (A chunked square product per chunk spends a
// snapshot per step and a two-block resolution per lane on every chunk.)

// Warp area (CLS_WARP_WORDS words): y blocks [0, 256), plane buffer 0
// [256, 512), the snapshot slots [512, 1792), plane buffer 1 [1792, 2048).

// Writes thread t's two 16-byte slots of a chunk (load_chunk_regs<32>) into a
// plane buffer: half h of block j at slot h*32 + j.
__device__ __forceinline__ void store_planes32(uint4* buf, const uint4 (&q)[classic::T / 4], uint32_t t) {
#pragma unroll
    for (int it = 0; it < classic::T / 4; ++it) {
        const uint32_t v = t + uint32_t(it) * 32;
        buf[(v & 1) * 32 + (v >> 1)] = q[it];
    }
}

// One round's tiles: lane t accumulates y_k * x-block (t - k) mod 32 of `cur`
// (k <= t) or `prev` (k > t), k < nby.  SNAP: the wrap round, whose lane t
// snapshots its accumulator at step min(t, nby - 1) (its lower anti-diagonal
// complete).
template <bool SNAP>
__device__ __forceinline__ void rect_tiles(const uint32_t* gA, const uint4* cur, const uint4* prev, uint2* slots,
                                           uint32_t t, uint32_t nby, classic::DiagAcc& s) {
    using classic::T;
#pragma unroll
    for (int w = 0; w < 2 * T; ++w) s.a[w] = 0;
#pragma unroll
    for (int w = 0; w < 2 * T - 2; ++w) s.b[w] = 0;
#pragma unroll
    for (int w = 0; w < T + 1; ++w) s.cc[w] = 0;
    const uint32_t snap_k = t < nby ? t : nby - 1;
#pragma unroll 4
    for (uint32_t k = 0; k < nby; ++k) {
        const uint32_t j = (t - k) & 31u;
        const uint4* src = k <= t ? cur : prev;
        const uint4 a0 = reinterpret_cast<const uint4*>(gA + k * T)[0];
        const uint4 a1 = reinterpret_cast<const uint4*>(gA + k * T)[1];
        const uint4 b0 = src[j], b1 = src[32 + j];
        uint32_t A[T], B[T];
        A[0] = a0.x; A[1] = a0.y; A[2] = a0.z; A[3] = a0.w;
        A[4] = a1.x; A[5] = a1.y; A[6] = a1.z; A[7] = a1.w;
        B[0] = b0.x; B[1] = b0.y; B[2] = b0.z; B[3] = b0.w;
        B[4] = b1.x; B[5] = b1.y; B[6] = b1.z; B[7] = b1.w;
        classic::tile_mac(A, B, s);
        if (SNAP && k == snap_k) {
#pragma unroll
            for (int w = 0; w < T; ++w) slots[w * 32 + t] = make_uint2(s.a[2 * w], s.a[2 * w + 1]);
#pragma unroll
            for (int w = 0; w < T - 1; ++w) slots[(T + w) * 32 + t] = make_uint2(s.b[2 * w], s.b[2 * w + 1]);
#pragma unroll
            for (int w = 0; w < T / 2; ++w)
                slots[(2 * T - 1 + w) * 32 + t] = make_uint2(s.cc[2 * w], s.cc[2 * w + 1]);
            slots[(2 * T - 1 + T / 2) * 32 + t] = make_uint2(s.cc[T], 0u);
        }
    }
}

// Output block blk0 + t from lane t's anti-diagonal value D (L = words 0..7,
// H = 8..15, O = 16): L_t + H_(t-1) + O_(t-2), lanes 0 and 1 taking the words
// of the previous round's lanes 31 and 30 from `cs` (zeros in the first
// round), then carried: kprev is the previous round's last add3 carry (0..2),
// cprev its lookahead carry out; both are updated for the next round.  Stores
// the block (clipped to rlen words) and leaves lane 31's H and O and lane
// 30's O in `cs`.
__device__ __forceinline__ void rect_epilogue(const uint32_t (&D)[classic::ACC], uint32_t* cs, uint32_t t,
                                              bool first, uint32_t& kprev, uint32_t& cprev, uint32_t* rr,
                                              uint32_t blk0, uint32_t rlen) {
    using classic::T;
    const uint32_t src1 = (t - 1) & 31u, src2 = (t - 2) & 31u;
    uint32_t L[T], H[T], r[T];
#pragma unroll
    for (int w = 0; w < T; ++w) {
        const uint32_t v = __shfl_sync(MI_FULL_MASK, D[T + w], src1);
        H[w] = t ? v : (first ? 0u : cs[w]);
        L[w] = D[w];
    }
    const uint32_t o = __shfl_sync(MI_FULL_MASK, D[2 * T], src2);
    const uint32_t O = t >= 2 ? o : (first ? 0u : cs[t == 0 ? T + 1 : T]);
    __syncwarp();  // lanes 0 and 1 have read the previous round's words
    if (t == 31) {
#pragma unroll
        for (int w = 0; w < T; ++w) cs[w] = D[T + w];
        cs[T] = D[2 * T];
    }
    if (t == 30) cs[T + 1] = D[2 * T];
    const uint32_t k = classic::add3_block(L, H, O, r);
    const uint32_t up = __shfl_up_sync(MI_FULL_MASK, k, 1);
    const uint32_t e = classic::add_word_block(r, t ? up : kprev);
    uint32_t cout;
    const uint32_t c = group_carry<32>(e != 0, classic::all_ones(r), cprev, &cout, nullptr);
    classic::add_word_block(r, c);
    classic::store_pairs(rr, (blk0 + t) * T, rlen, r);
    kprev = __shfl_sync(MI_FULL_MASK, k, 31);
    cprev = cout;
}

__device__ __forceinline__ void rect32_task(const Params& P, const Task& tk, uint32_t* sm) {
    using classic::ACC;
    using classic::PAIRS;
    using classic::T;
    const uint32_t t = threadIdx.x & 31u;
    const uint32_t chunks = tk.key - KEY_R32 + 1;  // 1..8 chunks of 32 blocks
    const uint32_t* sorted = P.scr + Scratch::sorted(P.n_ops);
    const mi_op op = P.ops[sorted[tk.first]];
    const bool a_long = op.la >= op.lb;
    const uint32_t* x = reinterpret_cast<const uint32_t*>(P.in + (a_long ? op.a_off : op.b_off));
    const uint32_t* y = reinterpret_cast<const uint32_t*>(P.in + (a_long ? op.b_off : op.a_off));
    const uint32_t nx = 2 * (a_long ? op.la : op.lb), ny = 2 * (a_long ? op.lb : op.la);
    uint32_t* rr = reinterpret_cast<uint32_t*>(P.out + op.r_off);
    const uint32_t rlen = 2 * (op.la + op.lb);
    const uint32_t nby = (ny + T - 1) / T;
    constexpr uint32_t W = 32 * T;  // words of a chunk
    uint32_t* gA = sm;
    uint4* buf0 = reinterpret_cast<uint4*>(sm + 256);
    uint2* slots = reinterpret_cast<uint2*>(sm + 512);
    uint4* buf1 = reinterpret_cast<uint4*>(sm + 512 + 32 * classic::PER_T);
    uint32_t* cs = sm + 512 + 2 * 10 * 32;  // snapshot pairs 10.. of lanes 0..4, free after the wrap round
    const uint32_t last = chunks - 1;

    uint4 q[T / 4];
    load_chunk_regs<32>(q, y, ny, 0, t);
#pragma unroll
    for (int it = 0; it < T / 4; ++it) reinterpret_cast<uint4*>(gA)[t + it * 32] = q[it];
    load_chunk_regs<32>(q, x, nx, 0, t);
    store_planes32(buf0, q, t);
    if (last) {
        load_chunk_regs<32>(q, x, nx, last * W, t);
        store_planes32(buf1, q, t);
    }
    uint4 nxt[T / 4];
    if (chunks > 2) load_chunk_regs<32>(nxt, x, nx, W, t);  // chunk 1; buf1 holds the last chunk until then
    __syncwarp();

    // the wrap round: chunk 0's lower anti-diagonals and the last chunk's upper ones
    classic::DiagAcc s;
    rect_tiles<true>(gA, buf0, last ? buf1 : buf0, slots, t, nby, s);
    uint32_t d1[ACC], d2[ACC];
    {
        uint32_t snap[2 * PAIRS];
#pragma unroll
        for (int w = 0; w < PAIRS; ++w) {
            const uint2 v = slots[w * 32 + t];
            snap[2 * w] = v.x;
            snap[2 * w + 1] = v.y;
        }
        classic::fold(snap, snap + 2 * T, snap + 4 * T - 2, d1);
        classic::fold(s.a, s.b, s.cc, d2);
        sub_cc(d2[0], d1[0]);
#pragma unroll
        for (int w = 1; w < ACC - 1; ++w) subc_cc(d2[w], d1[w]);
        subc(d2[ACC - 1], d1[ACC - 1]);
    }
#pragma unroll
    for (int w = 0; w < ACC / 2; ++w) slots[w * 32 + t] = make_uint2(d2[2 * w], d2[2 * w + 1]);  // own pairs 0..8
    slots[(ACC / 2) * 32 + t] = make_uint2(d2[ACC - 1], 0u);
    uint32_t kprev = 0, cprev = 0;
    rect_epilogue(d1, cs, t, true, kprev, cprev, rr, 0, rlen);

    for (uint32_t c = 1; c < chunks; ++c) {
        uint4* cur = (c & 1) ? buf1 : buf0;
        const uint4* prev = (c & 1) ? buf0 : buf1;
        if (c > 1 || chunks > 2) {  // chunk c replaces chunk c - 2 (or, for c = 1, the last chunk)
            __syncwarp();
            store_planes32(cur, nxt, t);
            if (c + 1 < chunks) load_chunk_regs<32>(nxt, x, nx, (c + 1) * W, t);
        }
        __syncwarp();
        rect_tiles<false>(gA, cur, prev, slots, t, nby, s);
        classic::fold(s.a, s.b, s.cc, d1);
        rect_epilogue(d1, cs, t, false, kprev, cprev, rr, c * 32, rlen);
    }
    // the last chunk's upper anti-diagonals, kept since the wrap round
#pragma unroll
    for (int w = 0; w < ACC / 2; ++w) {
        const uint2 v = slots[w * 32 + t];
        d2[2 * w] = v.x;
        d2[2 * w + 1] = v.y;
    }
    d2[ACC - 1] = slots[(ACC / 2) * 32 + t].x;
    __syncwarp();  // the last round's words in cs are visible
    rect_epilogue(d2, cs, t, false, kprev, cprev, rr, chunks * 32, rlen);
    __syncwarp();  // the warp's area is reused by its next task
}

// The R x C-word product of A and B in one parity-split accumulator, as
// classic::tile_mac does for 8 x 8 tiles: products with i + j even go to a
// (pairs at even columns), those with i + j odd to b (column k + 1 at b[k]),
// so every (lo, hi) pair is one wide multiply-add; each row is two carry
// chains whose single carry-outs land in cc (column C + i at cc[i]).
template <int R, int C>
struct RectAcc {
    uint32_t a[R + C], b[R + C - 2], cc[R + 1];
};

template <int R, int C>
__device__ __forceinline__ void rect_mac(const uint32_t (&A)[R], const uint32_t (&B)[C], RectAcc<R, C>& s) {
#pragma unroll
    for (int i = 0; i < R; ++i) {
        const int j0 = i & 1, j1 = 1 - j0;
        mad_lo_cc(s.a[i + j0], A[i], B[j0]);
        madc_hi_cc(s.a[i + j0 + 1], A[i], B[j0]);
#pragma unroll
        for (int j = j0 + 2; j < C; j += 2) {
            madc_lo_cc(s.a[i + j], A[i], B[j]);
            madc_hi_cc(s.a[i + j + 1], A[i], B[j]);
        }
        addc(s.cc[i + j0], 0u);
        mad_lo_cc(s.b[i + j1 - 1], A[i], B[j1]);
        madc_hi_cc(s.b[i + j1], A[i], B[j1]);
#pragma unroll
        for (int j = j1 + 2; j < C; j += 2) {
            madc_lo_cc(s.b[i + j - 1], A[i], B[j]);
            madc_hi_cc(s.b[i + j], A[i], B[j]);
        }
        addc(s.cc[i + j1], 0u);
    }
}

// The R + C words of the product from its accumulator (which fits them).
template <int R, int C>
__device__ __forceinline__ void rect_fold(RectAcc<R, C>& s, uint32_t (&f)[R + C]) {
#pragma unroll
    for (int c = 0; c < R + C; ++c) f[c] = s.a[c];
    add_cc(f[1], s.b[0]);
#pragma unroll
    for (int k = 1; k < R + C - 2; ++k) addc_cc(f[k + 1], s.b[k]);
    addc(f[R + C - 1], 0u);
    add_cc(f[C], s.cc[0]);
#pragma unroll
    for (int i = 1; i < R; ++i) addc_cc(f[C + i], s.cc[i]);
}

// Comb products, shorter operand y of at most 8 limbs (16 words, held in
// registers by every thread of the group): thread t multiplies its 16 words
// of the longer operand x by y (one parity-split accumulator, rect_mac), keeps
// the low 16 words and hands the high 16 to thread t+1, whose low words they
// overlap; one carry-lookahead pass over the group makes 16 result words per
// thread final, and the last thread's high words plus the carry-out open the
// next pass (512 words of x per pass of a warp) -- a few passes where the
// chunked square products would chain one chunk per 8 or 16 words.
template <int G>
__device__ __forceinline__ void comb_task(const Params& P, const Task& tk) {
    constexpr int K = 16, NBW = 16;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t g = lane / G, t = lane % G;
    if (g >= tk.count) return;  // groups synchronise only among their own lanes
    const uint32_t ki = tk.key - KEY_CMB;
    const uint32_t passes = ki < 3 ? 1u : ki - 2;
    const uint32_t* sorted = P.scr + Scratch::sorted(P.n_ops);
    const mi_op op = P.ops[sorted[tk.first + g]];
    const bool a_long = op.la >= op.lb;
    const uint32_t* x = reinterpret_cast<const uint32_t*>(P.in + (a_long ? op.a_off : op.b_off));
    const uint32_t* y = reinterpret_cast<const uint32_t*>(P.in + (a_long ? op.b_off : op.a_off));
    const uint32_t nx = 2 * (a_long ? op.la : op.lb), ny = 2 * (a_long ? op.lb : op.la);
    uint32_t* rr = reinterpret_cast<uint32_t*>(P.out + op.r_off);
    const uint32_t rlen = 2 * (op.la + op.lb);
    const uint32_t mask = group_lanes<G>();
    uint32_t B[NBW];
#pragma unroll
    for (int j = 0; j < NBW; j += 2) {  // limbs are 8-byte aligned pairs of words
        const uint2 v = uint32_t(j + 2) <= ny ? __ldg(reinterpret_cast<const uint2*>(y + j)) : make_uint2(0, 0);
        B[j] = v.x;
        B[j + 1] = v.y;
    }
    uint32_t pend[NBW];
#pragma unroll
    for (int j = 0; j < NBW; ++j) pend[j] = 0;
    for (uint32_t p = 0; p < passes; ++p) {
        const uint32_t base = (p * G + t) * K;
        uint32_t a[K];
#pragma unroll
        for (int i = 0; i < K; i += 2) {
            const uint2 v = base + i + 2 <= nx ? __ldcs(reinterpret_cast<const uint2*>(x + base + i)) : make_uint2(0, 0);
            a[i] = v.x;
            a[i + 1] = v.y;
        }
        uint32_t acc[K + NBW];
        {
            RectAcc<K, NBW> ra;
#pragma unroll
            for (int w = 0; w < K + NBW; ++w) ra.a[w] = 0;
#pragma unroll
            for (int w = 0; w < K + NBW - 2; ++w) ra.b[w] = 0;
#pragma unroll
            for (int w = 0; w <= K; ++w) ra.cc[w] = 0;
            rect_mac<K, NBW>(a, B, ra);
            rect_fold<K, NBW>(ra, acc);
        }
        // words [base, base + K): the low words plus the previous thread's
        // high words (the pending words for the group's first thread)
        uint32_t lo[K], hin[K], out[K];
#pragma unroll
        for (int j = 0; j < K; ++j) {
            const uint32_t v = __shfl_up_sync(mask, acc[K + j], 1, G);
            hin[j] = t == 0 ? pend[j] : v;
            lo[j] = acc[j];
        }
        bool gg, pp;
        uint32_t gc;
        chunk_add<uint32_t, K>(lo, hin, out, gg, pp);
        chunk_inc<uint32_t, K>(out, group_carry<G>(gg, pp, 0u, &gc, nullptr));
#pragma unroll
        for (int w = 0; w < K; w += 2)  // rows are 8-byte aligned and rlen even
            if (base + w < rlen) *reinterpret_cast<uint2*>(rr + base + w) = make_uint2(out[w], out[w + 1]);
        // the last thread's high words plus the group's carry-out open the next pass
        uint32_t c = gc;
#pragma unroll
        for (int j = 0; j < NBW; ++j) {
            const uint64_t v = uint64_t(__shfl_sync(mask, acc[K + j], G - 1, G)) + c;
            pend[j] = uint32_t(v);
            c = uint32_t(v >> 32);
        }
    }
    if (t == 0) {
        const uint32_t top = passes * G * K;
#pragma unroll
        for (int w = 0; w < NBW; w += 2)
            if (top + w < rlen) *reinterpret_cast<uint2*>(rr + top + w) = make_uint2(pend[w], pend[w + 1]);
    }
}

__global__ void __launch_bounds__(256, 2) k_rg_classic(Params P) {
    extern __shared__ __align__(16) uint32_t smem32[];
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    uint32_t* wsm = smem32 + warp * CLS_WARP_WORDS;
    __shared__ FamTab tab;
    const uint32_t ntasks = P.scr[Scratch::NTASKS + 1];
    pdl_trigger();
    load_tab(tab, P.scr, 1);
    __syncthreads();
    // each warp fetches its next task index while the current task runs
    uint32_t next = 0;
    if (lane == 0) next = atomicAdd(P.scr + Scratch::QUEUE + 1, 1u);
    for (;;) {
        const uint32_t t = __shfl_sync(MI_FULL_MASK, next, 0);
        if (t >= ntasks) break;
        if (lane == 0) next = atomicAdd(P.scr + Scratch::QUEUE + 1, 1u);
        const Task tk = decode_tab<1>(tab, t);
        switch (tk.key - KEY_CLS) {
            case 0: classic_task<1>(P, tk, wsm, nullptr); break;
            case 1: classic_task<2>(P, tk, wsm, nullptr); break;
            case 2: classic_task<4>(P, tk, wsm, nullptr); break;
            case 3: classic_task<8>(P, tk, wsm, nullptr); break;
            default: classic_task<16>(P, tk, wsm, nullptr); break;
        }
        __syncwarp();
    }
    pdl_wait();  // complete only after the task kernel launched before it
}

// 32-thread products over rounds (shorter operand of 17..128 limbs below the
// NTT crossover, or a longer one of more than 64): a family and a kernel of
// their own.  Two CTAs per SM at up to 128 registers: at three (80 registers)
// the tile loop could no longer read a few steps' operands ahead, and the
// list ran 1.62 ms (unrolled 2 deep, 48 bytes spilled) or 1.70 ms (not
// unrolled) against 1.51 ms.
__global__ void __launch_bounds__(256, 2) k_rg_r32(Params P) {
    extern __shared__ __align__(16) uint32_t smem32[];
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    uint32_t* wsm = smem32 + warp * R32_WARP_WORDS;
    __shared__ FamTab tab;
    const uint32_t ntasks = P.scr[Scratch::NTASKS + 7];
    pdl_trigger();
    load_tab(tab, P.scr, 7);
    __syncthreads();
    uint32_t next = 0;  // the next task index, fetched while the current task runs
    if (lane == 0) next = atomicAdd(P.scr + Scratch::QUEUE + 7, 1u);
    for (;;) {
        const uint32_t t = __shfl_sync(MI_FULL_MASK, next, 0);
        if (t >= ntasks) break;
        if (lane == 0) next = atomicAdd(P.scr + Scratch::QUEUE + 7, 1u);
        rect32_task(P, decode_tab<7>(tab, t), wsm);
    }
    pdl_wait();  // complete only after the task kernel launched before it
}

// Comb products (shorter operand of at most 8 limbs): a family and a kernel
// of their own, so that neither these nor the square products carry the
// other's code and registers.
__global__ void __launch_bounds__(256, 2) k_rg_comb(Params P) {
    const uint32_t lane = threadIdx.x & 31u;
    __shared__ FamTab tab;
    const uint32_t ntasks = P.scr[Scratch::NTASKS + 5];
    pdl_trigger();
    load_tab(tab, P.scr, 5);
    __syncthreads();
    uint32_t next = 0;  // the next task index, fetched while the current task runs
    if (lane == 0) next = atomicAdd(P.scr + Scratch::QUEUE + 5, 1u);
    for (;;) {
        const uint32_t t = __shfl_sync(MI_FULL_MASK, next, 0);
        if (t >= ntasks) break;
        if (lane == 0) next = atomicAdd(P.scr + Scratch::QUEUE + 5, 1u);
        const Task tk = decode_tab<5>(tab, t);
        const uint32_t ki = tk.key - KEY_CMB;
        if (ki == 0) comb_task<4>(P, tk);
        else if (ki == 1) comb_task<8>(P, tk);
        else if (ki == 2) comb_task<16>(P, tk);
        else comb_task<32>(P, tk);
        __syncwarp();
    }
    pdl_wait();  // complete only after the task kernel launched before it
}

// Products whose shorter operand has 129..256 limbs (below the NTT crossover):
// four 64-thread groups per block, one task = up to four products of one key.
__global__ void __launch_bounds__(256, 2) k_rg_c64(Params P) {
    extern __shared__ __align__(16) uint32_t smem32[];
    __shared__ uint32_t scr_warp[8];
    __shared__ uint32_t s_task[2];
    __shared__ FamTab tab;
    const uint32_t ntasks = P.scr[Scratch::NTASKS + 3];
    pdl_trigger();
    load_tab(tab, P.scr, 3);
    if (threadIdx.x == 0) s_task[0] = atomicAdd(P.scr + Scratch::QUEUE + 3, 1u);
    __syncthreads();
    for (uint32_t it = 0;; ++it) {
        const uint32_t t = s_task[it & 1];
        if (t >= ntasks) break;
        if (threadIdx.x == 0) s_task[(it + 1) & 1] = atomicAdd(P.scr + Scratch::QUEUE + 3, 1u);
        classic_task<64>(P, decode_tab<3>(tab, t), smem32, scr_warp);
        __syncthreads();  // the next index is visible; shared memory is reused
    }
    pdl_wait();  // complete only after the task kernel launched before it
}

// --- addition family -------------------------------------------------------------
//
// Warp tasks.  Additions of at most 32 limbs: groups of GS = pow2ceil(m)
// lanes, one limb per lane, 32/GS additions per task, one carry-lookahead
// pass per group.  Longer additions: one warp per addition, lane i of row r
// owning limb 32r + i, so every load and store of the warp is 256 contiguous
// bytes; rows are loaded eight at a time and resolved in order, each row's
// carry-out entering the next row's lookahead.

template <int GS>
__device__ __forceinline__ void add_short(const Params& P, const Task& tk) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t g = lane / GS, t = lane % GS;
    if (g >= tk.count) return;  // groups vote only among their own lanes
    const uint32_t* sorted = P.scr + Scratch::sorted(P.n_ops);
    const uint32_t idx = sorted[tk.first + g];
    const mi_op op = P.ops[idx];
    const uint32_t m = max(op.la, op.lb);
    const uint64_t x = t < op.la ? __ldcs(reinterpret_cast<const unsigned long long*>(P.in + op.a_off + t)) : 0;
    const uint64_t y = t < op.lb ? __ldcs(reinterpret_cast<const unsigned long long*>(P.in + op.b_off + t)) : 0;
    uint64_t s = x + y;
    uint32_t gc;
    s += group_carry<GS>(s < x, s == ~0ull, 0u, &gc, nullptr);
    if (t < m) P.out[op.r_off + t] = s;
    if (P.carry != nullptr) {
        if (t == m) P.carry[idx] = uint8_t(s);                     // limb m holds the carry-out
        else if (m == GS && t == GS - 1) P.carry[idx] = uint8_t(gc);
    }
}

// Rows r0 .. r0+RB-1 of an addition (lane i of row r: limb 32r + i), zero
// past each operand.
template <int RB>
__device__ __forceinline__ void load_rows(const unsigned long long* __restrict__ ar,
                                          const unsigned long long* __restrict__ br, uint32_t la, uint32_t lb,
                                          uint32_t r0, uint32_t lane, uint64_t (&x)[RB], uint64_t (&y)[RB]) {
#pragma unroll
    for (int r = 0; r < RB; ++r) {
        const uint32_t i = (r0 + r) * 32 + lane;
        x[r] = i < la ? __ldcs(ar + i) : 0;
        y[r] = i < lb ? __ldcs(br + i) : 0;
    }
}

// Sums rows r0 .. of x + y in order, each row's carry-out entering the next
// row's lookahead, and stores them (limb m, past the sum, is the carry-out).
template <int RB>
__device__ __forceinline__ void resolve_rows(const uint64_t (&x)[RB], const uint64_t (&y)[RB], uint32_t r0,
                                             uint32_t rows, uint32_t m, uint32_t lane, uint32_t& carry,
                                             uint64_t* __restrict__ rr, uint8_t* cflag) {
#pragma unroll
    for (int r = 0; r < RB; ++r) {
        if (r0 + r >= rows) break;  // uniform across the warp
        const uint32_t i = (r0 + r) * 32 + lane;
        uint64_t s = x[r] + y[r];
        uint32_t gc;
        s += group_carry<32>(s < x[r], s == ~0ull, carry, &gc, nullptr);
        carry = gc;
        if (i < m) __stcs(reinterpret_cast<unsigned long long*>(rr + i), s);
        else if (i == m && cflag != nullptr) *cflag = uint8_t(s);
    }
}

// One warp per addition of more than 32 limbs: batches of RB rows, the next
// batch's loads issued before the current batch is resolved, so that two
// batches are in flight while the carries of one are resolved.  The task's
// op descriptors are fetched at once into the warp's slots `desc` (lane o
// fetches op o's), so the ops of a task pay one descriptor latency.  Three
// 256-thread blocks per SM at up to 80 registers (at four, 64 registers, the
// descriptors spilled): the addition band of the 200000-op list 0.1115 ->
// 0.1055 ms against one batch of eight rows in flight; tasks of two or
// eight additions instead of four measured slower (0.110, 0.145 ms).
struct AddDesc {
    uint32_t idx, la, lb, pad;
    uint64_t a_off, b_off, r_off;
};

__device__ __forceinline__ void add_rows(const Params& P, const Task& tk, AddDesc* desc) {
    constexpr int RB = kAddRowBatch;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t* sorted = P.scr + Scratch::sorted(P.n_ops);
    if (lane < tk.count) {
        const uint32_t idx = sorted[tk.first + lane];
        const mi_op op = P.ops[idx];
        desc[lane] = AddDesc{idx, op.la, op.lb, 0u, op.a_off, op.b_off, op.r_off};
    }
    __syncwarp();
    for (uint32_t o = 0; o < tk.count; ++o) {
        const AddDesc d = desc[o];
        const uint32_t m = max(d.la, d.lb), rows = (m + 31) / 32;
        const unsigned long long* ar = reinterpret_cast<const unsigned long long*>(P.in + d.a_off);
        const unsigned long long* br = reinterpret_cast<const unsigned long long*>(P.in + d.b_off);
        uint64_t* rr = P.out + d.r_off;
        uint8_t* cflag = P.carry != nullptr ? P.carry + d.idx : nullptr;
        uint32_t carry = 0;
        uint64_t xa[RB], ya[RB], xb[RB], yb[RB];
        load_rows<RB>(ar, br, d.la, d.lb, 0, lane, xa, ya);
        for (uint32_t r0 = 0; r0 < rows; r0 += 2 * RB) {
            if (r0 + RB < rows) load_rows<RB>(ar, br, d.la, d.lb, r0 + RB, lane, xb, yb);
            resolve_rows<RB>(xa, ya, r0, rows, m, lane, carry, rr, cflag);
            if (r0 + RB >= rows) break;
            if (r0 + 2 * RB < rows) load_rows<RB>(ar, br, d.la, d.lb, r0 + 2 * RB, lane, xa, ya);
            resolve_rows<RB>(xb, yb, r0 + RB, rows, m, lane, carry, rr, cflag);
        }
        if (cflag != nullptr && m % 32 == 0 && lane == 0) *cflag = uint8_t(carry);
    }
    __syncwarp();  // the slots are rewritten by the warp's next task
}

__global__ void __launch_bounds__(256, 3) k_rg_add(Params P) {
    const uint32_t lane = threadIdx.x & 31u;
    __shared__ FamTab tab;
    __shared__ AddDesc desc[8][kAddRowOps];  // each warp's descriptor slots
    const uint32_t ntasks = P.scr[Scratch::NTASKS + 2];
    pdl_trigger();
    load_tab(tab, P.scr, 2);
    __syncthreads();
    uint32_t next = 0;  // the next task index, fetched while the current task runs
    if (lane == 0) next = atomicAdd(P.scr + Scratch::QUEUE + 2, 1u);
    for (;;) {
        const uint32_t t = __shfl_sync(MI_FULL_MASK, next, 0);
        if (t >= ntasks) break;
        if (lane == 0) next = atomicAdd(P.scr + Scratch::QUEUE + 2, 1u);
        const Task tk = decode_tab<2>(tab, t);
        switch (tk.key - KEY_ADD) {
            case 0: add_short<1>(P, tk); break;
            case 1: add_short<2>(P, tk); break;
            case 2: add_short<4>(P, tk); break;
            case 3: add_short<8>(P, tk); break;
            case 4: add_short<16>(P, tk); break;
            case 5: add_short<32>(P, tk); break;
            default: add_rows(P, tk, desc[threadIdx.x >> 5]); break;
        }
        __syncwarp();
    }
    pdl_wait();  // complete only after the task kernel launched before it
}

// --- host side -------------------------------------------------------------------

constexpr size_t kNttSmem = ntt32::MulSmem<11>::WORDS32 * 4 + 64;
constexpr size_t kClsSmem = size_t(8) * CLS_WARP_WORDS * 4;
constexpr size_t kR32Smem = size_t(8) * R32_WARP_WORDS * 4;
constexpr size_t kC64Smem = size_t(4) * C64_GROUP_WORDS * 4;

std::mutex g_init_mu;
bool g_init[64] = {};

mi_status init_device() {
    int dev = 0;
    MI_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return set_error(MI_ENODEV, "device %d out of range", dev);
    std::lock_guard<std::mutex> lk(g_init_mu);
    if (g_init[dev]) return MI_OK;
    // keys of each family in descending cost
    std::vector<uint16_t> order(K);
    for (int k = 0; k < K_NTT; ++k) order[KEY_NTT + k] = uint16_t(KEY_NTT + (K_NTT - 1 - k));
    // classical keys by descending cost: groups of 16, 8, 4, 2, 1 threads (one
    // chunk each); 32-thread products from 8 chunks down to 1
    for (int k = 0; k < K_CLS; ++k) order[KEY_CLS + k] = uint16_t(KEY_CLS + (K_CLS - 1 - k));
    for (int k = 0; k < K_R32; ++k) order[KEY_R32 + k] = uint16_t(KEY_R32 + (K_R32 - 1 - k));
    // the comb family, the most passes first
    const int comb[K_CMB] = {6, 5, 4, 3, 2, 1, 0};
    for (int k = 0; k < K_CMB; ++k) order[KEY_CMB + k] = uint16_t(KEY_CMB + comb[k]);
    for (int k = 0; k < K_ADD; ++k) order[KEY_ADD + k] = uint16_t(KEY_ADD + (K_ADD - 1 - k));
    for (int k = 0; k < K_C64; ++k) order[KEY_C64 + k] = uint16_t(KEY_C64 + (K_C64 - 1 - k));
    for (int k = 0; k < K_N48; ++k) order[KEY_N48 + k] = uint16_t(KEY_N48 + (K_N48 - 1 - k));
    for (int k = 0; k < K_N40; ++k) order[KEY_N40 + k] = uint16_t(KEY_N40 + (K_N40 - 1 - k));
    MI_CUDA_TRY(cudaMemcpyToSymbol(c_order, order.data(), sizeof(uint16_t) * K));
    MI_CUDA_TRY(cudaFuncSetAttribute(k_rg_ntt<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kNttSmem)));
    MI_CUDA_TRY(cudaFuncSetAttribute(k_rg_ntt<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kNttSmem)));
    MI_CUDA_TRY(cudaFuncSetAttribute(k_rg_ntt<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kNttSmem)));
    MI_CUDA_TRY(cudaFuncSetAttribute(k_rg_classic, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kClsSmem)));
    MI_CUDA_TRY(cudaFuncSetAttribute(k_rg_r32, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kR32Smem)));
    MI_CUDA_TRY(cudaFuncSetAttribute(k_rg_c64, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kC64Smem)));
    g_init[dev] = true;
    return MI_OK;
}

int persistent_grid(const void* kern, size_t smem) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 256, smem) != cudaSuccess || per_sm < 1)
        per_sm = 1;
    return sm_count() * per_sm;
}

}  // namespace rg

mi_status ragged_launch(mi_ctx ctx, const mi_op* ops, uint32_t n_ops, const uint64_t* in, uint64_t* out,
                        uint8_t* carry, void* scratch, size_t scratch_bytes, uint32_t ntt_min, cudaStream_t st) {
    using namespace rg;
    if (n_ops == 0) return MI_OK;
    if (ops == nullptr || in == nullptr || out == nullptr || scratch == nullptr)
        return set_error(MI_EINVAL, "ragged: null pointer");
    if (scratch_bytes < Scratch::words(n_ops) * 4) return set_error(MI_EINVAL, "ragged: scratch too small");
    MI_TRY(init_device());
    Params P;
    P.ops = ops;
    P.n_ops = n_ops;
    P.in = in;
    P.out = out;
    P.carry = carry;
    P.scr = static_cast<uint32_t*>(scratch);
    // classical groups hold at most 64 tiles (256 u64 limbs) of the shorter operand
    P.ntt_min = ntt_min < 1 ? 1 : (ntt_min > 257 ? 257 : ntt_min);
    P.ntt40_min = ctx->ragged_ntt40_min < 1 ? 1 : (ctx->ragged_ntt40_min > 257 ? 257 : ctx->ragged_ntt40_min);
    P.ntt = ctx->ntt.params;
    MI_CUDA_TRY(cudaMemsetAsync(P.scr, 0, (Scratch::KEYS) * 4, st));
    const uint32_t blocks = (n_ops + kBinRange - 1) / kBinRange;
    k_classify<<<blocks, 256, 0, st>>>(ops, n_ops, P.scr, P.ntt_min, P.ntt40_min);
    k_scan<<<1, 32 * NFAM, 0, st>>>(P.scr);  // the cursors were zeroed with the counts
    k_scatter<<<blocks, 256, 0, st>>>(n_ops, P.scr);
    // The task kernels: the first waits for the binning like any launch; each later one is a programmatic dependent launch that does not
    // wait at its start -- the families read the binned lists and write
    // disjoint results, so a kernel's blocks may start on the SMs that the
    // previous kernel's last tasks leave idle -- and waits for its predecessor
    // only before it completes, so that the last kernel completes after all.
    k_rg_ntt<0><<<persistent_grid((const void*)k_rg_ntt<0>, kNttSmem), 256, kNttSmem, st>>>(P);
    MI_CUDA_TRY(cudaGetLastError());
    MI_CUDA_TRY(launch_pdl(k_rg_ntt<1>, persistent_grid((const void*)k_rg_ntt<1>, kNttSmem), 256, kNttSmem, st, P));
    MI_CUDA_TRY(launch_pdl(k_rg_ntt<2>, persistent_grid((const void*)k_rg_ntt<2>, kNttSmem), 256, kNttSmem, st, P));
    MI_CUDA_TRY(launch_pdl(k_rg_r32, persistent_grid((const void*)k_rg_r32, kR32Smem), 256, kR32Smem, st, P));
    MI_CUDA_TRY(launch_pdl(k_rg_classic, persistent_grid((const void*)k_rg_classic, kClsSmem), 256, kClsSmem, st, P));
    // 64-thread classical groups serve shorter operands of 129..256 limbs below the crossover
    if (P.ntt_min > 129)
        MI_CUDA_TRY(launch_pdl(k_rg_c64, persistent_grid((const void*)k_rg_c64, kC64Smem), 256, kC64Smem, st, P));
    MI_CUDA_TRY(launch_pdl(k_rg_comb, persistent_grid((const void*)k_rg_comb, 0), 256, 0, st, P));
    MI_CUDA_TRY(launch_pdl(k_rg_add, persistent_grid((const void*)k_rg_add, 0), 256, 0, st, P));
    return MI_OK;
}

size_t ragged_scratch_words(uint32_t n_ops) { return rg::Scratch::words(n_ops); }
mi_status ragged_prepare() { return rg::init_device(); }

// --- the allocation-free variant ---------------------------------------------------
//
// Scratch for callers that cannot allocate device memory: a file-scope device
// array sized for at most MI_RAGGED_NOALLOC_MAX_OPS ops (about 0.5 MiB, held by
// every GPU that loads the library until the process exits).  In host code
// `g_noalloc_scratch` names a host-side stand-in, not device memory; the device
// address comes from cudaGetSymbolAddress, once per device, with that device
// current, on the first call there.
namespace rg {
static __device__ __align__(256) uint32_t g_noalloc_scratch[Scratch::words(MI_RAGGED_NOALLOC_MAX_OPS)];
std::mutex g_noalloc_mu;
void* g_noalloc_ptr[64] = {};

mi_status noalloc_scratch(void** out) {
    int dev = 0;
    MI_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return set_error(MI_ENODEV, "device %d out of range", dev);
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (g_noalloc_ptr[dev] == nullptr) {
        void* ptr = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_error(e, "cudaGetSymbolAddress(noalloc scratch)");
        g_noalloc_ptr[dev] = ptr;
    }
    *out = g_noalloc_ptr[dev];
    return MI_OK;
}
}  // namespace rg

}  // namespace mi

// Same work as mi_ragged_run, for callers that cannot allocate device memory
// (for example code that runs inside another framework's memory pool, or under
// a fixed device-memory budget, where a cudaMalloc would fail or is not
// allowed): the scratch is the library's static device array instead of a
// caller buffer.  No allocation, no free, no allocating library routine.
extern "C" mi_status mi_ragged_run_noalloc(mi_ctx ctx, const mi_op* ops, uint32_t n_ops, const uint64_t* in,
                                           uint64_t* out, uint8_t* carry_out, mi_stream stream) {
    using namespace mi;
    if (ctx == nullptr) return set_error(MI_EINVAL, "ragged_run_noalloc: null context");
    if (n_ops > MI_RAGGED_NOALLOC_MAX_OPS)
        return set_error(MI_EINVAL, "ragged_run_noalloc: %u ops exceed the static scratch limit of %u ops", n_ops,
                         MI_RAGGED_NOALLOC_MAX_OPS);
    if (n_ops == 0) return MI_OK;
    if (!aligned8(ops) || !aligned8(in) || !aligned8(out))
        return set_error(MI_EINVAL, "ragged_run_noalloc: ops, in and out must be 8-byte aligned");
    int cur = -1;
    MI_CUDA_TRY(cudaGetDevice(&cur));
    if (cur != ctx->device) MI_CUDA_TRY(cudaSetDevice(ctx->device));
    void* scratch = nullptr;
    MI_TRY(rg::noalloc_scratch(&scratch));
    return ragged_launch(ctx, ops, n_ops, in, out, carry_out, scratch, rg::Scratch::words(MI_RAGGED_NOALLOC_MAX_OPS) * 4,
                         ctx->ragged_ntt_min, reinterpret_cast<cudaStream_t>(stream));
}

// The skipped-op count of the last no-alloc run on the context's device, read
// from the static array (the count that mi_ragged_invalid reads from a caller
// scratch buffer).  Synchronous; allocates nothing.
extern "C" mi_status mi_ragged_invalid_noalloc(mi_ctx ctx, uint32_t* count) {
    using namespace mi;
    if (ctx == nullptr || count == nullptr) return set_error(MI_EINVAL, "ragged_invalid_noalloc: null pointer");
    int cur = -1;
    MI_CUDA_TRY(cudaGetDevice(&cur));
    if (cur != ctx->device) MI_CUDA_TRY(cudaSetDevice(ctx->device));
    void* scratch = nullptr;
    MI_TRY(rg::noalloc_scratch(&scratch));
    MI_CUDA_TRY(cudaMemcpy(count, static_cast<const uint32_t*>(scratch) + rg::Scratch::INVALID, 4,
                           cudaMemcpyDeviceToHost));
    return MI_OK;
}

namespace mi {
size_t ragged_invalid_word() { return rg::Scratch::INVALID; }

}  // namespace mi
