// kernels.h -- host launchers of the device kernels (internal to the library).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/midint.h"

namespace mi {

enum AddOp : int { ADD_PLAIN = 0, ADD_SIX = 1 };

// Batched addition on u64 or u32 limbs (op = ADD_PLAIN or ADD_SIX).
// Arguments are already validated; n > 0, limbs > 0.
// Device state of the additions wider than one block (decoupled look-back):
// `status` holds kWideTiles tile words, then the 64-bit tile counter, then the
// error word (set when a bounded wait gave up).  One per context; wide
// additions on one context must not overlap on the device.  The host side
// keeps the epoch of the last launch and the counter values issued so far.
constexpr uint32_t kWideTiles = 1u << 16;
struct WideState {
    uint32_t* status = nullptr;    // kWideTiles + 4 words
    uint32_t epoch = 0;            // of the last launch (tile words carry it)
    uint64_t issued = 0;           // tile counter values taken by earlier launches
    uint32_t spin_limit = 1u << 20;  // polls of an unpublished predecessor before giving up
    uint32_t withhold = 0;         // tests only: first tiles never publish (makes the waits run out)
    uint32_t round_tiles = kWideTiles;  // tiles per launch (at most kWideTiles)
};

// thread_bytes: operand bytes each thread owns (16, 32 or 64; raised where the
// instance would need a group of more than 1024 threads).  Instances wider
// than one group (limbs above kAddMaxLimbs64 u64 limbs) take the multi-block
// kernel, which needs `wide`.
mi_status launch_add_u64(const uint64_t* a, const uint64_t* b, uint64_t* r, uint8_t* carry, uint32_t n,
                         uint32_t limbs, int op, uint32_t thread_bytes, cudaStream_t st,
                         WideState* wide = nullptr);
mi_status launch_add_u32(const uint32_t* a, const uint32_t* b, uint32_t* r, uint8_t* carry, uint32_t n,
                         uint32_t limbs, uint32_t thread_bytes, cudaStream_t st, WideState* wide = nullptr);
// Size class of an addition of `bytes` per operand: ceil(log2(u64 limbs)).
uint32_t add_size_class(uint64_t bytes);

// Classical multiplication on u32 limb views (a u64 buffer with m limbs is a
// u32 buffer with 2m limbs).  full: r has 2*n32 limbs per instance, else n32.
// max_per_sm > 0 caps the full-product kernel's resident blocks per SM (by
// its shared-memory request).
mi_status launch_mul_classic(const uint32_t* a, const uint32_t* b, uint32_t* r, uint32_t n, uint32_t n32,
                             bool full, cudaStream_t st, uint32_t max_per_sm = 0);

// Low n32 limbs of a*b per instance (u32 limb views), n32 > 8.
mi_status launch_mul_lo(const uint32_t* a, const uint32_t* b, uint32_t* r, uint32_t n, uint32_t n32, cudaStream_t st);

// ((a^2 + b)(b^2 + b) + ab) mod 2^(32*n32) per instance (u32 limb views).
mi_status launch_poly(const uint32_t* a, const uint32_t* b, uint32_t* r, uint32_t n, uint32_t n32, cudaStream_t st);

// GMP word-format conversions (convert.cu): fields of `words` words of `size`
// bytes (1, 2, 4, 8), order 1 / -1, endian 1 (big) / 0, -1 (little).
mi_status launch_import(const void* src, uint64_t* dst, uint32_t n, uint32_t words, uint32_t size, int order,
                        int endian, uint32_t limbs, cudaStream_t st);
mi_status launch_export(const uint64_t* src, void* dst, uint32_t n, uint32_t limbs, uint32_t words, uint32_t size,
                        int order, int endian, uint32_t* counts, cudaStream_t st);

// Ragged batches (ragged.cu): device scratch words for n_ops, the word that
// counts skipped ops, the one-time per-device setup (call outside stream
// capture) and the asynchronous launch sequence.
size_t ragged_scratch_words(uint32_t n_ops);
size_t ragged_invalid_word();
mi_status ragged_prepare();
mi_status ragged_launch(mi_ctx ctx, const mi_op* ops, uint32_t n_ops, const uint64_t* in, uint64_t* out,
                        uint8_t* carry, void* scratch, size_t scratch_bytes, uint32_t ntt_min, cudaStream_t st);

// Largest u32 limb count the classical kernel takes per instance.
constexpr uint32_t kMulMaxN32 = 4096;
// Largest u64 limb count the addition kernels take per instance (one group of
// at most 1024 threads, 4 limbs each).
constexpr uint32_t kAddMaxLimbs64 = 4096;
// Largest u64 limb count of one instance of the multi-block addition.
constexpr uint32_t kAddWideMaxLimbs64 = 1u << 26;

}  // namespace mi
