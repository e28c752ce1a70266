// ctx.h -- the context object behind mi_ctx (internal to the library).
#pragma once

#include <mutex>

#include <cuda_runtime.h>

#include "kernels.h"
#include "ntt_host.h"
#include "tuning_table.h"

struct mi_ctx_s {
    int device = 0;
    cudaStream_t stream = nullptr;
    mi::NttTables ntt;  // resident twiddles of the three NTT primes
    // host-pointer pipeline: a copy-in stream, a copy-out stream and two
    // compute streams over a ring of staging slots, ordered by events
    static constexpr int kSlots = 3;
    cudaStream_t pipe[4] = {};  // 0 copy-in, 1 copy-out, 2 and 3 compute
    cudaEvent_t ev_in[kSlots] = {}, ev_k[kSlots] = {}, ev_out[kSlots] = {};
    void* stage[kSlots] = {};
    size_t stage_cap = 0;
    // by operation class (0 additions, 1 multiplications): chunks of a large
    // host-buffer batch, and whether kernels read mapped pinned buffers in place
    uint32_t host_chunks[2] = {mi::tuned::kHostChunks[0], mi::tuned::kHostChunks[1]};
    uint32_t host_zero_copy[2] = {mi::tuned::kHostZeroCopy[0], mi::tuned::kHostZeroCopy[1]};
    // zero-copy mode 1: resident blocks per SM of the classical product (0: all that fit)
    uint32_t host_zc_blocks[2] = {mi::tuned::kHostZcBlocks[0], mi::tuned::kHostZcBlocks[1]};
    std::mutex mu;  // serialises host-pointer calls on one context
    // ragged batches: products whose shorter operand has at least this many
    // u64 limbs go through the NTT kernel (at most 257: classical groups hold
    // 256 limbs of the shorter operand)
    uint32_t ragged_ntt_min = mi::tuned::kRaggedNttMin;
    uint32_t ragged_ntt40_min = mi::tuned::kRaggedNtt40Min;
    // mi_mul_u64: square products of at least this many u64 limbs use the NTT
    uint32_t plain_ntt_min = mi::tuned::kPlainNttMin;
    // mi_mul_lo_u64 and the u64 gpuMultiply wrapper: low halves of products
    // of at least this many u64 limbs come from the NTT kernel
    uint32_t lo_ntt_min = mi::tuned::kLoNttMin;
    // mi_poly_u64: composites of at least this many u64 limbs run on the NTT
    uint32_t poly_ntt_min = mi::tuned::kPolyNttMin;
    // multi-block additions: tile status words, counter and error word
    mi::WideState wide;
    // addition: operand bytes per thread by size class ceil(log2(u64 limbs))
    uint8_t add_thread_bytes[13] = {};
    mi_ctx_s() {
        for (int c = 0; c < 13; ++c) add_thread_bytes[c] = mi::tuned::kAddThreadBytes[c];
    }
};

struct mi_graph_s {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int device = 0;
};
