// ctx.h -- the context object behind mi_ctx (internal to the library).
#pragma once

#include <mutex>

#include <cuda_runtime.h>

#include "ntt_host.h"
#include "tuning_table.h"

struct mi_ctx_s {
    int device = 0;
    cudaStream_t stream = nullptr;
    mi::NttTables ntt;  // resident twiddles of the three NTT primes
    // host-pointer pipeline: two streams, each with its own device staging area
    cudaStream_t pipe[2] = {nullptr, nullptr};
    void* stage[2] = {nullptr, nullptr};
    size_t stage_cap = 0;
    std::mutex mu;  // serialises host-pointer calls on one context
    // ragged batches: products whose shorter operand has at least this many
    // u64 limbs go through the NTT kernel (at most 129: classical groups hold
    // 128 limbs of the shorter operand)
    uint32_t ragged_ntt_min = mi::tuned::kRaggedNttMin;
    // mi_mul_u64: square products of at least this many u64 limbs use the NTT
    uint32_t plain_ntt_min = mi::tuned::kPlainNttMin;
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
