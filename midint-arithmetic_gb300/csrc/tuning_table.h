// tuning_table.h -- defaults of the tunable launch choices, written by
// midint-arithmetic_gb300/autotune.py from measurements on NVIDIA GB300 (2026-12-04; the
// record of the run is midint-arithmetic_gb300/tuning.json).  Hand edits are
// overwritten by the next tuning run.
#pragma once

#include <cstdint>

namespace mi {
namespace tuned {

// mi_mul_u64: square products of at least this many u64 limbs use the NTT.
constexpr uint32_t kPlainNttMin = 96;
// mi_mul_lo_u64: low halves of products of at least this many u64 limbs come
// from the NTT kernel (2049 = never).
constexpr uint32_t kLoNttMin = 320;
// mi_poly_u64: composites of at least this many u64 limbs run their four
// products on the NTT (2049 = never).
constexpr uint32_t kPolyNttMin = 320;
// Ragged runs: products whose shorter operand has at least this many u64
// limbs use the NTT kernel (1..257), and so do those from kRaggedNtt40Min
// limbs whose NTT runs on 40-bit digits and three primes.
constexpr uint32_t kRaggedNttMin = 112;
constexpr uint32_t kRaggedNtt40Min = 96;
// Batched addition: bytes of each operand a thread owns (16, 32 or 64), by
// size class c = ceil(log2(u64 limbs)), c = 0..12.
constexpr uint8_t kAddThreadBytes[13] = {16, 16, 16, 16, 32, 32, 32, 32, 16, 32, 32, 64, 64};
// Host-buffer calls, by operation class {additions, multiplications}: chunks a
// large batch is cut into for copy/compute overlap, and the zero-copy mode for
// mapped pinned buffers (0 copies, 1 kernels read and write in place, 2 kernels
// read the operands in place and the results are copied out).
constexpr uint32_t kHostChunks[2] = {6, 3};
constexpr uint32_t kHostZeroCopy[2] = {2, 1};
// Zero-copy mode 1: resident blocks per SM of the classical product kernel
// (0: as many as fit).
constexpr uint32_t kHostZcBlocks[2] = {0, 2};

}  // namespace tuned
}  // namespace mi
