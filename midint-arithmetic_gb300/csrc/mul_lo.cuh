// mul_lo.cuh -- shape and launch of the low-half product kernels (mul_lo.cu,
// poly.cu): NH threads per instance for NB = 2*NH blocks of T limbs, a block of
// 256 threads holds 256/NH instances and strides over the batch.
#pragma once

#include "common.cuh"
#include "kernels.h"
#include "mul_core.cuh"

namespace mi {

template <int NH>
struct LoShape {
    static constexpr int BLOCK = NH > 256 ? NH : 256;
    static constexpr int IPB = BLOCK / NH;
    static constexpr int NB = 2 * NH;
    static constexpr int WPAD = NB * classic::T;  // words per operand
    static constexpr size_t SMEM = size_t(2 * IPB * WPAD + BLOCK * classic::PER_T) * 4;
};

using LoKernel = void (*)(const uint32_t*, const uint32_t*, uint32_t*, uint32_t, uint32_t);

// Launches kern (a low-half kernel with NH threads per instance, which starts
// with pdl_wait) with launch_pdl.
template <int NH>
mi_status launch_lo(LoKernel kern, const uint32_t* a, const uint32_t* b, uint32_t* r, uint32_t n, uint32_t n32,
                    cudaStream_t st) {
    using S = LoShape<NH>;
    MI_TRY(ensure_dyn_smem(kern, S::SMEM));
    uint64_t blocks = (uint64_t(n) + S::IPB - 1) / S::IPB;
    const uint64_t cap = uint64_t(sm_count()) * 32;
    if (blocks > cap) blocks = cap;
    MI_CUDA_TRY(launch_pdl(kern, dim3(uint32_t(blocks)), dim3(S::BLOCK), S::SMEM, st, a, b, r, n, n32));
    return MI_OK;
}

// NH for n32 limbs: NB = pow2ceil(blocks of T limbs), at least 2.
inline uint32_t lo_threads(uint32_t n32) {
    const uint32_t nb = pow2ceil((n32 + classic::T - 1) / classic::T);
    return nb < 2 ? 1 : nb / 2;
}

}  // namespace mi
