// calib.cu -- integer-multiply-pipe calibration microbenchmark.
//
// Counterpart of the reference's scalar-op latency loops additionKer /
// multiplyKer / modulusKer and testBasicOps (cuda/ker-helpers.cu.h:193-317),
// turned into a throughput measurement of the instruction form the
// multiplication kernels are built from: a 32x32-bit partial product added
// into a carry chain as mad.lo.cc + madc.hi.cc on the same operands (which the
// compiler issues as one wide multiply-add).  Every thread runs kChains
// independent chains with few enough registers for full occupancy, so the
// rate it reaches is the ceiling for 32x32-bit partial products on this GPU.
#include "common.cuh"

namespace mi {
namespace {

constexpr int kChains = 8;
constexpr int kProdPerStep = 2;  // two partial products (four multiply-adds) per chain step

__global__ void __launch_bounds__(256) k_imad_peak(uint32_t iters, uint32_t seed, uint32_t* out) {
    uint32_t a = seed ^ threadIdx.x, b = seed * 2654435761u + blockIdx.x;
    uint32_t acc[kChains][4];
#pragma unroll
    for (int c = 0; c < kChains; ++c)
#pragma unroll
        for (int w = 0; w < 4; ++w) acc[c][w] = a + 7 * c + w;
    for (uint32_t it = 0; it < iters; ++it) {
#pragma unroll
        for (int c = 0; c < kChains; ++c) {
            const uint32_t bc = b + c;
            mad_lo_cc(acc[c][0], a, bc);
            madc_hi_cc(acc[c][1], a, bc);
            madc_lo_cc(acc[c][2], a ^ 1u, bc);
            madc_hi_cc(acc[c][3], a ^ 1u, bc);
        }
        a += acc[0][3];
    }
    uint32_t s = 0;
#pragma unroll
    for (int c = 0; c < kChains; ++c)
#pragma unroll
        for (int w = 0; w < 4; ++w) s ^= acc[c][w];
    if (s == 0x9e3779b9u) out[0] = s;  // keeps the work observable
}

}  // namespace
}  // namespace mi

using namespace mi;

extern "C" mi_status mi_calib_mul32_peak(uint32_t iters, double* products_per_s, double* seconds) {
    if (products_per_s == nullptr) return set_error(MI_EINVAL, "calib: null output");
    if (iters == 0) iters = 20000;
    int blocks_per_sm = 0;
    MI_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, k_imad_peak, 256, 0));
    if (blocks_per_sm < 1) blocks_per_sm = 1;
    const uint32_t blocks = uint32_t(sm_count() * blocks_per_sm);
    uint32_t* d_out = nullptr;
    MI_CUDA_TRY(cudaMalloc(&d_out, 4));
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    k_imad_peak<<<blocks, 256>>>(iters / 8, 1u, d_out);  // warm-up
    cudaEventRecord(e0);
    k_imad_peak<<<blocks, 256>>>(iters, 2u, d_out);
    cudaEventRecord(e1);
    cudaError_t err = cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(d_out);
    if (err != cudaSuccess) return cuda_error(err, "calib kernel");
    const double prods = double(blocks) * 256.0 * iters * kChains * kProdPerStep;
    *products_per_s = prods / (double(ms) * 1e-3);
    if (seconds) *seconds = double(ms) * 1e-3;
    return MI_OK;
}
