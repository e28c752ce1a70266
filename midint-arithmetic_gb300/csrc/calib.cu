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

// Host-link streaming by the SMs over mapped pinned host memory (the access
// pattern of the zero-copy host-buffer calls): 16-byte loads, stores, or a
// copy, grid-strided over n 16-byte words.
__global__ void __launch_bounds__(256) k_link_read(const uint4* __restrict__ p, size_t n, uint4* __restrict__ sink) {
    uint4 x = make_uint4(0, 0, 0, 0);
    for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x) {
        const uint4 v = __ldcs(p + i);
        x.x ^= v.x, x.y ^= v.y, x.z ^= v.z, x.w ^= v.w;
    }
    if ((x.x & x.y & x.z & x.w) == 0xffffffffu) sink[0] = x;  // keeps the loads observable
}
__global__ void __launch_bounds__(256) k_link_write(uint4* __restrict__ p, size_t n) {
    for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x)
        __stcs(p + i, make_uint4(uint32_t(i), 1u, 2u, 3u));
}
__global__ void __launch_bounds__(256) k_link_copy(const uint4* __restrict__ s, uint4* __restrict__ d, size_t n) {
    for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x)
        __stcs(d + i, __ldcs(s + i));
}

// The device address of a mapped host buffer, or null.
void* mapped(const void* p) {
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return at.type == cudaMemoryTypeHost ? at.devicePointer : nullptr;
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
    cudaError_t err = cudaGetLastError();  // a failed launch would leave an empty timed region
    if (err == cudaSuccess) err = cudaEventSynchronize(e1);
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

extern "C" mi_status mi_calib_host_link(const void* host_src, void* host_dst, size_t bytes, double* read_gbs,
                                        double* write_gbs, double* both_gbs) {
    if (host_src == nullptr || host_dst == nullptr || read_gbs == nullptr || write_gbs == nullptr ||
        both_gbs == nullptr)
        return set_error(MI_EINVAL, "calib_host_link: null pointer");
    if (bytes < 32 || bytes % 32 != 0 || !aligned16(host_src) || !aligned16(host_dst))
        return set_error(MI_EINVAL, "calib_host_link: bytes must be a positive multiple of 32 on 16-byte aligned buffers");
    const uint4* src = static_cast<const uint4*>(mapped(host_src));
    uint4* dst = static_cast<uint4*>(mapped(host_dst));
    if (src == nullptr || dst == nullptr)
        return set_error(MI_EINVAL, "calib_host_link: buffers must be pinned host memory mapped for the device");
    const size_t n = bytes / 16;
    const uint32_t blocks = uint32_t(sm_count() * 2);
    uint4* sink = nullptr;
    MI_CUDA_TRY(cudaMalloc(&sink, 16));
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best[3] = {1e30f, 1e30f, 1e30f};
    cudaError_t err = cudaSuccess;
    for (int it = 0; it < 6 && err == cudaSuccess; ++it) {  // the first round warms up
        for (int k = 0; k < 3 && err == cudaSuccess; ++k) {
            cudaEventRecord(e0);
            if (k == 0) k_link_read<<<blocks, 256>>>(src, n, sink);
            else if (k == 1) k_link_write<<<blocks, 256>>>(dst, n);
            else k_link_copy<<<blocks, 256>>>(src, dst, n / 2);  // bytes/2 each way
            cudaEventRecord(e1);
            err = cudaGetLastError();
            if (err == cudaSuccess) err = cudaEventSynchronize(e1);
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (it > 0 && ms < best[k]) best[k] = ms;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(sink);
    if (err != cudaSuccess) return cuda_error(err, "calib_host_link kernel");
    *read_gbs = double(bytes) / (double(best[0]) * 1e-3) / 1e9;
    *write_gbs = double(bytes) / (double(best[1]) * 1e-3) / 1e9;
    *both_gbs = double(bytes) / (double(best[2]) * 1e-3) / 1e9;
    return MI_OK;
}
