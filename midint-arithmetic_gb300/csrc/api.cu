// api.cu -- the C ABI (include/midint.h): contexts, argument checks, status
// codes, the reference-shaped host-pointer wrappers and the pipelined
// host-buffer calls.
//
// The reference's drivers (cuda/main.cu:39-162, 221-356) allocate, copy, launch
// on the default stream and ignore every error (gpuAssert prints and returns,
// cuda/helper.h:13-19).  Here device-pointer calls never allocate, launch on the
// caller's stream and return a status; only the host-pointer calls move data,
// through staging buffers the context keeps.
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <atomic>
#include <map>
#include <mutex>
#include <utility>

#include "common.cuh"
#include "ctx.h"
#include "kernels.h"
#include "ntt_host.h"

namespace mi {

namespace {
thread_local char g_err[512] = "";
}

mi_status set_error(mi_status st, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
    return st;
}

mi_status cuda_error(cudaError_t e, const char* what) {
    const mi_status st = (e == cudaErrorMemoryAllocation)                                   ? MI_ENOMEM
                         : (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver ||
                            e == cudaErrorInvalidDevice)                                     ? MI_ENODEV
                                                                                             : MI_ECUDA;
    return set_error(st, "%s: %s (%s)", what, cudaGetErrorName(e), cudaGetErrorString(e));
}

int sm_count() {
    static std::atomic<int> cache[64];  // zero-initialised (static storage)
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 152;
    int v = cache[dev].load(std::memory_order_relaxed);
    if (v == 0) {
        if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0) v = 152;
        cache[dev].store(v, std::memory_order_relaxed);
    }
    return v;
}

mi_status ensure_dyn_smem(const void* kern, size_t bytes) {
    static std::mutex mu;
    static std::map<std::pair<const void*, int>, size_t> limit;
    int dev = 0;
    MI_CUDA_TRY(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(mu);
    size_t& cur = limit[{kern, dev}];
    if (cur >= bytes) return MI_OK;
    MI_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(bytes)));
    cur = bytes;
    return MI_OK;
}

}  // namespace mi

using namespace mi;

namespace {

// NULL is CUDA's default stream, as everywhere in the CUDA runtime; callers
// that want the context's own stream pass mi_ctx_stream(ctx).
cudaStream_t pick_stream(mi_ctx, mi_stream s) { return reinterpret_cast<cudaStream_t>(s); }

mi_status check_ctx(mi_ctx ctx) {
    if (ctx == nullptr) return set_error(MI_EINVAL, "null context");
    int cur = -1;
    MI_CUDA_TRY(cudaGetDevice(&cur));
    if (cur != ctx->device) MI_CUDA_TRY(cudaSetDevice(ctx->device));
    return MI_OK;
}

mi_status check_batch(const void* a, const void* b, const void* r, uint32_t limbs, uint32_t max_limbs,
                      const char* op) {
    if (a == nullptr || b == nullptr || r == nullptr) return set_error(MI_EINVAL, "%s: null buffer", op);
    if (limbs == 0) return set_error(MI_EINVAL, "%s: zero limbs", op);
    if (limbs > max_limbs) return set_error(MI_EINVAL, "%s: %u limbs exceeds the maximum %u", op, limbs, max_limbs);
    return MI_OK;
}

// Operand bytes per thread of an addition from the context's tuning table.
uint32_t add_bytes(mi_ctx ctx, uint32_t limbs, int limb_bytes) {
    return ctx->add_thread_bytes[add_size_class(uint64_t(limbs) * uint32_t(limb_bytes))];
}

mi_status add_any(mi_ctx ctx, const void* a, const void* b, void* r, uint8_t* carry, uint32_t n, uint32_t limbs,
                  mi_stream stream, int limb_bytes, int op) {
    const uint32_t maxl = kAddWideMaxLimbs64 * (8 / limb_bytes);
    MI_TRY(check_batch(a, b, r, limbs, maxl, op == ADD_SIX ? "add6" : "add"));
    const size_t bytes = size_t(n) * limbs * limb_bytes;
    if (partial_overlap(a, bytes, r, bytes) || partial_overlap(b, bytes, r, bytes))
        return set_error(MI_EINVAL, "add: result partially overlaps an operand");
    if (carry != nullptr && (any_overlap(carry, n, r, bytes) || any_overlap(carry, n, a, bytes) ||
                             any_overlap(carry, n, b, bytes)))
        return set_error(MI_EINVAL, "add: carry_out overlaps a limb buffer");
    if (n == 0) return MI_OK;
    MI_TRY(check_ctx(ctx));
    cudaStream_t st = pick_stream(ctx, stream);
    const uint32_t tb = add_bytes(ctx, limbs, limb_bytes);
    if (limb_bytes == 8)
        return launch_add_u64(static_cast<const uint64_t*>(a), static_cast<const uint64_t*>(b),
                              static_cast<uint64_t*>(r), carry, n, limbs, op, tb, st, &ctx->wide);
    return launch_add_u32(static_cast<const uint32_t*>(a), static_cast<const uint32_t*>(b),
                          static_cast<uint32_t*>(r), carry, n, limbs, tb, st, &ctx->wide);
}

// pick_ntt: a low half of at least ctx->lo_ntt_min u64 limbs comes from the
// NTT kernel (same result; the NTT's cost grows as L lg L, the classical low
// half's as limbs^2)
mi_status mul_any(mi_ctx ctx, const void* a, const void* b, void* r, uint32_t n, uint32_t limbs, mi_stream stream,
                  int limb_bytes, bool full, bool pick_ntt = false) {
    const uint32_t maxl = kMulMaxN32 / (limb_bytes / 4);
    MI_TRY(check_batch(a, b, r, limbs, maxl, full ? "mul_full" : "mul_lo"));
    const size_t in_bytes = size_t(n) * limbs * limb_bytes;
    const size_t out_bytes = in_bytes * (full ? 2 : 1);
    if (n > 0 && (any_overlap(r, out_bytes, a, in_bytes) || any_overlap(r, out_bytes, b, in_bytes)))
        return set_error(MI_EINVAL, "mul: result overlaps an operand");
    if (n == 0) return MI_OK;
    MI_TRY(check_ctx(ctx));
    // (the NTT kernels read 8-byte words: rows that are only 4-byte aligned
    // take the classical kernel, which reads 32-bit words)
    if (pick_ntt && !full && limb_bytes == 8 && limbs >= ctx->lo_ntt_min && limbs <= kNttMaxLimbs &&
        aligned8(a) && aligned8(b) && aligned8(r))
        return launch_mul_ntt(static_cast<const uint64_t*>(a), static_cast<const uint64_t*>(b),
                              static_cast<uint64_t*>(r), n, limbs, ctx->ntt.params, pick_stream(ctx, stream), true);
    const uint32_t n32 = limbs * uint32_t(limb_bytes / 4);
    return launch_mul_classic(static_cast<const uint32_t*>(a), static_cast<const uint32_t*>(b),
                              static_cast<uint32_t*>(r), n, n32, full, pick_stream(ctx, stream));
}

mi_status mul_ntt(mi_ctx ctx, const uint64_t* a, const uint64_t* b, uint64_t* r, uint32_t n, uint32_t limbs,
                  mi_stream stream) {
    MI_TRY(check_batch(a, b, r, limbs, kNttMaxLimbs, "mul_ntt"));
    if (!aligned8(a) || !aligned8(b) || !aligned8(r)) return set_error(MI_EINVAL, "mul_ntt: buffers not 8-byte aligned");
    const size_t in_bytes = size_t(n) * limbs * 8;
    if (n > 0 && (any_overlap(r, 2 * in_bytes, a, in_bytes) || any_overlap(r, 2 * in_bytes, b, in_bytes)))
        return set_error(MI_EINVAL, "mul_ntt: result overlaps an operand");
    if (n == 0) return MI_OK;
    MI_TRY(check_ctx(ctx));
    return launch_mul_ntt(a, b, r, n, limbs, ctx->ntt.params, pick_stream(ctx, stream));
}


// --- default contexts for the reference-shaped host-pointer wrappers -------
std::mutex g_default_mu;
mi_ctx g_default[64] = {};

mi_status default_ctx(mi_ctx* out) {
    int dev = 0;
    MI_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return set_error(MI_ENODEV, "device index %d out of range", dev);
    std::lock_guard<std::mutex> lk(g_default_mu);
    if (g_default[dev] == nullptr) MI_TRY(mi_ctx_create(dev, &g_default[dev]));
    *out = g_default[dev];
    return MI_OK;
}

mi_status ensure_stage(mi_ctx ctx, size_t bytes) {
    if (bytes <= ctx->stage_cap) return MI_OK;
    for (int i = 0; i < mi_ctx_s::kSlots; ++i) {
        if (ctx->stage[i]) cudaFree(ctx->stage[i]);
        ctx->stage[i] = nullptr;
    }
    ctx->stage_cap = 0;
    size_t cap = 1;
    while (cap < bytes) cap <<= 1;
    for (int i = 0; i < mi_ctx_s::kSlots; ++i) MI_CUDA_TRY(cudaMalloc(&ctx->stage[i], cap));
    ctx->stage_cap = cap;
    return MI_OK;
}

// The device address of a mapped pinned host buffer that kernels may read or
// write in place, or null.  Buffers that are not 8-byte aligned are not used
// in place (the staging buffers of the copy path are): the u64 and NTT
// kernels read whole 8-byte words.
void* mapped_host(const void* p) {
    if (!aligned8(p)) return nullptr;
    cudaPointerAttributes attr;
    if (cudaPointerGetAttributes(&attr, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return attr.type == cudaMemoryTypeHost ? attr.devicePointer : nullptr;
}

// MI_ETIMEOUT (and the error word cleared) when a multi-block addition of the
// context gave up a bounded wait; call after its stream has been synchronised.
mi_status wide_status(mi_ctx ctx) {
    uint32_t err = 0;
    MI_CUDA_TRY(cudaMemcpy(&err, ctx->wide.status + kWideTiles + 2, 4, cudaMemcpyDeviceToHost));
    if (err == 0) return MI_OK;
    MI_CUDA_TRY(cudaMemset(ctx->wide.status + kWideTiles + 2, 0, 4));
    return set_error(MI_ETIMEOUT, "a multi-block addition gave up waiting for a predecessor tile");
}

// Runs `launch(da, db, dr, dcarry, count, stream, max_per_sm)` over a batch of
// host buffers, with the tuning of operation class `cls` (max_per_sm is the
// class's zero-copy occupancy cap in mode 1, else 0).  Zero-copy mode 2 with
// mapped pinned operands: the kernels read the operands in place and only the
// results go through the staging slots and the copy-out stream (the two
// directions of the host link then run at once).  Zero-copy mode 1 with
// every buffer mapped pinned memory: one
// launch reads and writes them in place.  Mode 3 with mapped pinned results:
// the operands go through the staging slots on the copy-in stream and the
// kernels write the results in place (no copy-out).  Otherwise the batch is cut into
// chunks that cycle through kSlots device staging slots: chunk c copies in on
// the copy-in stream (after the slot's previous copy-out), computes on compute
// stream c % 2 (always the first compute stream when `one_compute_stream`: for
// kernels that share context state between launches) and copies out on the
// copy-out stream, so copies in both
// directions and the kernels of neighbouring chunks overlap.
enum { HOST_ADD = 0, HOST_MUL = 1 };  // operation classes of the host tuning knobs

template <typename F>
mi_status host_pipeline(mi_ctx ctx, int cls, const void* h_a, const void* h_b, void* h_r, uint8_t* h_carry,
                        uint32_t n, size_t in_row, size_t out_row, F launch, bool one_compute_stream = false) {
    if (n == 0) return MI_OK;
    MI_TRY(check_ctx(ctx));
    std::lock_guard<std::mutex> lk(ctx->mu);
    // zero-copy reads of the operands (modes 1 and 2) when both are mapped
    const char* za = nullptr;
    const char* zb = nullptr;
    const uint32_t mode = ctx->host_zero_copy[cls];
    if (mode == 1 || mode == 2) {
        za = static_cast<const char*>(mapped_host(h_a));
        zb = static_cast<const char*>(mapped_host(h_b));
        if (!za || !zb) za = zb = nullptr;
    }
    if (za && mode == 1) {
        void* dr = mapped_host(h_r);
        void* dc = h_carry ? mapped_host(h_carry) : nullptr;
        if (dr && (dc || !h_carry)) {
            MI_TRY(launch(const_cast<char*>(za), const_cast<char*>(zb), dr, static_cast<uint8_t*>(dc), n,
                          ctx->pipe[2], ctx->host_zc_blocks[cls]));
            MI_CUDA_TRY(cudaStreamSynchronize(ctx->pipe[2]));
            return MI_OK;
        }
    }
    // mode 3: the operands are copied in by chunks and the kernels write the
    // results in place when they (and the carries) are mapped pinned memory
    char* zr = nullptr;
    uint8_t* zc = nullptr;
    if (mode == 3) {
        zr = static_cast<char*>(mapped_host(h_r));
        zc = h_carry ? static_cast<uint8_t*>(mapped_host(h_carry)) : nullptr;
        if (h_carry && !zc) zr = nullptr;
    }
    const size_t per_inst = 2 * in_row + out_row + (h_carry ? 1 : 0);
    uint64_t chunk = (uint64_t(n) + ctx->host_chunks[cls] - 1) / ctx->host_chunks[cls];
    const uint64_t max_chunk = (64ull << 20) / per_inst;  // at most 64 MiB per slot
    if (chunk > max_chunk) chunk = max_chunk;
    if (chunk == 0) chunk = 1;
    const size_t off_b = ((chunk * in_row + 255) / 256) * 256;
    const size_t off_r = off_b + ((chunk * in_row + 255) / 256) * 256;
    const size_t off_c = off_r + ((chunk * out_row + 255) / 256) * 256;
    MI_TRY(ensure_stage(ctx, off_c + chunk + 256));
    cudaStream_t cin = ctx->pipe[0], cout = ctx->pipe[1];
    int c = 0;
    for (uint64_t base = 0; base < n; base += chunk, ++c) {
        const uint32_t cnt = uint32_t((n - base) < chunk ? (n - base) : chunk);
        const int slot = c % mi_ctx_s::kSlots;
        cudaStream_t comp = ctx->pipe[one_compute_stream ? 2 : 2 + (c & 1)];
        char* stg = static_cast<char*>(ctx->stage[slot]);
        if (za) {
            // mode 2: the kernel reads this chunk's operands in place and
            // writes the staging slot once its previous copy-out is done
            if (c >= mi_ctx_s::kSlots) MI_CUDA_TRY(cudaStreamWaitEvent(comp, ctx->ev_out[slot], 0));
            MI_TRY(launch(const_cast<char*>(za) + base * in_row, const_cast<char*>(zb) + base * in_row, stg + off_r,
                          h_carry ? reinterpret_cast<uint8_t*>(stg + off_c) : nullptr, cnt, comp, 0u));
        } else {
            // the slot is free once its last reader is done: its copy-out,
            // or in mode 3 the kernel itself
            if (c >= mi_ctx_s::kSlots) MI_CUDA_TRY(cudaStreamWaitEvent(cin, zr ? ctx->ev_k[slot] : ctx->ev_out[slot], 0));
            MI_CUDA_TRY(cudaMemcpyAsync(stg, static_cast<const char*>(h_a) + base * in_row, cnt * in_row,
                                        cudaMemcpyHostToDevice, cin));
            MI_CUDA_TRY(cudaMemcpyAsync(stg + off_b, static_cast<const char*>(h_b) + base * in_row, cnt * in_row,
                                        cudaMemcpyHostToDevice, cin));
            MI_CUDA_TRY(cudaEventRecord(ctx->ev_in[slot], cin));
            MI_CUDA_TRY(cudaStreamWaitEvent(comp, ctx->ev_in[slot], 0));
            if (zr) {
                MI_TRY(launch(stg, stg + off_b, zr + base * out_row, zc ? zc + base : nullptr, cnt, comp, 0u));
                MI_CUDA_TRY(cudaEventRecord(ctx->ev_k[slot], comp));
                continue;
            }
            MI_TRY(launch(stg, stg + off_b, stg + off_r, h_carry ? reinterpret_cast<uint8_t*>(stg + off_c) : nullptr,
                          cnt, comp, 0u));
        }
        MI_CUDA_TRY(cudaEventRecord(ctx->ev_k[slot], comp));
        MI_CUDA_TRY(cudaStreamWaitEvent(cout, ctx->ev_k[slot], 0));
        MI_CUDA_TRY(cudaMemcpyAsync(static_cast<char*>(h_r) + base * out_row, stg + off_r, cnt * out_row,
                                    cudaMemcpyDeviceToHost, cout));
        if (h_carry)
            MI_CUDA_TRY(cudaMemcpyAsync(h_carry + base, stg + off_c, cnt, cudaMemcpyDeviceToHost, cout));
        MI_CUDA_TRY(cudaEventRecord(ctx->ev_out[slot], cout));
    }
    if (zr) {
        MI_CUDA_TRY(cudaStreamSynchronize(ctx->pipe[2]));
        MI_CUDA_TRY(cudaStreamSynchronize(ctx->pipe[3]));
    } else {
        MI_CUDA_TRY(cudaStreamSynchronize(cout));
    }
    return MI_OK;
}

}  // namespace

extern "C" {

int mi_version(void) { return 100; }

const char* mi_status_string(int status) {
    switch (status) {
        case MI_OK: return "MI_OK";
        case MI_EINVAL: return "MI_EINVAL: invalid argument";
        case MI_ENOMEM: return "MI_ENOMEM: out of memory";
        case MI_ECUDA: return "MI_ECUDA: CUDA error";
        case MI_ETIMEOUT: return "MI_ETIMEOUT: bounded device wait timed out";
        case MI_ENODEV: return "MI_ENODEV: no usable CUDA device";
        case MI_ENOTSUP: return "MI_ENOTSUP: not supported";
        default: return "unknown status";
    }
}

const char* mi_last_error(void) { return g_err; }

mi_status mi_ctx_create(int device, mi_ctx* out) {
    if (out == nullptr) return set_error(MI_EINVAL, "mi_ctx_create: null out");
    *out = nullptr;
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) return set_error(MI_ENODEV, "no CUDA device (%s)", cudaGetErrorName(e));
    if (device < 0 || device >= count) return set_error(MI_ENODEV, "device %d not present (%d devices)", device, count);
    MI_CUDA_TRY(cudaSetDevice(device));
    mi_ctx ctx = new (std::nothrow) mi_ctx_s();
    if (ctx == nullptr) return set_error(MI_ENOMEM, "mi_ctx_create: host allocation");
    ctx->device = device;
    mi_status st = MI_OK;
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess)
        st = set_error(MI_ECUDA, "mi_ctx_create: stream creation failed");
    for (int i = 0; i < 4 && st == MI_OK; ++i)
        if (cudaStreamCreateWithFlags(&ctx->pipe[i], cudaStreamNonBlocking) != cudaSuccess)
            st = set_error(MI_ECUDA, "mi_ctx_create: stream creation failed");
    for (int i = 0; i < mi_ctx_s::kSlots && st == MI_OK; ++i)
        if (cudaEventCreateWithFlags(&ctx->ev_in[i], cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&ctx->ev_k[i], cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&ctx->ev_out[i], cudaEventDisableTiming) != cudaSuccess)
            st = set_error(MI_ECUDA, "mi_ctx_create: event creation failed");
    if (st == MI_OK) st = ntt_tables_create(&ctx->ntt);
    if (st == MI_OK) {
        const size_t wb = (size_t(kWideTiles) + 4) * 4;
        if (cudaMalloc(&ctx->wide.status, wb) != cudaSuccess || cudaMemset(ctx->wide.status, 0, wb) != cudaSuccess)
            st = set_error(MI_ENOMEM, "mi_ctx_create: multi-block addition state");
    }
    if (st != MI_OK) {
        mi_ctx_destroy(ctx);
        return st;
    }
    *out = ctx;
    return MI_OK;
}

mi_status mi_ctx_destroy(mi_ctx ctx) {
    if (ctx == nullptr) return MI_OK;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    for (int i = 0; i < 4; ++i) {
        if (ctx->pipe[i]) {
            cudaStreamSynchronize(ctx->pipe[i]);
            cudaStreamDestroy(ctx->pipe[i]);
        }
    }
    for (int i = 0; i < mi_ctx_s::kSlots; ++i) {
        if (ctx->stage[i]) cudaFree(ctx->stage[i]);
        if (ctx->ev_in[i]) cudaEventDestroy(ctx->ev_in[i]);
        if (ctx->ev_k[i]) cudaEventDestroy(ctx->ev_k[i]);
        if (ctx->ev_out[i]) cudaEventDestroy(ctx->ev_out[i]);
    }
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    if (ctx->wide.status) cudaFree(ctx->wide.status);
    ntt_tables_destroy(&ctx->ntt);
    delete ctx;
    return MI_OK;
}

mi_status mi_ctx_synchronize(mi_ctx ctx) {
    MI_TRY(check_ctx(ctx));
    MI_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return MI_OK;
}

mi_stream mi_ctx_stream(mi_ctx ctx) { return ctx ? reinterpret_cast<mi_stream>(ctx->stream) : nullptr; }

mi_status mi_ctx_set_crossover(mi_ctx ctx, uint32_t ragged_ntt_min, uint32_t plain_ntt_min) {
    if (ctx == nullptr) return set_error(MI_EINVAL, "null context");
    if (ragged_ntt_min < 1 || ragged_ntt_min > 257)
        return set_error(MI_EINVAL, "ragged_ntt_min %u outside 1..257", ragged_ntt_min);
    if (plain_ntt_min < 1 || plain_ntt_min > kNttMaxLimbs + 1)
        return set_error(MI_EINVAL, "plain_ntt_min %u outside 1..%u", plain_ntt_min, kNttMaxLimbs + 1);
    ctx->ragged_ntt_min = ragged_ntt_min;
    ctx->plain_ntt_min = plain_ntt_min;
    return MI_OK;
}

mi_status mi_ctx_device_status(mi_ctx ctx) {
    MI_TRY(check_ctx(ctx));
    MI_CUDA_TRY(cudaDeviceSynchronize());
    return wide_status(ctx);
}

mi_status mi_ctx_set_tuning(mi_ctx ctx, int knob, uint32_t cls, uint32_t value) {
    if (ctx == nullptr) return set_error(MI_EINVAL, "null context");
    switch (knob) {
        case MI_TUNE_PLAIN_NTT_MIN:
            if (value < 1 || value > kNttMaxLimbs + 1)
                return set_error(MI_EINVAL, "plain_ntt_min %u outside 1..%u", value, kNttMaxLimbs + 1);
            ctx->plain_ntt_min = value;
            return MI_OK;
        case MI_TUNE_RAGGED_NTT_MIN:
            if (cls > 1) return set_error(MI_EINVAL, "ragged crossover class %u not 0 or 1", cls);
            if (value < 1 || value > 257) return set_error(MI_EINVAL, "ragged_ntt_min %u outside 1..257", value);
            (cls == 0 ? ctx->ragged_ntt_min : ctx->ragged_ntt40_min) = value;
            return MI_OK;
        case MI_TUNE_LO_NTT_MIN:
            if (value < 1 || value > kNttMaxLimbs + 1)
                return set_error(MI_EINVAL, "lo_ntt_min %u outside 1..%u", value, kNttMaxLimbs + 1);
            ctx->lo_ntt_min = value;
            return MI_OK;
        case MI_TUNE_POLY_NTT_MIN:
            if (value < 1 || value > kNttMaxLimbs + 1)
                return set_error(MI_EINVAL, "poly_ntt_min %u outside 1..%u", value, kNttMaxLimbs + 1);
            ctx->poly_ntt_min = value;
            return MI_OK;
        case MI_TUNE_ADD_THREAD_BYTES:
            if (cls > 12) return set_error(MI_EINVAL, "addition size class %u outside 0..12", cls);
            if (value != 16 && value != 32 && value != 64)
                return set_error(MI_EINVAL, "addition bytes per thread %u not 16, 32 or 64", value);
            ctx->add_thread_bytes[cls] = uint8_t(value);
            return MI_OK;
        case MI_TUNE_HOST_CHUNKS:
            if (cls > 1) return set_error(MI_EINVAL, "host operation class %u not 0 or 1", cls);
            if (value < 1 || value > 64) return set_error(MI_EINVAL, "host chunks %u outside 1..64", value);
            ctx->host_chunks[cls] = value;
            return MI_OK;
        case MI_TUNE_HOST_ZERO_COPY:
            if (cls > 1) return set_error(MI_EINVAL, "host operation class %u not 0 or 1", cls);
            if (value > 3) return set_error(MI_EINVAL, "host zero-copy mode %u not 0, 1, 2 or 3", value);
            ctx->host_zero_copy[cls] = value;
            return MI_OK;
        case MI_TUNE_HOST_ZC_BLOCKS:
            if (cls > 1) return set_error(MI_EINVAL, "host operation class %u not 0 or 1", cls);
            if (value > 3) return set_error(MI_EINVAL, "zero-copy blocks per SM %u outside 0..3", value);
            ctx->host_zc_blocks[cls] = value;
            return MI_OK;
        case MI_TUNE_WIDE_SPIN_LIMIT:
            if (value < 1) return set_error(MI_EINVAL, "spin limit must be at least 1");
            ctx->wide.spin_limit = value;
            return MI_OK;
        case MI_TUNE_WIDE_WITHHOLD:
            if (value > 1) return set_error(MI_EINVAL, "withhold %u not 0 or 1", value);
            ctx->wide.withhold = value;
            return MI_OK;
        case MI_TUNE_WIDE_ROUND_TILES:
            if (value < 1 || value > kWideTiles)
                return set_error(MI_EINVAL, "tiles per round %u outside 1..%u", value, kWideTiles);
            ctx->wide.round_tiles = value;
            return MI_OK;
        default: return set_error(MI_EINVAL, "unknown tuning knob %d", knob);
    }
}

mi_status mi_ctx_get_tuning(mi_ctx ctx, int knob, uint32_t cls, uint32_t* value) {
    if (ctx == nullptr || value == nullptr) return set_error(MI_EINVAL, "null context or value");
    switch (knob) {
        case MI_TUNE_PLAIN_NTT_MIN: *value = ctx->plain_ntt_min; return MI_OK;
        case MI_TUNE_RAGGED_NTT_MIN:
            if (cls > 1) return set_error(MI_EINVAL, "ragged crossover class %u not 0 or 1", cls);
            *value = cls == 0 ? ctx->ragged_ntt_min : ctx->ragged_ntt40_min;
            return MI_OK;
        case MI_TUNE_LO_NTT_MIN: *value = ctx->lo_ntt_min; return MI_OK;
        case MI_TUNE_POLY_NTT_MIN: *value = ctx->poly_ntt_min; return MI_OK;
        case MI_TUNE_ADD_THREAD_BYTES:
            if (cls > 12) return set_error(MI_EINVAL, "addition size class %u outside 0..12", cls);
            *value = ctx->add_thread_bytes[cls];
            return MI_OK;
        case MI_TUNE_HOST_CHUNKS:
        case MI_TUNE_HOST_ZERO_COPY:
        case MI_TUNE_HOST_ZC_BLOCKS:
            if (cls > 1) return set_error(MI_EINVAL, "host operation class %u not 0 or 1", cls);
            *value = knob == MI_TUNE_HOST_CHUNKS ? ctx->host_chunks[cls]
                     : knob == MI_TUNE_HOST_ZERO_COPY ? ctx->host_zero_copy[cls]
                                                     : ctx->host_zc_blocks[cls];
            return MI_OK;
        case MI_TUNE_WIDE_SPIN_LIMIT: *value = ctx->wide.spin_limit; return MI_OK;
        case MI_TUNE_WIDE_WITHHOLD: *value = ctx->wide.withhold; return MI_OK;
        case MI_TUNE_WIDE_ROUND_TILES: *value = ctx->wide.round_tiles; return MI_OK;
        default: return set_error(MI_EINVAL, "unknown tuning knob %d", knob);
    }
}

mi_status mi_add_u64(mi_ctx ctx, const uint64_t* a, const uint64_t* b, uint64_t* r, uint8_t* carry_out, uint32_t n,
                     uint32_t limbs, mi_stream stream) {
    return add_any(ctx, a, b, r, carry_out, n, limbs, stream, 8, ADD_PLAIN);
}

mi_status mi_add_u32(mi_ctx ctx, const uint32_t* a, const uint32_t* b, uint32_t* r, uint8_t* carry_out, uint32_t n,
                     uint32_t limbs, mi_stream stream) {
    return add_any(ctx, a, b, r, carry_out, n, limbs, stream, 4, ADD_PLAIN);
}

mi_status mi_add6_u64(mi_ctx ctx, const uint64_t* a, const uint64_t* b, uint64_t* r, uint32_t n, uint32_t limbs,
                      mi_stream stream) {
    return add_any(ctx, a, b, r, nullptr, n, limbs, stream, 8, ADD_SIX);
}

mi_status mi_mul_lo_u64(mi_ctx ctx, const uint64_t* a, const uint64_t* b, uint64_t* r, uint32_t n, uint32_t limbs,
                        mi_stream stream) {
    return mul_any(ctx, a, b, r, n, limbs, stream, 8, false, true);
}
mi_status mi_mul_lo_u32(mi_ctx ctx, const uint32_t* a, const uint32_t* b, uint32_t* r, uint32_t n, uint32_t limbs,
                        mi_stream stream) {
    return mul_any(ctx, a, b, r, n, limbs, stream, 4, false);
}
mi_status mi_mul_full_u64(mi_ctx ctx, const uint64_t* a, const uint64_t* b, uint64_t* r, uint32_t n, uint32_t limbs,
                          mi_stream stream) {
    return mul_any(ctx, a, b, r, n, limbs, stream, 8, true);
}
mi_status mi_mul_full_u32(mi_ctx ctx, const uint32_t* a, const uint32_t* b, uint32_t* r, uint32_t n, uint32_t limbs,
                          mi_stream stream) {
    return mul_any(ctx, a, b, r, n, limbs, stream, 4, true);
}

mi_status mi_poly_u64(mi_ctx ctx, const uint64_t* a, const uint64_t* b, uint64_t* r, uint32_t n, uint32_t limbs,
                      mi_stream stream) {
    MI_TRY(check_batch(a, b, r, limbs, kMulMaxN32 / 2, "poly"));
    const size_t bytes = size_t(n) * limbs * 8;
    if (n > 0 && (any_overlap(r, bytes, a, bytes) || any_overlap(r, bytes, b, bytes)))
        return set_error(MI_EINVAL, "poly: result overlaps an operand");
    if (n == 0) return MI_OK;
    MI_TRY(check_ctx(ctx));
    // from the tuned crossover on, the four products run on transforms (the
    // reference's polyFttKer); below it, the classical form (polyKerQ)
    if (limbs >= ctx->poly_ntt_min && aligned8(a) && aligned8(b) && aligned8(r))
        return launch_poly_ntt(a, b, r, n, limbs, ctx->ntt.params, pick_stream(ctx, stream));
    return launch_poly(reinterpret_cast<const uint32_t*>(a), reinterpret_cast<const uint32_t*>(b),
                       reinterpret_cast<uint32_t*>(r), n, 2 * limbs, pick_stream(ctx, stream));
}

static mi_status check_format(uint32_t words, uint32_t size, int order, int endian, uint32_t limbs, const char* op) {
    if (words == 0 || limbs == 0) return set_error(MI_EINVAL, "%s: zero words or limbs", op);
    if (size != 1 && size != 2 && size != 4 && size != 8)
        return set_error(MI_EINVAL, "%s: word size %u not 1, 2, 4 or 8", op, size);
    if (order != 1 && order != -1) return set_error(MI_EINVAL, "%s: order %d not 1 or -1", op, order);
    if (endian < -1 || endian > 1) return set_error(MI_EINVAL, "%s: endian %d not -1, 0 or 1", op, endian);
    return MI_OK;
}

mi_status mi_import_words(mi_ctx ctx, const void* src, uint32_t n, uint32_t words, uint32_t size, int order,
                          int endian, uint64_t* dst, uint32_t limbs, mi_stream stream) {
    if (src == nullptr || dst == nullptr) return set_error(MI_EINVAL, "import: null buffer");
    MI_TRY(check_format(words, size, order, endian, limbs, "import"));
    if ((reinterpret_cast<uintptr_t>(src) % size) != 0 || (reinterpret_cast<uintptr_t>(dst) & 7u) != 0)
        return set_error(MI_EINVAL, "import: src must be aligned to its word size, dst to 8 bytes");
    if (n > 0 && any_overlap(src, size_t(n) * words * size, dst, size_t(n) * limbs * 8))
        return set_error(MI_EINVAL, "import: src and dst overlap");
    if (n == 0) return MI_OK;
    MI_TRY(check_ctx(ctx));
    return launch_import(src, dst, n, words, size, order, endian, limbs, pick_stream(ctx, stream));
}

mi_status mi_export_words(mi_ctx ctx, const uint64_t* src, uint32_t n, uint32_t limbs, void* dst, uint32_t words,
                          uint32_t size, int order, int endian, uint32_t* counts, mi_stream stream) {
    if (src == nullptr || dst == nullptr) return set_error(MI_EINVAL, "export: null buffer");
    MI_TRY(check_format(words, size, order, endian, limbs, "export"));
    if ((reinterpret_cast<uintptr_t>(dst) % size) != 0 || (reinterpret_cast<uintptr_t>(src) & 7u) != 0 ||
        (reinterpret_cast<uintptr_t>(counts) & 3u) != 0)
        return set_error(MI_EINVAL, "export: dst must be aligned to its word size, src to 8 bytes, counts to 4");
    const size_t sb = size_t(n) * limbs * 8, db = size_t(n) * words * size;
    if (n > 0 && (any_overlap(src, sb, dst, db) || (counts && (any_overlap(counts, size_t(n) * 4, dst, db) ||
                                                              any_overlap(counts, size_t(n) * 4, src, sb)))))
        return set_error(MI_EINVAL, "export: buffers overlap");
    if (n == 0) return MI_OK;
    MI_TRY(check_ctx(ctx));
    return launch_export(src, dst, n, limbs, words, size, order, endian, counts, pick_stream(ctx, stream));
}

mi_status mi_mul_ntt_u64(mi_ctx ctx, const uint64_t* a, const uint64_t* b, uint64_t* r, uint32_t n, uint32_t limbs,
                         mi_stream stream) {
    return mul_ntt(ctx, a, b, r, n, limbs, stream);
}

mi_status mi_mul_u64(mi_ctx ctx, const uint64_t* a, const uint64_t* b, uint64_t* r, uint32_t n, uint32_t limbs,
                     mi_stream stream) {
    if (ctx == nullptr) return set_error(MI_EINVAL, "null context");
    if (limbs >= ctx->plain_ntt_min && limbs <= kNttMaxLimbs && aligned8(a) && aligned8(b) && aligned8(r))
        return mul_ntt(ctx, a, b, r, n, limbs, stream);
    return mul_any(ctx, a, b, r, n, limbs, stream, 8, true);
}

// --- reference-shaped host-pointer wrappers ---------------------------------

mi_status mi_compat_gpuAdd_u64(int num_instances, uint32_t m, const uint64_t* h_as, const uint64_t* h_bs,
                               uint64_t* h_rs) {
    if (num_instances < 0) return set_error(MI_EINVAL, "gpuAdd: negative num_instances");
    MI_TRY(check_batch(h_as, h_bs, h_rs, m, kAddWideMaxLimbs64, "gpuAdd"));
    mi_ctx ctx;
    MI_TRY(default_ctx(&ctx));
    return mi_host_add_u64(ctx, h_as, h_bs, h_rs, nullptr, uint32_t(num_instances), m);
}

mi_status mi_compat_gpuAdd_u32(int num_instances, uint32_t m, const uint32_t* h_as, const uint32_t* h_bs,
                               uint32_t* h_rs) {
    if (num_instances < 0) return set_error(MI_EINVAL, "gpuAdd: negative num_instances");
    MI_TRY(check_batch(h_as, h_bs, h_rs, m, 2 * kAddWideMaxLimbs64, "gpuAdd"));
    mi_ctx ctx;
    MI_TRY(default_ctx(&ctx));
    const size_t row = size_t(m) * 4;
    const mi_status st = host_pipeline(ctx, HOST_ADD, h_as, h_bs, h_rs, nullptr, uint32_t(num_instances), row, row,
                         [ctx, m, tb = add_bytes(ctx, m, 4)](void* da, void* db, void* dr, uint8_t*, uint32_t cnt,
                                                              cudaStream_t st, uint32_t) {
                             return launch_add_u32(static_cast<uint32_t*>(da), static_cast<uint32_t*>(db),
                                                   static_cast<uint32_t*>(dr), nullptr, cnt, m, tb, st, &ctx->wide);
                         },
                         m > 2 * kAddMaxLimbs64);
    return st == MI_OK && m > 2 * kAddMaxLimbs64 ? wide_status(ctx) : st;
}

mi_status mi_compat_gpuMultiply_u64(int num_instances, uint32_t m, const uint64_t* h_as, const uint64_t* h_bs,
                                    uint64_t* h_rs) {
    if (num_instances < 0) return set_error(MI_EINVAL, "gpuMultiply: negative num_instances");
    MI_TRY(check_batch(h_as, h_bs, h_rs, m, kMulMaxN32 / 2, "gpuMultiply"));
    mi_ctx ctx;
    MI_TRY(default_ctx(&ctx));
    const size_t row = size_t(m) * 8;
    const bool ntt = m >= ctx->lo_ntt_min && m <= kNttMaxLimbs;  // as mi_mul_lo_u64 picks (the buffers the
                                                                  // kernels see are 8-byte aligned)
    return host_pipeline(ctx, HOST_MUL, h_as, h_bs, h_rs, nullptr, uint32_t(num_instances), row, row,
                         [ctx, m, ntt](void* da, void* db, void* dr, uint8_t*, uint32_t cnt, cudaStream_t st,
                                       uint32_t cap) {
                             if (ntt)
                                 return launch_mul_ntt(static_cast<uint64_t*>(da), static_cast<uint64_t*>(db),
                                                       static_cast<uint64_t*>(dr), cnt, m, ctx->ntt.params, st, true);
                             return launch_mul_classic(static_cast<uint32_t*>(da), static_cast<uint32_t*>(db),
                                                       static_cast<uint32_t*>(dr), cnt, 2 * m, false, st, cap);
                         });
}

mi_status mi_compat_gpuMultiply_u32(int num_instances, uint32_t m, const uint32_t* h_as, const uint32_t* h_bs,
                                    uint32_t* h_rs) {
    if (num_instances < 0) return set_error(MI_EINVAL, "gpuMultiply: negative num_instances");
    MI_TRY(check_batch(h_as, h_bs, h_rs, m, kMulMaxN32, "gpuMultiply"));
    mi_ctx ctx;
    MI_TRY(default_ctx(&ctx));
    const size_t row = size_t(m) * 4;
    return host_pipeline(ctx, HOST_MUL, h_as, h_bs, h_rs, nullptr, uint32_t(num_instances), row, row,
                         [m](void* da, void* db, void* dr, uint8_t*, uint32_t cnt, cudaStream_t st, uint32_t cap) {
                             return launch_mul_classic(static_cast<uint32_t*>(da), static_cast<uint32_t*>(db),
                                                       static_cast<uint32_t*>(dr), cnt, m, false, st, cap);
                         });
}

mi_status mi_compat_gpuMulFFT_u16(int num_instances, uint32_t M, const uint16_t* h_as, const uint16_t* h_bs,
                                  uint32_t* h_rs) {
    if (num_instances < 0) return set_error(MI_EINVAL, "gpuMulFFT: negative num_instances");
    if (M == 0 || M % 4 != 0 || M / 4 > kNttMaxLimbs)
        return set_error(MI_EINVAL, "gpuMulFFT: M = %u u16 digits must be a multiple of 4, at most %u", M,
                         4 * kNttMaxLimbs);
    if (h_as == nullptr || h_bs == nullptr || h_rs == nullptr) return set_error(MI_EINVAL, "gpuMulFFT: null buffer");
    mi_ctx ctx;
    MI_TRY(default_ctx(&ctx));
    const uint32_t m = M / 4;  // u64 limbs
    const size_t row = size_t(m) * 8;
    // the NTT kernel, storing the low M digits (m limbs) of each product
    return host_pipeline(ctx, HOST_MUL, h_as, h_bs, h_rs, nullptr, uint32_t(num_instances), row, row,
                         [ctx, m](void* da, void* db, void* dr, uint8_t*, uint32_t cnt, cudaStream_t st, uint32_t) {
                             return launch_mul_ntt(static_cast<uint64_t*>(da), static_cast<uint64_t*>(db),
                                                   static_cast<uint64_t*>(dr), cnt, m, ctx->ntt.params, st, true);
                         });
}

// --- ragged batches ----------------------------------------------------------

mi_status mi_ragged_scratch_bytes(uint32_t n_ops, size_t* bytes) {
    if (bytes == nullptr) return set_error(MI_EINVAL, "ragged_scratch_bytes: null out");
    *bytes = ragged_scratch_words(n_ops) * 4;
    return MI_OK;
}

mi_status mi_ragged_run(mi_ctx ctx, const mi_op* ops, uint32_t n_ops, const uint64_t* in, uint64_t* out,
                        uint8_t* carry_out, void* scratch, size_t scratch_bytes, mi_stream stream) {
    if (n_ops == 0) return MI_OK;
    if (!aligned8(ops) || !aligned8(in) || !aligned8(out))
        return set_error(MI_EINVAL, "ragged_run: ops, in and out must be 8-byte aligned");
    MI_TRY(check_ctx(ctx));
    return ragged_launch(ctx, ops, n_ops, in, out, carry_out, scratch, scratch_bytes, ctx->ragged_ntt_min,
                         pick_stream(ctx, stream));
}

mi_status mi_ragged_invalid(const void* scratch, uint32_t* count) {
    if (scratch == nullptr || count == nullptr) return set_error(MI_EINVAL, "ragged_invalid: null pointer");
    MI_CUDA_TRY(cudaMemcpy(count, static_cast<const uint32_t*>(scratch) + ragged_invalid_word(), 4,
                           cudaMemcpyDeviceToHost));
    return MI_OK;
}

mi_status mi_ragged_graph_create(mi_ctx ctx, const mi_op* ops, uint32_t n_ops, const uint64_t* in, uint64_t* out,
                                 uint8_t* carry_out, void* scratch, size_t scratch_bytes, mi_graph* graph) {
    if (graph == nullptr) return set_error(MI_EINVAL, "ragged_graph_create: null out");
    *graph = nullptr;
    if (!aligned8(ops) || !aligned8(in) || !aligned8(out))
        return set_error(MI_EINVAL, "ragged_graph_create: ops, in and out must be 8-byte aligned");
    MI_TRY(check_ctx(ctx));
    MI_TRY(ragged_prepare());  // constant tables and attributes, outside the capture
    cudaStream_t cs = nullptr;
    MI_CUDA_TRY(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    mi_graph g = new (std::nothrow) mi_graph_s();
    if (g == nullptr) {
        cudaStreamDestroy(cs);
        return set_error(MI_ENOMEM, "ragged_graph_create: host allocation");
    }
    g->device = ctx->device;
    mi_status st = MI_OK;
    cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) st = cuda_error(e, "cudaStreamBeginCapture");
    if (st == MI_OK) {
        const mi_status launched =
            ragged_launch(ctx, ops, n_ops, in, out, carry_out, scratch, scratch_bytes, ctx->ragged_ntt_min, cs);
        e = cudaStreamEndCapture(cs, &g->graph);
        if (launched != MI_OK) st = launched;
        else if (e != cudaSuccess) st = cuda_error(e, "cudaStreamEndCapture");
    }
    if (st == MI_OK && g->graph != nullptr) {
        e = cudaGraphInstantiate(&g->exec, g->graph, 0);
        if (e != cudaSuccess) st = cuda_error(e, "cudaGraphInstantiate");
    }
    cudaStreamDestroy(cs);
    if (st != MI_OK) {
        mi_graph_destroy(g);
        return st;
    }
    *graph = g;
    return MI_OK;
}

mi_status mi_graph_launch(mi_graph graph, mi_stream stream) {
    if (graph == nullptr || graph->exec == nullptr) return set_error(MI_EINVAL, "graph_launch: null graph");
    MI_CUDA_TRY(cudaSetDevice(graph->device));
    MI_CUDA_TRY(cudaGraphLaunch(graph->exec, reinterpret_cast<cudaStream_t>(stream)));
    return MI_OK;
}

mi_status mi_graph_destroy(mi_graph graph) {
    if (graph == nullptr) return MI_OK;
    if (graph->exec) cudaGraphExecDestroy(graph->exec);
    if (graph->graph) cudaGraphDestroy(graph->graph);
    delete graph;
    return MI_OK;
}

// --- host-buffer end-to-end calls -------------------------------------------

mi_status mi_host_add_u64(mi_ctx ctx, const uint64_t* h_a, const uint64_t* h_b, uint64_t* h_r, uint8_t* h_carry,
                          uint32_t n, uint32_t limbs) {
    MI_TRY(check_batch(h_a, h_b, h_r, limbs, kAddWideMaxLimbs64, "host_add"));
    if (ctx == nullptr) return set_error(MI_EINVAL, "null context");
    const size_t row = size_t(limbs) * 8;
    const mi_status st = host_pipeline(ctx, HOST_ADD, h_a, h_b, h_r, h_carry, n, row, row,
                         [ctx, limbs, tb = add_bytes(ctx, limbs, 8)](void* da, void* db, void* dr, uint8_t* dc,
                                                                      uint32_t cnt, cudaStream_t st, uint32_t) {
                             return launch_add_u64(static_cast<uint64_t*>(da), static_cast<uint64_t*>(db),
                                                   static_cast<uint64_t*>(dr), dc, cnt, limbs, ADD_PLAIN, tb, st,
                                                   &ctx->wide);
                         },
                         limbs > kAddMaxLimbs64);
    return st == MI_OK && limbs > kAddMaxLimbs64 ? wide_status(ctx) : st;
}

mi_status mi_host_mul_full_u64(mi_ctx ctx, const uint64_t* h_a, const uint64_t* h_b, uint64_t* h_r, uint32_t n,
                               uint32_t limbs) {
    MI_TRY(check_batch(h_a, h_b, h_r, limbs, kMulMaxN32 / 2, "host_mul_full"));
    if (ctx == nullptr) return set_error(MI_EINVAL, "null context");
    const size_t row = size_t(limbs) * 8;
    return host_pipeline(ctx, HOST_MUL, h_a, h_b, h_r, nullptr, n, row, 2 * row,
                         [limbs](void* da, void* db, void* dr, uint8_t*, uint32_t cnt, cudaStream_t st, uint32_t cap) {
                             return launch_mul_classic(static_cast<uint32_t*>(da), static_cast<uint32_t*>(db),
                                                       static_cast<uint32_t*>(dr), cnt, 2 * limbs, true, st, cap);
                         });
}

}  // extern "C"
