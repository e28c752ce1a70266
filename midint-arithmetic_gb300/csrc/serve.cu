// serve.cu -- the request loop: continuous batching of ragged requests.
//
// (No reference counterpart: the reference's driver runs one synchronous
// batch per size, cuda/main.cu:661-746.)
//
// A server owns `slots` batch slots; each slot has its own stream, a device
// arena (ops, input pool, output pool, carry bytes, ragged scratch) and a
// pinned host staging arena of the same layout.  One loop thread:
//  * admits queued requests FIFO into the next free slot while the slot's
//    arena has room (memory-based admission) and the op cap allows -- so
//    requests that arrive while other batches are on the GPU join the next
//    batch as soon as a slot frees up;
//  * packs them (ops rebased onto the batch pools, operands copied into
//    pinned memory), enqueues copy-in, the ragged run (ragged.cu), copy-out
//    and an event on the slot's stream -- batches of different slots overlap
//    on the device;
//  * polls the in-flight slots' events, copies finished results into the
//    callers' buffers and wakes their waiters.
// With `batching` = 0 every batch is exactly one request and there is one
// slot: the plain per-request launch, the baseline the loop is measured
// against.  Results do not depend on what else is in a batch: every op is
// computed independently, and the tests check each result alone and in the mix.
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "common.cuh"
#include "ctx.h"
#include "kernels.h"

namespace {

using clk = std::chrono::steady_clock;

uint64_t now_ns() {
    return uint64_t(std::chrono::duration_cast<std::chrono::nanoseconds>(clk::now().time_since_epoch()).count());
}

struct Request {
    uint64_t ticket;
    const mi_op* ops;
    uint32_t n_ops;
    const uint64_t* in;
    size_t in_limbs;
    uint64_t* out;
    size_t out_limbs;
    uint8_t* carry;
    uint64_t t_submit = 0, t_admit = 0, t_done = 0;
    mi_status status = MI_OK;
    bool done = false;
    // placement inside the batch
    uint32_t op_base = 0;
    size_t in_base = 0, out_base = 0;
};

size_t round_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// Arena layout of one slot for a batch of n ops / in limbs / out limbs.
struct Layout {
    size_t ops, in, out, carry, scratch, total;
    static Layout of(size_t n_ops, size_t in_limbs, size_t out_limbs) {
        Layout L;
        L.ops = 0;
        L.in = round_up(n_ops * sizeof(mi_op), 256);
        L.out = L.in + round_up(in_limbs * 8, 256);
        L.carry = L.out + round_up(out_limbs * 8, 256);
        L.scratch = L.carry + round_up(n_ops, 256);
        L.total = L.scratch + round_up(mi::ragged_scratch_words(uint32_t(n_ops)) * 4, 256);
        return L;
    }
};

struct Slot {
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    char* dev = nullptr;
    char* host = nullptr;
    size_t cap = 0;
    bool busy = false;
    std::vector<Request*> reqs;
    Layout lay{};
    uint32_t n_ops = 0;
};

}  // namespace

struct mi_server_s {
    mi_ctx ctx = nullptr;
    mi_server_config cfg{};
    std::vector<Slot> slots;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Request*> queue;
    std::unordered_map<uint64_t, Request*> reqs;
    uint64_t next_ticket = 1;
    bool stop = false;
    std::thread loop;
    // statistics
    std::atomic<uint64_t> batches{0}, ops_done{0}, reqs_done{0};
    mi_status loop_error = MI_OK;

    void run();
    bool launch(Slot& s, std::vector<Request*>& batch);
    void finish(Slot& s);
};

void mi_server_s::run() {
    cudaSetDevice(ctx->device);
    for (;;) {
        std::vector<Request*> batch;
        Slot* free_slot = nullptr;
        {
            std::unique_lock<std::mutex> lk(mu);
            bool any_busy = false;
            for (auto& s : slots) any_busy = any_busy || s.busy;
            if (stop && queue.empty() && !any_busy) return;
            for (auto& s : slots)
                if (!s.busy) {
                    free_slot = &s;
                    break;
                }
            if (free_slot && !queue.empty()) {
                // admission: FIFO while the slot's arena has room
                size_t n = 0, in = 0, out = 0;
                while (!queue.empty()) {
                    Request* r = queue.front();
                    const size_t n2 = n + r->n_ops, in2 = in + r->in_limbs, out2 = out + r->out_limbs;
                    const bool fits = Layout::of(n2, in2, out2).total <= free_slot->cap &&
                                      (cfg.max_batch_ops == 0 || n2 <= cfg.max_batch_ops || batch.empty());
                    if (!batch.empty() && (!fits || !cfg.batching)) break;
                    r->op_base = uint32_t(n);
                    r->in_base = in;
                    r->out_base = out;
                    n = n2;
                    in = in2;
                    out = out2;
                    batch.push_back(r);
                    queue.pop_front();
                    if (!cfg.batching) break;
                }
            } else if (!any_busy && !stop) {
                cv_work.wait_for(lk, std::chrono::milliseconds(50));
                continue;
            }
        }
        if (!batch.empty()) {
            const uint64_t t = now_ns();
            for (Request* r : batch) r->t_admit = t;
            if (!launch(*free_slot, batch)) {
                std::lock_guard<std::mutex> lk(mu);
                for (Request* r : batch) {
                    r->done = true;
                    r->t_done = now_ns();
                    if (r->status == MI_OK) r->status = MI_ECUDA;
                }
                cv_done.notify_all();
            }
        }
        // completions
        bool progressed = false;
        for (auto& s : slots) {
            if (!s.busy) continue;
            const cudaError_t q = cudaEventQuery(s.done);
            if (q == cudaErrorNotReady) continue;
            if (q != cudaSuccess) {
                std::lock_guard<std::mutex> lk(mu);
                loop_error = mi::cuda_error(q, "server batch");
                for (Request* r : s.reqs) {
                    r->status = MI_ECUDA;
                    r->done = true;
                    r->t_done = now_ns();
                }
                s.reqs.clear();
                s.busy = false;
                cv_done.notify_all();
                continue;
            }
            finish(s);
            progressed = true;
        }
        if (batch.empty() && !progressed) std::this_thread::sleep_for(std::chrono::microseconds(20));
    }
}

bool mi_server_s::launch(Slot& s, std::vector<Request*>& batch) {
    size_t n = 0, in = 0, out = 0;
    for (Request* r : batch) {
        n += r->n_ops;
        in += r->in_limbs;
        out += r->out_limbs;
    }
    const Layout L = Layout::of(n, in, out);
    if (L.total > s.cap) {  // a single request larger than the arena: grow it
        if (s.dev) cudaFree(s.dev);
        if (s.host) cudaFreeHost(s.host);
        s.dev = nullptr;
        s.host = nullptr;
        s.cap = 0;
        if (cudaMalloc(&s.dev, L.total) != cudaSuccess || cudaMallocHost(&s.host, L.total) != cudaSuccess) {
            for (Request* r : batch) r->status = MI_ENOMEM;
            return false;
        }
        s.cap = L.total;
    }
    // pack into pinned staging: ops rebased onto the batch pools, operands
    mi_op* hops = reinterpret_cast<mi_op*>(s.host + L.ops);
    uint64_t* hin = reinterpret_cast<uint64_t*>(s.host + L.in);
    for (Request* r : batch) {
        for (uint32_t i = 0; i < r->n_ops; ++i) {
            mi_op o = r->ops[i];
            o.a_off += r->in_base;
            o.b_off += r->in_base;
            o.r_off += r->out_base;
            hops[r->op_base + i] = o;
        }
        std::memcpy(hin + r->in_base, r->in, r->in_limbs * 8);
    }
    cudaStream_t st = s.stream;
    bool ok = cudaMemcpyAsync(s.dev + L.ops, s.host + L.ops, n * sizeof(mi_op), cudaMemcpyHostToDevice, st) ==
                  cudaSuccess &&
              cudaMemcpyAsync(s.dev + L.in, s.host + L.in, in * 8, cudaMemcpyHostToDevice, st) == cudaSuccess;
    if (ok) {
        const mi_status rs = mi::ragged_launch(
            ctx, reinterpret_cast<const mi_op*>(s.dev + L.ops), uint32_t(n), reinterpret_cast<uint64_t*>(s.dev + L.in),
            reinterpret_cast<uint64_t*>(s.dev + L.out), reinterpret_cast<uint8_t*>(s.dev + L.carry), s.dev + L.scratch,
            L.total - L.scratch, ctx->ragged_ntt_min, st);
        ok = rs == MI_OK;
    }
    ok = ok && cudaMemcpyAsync(s.host + L.out, s.dev + L.out, out * 8, cudaMemcpyDeviceToHost, st) == cudaSuccess &&
         cudaMemcpyAsync(s.host + L.carry, s.dev + L.carry, n, cudaMemcpyDeviceToHost, st) == cudaSuccess &&
         cudaEventRecord(s.done, st) == cudaSuccess;
    if (!ok) return false;
    s.busy = true;
    s.reqs = batch;
    s.lay = L;
    s.n_ops = uint32_t(n);
    batches.fetch_add(1);
    return true;
}

void mi_server_s::finish(Slot& s) {
    const uint64_t* hout = reinterpret_cast<const uint64_t*>(s.host + s.lay.out);
    const uint8_t* hcarry = reinterpret_cast<const uint8_t*>(s.host + s.lay.carry);
    for (Request* r : s.reqs) {
        std::memcpy(r->out, hout + r->out_base, r->out_limbs * 8);
        if (r->carry) std::memcpy(r->carry, hcarry + r->op_base, r->n_ops);
    }
    std::lock_guard<std::mutex> lk(mu);
    const uint64_t t = now_ns();
    for (Request* r : s.reqs) {
        r->t_done = t;
        r->done = true;
        ops_done.fetch_add(r->n_ops);
        reqs_done.fetch_add(1);
    }
    s.reqs.clear();
    s.busy = false;
    cv_done.notify_all();
}

using namespace mi;

extern "C" {

mi_status mi_server_create(mi_ctx ctx, const mi_server_config* cfg, mi_server* out) {
    if (ctx == nullptr || cfg == nullptr || out == nullptr) return set_error(MI_EINVAL, "server_create: null argument");
    *out = nullptr;
    if (cfg->slots < 1 || cfg->slots > 8) return set_error(MI_EINVAL, "server_create: slots %u outside 1..8", cfg->slots);
    MI_CUDA_TRY(cudaSetDevice(ctx->device));
    MI_TRY(ragged_prepare());
    size_t budget = cfg->device_bytes;
    if (budget == 0) {
        size_t free_b = 0, total_b = 0;
        MI_CUDA_TRY(cudaMemGetInfo(&free_b, &total_b));
        budget = free_b / 4;
    }
    mi_server s = new (std::nothrow) mi_server_s();
    if (s == nullptr) return set_error(MI_ENOMEM, "server_create: host allocation");
    s->ctx = ctx;
    s->cfg = *cfg;
    const uint32_t nslots = cfg->batching ? cfg->slots : 1;
    s->slots.resize(nslots);
    const size_t per = budget / nslots;
    mi_status st = MI_OK;
    for (auto& sl : s->slots) {
        if (cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming) != cudaSuccess) {
            st = set_error(MI_ECUDA, "server_create: stream/event");
            break;
        }
        if (cudaMalloc(&sl.dev, per) != cudaSuccess || cudaMallocHost(&sl.host, per) != cudaSuccess) {
            st = set_error(MI_ENOMEM, "server_create: arena of %zu bytes", per);
            break;
        }
        sl.cap = per;
    }
    if (st != MI_OK) {
        for (auto& sl : s->slots) {
            if (sl.dev) cudaFree(sl.dev);
            if (sl.host) cudaFreeHost(sl.host);
            if (sl.stream) cudaStreamDestroy(sl.stream);
            if (sl.done) cudaEventDestroy(sl.done);
        }
        delete s;
        return st;
    }
    s->loop = std::thread([s] { s->run(); });
    *out = s;
    return MI_OK;
}

mi_status mi_server_destroy(mi_server s) {
    if (s == nullptr) return MI_OK;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv_work.notify_all();
    if (s->loop.joinable()) s->loop.join();
    cudaSetDevice(s->ctx->device);
    for (auto& sl : s->slots) {
        if (sl.stream) cudaStreamSynchronize(sl.stream);
        if (sl.dev) cudaFree(sl.dev);
        if (sl.host) cudaFreeHost(sl.host);
        if (sl.stream) cudaStreamDestroy(sl.stream);
        if (sl.done) cudaEventDestroy(sl.done);
    }
    for (auto& kv : s->reqs) delete kv.second;
    delete s;
    return MI_OK;
}

mi_status mi_server_submit(mi_server s, const mi_op* ops, uint32_t n_ops, const uint64_t* in, size_t in_limbs,
                           uint64_t* out, size_t out_limbs, uint8_t* carry_out, uint64_t* ticket) {
    if (s == nullptr || ticket == nullptr) return set_error(MI_EINVAL, "server_submit: null argument");
    if (n_ops == 0 || ops == nullptr || in == nullptr || out == nullptr)
        return set_error(MI_EINVAL, "server_submit: empty request or null buffer");
    for (uint32_t i = 0; i < n_ops; ++i) {  // ops must stay inside the request's pools
        const mi_op& o = ops[i];
        const uint64_t rl = o.kind == MI_OP_ADD ? (o.la > o.lb ? o.la : o.lb) : uint64_t(o.la) + o.lb;
        if (o.a_off + o.la > in_limbs || o.b_off + o.lb > in_limbs || o.r_off + rl > out_limbs)
            return set_error(MI_EINVAL, "server_submit: op %u reaches outside the request's pools", i);
    }
    Request* r = new (std::nothrow) Request();
    if (r == nullptr) return set_error(MI_ENOMEM, "server_submit: host allocation");
    r->ops = ops;
    r->n_ops = n_ops;
    r->in = in;
    r->in_limbs = in_limbs;
    r->out = out;
    r->out_limbs = out_limbs;
    r->carry = carry_out;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (s->stop) {
            delete r;
            return set_error(MI_EINVAL, "server_submit: server stopping");
        }
        r->ticket = s->next_ticket++;
        r->t_submit = now_ns();
        s->reqs[r->ticket] = r;
        s->queue.push_back(r);
    }
    s->cv_work.notify_one();
    *ticket = r->ticket;
    return MI_OK;
}

mi_status mi_server_wait(mi_server s, uint64_t ticket, int timeout_ms) {
    if (s == nullptr) return set_error(MI_EINVAL, "server_wait: null server");
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end()) return set_error(MI_EINVAL, "server_wait: unknown ticket %llu", (unsigned long long)ticket);
    Request* r = it->second;
    auto pred = [r] { return r->done; };
    if (timeout_ms < 0)
        s->cv_done.wait(lk, pred);
    else if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), pred))
        return set_error(MI_ETIMEOUT, "server_wait: ticket %llu not done", (unsigned long long)ticket);
    return r->status;
}

mi_status mi_server_request_times(mi_server s, uint64_t ticket, uint64_t* submit_ns, uint64_t* admit_ns,
                                  uint64_t* done_ns) {
    if (s == nullptr) return set_error(MI_EINVAL, "server_request_times: null server");
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end()) return set_error(MI_EINVAL, "server_request_times: unknown ticket");
    const Request* r = it->second;
    if (submit_ns) *submit_ns = r->t_submit;
    if (admit_ns) *admit_ns = r->t_admit;
    if (done_ns) *done_ns = r->t_done;
    return r->done ? r->status : MI_ETIMEOUT;
}

mi_status mi_server_release(mi_server s, uint64_t ticket) {
    if (s == nullptr) return set_error(MI_EINVAL, "server_release: null server");
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end()) return set_error(MI_EINVAL, "server_release: unknown ticket");
    if (!it->second->done) return set_error(MI_EINVAL, "server_release: request still in flight");
    delete it->second;
    s->reqs.erase(it);
    return MI_OK;
}

mi_status mi_server_stats(mi_server s, uint64_t* batches, uint64_t* requests, uint64_t* ops) {
    if (s == nullptr) return set_error(MI_EINVAL, "server_stats: null server");
    if (batches) *batches = s->batches.load();
    if (requests) *requests = s->reqs_done.load();
    if (ops) *ops = s->ops_done.load();
    return s->loop_error;
}

}  // extern "C"
