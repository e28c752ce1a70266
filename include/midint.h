/*
 * midint.h -- C ABI of the GB300 (sm_103a) batched midsize big-integer library.
 *
 * A "batch" is n independent instances stored back to back: instance i of an
 * operand with `limbs` limbs occupies limbs [i*limbs, (i+1)*limbs), limb 0 is
 * the least significant one (the layout of the reference's drivers and of its
 * GMP oracle, cuda/helper.h:116 GMP_ORDER -1).  Limbs are uint64_t (`_u64`
 * entry points) or uint32_t (`_u32`).
 *
 * Every entry point returns an mi_status and never aborts.  Device-pointer
 * entry points are asynchronous on the given stream (NULL = CUDA's default
 * stream, mi_ctx_stream(ctx) = the context's own) and never allocate; the caller owns every buffer it passes and the
 * library never frees it.  Host-pointer entry points ("compat" and "host")
 * copy through device buffers that the context keeps and grows on demand, and
 * return when the result is in host memory.
 *
 * Replaces the reference's kernel drivers in cuda/main.cu (gpuAdd :39-44,
 * gpuMultiply :221-226, gpuMulFFT :415-420) and the kernels they launch
 * (baddKer cuda/ker-addition.cu.h:227-260, bmulKerQ
 * cuda/ker-classic-mul.cu.h:468-498, bmulFFT cuda/ker-fft-mul.cu.h:427-454).
 * The reference fixes the size as a template parameter; here it is a runtime
 * argument.
 */
#ifndef MIDINT_H
#define MIDINT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum mi_status {
    MI_OK = 0,
    MI_EINVAL = 1,   /* null pointer, zero/oversized length, misaligned buffer */
    MI_ENOMEM = 2,   /* a device or pinned-host allocation failed            */
    MI_ECUDA = 3,    /* a CUDA runtime call or a kernel launch failed         */
    MI_ETIMEOUT = 4, /* a bounded device-side wait gave up (no hang)          */
    MI_ENODEV = 5,   /* no usable CUDA device                                  */
    MI_ENOTSUP = 6   /* combination of arguments not supported                 */
} mi_status;

/* Opaque per-device context: resident NTT twiddle tables, staging buffers for
 * the host-pointer calls, the tuned dispatch table and one CUDA stream. */
typedef struct mi_ctx_s* mi_ctx;

/* A cudaStream_t passed as a plain pointer (NULL = CUDA's default stream). */
typedef void* mi_stream;

/* Largest operand length, in u64 limbs, of the plain multiplication kernels
 * (classical, NTT, poly): 131072 bits, the largest size the reference's
 * drivers run (cuda/main.cu:693-703).  u32 entry points accept twice as many
 * limbs; additions take up to 4096 u64 limbs; ragged ops up to 1024. */
#define MI_MAX_LIMBS_U64 2048u

/* ---------------------------------------------------------------------------
 * Library / context
 * ------------------------------------------------------------------------- */

/* Version as 10000*major + 100*minor + patch. */
int mi_version(void);

/* Static text for a status code. */
const char* mi_status_string(int status);

/* Detail of the last failure on the calling thread ("" if none). */
const char* mi_last_error(void);

/* Creates a context on `device` (cudaSetDevice semantics, checked). */
mi_status mi_ctx_create(int device, mi_ctx* out);

/* Destroys a context, after waiting for its stream. NULL is accepted. */
mi_status mi_ctx_destroy(mi_ctx ctx);

/* Waits for all work queued on the context's stream. */
mi_status mi_ctx_synchronize(mi_ctx ctx);

/* The context's own stream, as a cudaStream_t. */
mi_stream mi_ctx_stream(mi_ctx ctx);

/* Classical/NTT crossovers of a context, in u64 limbs: ragged runs send a
 * product through the NTT kernel when its shorter operand has at least
 * ragged_ntt_min limbs (1..257; classical groups hold at most 256), and
 * mi_mul_u64 does so when its operands have at least plain_ntt_min limbs
 * (1..2049; 2049 = never).  Defaults come from the committed tuning table.
 * (mi_mul_lo_u64 has its own crossover, MI_TUNE_LO_NTT_MIN.) */
mi_status mi_ctx_set_crossover(mi_ctx ctx, uint32_t ragged_ntt_min, uint32_t plain_ntt_min);

/* Tunable launch choices of a context.  A new context starts from the table
 * that the project's autotuner measured and committed; these calls override
 * one entry (the autotuner itself sweeps candidates through them).
 *   MI_TUNE_PLAIN_NTT_MIN    cls ignored; value 1..2049 (as plain_ntt_min)
 *   MI_TUNE_RAGGED_NTT_MIN   cls 0: value 1..257 (as ragged_ntt_min);
 *                            cls 1: value 1..257, products whose NTT runs
 *                            on 40-bit digits and three primes (their
 *                            digits fill at most 5/8 of the transform
 *                            length) use the NTT kernel from this many
 *                            limbs of the shorter operand on, even below
 *                            ragged_ntt_min
 *   MI_TUNE_LO_NTT_MIN       cls ignored; value 1..2049: mi_mul_lo_u64 and
 *                            the u64 gpuMultiply wrapper compute the low
 *                            half with the NTT kernel from this many limbs
 *                            on (2049 = never)
 *   MI_TUNE_ADD_THREAD_BYTES cls = ceil(log2(u64 limbs)) 0..12 of the
 *                            operands; value = bytes of each operand one
 *                            thread owns: 16, 32 or 64
 *   MI_TUNE_HOST_CHUNKS      cls = 0 additions, 1 multiplications; value
 *                            1..64: chunks a host-buffer batch is cut into
 *                            for copy/compute overlap
 *   MI_TUNE_HOST_ZERO_COPY   cls as above; value 0: copies both ways;
 *                            1: when every buffer is mapped pinned memory,
 *                            the kernel reads and writes them in place;
 *                            2: when the operands are mapped pinned memory,
 *                            the kernel reads them in place and the results
 *                            are copied out in chunks (the buffers must hold
 *                            the whole batch, as for the copies);
 *                            3: when the results are mapped pinned memory,
 *                            the operands are copied in by chunks and the
 *                            kernels write the results in place */
enum {
    MI_TUNE_PLAIN_NTT_MIN = 0,
    MI_TUNE_RAGGED_NTT_MIN = 1,
    MI_TUNE_ADD_THREAD_BYTES = 2,
    MI_TUNE_HOST_CHUNKS = 3,
    MI_TUNE_HOST_ZERO_COPY = 4,
    MI_TUNE_WIDE_SPIN_LIMIT = 5, /* cls ignored; polls of an unpublished
                                  * predecessor before a multi-block addition
                                  * gives up (default 2^20, about 70 ms) */
    MI_TUNE_WIDE_WITHHOLD = 6,   /* cls ignored; 0 or 1.  Failure injection for
                                  * tests: the first tile of every instance
                                  * never publishes its carry, so the waits of
                                  * its successors run out (bounded) */
    MI_TUNE_WIDE_ROUND_TILES = 7, /* cls ignored; 1..65536: tiles (2048 u64 limbs
                                   * each) per multi-block launch; an instance
                                   * may not need more (default 65536) */
    MI_TUNE_HOST_ZC_BLOCKS = 8,   /* cls as for MI_TUNE_HOST_CHUNKS; value 0..3:
                                   * with zero-copy mode 1, at most this many
                                   * blocks per SM for the classical
                                   * multiplication kernel (0: as many as fit).
                                   * Fewer resident blocks make the first
                                   * results leave over the host link sooner */
    MI_TUNE_LO_NTT_MIN = 9,
    MI_TUNE_POLY_NTT_MIN = 10     /* cls ignored; value 1..2049: mi_poly_u64
                                   * runs its four products on number-theoretic
                                   * transforms from this many limbs on
                                   * (2049 = never) */
};
mi_status mi_ctx_set_tuning(mi_ctx ctx, int knob, uint32_t cls, uint32_t value);

/* Waits for all work on the context's device, then reports (and clears) the
 * context's device-side error state: MI_ETIMEOUT when a bounded wait of a
 * multi-block addition gave up since the last report, else MI_OK. */
mi_status mi_ctx_device_status(mi_ctx ctx);
mi_status mi_ctx_get_tuning(mi_ctx ctx, int knob, uint32_t cls, uint32_t* value);

/* ---------------------------------------------------------------------------
 * Batched addition  r = (a + b) mod 2^(bits*limbs), carry_out[i] = carry bit.
 * Replaces baddKer<Base,IPB,M,Q> (cuda/ker-addition.cu.h:227-260) as launched
 * by gpuAdd (cuda/main.cu:39-119).  The reference discards the carry-out;
 * carry_out may be NULL to do the same.  a, b, r: n*limbs limbs each.
 * r may alias a or b exactly (in-place), but must not partially overlap.
 * limbs <= 2^26 u64 limbs (2^27 u32): instances wider than 4096 u64 limbs run
 * a multi-block kernel whose tiles chain their carries by decoupled
 * look-back with bounded waits; such calls on one context must not overlap on
 * the device, and a wait that gave up is reported by mi_ctx_device_status
 * (and by the host-buffer calls) as MI_ETIMEOUT.
 * ------------------------------------------------------------------------- */
mi_status mi_add_u64(mi_ctx ctx, const uint64_t* a, const uint64_t* b, uint64_t* r,
                     uint8_t* carry_out, uint32_t n, uint32_t limbs, mi_stream stream);
mi_status mi_add_u32(mi_ctx ctx, const uint32_t* a, const uint32_t* b, uint32_t* r,
                     uint8_t* carry_out, uint32_t n, uint32_t limbs, mi_stream stream);

/* Fused six-addition composite r = 6a + 10b (mod 2^(bits*limbs)), the value of
 * the reference's chain t1=a+b, t2=2t1, t3=t2+b, t4=2t3, t5=t4+t3, r=t5+b,
 * formed per limb as 6a_i + 10b_i with one carry pass.  Replaces a6pb10Ker
 * (cuda/ker-addition.cu.h:266-328). */
mi_status mi_add6_u64(mi_ctx ctx, const uint64_t* a, const uint64_t* b, uint64_t* r,
                      uint32_t n, uint32_t limbs, mi_stream stream);

/* ---------------------------------------------------------------------------
 * Classical (quadratic) multiplication.
 * mi_mul_lo_*:   r = a*b mod 2^(bits*limbs)   (n*limbs limbs)  -- the
 *                reference's bmulKerQ semantics (cuda/ker-classic-mul.cu.h:
 *                468-498, driven by gpuMultiply cuda/main.cu:221-315).
 *                mi_mul_lo_u64 switches to the exact NTT kernel, storing the
 *                low limbs only, from MI_TUNE_LO_NTT_MIN limbs on (tuned:
 *                where the NTT's full product costs less than the classical
 *                low half); the result is the same either way.
 * mi_mul_full_*: r = a*b                      (n*2*limbs limbs).
 * r must not overlap a or b.
 * ------------------------------------------------------------------------- */
mi_status mi_mul_lo_u64(mi_ctx ctx, const uint64_t* a, const uint64_t* b, uint64_t* r,
                        uint32_t n, uint32_t limbs, mi_stream stream);
mi_status mi_mul_lo_u32(mi_ctx ctx, const uint32_t* a, const uint32_t* b, uint32_t* r,
                        uint32_t n, uint32_t limbs, mi_stream stream);
mi_status mi_mul_full_u64(mi_ctx ctx, const uint64_t* a, const uint64_t* b, uint64_t* r,
                          uint32_t n, uint32_t limbs, mi_stream stream);
mi_status mi_mul_full_u32(mi_ctx ctx, const uint32_t* a, const uint32_t* b, uint32_t* r,
                          uint32_t n, uint32_t limbs, mi_stream stream);

/* Fused polynomial composite r = ((a^2 + b)(b^2 + b) + ab) mod 2^(64*limbs),
 * every intermediate mod 2^(64*limbs) and held on chip, limbs <= 2048.
 * Replaces polyKerQ (cuda/ker-classic-mul.cu.h:500-575), four classical
 * low-half products, and from MI_TUNE_POLY_NTT_MIN limbs on polyFttKer
 * (cuda/ker-fft-mul.cu.h:456-509), the same four products on exact
 * number-theoretic transforms; the result is the same either way. */
mi_status mi_poly_u64(mi_ctx ctx, const uint64_t* a, const uint64_t* b, uint64_t* r,
                      uint32_t n, uint32_t limbs, mi_stream stream);

/* ---------------------------------------------------------------------------
 * GMP word formats.  The reference moves every operand through mpz_import /
 * mpz_export with order -1 and 4-byte native words (cuda/helper.h:116,
 * 146-170), the same bytes as this library's limbs; these convert batches in
 * any other mpz_import / mpz_export word format on the device.  A field is
 * `words` words of `size` bytes (1, 2, 4 or 8) per instance; order 1 = most
 * significant word first, -1 = least significant first; endian 1 = big-endian
 * bytes within a word, 0 or -1 = little-endian (native on every supported
 * host); nails are not supported.
 * mi_import_words: n fields -> n*limbs u64 limbs (values mod 2^(64*limbs),
 *   shorter fields zero-extended), like mpz_import per instance.  src aligned
 *   to `size`.
 * mi_export_words: n*limbs limbs -> n fixed-width fields: the value's words at
 *   the least significant end of the field (the start for order -1, the end for
 *   order 1), zero words elsewhere -- mpz_export's words right- or
 *   left-aligned in the field; a value wider than the field keeps its low
 *   words.  counts (nullable) receives mpz_export's count of significant words
 *   per instance (0 for zero; more than `words` when the value did not fit).
 * ------------------------------------------------------------------------- */
mi_status mi_import_words(mi_ctx ctx, const void* src, uint32_t n, uint32_t words, uint32_t size,
                          int order, int endian, uint64_t* dst, uint32_t limbs, mi_stream stream);
mi_status mi_export_words(mi_ctx ctx, const uint64_t* src, uint32_t n, uint32_t limbs, void* dst,
                          uint32_t words, uint32_t size, int order, int endian, uint32_t* counts,
                          mi_stream stream);

/* ---------------------------------------------------------------------------
 * Exact NTT multiplication r = a*b (n*2*limbs limbs), limbs <= 2048: every u64
 * limb is one digit and five 30-bit primes carry the convolution, or, when
 * 48-bit digits fit the same power-of-two length (2*ceil(4*limbs/3) <= L),
 * 48-bit digits on four of the primes (Shoup and Montgomery products on
 * 32-bit residues); Garner's CRT and the final carry run in the same kernel.  Replaces bmulFFT<P,M,Q>
 * (cuda/ker-fft-mul.cu.h:427-454) as launched by gpuMulFFT
 * (cuda/main.cu:415-520); unlike it, the result is exact at every size.
 * mi_mul_u64 picks the classical or the NTT kernel by size.
 * r must not overlap a or b.  mi_mul_ntt_u64 needs 8-byte aligned buffers
 * (MI_EINVAL otherwise); mi_mul_u64, mi_mul_lo_u64 and mi_poly_u64 use the
 * transforms only for 8-byte aligned buffers and the classical kernels
 * (which read 32-bit words) for the others.
 * ------------------------------------------------------------------------- */
mi_status mi_mul_ntt_u64(mi_ctx ctx, const uint64_t* a, const uint64_t* b, uint64_t* r,
                         uint32_t n, uint32_t limbs, mi_stream stream);
mi_status mi_mul_u64(mi_ctx ctx, const uint64_t* a, const uint64_t* b, uint64_t* r,
                     uint32_t n, uint32_t limbs, mi_stream stream);

/* ---------------------------------------------------------------------------
 * Host-pointer compatibility wrappers with the shapes of the reference's
 * drivers: synchronous, the context is a lazily created one on the current
 * device, buffers are caller-owned host memory (pinned or pageable), output
 * truncated to m limbs exactly as the reference does.
 *   gpuAdd<Base,m>      cuda/main.cu:39-44
 *   gpuMultiply<Base,m> cuda/main.cu:221-226
 * ------------------------------------------------------------------------- */
mi_status mi_compat_gpuAdd_u64(int num_instances, uint32_t m, const uint64_t* h_as,
                               const uint64_t* h_bs, uint64_t* h_rs);
mi_status mi_compat_gpuAdd_u32(int num_instances, uint32_t m, const uint32_t* h_as,
                               const uint32_t* h_bs, uint32_t* h_rs);
mi_status mi_compat_gpuMultiply_u64(int num_instances, uint32_t m, const uint64_t* h_as,
                                    const uint64_t* h_bs, uint64_t* h_rs);
mi_status mi_compat_gpuMultiply_u32(int num_instances, uint32_t m, const uint32_t* h_as,
                                    const uint32_t* h_bs, uint32_t* h_rs);
/* gpuMulFFT<FftPrime32, M> (cuda/main.cu:415-420): M 16-bit digits per
 * instance in, the low M digits of the product out, packed as u16 digits at
 * digit offset i*M of the output buffer (its first half; the buffer holds M
 * u32 words per instance), exactly where the reference's kernel writes them
 * (cuda/ker-fft-mul.cu.h:451-452).  This is the exact result the reference's
 * disabled validation expects (cuda/main.cu:598-608).  M must be a multiple
 * of 4 and at most 8192 (the largest M the reference's kernel can launch:
 * M/8 threads per block at its Q = 4). */
mi_status mi_compat_gpuMulFFT_u16(int num_instances, uint32_t M, const uint16_t* h_as,
                                  const uint16_t* h_bs, uint32_t* h_rs);

/* ---------------------------------------------------------------------------
 * Host-buffer end-to-end calls on an explicit context: copy in, compute, copy
 * out, on the context's stream, pipelined in chunks so that copies overlap the
 * kernels.  Same semantics as the device-pointer calls above.
 * ------------------------------------------------------------------------- */
mi_status mi_host_add_u64(mi_ctx ctx, const uint64_t* h_a, const uint64_t* h_b,
                          uint64_t* h_r, uint8_t* h_carry, uint32_t n, uint32_t limbs);
mi_status mi_host_mul_full_u64(mi_ctx ctx, const uint64_t* h_a, const uint64_t* h_b,
                               uint64_t* h_r, uint32_t n, uint32_t limbs);

/* ---------------------------------------------------------------------------
 * Ragged batches: one list of adds and multiplies of uneven lengths, run by
 * persistent kernels that bin the list by size class on the device.  No
 * reference counterpart: the reference launches one kernel per operation and
 * size (cuda/main.cu:661-746) with both operands of one compile-time size.
 *
 * Each op reads a (la limbs) and b (lb limbs) from the u64 input pool at limb
 * offsets a_off, b_off and writes its result at limb offset r_off of the
 * output pool: an add writes max(la, lb) limbs (the sum modulo 2^(64 max))
 * and, if carry_out is given, carry_out[op index]; a multiply writes la + lb
 * limbs (the full product).  1 <= la, lb <= 1024.  Results must not overlap
 * each other or the inputs.  ops, in and out must be 8-byte aligned.  Ops with a bad kind or length are skipped and
 * counted (mi_ragged_invalid).
 * ------------------------------------------------------------------------- */
#define MI_OP_ADD 0u
#define MI_OP_MUL 1u

typedef struct mi_op {
    uint32_t kind;  /* MI_OP_ADD or MI_OP_MUL */
    uint32_t la;    /* limbs of a */
    uint32_t lb;    /* limbs of b */
    uint32_t flags; /* reserved, 0 */
    uint64_t a_off; /* limb offset of a in the input pool */
    uint64_t b_off; /* limb offset of b in the input pool */
    uint64_t r_off; /* limb offset of the result in the output pool */
} mi_op;

/* Device scratch a ragged run needs for n_ops operations. */
mi_status mi_ragged_scratch_bytes(uint32_t n_ops, size_t* bytes);

/* Runs the ops (device arrays) asynchronously on `stream`: classify, scan,
 * scatter, then one persistent kernel per family (NTT products, classical
 * rectangular products, additions), each consuming its tasks longest first
 * from an atomic queue.  `scratch` is caller-owned device memory of at least
 * mi_ragged_scratch_bytes(n_ops).  The first call on a device loads the
 * size-class order tables; make it before capturing a stream. */
mi_status mi_ragged_run(mi_ctx ctx, const mi_op* ops, uint32_t n_ops, const uint64_t* in, uint64_t* out,
                        uint8_t* carry_out, void* scratch, size_t scratch_bytes, mi_stream stream);

/* Number of ops the last run on this scratch skipped as invalid (synchronous). */
mi_status mi_ragged_invalid(const void* scratch, uint32_t* count);

/* The ragged run of mi_ragged_run for callers that cannot allocate device
 * memory -- code that runs inside another framework's memory pool or under a
 * fixed device-memory budget, where a cudaMalloc would fail or is not
 * allowed.  It allocates nothing: its scratch is a static device array of the
 * library sized for at most MI_RAGGED_NOALLOC_MAX_OPS ops (about 0.5 MiB, held
 * by every GPU that loads the library until the process exits); larger lists
 * are refused with MI_EINVAL.  The first call on a device looks the array up
 * (and loads the size-class tables); make it before capturing any stream.
 * All calls share the array, so calls whose work overlaps on the GPU race:
 * order them on one stream.  The context is created beforehand as usual.
 * The array's device address is looked up once per device and kept for the
 * life of the process, so the library is not usable on a device after a
 * cudaDeviceReset there (its contexts are not either).
 * No counterpart in the reference. */
#define MI_RAGGED_NOALLOC_MAX_OPS 65536u
mi_status mi_ragged_run_noalloc(mi_ctx ctx, const mi_op* ops, uint32_t n_ops, const uint64_t* in, uint64_t* out,
                                uint8_t* carry_out, mi_stream stream);

/* Number of ops the last mi_ragged_run_noalloc on the context's device
 * skipped as invalid, read from the static array (synchronous, allocates
 * nothing).  No counterpart in the reference. */
mi_status mi_ragged_invalid_noalloc(mi_ctx ctx, uint32_t* count);

/* The same run captured once into a CUDA graph and replayed. */
typedef struct mi_graph_s* mi_graph;
mi_status mi_ragged_graph_create(mi_ctx ctx, const mi_op* ops, uint32_t n_ops, const uint64_t* in, uint64_t* out,
                                 uint8_t* carry_out, void* scratch, size_t scratch_bytes, mi_graph* graph);
mi_status mi_graph_launch(mi_graph graph, mi_stream stream);
mi_status mi_graph_destroy(mi_graph graph);

/* ---------------------------------------------------------------------------
 * Serving: a request loop with continuous batching.  No reference
 * counterpart (the reference runs one synchronous batch per size).
 *
 * A request is a ragged op list (mi_op, offsets into the request's own pools)
 * with host buffers that stay valid until it completes.  A loop thread
 * admits queued requests FIFO into the next free batch slot while the slot's
 * device arena has room (memory-based admission), so requests that arrive
 * while other batches are on the GPU join the next batch; each slot has its
 * own stream, so batches overlap on the device.  batching = 0 gives the plain
 * per-request form: one request per launch, one slot.
 * ------------------------------------------------------------------------- */
typedef struct mi_server_s* mi_server;

typedef struct mi_server_config {
    size_t device_bytes;    /* device memory for in-flight batches (0 = 1/4 of free memory) */
    uint32_t slots;         /* batches in flight at once, 1..8 */
    uint32_t max_batch_ops; /* cap on ops per batch (0 = none) */
    uint32_t batching;      /* 1 = continuous batching, 0 = one request per launch */
    uint32_t reserved;      /* 0 */
} mi_server_config;

mi_status mi_server_create(mi_ctx ctx, const mi_server_config* config, mi_server* server);
/* Finishes every queued and in-flight request, then frees the server. */
mi_status mi_server_destroy(mi_server server);
/* Queues a request; non-blocking.  Ops must stay inside the request's pools
 * (in: in_limbs limbs, out: out_limbs limbs); carry_out may be NULL. */
mi_status mi_server_submit(mi_server server, const mi_op* ops, uint32_t n_ops, const uint64_t* in,
                           size_t in_limbs, uint64_t* out, size_t out_limbs, uint8_t* carry_out,
                           uint64_t* ticket);
/* Waits for a request (timeout_ms < 0: no limit); MI_ETIMEOUT if not done. */
mi_status mi_server_wait(mi_server server, uint64_t ticket, int timeout_ms);
/* Host steady-clock times (ns) of submission, admission and completion. */
mi_status mi_server_request_times(mi_server server, uint64_t ticket, uint64_t* submit_ns,
                                  uint64_t* admit_ns, uint64_t* done_ns);
/* Forgets a finished request. */
mi_status mi_server_release(mi_server server, uint64_t ticket);
/* Batches launched, requests and ops finished so far. */
mi_status mi_server_stats(mi_server server, uint64_t* batches, uint64_t* requests, uint64_t* ops);

/* ---------------------------------------------------------------------------
 * Calibration: throughput of the integer multiply pipe on this device, in
 * 32x32-bit partial products per second, measured with independent carry
 * chains of the instruction mix the multiplication kernels issue
 * (mad.lo.cc / madc.hi.cc).  The denominator of the multiplication kernels'
 * roofline.  Counterpart of testBasicOps (cuda/ker-helpers.cu.h:226-317).
 * iters = 0 picks a default (~tens of ms).  Synchronous; current device.
 * ------------------------------------------------------------------------- */
mi_status mi_calib_mul32_peak(uint32_t iters, double* products_per_s, double* seconds);

/* Calibration of the host link as the zero-copy host-buffer calls use it:
 * the SMs streaming `bytes` of mapped pinned host memory in 16-byte accesses
 * -- reads of host_src, writes of host_dst, and a copy of bytes/2 from one to
 * the other (both directions at once) -- in GB/s of bytes moved, best of 5.
 * bytes a positive multiple of 32, both buffers 16-byte aligned, pinned and
 * mapped (cudaHostAlloc under unified addressing).  The denominator of the
 * end-to-end roofline.  Synchronous; current device.  No counterpart in the
 * reference (its drivers copy with cudaMemcpy only). */
mi_status mi_calib_host_link(const void* host_src, void* host_dst, size_t bytes, double* read_gbs,
                             double* write_gbs, double* both_gbs);

/* ---------------------------------------------------------------------------
 * One NTT on a single caller-chosen prime, in 64-bit Montgomery fields (a
 * separate radix-8 transform, csrc/ntt.cuh, that can run the reference's own
 * primes; the multiplication kernels use the 30-bit transform of
 * mi_ntt32_raw below): conv = 0 gives the forward transform of `a` in natural
 * order (the reference's fft, cuda/ker-fft-mul.cu.h:304-348), conv = 1 the
 * cyclic convolution of a and b mod p (bmulFFTvalid,
 * cuda/ker-fft-mul.cu.h:512-554).  p odd < 2^62, g of order 2^two_adicity
 * (two_adicity >= 12), len a power of two in [8, 2048]; host buffers of len
 * words; synchronous.  Used to check a transform of the reference's shape
 * against the reference's known answers.
 * ------------------------------------------------------------------------- */
mi_status mi_ntt_raw(uint64_t p, uint64_t g, uint32_t two_adicity, uint32_t len, int conv,
                     const uint64_t* h_a, const uint64_t* h_b, uint64_t* h_out);

/* ---------------------------------------------------------------------------
 * The transform that the NTT multiplication kernels run (csrc/ntt32.cuh), on
 * its own, on production prime number `prime` (0..4, the five 30-bit primes
 * of mi_ntt32_prime) with the context's resident twiddles: conv = 0 gives the
 * forward transform of `a` in natural order, X_k = sum_i a_i w^(ik) mod p with
 * w = g^((p-1)/len); conv = 1 the cyclic convolution of a and b mod p, by the
 * same per-prime steps as a multiplication (b scaled by 2^32/L, lockstep
 * forward transforms, Montgomery pointwise product, inverse transform).
 * Replaces the role of the reference's fft / bmulFFTvalid
 * (cuda/ker-fft-mul.cu.h:304-348, 512-554) as the transform-level check.
 * len a power of two in [256, 4096]; inputs are reduced mod p; host buffers
 * of len words; synchronous.
 * ------------------------------------------------------------------------- */
mi_status mi_ntt32_raw(mi_ctx ctx, uint32_t prime, uint32_t len, int conv, const uint32_t* h_a,
                       const uint32_t* h_b, uint32_t* h_out);

/* Prime number `prime` (0..4) of the NTT multiplication kernels and its
 * primitive root. */
mi_status mi_ntt32_prime(uint32_t prime, uint32_t* p, uint32_t* g);

#ifdef __cplusplus
}
#endif

#endif /* MIDINT_H */
