"""Python host mirror of the library's C ABI (include/midint.h).

Two layers, both thin ctypes bindings over libmidint_gb300.so:

* Reference-shaped drivers with the names and argument meaning of the
  reference's cuda/main.cu: ``gpuAdd(Base, m, num_instances, h_as, h_bs,
  h_rs)`` (cuda/main.cu:39-44) and ``gpuMultiply(Base, m, ...)``
  (cuda/main.cu:221-226) on host numpy arrays, with ``U64bits`` / ``U32bits``
  standing for the reference's limb traits (cuda/ker-helpers.cu.h:12-28).
  Unlike the reference, which prints CUDA errors and carries on
  (cuda/helper.h:13-19), every failure raises MidintError.
* Device-pointer calls on a Context (``add``, ``add6``, ``mul_lo``,
  ``mul_full``): arguments are CUDA device pointers (ints) or objects with a
  ``data_ptr()`` method such as torch tensors; the call is asynchronous on the
  given stream.

There is no fallback: if the shared library is missing the first call raises.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmidint_gb300.so")

MI_OK, MI_EINVAL, MI_ENOMEM, MI_ECUDA, MI_ETIMEOUT, MI_ENODEV, MI_ENOTSUP = range(7)
MAX_LIMBS_U64 = 2048
RAGGED_NOALLOC_MAX_OPS = 65536

# Every symbol include/midint.h declares, with (restype, argtypes).
_P, _U32, _I = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_int
_S = ctypes.c_int  # mi_status
(TUNE_PLAIN_NTT_MIN, TUNE_RAGGED_NTT_MIN, TUNE_ADD_THREAD_BYTES, TUNE_HOST_CHUNKS, TUNE_HOST_ZERO_COPY,
 TUNE_WIDE_SPIN_LIMIT, TUNE_WIDE_WITHHOLD, TUNE_WIDE_ROUND_TILES, TUNE_HOST_ZC_BLOCKS, TUNE_LO_NTT_MIN,
 TUNE_POLY_NTT_MIN) = range(11)
SIGNATURES = {
    "mi_version": (_I, []),
    "mi_status_string": (ctypes.c_char_p, [_I]),
    "mi_last_error": (ctypes.c_char_p, []),
    "mi_ctx_create": (_S, [_I, ctypes.POINTER(_P)]),
    "mi_ctx_destroy": (_S, [_P]),
    "mi_ctx_synchronize": (_S, [_P]),
    "mi_ctx_stream": (_P, [_P]),
    "mi_ctx_set_crossover": (_S, [_P, _U32, _U32]),
    "mi_ctx_set_tuning": (_S, [_P, _I, _U32, _U32]),
    "mi_ctx_get_tuning": (_S, [_P, _I, _U32, _P]),
    "mi_ctx_device_status": (_S, [_P]),
    "mi_add_u64": (_S, [_P, _P, _P, _P, _P, _U32, _U32, _P]),
    "mi_add_u32": (_S, [_P, _P, _P, _P, _P, _U32, _U32, _P]),
    "mi_add6_u64": (_S, [_P, _P, _P, _P, _U32, _U32, _P]),
    "mi_mul_lo_u64": (_S, [_P, _P, _P, _P, _U32, _U32, _P]),
    "mi_mul_lo_u32": (_S, [_P, _P, _P, _P, _U32, _U32, _P]),
    "mi_mul_full_u64": (_S, [_P, _P, _P, _P, _U32, _U32, _P]),
    "mi_mul_full_u32": (_S, [_P, _P, _P, _P, _U32, _U32, _P]),
    "mi_compat_gpuAdd_u64": (_S, [_I, _U32, _P, _P, _P]),
    "mi_compat_gpuAdd_u32": (_S, [_I, _U32, _P, _P, _P]),
    "mi_compat_gpuMultiply_u64": (_S, [_I, _U32, _P, _P, _P]),
    "mi_compat_gpuMultiply_u32": (_S, [_I, _U32, _P, _P, _P]),
    "mi_host_add_u64": (_S, [_P, _P, _P, _P, _P, _U32, _U32]),
    "mi_host_mul_full_u64": (_S, [_P, _P, _P, _P, _U32, _U32]),
    "mi_calib_mul32_peak": (_S, [_U32, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]),
    "mi_calib_host_link": (_S, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_double),
                                ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]),
    "mi_mul_ntt_u64": (_S, [_P, _P, _P, _P, _U32, _U32, _P]),
    "mi_poly_u64": (_S, [_P, _P, _P, _P, _U32, _U32, _P]),
    "mi_import_words": (_S, [_P, _P, _U32, _U32, _U32, _I, _I, _P, _U32, _P]),
    "mi_export_words": (_S, [_P, _P, _U32, _U32, _P, _U32, _U32, _I, _I, _P, _P]),
    "mi_mul_u64": (_S, [_P, _P, _P, _P, _U32, _U32, _P]),
    "mi_compat_gpuMulFFT_u16": (_S, [_I, _U32, _P, _P, _P]),
    "mi_ntt_raw": (_S, [ctypes.c_uint64, ctypes.c_uint64, _U32, _U32, _I, _P, _P, _P]),
    "mi_ntt32_raw": (_S, [_P, _U32, _U32, _I, _P, _P, _P]),
    "mi_ntt32_prime": (_S, [_U32, ctypes.POINTER(_U32), ctypes.POINTER(_U32)]),
    "mi_ragged_scratch_bytes": (_S, [_U32, ctypes.POINTER(ctypes.c_size_t)]),
    "mi_ragged_run": (_S, [_P, _P, _U32, _P, _P, _P, _P, ctypes.c_size_t, _P]),
    "mi_ragged_invalid": (_S, [_P, ctypes.POINTER(_U32)]),
    "mi_ragged_run_noalloc": (_S, [_P, _P, _U32, _P, _P, _P, _P]),
    "mi_ragged_invalid_noalloc": (_S, [_P, ctypes.POINTER(_U32)]),
    "mi_ragged_graph_create": (_S, [_P, _P, _U32, _P, _P, _P, _P, ctypes.c_size_t, ctypes.POINTER(_P)]),
    "mi_graph_launch": (_S, [_P, _P]),
    "mi_graph_destroy": (_S, [_P]),
    "mi_server_create": (_S, [_P, _P, ctypes.POINTER(_P)]),
    "mi_server_destroy": (_S, [_P]),
    "mi_server_submit": (_S, [_P, _P, _U32, _P, ctypes.c_size_t, _P, ctypes.c_size_t, _P,
                              ctypes.POINTER(ctypes.c_uint64)]),
    "mi_server_wait": (_S, [_P, ctypes.c_uint64, _I]),
    "mi_server_request_times": (_S, [_P, ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint64),
                                     ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64)]),
    "mi_server_release": (_S, [_P, ctypes.c_uint64]),
    "mi_server_stats": (_S, [_P, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64),
                             ctypes.POINTER(ctypes.c_uint64)]),
}


class ServerConfig(ctypes.Structure):
    """struct mi_server_config of include/midint.h."""
    _fields_ = [("device_bytes", ctypes.c_size_t), ("slots", ctypes.c_uint32), ("max_batch_ops", ctypes.c_uint32),
                ("batching", ctypes.c_uint32), ("reserved", ctypes.c_uint32)]

MI_OP_ADD, MI_OP_MUL = 0, 1
# struct mi_op of include/midint.h (40 bytes)
OP_DTYPE = np.dtype([("kind", "<u4"), ("la", "<u4"), ("lb", "<u4"), ("flags", "<u4"),
                     ("a_off", "<u8"), ("b_off", "<u8"), ("r_off", "<u8")])


class MidintError(RuntimeError):
    def __init__(self, status: int, detail: str):
        super().__init__(f"{_status_name(status)}: {detail}")
        self.status = status
        self.detail = detail


_lib: ctypes.CDLL | None = None


def load() -> ctypes.CDLL:
    """Loads libmidint_gb300.so (built by build.py); raises if it is absent."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is not built: run `python midint-arithmetic_gb300/build.py`")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _status_name(st: int) -> str:
    try:
        return load().mi_status_string(st).decode()
    except Exception:  # pragma: no cover - only when the library itself is missing
        return f"status {st}"


def check(st: int) -> None:
    if st != MI_OK:
        raise MidintError(st, load().mi_last_error().decode())


def _ptr(x) -> int | None:
    if x is None:
        return None
    if isinstance(x, int):
        return x
    if isinstance(x, np.ndarray):
        return x.ctypes.data
    return x.data_ptr()


class Context:
    """An mi_ctx: one device, its own stream, resident tables and staging."""

    def __init__(self, device: int = 0):
        h = ctypes.c_void_p()
        check(load().mi_ctx_create(device, ctypes.byref(h)))
        self.handle = h.value
        self.device = device

    @property
    def stream(self) -> int:
        return load().mi_ctx_stream(self.handle) or 0

    def synchronize(self) -> None:
        check(load().mi_ctx_synchronize(self.handle))

    def set_crossover(self, ragged_ntt_min: int, plain_ntt_min: int) -> None:
        check(load().mi_ctx_set_crossover(self.handle, ragged_ntt_min, plain_ntt_min))

    def set_tuning(self, knob: int, cls: int, value: int) -> None:
        """Overrides one entry of the context's tuning table (TUNE_* knobs)."""
        check(load().mi_ctx_set_tuning(self.handle, knob, cls, value))

    def device_status(self) -> int:
        """Waits for the device, then MI_OK or MI_ETIMEOUT (a bounded wait of a
        multi-block addition gave up); the state is cleared by reading it."""
        return load().mi_ctx_device_status(self.handle)

    def get_tuning(self, knob: int, cls: int = 0) -> int:
        v = ctypes.c_uint32()
        check(load().mi_ctx_get_tuning(self.handle, knob, cls, ctypes.byref(v)))
        return v.value

    def close(self) -> None:
        if self.handle:
            load().mi_ctx_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):  # pragma: no cover
        try:
            self.close()
        except Exception:
            pass

    # --- device-pointer calls ---------------------------------------------
    def add(self, a, b, r, n: int, limbs: int, carry=None, limb_bits: int = 64, stream=None) -> None:
        f = load().mi_add_u64 if limb_bits == 64 else load().mi_add_u32
        check(f(self.handle, _ptr(a), _ptr(b), _ptr(r), _ptr(carry), n, limbs, _ptr(stream)))

    def add6(self, a, b, r, n: int, limbs: int, stream=None) -> None:
        check(load().mi_add6_u64(self.handle, _ptr(a), _ptr(b), _ptr(r), n, limbs, _ptr(stream)))

    def mul_lo(self, a, b, r, n: int, limbs: int, limb_bits: int = 64, stream=None) -> None:
        f = load().mi_mul_lo_u64 if limb_bits == 64 else load().mi_mul_lo_u32
        check(f(self.handle, _ptr(a), _ptr(b), _ptr(r), n, limbs, _ptr(stream)))

    def mul_full(self, a, b, r, n: int, limbs: int, limb_bits: int = 64, stream=None) -> None:
        f = load().mi_mul_full_u64 if limb_bits == 64 else load().mi_mul_full_u32
        check(f(self.handle, _ptr(a), _ptr(b), _ptr(r), n, limbs, _ptr(stream)))

    def import_words(self, src, n: int, words: int, size: int, order: int, endian: int, dst, limbs: int,
                     stream=None) -> None:
        """GMP word fields (mpz_import conventions) -> u64 limbs, on the device."""
        check(load().mi_import_words(self.handle, _ptr(src), n, words, size, order, endian, _ptr(dst), limbs,
                                     _ptr(stream)))

    def export_words(self, src, n: int, limbs: int, dst, words: int, size: int, order: int, endian: int,
                     counts=None, stream=None) -> None:
        """u64 limbs -> fixed-width GMP word fields (mpz_export conventions), on the device."""
        check(load().mi_export_words(self.handle, _ptr(src), n, limbs, _ptr(dst), words, size, order, endian,
                                     _ptr(counts), _ptr(stream)))

    def poly(self, a, b, r, n: int, limbs: int, stream=None) -> None:
        """((a^2 + b)(b^2 + b) + ab) mod 2^(64*limbs), fused (u64 limbs)."""
        check(load().mi_poly_u64(self.handle, _ptr(a), _ptr(b), _ptr(r), n, limbs, _ptr(stream)))

    def mul_ntt(self, a, b, r, n: int, limbs: int, stream=None) -> None:
        """Exact full product by NTT (u64 limbs, limbs <= 2048)."""
        check(load().mi_mul_ntt_u64(self.handle, _ptr(a), _ptr(b), _ptr(r), n, limbs, _ptr(stream)))

    def mul(self, a, b, r, n: int, limbs: int, stream=None) -> None:
        """Full product, classical or NTT by size (u64 limbs)."""
        check(load().mi_mul_u64(self.handle, _ptr(a), _ptr(b), _ptr(r), n, limbs, _ptr(stream)))

    # --- ragged batches ------------------------------------------------------
    def ragged_run(self, ops, n_ops: int, pool_in, pool_out, scratch, scratch_bytes: int, carry=None,
                   stream=None) -> None:
        """Runs a ragged list of mi_op records (device array) on the device."""
        check(load().mi_ragged_run(self.handle, _ptr(ops), n_ops, _ptr(pool_in), _ptr(pool_out), _ptr(carry),
                                   _ptr(scratch), scratch_bytes, _ptr(stream)))

    def ragged_run_noalloc(self, ops, n_ops: int, pool_in, pool_out, carry=None, stream=None) -> None:
        """The ragged run on the library's static scratch (no device allocation)."""
        check(load().mi_ragged_run_noalloc(self.handle, _ptr(ops), n_ops, _ptr(pool_in), _ptr(pool_out), _ptr(carry),
                                           _ptr(stream)))

    def ragged_invalid_noalloc(self) -> int:
        """Ops the last no-alloc ragged run on this device skipped as invalid."""
        v = ctypes.c_uint32()
        check(load().mi_ragged_invalid_noalloc(self.handle, ctypes.byref(v)))
        return v.value

    def ragged_graph(self, ops, n_ops: int, pool_in, pool_out, scratch, scratch_bytes: int, carry=None) -> "Graph":
        h = ctypes.c_void_p()
        check(load().mi_ragged_graph_create(self.handle, _ptr(ops), n_ops, _ptr(pool_in), _ptr(pool_out),
                                            _ptr(carry), _ptr(scratch), scratch_bytes, ctypes.byref(h)))
        return Graph(h.value)

    # --- host-buffer end-to-end calls --------------------------------------
    def host_add(self, h_a: np.ndarray, h_b: np.ndarray, h_r: np.ndarray, h_carry: np.ndarray | None,
                 n: int, limbs: int) -> None:
        check(load().mi_host_add_u64(self.handle, _ptr(h_a), _ptr(h_b), _ptr(h_r), _ptr(h_carry), n, limbs))

    def host_mul_full(self, h_a: np.ndarray, h_b: np.ndarray, h_r: np.ndarray, n: int, limbs: int) -> None:
        check(load().mi_host_mul_full_u64(self.handle, _ptr(h_a), _ptr(h_b), _ptr(h_r), n, limbs))


class Graph:
    """A captured ragged run (mi_graph)."""

    def __init__(self, handle):
        self.handle = handle

    def launch(self, stream=None) -> None:
        check(load().mi_graph_launch(self.handle, _ptr(stream)))

    def close(self) -> None:
        if self.handle:
            load().mi_graph_destroy(self.handle)
            self.handle = None

    def __del__(self):  # pragma: no cover
        try:
            self.close()
        except Exception:
            pass


class Server:
    """A request loop (mi_server) on a context: continuous batching, or one
    request per launch with batching=False."""

    def __init__(self, ctx: "Context", device_bytes: int = 1 << 30, slots: int = 3, max_batch_ops: int = 0,
                 batching: bool = True):
        cfg = ServerConfig(device_bytes, slots, max_batch_ops, 1 if batching else 0, 0)
        h = ctypes.c_void_p()
        check(load().mi_server_create(ctx.handle, ctypes.byref(cfg), ctypes.byref(h)))
        self.handle = h.value
        self._keep = {}

    def submit(self, ops: np.ndarray, pool_in: np.ndarray, out: np.ndarray, carry: np.ndarray | None = None) -> int:
        """Queues a request (host arrays, kept alive until released)."""
        t = ctypes.c_uint64()
        check(load().mi_server_submit(self.handle, _ptr(ops), ops.size, _ptr(pool_in), pool_in.size, _ptr(out),
                                      out.size, _ptr(carry), ctypes.byref(t)))
        self._keep[t.value] = (ops, pool_in, out, carry)
        return t.value

    def wait(self, ticket: int, timeout_ms: int = -1) -> None:
        check(load().mi_server_wait(self.handle, ticket, timeout_ms))

    def times(self, ticket: int):
        s, a, d = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64()
        check(load().mi_server_request_times(self.handle, ticket, ctypes.byref(s), ctypes.byref(a), ctypes.byref(d)))
        return s.value, a.value, d.value

    def release(self, ticket: int) -> None:
        check(load().mi_server_release(self.handle, ticket))
        self._keep.pop(ticket, None)

    def stats(self):
        b, r, o = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64()
        check(load().mi_server_stats(self.handle, ctypes.byref(b), ctypes.byref(r), ctypes.byref(o)))
        return b.value, r.value, o.value

    def close(self) -> None:
        if self.handle:
            load().mi_server_destroy(self.handle)
            self.handle = None
            self._keep.clear()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def ragged_scratch_bytes(n_ops: int) -> int:
    v = ctypes.c_size_t()
    check(load().mi_ragged_scratch_bytes(n_ops, ctypes.byref(v)))
    return v.value


def ragged_invalid(scratch) -> int:
    v = ctypes.c_uint32()
    check(load().mi_ragged_invalid(_ptr(scratch), ctypes.byref(v)))
    return v.value


def calib_mul32_peak(iters: int = 0) -> float:
    """Measured 32x32-bit partial products per second on the current device."""
    v, t = ctypes.c_double(), ctypes.c_double()
    check(load().mi_calib_mul32_peak(iters, ctypes.byref(v), ctypes.byref(t)))
    return v.value


def calib_host_link(src, dst, nbytes: int) -> tuple[float, float, float]:
    """SM-driven host-link rates over mapped pinned host buffers (pointers or
    pinned tensors): (read, write, both directions) in GB/s."""
    r, w, b = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    check(load().mi_calib_host_link(_ptr(src), _ptr(dst), nbytes, ctypes.byref(r), ctypes.byref(w), ctypes.byref(b)))
    return r.value, w.value, b.value


def ntt_raw(p: int, g: int, two_adicity: int, a: np.ndarray, b: np.ndarray | None = None) -> np.ndarray:
    """Forward NTT of `a` (natural order) or, with `b`, the cyclic convolution
    of a and b mod p, computed on the GPU by the library's transform code."""
    a = np.ascontiguousarray(a, dtype=np.uint64)
    out = np.empty_like(a)
    bb = None if b is None else np.ascontiguousarray(b, dtype=np.uint64)
    check(load().mi_ntt_raw(p, g, two_adicity, a.size, 0 if b is None else 1, _ptr(a), _ptr(bb), _ptr(out)))
    return out


def ntt32_prime(q: int) -> tuple[int, int]:
    """(p, g): production prime q (0..4) of the NTT multiplication kernels and
    its primitive root."""
    p, g = ctypes.c_uint32(), ctypes.c_uint32()
    check(load().mi_ntt32_prime(q, ctypes.byref(p), ctypes.byref(g)))
    return p.value, g.value


def ntt32_raw(ctx: "Context", q: int, a: np.ndarray, b: np.ndarray | None = None) -> np.ndarray:
    """The multiplication kernels' transform on production prime q: forward
    NTT of `a` (natural order) or, with `b`, the cyclic convolution mod p."""
    a = np.ascontiguousarray(a, dtype=np.uint32)
    out = np.empty_like(a)
    bb = None if b is None else np.ascontiguousarray(b, dtype=np.uint32)
    check(load().mi_ntt32_raw(ctx.handle, q, a.size, 0 if b is None else 1, _ptr(a), _ptr(bb), _ptr(out)))
    return out


# --- reference-shaped drivers --------------------------------------------------

class U64bits:
    """Limb traits of cuda/ker-helpers.cu.h:12-19."""
    uint_t = np.uint64
    bits = 64
    HIGHEST = 0xFFFFFFFFFFFFFFFF


class U32bits:
    """Limb traits of cuda/ker-helpers.cu.h:21-28."""
    uint_t = np.uint32
    bits = 32
    HIGHEST = 0xFFFFFFFF


def _host_args(Base, m, num_instances, arrays):
    for x in arrays:
        if not isinstance(x, np.ndarray) or x.dtype != Base.uint_t or not x.flags.c_contiguous:
            raise MidintError(MI_EINVAL, f"expected C-contiguous {np.dtype(Base.uint_t).name} arrays")
        if x.size < num_instances * m:
            raise MidintError(MI_EINVAL, f"array of {x.size} limbs holds fewer than {num_instances}x{m}")


def gpuAdd(Base, m: int, num_instances: int, h_as: np.ndarray, h_bs: np.ndarray, h_rs: np.ndarray) -> None:
    """gpuAdd<Base, m>(num_instances, h_as, h_bs, h_rs): h_rs = (h_as + h_bs) mod 2^(bits*m)."""
    _host_args(Base, m, num_instances, (h_as, h_bs, h_rs))
    f = load().mi_compat_gpuAdd_u64 if Base.bits == 64 else load().mi_compat_gpuAdd_u32
    check(f(num_instances, m, _ptr(h_as), _ptr(h_bs), _ptr(h_rs)))


class FftPrime32:
    """The reference's 32-bit NTT prime traits (cuda/ker-fft-mul.cu.h:59-72)."""
    uhlf_t = np.uint16
    uint_t = np.uint32
    p, g, n = 3221225473, 13, 30


def gpuMulFFT(P, m: int, num_instances: int, h_as: np.ndarray, h_bs: np.ndarray, h_rs: np.ndarray) -> None:
    """gpuMulFFT<FftPrime32, m>(num_instances, h_as, h_bs, h_rs): m u16 digits
    per instance; the low m digits of each product are packed as u16 digits at
    digit offset i*m of h_rs (whose size is m u32 words per instance), as in the
    reference's kernel.  Exact, unlike the reference's."""
    if P is not FftPrime32:
        raise MidintError(MI_ENOTSUP, "only the FftPrime32 (u16 digit) shape is provided")
    for x, dt in ((h_as, np.uint16), (h_bs, np.uint16), (h_rs, np.uint32)):
        if not isinstance(x, np.ndarray) or x.dtype != dt or not x.flags.c_contiguous:
            raise MidintError(MI_EINVAL, "expected C-contiguous uint16 inputs and a uint32 output")
    if h_as.size < num_instances * m or h_bs.size < num_instances * m or h_rs.size < num_instances * m:
        raise MidintError(MI_EINVAL, "arrays too short")
    check(load().mi_compat_gpuMulFFT_u16(num_instances, m, _ptr(h_as), _ptr(h_bs), _ptr(h_rs)))


def gpuMultiply(Base, m: int, num_instances: int, h_as: np.ndarray, h_bs: np.ndarray, h_rs: np.ndarray) -> None:
    """gpuMultiply<Base, m>(num_instances, h_as, h_bs, h_rs): h_rs = (h_as * h_bs) mod 2^(bits*m)."""
    _host_args(Base, m, num_instances, (h_as, h_bs, h_rs))
    f = load().mi_compat_gpuMultiply_u64 if Base.bits == 64 else load().mi_compat_gpuMultiply_u32
    check(f(num_instances, m, _ptr(h_as), _ptr(h_bs), _ptr(h_rs)))
