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
MAX_LIMBS_U64 = 1024

# Every symbol include/midint.h declares, with (restype, argtypes).
_P, _U32, _I = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_int
_S = ctypes.c_int  # mi_status
SIGNATURES = {
    "mi_version": (_I, []),
    "mi_status_string": (ctypes.c_char_p, [_I]),
    "mi_last_error": (ctypes.c_char_p, []),
    "mi_ctx_create": (_S, [_I, ctypes.POINTER(_P)]),
    "mi_ctx_destroy": (_S, [_P]),
    "mi_ctx_synchronize": (_S, [_P]),
    "mi_ctx_stream": (_P, [_P]),
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
    "mi_mul_ntt_u64": (_S, [_P, _P, _P, _P, _U32, _U32, _P]),
    "mi_mul_u64": (_S, [_P, _P, _P, _P, _U32, _U32, _P]),
    "mi_compat_gpuMulFFT_u16": (_S, [_I, _U32, _P, _P, _P]),
    "mi_ntt_raw": (_S, [ctypes.c_uint64, ctypes.c_uint64, _U32, _U32, _I, _P, _P, _P]),
}


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

    def mul_ntt(self, a, b, r, n: int, limbs: int, stream=None) -> None:
        """Exact full product by NTT (u64 limbs, limbs <= 1024)."""
        check(load().mi_mul_ntt_u64(self.handle, _ptr(a), _ptr(b), _ptr(r), n, limbs, _ptr(stream)))

    def mul(self, a, b, r, n: int, limbs: int, stream=None) -> None:
        """Full product, classical or NTT by size (u64 limbs)."""
        check(load().mi_mul_u64(self.handle, _ptr(a), _ptr(b), _ptr(r), n, limbs, _ptr(stream)))

    # --- host-buffer end-to-end calls --------------------------------------
    def host_add(self, h_a: np.ndarray, h_b: np.ndarray, h_r: np.ndarray, h_carry: np.ndarray | None,
                 n: int, limbs: int) -> None:
        check(load().mi_host_add_u64(self.handle, _ptr(h_a), _ptr(h_b), _ptr(h_r), _ptr(h_carry), n, limbs))

    def host_mul_full(self, h_a: np.ndarray, h_b: np.ndarray, h_r: np.ndarray, n: int, limbs: int) -> None:
        check(load().mi_host_mul_full_u64(self.handle, _ptr(h_a), _ptr(h_b), _ptr(h_r), n, limbs))


def calib_mul32_peak(iters: int = 0) -> float:
    """Measured 32x32-bit partial products per second on the current device."""
    v, t = ctypes.c_double(), ctypes.c_double()
    check(load().mi_calib_mul32_peak(iters, ctypes.byref(v), ctypes.byref(t)))
    return v.value


def ntt_raw(p: int, g: int, two_adicity: int, a: np.ndarray, b: np.ndarray | None = None) -> np.ndarray:
    """Forward NTT of `a` (natural order) or, with `b`, the cyclic convolution
    of a and b mod p, computed on the GPU by the library's transform code."""
    a = np.ascontiguousarray(a, dtype=np.uint64)
    out = np.empty_like(a)
    bb = None if b is None else np.ascontiguousarray(b, dtype=np.uint64)
    check(load().mi_ntt_raw(p, g, two_adicity, a.size, 0 if b is None else 1, _ptr(a), _ptr(bb), _ptr(out)))
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
