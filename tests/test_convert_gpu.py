"""GMP word-format conversions on the device (mi_import_words /
mi_export_words) against the oracle's restatement, which test_oracle.py pins
on GMP's own mpz_import / mpz_export."""
from __future__ import annotations

import numpy as np
import pytest
import torch

import midint
import oracle as O

pytestmark = pytest.mark.gpu

FORMATS = [(order, size, endian) for order in (-1, 1) for size in (1, 2, 4, 8) for endian in (-1, 0, 1)]


def _dev_bytes(x: np.ndarray, extra: int = 64):
    b = np.ascontiguousarray(x).view(np.uint8)
    t = torch.zeros(b.size + extra, dtype=torch.uint8, device="cuda:0")
    t[: b.size] = torch.from_numpy(b.copy()).to("cuda:0")
    return t


@pytest.mark.parametrize("order,size,endian", FORMATS)
def test_import_export_match_oracle(ctx, order, size, endian):
    rng = np.random.default_rng(size * 13 + order * 3 + endian)
    s = torch.cuda.current_stream().cuda_stream
    for limbs, words in ((4, 32 // size), (4, 32 // size + 5), (7, 2), (1, 8 // size), (33, 264 // size + 1)):
        n = 37
        x = rng.integers(0, 2**64, size=n * limbs, dtype=np.uint64)
        x[:limbs] = 0
        x[limbs:2 * limbs] = np.uint64(2**64 - 1)
        x[2 * limbs + 1:3 * limbs] = 0
        want_field, want_counts = O.export_words(x, n, limbs, words, size, order, endian)
        dx = _dev_bytes(x)
        field = torch.full((want_field.size + 64,), 0xA5, dtype=torch.uint8, device="cuda:0")
        counts = torch.full((n + 4,), 0xFFFFFFFF, dtype=torch.int64, device="cuda:0").view(torch.int32)
        ctx.export_words(dx, n, limbs, field, words, size, order, endian, counts=counts, stream=s)
        torch.cuda.synchronize()
        got = field.cpu().numpy()
        assert np.array_equal(got[: want_field.size], want_field)
        assert (got[want_field.size:] == 0xA5).all(), "export wrote past the batch"
        assert np.array_equal(counts.cpu().numpy().view(np.uint32)[:n], want_counts)
        # and back: fields -> limbs
        dst = torch.full((n * limbs + 8,), -1, dtype=torch.int64, device="cuda:0")
        ctx.import_words(field, n, words, size, order, endian, dst, limbs, stream=s)
        torch.cuda.synchronize()
        back = dst.cpu().numpy().view(np.uint64)
        assert np.array_equal(back[: n * limbs], O.import_words(want_field, n, words, size, order, endian, limbs))
        assert (back[n * limbs:] == np.uint64(2**64 - 1)).all(), "import wrote past the batch"
        if words * size >= limbs * 8:
            assert np.array_equal(back[: n * limbs], x)


def test_reference_format_is_the_limb_bytes(ctx):
    # the reference's mpz order -1, 4-byte native words: identical bytes
    rng = np.random.default_rng(2)
    x = rng.integers(0, 2**64, size=9 * 16, dtype=np.uint64)
    dx = _dev_bytes(x)
    field = torch.zeros(x.nbytes, dtype=torch.uint8, device="cuda:0")
    ctx.export_words(dx, 9, 16, field, 32, 4, -1, 0, stream=torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert np.array_equal(field.cpu().numpy(), x.view(np.uint8))


def test_big_endian_byte_strings(ctx):
    # order 1, 1-byte words: the big-endian byte string of each value
    vals = [0, 1, 255, 256, 2**200 + 12345, 2**256 - 1]
    limbs, nbytes = 4, 32
    x = O.from_ints(vals, limbs)
    dx = _dev_bytes(x)
    field = torch.zeros(len(vals) * nbytes, dtype=torch.uint8, device="cuda:0")
    ctx.export_words(dx, len(vals), limbs, field, nbytes, 1, 1, 1, stream=torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    got = field.cpu().numpy().reshape(len(vals), nbytes)
    for i, v in enumerate(vals):
        assert bytes(got[i]) == v.to_bytes(nbytes, "big")


def test_conversion_argument_errors(ctx):
    buf = torch.zeros(256, dtype=torch.uint8, device="cuda:0")
    p = buf.data_ptr()
    with pytest.raises(midint.MidintError):
        ctx.import_words(p, 1, 4, 3, -1, 0, p + 128, 2)          # size 3
    with pytest.raises(midint.MidintError):
        ctx.import_words(p, 1, 4, 4, 0, 0, p + 128, 2)           # order 0
    with pytest.raises(midint.MidintError):
        ctx.export_words(p, 1, 2, p + 4, 4, 4, -1, 2)            # endian 2
    with pytest.raises(midint.MidintError):
        ctx.export_words(p, 1, 2, p + 8, 4, 4, -1, 0)            # overlap
    with pytest.raises(midint.MidintError):
        ctx.import_words(p + 2, 1, 4, 4, -1, 0, p + 128, 2)      # misaligned src
    ctx.import_words(p, 0, 4, 4, -1, 0, p + 128, 2)              # empty batch
