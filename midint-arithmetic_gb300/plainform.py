"""The plain per-size-launch form of a ragged batch.

The baseline the ragged kernels are measured against: the library's own
per-operation kernels, one launch per (operation, power-of-two size class),
with both operands of every op zero-padded to the class size P =
pow2ceil(max(la, lb)).  Additions run mi_add_u64 on P limbs (carry-out
kept), multiplications mi_mul_u64 on P limbs (classical or NTT by the
context's crossover).  Padding happens once on the host in prepare(); run()
launches only device work.
"""
from __future__ import annotations

import numpy as np


class PlainBatch:
    def __init__(self, ops: np.ndarray, pool: np.ndarray, device="cuda:0"):
        import torch

        self.torch = torch
        self.groups = []
        la = ops["la"].astype(np.int64)
        lb = ops["lb"].astype(np.int64)
        m = np.maximum(la, lb)
        P = (1 << np.ceil(np.log2(m)).astype(np.int64))
        for kind in (0, 1):
            for p in np.unique(P[ops["kind"] == kind]):
                idx = np.nonzero((ops["kind"] == kind) & (P == p))[0]
                A = self._pad(pool, ops["a_off"][idx], la[idx], int(p))
                B = self._pad(pool, ops["b_off"][idx], lb[idx], int(p))
                n = idx.size
                g = {"kind": kind, "P": int(p), "idx": idx,
                     "a": torch.from_numpy(A.view(np.int64)).to(device),
                     "b": torch.from_numpy(B.view(np.int64)).to(device),
                     "r": torch.empty(n * int(p) * (1 if kind == 0 else 2), dtype=torch.int64, device=device),
                     "c": torch.empty(n, dtype=torch.uint8, device=device) if kind == 0 else None}
                self.groups.append(g)

    @staticmethod
    def _pad(pool, offs, lens, p):
        n = offs.size
        cols = np.arange(p, dtype=np.int64)[None, :]
        src = offs.astype(np.int64)[:, None] + cols
        mask = cols < lens[:, None]
        out = np.zeros((n, p), np.uint64)
        out[mask] = pool[src[mask]]
        return out.ravel()

    def run(self, ctx, stream) -> int:
        """Launches every class; returns the number of launches."""
        for g in self.groups:
            n = g["idx"].size
            if g["kind"] == 0:
                ctx.add(g["a"], g["b"], g["r"], n, g["P"], carry=g["c"], stream=stream)
            else:
                ctx.mul(g["a"], g["b"], g["r"], n, g["P"], stream=stream)
        return len(self.groups)

    def results(self, ops: np.ndarray, out_limbs: int):
        """The ragged output pool (and add carry-outs) rebuilt from the padded results."""
        out = np.zeros(out_limbs, np.uint64)
        carry = np.zeros(ops.size, np.uint8)
        la = ops["la"].astype(np.int64)
        lb = ops["lb"].astype(np.int64)
        for g in self.groups:
            idx, p = g["idx"], g["P"]
            width = p if g["kind"] == 0 else 2 * p
            R = g["r"].cpu().numpy().view(np.uint64).reshape(-1, width)
            rl = np.maximum(la[idx], lb[idx]) if g["kind"] == 0 else la[idx] + lb[idx]
            cols = np.arange(width, dtype=np.int64)[None, :]
            mask = cols < rl[:, None]
            dst = ops["r_off"][idx].astype(np.int64)[:, None] + cols
            out[dst[mask]] = R[mask]
            if g["kind"] == 0:
                c = g["c"].cpu().numpy()
                m = np.maximum(la[idx], lb[idx])
                # the carry of an m-limb sum is limb m of the padded sum, or the
                # padded carry-out when m == P
                inner = m < p
                carry[idx[~inner]] = c[~inner]
                carry[idx[inner]] = R[np.nonzero(inner)[0], m[inner]].astype(np.uint8)
        return out, carry
