"""Learned cost model for the extension scheduler (host side).

A 2 x 64 MLP (BF16 weights, FP32 accumulation) predicts log(1 + cells) of a
ksw_extend2 job; trained on the GPU by the library's own forward, backward
and Adam kernels (csrc/cost_mlp.cu) on per-job cell counts the extension
kernel itself logs.  Its prediction becomes the cost key the persistent
extension kernels issue jobs by; it never changes a result.  The plain
bound qlen x min(tlen, qlen + w) is both the fallback and the yardstick.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib

F = 8
H = 64
N_PARAMS = H * F + H * H + H + H + H + 1
WEIGHTS_BYTES = 2 * (H * F + H * H + H) + 4 * (H + H + 1)


def bf16_bits(x: np.ndarray) -> np.ndarray:
    """float32 -> BF16 bit patterns, round to nearest even (as __float2bfloat16)."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = ((u >> 16) & 1) + 0x7FFF
    return ((u + r) >> 16).astype(np.uint16)


def bf16_value(bits: np.ndarray) -> np.ndarray:
    return (bits.astype(np.uint32) << 16).view(np.float32)


def pack_weights(master: np.ndarray) -> np.ndarray:
    """Flat FP32 parameters (w1|w2|w3|b1|b2|b3) -> the bytes of bsb_mlp_weights_t."""
    m = np.asarray(master, np.float32)
    w = bf16_bits(m[: H * F + H * H + H])
    b = m[H * F + H * H + H:]
    return np.concatenate([w.view(np.uint8), b.astype(np.float32).view(np.uint8)])


def init_params(seed: int = 1234) -> np.ndarray:
    rng = np.random.Generator(np.random.PCG64(seed))
    w1 = rng.uniform(-1, 1, H * F) * np.sqrt(6.0 / F) * 0.5
    w2 = rng.uniform(-1, 1, H * H) * np.sqrt(6.0 / H) * 0.5
    w3 = rng.uniform(-1, 1, H) * np.sqrt(6.0 / H) * 0.5
    b = np.zeros(2 * H + 1)
    b[-1] = 7.0                     # log1p(cells) is ~ 6-10 for these jobs
    return np.concatenate([w1, w2, w3, b]).astype(np.float32)


class CostModel:
    """Device-resident model state: BF16 weights, FP32 master copy, Adam moments."""

    def __init__(self, ctx, seed: int = 1234):
        import torch
        self.ctx, self.L, self.torch = ctx, ctx.L, torch
        p = init_params(seed)
        self.master = torch.from_numpy(p).cuda()
        self.m = torch.zeros(N_PARAMS, dtype=torch.float32, device="cuda")
        self.v = torch.zeros(N_PARAMS, dtype=torch.float32, device="cuda")
        self.grad = torch.zeros(N_PARAMS + 1, dtype=torch.float32, device="cuda")
        self.w = torch.from_numpy(pack_weights(p)).cuda()
        self.step = 0
        torch.cuda.synchronize()

    def params(self) -> np.ndarray:
        self.torch.cuda.synchronize()
        return self.master.cpu().numpy()

    def weights_bits(self):
        self.torch.cuda.synchronize()
        raw = self.w.cpu().numpy()
        nw = H * F + H * H + H
        return raw[: 2 * nw].view(np.uint16), raw[2 * nw:].view(np.float32)

    def _p(self, t):
        return ctypes.c_void_p(t.data_ptr())

    def features(self, d_jobs, n, d_seq, seq_bytes):
        torch = self.torch
        feat = torch.empty((n, F), dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        _lib.check(self.ctx.handle, self.L.bsb_cost_features(self.ctx.handle, self._p(d_jobs), n, self._p(d_seq),
                                                              seq_bytes, self._p(feat)))
        _lib.check(self.ctx.handle, self.L.bsb_sync(self.ctx.handle))
        return feat

    def forward(self, feat, want_key=False):
        torch = self.torch
        n = feat.shape[0]
        pred = torch.empty(n, dtype=torch.float32, device="cuda")
        key = torch.empty(n, dtype=torch.int32, device="cuda") if want_key else None
        torch.cuda.synchronize()
        _lib.check(self.ctx.handle, self.L.bsb_mlp_forward(self.ctx.handle, self._p(self.w), self._p(feat), n,
                                                            self._p(pred), self._p(key) if key is not None else None))
        _lib.check(self.ctx.handle, self.L.bsb_sync(self.ctx.handle))
        return (pred, key) if want_key else pred

    def backward(self, feat, target):
        torch = self.torch
        torch.cuda.synchronize()
        _lib.check(self.ctx.handle, self.L.bsb_mlp_backward(self.ctx.handle, self._p(self.w), self._p(feat),
                                                             self._p(target), feat.shape[0], self._p(self.grad)))
        _lib.check(self.ctx.handle, self.L.bsb_sync(self.ctx.handle))
        return self.grad

    def adam(self, lr):
        self.step += 1
        _lib.check(self.ctx.handle, self.L.bsb_mlp_adam(self.ctx.handle, self._p(self.w), self._p(self.master),
                                                         self._p(self.m), self._p(self.v), self._p(self.grad),
                                                         ctypes.c_float(lr), self.step))

    def train(self, feat, target, epochs: int = 4, batch: int = 8192, lr: float = 3e-3, seed: int = 7):
        """Minibatch Adam on (feat, target = log1p(cells)); returns the loss per epoch."""
        torch = self.torch
        n = feat.shape[0]
        g = torch.Generator(device="cpu").manual_seed(seed)
        losses = []
        for _ in range(epochs):
            perm = torch.randperm(n, generator=g).cuda()
            tot = 0.0
            nb = 0
            for s in range(0, n - batch + 1, batch):
                idx = perm[s:s + batch]
                fb = feat[idx].contiguous()
                tb = target[idx].contiguous()
                self.backward(fb, tb)
                tot += float(self.grad[N_PARAMS].item())   # loss of this batch, before the update
                self.adam(lr)
                nb += 1
            torch.cuda.synchronize()
            losses.append(tot / max(1, nb))
        return losses


def spearman(a: np.ndarray, b: np.ndarray) -> float:
    ra = np.argsort(np.argsort(a, kind="stable"), kind="stable").astype(np.float64)
    rb = np.argsort(np.argsort(b, kind="stable"), kind="stable").astype(np.float64)
    ra -= ra.mean()
    rb -= rb.mean()
    return float((ra * rb).sum() / np.sqrt((ra * ra).sum() * (rb * rb).sum()))


def mape(pred_cells: np.ndarray, cells: np.ndarray) -> float:
    c = np.maximum(cells.astype(np.float64), 1.0)
    return float(np.mean(np.abs(pred_cells - c) / c))


def calibrated_bound(bound: np.ndarray, cells: np.ndarray) -> np.ndarray:
    """The plain bound rescaled by its mean ratio to the logged cells, so its MAPE is comparable."""
    k = cells.sum() / max(1.0, float(bound.sum()))
    return bound * k
