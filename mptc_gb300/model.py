"""Learned candidate proposal: model wrapper, training-example sampler and
training loop over the C ABI (mptc_model_*). Training runs on the GPU in the
library's own tensor-core kernels; this module only prepares index arrays.

Layers (flat fp32 parameter vector, weight [in x out] then bias per layer):
f1 64(54 used) -> 128, f2 128 -> 128, f3 128 -> 64 (block MLP, ReLU between),
g1 32 -> 128, g2 128 -> 64 (candidate MLP over the index word's bits).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from ._lib import check, dev_ptr, lib

LAYERS = [(64, 128), (128, 128), (128, 64), (32, 128), (128, 64)]


def param_slices():
    out, o = [], 0
    for i, n in LAYERS:
        out.append(((o, o + i * n, (i, n)), (o + i * n, o + i * n + n, (n,))))
        o += i * n + n
    return out, o


def _example_ptrs(rgb, stb, blocks, cands):
    """Checked device pointers of a training batch: the frame's pixels and
    stb blocks, B block indices and B x C candidate words (4-byte integers)."""
    if cands.dim() != 2 or blocks.numel() != cands.shape[0]:
        raise ValueError(f"blocks {tuple(blocks.shape)} and cands {tuple(cands.shape)} do not match (B, B x C)")
    B, C = cands.shape
    return (dev_ptr(rgb, "rgb", 1, 48), dev_ptr(stb, "stb", 8, 1), dev_ptr(blocks, "blocks", 4, B),
            dev_ptr(cands, "cands", 4, B * C))


class ProposalModel:
    def __init__(self, seed: int = 0):
        h = ctypes.c_void_p()
        check(lib().mptc_model_create(ctypes.c_uint64(seed), ctypes.byref(h)))
        self._m = h
        self.n_params = int(lib().mptc_model_num_params())
        if self.n_params != param_slices()[1]:
            raise RuntimeError(f"library has {self.n_params} parameters, LAYERS describe {param_slices()[1]}")

    @property
    def handle(self):
        return self._m

    def close(self):
        if getattr(self, "_m", None):
            lib().mptc_model_destroy(self._m)
            self._m = None

    def __del__(self):  # pragma: no cover
        try:
            self.close()
        except Exception:
            pass

    def params(self) -> np.ndarray:
        p = np.empty(self.n_params, np.float32)
        check(lib().mptc_model_get_params(self._m, p.ctypes.data))
        return p

    def set_params(self, p: np.ndarray) -> None:
        p = np.ascontiguousarray(p, dtype=np.float32)
        if p.size != self.n_params:
            raise ValueError(f"params: {p.size} values given, {self.n_params} expected")
        check(lib().mptc_model_set_params(self._m, p.ctypes.data))

    def grads(self, rgb, width, stb, blocks, cands):
        """Loss and flat gradient on device tensors (blocks: B int32, cands: B x C int32)."""
        g = np.empty(self.n_params, np.float32)
        loss = ctypes.c_float(0)
        B, C = cands.shape
        rgb_p, stb_p, blk_p, cand_p = _example_ptrs(rgb, stb, blocks, cands)
        check(lib().mptc_model_grads(self._m, rgb_p, width, stb_p, blk_p, cand_p, B, C, g.ctypes.data,
                                     ctypes.byref(loss), None))
        return float(loss.value), g

    def train_step(self, rgb, width, stb, blocks, cands, lr=1e-3, weight_decay=1e-4, stream=None) -> float:
        loss = ctypes.c_float(0)
        B, C = cands.shape
        s = ctypes.c_void_p(stream.cuda_stream if stream is not None else 0)
        rgb_p, stb_p, blk_p, cand_p = _example_ptrs(rgb, stb, blocks, cands)
        check(lib().mptc_model_train_step(self._m, rgb_p, width, stb_p, blk_p, cand_p, B, C, lr, weight_decay,
                                          ctypes.byref(loss), s))
        return float(loss.value)

    def embed(self, rgb, width, stb, blocks, n_blocks, out_blocks, words=None, word_stride=1, n_words=0,
              out_words=None):
        check(lib().mptc_model_embed(self._m, rgb.data_ptr() if rgb is not None else None, width,
                                     stb.data_ptr() if stb is not None else None,
                                     blocks.data_ptr() if blocks is not None else None, n_blocks,
                                     out_blocks.data_ptr() if out_blocks is not None else None,
                                     words.data_ptr() if words is not None else None, word_stride, n_words,
                                     out_words.data_ptr() if out_words is not None else None, None))

    def save(self, path: str) -> None:
        check(lib().mptc_model_save(self._m, path.encode()))

    def load(self, path: str) -> None:
        check(lib().mptc_model_load(self._m, path.encode()))


@dataclass
class Examples:
    blocks: np.ndarray   # B int32 block indices
    cands: np.ndarray    # B x C uint32 index words, the accepted one first


def sample_examples(rng: np.random.Generator, bw: int, bh: int, sa: int, motion: np.ndarray,
                    prev_final: np.ndarray, B: int, C: int) -> Examples | None:
    """(block, accepted inter candidate) pairs of one frame plus C-1 other
    in-window candidates of the same block as negatives."""
    m = motion.reshape(-1, 2).astype(np.int64)
    inter = np.nonzero((m[:, 0] >= 128) & ~((m[:, 0] == 255) & (m[:, 1] == 255)))[0]
    if inter.size == 0:
        return None
    pick = inter[rng.integers(0, inter.size, B)]
    bx, by = pick % bw, pick // bw
    words = (prev_final >> np.uint64(32)).astype(np.uint32)
    pos_i = bx + m[pick, 0] - 128 - sa
    pos_j = by + m[pick, 1] - 128 - sa
    cands = np.empty((B, C), np.uint32)
    cands[:, 0] = words[pos_j * bw + pos_i]
    # negatives: random in-bounds window positions (re-drawn when out of bounds)
    di = rng.integers(-sa, sa, (B, C - 1))
    dj = rng.integers(-sa, sa, (B, C - 1))
    ni = np.clip(bx[:, None] + di, 0, bw - 1)
    nj = np.clip(by[:, None] + dj, 0, bh - 1)
    cands[:, 1:] = words[nj * bw + ni]
    return Examples(pick.astype(np.int32), cands)
