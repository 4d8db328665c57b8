"""Batched multi-stream encoding over the C ABI (mptc_batch_*).

One call encodes one frame of every stream; the streams may have different
resolutions. Frames enter through ``upload`` (host arrays or device tensors)
and results leave through ``fetch``; between the two the work of all streams
runs as one CUDA graph with a concurrent branch per stream.
"""
from __future__ import annotations

import ctypes

import numpy as np

from ._lib import Config, check, dev_ptr, lib


class BatchEncoder:
    def __init__(self, sizes: list[tuple[int, int]], search_area: int = 8, err_threshold: int = 5,
                 intra_interval: int = 16):
        self.sizes = list(sizes)
        self.n = len(sizes)
        self.intra_interval = intra_interval
        w = (ctypes.c_int32 * self.n)(*[s[0] for s in sizes])
        h = (ctypes.c_int32 * self.n)(*[s[1] for s in sizes])
        cfg = Config(search_area, err_threshold, intra_interval, 0)
        handle = ctypes.c_void_p()
        check(lib().mptc_batch_create(ctypes.byref(cfg), self.n, w, h, ctypes.byref(handle)))
        self._b = handle
        self._num = [1] * self.n
        self._next_intra = [True] * self.n

    def close(self) -> None:
        if getattr(self, "_b", None):
            lib().mptc_batch_destroy(self._b)
            self._b = None

    def __del__(self):  # pragma: no cover - best effort
        try:
            self.close()
        except Exception:
            pass

    def set_model(self, model, k: int = 8) -> None:
        check(lib().mptc_batch_set_model(self._b, model.handle if model is not None else None,
                                         int(k) if model is not None else 0))

    def nblk(self, i: int) -> int:
        return (self.sizes[i][0] // 4) * (self.sizes[i][1] // 4)

    def upload(self, i: int, frame, stream=None) -> None:
        """frame: (H, W, 3) uint8 numpy array or CUDA tensor."""
        w, h = self.sizes[i]
        if tuple(frame.shape) != (h, w, 3):
            raise ValueError(f"frame: shape {tuple(frame.shape)}, expected ({h}, {w}, 3)")
        if getattr(frame, "is_cuda", False):
            ptr = dev_ptr(frame, "frame", 1, h * w * 3)
        else:
            frame = np.ascontiguousarray(frame.numpy() if hasattr(frame, "numpy") else frame, dtype=np.uint8)
            ptr = frame.ctypes.data
        s = ctypes.c_void_p(stream.cuda_stream if stream is not None else 0)
        check(lib().mptc_batch_upload(self._b, i, ptr, s))

    def schedule(self) -> list[bool]:
        """Intra flags of the next step: the reference's intra-interval rule per stream."""
        out = []
        for i in range(self.n):
            out.append(self._next_intra[i])
            if self._num[i] <= self.intra_interval:
                self._next_intra[i] = False
                if self._num[i] == self.intra_interval:
                    self._next_intra[i] = True
                    self._num[i] = 1
                else:
                    self._num[i] += 1
        return out

    def encode(self, is_intra: list[bool] | None = None, stream=None) -> list[bool]:
        flags = self.schedule() if is_intra is None else list(is_intra)
        arr = (ctypes.c_int32 * self.n)(*[int(bool(f)) for f in flags])
        s = ctypes.c_void_p(stream.cuda_stream if stream is not None else 0)
        check(lib().mptc_batch_encode(self._b, arr, s))
        return flags

    def encode_run(self, frames, finals, motions, uniques, n_uniques, is_intra, stream=None) -> None:
        """A run of F frames of every stream (mptc_batch_encode_run): frames[i]
        a CUDA uint8 tensor (F, H_i, W_i, 3); finals[i] (F, nblk_i) int64,
        motions[i] (F, 2 nblk_i) uint8, uniques[i] (F, nblk_i) int32 and
        n_uniques[i] (F,) int32 CUDA tensors receive stream i's outputs;
        is_intra[i]: F flags."""
        if len(frames) != self.n:
            raise ValueError(f"{len(frames)} frame runs for {self.n} streams")
        F = int(frames[0].shape[0])
        ptr = lambda xs: (ctypes.c_void_p * self.n)(*xs)  # noqa: E731
        fr, fi, mo, un, nu, flags = [], [], [], [], [], []
        for i in range(self.n):
            w, h = self.sizes[i]
            n = self.nblk(i)
            if tuple(frames[i].shape) != (F, h, w, 3):
                raise ValueError(f"stream {i}: frames {tuple(frames[i].shape)}, expected ({F}, {h}, {w}, 3)")
            fr.append(dev_ptr(frames[i], "frames", 1, F * h * w * 3))
            fi.append(dev_ptr(finals[i], "final", 8, F * n))
            mo.append(dev_ptr(motions[i], "motion", 1, F * 2 * n))
            un.append(dev_ptr(uniques[i], "unique", 4, F * n))
            nu.append(dev_ptr(n_uniques[i], "n_unique", 4, F))
            if len(is_intra[i]) != F:
                raise ValueError(f"stream {i}: {len(is_intra[i])} intra flags for {F} frames")
            flags.extend(int(bool(x)) for x in is_intra[i])
        arr = (ctypes.c_int32 * len(flags))(*flags)
        s = ctypes.c_void_p(stream.cuda_stream if stream is not None else 0)
        check(lib().mptc_batch_encode_run(self._b, F, ptr(fr), arr, ptr(fi), ptr(mo), ptr(un), ptr(nu), s))

    def autotune(self, is_intra: list[bool], stream=None) -> dict:
        """Times the launch shapes on the current inputs and keeps the fastest;
        returns the chosen inter warps per CTA, intra CTAs per stream (0: all)
        and the scoring's dictionary slice per stage (4 or 8: 64 or 128 words
        per MMA)."""
        arr = (ctypes.c_int32 * self.n)(*[int(bool(f)) for f in is_intra])
        w, c, r = ctypes.c_int32(0), ctypes.c_int32(0), ctypes.c_int32(0)
        s = ctypes.c_void_p(stream.cuda_stream if stream is not None else 0)
        check(lib().mptc_batch_autotune(self._b, arr, ctypes.byref(w), ctypes.byref(c), ctypes.byref(r), s))
        return {"inter_warps_per_cta": w.value, "intra_ctas_per_stream": c.value, "score_rows_per_stage": r.value}

    def fetch(self, i: int, stream=None):
        n = self.nblk(i)
        fin = np.empty(n, np.uint64)
        mot = np.empty(2 * n, np.uint8)
        uni = np.empty(n, np.uint32)
        nu = ctypes.c_uint32(0)
        s = ctypes.c_void_p(stream.cuda_stream if stream is not None else 0)
        check(lib().mptc_batch_fetch(self._b, i, fin.ctypes.data, mot.ctypes.data, uni.ctypes.data,
                                     ctypes.byref(nu), s))
        return fin, mot, uni[: nu.value]
