"""Host-side mirror of the reference encoder loop over the C ABI.

``Encoder`` owns an ``mptc_ctx`` for one stream resolution and exposes the
two calls the reference makes per frame (``DXTImage(...)`` + ``Reencode``,
codec/codec.cpp:1388-1394) on device tensors or on host arrays. Device memory
and streams come from PyTorch; the work runs in libmptc_gb300.so.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from ._lib import Config, FrameStats, KernelTime, check, dev_ptr, host_ptr, lib


def intra_schedule(n: int, interval: int) -> list[bool]:
    """Intra flags of n frames: the first frame intra, then every interval-th
    (CompressMultiUnique's set_intra / intra_num loop, codec/codec.cpp:1462-1469)."""
    out, num, nxt = [], 1, True
    for _ in range(n):
        out.append(nxt)
        if num <= interval:
            nxt = False
            if num == interval:
                nxt, num = True, 1
            else:
                num += 1
    return out


@dataclass
class FrameOutput:
    final: np.ndarray    # u64 per block (PhysicalDXTBlock)
    motion: np.ndarray   # u8, (x, y) per block
    unique: np.ndarray   # u32 unique palette in raster order
    stb: np.ndarray | None = None


@dataclass
class StreamOutput:
    """Outputs of a run of frames (encode_stream_host), one row per frame."""
    final: np.ndarray     # (frames, nblk) u64
    motion: np.ndarray    # (frames, 2 * nblk) u8
    unique: np.ndarray    # (frames, nblk) u32: frame k's palette is unique[k, :n_unique[k]]
    n_unique: np.ndarray  # (frames,) u32

    def frame(self, k: int) -> FrameOutput:
        return FrameOutput(self.final[k], self.motion[k], self.unique[k, : int(self.n_unique[k])])


class Encoder:
    """One MPTC stream of fixed resolution (width, height multiples of 4)."""

    def __init__(self, width: int, height: int, search_area: int = 8, err_threshold: int = 5,
                 intra_interval: int = 16, intra_sweeps: int = 0):
        self.width, self.height = width, height
        self.bw, self.bh = width // 4, height // 4
        self.nblk = self.bw * self.bh
        self.intra_interval = intra_interval
        cfg = Config(search_area, err_threshold, intra_interval, intra_sweeps)
        h = ctypes.c_void_p()
        check(lib().mptc_ctx_create(ctypes.byref(cfg), width, height, ctypes.byref(h)))
        self._ctx = h
        self._intra_num = 1
        self._next_intra = True

    def close(self) -> None:
        if getattr(self, "_ctx", None):
            lib().mptc_ctx_destroy(self._ctx)
            self._ctx = None

    def __del__(self):  # pragma: no cover - best effort
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self) -> ctypes.c_void_p:
        return self._ctx

    # -- device API ---------------------------------------------------------
    def _frame_ptrs(self, final, motion, unique, n_unique, frames: int = 1):
        n = self.nblk
        return (dev_ptr(final, "final", 8, frames * n), dev_ptr(motion, "motion", 1, frames * 2 * n),
                dev_ptr(unique, "unique", 4, frames * n), dev_ptr(n_unique, "n_unique", 4, frames))

    def encode_frame_device(self, rgb, prev_final, stb, final, motion, unique, n_unique, stream=None):
        """All arguments are torch CUDA tensors (prev_final and stb may be None):
        rgb (height, width, 3) uint8, prev_final/stb/final nblk int64, motion
        2*nblk uint8, unique nblk int32, n_unique one int32."""
        n = self.nblk
        outs = self._frame_ptrs(final, motion, unique, n_unique)
        s = ctypes.c_void_p(stream.cuda_stream if stream is not None else 0)
        check(lib().mptc_encode_frame(self._ctx, dev_ptr(rgb, "rgb", 1, 48 * n),
                                      dev_ptr(prev_final, "prev_final", 8, n) if prev_final is not None else None,
                                      dev_ptr(stb, "stb", 8, n) if stb is not None else None, *outs, s),
              self._ctx)

    def encode_stream_device(self, frames, final, motion, unique, n_unique, is_intra=None, stream=None) -> None:
        """A run of frames on the device (mptc_encode_stream_device): frames is a
        CUDA uint8 tensor (n, height, width, 3); final (n, nblk) int64, motion
        (n, 2*nblk) uint8, unique (n, nblk) int32 and n_unique (n,) int32 CUDA
        tensors receive each frame's outputs. Intra frames run on a second
        lane, concurrently with the inter frames before them. is_intra: a flag
        per frame, or None for the reference's schedule."""
        n = frames.shape[0]
        if tuple(frames.shape[1:]) != (self.height, self.width, 3):
            raise ValueError(f"frames: shape {tuple(frames.shape)}, expected (n, {self.height}, {self.width}, 3)")
        src = dev_ptr(frames, "frames", 1, n * 48 * self.nblk)
        outs = self._frame_ptrs(final, motion, unique, n_unique, n)
        flags = np.array([self._intra_flag(None if is_intra is None else is_intra[k]) for k in range(n)],
                         dtype=np.int32)
        s = ctypes.c_void_p(stream.cuda_stream if stream is not None else 0)
        check(lib().mptc_encode_stream_device(self._ctx, src, n, flags.ctypes.data, *outs, s), self._ctx)

    def dxt1_encode_device(self, rgb, stb, orig_err, stream=None):
        n = self.nblk
        s = ctypes.c_void_p(stream.cuda_stream if stream is not None else 0)
        check(lib().mptc_dxt1_encode(self._ctx, dev_ptr(rgb, "rgb", 1, 48 * n), dev_ptr(stb, "stb", 8, n),
                                     dev_ptr(orig_err, "orig_err", 4, n) if orig_err is not None else None, s),
              self._ctx)

    def reencode_device(self, rgb, stb, orig_err, prev_final, final, motion, unique, n_unique,
                        stream=None):
        n = self.nblk
        outs = self._frame_ptrs(final, motion, unique, n_unique)
        s = ctypes.c_void_p(stream.cuda_stream if stream is not None else 0)
        check(lib().mptc_reencode(self._ctx, dev_ptr(rgb, "rgb", 1, 48 * n), dev_ptr(stb, "stb", 8, n),
                                  dev_ptr(orig_err, "orig_err", 4, n),
                                  dev_ptr(prev_final, "prev_final", 8, n) if prev_final is not None else None,
                                  *outs, s), self._ctx)

    def stats(self, stream=None) -> FrameStats:
        st = FrameStats()
        s = ctypes.c_void_p(stream.cuda_stream if stream is not None else 0)
        check(lib().mptc_last_frame_stats(self._ctx, ctypes.byref(st), s), self._ctx)
        return st

    def set_model(self, model, k: int = 8) -> None:
        """Attach a ProposalModel to the inter search (k proposals), or detach (None)."""
        check(lib().mptc_ctx_set_model(self._ctx, model.handle if model is not None else None,
                                       int(k) if model is not None else 0), self._ctx)

    def kernel_launches(self) -> int:
        """Kernels launched on this context since the last call."""
        n = ctypes.c_uint64()
        check(lib().mptc_kernel_launches(self._ctx, ctypes.byref(n)), self._ctx)
        return int(n.value)

    def set_kernel_timing(self, enable: bool) -> None:
        check(lib().mptc_set_kernel_timing(self._ctx, int(enable)), self._ctx)

    def kernel_times(self) -> dict:
        """{kernel name: (launches, total ms)} since the last call."""
        arr = (KernelTime * 16)()
        n = ctypes.c_int32(0)
        check(lib().mptc_kernel_times(self._ctx, arr, 16, ctypes.byref(n)), self._ctx)
        return {arr[i].name.decode(): (arr[i].launches, arr[i].total_ms) for i in range(n.value)}

    # -- host API -----------------------------------------------------------
    def _intra_flag(self, is_intra: bool | None) -> bool:
        """The caller's flag, or the next one of the reference's schedule."""
        if is_intra is not None:
            return bool(is_intra)
        flag = self._next_intra
        if self._intra_num <= self.intra_interval:
            self._next_intra = False
            if self._intra_num == self.intra_interval:
                self._next_intra = True
                self._intra_num = 1
            else:
                self._intra_num += 1
        return flag

    def encode_stream_host(self, frames: np.ndarray, is_intra=None,
                           out: StreamOutput | None = None) -> StreamOutput:
        """A run of frames (frames, height, width, 3) from host memory in one
        call (mptc_encode_stream_host); the stream continues across calls.
        is_intra: a flag per frame, or None for the reference's schedule.
        With pinned frames and outputs the uploads and downloads overlap the
        encode; otherwise the frames go one by one."""
        f = np.ascontiguousarray(frames, dtype=np.uint8)
        if f.ndim != 4 or f.shape[1:] != (self.height, self.width, 3):
            raise ValueError(f"frames: shape {f.shape}, expected (n, {self.height}, {self.width}, 3)")
        n, nb = f.shape[0], self.nblk
        if out is None:
            out = StreamOutput(np.empty((n, nb), np.uint64), np.empty((n, 2 * nb), np.uint8),
                               np.empty((n, nb), np.uint32), np.empty(n, np.uint32))
        ptrs = (host_ptr(out.final, "final", np.uint64, n * nb), host_ptr(out.motion, "motion", np.uint8, n * 2 * nb),
                host_ptr(out.unique, "unique", np.uint32, n * nb), host_ptr(out.n_unique, "n_unique", np.uint32, n))
        flags = np.array([self._intra_flag(None if is_intra is None else is_intra[k]) for k in range(n)],
                         dtype=np.int32)
        check(lib().mptc_encode_stream_host(self._ctx, f.ctypes.data, n, flags.ctypes.data, *ptrs, None),
              self._ctx)
        return out

    def encode_frame_host(self, frame: np.ndarray, is_intra: bool | None = None,
                          want_stb: bool = False, out: FrameOutput | None = None) -> FrameOutput:
        """One frame from host memory; successive calls form a stream. With
        is_intra=None the reference's intra-interval schedule is applied
        (frame 1 intra, then every intra_interval-th, codec/codec.cpp:1462-1469)."""
        f = np.ascontiguousarray(frame, dtype=np.uint8)
        if f.shape != (self.height, self.width, 3):
            raise ValueError(f"frame: shape {f.shape}, expected ({self.height}, {self.width}, 3)")
        nb = self.nblk
        if out is None:
            out = FrameOutput(np.empty(nb, np.uint64), np.empty(2 * nb, np.uint8), np.empty(nb, np.uint32),
                              np.empty(nb, np.uint64) if want_stb else None)
        ptrs = (host_ptr(out.final, "final", np.uint64, nb), host_ptr(out.motion, "motion", np.uint8, 2 * nb),
                host_ptr(out.unique, "unique", np.uint32, nb))
        stb = host_ptr(out.stb, "stb", np.uint64, nb) if out.stb is not None else None
        is_intra = self._intra_flag(is_intra)
        nu = ctypes.c_uint32(0)
        check(lib().mptc_encode_frame_host(self._ctx, f.ctypes.data, int(bool(is_intra)), stb, *ptrs,
                                           ctypes.byref(nu), None),
              self._ctx)
        return FrameOutput(out.final, out.motion, out.unique[: nu.value], out.stb)
