"""MPTC stream writer: ctypes binding of ``libmptc_host.so`` (include/mptc_host.h).

Turns the per-frame arrays the encoder returns (final blocks, motion codes,
unique palette) into the bytes of an MPTC stream, identical to the stream the
reference encoder's ``CompressMultiUnique`` (codec/codec.cpp:1307-1532) writes
for the same frames. Host-only: no GPU is needed.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from ._lib import MptcError

_HERE = os.path.dirname(os.path.abspath(__file__))
HOST_LIB_PATH = os.path.join(_HERE, "libmptc_host.so")

HOST_EXPORTED = [
    "mptc_stream_writer_create", "mptc_stream_writer_destroy", "mptc_stream_writer_add_frame",
    "mptc_stream_writer_finish", "mptc_stream_writer_frame_sizes",
]

_HOST = None


def host_lib() -> ctypes.CDLL:
    global _HOST
    if _HOST is None:
        if not os.path.exists(HOST_LIB_PATH):
            raise RuntimeError(f"{HOST_LIB_PATH} is missing: run __graft_entry__.build()")
        L = ctypes.CDLL(HOST_LIB_PATH)
        vp, i32 = ctypes.c_void_p, ctypes.c_int32
        L.mptc_stream_writer_create.argtypes = [i32, i32, i32, i32, i32, ctypes.POINTER(vp)]
        L.mptc_stream_writer_destroy.argtypes = [vp]
        L.mptc_stream_writer_add_frame.argtypes = [vp, vp, vp, vp, ctypes.c_uint32]
        L.mptc_stream_writer_finish.argtypes = [vp, vp, ctypes.POINTER(ctypes.c_uint64)]
        L.mptc_stream_writer_frame_sizes.argtypes = [vp, ctypes.POINTER(ctypes.c_uint32), vp]
        _HOST = L
    return _HOST


def _check(rc: int, what: str) -> None:
    if rc != 0:
        raise MptcError(rc, what)


class StreamWriter:
    """One MPTC stream. Frame sizes must be multiples of 256 pixels (the
    endpoint wavelet works on 64x64-block tiles)."""

    def __init__(self, width: int, height: int, search_area: int, unique_interval: int,
                 total_frames: int):
        self._h = ctypes.c_void_p()
        self.blocks = (width // 4) * (height // 4)
        _check(host_lib().mptc_stream_writer_create(width, height, search_area, unique_interval,
                                                     total_frames, ctypes.byref(self._h)),
               f"stream writer for {width}x{height}, search area {search_area}, "
               f"unique interval {unique_interval}, {total_frames} frames")

    def add_frame(self, final: np.ndarray, motion: np.ndarray, unique: np.ndarray) -> None:
        final = np.ascontiguousarray(final, dtype=np.uint64).reshape(-1)
        motion = np.ascontiguousarray(motion, dtype=np.uint8).reshape(-1)
        unique = np.ascontiguousarray(unique, dtype=np.uint32).reshape(-1)
        if final.size != self.blocks or motion.size != 2 * self.blocks:
            raise ValueError(f"frame arrays do not match {self.blocks} blocks")
        _check(host_lib().mptc_stream_writer_add_frame(self._h, final.ctypes.data, motion.ctypes.data,
                                                        unique.ctypes.data if unique.size else None,
                                                        unique.size), "add_frame")

    def frame_sizes(self) -> tuple[int, list[int]]:
        """(motion bytes, [Y1, C1, Y2, C2] endpoint bytes) of the last frame."""
        mb = ctypes.c_uint32()
        ep = np.zeros(4, np.uint32)
        _check(host_lib().mptc_stream_writer_frame_sizes(self._h, ctypes.byref(mb), ep.ctypes.data),
               "frame_sizes")
        return int(mb.value), [int(x) for x in ep]

    def finish(self) -> bytes:
        n = ctypes.c_uint64()
        _check(host_lib().mptc_stream_writer_finish(self._h, None, ctypes.byref(n)), "finish")
        buf = np.empty(n.value, np.uint8)
        _check(host_lib().mptc_stream_writer_finish(self._h, buf.ctypes.data, ctypes.byref(n)), "finish")
        return buf.tobytes()

    def close(self) -> None:
        if self._h:
            host_lib().mptc_stream_writer_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def write_stream(frames, width: int, height: int, search_area: int, unique_interval: int) -> bytes:
    """Stream bytes of encoded frames: each item has ``final``, ``motion`` and
    ``unique`` arrays (or is a (final, motion, unique) tuple)."""
    frames = list(frames)
    w = StreamWriter(width, height, search_area, unique_interval, len(frames))
    try:
        for f in frames:
            if isinstance(f, tuple):
                w.add_frame(*f)
            else:
                w.add_frame(f.final, f.motion, f.unique)
        return w.finish()
    finally:
        w.close()
