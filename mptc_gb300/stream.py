"""MPTC stream writer and reader: ctypes binding of ``libmptc_host.so``
(include/mptc_host.h).

The writer turns the per-frame arrays the encoder returns (final blocks,
motion codes, unique palette) into the bytes of an MPTC stream, identical to
the stream the reference encoder's ``CompressMultiUnique``
(codec/codec.cpp:1307-1532) writes for the same frames. The reader walks a
stream and entropy-decodes each frame's parts for the GPU decoder
(``mptc_gb300.decoder``). Host-only: no GPU is needed.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from ._lib import MptcError, host_ptr

_HERE = os.path.dirname(os.path.abspath(__file__))
HOST_LIB_PATH = os.path.join(_HERE, "libmptc_host.so")

HOST_EXPORTED = [
    "mptc_stream_writer_create", "mptc_stream_writer_destroy", "mptc_stream_writer_add_frame",
    "mptc_stream_writer_add_frame_coefficients", "mptc_stream_writer_add_frames",
    "mptc_stream_writer_add_frames_coefficients", "mptc_stream_writer_finish",
    "mptc_stream_writer_frame_sizes", "mptc_stream_reader_open", "mptc_stream_reader_destroy",
    "mptc_stream_reader_info", "mptc_stream_reader_next", "mptc_stream_reader_next_frames",
]


class StreamInfo(ctypes.Structure):
    _fields_ = [("width", ctypes.c_int32), ("height", ctypes.c_int32), ("search_area", ctypes.c_int32),
                ("unique_interval", ctypes.c_int32), ("groups", ctypes.c_uint32),
                ("frames", ctypes.c_uint32), ("max_unique_count", ctypes.c_uint32),
                ("max_compressed_palette", ctypes.c_uint32),
                ("max_compressed_motion_indices", ctypes.c_uint32),
                ("max_compressed_ep_y", ctypes.c_uint32), ("max_compressed_ep_c", ctypes.c_uint32)]


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
        L.mptc_stream_writer_add_frame_coefficients.argtypes = [vp, vp, vp, vp, ctypes.c_uint32]
        L.mptc_stream_writer_add_frames.argtypes = [vp, i32, vp, vp, vp, vp]
        L.mptc_stream_writer_add_frames_coefficients.argtypes = [vp, i32, vp, vp, vp, vp]
        L.mptc_stream_reader_open.argtypes = [vp, ctypes.c_uint64, ctypes.POINTER(vp)]
        L.mptc_stream_reader_destroy.argtypes = [vp]
        L.mptc_stream_reader_info.argtypes = [vp, ctypes.POINTER(StreamInfo)]
        L.mptc_stream_reader_next.argtypes = [vp, vp, vp, vp, ctypes.POINTER(ctypes.c_uint32)]
        L.mptc_stream_reader_next_frames.argtypes = [vp, i32, vp, vp, vp, vp, ctypes.POINTER(i32)]
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

    def add_frame_coefficients(self, coeff: np.ndarray, motion: np.ndarray, unique: np.ndarray) -> None:
        """A frame whose endpoint images are already transformed: ``coeff`` is
        the six coefficient planes [Y1|Co1|Cg1|Y2|Co2|Cg2], blocks bytes each."""
        coeff = np.ascontiguousarray(coeff, dtype=np.uint8).reshape(-1)
        motion = np.ascontiguousarray(motion, dtype=np.uint8).reshape(-1)
        unique = np.ascontiguousarray(unique, dtype=np.uint32).reshape(-1)
        if coeff.size != 6 * self.blocks or motion.size != 2 * self.blocks:
            raise ValueError(f"frame arrays do not match {self.blocks} blocks")
        _check(host_lib().mptc_stream_writer_add_frame_coefficients(
            self._h, coeff.ctypes.data, motion.ctypes.data, unique.ctypes.data if unique.size else None,
            unique.size), "add_frame_coefficients")

    def add_frames(self, final: np.ndarray, motion: np.ndarray, unique: np.ndarray, n_unique: np.ndarray,
                   coefficients: bool = False) -> None:
        """A run of F frames in one call, coded on all host cores: final (F,
        blocks) u64 (or, with coefficients=True, (F, 6 * blocks) u8 coefficient
        planes), motion (F, 2 * blocks) u8, unique (F, blocks) u32 with frame
        f's palette in unique[f, :n_unique[f]], n_unique (F,) u32 — the
        layout of Encoder.encode_stream_host's StreamOutput."""
        f = int(np.shape(n_unique)[0])
        n = self.blocks
        nu = np.ascontiguousarray(n_unique, dtype=np.uint32).reshape(-1)
        if coefficients:
            src = np.ascontiguousarray(final, dtype=np.uint8)
            src_ptr = host_ptr(src.reshape(-1), "coeff", np.uint8, 6 * n * f)
        else:
            src = np.ascontiguousarray(final, dtype=np.uint64)
            src_ptr = host_ptr(src.reshape(-1), "final", np.uint64, n * f)
        mot = np.ascontiguousarray(motion, dtype=np.uint8)
        uni = np.ascontiguousarray(unique, dtype=np.uint32)
        ptrs = (host_ptr(mot.reshape(-1), "motion", np.uint8, 2 * n * f),
                host_ptr(uni.reshape(-1), "unique", np.uint32, n * f), nu.ctypes.data)
        call = (host_lib().mptc_stream_writer_add_frames_coefficients if coefficients
                else host_lib().mptc_stream_writer_add_frames)
        _check(call(self._h, f, src_ptr, *ptrs), "add_frames")

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


def write_stream(frames, width: int, height: int, search_area: int, unique_interval: int,
                 chunk_frames: int | None = None) -> bytes:
    """Stream bytes of encoded frames: each item has ``final``, ``motion`` and
    ``unique`` arrays (or is a (final, motion, unique) tuple). The frames are
    coded in add_frames calls of ``chunk_frames`` frames each (default: twice
    the host's cores, the writer's own chunk), so that only one chunk's
    stacked arrays are held at a time; the bytes do not depend on the chunk."""
    frames = [f if isinstance(f, tuple) else (f.final, f.motion, f.unique) for f in frames]
    w = StreamWriter(width, height, search_area, unique_interval, len(frames))
    step = chunk_frames if chunk_frames is not None else 2 * (os.cpu_count() or 1)
    if step < 1:
        raise ValueError("chunk_frames must be positive")
    try:
        n = w.blocks
        for c0 in range(0, len(frames), step):
            part = frames[c0:c0 + step]
            final = np.stack([np.asarray(f[0], np.uint64).reshape(-1) for f in part])
            motion = np.stack([np.asarray(f[1], np.uint8).reshape(-1) for f in part])
            n_unique = np.array([np.size(f[2]) for f in part], np.uint32)
            if final.shape[1] != n or motion.shape[1] != 2 * n or (n_unique > n).any():
                raise ValueError(f"frame arrays do not match {n} blocks")
            unique = np.zeros((len(part), n), np.uint32)
            for k, f in enumerate(part):
                unique[k, : n_unique[k]] = np.asarray(f[2], np.uint32).reshape(-1)
            w.add_frames(final, motion, unique, n_unique)
        return w.finish()
    finally:
        w.close()


class StreamReader:
    """Walks an MPTC stream and entropy-decodes each frame's parts (the host
    half of the reference decoder's GetFrame, codec/decoder.cpp:256-414)."""

    def __init__(self, data: bytes):
        self._buf = np.frombuffer(data, np.uint8)
        self._h = ctypes.c_void_p()
        _check(host_lib().mptc_stream_reader_open(self._buf.ctypes.data if self._buf.size else None,
                                                   self._buf.size, ctypes.byref(self._h)),
               "stream header")
        self.info = StreamInfo()
        _check(host_lib().mptc_stream_reader_info(self._h, ctypes.byref(self.info)), "stream info")
        self.blocks = (self.info.width // 4) * (self.info.height // 4)

    def next_frame(self, motion=None, coeff=None, unique=None):
        """(motion u8[2n], coeff u8[6n], unique u32[n_unique]) of the next frame,
        or None after the last one. Output arrays may be passed in for reuse."""
        n = self.blocks
        motion = np.empty(2 * n, np.uint8) if motion is None else motion
        coeff = np.empty(6 * n, np.uint8) if coeff is None else coeff
        unique = np.empty(n, np.uint32) if unique is None else unique
        ptrs = (host_ptr(motion, "motion", np.uint8, 2 * n), host_ptr(coeff, "coeff", np.uint8, 6 * n),
                host_ptr(unique, "unique", np.uint32, n))
        nu = ctypes.c_uint32()
        rc = host_lib().mptc_stream_reader_next(self._h, *ptrs, ctypes.byref(nu))
        if rc == 5:  # MPTC_ESTATE: no frames left
            return None
        _check(rc, "stream frame")
        return motion, coeff, unique[: nu.value]

    def next_frames(self, max_frames: int):
        """Up to max_frames next frames, their parts decoded on all host cores:
        (motion (F, 2n) u8, coeff (F, 6n) u8, unique (F, n) u32, n_unique (F,)
        u32) with F frames read (0 at the end of the stream)."""
        n = self.blocks
        motion = np.empty((max_frames, 2 * n), np.uint8)
        coeff = np.empty((max_frames, 6 * n), np.uint8)
        unique = np.empty((max_frames, n), np.uint32)
        nu = np.zeros(max_frames, np.uint32)
        got = ctypes.c_int32(0)
        rc = host_lib().mptc_stream_reader_next_frames(self._h, max_frames, motion.ctypes.data, coeff.ctypes.data,
                                                       unique.ctypes.data, nu.ctypes.data, ctypes.byref(got))
        if rc == 5:  # MPTC_ESTATE: no frames left
            got.value = 0
        else:
            _check(rc, "stream frames")
        f = got.value
        return motion[:f], coeff[:f], unique[:f], nu[:f]

    def __iter__(self):
        while True:
            f = self.next_frame()
            if f is None:
                return
            yield f

    def close(self) -> None:
        if self._h:
            host_lib().mptc_stream_reader_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
