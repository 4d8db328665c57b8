"""Seeded synthetic RGB8 video for the MPTC encoder workloads.

The generator itself is integer C (``csrc/synth_frames.c``) so that a seed
gives the same bytes on every host. Workload presets follow the five encoder
configurations the project measures: a 256x256 smoke stream, 720p with a scene
cut, 1080p, a mixed-resolution multi-stream batch and a 2160p stress case.
Widths that are not multiples of 4 (854) are padded to the next multiple of 4
by the caller; the generator itself takes any size.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass, replace

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None


class _Cfg(ctypes.Structure):
    _fields_ = [
        ("width", ctypes.c_int), ("height", ctypes.c_int),
        ("period_min", ctypes.c_int), ("period_max", ctypes.c_int),
        ("amp_min", ctypes.c_int), ("amp_max", ctypes.c_int),
        ("n_squares", ctypes.c_int), ("square_size", ctypes.c_int),
        ("speed_min", ctypes.c_int), ("speed_max", ctypes.c_int),
        ("cut_every", ctypes.c_int),
        ("seed", ctypes.c_uint64),
    ]


def _lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "libmptc_synth.so")
        if not os.path.exists(path):
            raise RuntimeError(f"{path} is missing: run __graft_entry__.build() first")
        lib = ctypes.CDLL(path)
        lib.mptc_synth_frames.argtypes = [ctypes.POINTER(_Cfg), ctypes.c_int, ctypes.c_int,
                                          ctypes.c_void_p]
        lib.mptc_synth_frames.restype = ctypes.c_int
        _LIB = lib
    return _LIB


@dataclass(frozen=True)
class StreamSpec:
    width: int
    height: int
    frames: int
    period_min: int = 32
    period_max: int = 256
    amp_min: int = 20
    amp_max: int = 50
    n_squares: int = 1
    square_size: int = 64
    speed_min: int = 2
    speed_max: int = 2
    cut_every: int = 0
    seed: int = 1000

    def padded(self, multiple: int = 4) -> "StreamSpec":
        w = (self.width + multiple - 1) // multiple * multiple
        h = (self.height + multiple - 1) // multiple * multiple
        return replace(self, width=w, height=h)

    def generate(self, first: int = 0, count: int | None = None) -> np.ndarray:
        """Frames [first, first+count) as a (count, H, W, 3) uint8 array."""
        count = self.frames - first if count is None else count
        out = np.empty((count, self.height, self.width, 3), dtype=np.uint8)
        c = _Cfg(self.width, self.height, self.period_min, self.period_max, self.amp_min,
                 self.amp_max, self.n_squares, self.square_size, self.speed_min, self.speed_max,
                 self.cut_every, self.seed)
        rc = _lib().mptc_synth_frames(ctypes.byref(c), first, count, out.ctypes.data)
        if rc != 0:
            raise ValueError(f"invalid synthetic stream spec {self}")
        return out


# Workload presets (search_area 8, threshold 5, intra interval 16 unless noted).
SMOKE_256 = StreamSpec(256, 256, 16)
HD720 = StreamSpec(1280, 720, 64, period_min=64, period_max=512, n_squares=4, square_size=128,
                   speed_min=1, speed_max=4, cut_every=32)
FHD1080 = StreamSpec(1920, 1080, 120)
FHD1080_TRAIN = StreamSpec(1920, 1080, 200, seed=5000)
# calibration frames of the learned proposal's K: neither trained on nor measured
FHD1080_CALIB = StreamSpec(1920, 1080, 16, seed=7000)
UHD2160 = StreamSpec(3840, 2160, 60, period_min=128, period_max=1024, n_squares=16,
                     square_size=256, speed_min=1, speed_max=4, cut_every=20)


def mixed_batch(frames: int = 30) -> list[StreamSpec]:
    """32 streams: 8 each of 854x480 (padded to 856), 720p, 1080p, 1440p."""
    sizes = [(854, 480), (1280, 720), (1920, 1080), (2560, 1440)]
    out = []
    for k, (w, h) in enumerate(sizes):
        for s in range(8):
            out.append(StreamSpec(w, h, frames, seed=1000 + 8 * k + s).padded(4))
    return out


def uhd_streams() -> list[StreamSpec]:
    return [replace(UHD2160, seed=1000 + s) for s in range(4)]


def pad_edge(frames: np.ndarray, multiple: int) -> np.ndarray:
    """Frames (..., H, W, 3) padded on the right and bottom to multiples of
    `multiple` pixels by repeating the last column and row. The reference's
    stream writer needs frame sizes that are multiples of 256 pixels (its
    endpoint wavelet works on 64x64-block tiles, codec/image_processing.h:293-294)
    and its block gather needs widths that are multiples of 4
    (codec/dxt_image.cpp:128-139)."""
    h, w = frames.shape[-3], frames.shape[-2]
    ph = (h + multiple - 1) // multiple * multiple - h
    pw = (w + multiple - 1) // multiple * multiple - w
    if ph == 0 and pw == 0:
        return frames
    widths = [(0, 0)] * (frames.ndim - 3) + [(0, ph), (0, pw), (0, 0)]
    return np.pad(frames, widths, mode="edge")
