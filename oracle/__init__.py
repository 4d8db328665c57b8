"""ORACLE — test infrastructure only.

ctypes binding of ``libmptc_oracle.so``, the CPU restatement of the MPTC
encoder hot path (stb_dxt DXT1 encode + DXTImage::Reencode index search).
Only tests, the smoke check and the CPU-baseline leg of bench.py use it, as the
checker. The product path (``mptc_gb300``) never imports it.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None


class Stats(ctypes.Structure):
    _fields_ = [("inter_visited", ctypes.c_int64), ("intra_visited", ctypes.c_int64),
                ("refits", ctypes.c_int64), ("n_inter", ctypes.c_int32),
                ("n_intra", ctypes.c_int32), ("n_unique", ctypes.c_int32)]


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "libmptc_oracle.so")
        if not os.path.exists(path):
            raise RuntimeError(f"{path} is missing: run `make -C oracle` (or build())")
        L = ctypes.CDLL(path)
        vp, i32 = ctypes.c_void_p, ctypes.c_int
        L.mo_stb_encode_block.argtypes = [vp]
        L.mo_stb_encode_block.restype = ctypes.c_uint64
        L.mo_dxt1_encode_frame.argtypes = [vp, i32, i32, vp]
        L.mo_block_error.argtypes = [vp, ctypes.c_uint64]
        L.mo_refit.argtypes = [vp, ctypes.c_uint32, vp, vp, ctypes.POINTER(i32)]
        L.mo_reencode_frame_mt.argtypes = [vp, i32, i32, vp, vp, i32, ctypes.c_int32, vp, vp, vp,
                                           ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(Stats),
                                           i32]
        L.mo_frame_psnr.argtypes = [vp, i32, i32, vp, vp]
        L.mo_frame_psnr.restype = ctypes.c_double
        L.mo_decoded_sse.argtypes = [vp, i32, i32, vp]
        L.mo_decoded_sse.restype = ctypes.c_uint64
        _LIB = L
    return _LIB


def _ptr(a: np.ndarray):
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data


def stb_encode_block(rgba: np.ndarray) -> int:
    a = np.ascontiguousarray(rgba, dtype=np.uint8).reshape(64)
    return int(lib().mo_stb_encode_block(_ptr(a)))


def dxt1_encode(frame: np.ndarray) -> np.ndarray:
    h, w, _ = frame.shape
    f = np.ascontiguousarray(frame, dtype=np.uint8)
    out = np.empty((h // 4) * (w // 4), dtype=np.uint64)
    if lib().mo_dxt1_encode_frame(_ptr(f), w, h, _ptr(out)) != 0:
        raise ValueError("invalid frame size")
    return out


def block_error(px48: np.ndarray, block: int) -> int:
    a = np.ascontiguousarray(px48, dtype=np.uint8).reshape(48)
    return int(lib().mo_block_error(_ptr(a), ctypes.c_uint64(block)))


def refit(px48: np.ndarray, interp: int):
    a = np.ascontiguousarray(px48, dtype=np.uint8).reshape(48)
    e1 = np.zeros(3, np.uint8)
    e2 = np.zeros(3, np.uint8)
    valid = ctypes.c_int(0)
    err = lib().mo_refit(_ptr(a), ctypes.c_uint32(interp), _ptr(e1), _ptr(e2), ctypes.byref(valid))
    return int(err), e1, e2, bool(valid.value)


def decoded_sse(frame: np.ndarray, blocks: np.ndarray) -> int:
    """Squared error of a frame against its decoded DXT1 blocks (u64 each)."""
    h, w, _ = frame.shape
    f = np.ascontiguousarray(frame, dtype=np.uint8)
    b = np.ascontiguousarray(blocks, dtype=np.uint64)
    assert b.size == (h // 4) * (w // 4)
    return int(lib().mo_decoded_sse(_ptr(f), w, h, _ptr(b)))


@dataclass
class FrameResult:
    stb: np.ndarray        # u64 per block
    final: np.ndarray      # u64 per block
    motion: np.ndarray     # u8, 2 per block
    unique: np.ndarray     # u32 unique palette (raster order)
    stats: Stats
    psnr: float


def reencode(frame: np.ndarray, stb: np.ndarray, prev_final: np.ndarray | None, search_area: int,
             threshold: int, threads: int = 1, want_psnr: bool = True) -> FrameResult:
    h, w, _ = frame.shape
    f = np.ascontiguousarray(frame, dtype=np.uint8)
    nblk = (h // 4) * (w // 4)
    stb = np.ascontiguousarray(stb, dtype=np.uint64)
    final = np.empty(nblk, np.uint64)
    motion = np.empty(2 * nblk, np.uint8)
    uniq = np.empty(nblk, np.uint32)
    nu = ctypes.c_uint32(0)
    st = Stats()
    prev_p = None
    if prev_final is not None:
        prev_final = np.ascontiguousarray(prev_final, dtype=np.uint64)
        prev_p = _ptr(prev_final)
    rc = lib().mo_reencode_frame_mt(_ptr(f), w, h, _ptr(stb), prev_p, search_area, threshold,
                                    _ptr(final), _ptr(motion), _ptr(uniq), ctypes.byref(nu),
                                    ctypes.byref(st), threads)
    if rc != 0:
        raise ValueError(f"oracle reencode failed ({rc})")
    psnr = float(lib().mo_frame_psnr(_ptr(f), w, h, _ptr(final), _ptr(stb))) if want_psnr else float("nan")
    return FrameResult(stb, final, motion, uniq[: nu.value].copy(), st, psnr)


def encode_stream(frames: np.ndarray, search_area: int = 8, threshold: int = 5,
                  intra_interval: int = 16, threads: int = 1, want_psnr: bool = True):
    """Whole-stream hot path: frame 1 intra, then every intra_interval-th frame
    (codec/codec.cpp:1379-1469); inter frames search the previous final blocks."""
    out = []
    prev = None
    intra_num = 1
    set_intra = True
    for f in frames:
        stb = dxt1_encode(f)
        r = reencode(f, stb, None if set_intra else prev, search_area, threshold, threads, want_psnr)
        out.append(r)
        if intra_num <= intra_interval:
            set_intra = False
            if intra_num == intra_interval:
                set_intra = True
                intra_num = 1
            else:
                intra_num += 1
        prev = r.final
    return out
