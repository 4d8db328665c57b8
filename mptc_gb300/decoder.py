"""GPU decode of MPTC streams and the GPU endpoint transform.

``Decoder`` rebuilds each frame's physical DXT1 blocks on the GPU from the
parts ``StreamReader`` entropy-decodes on the host: the GPU half of the
reference decoder's GetFrame (codec/decoder.cpp:68-254). The blocks stay in
device memory (a DXT1 texture ready for upload), with no graphics API.
``endpoint_coefficients`` is the encoder-side transform (CompressEndpoint,
codec/codec.cpp:804-838) for ``StreamWriter.add_frame_coefficients``.
"""
from __future__ import annotations

import ctypes

import numpy as np

from ._lib import MptcError, dev_ptr, lib
from .stream import StreamReader


def _stream_ptr(stream) -> ctypes.c_void_p:
    return ctypes.c_void_p(stream.cuda_stream if stream is not None else 0)


def endpoint_coefficients(width: int, height: int, blocks_dev, coeff_dev, stream=None) -> None:
    """blocks_dev: torch CUDA tensor of width/4*height/4 u64 (int64) blocks;
    coeff_dev: torch CUDA uint8 tensor of 6 * blocks bytes."""
    n = (width // 4) * (height // 4)
    rc = lib().mptc_endpoint_coefficients(width, height, dev_ptr(blocks_dev, "blocks", 8, n),
                                          dev_ptr(coeff_dev, "coeff", 1, 6 * n), _stream_ptr(stream))
    if rc != 0:
        raise MptcError(rc, f"endpoint_coefficients {width}x{height}")


class Decoder:
    """Per-stream GPU decoder state (frame size and search area from the header)."""

    def __init__(self, width: int, height: int, search_area: int):
        import torch
        self.width, self.height, self.search_area = width, height, search_area
        self.blocks = (width // 4) * (height // 4)
        h = ctypes.c_void_p()
        rc = lib().mptc_decoder_create(width, height, search_area, ctypes.byref(h))
        if rc != 0:
            raise MptcError(rc, f"decoder for {width}x{height}, search area {search_area}")
        self._h = h
        dev = torch.device("cuda")
        n = self.blocks
        self._coeff = torch.empty(6 * n, dtype=torch.uint8, device=dev)
        self._motion = torch.empty(2 * n, dtype=torch.uint8, device=dev)
        self._unique = torch.empty(max(n, 1), dtype=torch.int32, device=dev)
        self._frames = [torch.empty(n, dtype=torch.int64, device=dev) for _ in range(2)]
        self._cur = -1

    def decode_frame(self, motion, coeff, unique, stream=None):
        """Device-side decode of one frame from host arrays (numpy) or CUDA
        tensors; returns the device tensor of blocks (valid until the frame
        after next is decoded)."""
        import torch
        n_unique = int(unique.size if isinstance(unique, np.ndarray) else unique.numel())
        n = self.blocks
        for name, a, want in (("motion", motion, 2 * n), ("coeff", coeff, 6 * n)):
            size = a.size if isinstance(a, np.ndarray) else a.numel()
            if size != want:
                raise ValueError(f"{name}: {size} bytes given, {want} expected")
        if n_unique > n:
            raise ValueError(f"unique: {n_unique} entries given, at most {n} expected")
        s = stream if stream is not None else torch.cuda.current_stream()
        with torch.cuda.stream(s):  # staging copies ordered with the decode kernels
            for dst, src in ((self._motion, motion), (self._coeff, coeff)):
                dst.copy_(torch.from_numpy(src) if isinstance(src, np.ndarray) else src)
            if n_unique:
                u = unique.view(np.int32) if isinstance(unique, np.ndarray) else unique.view(torch.int32)
                self._unique[:n_unique].copy_(torch.from_numpy(u) if isinstance(u, np.ndarray) else u)
        prev = self._frames[self._cur].data_ptr() if self._cur >= 0 else None
        self._cur = (self._cur + 1) % 2
        out = self._frames[self._cur]
        rc = lib().mptc_decode_frame(self._h, self._coeff.data_ptr(), self._motion.data_ptr(),
                                     self._unique.data_ptr(), n_unique, prev, out.data_ptr(),
                                     _stream_ptr(s))
        if rc != 0:
            raise MptcError(rc, lib().mptc_decoder_last_error(self._h).decode())
        return out

    def check(self, stream=None) -> None:
        """Raises if a frame decoded since the last check held invalid codes."""
        import torch
        s = stream if stream is not None else torch.cuda.current_stream()
        flags = ctypes.c_uint32()
        rc = lib().mptc_decoder_check(self._h, _stream_ptr(s), ctypes.byref(flags))
        if rc != 0:
            raise MptcError(rc, lib().mptc_decoder_last_error(self._h).decode())

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().mptc_decoder_destroy(self._h)
            self._h = None

    def __del__(self):  # pragma: no cover - best effort
        try:
            self.close()
        except Exception:
            pass


def decode_stream(data: bytes) -> list[np.ndarray]:
    """All frames of a stream as host arrays of u64 physical blocks."""
    rd = StreamReader(data)
    dec = Decoder(rd.info.width, rd.info.height, rd.info.search_area)
    out = []
    try:
        for motion, coeff, unique in rd:
            blocks = dec.decode_frame(motion, coeff, unique)
            out.append(blocks.cpu().numpy().view(np.uint64).copy())
        dec.check()
    finally:
        dec.close()
        rd.close()
    return out
