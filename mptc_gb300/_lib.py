"""ctypes binding of ``libmptc_gb300.so`` (the C ABI in include/mptc_gb300.h).

Loading fails loudly when the library is missing: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libmptc_gb300.so")

MPTC_OK, MPTC_EINVAL, MPTC_ENOMEM, MPTC_ETIMEOUT, MPTC_ECUDA, MPTC_ESTATE = range(6)
STATUS_NAMES = {0: "MPTC_OK", 1: "MPTC_EINVAL", 2: "MPTC_ENOMEM", 3: "MPTC_ETIMEOUT",
                4: "MPTC_ECUDA", 5: "MPTC_ESTATE"}

# Every symbol include/mptc_gb300.h declares.
EXPORTED = [
    "mptc_ctx_create", "mptc_ctx_destroy", "mptc_dxt1_encode", "mptc_reencode",
    "mptc_encode_frame", "mptc_encode_frame_host", "mptc_encode_stream_host", "mptc_encode_stream_device",
    "mptc_last_frame_stats",
    "mptc_last_error",
    "mptc_version", "mptc_built_arch", "mptc_set_kernel_timing", "mptc_kernel_times",
    "mptc_alu_probe", "mptc_encode_frame_noalloc", "mptc_batch_create", "mptc_batch_destroy",
    "mptc_batch_input", "mptc_batch_output", "mptc_batch_upload", "mptc_batch_fetch",
    "mptc_batch_encode", "mptc_batch_autotune", "mptc_model_num_params", "mptc_model_create",
    "mptc_model_destroy", "mptc_model_get_params", "mptc_model_set_params", "mptc_model_train_step",
    "mptc_model_grads", "mptc_model_embed", "mptc_model_save", "mptc_model_load",
    "mptc_ctx_set_model", "mptc_decoded_sse", "mptc_batch_set_model",
    "mptc_endpoint_coefficients", "mptc_decoder_create", "mptc_decoder_destroy", "mptc_decode_frame",
    "mptc_decoder_check", "mptc_decoder_last_error", "mptc_kernel_launches", "mptc_candidate_errors",
    "mptc_learned_proposals", "mptc_ctx_set_learned_shape", "mptc_batch_encode_run",
]

NOALLOC_MAX_BLOCKS = 131072  # MPTC_NOALLOC_MAX_BLOCKS


class Config(ctypes.Structure):
    _fields_ = [("search_area", ctypes.c_int32), ("err_threshold", ctypes.c_int32),
                ("intra_interval", ctypes.c_int32), ("intra_sweeps", ctypes.c_int32)]


class FrameStats(ctypes.Structure):
    _fields_ = [("n_inter", ctypes.c_uint32), ("n_intra", ctypes.c_uint32),
                ("n_unique", ctypes.c_uint32), ("is_intra", ctypes.c_uint32),
                ("n_fallback", ctypes.c_uint32)]


class KernelTime(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char * 32), ("launches", ctypes.c_int32),
                ("total_ms", ctypes.c_double)]


class MptcError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


def dev_ptr(t, name: str, itemsize: int, count: int) -> int:
    """The device pointer of a tensor argument, after checking it: the C ABI
    takes plain pointers and cannot see a buffer's size, so a short, strided
    or mistyped tensor would be read or written past its end on the device.
    Requires an integer tensor of `itemsize`-byte elements, contiguous, with
    at least `count` elements, on a CUDA device."""
    if t.is_floating_point() or t.is_complex() or t.element_size() != itemsize:
        raise ValueError(f"{name}: {t.dtype} given, an integer type of {itemsize} bytes expected")
    if not t.is_contiguous():
        raise ValueError(f"{name}: not contiguous")
    if t.numel() < count:
        raise ValueError(f"{name}: {t.numel()} elements given, at least {count} expected")
    if not t.is_cuda:
        raise ValueError(f"{name}: not a CUDA tensor")
    return t.data_ptr()


def host_ptr(a: np.ndarray, name: str, dtype, count: int) -> int:
    """The same checks for a host output array: exact dtype, C-contiguous,
    writable, at least `count` elements."""
    if a.dtype != np.dtype(dtype):
        raise ValueError(f"{name}: {a.dtype} given, {np.dtype(dtype)} expected")
    if not a.flags.c_contiguous or not a.flags.writeable:
        raise ValueError(f"{name}: not a writable C-contiguous array")
    if a.size < count:
        raise ValueError(f"{name}: {a.size} elements given, at least {count} expected")
    return a.ctypes.data


_LIB = None


def lib() -> ctypes.CDLL:
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: run __graft_entry__.build() "
                               "(the encoder has no CPU fallback)")
        L = ctypes.CDLL(LIB_PATH)
        vp, i32, u32p = ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p
        L.mptc_ctx_create.argtypes = [ctypes.POINTER(Config), i32, i32, ctypes.POINTER(vp)]
        L.mptc_ctx_destroy.argtypes = [vp]
        L.mptc_dxt1_encode.argtypes = [vp, vp, vp, vp, vp]
        L.mptc_reencode.argtypes = [vp, vp, vp, vp, vp, vp, vp, vp, u32p, vp]
        L.mptc_encode_frame.argtypes = [vp, vp, vp, vp, vp, vp, vp, u32p, vp]
        L.mptc_encode_frame_host.argtypes = [vp, vp, i32, vp, vp, vp, vp, u32p, vp]
        L.mptc_encode_stream_host.argtypes = [vp, vp, i32, vp, vp, vp, vp, vp, vp]
        L.mptc_encode_stream_device.argtypes = [vp, vp, i32, vp, vp, vp, vp, vp, vp]
        L.mptc_last_frame_stats.argtypes = [vp, ctypes.POINTER(FrameStats), vp]
        L.mptc_last_error.argtypes = [vp]
        L.mptc_last_error.restype = ctypes.c_char_p
        L.mptc_set_kernel_timing.argtypes = [vp, i32]
        L.mptc_kernel_times.argtypes = [vp, ctypes.POINTER(KernelTime), i32,
                                        ctypes.POINTER(ctypes.c_int32)]
        L.mptc_alu_probe.argtypes = [i32, i32, vp, ctypes.POINTER(ctypes.c_double), vp]
        L.mptc_encode_frame_noalloc.argtypes = [ctypes.POINTER(Config), i32, i32, vp, vp, vp, vp, vp,
                                                vp, u32p, vp]
        L.mptc_batch_create.argtypes = [ctypes.POINTER(Config), i32, vp, vp, ctypes.POINTER(vp)]
        L.mptc_batch_destroy.argtypes = [vp]
        L.mptc_batch_input.argtypes = [vp, i32, ctypes.POINTER(vp)]
        L.mptc_batch_output.argtypes = [vp, i32, ctypes.POINTER(vp), ctypes.POINTER(vp),
                                        ctypes.POINTER(vp), ctypes.POINTER(vp)]
        L.mptc_batch_upload.argtypes = [vp, i32, vp, vp]
        L.mptc_batch_fetch.argtypes = [vp, i32, vp, vp, vp, ctypes.POINTER(ctypes.c_uint32), vp]
        L.mptc_batch_encode.argtypes = [vp, vp, vp]
        L.mptc_batch_autotune.argtypes = [vp, vp, ctypes.POINTER(i32), ctypes.POINTER(i32), ctypes.POINTER(i32), vp]
        fp = ctypes.POINTER(ctypes.c_float)
        L.mptc_model_num_params.restype = ctypes.c_int64
        L.mptc_model_create.argtypes = [ctypes.c_uint64, ctypes.POINTER(vp)]
        L.mptc_model_destroy.argtypes = [vp]
        L.mptc_model_get_params.argtypes = [vp, vp]
        L.mptc_model_set_params.argtypes = [vp, vp]
        L.mptc_model_train_step.argtypes = [vp, vp, i32, vp, vp, vp, i32, i32, ctypes.c_float,
                                            ctypes.c_float, fp, vp]
        L.mptc_model_grads.argtypes = [vp, vp, i32, vp, vp, vp, i32, i32, vp, fp, vp]
        L.mptc_model_embed.argtypes = [vp, vp, i32, vp, vp, i32, vp, vp, i32, i32, vp, vp]
        L.mptc_model_save.argtypes = [vp, ctypes.c_char_p]
        L.mptc_model_load.argtypes = [vp, ctypes.c_char_p]
        L.mptc_ctx_set_model.argtypes = [vp, vp, i32]
        L.mptc_decoded_sse.argtypes = [vp, i32, i32, vp, vp, vp]
        L.mptc_learned_proposals.argtypes = [vp, vp, vp, vp, vp, vp]
        L.mptc_batch_encode_run.argtypes = [vp, i32, vp, vp, vp, vp, vp, vp, vp]
        L.mptc_ctx_set_learned_shape.argtypes = [vp, i32]
        L.mptc_candidate_errors.argtypes = [vp, i32, i32, vp, vp, vp, i32, i32, vp, vp]
        L.mptc_batch_set_model.argtypes = [vp, vp, i32]
        L.mptc_endpoint_coefficients.argtypes = [i32, i32, vp, vp, vp]
        L.mptc_decoder_create.argtypes = [i32, i32, i32, ctypes.POINTER(vp)]
        L.mptc_decoder_destroy.argtypes = [vp]
        L.mptc_decode_frame.argtypes = [vp, vp, vp, vp, ctypes.c_uint32, vp, vp, vp]
        L.mptc_decoder_check.argtypes = [vp, vp, ctypes.POINTER(ctypes.c_uint32)]
        L.mptc_decoder_last_error.argtypes = [vp]
        L.mptc_decoder_last_error.restype = ctypes.c_char_p
        L.mptc_kernel_launches.argtypes = [vp, ctypes.POINTER(ctypes.c_uint64)]
        L.mptc_version.restype = i32
        L.mptc_built_arch.restype = i32
        for name in EXPORTED:
            if name not in ("mptc_last_error", "mptc_version", "mptc_built_arch",
                            "mptc_model_num_params", "mptc_decoder_last_error"):
                getattr(L, name).restype = ctypes.c_int
        _LIB = L
    return _LIB


def check(status: int, ctx=None) -> None:
    if status != MPTC_OK:
        msg = lib().mptc_last_error(ctx).decode() if ctx else ""
        raise MptcError(status, msg)
