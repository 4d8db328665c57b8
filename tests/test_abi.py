"""The C-ABI libraries load without a GPU and export every function the public
headers declare (no compute calls: these run on CPU-only machines)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(ROOT, "include")
DECL = re.compile(r"^[A-Za-z_][\w \t]*?\*?\s*\b(mptc_\w+)\s*\(", re.M)


def declared(header: str) -> list[str]:
    text = open(os.path.join(INCLUDE, header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(DECL.findall(text)))


def _load(path):
    if not os.path.exists(path):
        pytest.fail(f"{path} is missing: __graft_entry__.build() must run first")
    return ctypes.CDLL(path)


def test_gb300_library_exports_header():
    from mptc_gb300 import _lib
    names = declared("mptc_gb300.h")
    assert len(names) >= 30
    L = _load(_lib.LIB_PATH)
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, f"declared but not exported: {missing}"
    assert sorted(_lib.EXPORTED) == names


def test_host_library_exports_header():
    from mptc_gb300 import stream
    names = declared("mptc_host.h")
    assert names == sorted(stream.HOST_EXPORTED)
    L = _load(stream.HOST_LIB_PATH)
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, f"declared but not exported: {missing}"


def test_version_and_arch_need_no_gpu():
    from mptc_gb300 import _lib
    L = _load(_lib.LIB_PATH)
    L.mptc_version.restype = ctypes.c_int32
    L.mptc_built_arch.restype = ctypes.c_int32
    assert L.mptc_version() > 0
    assert L.mptc_built_arch() == 1030


def test_default_intra_schedule_matches_reference_loop():
    """The encoder's default intra flags (used by the per-frame and the stream
    calls) follow the reference's schedule: the first frame intra, then every
    intra_interval-th (codec/codec.cpp:1462-1469), as intra_schedule (used by
    the bench and the training loop) and the oracle's stream loop do."""
    from mptc_gb300.encoder import Encoder, intra_schedule
    for interval in (1, 2, 5, 16):
        enc = Encoder.__new__(Encoder)  # the schedule state only: no context
        enc.intra_interval, enc._intra_num, enc._next_intra = interval, 1, True
        flags = [enc._intra_flag(None) for _ in range(70)]
        assert flags == intra_schedule(70, interval)
        assert enc._intra_flag(True) is True and enc._intra_flag(False) is False


def test_buffer_checks_before_the_abi():
    """The Python wrappers check every buffer before its pointer crosses the
    C ABI (which cannot see sizes): type, contiguity, length, then device."""
    import numpy as np
    import torch

    from mptc_gb300._lib import dev_ptr, host_ptr
    with pytest.raises(ValueError, match="integer type of 4 bytes"):
        dev_ptr(torch.zeros(8, dtype=torch.float32), "unique", 4, 8)
    with pytest.raises(ValueError, match="integer type of 8 bytes"):
        dev_ptr(torch.zeros(8, dtype=torch.int32), "final", 8, 8)
    with pytest.raises(ValueError, match="not contiguous"):
        dev_ptr(torch.zeros((8, 8), dtype=torch.int32)[:, 0], "unique", 4, 8)
    with pytest.raises(ValueError, match="at least 9 expected"):
        dev_ptr(torch.zeros(8, dtype=torch.int32), "unique", 4, 9)
    with pytest.raises(ValueError, match="not a CUDA tensor"):
        dev_ptr(torch.zeros(8, dtype=torch.int32), "unique", 4, 8)
    a = np.zeros(8, np.uint32)
    assert host_ptr(a, "unique", np.uint32, 8) == a.ctypes.data
    with pytest.raises(ValueError, match="uint64 expected"):
        host_ptr(a, "final", np.uint64, 4)
    with pytest.raises(ValueError, match="at least 9 expected"):
        host_ptr(a, "unique", np.uint32, 9)
    with pytest.raises(ValueError, match="C-contiguous"):
        host_ptr(np.zeros((8, 8), np.uint32)[:, 0], "unique", np.uint32, 8)
    ro = np.zeros(8, np.uint32)
    ro.flags.writeable = False
    with pytest.raises(ValueError, match="C-contiguous"):
        host_ptr(ro, "unique", np.uint32, 8)


def test_product_path_never_reaches_the_oracle():
    """The package (Python bindings, CUDA sources, host C++) and the public
    headers name nothing under oracle/: the oracle is test infrastructure, and
    the product path has no CPU fallback through it."""
    pkg = os.path.join(ROOT, "mptc_gb300")
    files = [os.path.join(d, f) for d, _, fs in os.walk(pkg) for f in fs
             if f.endswith((".py", ".cu", ".cuh", ".h", ".cpp", ".c")) and "__pycache__" not in d]
    files += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    assert len(files) > 20
    for path in files:
        text = open(path, encoding="utf-8").read()
        assert not re.search(r"\boracle\b|mptc_oracle|libmptc_oracle", text), path
