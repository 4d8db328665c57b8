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
    intra_interval-th (codec/codec.cpp:1462-1469), as bench.intra_schedule
    and the oracle's stream loop do."""
    from mptc_gb300.encoder import Encoder

    import bench
    for interval in (1, 2, 5, 16):
        enc = Encoder.__new__(Encoder)  # the schedule state only: no context
        enc.intra_interval, enc._intra_num, enc._next_intra = interval, 1, True
        flags = [enc._intra_flag(None) for _ in range(70)]
        assert flags == bench.intra_schedule(70, interval)
        assert enc._intra_flag(True) is True and enc._intra_flag(False) is False
