"""The drop-in binding compiles and links against the reference codec.

tests/c/dxtimage_binding.cpp fills a reference MPTC::DXTImage from
libmptc_gb300 and hands it to the reference's EntropyEncode. This test builds
it together with the reference's own codec/codec.cpp, codec/dxt_image.cpp and
the sources they need, against include/mptc_gb300.h, into a shared object
linked with libmptc_gb300.so and no undefined symbols: the binding a
maintainer adds is checked by the compiler and the linker,
not only shown. It needs the reference sources, named by the environment
variable MPTC_REFERENCE; without it the test is skipped. Link-only: no GPU.
"""
import os
import shutil
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("MPTC_REFERENCE", "")


@pytest.mark.skipif(not (REF and os.path.isfile(os.path.join(REF, "codec", "codec.cpp"))),
                    reason="the reference sources are not available (set MPTC_REFERENCE)")
@pytest.mark.skipif(shutil.which("g++") is None, reason="no C++ compiler")
def test_binding_links_with_reference_codec():
    lib = os.path.join(ROOT, "mptc_gb300", "libmptc_gb300.so")
    if not os.path.exists(lib):
        pytest.skip("libmptc_gb300.so is not built")
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    srcs = [os.path.join(ROOT, "tests", "c", "dxtimage_binding.cpp")] + [
        os.path.join(REF, p) for p in ("codec/codec.cpp", "codec/dxt_image.cpp", "codec/image.cpp",
                                       "codec/wavelet.cpp", "codec/image_processing.cpp",
                                       "entropy/arithmetic_codec.cpp")]
    with tempfile.TemporaryDirectory() as td:
        out = os.path.join(td, "libbinding.so")
        cmd = ["g++", "-std=gnu++11", "-O1", "-w", "-fms-extensions", "-fPIC", "-shared", "-Wl,--no-undefined",
               "-I", os.path.join(ROOT, "include"), "-I", os.path.join(REF, "codec"),
               "-I", os.path.join(REF, "entropy"), "-I", os.path.join(REF, "Include"), *srcs,
               "-L", os.path.join(ROOT, "mptc_gb300"), "-lmptc_gb300", "-L", os.path.join(cuda, "lib64"),
               "-lcudart", "-lpthread", "-o", out]
        r = subprocess.run(cmd, capture_output=True, text=True, cwd=td)
        assert r.returncode == 0, r.stderr[-4000:]
        nm = subprocess.run(["nm", "-D", "--defined-only", out], capture_output=True, text=True)
        assert "EncodeFrameOnGpu" in nm.stdout and "EncodeRecordsOnGpu" in nm.stdout
        und = subprocess.run(["nm", "-D", "--undefined-only", out], capture_output=True, text=True).stdout
        assert "mptc_encode_frame_host" in und and "mptc_ctx_create" in und
