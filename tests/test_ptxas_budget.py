"""Resource budget of the hot kernels, from ptxas's own report (CPU only: nvcc
cross-compiles for sm_103a without a GPU). The launch shapes rely on these
figures: the inter run kernel runs 8 CTAs of 4 warps per SM (64 registers,
under 28 KB of shared memory each, no spills), the intra dataflow 4 CTAs of
256 threads per SM (64 registers)."""
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "mptc_gb300", "csrc")
FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-lineinfo", "-std=c++17", "-fmad=false",
         "-Xcompiler", "-fPIC", "-Xptxas", "-v"]
ENTRY = re.compile(r"Compiling entry function '(\S+)' for 'sm_103a'\n(?:.*\n)*?.*?(\d+) bytes spill stores, "
                   r"(\d+) bytes spill loads\n.*?Used (\d+) registers(?:.*?(\d+) bytes smem)?")


@pytest.fixture(scope="module")
def report():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    p = subprocess.run([nvcc, *FLAGS, "-c", "mptc_api.cu", "-o", os.devnull], cwd=CSRC, capture_output=True,
                       text=True, timeout=600)
    assert p.returncode == 0, p.stderr[-2000:]
    out = {}
    for name, st, ld, regs, smem in ENTRY.findall(p.stdout + p.stderr):
        out[name] = dict(spill=int(st) + int(ld), regs=int(regs), smem=int(smem or 0))
    assert out, "no ptxas report"
    return out


def _find(report, pattern):
    hits = {k: v for k, v in report.items() if re.search(pattern, k)}
    assert hits, pattern
    return hits


def test_inter_run_kernel_fits_eight_ctas_per_sm(report):
    # inter_run_kernel<WARPS=4, RUN=8, SA=8>: the default search area, window constants folded
    for v in _find(report, r"inter_run_kernelILi4ELi8ELi8E").values():
        assert v["spill"] == 0 and v["regs"] <= 64 and v["smem"] <= 28 * 1024, v


def test_streaming_kernels_do_not_spill(report):
    for pat in (r"inter_overflow_kernel", r"dxt1_encode_kernel", r"unique_scan_kernel", r"pending_scan_kernel",
                r"weight_desc_kernel"):
        for name, v in _find(report, pat).items():
            assert v["spill"] == 0, (name, v)


def test_intra_dataflow_fits_four_ctas_per_sm(report):
    for v in _find(report, r"intra_search_kernelILi256E").values():
        assert v["regs"] <= 64, v
