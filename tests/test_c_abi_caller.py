"""The public headers are a C ABI: a plain C99 program (and the same source as
C++) includes both headers, links both libraries and calls them (CPU only:
the GPU-free calls and the host stream writer/reader)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "c", "abi_caller.c")
LIBDIR = os.path.join(ROOT, "mptc_gb300")
CUDA_LIB = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "lib64")


@pytest.mark.parametrize("compiler,flags", [("gcc", ["-std=c99", "-pedantic"]),
                                            ("g++", ["-x", "c++", "-std=c++17", "-pedantic"])])
def test_c_program_includes_links_and_calls_the_abi(tmp_path, compiler, flags):
    if not shutil.which(compiler):
        pytest.skip(f"{compiler} not available")
    for lib in ("libmptc_gb300.so", "libmptc_host.so"):
        if not os.path.exists(os.path.join(LIBDIR, lib)):
            pytest.fail(f"{lib} is missing: __graft_entry__.build() must run first")
    exe = str(tmp_path / "abi_caller")
    cmd = [compiler, *flags, "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"), SRC, "-o", exe,
           "-x", "none", "-L", LIBDIR, "-lmptc_host", "-lmptc_gb300", f"-Wl,-rpath,{LIBDIR}",
           f"-Wl,-rpath-link,{CUDA_LIB}"]
    p = subprocess.run(cmd, capture_output=True, text=True, timeout=120)
    assert p.returncode == 0, p.stderr[-3000:]
    env = dict(os.environ)
    env["LD_LIBRARY_PATH"] = os.pathsep.join(x for x in (CUDA_LIB, env.get("LD_LIBRARY_PATH", "")) if x)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=60, env=env)
    assert r.returncode == 0 and r.stdout.startswith("ok "), (r.returncode, r.stdout, r.stderr)
