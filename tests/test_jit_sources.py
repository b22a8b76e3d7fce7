"""The kernels the drop-in headers generate for user functors (the
single-pass look-back scan and the one-launch in-order fold) compile with
NVRTC for sm_103a, with the options libbcx uses at run time -- checked on the
host, no GPU needed.  The program tests/cpp/jit_sources.cpp prints the
generated sources for scalar, user-function and struct element types."""
import ctypes
import glob
import os
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
SRC = ROOT / "tests" / "cpp" / "jit_sources.cpp"
OPTIONS = [b"--gpu-architecture=sm_103a", b"-std=c++17", b"-default-device"]


def _nvrtc():
    cands = []
    for home in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if home:
            cands += sorted(glob.glob(os.path.join(home, "lib64", "libnvrtc.so*")))
    for c in cands:
        try:
            return ctypes.CDLL(c)
        except OSError:
            continue
    return None


def _sources(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = tmp_path / "jit_sources"
    r = subprocess.run([cxx, "-std=c++17", "-O0", "-Wall", "-Werror", f"-I{ROOT / 'include'}", str(SRC), "-o",
                        str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
    parts = out.split("//@@ ")[1:]
    return [(p.split("\n", 1)[0].strip(), p.split("\n", 1)[1]) for p in parts]


def test_generated_kernels_compile_for_sm103a(tmp_path):
    nv = _nvrtc()
    if nv is None:
        pytest.skip("libnvrtc not found")
    srcs = _sources(tmp_path)
    assert len(srcs) >= 10
    for name, src in srcs:
        prog = ctypes.c_void_p()
        assert nv.nvrtcCreateProgram(ctypes.byref(prog), src.encode(), b"bcx_jit.cu", 0, None, None) == 0
        opts = (ctypes.c_char_p * len(OPTIONS))(*OPTIONS)
        rc = nv.nvrtcCompileProgram(prog, len(OPTIONS), opts)
        size = ctypes.c_size_t()
        nv.nvrtcGetProgramLogSize(prog, ctypes.byref(size))
        log = ctypes.create_string_buffer(size.value + 1)
        nv.nvrtcGetProgramLog(prog, log)
        nv.nvrtcDestroyProgram(ctypes.byref(prog))
        assert rc == 0, f"{name}:\n{log.value.decode()}\n{src[-3000:]}"
        assert name.encode() in src.encode()
