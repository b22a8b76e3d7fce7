"""The boost::compute drop-in headers: reference-style C++ callers compile
unchanged (apart from include paths) and, on a GPU, produce the reference's
known answers (tests/cpp/drop_in_test.cpp)."""
import os
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
SRC = ROOT / "tests" / "cpp" / "drop_in_test.cpp"
LIBDIR = ROOT / "compute_gb300"


def _compile(out: Path, link: bool) -> subprocess.CompletedProcess:
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    cmd = [cxx, "-std=c++17", "-O2", "-Wall", "-Werror", f"-I{ROOT / 'include'}", str(SRC), "-o", str(out)]
    if link:
        cmd += [f"-L{LIBDIR}", "-lbcx", f"-Wl,-rpath,{LIBDIR}"]
    else:
        cmd = cmd[:-2] + ["-c", "-o", str(out)]
    return subprocess.run(cmd, capture_output=True, text=True)


def test_headers_compile(tmp_path):
    r = _compile(tmp_path / "drop_in_test.o", link=False)
    assert r.returncode == 0, r.stderr


@pytest.mark.gpu
def test_drop_in_program_on_gpu(tmp_path, cuda):
    if not (LIBDIR / "libbcx.so").exists():
        pytest.fail("libbcx.so is not built")
    exe = tmp_path / "drop_in_test"
    r = _compile(exe, link=True)
    assert r.returncode == 0, r.stderr
    run = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600,
                         env=dict(os.environ, BOOST_COMPUTE_DEFAULT_DEVICE="0"))
    assert run.returncode == 0, run.stdout + run.stderr
    assert run.stdout.strip().endswith("OK (0 failures)"), run.stdout
