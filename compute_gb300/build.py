"""Builds libbcx.so (the sm_103a kernels and the C ABI) in-tree.

Every ``.cu``/``.cpp`` file under ``compute_gb300/csrc`` is compiled to an
object in parallel with nvcc for ``sm_103a`` only, then linked into
``compute_gb300/libbcx.so`` (static CUDA runtime, NVRTC for the JIT path).
Objects are rebuilt only when a source or header is newer than them.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libbcx.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found (set NVCC or install the CUDA toolkit)")


def cuda_home() -> Path:
    return Path(nvcc()).resolve().parent.parent


def _flags() -> list[str]:
    return ARCH + [
        "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
        "-Xcompiler", "-fPIC", "-Xcompiler", "-O3",
        f"-I{ROOT / 'include'}", f"-I{CSRC}",
    ]


def _headers() -> list[Path]:
    return list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list((ROOT / "include").glob("*.h"))


def _compile(src: Path, obj: Path, extra: list[str], verbose: bool) -> str:
    cmd = [nvcc()] + _flags() + extra + ["-c", str(src), "-o", str(obj)]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src.name}:\n{r.stdout}\n{r.stderr}")
    return r.stderr


def build(verbose: bool = False, ptxas_info: bool = False, jobs: int | None = None) -> Path:
    BUILD.mkdir(exist_ok=True)
    sources = sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")))
    hdr_mtime = max((h.stat().st_mtime for h in _headers()), default=0.0)
    extra = ["-Xptxas", "-v"] if ptxas_info else []
    todo = []
    objs = []
    for src in sources:
        obj = BUILD / (src.name + ".o")
        objs.append(obj)
        if ptxas_info or not obj.exists() or obj.stat().st_mtime < max(src.stat().st_mtime, hdr_mtime):
            todo.append((src, obj))
    logs = {}
    if todo:
        n = jobs or min(len(todo), os.cpu_count() or 4)
        with cf.ThreadPoolExecutor(max_workers=n) as ex:
            futs = {ex.submit(_compile, s, o, extra, verbose): s for s, o in todo}
            for f in cf.as_completed(futs):
                logs[futs[f].name] = f.result()
    if ptxas_info:
        for name, log in sorted(logs.items()):
            print(f"== {name}\n{log}")
    lib_mtime = LIB.stat().st_mtime if LIB.exists() else 0.0
    if todo or lib_mtime < max(o.stat().st_mtime for o in objs):
        cuda_lib = cuda_home() / "lib64"
        cmd = [nvcc()] + ARCH + ["-shared", "-cudart", "static", "-o", str(LIB)] + [str(o) for o in objs] + [
            f"-L{cuda_lib}", "-lnvrtc", "-Xlinker", f"-rpath,{cuda_lib}"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, ptxas_info="--ptxas" in sys.argv)
    print(LIB)
