"""In-tree build of the native engine: ``vmps_gb300/libvmps_gb300.so``.

Compiles the CUDA kernels for sm_103a only and the host C++ with g++, in
parallel, then links one shared library with the CUDA runtime.  No cmake, no
torch extension machinery: the library exposes a plain C ABI
(``include/vmps_gb300.h``) and is loaded with ctypes.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libvmps_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _cuda_home() -> str:
    for cand in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if cand and os.path.exists(os.path.join(cand, "bin", "nvcc")):
            return cand
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build vmps_gb300")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout)


def _sources():
    cu = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    cpp = sorted(f for f in os.listdir(CSRC) if f.endswith(".cpp"))
    return cu, cpp


def _stale(objs: list[str]) -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps.append(os.path.join(ROOT, "include", "vmps_gb300.h"))
    deps.append(os.path.abspath(__file__))
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    cu, cpp = _sources()
    os.makedirs(OUT_DIR, exist_ok=True)
    objs = [os.path.join(OUT_DIR, f + ".o") for f in cu + cpp]
    if not force and not _stale(objs):
        return LIB
    inc = ["-I", CSRC, "-I", os.path.join(ROOT, "include")]
    jobs = []
    for f in cu:
        jobs.append([nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                     "--expt-relaxed-constexpr", *inc, "-c", os.path.join(CSRC, f),
                     "-o", os.path.join(OUT_DIR, f + ".o")])
    for f in cpp:
        jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-Wall", "-Wno-unused-function",
                     "-I", os.path.join(cuda, "include"), *inc, "-c", os.path.join(CSRC, f),
                     "-o", os.path.join(OUT_DIR, f + ".o")])
    with ThreadPoolExecutor(max_workers=max(2, len(jobs))) as ex:
        for fut in [ex.submit(_run, j) for j in jobs]:
            fut.result()
    tmp = LIB + ".tmp"
    _run([nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart", "-lcublas", "-lcusolver", "-ldl", "-lpthread"])
    os.replace(tmp, LIB)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
