"""Builds the sm_103a shared library ``voxurf_gb300/lib/libvoxurf_gb300.so``.

One ``nvcc -c`` per translation unit, run in parallel, then one ``nvcc
-shared`` link.  No CMake, no torch extension machinery: the library is a
plain C ABI (``include/voxurf_gb300.h``) loaded with ctypes.  A rebuild is
skipped when the library is newer than every source and header.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
REPO_DIR = os.path.dirname(PKG_DIR)
CSRC_DIR = os.path.join(PKG_DIR, "csrc")
INCLUDE_DIR = os.path.join(REPO_DIR, "include")
LIB_DIR = os.path.join(PKG_DIR, "lib")
BUILD_DIR = os.path.join(PKG_DIR, "_build")
LIB_NAME = "libvoxurf_gb300.so"
LIB_PATH = os.path.join(LIB_DIR, LIB_NAME)

ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
    "-Xcompiler", "-fPIC", "-Xcompiler", "-O3",
    "-Xptxas", "-warn-spills",
]


def nvcc_path() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the voxurf_gb300 CUDA library cannot be built")


def sources() -> list[str]:
    return sorted(os.path.join(CSRC_DIR, f) for f in os.listdir(CSRC_DIR) if f.endswith(".cu"))


def _deps() -> list[str]:
    hdrs = [os.path.join(CSRC_DIR, f) for f in os.listdir(CSRC_DIR) if f.endswith((".cuh", ".h"))]
    hdrs += [os.path.join(INCLUDE_DIR, f) for f in os.listdir(INCLUDE_DIR) if f.endswith(".h")]
    return sources() + hdrs + [os.path.abspath(__file__)]


def is_stale() -> bool:
    if not os.path.exists(LIB_PATH):
        return True
    t = os.path.getmtime(LIB_PATH)
    return any(os.path.getmtime(p) > t for p in _deps())


def _compile(nvcc: str, src: str, extra: list[str]) -> tuple[str, str]:
    obj = os.path.join(BUILD_DIR, os.path.basename(src)[:-3] + ".o")
    cmd = [nvcc, *ARCH_FLAGS, *NVCC_FLAGS, *extra, "-I", INCLUDE_DIR, "-I", CSRC_DIR, "-c", src, "-o", obj]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed on {os.path.basename(src)}:\n{' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    return obj, res.stderr


def build(force: bool = False, verbose: bool = False, jobs: int | None = None, extra_flags: list[str] | None = None) -> str:
    """Compiles every ``csrc/*.cu`` for sm_103a and links the shared library.

    Returns the path of the library.  Raises RuntimeError on any failure.
    """
    if not force and not is_stale():
        return LIB_PATH
    nvcc = nvcc_path()
    os.makedirs(BUILD_DIR, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    extra = list(extra_flags or [])
    srcs = sources()
    jobs = jobs or min(len(srcs), max(1, os.cpu_count() or 1))
    objs = []
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        futs = {ex.submit(_compile, nvcc, s, extra): s for s in srcs}
        for f in cf.as_completed(futs):
            obj, log = f.result()
            objs.append(obj)
            if verbose and log.strip():
                print(f"[{os.path.basename(futs[f])}]\n{log}", file=sys.stderr)
    tmp = LIB_PATH + ".tmp"
    cmd = [nvcc, *ARCH_FLAGS, "-shared", "-Xcompiler", "-fPIC", *sorted(objs), "-o", tmp]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
