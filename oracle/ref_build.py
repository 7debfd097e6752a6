"""ORACLE — test infrastructure only (never imported by the product).

Build recipe for the reference's own CUDA kernels.  Each of the reference's
kernel files (lib/cuda/render_utils_kernel.cu, total_variation_kernel.cu,
adam_upd_kernel.cu, ub360_utils_kernel.cu) is compiled where it lies in the
reference checkout, unmodified, by nvcc into PTX for compute_103a under
``oracle/_ref/``.  The flags are the ones ``torch.utils.cpp_extension.load``
gives the reference's JIT build (lib/voxurf_fine.py:17-22, lib/grid.py:12-24:
PyTorch's common nvcc flags, C++17, nvcc's defaults otherwise, which include
``--fmad=true``), plus ``-include oracle/ref_compat.h`` so that the files'
``tensor.type()`` dispatch compiles against this PyTorch.

PTX (text) is what travels to the GPU machine: it carries no host code, so
it does not depend on the host architecture, and the CUDA driver there
compiles it for the GPU at load time (``oracle/ref_cuda.py``), as ptxas does
in the reference's own build.  Nothing here runs on the GPU machine, where
the reference checkout is absent: the GPU tests use the prebuilt files or
skip.

    VOXURF_REFERENCE=<reference checkout> python oracle/ref_build.py [--force]
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
import sysconfig

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_ref")
COMPAT = os.path.join(HERE, "ref_compat.h")
UNITS = ("render_utils", "total_variation", "adam_upd", "ub360_utils")
DEFAULT_REFERENCE = "/root/reference"


def reference_root() -> str | None:
    """The reference checkout (the directory holding lib/cuda), or None."""
    root = os.environ.get("VOXURF_REFERENCE", DEFAULT_REFERENCE)
    return root if os.path.isdir(os.path.join(root, "lib", "cuda")) else None


def ptx_path(unit: str) -> str:
    return os.path.join(OUT_DIR, unit + ".ptx")


def _flags() -> list[str]:
    import torch.utils.cpp_extension as ext

    inc = []
    for p in ext.include_paths():
        inc += ["-I", p]
    inc += ["-I", sysconfig.get_paths()["include"]]
    return ["-ptx", "-arch=compute_103a", "-std=c++17", *ext.COMMON_NVCC_FLAGS, "-include", COMPAT, *inc]


def _compile(nvcc: str, flags: list[str], src: str, out: str) -> None:
    tmp = out + ".tmp"
    res = subprocess.run([nvcc, *flags, src, "-o", tmp], capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{res.stderr[-4000:]}")
    os.replace(tmp, out)


def build(force: bool = False) -> list[str]:
    """Compiles the reference kernel files that are missing or stale.
    Returns the PTX paths, or [] when the reference checkout is absent."""
    root = reference_root()
    if root is None:
        return []
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    os.makedirs(OUT_DIR, exist_ok=True)
    jobs = []
    for u in UNITS:
        src = os.path.join(root, "lib", "cuda", u + "_kernel.cu")
        out = ptx_path(u)
        stale = force or not os.path.exists(out) or os.path.getmtime(out) < max(
            os.path.getmtime(src), os.path.getmtime(COMPAT), os.path.getmtime(os.path.abspath(__file__)))
        if stale:
            jobs.append((src, out))
    if jobs:
        flags = _flags()
        with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            for f in [ex.submit(_compile, nvcc, flags, s, o) for s, o in jobs]:
                f.result()
    return [ptx_path(u) for u in UNITS]


if __name__ == "__main__":
    paths = build(force="--force" in sys.argv)
    print("\n".join(paths) if paths else "reference checkout not found: nothing built")
