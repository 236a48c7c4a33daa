"""Build recipe for oracle/_ref: the reference's own CUDA kernels, compiled from
the reference's sources where they lie, as device-only modules.

TEST INFRASTRUCTURE ONLY.  The reference's GPU path has two hand-written CUDA
files (cunusht/c/pointing.cu, cunusht/c/doubling.cu; built by its CMake with
nanobind, cunusht/c/CMakeLists.txt).  Neither CMake nor nanobind is used
here: each file is compiled on its own by nvcc into a cubin for sm_103a, with
oracle/ref_stub standing in for the nanobind headers.  A cubin holds only
device code, so the same file runs on any host architecture; the harness
(oracle/ref_kernels.py) loads it through the CUDA driver API and launches the
reference's kernels exactly as its host wrappers do.

Outputs go to oracle/_ref/ only (git-ignored; it travels with the working
tree).  When the reference sources are absent (the GPU machine), the prebuilt
cubins are used as they are.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
STUB = os.path.join(HERE, "ref_stub")
REF_SRC = "/root/reference/cunusht/c"
MODULES = ("pointing", "doubling")


def cubin_path(name: str) -> str:
    return os.path.join(OUT, name + ".cubin")


def _nvcc() -> str:
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def build_ref(force: bool = False, verbose: bool = False) -> list[str]:
    """Compile the reference kernels into oracle/_ref/<name>.cubin when the
    reference sources are present; return the cubins that exist afterwards."""
    have_src = os.path.isdir(REF_SRC)
    os.makedirs(OUT, exist_ok=True)
    built = []
    for name in MODULES:
        src = os.path.join(REF_SRC, name + ".cu")
        dst = cubin_path(name)
        if have_src and os.path.exists(src):
            stale = force or not os.path.exists(dst) or os.path.getmtime(src) > os.path.getmtime(dst)
            if stale:
                cmd = [_nvcc(), "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17",
                       "-w", "-I", STUB, "-I", REF_SRC, src, "-o", dst]
                r = subprocess.run(cmd, capture_output=True, text=True)
                if verbose or r.returncode != 0:
                    sys.stderr.write(r.stdout + r.stderr)
                if r.returncode != 0:
                    raise RuntimeError("nvcc failed on the reference source: " + " ".join(cmd))
        if os.path.exists(dst):
            built.append(dst)
    return built


if __name__ == "__main__":
    for p in build_ref(force="--force" in sys.argv, verbose=True):
        print(p)
