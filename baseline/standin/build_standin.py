"""Build recipe for the library stand-in (benchmark comparator only): one
nvcc call linking cuBLAS and cuSOLVER into baseline/standin/libsf_standin.so."""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / "sf_standin.cu"
LIB = HERE / "libsf_standin.so"


def build(force: bool = False) -> Path:
    if not force and LIB.exists() and LIB.stat().st_mtime >= SRC.stat().st_mtime:
        return LIB
    nvcc = os.environ.get("NVCC") or "/usr/local/cuda/bin/nvcc"
    if not Path(nvcc).exists():
        nvcc = "nvcc"
    cmd = [nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
           "-shared", str(SRC), "-o", str(LIB), "-lcublas", "-lcusolver", "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"stand-in build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(force=True))
