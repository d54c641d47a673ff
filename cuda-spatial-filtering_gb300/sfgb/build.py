"""Build recipe for the sm_103a library (no cmake): nvcc compiles each
translation unit in parallel, then links one shared library in-tree."""
from __future__ import annotations

import os
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = ROOT / "csrc"
BUILD = ROOT / "_build"
LIB = PKG / "libsfgb.so"
SOURCES = ["sf_corr.cu", "sf_eig.cu", "sf_eig_topk.cu", "sf_beam.cu", "sf_capi.cu", "sf_noalloc.cu",
           "sf_spectra.cu", "sf_steering.cu", "sf_batch.cu", "sf_batch_capi.cu", "sf_mlp.cu", "sf_proposer.cu", "sf_refine.cu",
           "sf_eig_small.cu"]
HEADERS = ["sf_common.cuh", "sf_plan.cuh", "sf_batch.cuh"]
NVCC_FLAGS = [
    "-gencode", "arch=compute_103a,code=sm_103a",
    "-O3", "-lineinfo", "-std=c++17",
    "-Xcompiler", "-fPIC",
]


def _nvcc() -> str:
    cand = os.environ.get("NVCC") or "/usr/local/cuda/bin/nvcc"
    return cand if Path(cand).exists() else "nvcc"


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    hdrs = [CSRC / h for h in HEADERS] + [ROOT.parent / "include" / "sf_capi.h"]
    objs = []
    jobs = []
    for src in SOURCES:
        obj = BUILD / (Path(src).stem + ".o")
        objs.append(obj)
        if force or _stale(obj, [CSRC / src] + hdrs):
            cmd = [_nvcc(), *NVCC_FLAGS, "-c", str(CSRC / src), "-o", str(obj)]
            jobs.append(cmd)

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose:
            print(r.stdout, r.stderr)

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        list(ex.map(run, jobs))
    if force or jobs or _stale(LIB, objs):
        cmd = [_nvcc(), "-shared", "-o", str(LIB), *map(str, objs), "-lcudart"]
        run(cmd)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
