"""Build recipe for the oracle's C restatement (gcc -O3 -fopenmp, shared
library in oracle/_build/).  Test infrastructure only."""
from __future__ import annotations

import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / "sf_oracle.c"
OUT_DIR = HERE / "_build"
LIB = OUT_DIR / "libsforacle.so"


def build(force: bool = False) -> Path:
    OUT_DIR.mkdir(exist_ok=True)
    if force or not LIB.exists() or LIB.stat().st_mtime < SRC.stat().st_mtime:
        cmd = ["gcc", "-O3", "-fopenmp", "-fPIC", "-shared", "-std=c11", str(SRC), "-o", str(LIB), "-lm"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"oracle build failed: {r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(force=True))
