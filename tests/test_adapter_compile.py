"""The C++ adapters (include/sf_pipeline.hpp) compile as drop-ins (CPU only:
compile, no link, no GPU).

* Against the harness's restatement of the host framework's interfaces.
* Against the reference's own include/spatial/pipeline_base.hpp, whenever
  SF_REFERENCE_ROOT names a checkout of the reference (its GPUPipeline header
  is self-contained); skipped otherwise.
"""
import os
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
HARNESS = ROOT / "tests" / "cpp" / "adapter_harness.cpp"


def _nvcc():
    cand = os.environ.get("NVCC") or "/usr/local/cuda/bin/nvcc"
    if Path(cand).exists():
        return cand
    return shutil.which("nvcc")


def _compile(extra, tmp_path):
    nvcc = _nvcc()
    if nvcc is None:
        pytest.skip("nvcc not available")
    cmd = [nvcc, "-std=c++17", "-c", "-I", str(ROOT / "include"), *extra, str(HARNESS), "-o",
           str(tmp_path / "harness.o")]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr


def test_adapters_compile_against_restated_interfaces(tmp_path):
    _compile([], tmp_path)


def test_adapters_compile_against_reference_pipeline_base(tmp_path):
    ref = os.environ.get("SF_REFERENCE_ROOT")
    if not ref or not (Path(ref) / "include" / "spatial" / "pipeline_base.hpp").exists():
        pytest.skip("SF_REFERENCE_ROOT does not name a reference checkout")
    _compile(["-DSF_REFERENCE_PIPELINE_BASE", "-I", str(Path(ref) / "include")], tmp_path)
