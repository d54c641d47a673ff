"""Generate golden vectors from the reference's own Python implementation.

Run where a reference checkout exists, with its path in SF_REFERENCE_ROOT:

    SF_REFERENCE_ROOT=/path/to/cuda-spatial-filtering python tests/golden/make_golden.py

It imports ``scripts/adaptive_detection_reference.py`` from the reference
(detect_k, build_null_projection, build_shrink_projection,
apply_projection_to_weights, beamform; lines 11-77) and records its outputs on
seeded inputs into ``adaptive_reference_golden.npz``.  The GPU machine never reads
the reference: tests only load the committed ``.npz``.
"""
from __future__ import annotations

import importlib.util
import os
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent


def load_reference_module():
    if not os.environ.get("SF_REFERENCE_ROOT"):
        raise SystemExit("set SF_REFERENCE_ROOT to the reference checkout")
    root = Path(os.environ["SF_REFERENCE_ROOT"])
    path = root / "scripts" / "adaptive_detection_reference.py"
    spec = importlib.util.spec_from_file_location("adaptive_detection_reference", path)
    mod = importlib.util.module_from_spec(spec)
    sys.modules["adaptive_detection_reference"] = mod
    spec.loader.exec_module(mod)
    return mod


def main() -> int:
    ref = load_reference_module()
    rng = np.random.Generator(np.random.PCG64(20241203))
    out: dict[str, np.ndarray] = {}

    # 1. The reference's own known-answer self tests (adaptive_detection_reference.py:86-132)
    results = ref.run_self_tests()
    out["selftest_names"] = np.array([r.name for r in results])
    out["selftest_passed"] = np.array([r.passed for r in results])

    # 2. detect_k on eigenvalue spectra: noise-like spectra with 0..4 strong modes,
    #    several deltas, including exact-threshold ties.
    spectra = []
    deltas = []
    ks = []
    for case in range(64):
        n = int(rng.choice([4, 16, 36, 64]))
        noise = np.sort(rng.gamma(20.0, 1.0 / 20.0, size=n))
        nsig = int(rng.integers(0, 5))
        vals = noise.copy()
        if nsig:
            vals[n - nsig:] += rng.uniform(5.0, 300.0, size=nsig)
        vals = np.sort(vals).astype(np.float32)
        for delta in (0.5, 0.8416, 3.0, 10.0):
            spectra.append(np.pad(vals, (0, 64 - n), constant_values=np.nan))
            deltas.append(delta)
            ks.append(ref.detect_k(vals.astype(np.float64), delta))
    out["detect_spectra"] = np.array(spectra, dtype=np.float32)
    out["detect_delta"] = np.array(deltas, dtype=np.float64)
    out["detect_k"] = np.array(ks, dtype=np.int32)

    # 3. Null / shrink projections, weight projection and beamforming on random
    #    Hermitian eigen-systems.
    n, nb, nt = 24, 3, 32
    cases_v, cases_l, cases_k = [], [], []
    null_p, shrink_p, w_in, w_null, x_in, y_null, y_orig = [], [], [], [], [], [], []
    for case in range(6):
        a = rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))
        h = a @ a.conj().T
        lam, v = np.linalg.eigh(h)
        k = case % 5
        cases_v.append(v)
        cases_l.append(lam)
        cases_k.append(k)
        pn = ref.build_null_projection(v, lam, k)
        ps = ref.build_shrink_projection(v, lam, k)
        w = rng.normal(size=(nb, n)) + 1j * rng.normal(size=(nb, n))
        x = rng.normal(size=(n, nt)) + 1j * rng.normal(size=(n, nt))
        wp = ref.apply_projection_to_weights(w, pn)
        null_p.append(pn)
        shrink_p.append(ps)
        w_in.append(w)
        w_null.append(wp)
        x_in.append(x)
        y_null.append(ref.beamform(x, wp))
        y_orig.append(ref.beamform(x, w))
    out["proj_evecs"] = np.array(cases_v)
    out["proj_evals"] = np.array(cases_l)
    out["proj_k"] = np.array(cases_k, dtype=np.int32)
    out["proj_null"] = np.array(null_p)
    out["proj_shrink"] = np.array(shrink_p)
    out["proj_weights"] = np.array(w_in)
    out["proj_weights_null"] = np.array(w_null)
    out["proj_samples"] = np.array(x_in)
    out["proj_beam_null"] = np.array(y_null)
    out["proj_beam_orig"] = np.array(y_orig)

    np.savez_compressed(HERE / "adaptive_reference_golden.npz", **out)
    print("wrote", HERE / "adaptive_reference_golden.npz")
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
