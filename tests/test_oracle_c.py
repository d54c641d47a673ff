"""The C restatement agrees with the numpy oracle (CPU only)."""
import numpy as np
import pytest

import sf_oracle as orc

sfc = pytest.importorskip("sf_oracle_c")


@pytest.mark.parametrize("shrink,k_rule", [(False, 0), (True, 0), (False, 1), (False, 2)])
def test_c_chain_matches_numpy_oracle(shrink, k_rule):
    sh = orc.Shape(3, 4, 16, 12, 3, 4, 2)
    samples, scales, _ = orc.synth_inputs(sh, seed=3, n_interferers=2, frac_channels=0.7)
    w = orc.synth_weights(sh)
    tau = np.linspace(-5, 5, sh.R)
    d = orc.receiver_factors(sh, phasors=orc.fine_delay_phasors(sh, tau, 0.0, 781250.0, 64))
    delays = [0, 3, -2, 16]
    off = orc.sample_offsets(sh, delays)
    fixed = np.array([2, 1, 0])
    delta = {0: 0.0, 1: 3.0, 2: 10.0}[k_rule]
    ref = orc.adaptive_chain(sh, samples, scales, w, k_fixed=fixed, shrink=shrink, delays=delays, d=d,
                             detect=(k_rule == 1), delta=delta,
                             k_rule=(lambda lam: orc.detect_k_noise_floor(lam, 10.0)) if k_rule == 2 else None)
    got = sfc.adaptive_chain(sh, samples, scales, off, w.astype(np.float32), d, fixed_k=fixed,
                             k_rule=k_rule, delta=delta, shrink=shrink, nthreads=2)
    assert np.array_equal(got["vis"], ref["vis"])
    assert np.allclose(got["evals"], ref["evals"], atol=1e-9 * np.abs(ref["evals"]).max())
    assert np.array_equal(got["counts"], ref["counts"])
    assert np.allclose(got["beams"], ref["beams"], atol=1e-7 * np.abs(ref["beams"]).max())


def test_c_correlate_exact_extremes():
    sh = orc.Shape(2, 2, 8, 6, 3, 3, 1)
    rng = np.random.default_rng(0)
    samples = rng.integers(-128, 128, size=sh.samples_shape(), dtype=np.int8)
    scales = rng.integers(-300, 300, size=sh.scales_shape()).astype(np.int16)
    off = orc.sample_offsets(sh, [2, -8])
    re, im = orc.aligned_samples(sh, samples, scales, off)
    assert np.array_equal(sfc.correlate(sh, samples, scales, off, nthreads=2), orc.correlate(sh, re, im))
