"""The oracle against the reference's own golden vectors (CPU only)."""
from pathlib import Path

import numpy as np
import pytest

import sf_oracle as orc
from case_checks import check_case, oracle_outputs, oracle_shape, _power
from reference_cases import build_cases

GOLDEN = Path(__file__).resolve().parent / "golden" / "adaptive_reference_golden.npz"
CASES = build_cases()


@pytest.mark.parametrize("case", CASES, ids=[c.name for c in CASES])
def test_oracle_reproduces_reference_test_goldens(case):
    out = oracle_outputs(case)
    check_case(case, out)


def test_oracle_shrink_rank_two_exceeds_null():
    case = next(c for c in CASES if c.name == "AdaptiveShrinkRankTwo")
    sh = oracle_shape(case)
    null = orc.adaptive_chain(sh, case.samples, case.scales, case.weights, k_fixed=[1])
    shrink = orc.adaptive_chain(sh, case.samples, case.scales, case.weights, k_fixed=[1], shrink=True)
    pn = _power(orc.half_output(null["beams"]).astype(np.float32))
    ps = _power(orc.half_output(shrink["beams"]).astype(np.float32))
    assert ps > pn + 1e-6


def test_reference_python_selftests_recorded_passing():
    g = np.load(GOLDEN)
    assert g["selftest_passed"].all(), g["selftest_names"]


def test_detect_k_matches_reference_python():
    g = np.load(GOLDEN)
    for spec, delta, k in zip(g["detect_spectra"], g["detect_delta"], g["detect_k"]):
        vals = spec[~np.isnan(spec)]
        assert orc.detect_k_f64(vals, delta) == k
        # the device rule runs in float32; away from exact ties it agrees
        assert orc.detect_k_f32(vals, delta) == k


def test_projections_weights_beams_match_reference_python():
    g = np.load(GOLDEN)
    for i in range(len(g["proj_k"])):
        v, lam, k = g["proj_evecs"][i], g["proj_evals"][i], int(g["proj_k"][i])
        pn = orc.null_projection(v, k)
        ps = orc.shrink_projection(v, lam, k)
        assert np.allclose(pn, g["proj_null"][i], atol=1e-12)
        assert np.allclose(ps, g["proj_shrink"][i], atol=1e-9)
        w = g["proj_weights"][i]
        assert np.allclose(w @ pn, g["proj_weights_null"][i], atol=1e-12)
        x = g["proj_samples"][i]
        assert np.allclose((w @ pn) @ x, g["proj_beam_null"][i], atol=1e-10)
        assert np.allclose(w @ x, g["proj_beam_orig"][i], atol=1e-10)


def test_reference_selftest_vectors_directly():
    # adaptive_detection_reference.py:86-132, restated
    assert orc.detect_k_f64([0.0, 0.0, 100.0, 100.0], 0.8416) == 0
    assert orc.detect_k_f64(np.zeros(4), 0.5) == 0
    assert orc.detect_k_f64([0.0, 0.0, 0.0, 100.0], 0.5) == 1
    assert orc.detect_k_f64([0.0, 0.0, 100.0, 100.0], 0.5) == 2
    for fn in (orc.detect_k_f32,):
        assert fn([0.0, 0.0, 0.0, 100.0], 0.5) == 1
        assert fn([0.0, 0.0, 100.0, 100.0], 0.5) == 2
    eye = np.eye(4, dtype=complex)
    assert np.allclose(orc.null_projection(eye, 1), np.diag([1, 1, 1, 0]))
    assert np.allclose(orc.shrink_projection(eye, np.array([1.0, 2.0, 3.0, 12.0]), 1),
                       np.diag([1, 1, 1, 1 / 6]))


def test_conjugation_convention_complex_phase_kat():
    # tests/test_beamforming.cpp:49-79: receiver 0 = [1+1j, 2+2j], receiver 1 =
    # [2+2j, 1j] -> baseline(0,1) = sum x0 conj(x1) = 6-2j, autos 10 and 9.
    sh = orc.Shape(1, 1, 2, 2, 2, 1, 1)
    s = np.zeros(sh.samples_shape(), np.int8)
    x0 = [(1, 1), (2, 2)]
    x1 = [(2, 2), (0, 1)]
    for t in range(2):
        for j in range(3):
            s[0, j, 0, t, 0, :, :] = x0[t]
            s[0, j, 0, t, 1, :, :] = x1[t]
    sc = np.ones(sh.scales_shape(), np.int16)
    re, im = orc.aligned_samples(sh, s, sc, orc.sample_offsets(sh))
    vis = orc.correlate(sh, re, im)
    assert tuple(vis[0, 0, 0, 0]) == (10, 0)
    assert tuple(vis[0, 1, 0, 0]) == (6, -2)
    assert tuple(vis[0, 2, 0, 0]) == (9, 0)


def test_correlate_matches_bruteforce_loops():
    sh = orc.Shape(2, 2, 4, 6, 3, 2, 1)
    rng = np.random.default_rng(3)
    s = rng.integers(-128, 128, size=sh.samples_shape(), dtype=np.int8)
    sc = rng.integers(-3, 4, size=sh.scales_shape()).astype(np.int16)
    delays = [1, -2]
    off = orc.sample_offsets(sh, delays)
    re, im = orc.aligned_samples(sh, s, sc, off)
    vis = orc.correlate(sh, re, im)
    for c in range(sh.C):
        for j in range(sh.R):
            for i in range(j + 1):
                b = orc.baseline_index(i, j)
                for p in range(2):
                    for q in range(2):
                        acc = 0
                        for t in range(sh.T):
                            f_i, n_i = divmod(i, sh.Rpp)
                            f_j, n_j = divmod(j, sh.Rpp)
                            qi, qj = t + off[f_i], t + off[f_j]
                            xi = complex(*s[c, qi // sh.Tp, f_i, qi % sh.Tp, n_i, p]) * int(sc[c, qi // sh.Tp, i, p])
                            xj = complex(*s[c, qj // sh.Tp, f_j, qj % sh.Tp, n_j, q]) * int(sc[c, qj // sh.Tp, j, q])
                            acc += xi * xj.conjugate()
                        assert vis[c, b, p, q, 0] == int(acc.real) and vis[c, b, p, q, 1] == int(acc.imag)


def test_eig_oracle_residual_and_orthogonality():
    sh = orc.Shape(2, 4, 64, 36, 9, 4, 2)
    s, sc, _ = orc.synth_inputs(sh, seed=0, n_interferers=2, frac_channels=0.5)
    w = orc.synth_weights(sh)
    r = orc.adaptive_chain(sh, s, sc, w, k_fixed=[1, 1])
    # with K = 1 the un-whitened unit vector u gives (I - u u^H) u = 0, so the
    # projected weights null it exactly (for K > 1 the un-whitened columns are
    # not mutually orthogonal and P is not an orthogonal projector, as in the
    # reference)
    for c in range(sh.C):
        for p in range(2):
            u = r["evecs"][c, p].T[:, -1:]
            wp = r["w_eff"][c, p, sh.B:]
            assert np.max(np.abs(wp @ u)) < 1e-9
    r2 = orc.adaptive_chain(sh, s, sc, w, k_fixed=[2, 2])
    for c in range(sh.C):
        for p in range(2):
            u = r2["evecs"][c, p].T[:, -2:]
            assert np.allclose(r2["proj"][c, p], np.eye(sh.R) - u @ u.conj().T, atol=1e-12)
