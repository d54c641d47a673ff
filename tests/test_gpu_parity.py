"""CUDA path vs the oracle and the reference's golden values (GPU only).

Integer work (visibilities) must be bit-exact.  Floating-point tolerances:
  beams       fp16 output of an fp32 sum: |y - y_ref| <= 2^-9 |y_ref| + 2^-6 (abs)
  eigenvalues |lambda - lambda_lapack| <= 2e-5 ||A||_2  (fp32 Jacobi vs FP64 LAPACK)
  residual    ||A v - lambda v|| <= 1e-4 ||A||_2, orthogonality ||V^H V - I|| <= 1e-4
  projector   ||P - P_ref||_max <= 2e-3 when the nulled eigenvalues are separated
"""
import numpy as np
import pytest
import torch

import sf_oracle as orc
import sfgb
from case_checks import check_case, oracle_outputs, oracle_shape, _power
from reference_cases import build_cases

pytestmark = pytest.mark.gpu

CASES = build_cases()


def _dev(x, dtype):
    return torch.as_tensor(np.ascontiguousarray(x)).to(device="cuda").view(dtype)


def gpu_case_outputs(case):
    C, F, Tp, R, Rpp, P, B = case.shape
    out = sfgb.SingleHostMemoryOutput()
    if case.path == "corr_beam":
        pipe = sfgb.LambdaCorrBeamOnlyGPUPipeline(case.shape, case.weights)
    elif case.path == "lambda_gpu":
        pipe = sfgb.LambdaGPUPipeline(case.shape, case.weights)
    else:
        a = case.adaptive
        pipe = sfgb.LambdaAdaptiveBeamformedSpectraPipeline(
            case.shape, case.weights, nr_signal_eigenvectors={0: a.get("k", 0)},
            shrink_eigenvalues=a.get("shrink", False), detect_signal_eigenmodes=a.get("detect", False),
            detection_threshold_delta=a.get("delta", 3.0))
    pipe.set_output(out)
    if case.delays is not None:
        pipe.set_subpacket_delays(case.delays)
    if case.gains is not None:
        pipe.set_antenna_gains(case.gains)
    pipe.execute_pipeline(sfgb.PacketData(case.samples, case.scales))
    pipe.dump_visibilities()
    rc, bits = pipe.plan.status()
    assert rc == 0 and bits == 0, f"device status bits 0x{bits:x}"
    res = {"beam_half": out.beam_data.astype(np.float32), "vis": out.visibilities}
    if out.eigenvalues is not None:
        res["evals"] = out.eigenvalues
        ev = out.eigenvectors
        res["evecs"] = ev[..., 0] + 1j * ev[..., 1]
    if out.nulled_eigenmode_counts is not None:
        res["counts"] = out.nulled_eigenmode_counts
    pipe.plan.close()
    return res


@pytest.mark.parametrize("case", CASES, ids=[c.name for c in CASES])
def test_reference_goldens_through_the_c_abi(case):
    out = gpu_case_outputs(case)
    check_case(case, out)
    ref = oracle_outputs(case)
    assert np.array_equal(out["vis"], ref["vis"]), f"{case.name}: float visibilities differ from oracle"


def test_shrink_rank_two_exceeds_null_on_gpu():
    case = next(c for c in CASES if c.name == "AdaptiveShrinkRankTwo")
    import copy
    null_case = copy.copy(case)
    null_case.adaptive = {"k": 1, "shrink": False}
    pn = _power(gpu_case_outputs(null_case)["beam_half"])
    ps = _power(gpu_case_outputs(case)["beam_half"])
    assert ps > pn + 1e-6


# --------------------------------------------------------------------------
# Correlator: bit-exact int32 against the exact-integer oracle
# --------------------------------------------------------------------------
def _correlate_gpu(sh, samples, scales, window, delays=None):
    plan = sfgb.Plan(sh.C, sh.F, sh.Tp, sh.R, sh.Rpp, sh.P, sh.B)
    if delays is not None:
        plan.set_subpacket_delays(delays)
    s = _dev(samples, torch.int8)
    sc = _dev(scales, torch.int16)
    vis = torch.full(plan.vis_shape(), -7, dtype=torch.int32, device="cuda")
    plan.correlate(s, sc, window, vis)
    torch.cuda.synchronize()
    rc, bits = plan.status()
    assert rc == 0 and bits == 0, f"device status 0x{bits:x}"
    plan.close()
    return vis.cpu().numpy()


@pytest.mark.parametrize("R,F,Tp,P,window,delays", [
    (36, 4, 64, 4, sfgb.SF_WINDOW_ALIGNED, [0, 5, -7, 64]),
    (36, 4, 64, 4, sfgb.SF_WINDOW_PACKET, None),
    (4, 1, 8, 1, sfgb.SF_WINDOW_ALIGNED, [0]),
    (6, 3, 8, 3, sfgb.SF_WINDOW_ALIGNED, [0, 3, -4]),
    (16, 2, 64, 2, sfgb.SF_WINDOW_ALIGNED, [-64, 17]),
    (32, 4, 32, 5, sfgb.SF_WINDOW_ALIGNED, [1, 2, 3, -32]),
    (40, 4, 64, 3, sfgb.SF_WINDOW_ALIGNED, [0, 0, 1, 1]),
    (48, 6, 16, 9, sfgb.SF_WINDOW_ALIGNED, [0, -16, 16, 5, -5, 9]),
    # 9.4 KB packets: the ring holds one stage's packets but not two, so each
    # stage is closed before the next one's packets are acquired
    (48, 4, 48, 9, sfgb.SF_WINDOW_ALIGNED, [0, 12, -48, 48]),
])
def test_correlator_bit_exact_random(R, F, Tp, P, window, delays):
    sh = orc.Shape(3, F, Tp, R, R // F, P, 1)
    rng = np.random.default_rng(R * 1000 + Tp)
    samples = rng.integers(-128, 128, size=sh.samples_shape(), dtype=np.int8)
    scales = rng.integers(-1, 2, size=sh.scales_shape()).astype(np.int16)
    off = orc.sample_offsets(sh, delays, mode="aligned" if window == sfgb.SF_WINDOW_ALIGNED else "packet")
    re, im = orc.aligned_samples(sh, samples, scales, off)
    ref = orc.correlate(sh, re, im)
    got = _correlate_gpu(sh, samples, scales, window, delays)
    assert np.array_equal(got, ref)


def test_correlator_exact_at_full_scale():
    """Every sample at -128/127 over 4096 samples: partial sums reach 2^27, so
    exactness relies on the 1024-sample fp32 chunks drained into int32."""
    sh = orc.Shape(2, 4, 64, 36, 9, 64, 1)
    rng = np.random.default_rng(7)
    samples = np.where(rng.random(sh.samples_shape()) < 0.5, -128, 127).astype(np.int8)
    scales = np.ones(sh.scales_shape(), np.int16)
    re, im = orc.aligned_samples(sh, samples, scales, orc.sample_offsets(sh))
    ref = orc.correlate(sh, re, im)
    assert np.abs(ref).max() > 2 ** 24
    got = _correlate_gpu(sh, samples, scales, sfgb.SF_WINDOW_ALIGNED, [0, 0, 0, 0])
    assert np.array_equal(got, ref)


def test_correlator_many_channels_persistent_loop():
    """More channels than SMs: every CTA walks several channels."""
    sh = orc.Shape(400, 1, 16, 8, 8, 2, 1)
    rng = np.random.default_rng(11)
    samples = rng.integers(-128, 128, size=sh.samples_shape(), dtype=np.int8)
    scales = rng.integers(0, 3, size=sh.scales_shape()).astype(np.int16)
    re, im = orc.aligned_samples(sh, samples, scales, orc.sample_offsets(sh, [3]))
    ref = orc.correlate(sh, re, im)
    got = _correlate_gpu(sh, samples, scales, sfgb.SF_WINDOW_ALIGNED, [3])
    assert np.array_equal(got, ref)


# --------------------------------------------------------------------------
# Eigensolver, projector, beams on LAMBDA-shaped synthetic data
# --------------------------------------------------------------------------
def _run_adaptive_gpu(sh, samples, scales, weights, k_rule, delta, shrink=False, fixed=None,
                      gains=None, fine=None, want_evecs=True):
    plan = sfgb.Plan(sh.C, sh.F, sh.Tp, sh.R, sh.Rpp, sh.P, sh.B)
    plan.set_weights(weights)
    if fixed is not None:
        plan.set_fixed_counts(fixed)
    if gains is not None:
        plan.set_antenna_gains(gains)
    if fine is not None:
        plan.set_fine_delays(*fine)
    s = _dev(samples, torch.int8)
    sc = _dev(scales, torch.int16)
    vis = torch.empty(plan.vis_shape(), dtype=torch.int32, device="cuda")
    ev = torch.empty((sh.C, 2, sh.R), dtype=torch.float32, device="cuda")
    vec = torch.empty((sh.C, 2, sh.R, sh.R, 2), dtype=torch.float32, device="cuda")
    cnt = torch.empty((sh.C, 2), dtype=torch.int32, device="cuda")
    beams = torch.empty(plan.beams_shape(2), dtype=torch.float16, device="cuda")
    plan.run_adaptive(s, sc, k_rule, delta, shrink, vis, ev, vec if want_evecs else None, cnt, beams)
    torch.cuda.synchronize()
    rc, bits = plan.status()
    assert rc == 0 and bits == 0, f"device status 0x{bits:x}"
    out = {"vis": vis.cpu().numpy(), "evals": ev.cpu().numpy(), "counts": cnt.cpu().numpy(),
           "beams": beams.cpu().numpy().astype(np.float32)}
    if want_evecs:
        v = vec.cpu().numpy()
        out["evecs"] = v[..., 0] + 1j * v[..., 1]
    plan.close()
    return out


@pytest.fixture(scope="module")
def lambda_cfg():
    sh = orc.Shape(16, 4, 64, 36, 9, 16, 4)
    samples, scales, rfi = orc.synth_inputs(sh, seed=0, n_interferers=2, frac_channels=0.5)
    weights = orc.synth_weights(sh)
    return sh, samples, scales, weights, rfi


def test_eig_against_lapack(lambda_cfg):
    sh, samples, scales, weights, rfi = lambda_cfg
    got = _run_adaptive_gpu(sh, samples, scales, weights, sfgb.SF_K_FIXED, 0.0, fixed=np.full(sh.C, 2))
    ref = orc.adaptive_chain(sh, samples, scales, weights, k_fixed=np.full(sh.C, 2))
    assert np.array_equal(got["vis"], ref["vis"])
    vc = orc.scaled_visibilities(sh, ref["vis"], orc.receiver_factors(sh))
    for p in range(2):
        m = orc.unpack_hermitian(sh, vc, p, p)
        for c in range(sh.C):
            a, _ = orc.whiten(m[c])
            norm = np.linalg.norm(a, 2)
            lam = got["evals"][c, p].astype(np.float64)
            assert np.all(np.diff(lam) >= -1e-6 * norm)
            assert np.max(np.abs(lam - ref["evals"][c, p])) <= 2e-5 * norm
    # eigenvector quality on the whitened matrices: residual and orthogonality
    sh1 = sh
    plan = sfgb.Plan(sh1.C, sh1.F, sh1.Tp, sh1.R, sh1.Rpp, sh1.P, sh1.B)
    vis = _dev(ref["vis"].astype(np.int32), torch.int32)
    ev = torch.empty((sh.C, 2, sh.R), dtype=torch.float32, device="cuda")
    vec = torch.empty((sh.C, 2, sh.R, sh.R, 2), dtype=torch.float32, device="cuda")
    plan.covariance_eig(vis, sfgb.SF_EIG_SAME_POL_WHITENED, sfgb.SF_K_FIXED, 0.0, True, ev, vec)
    torch.cuda.synchronize()
    lam = ev.cpu().numpy().astype(np.float64)
    v = vec.cpu().numpy()
    V = (v[..., 0] + 1j * v[..., 1]).astype(np.complex128)
    plan.close()
    for p in range(2):
        m = orc.unpack_hermitian(sh, vc, p, p)
        for c in range(sh.C):
            a, _ = orc.whiten(m[c])
            norm = np.linalg.norm(a, 2)
            U = V[c, p].T  # columns = eigenvectors
            res = np.linalg.norm(a @ U - U * lam[c, p][None, :], axis=0).max()
            assert res <= 1e-4 * norm
            assert np.abs(U.conj().T @ U - np.eye(sh.R)).max() <= 1e-4


def test_adaptive_null_projection_and_beams(lambda_cfg):
    sh, samples, scales, weights, rfi = lambda_cfg
    fixed = np.full(sh.C, 2)
    got = _run_adaptive_gpu(sh, samples, scales, weights, sfgb.SF_K_FIXED, 0.0, fixed=fixed)
    ref = orc.adaptive_chain(sh, samples, scales, weights, k_fixed=fixed)
    yr = ref["beams"]
    yb = got["beams"][..., 0] + 1j * got["beams"][..., 1]
    err = np.abs(yb - yr)
    tol = 2.0 ** -9 * np.abs(yr) + 2.0 ** -6 + 1e-3 * np.abs(yr).max(axis=-1, keepdims=True)
    assert np.all(err[:, :, :sh.B] <= 2.0 ** -9 * np.abs(yr[:, :, :sh.B]) + 2.0 ** -6)
    assert np.all(err <= tol)
    # projected eigenvectors (the RFI subspace) match LAPACK's: compare the projectors
    for c in range(sh.C):
        for p in range(2):
            if not rfi[c]:
                continue
            U = got["evecs"][c, p].T[:, -2:]
            Ur = ref["evecs"][c, p].T[:, -2:]
            assert np.abs(U @ U.conj().T - Ur @ Ur.conj().T).max() <= 2e-3


def test_plain_chain_at_golden_test_size():
    """The plain chain at the reference's golden-test size: 36 antennas, 2 pols,
    8 channels, 1024 samples (I, Q = clip(round(N(0, 16^2)), -127, 127), seed 0),
    per-channel per-pol covariance, eigendecomposition, null the top k = 1
    eigenvector, one beam with unit-modulus weights of uniform random phase."""
    sh = orc.Shape(8, 4, 64, 36, 9, 16, 1)
    samples, scales, _ = orc.synth_inputs(sh, seed=0)
    rng = np.random.Generator(np.random.PCG64(0))
    ph = rng.uniform(0.0, 2.0 * np.pi, size=(sh.C, 2, sh.B, sh.R))
    weights = np.stack([np.cos(ph), np.sin(ph)], axis=-1).astype(np.float16)
    fixed = np.ones(sh.C, np.int32)
    got = _run_adaptive_gpu(sh, samples, scales, weights, sfgb.SF_K_FIXED, 0.0, fixed=fixed)
    ref = orc.adaptive_chain(sh, samples, scales, weights, k_fixed=fixed)
    assert np.array_equal(got["vis"], ref["vis"])  # int32 visibilities bit-exact
    assert np.array_equal(got["counts"], np.ones((sh.C, 2), np.int32))
    vc = orc.scaled_visibilities(sh, ref["vis"], orc.receiver_factors(sh))
    for p in range(2):
        m = orc.unpack_hermitian(sh, vc, p, p)
        for c in range(sh.C):
            assert np.all(np.real(np.diag(m[c])) >= 0)  # non-negative autocorrelations
            assert np.allclose(m[c], m[c].conj().T)  # Hermitian covariance
            a, _ = orc.whiten(m[c])
            norm = np.linalg.norm(a, 2)
            assert np.max(np.abs(got["evals"][c, p] - ref["evals"][c, p])) <= 2e-5 * norm
    yr = ref["beams"]
    yb = got["beams"][..., 0] + 1j * got["beams"][..., 1]
    err = np.abs(yb - yr)
    assert np.all(err[:, :, :sh.B] <= 2.0 ** -9 * np.abs(yr[:, :, :sh.B]) + 2.0 ** -6)
    assert np.all(err <= 2.0 ** -9 * np.abs(yr) + 2.0 ** -6 + 1e-3 * np.abs(yr).max(axis=-1, keepdims=True))


def test_adaptive_detection_counts_match_oracle(lambda_cfg):
    sh, samples, scales, weights, rfi = lambda_cfg
    got = _run_adaptive_gpu(sh, samples, scales, weights, sfgb.SF_K_DETECT, 3.0)
    ref = orc.adaptive_chain(sh, samples, scales, weights, detect=True, delta=3.0)
    # detection on the device runs on fp32 eigenvalues; decide with the oracle
    # rule applied to the device's own eigenvalues and compare
    for c in range(sh.C):
        for p in range(2):
            assert got["counts"][c, p] == orc.detect_k_f32(got["evals"][c, p], 3.0)
    assert np.mean(got["counts"] == ref["counts"]) >= 0.9
    # interfered channels detect both interferers
    assert np.all(got["counts"][rfi] >= 2)


def test_gains_and_fine_delays_folded(lambda_cfg):
    sh, samples, scales, weights, rfi = lambda_cfg
    rng = np.random.default_rng(5)
    gains = (rng.normal(1, 0.1, (sh.C, 2, sh.R)) + 1j * rng.normal(0, 0.1, (sh.C, 2, sh.R))).astype(np.complex64)
    tau = rng.uniform(-5, 5, sh.R).astype(np.float32)
    fine = (tau, 0.0, 781250.0, 64)
    fixed = np.full(sh.C, 1)
    got = _run_adaptive_gpu(sh, samples, scales, weights, sfgb.SF_K_FIXED, 0.0, fixed=fixed,
                            gains=gains, fine=fine)
    ph = orc.fine_delay_phasors(sh, tau, 0.0, 781250.0, 64)
    d = orc.receiver_factors(sh, gains=gains, phasors=ph)
    ref = orc.adaptive_chain(sh, samples, scales, weights, k_fixed=fixed, d=d)
    yr = ref["beams"]
    yb = got["beams"][..., 0] + 1j * got["beams"][..., 1]
    tol = 2.0 ** -9 * np.abs(yr) + 2.0 ** -6 + 2e-3 * np.abs(yr).max(axis=-1, keepdims=True)
    assert np.all(np.abs(yb - yr) <= tol)


# --------------------------------------------------------------------------
# Top-K eigensolver (tridiagonal + bisection + inverse iteration): the path the
# adaptive chain takes when no eigenvector output is requested
# --------------------------------------------------------------------------
def _beams_close(got, ref_beams, rel_peak=1e-3):
    yb = got[..., 0] + 1j * got[..., 1]
    tol = 2.0 ** -9 * np.abs(ref_beams) + 2.0 ** -6 + rel_peak * np.abs(ref_beams).max(axis=-1, keepdims=True)
    return np.abs(yb - ref_beams) <= tol


@pytest.mark.parametrize("shrink", [False, True])
def test_topk_path_eigenvalues_and_beams(lambda_cfg, shrink):
    sh, samples, scales, weights, rfi = lambda_cfg
    fixed = np.full(sh.C, 2)
    got = _run_adaptive_gpu(sh, samples, scales, weights, sfgb.SF_K_FIXED, 0.0, shrink=shrink, fixed=fixed,
                            want_evecs=False)
    ref = orc.adaptive_chain(sh, samples, scales, weights, k_fixed=fixed, shrink=shrink)
    vc = orc.scaled_visibilities(sh, ref["vis"], orc.receiver_factors(sh))
    for p in range(2):
        m = orc.unpack_hermitian(sh, vc, p, p)
        for c in range(sh.C):
            a, _ = orc.whiten(m[c])
            norm = np.linalg.norm(a, 2)
            assert np.max(np.abs(got["evals"][c, p] - ref["evals"][c, p])) <= 2e-5 * norm
    ok = _beams_close(got["beams"], ref["beams"])
    assert ok.all(), f"{(~ok).sum()} beam samples outside tolerance"


def test_topk_path_matches_jacobi_path(lambda_cfg):
    sh, samples, scales, weights, rfi = lambda_cfg
    fixed = np.full(sh.C, 3)
    a = _run_adaptive_gpu(sh, samples, scales, weights, sfgb.SF_K_FIXED, 0.0, fixed=fixed, want_evecs=False)
    b = _run_adaptive_gpu(sh, samples, scales, weights, sfgb.SF_K_FIXED, 0.0, fixed=fixed, want_evecs=True)
    ya = a["beams"][..., 0] + 1j * a["beams"][..., 1]
    assert _beams_close(b["beams"], ya, rel_peak=2e-3).all()


def test_topk_path_detection(lambda_cfg):
    sh, samples, scales, weights, rfi = lambda_cfg
    got = _run_adaptive_gpu(sh, samples, scales, weights, sfgb.SF_K_DETECT, 3.0, want_evecs=False)
    for c in range(sh.C):
        for p in range(2):
            assert got["counts"][c, p] == orc.detect_k_f32(got["evals"][c, p], 3.0)
    assert np.all(got["counts"][rfi] >= 2)
    ref = orc.adaptive_chain(sh, samples, scales, weights, detect=True, delta=3.0)
    ok = _beams_close(got["beams"], ref["beams"])
    # channels whose K agrees with the FP64 oracle must agree in their beams
    same = got["counts"] == ref["counts"]
    assert ok[same].all()


@pytest.mark.parametrize("case", [c for c in CASES if c.path == "adaptive"],
                         ids=[c.name for c in CASES if c.path == "adaptive"])
def test_reference_adaptive_goldens_topk_path(case):
    sh = oracle_shape(case)
    a = case.adaptive
    rule = sfgb.SF_K_DETECT if a.get("detect") else sfgb.SF_K_FIXED
    got = _run_adaptive_gpu(sh, case.samples, case.scales, case.weights, rule, a.get("delta", 3.0),
                            shrink=a.get("shrink", False), fixed=np.full(sh.C, a.get("k", 0)),
                            want_evecs=False)
    out = {"beam_half": got["beams"], "counts": got["counts"], "evals": got["evals"]}
    e = dict(case.expect)
    import copy
    c2 = copy.copy(case)
    c2.expect = {k: v for k, v in e.items() if k not in ("evals", "principal_evec")}
    check_case(c2, out)


# --------------------------------------------------------------------------
# Stream permutation (reorder_streams, set_stream_permutation)
# --------------------------------------------------------------------------
def _random_stream_perm(sh, seed, n_zero=3):
    rng = np.random.default_rng(seed)
    src = rng.permutation(2 * sh.R)
    recv = (src // 2).astype(np.int32)
    pol = (src % 2).astype(np.int32)
    recv[rng.choice(2 * sh.R, n_zero, replace=False)] = -1  # zero streams
    recv[5] = recv[9] if recv[9] >= 0 else 0  # a source used twice
    pol[5] = pol[9]
    return recv, pol


@pytest.mark.parametrize("window,delays", [(sfgb.SF_WINDOW_ALIGNED, [0, 5, -7, 64]),
                                           (sfgb.SF_WINDOW_PACKET, None)])
def test_stream_permutation_correlation_bit_exact(window, delays):
    sh = orc.Shape(3, 4, 64, 36, 9, 4, 1)
    rng = np.random.default_rng(17)
    samples = rng.integers(-128, 128, size=sh.samples_shape(), dtype=np.int8)
    scales = rng.integers(-1, 3, size=sh.scales_shape()).astype(np.int16)
    recv, pol = _random_stream_perm(sh, 4)
    plan = sfgb.Plan(sh.C, sh.F, sh.Tp, sh.R, sh.Rpp, sh.P, sh.B)
    if delays is not None:
        plan.set_subpacket_delays(delays)
    plan.set_stream_permutation(recv, pol)
    vis = torch.empty(plan.vis_shape(), dtype=torch.int32, device="cuda")
    plan.correlate(_dev(samples, torch.int8), _dev(scales, torch.int16), window, vis)
    torch.cuda.synchronize()
    rc, bits = plan.status()
    assert rc == 0 and bits == 0
    got = vis.cpu().numpy()
    # back to the identity: plain correlation again
    plan.set_stream_permutation(None, None)
    vis2 = torch.empty(plan.vis_shape(), dtype=torch.int32, device="cuda")
    plan.correlate(_dev(samples, torch.int8), _dev(scales, torch.int16), window, vis2)
    torch.cuda.synchronize()
    plain = vis2.cpu().numpy()
    plan.close()
    off = orc.sample_offsets(sh, delays, mode="aligned" if window == sfgb.SF_WINDOW_ALIGNED else "packet")
    re, im = orc.aligned_samples(sh, samples, scales, off)
    pre, pim = orc.permute_streams(sh, re, im, recv, pol)
    assert np.array_equal(got, orc.correlate(sh, pre, pim))
    assert np.array_equal(plain, orc.correlate(sh, re, im))


def test_stream_permutation_adaptive_chain_with_gains(lambda_cfg):
    sh, samples, scales, weights, rfi = lambda_cfg
    recv, pol = _random_stream_perm(sh, 8, n_zero=0)
    rng = np.random.default_rng(23)
    gains = (rng.uniform(0.5, 1.5, (sh.C, 2, sh.R)) * np.exp(1j * rng.uniform(0, 2 * np.pi, (sh.C, 2, sh.R))))
    tau = rng.uniform(-5.0, 5.0, sh.R).astype(np.float32)
    fixed = np.full(sh.C, 2)
    plan = sfgb.Plan(sh.C, sh.F, sh.Tp, sh.R, sh.Rpp, sh.P, sh.B)
    plan.set_weights(weights)
    plan.set_fixed_counts(fixed)
    plan.set_antenna_gains(gains)
    plan.set_fine_delays(tau, 0.0, 781250.0, 64)
    plan.set_stream_permutation(recv, pol)
    s, sc = _dev(samples, torch.int8), _dev(scales, torch.int16)
    vis = torch.empty(plan.vis_shape(), dtype=torch.int32, device="cuda")
    cnt = torch.empty((sh.C, 2), dtype=torch.int32, device="cuda")
    beams = torch.empty(plan.beams_shape(2), dtype=torch.float16, device="cuda")
    plan.run_adaptive(s, sc, sfgb.SF_K_FIXED, 0.0, False, vis, None, None, cnt, beams)
    torch.cuda.synchronize()
    rc, bits = plan.status()
    assert rc == 0 and bits == 0
    plan.close()
    ph = orc.fine_delay_phasors(sh, tau, 0.0, 781250.0, 64)
    d = orc.permuted_factors(sh, recv, pol, gains=gains, phasors=ph)
    ref = orc.adaptive_chain(sh, samples, scales, weights, k_fixed=fixed, d=d, perm=(recv, pol))
    assert np.array_equal(vis.cpu().numpy(), ref["vis"])
    yr = ref["beams"]
    yb = beams.cpu().numpy().astype(np.float32)
    yb = yb[..., 0] + 1j * yb[..., 1]
    err = np.abs(yb - yr)
    assert np.all(err[:, :, :sh.B] <= 2.0 ** -9 * np.abs(yr[:, :, :sh.B]) + 2.0 ** -6 +
                  2e-3 * np.abs(yr[:, :, :sh.B]).max(axis=-1, keepdims=True))
    assert np.all(err <= 2.0 ** -9 * np.abs(yr) + 2.0 ** -6 + 2e-3 * np.abs(yr).max(axis=-1, keepdims=True))


def test_stream_permutation_rejects_bad_tables():
    sh = orc.Shape(2, 4, 64, 36, 9, 2, 1)
    plan = sfgb.Plan(sh.C, sh.F, sh.Tp, sh.R, sh.Rpp, sh.P, sh.B)
    good_r = np.arange(2 * sh.R, dtype=np.int32) // 2
    good_p = np.arange(2 * sh.R, dtype=np.int32) % 2
    bad_r = good_r.copy()
    bad_r[3] = sh.R
    with pytest.raises(RuntimeError):
        plan.set_stream_permutation(bad_r, good_p)
    bad_p = good_p.copy()
    bad_p[4] = 2
    with pytest.raises(RuntimeError):
        plan.set_stream_permutation(good_r, bad_p)
    with pytest.raises(ValueError):
        plan.set_stream_permutation(good_r[:-2], good_p[:-2])
    pipe = sfgb.LambdaGPUPipeline((sh.C, sh.F, sh.Tp, sh.R, sh.Rpp, sh.P, sh.B), orc.synth_weights(sh))
    with pytest.raises(RuntimeError):
        pipe.set_stream_permutation(list(good_r[:-1]), list(good_p[:-1]))
    pipe.set_stream_permutation(list(good_r), list(good_p))  # identity table is accepted
    pipe.plan.close()
    plan.close()


# --------------------------------------------------------------------------
# Balanced work split: with more channels than SMs, the channels past the
# whole-channel share are cut into stage ranges spread over every CTA; their
# partial visibilities are added with integer atomics.  160 channels of 1024
# samples: 8 tail channels, each cut across many CTAs.
# --------------------------------------------------------------------------
@pytest.fixture(scope="module")
def split_case():
    sh = orc.Shape(160, 4, 64, 36, 9, 16, 4)
    samples, scales, _ = orc.synth_inputs(sh, seed=31, n_interferers=2, frac_channels=0.5)
    weights = orc.synth_weights(sh, seed=32)
    return sh, samples, scales, weights


def test_correlator_split_channels_scaled_packets():
    """Pieces with non-unit packet scales (the general conversion path).
    Amplitudes stay where every 1024-sample fp32 Gram partial is an exact
    integer (|x s| <= 96: 1024 x 96^2 < 2^24), so the result is bit-exact."""
    import os
    import sf_oracle_c as sfc
    sh = orc.Shape(160, 4, 64, 36, 9, 16, 1)
    rng = np.random.default_rng(34)
    samples = rng.integers(-32, 33, size=sh.samples_shape()).astype(np.int8)
    scales = np.where(rng.random(sh.scales_shape()) < 0.3, rng.integers(2, 4, size=sh.scales_shape()), 1).astype(np.int16)
    delays = [3, -9, 0, 40]
    got = _correlate_gpu(sh, samples, scales, sfgb.SF_WINDOW_ALIGNED, delays)
    ref = sfc.correlate(sh, samples, scales, orc.sample_offsets(sh, delays), nthreads=os.cpu_count())
    assert np.array_equal(got, ref)


@pytest.mark.parametrize("window,delays", [(sfgb.SF_WINDOW_ALIGNED, [0, 5, -7, 64]),
                                           (sfgb.SF_WINDOW_PACKET, None)])
def test_correlator_split_channels_bit_exact(split_case, window, delays):
    import os
    import sf_oracle_c as sfc
    sh, samples, scales, _ = split_case
    got = _correlate_gpu(sh, samples, scales, window, delays)
    mode = "aligned" if window == sfgb.SF_WINDOW_ALIGNED else "packet"
    ref = sfc.correlate(sh, samples, scales, orc.sample_offsets(sh, delays, mode=mode), nthreads=os.cpu_count())
    assert np.array_equal(got, ref)


def _beam_close(got, ref_beams, B):
    yb = got[..., 0] + 1j * got[..., 1]
    err = np.abs(yb - ref_beams)
    scale = np.abs(ref_beams).max(axis=-1, keepdims=True)
    bound = 2.0 ** -9 * np.abs(ref_beams) + 2.0 ** -6 + 2e-3 * scale
    assert np.all(err[:, :, :B] <= bound[:, :, :B])
    assert np.all(err <= bound)


def test_adaptive_chain_split_channels(split_case):
    sh, samples, scales, weights = split_case
    fixed = np.full(sh.C, 2)
    got = _run_adaptive_gpu(sh, samples, scales, weights, sfgb.SF_K_FIXED, 0.0, fixed=fixed, want_evecs=False)
    ref = orc.adaptive_chain(sh, samples, scales, weights, k_fixed=fixed)
    assert np.array_equal(got["vis"], ref["vis"])
    _beam_close(got["beams"], ref["beams"], sh.B)


def test_corr_beam_fused_split_channels(split_case):
    sh, samples, scales, weights = split_case
    plan = sfgb.Plan(sh.C, sh.F, sh.Tp, sh.R, sh.Rpp, sh.P, sh.B)
    plan.set_weights(weights)
    s, sc = _dev(samples, torch.int8), _dev(scales, torch.int16)
    vis = torch.full(plan.vis_shape(), -7, dtype=torch.int32, device="cuda")
    beams = torch.empty(plan.beams_shape(1), dtype=torch.float16, device="cuda")
    plan.run_corr_beam(s, sc, vis, beams)
    torch.cuda.synchronize()
    rc, bits = plan.status()
    assert rc == 0 and bits == 0
    plan.close()
    ref = orc.corr_beam_chain(sh, samples, scales, weights)
    assert np.array_equal(vis.cpu().numpy(), ref["vis"])
    _beam_close(beams.cpu().numpy().astype(np.float32), ref["beams"], sh.B)


def test_shallow_packet_ring_corr_beam_split_channels():
    """Tp = 48, R = 48: an eight-slot packet ring, too shallow to hold two
    stages' packets at once, so the converters close every stage before the
    next one is acquired; 200 channels also split into single-stage pieces."""
    sh = orc.Shape(200, 4, 48, 48, 12, 9, 4)
    samples, scales, _ = orc.synth_inputs(sh, seed=41, n_interferers=2, frac_channels=0.5)
    weights = orc.synth_weights(sh, seed=42)
    plan = sfgb.Plan(sh.C, sh.F, sh.Tp, sh.R, sh.Rpp, sh.P, sh.B)
    plan.set_weights(weights)
    s, sc = _dev(samples, torch.int8), _dev(scales, torch.int16)
    vis = torch.full(plan.vis_shape(), -7, dtype=torch.int32, device="cuda")
    beams = torch.empty(plan.beams_shape(1), dtype=torch.float16, device="cuda")
    plan.run_corr_beam(s, sc, vis, beams)
    torch.cuda.synchronize()
    rc, bits = plan.status()
    assert rc == 0 and bits == 0
    plan.close()
    ref = orc.corr_beam_chain(sh, samples, scales, weights)
    assert np.array_equal(vis.cpu().numpy(), ref["vis"])
    _beam_close(beams.cpu().numpy().astype(np.float32), ref["beams"], sh.B)


# --------------------------------------------------------------------------
# Odd receiver and beam counts: the beamformer's weight tile is built from
# its nonzero entries only (rows 2 (p NB + b) + {0, 1}, columns 4 r + 2 p +
# {0, 1}); rows past 4 NB and columns past 4 R stay the zeros written at
# kernel start.  R = 13 (one FPGA), R = 34 (the beamformer's compact last K
# atom with 8 of its 16 values padding) and R = 45 (five FPGAs, 10 beams per
# pol over two slots: 40 of 48 tile rows).
# --------------------------------------------------------------------------
@pytest.mark.parametrize("shape", [(24, 1, 16, 13, 13, 16, 3), (24, 2, 16, 34, 17, 16, 3),
                                   (40, 5, 16, 45, 9, 16, 5)])
def test_odd_receiver_and_beam_counts(shape):
    sh = orc.Shape(*shape)
    samples, scales, _ = orc.synth_inputs(sh, seed=51, n_interferers=1, frac_channels=0.5)
    weights = orc.synth_weights(sh, seed=52)
    # fused corr + beam (one slot)
    plan = sfgb.Plan(sh.C, sh.F, sh.Tp, sh.R, sh.Rpp, sh.P, sh.B)
    plan.set_weights(weights)
    s, sc = _dev(samples, torch.int8), _dev(scales, torch.int16)
    vis = torch.full(plan.vis_shape(), -7, dtype=torch.int32, device="cuda")
    beams = torch.empty(plan.beams_shape(1), dtype=torch.float16, device="cuda")
    plan.run_corr_beam(s, sc, vis, beams)
    torch.cuda.synchronize()
    rc, bits = plan.status()
    assert rc == 0 and bits == 0
    plan.close()
    ref = orc.corr_beam_chain(sh, samples, scales, weights)
    assert np.array_equal(vis.cpu().numpy(), ref["vis"])
    _beam_close(beams.cpu().numpy().astype(np.float32), ref["beams"], sh.B)
    # adaptive chain: beams of both slots from the eigensolver's effective weights
    fixed = np.full(sh.C, 1)
    got = _run_adaptive_gpu(sh, samples, scales, weights, sfgb.SF_K_FIXED, 0.0, fixed=fixed, want_evecs=False)
    ref = orc.adaptive_chain(sh, samples, scales, weights, k_fixed=fixed)
    assert np.array_equal(got["vis"], ref["vis"])
    _beam_close(got["beams"], ref["beams"], sh.B)
