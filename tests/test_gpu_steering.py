"""Steering-weight synthesis on the device (sf_set_steering_weights) vs the
oracle restatement of compute_steering_weights, and through a chain (GPU only).

The kernel and the oracle both evaluate the phase in float64 and round
float64 -> float32 -> fp16; their sin/cos and fused multiply-adds can differ in
the last double bits, which moves an fp16 result by one unit in the last place
only when it sits on a rounding boundary: at most 1 fp16 ulp, and rarely.
The reference's own tests allow 2e-3 against the formula
(tests/test_pipeline.cu:1398-1432); null inputs must be exactly zero
(tests/test_pipeline.cu:1435-1489).
"""
import math

import numpy as np
import pytest
import torch

import sf_oracle as orc
import sfgb
from sfgb import pointing as pt

pytestmark = pytest.mark.gpu

NOW = 1.7648e9


def _fp16_ulp(x):
    a = np.abs(x.astype(np.float32))
    e = np.floor(np.log2(np.maximum(a, 2.0 ** -14)))
    return 2.0 ** (e - 10)


def _steered_beams(sh, samples, scales, steer_args, window=sfgb.SF_WINDOW_PACKET):
    plan = sfgb.Plan(sh.C, sh.F, sh.Tp, sh.R, sh.Rpp, sh.P, sh.B)
    plan.set_weights(np.zeros((sh.C, 2, sh.B, sh.R, 2), np.float16))
    plan.set_steering_weights(*steer_args)
    s = torch.as_tensor(samples).cuda()
    sc = torch.as_tensor(scales).cuda()
    beams = torch.empty(plan.beams_shape(1), dtype=torch.float16, device="cuda")
    plan.beamform(s, sc, window, 1, beams)
    torch.cuda.synchronize()
    rc, bits = plan.status()
    assert rc == 0 and bits == 0
    plan.close()
    return beams.cpu().numpy()


def _probe_inputs(sh):
    """Samples that make beam (c, p, m) at time t = R * k + r equal to
    scale * w[c][p][m][r] for every k: receiver r is 1 at t % R == r, else 0."""
    samples = np.zeros(sh.samples_shape(), np.int8)
    for f in range(sh.F):
        for n in range(sh.Rpp):
            r = f * sh.Rpp + n
            for pkt in range(sh.P):
                for tt in range(sh.Tp):
                    if (pkt * sh.Tp + tt) % sh.R == r:
                        samples[:, pkt, f, tt, n, :, 0] = 1
    scales = np.ones(sh.scales_shape(), np.int16)
    return samples, scales


def _weights_via_beams(sh, steer_args):
    """The plan's weights read back through a beamforming run on probe
    samples (exact: unit samples, unit scales, fp16 weights)."""
    samples, scales = _probe_inputs(sh)
    y = _steered_beams(sh, samples, scales, steer_args)  # [C][2][B][T][2]
    w = np.zeros((sh.C, 2, sh.B, sh.R, 2), np.float16)
    for r in range(sh.R):
        w[:, :, :, r, :] = y[:, :, :, r, :]
    return w


@pytest.fixture(scope="module")
def geometry():
    rng = np.random.default_rng(7)
    sh = orc.Shape(12, 4, 16, 36, 9, 3, 8)
    az = rng.uniform(0, 2 * np.pi, sh.B)
    el = rng.uniform(np.radians(20), np.radians(90), sh.B)
    dircos = np.stack([np.sin(az) * np.cos(el), np.cos(az) * np.cos(el), np.sin(el)], axis=1)
    enu = rng.uniform(-150.0, 150.0, (sh.R, 3))
    enu[:, 2] = rng.uniform(-3.0, 3.0, sh.R)
    connected = np.ones(sh.R, np.int32)
    connected[[0, 2, 17]] = 0
    cal = rng.uniform(0.6, 1.4, (sh.C, 2, sh.R)) * np.exp(1j * rng.uniform(0, 2 * np.pi, (sh.C, 2, sh.R)))
    return sh, dircos, enu, connected, cal


@pytest.mark.parametrize("with_cal", [False, True])
def test_steering_weights_match_oracle(geometry, with_cal):
    sh, dircos, enu, connected, cal = geometry
    args = (dircos, enu, connected, 1.2e9, 781250.0, 64, cal if with_cal else None)
    got = _weights_via_beams(sh, args).astype(np.float32)
    ref = orc.steering_weights(sh, dircos, enu, connected, 1.2e9, 781250.0, 64,
                               cal if with_cal else None).astype(np.float32)
    diff = np.abs(got - ref)
    assert np.all(diff <= _fp16_ulp(ref)), f"max diff {diff.max()}"
    assert np.mean(diff == 0) > 0.995
    assert np.all(got[:, :, :, [0, 2, 17]] == 0.0)


def test_reference_steering_case_radec_target():
    """ComputeSteeringWeightsMatchesGeometricPhaseFormula
    (tests/test_pipeline.cu:1362-1433) through the device synthesis."""
    sh = orc.Shape(4, 1, 16, 4, 4, 2, 1)
    pos = {100: (0.0, 0.0, 0.0), 101: (25.0, -10.0, 1.5), 102: (-12.5, 30.0, -2.0), 103: (8.0, 8.0, 0.5)}
    mapping = {0: 100, 1: 101, 2: 102, 3: 103}
    targets = [{"mode": "radec", "ra_deg": 83.633, "dec_deg": 22.014}]
    dircos, enu, conn = pt.steering_geometry(sh.B, sh.R, targets, pos, mapping, NOW, 52.91, 6.87, 30.0)
    w = _weights_via_beams(sh, (dircos, enu, conn, 1.4e9, 1.0e5, 64, None)).astype(np.float32)
    dc = pt.topocentric_direction(83.633, 22.014, NOW, 52.91, 6.87, 30.0)
    for c in range(sh.C):
        f = pt.channel_to_frequency_hz(64 + c, 1.4e9, 1.0e5)
        for r in range(sh.R):
            e = pos[mapping[r]]
            ph = -2.0 * math.pi * f / pt.SPEED_OF_LIGHT * (dc[0] * e[0] + dc[1] * e[1] + dc[2] * e[2])
            for p in range(2):
                assert abs(w[c, p, 0, r, 0] - math.cos(ph) / sh.R) < 2e-3
                assert abs(w[c, p, 0, r, 1] - math.sin(ph) / sh.R) < 2e-3


def test_reference_steering_case_null_antennas():
    """ComputeSteeringWeightsZeroesNullAntennas (tests/test_pipeline.cu:1435-1489)."""
    sh = orc.Shape(3, 1, 16, 4, 4, 2, 2)
    pos = {100: (0.0, 0.0, 0.0), 101: (25.0, -10.0, 1.5)}
    mapping = {0: -100, 1: 100, 2: -100, 3: 101}
    dircos, enu, conn = pt.steering_geometry(sh.B, sh.R, [{"mode": "zenith"}], pos, mapping, NOW)
    w = _weights_via_beams(sh, (dircos, enu, conn, 1.4e9, 1.0e5, 0, None)).astype(np.float32)
    assert np.all(w[:, :, :, [0, 2]] == 0.0)
    amp = np.hypot(w[..., 0], w[..., 1])
    assert np.all(np.abs(amp[:, :, :, [1, 3]] - 1.0 / sh.R) < 2e-3)


def test_steered_adaptive_chain(geometry):
    """A chain run on steered weights equals the oracle chain on the oracle's
    steering weights (beam tolerance of the parity tests plus the 1-ulp
    weight allowance)."""
    sh0, dircos, enu, connected, cal = geometry
    sh = orc.Shape(sh0.C, sh0.F, 64, sh0.R, sh0.Rpp, 4, sh0.B)
    samples, scales, _ = orc.synth_inputs(sh, seed=5, n_interferers=2, frac_channels=0.5)
    plan = sfgb.Plan(sh.C, sh.F, sh.Tp, sh.R, sh.Rpp, sh.P, sh.B)
    plan.set_weights(np.zeros((sh.C, 2, sh.B, sh.R, 2), np.float16))
    plan.set_steering_weights(dircos, enu, connected, 1.2e9, 781250.0, 64, cal)
    fixed = np.full(sh.C, 2)
    plan.set_fixed_counts(fixed)
    s, sc = torch.as_tensor(samples).cuda(), torch.as_tensor(scales).cuda()
    cnt = torch.empty((sh.C, 2), dtype=torch.int32, device="cuda")
    beams = torch.empty(plan.beams_shape(2), dtype=torch.float16, device="cuda")
    plan.run_adaptive(s, sc, sfgb.SF_K_FIXED, 0.0, False, None, None, None, cnt, beams)
    torch.cuda.synchronize()
    rc, bits = plan.status()
    assert rc == 0 and bits == 0
    plan.close()
    w = orc.steering_weights(sh, dircos, enu, connected, 1.2e9, 781250.0, 64, cal)
    ref = orc.adaptive_chain(sh, samples, scales, w, k_fixed=fixed)
    yb = beams.cpu().numpy().astype(np.float32)
    yb = yb[..., 0] + 1j * yb[..., 1]
    yr = ref["beams"]
    err = np.abs(yb - yr)
    scale = np.abs(yr).max(axis=-1, keepdims=True)
    assert np.all(err[:, :, :sh.B] <= 2.0 ** -9 * np.abs(yr[:, :, :sh.B]) + 2.0 ** -6 + 2e-3 * scale[:, :, :sh.B])
    assert np.all(err <= 2.0 ** -9 * np.abs(yr) + 2.0 ** -6 + 2e-3 * scale)


def test_steering_rejects_bad_input(geometry):
    sh, dircos, enu, connected, cal = geometry
    plan = sfgb.Plan(sh.C, sh.F, sh.Tp, sh.R, sh.Rpp, sh.P, sh.B)
    bad = np.array(dircos)
    bad[1, 1] = np.nan
    with pytest.raises(sfgb.SfError) as e:
        plan.set_steering_weights(bad, enu, connected, 1.2e9, 781250.0, 64)
    assert e.value.code == 1
    plan.close()
