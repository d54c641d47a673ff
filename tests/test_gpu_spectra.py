"""Beam spectra tails vs the oracle (GPU only).

Both kernels read fp16 beams and compute in fp32; the oracle transforms the
same fp16 values in float64 (numpy's FFT, pinned to the DFT definition in
test_oracle_spectra.py).  Tolerances, per output row (one (channel, pol, beam)):
  whole-integration power  |S - S_ref| <= 2e-5 mean(S_ref) + 1e-6 S_ref
  per-packet magnitude sum |S - S_ref| <= 2e-5 mean(S_ref) + 1e-6 S_ref
(fp32 FFT rounding grows like log2 N; per-bin errors scale with the row's
energy, not the bin's own value, hence the mean term).  Against the oracle's
float64 beams the fp16 rounding of the beams adds ~2^-11 relative per sample:
  chain spectra            |S - S_ref| <= 3e-3 mean(S_ref)
"""
import numpy as np
import pytest
import torch

import sf_oracle as orc
import sfgb

pytestmark = pytest.mark.gpu


def _random_beams(rng, C, nb, T, scale=100.0):
    b = rng.normal(0.0, scale, (C, 2, nb, T, 2)).astype(np.float16)
    return b


def _dev16(x):
    return torch.as_tensor(np.ascontiguousarray(x)).to(device="cuda")


def _plan_for(T, Tp=64, C=3, B=2):
    P = T // Tp
    return sfgb.Plan(C, 1, Tp, 4, 4, P, B)


def _row_close(got, ref, rel_mean, rel_bin):
    m = np.abs(ref).mean(axis=-1, keepdims=True)
    err = np.abs(got - ref)
    bound = rel_mean * m + rel_bin * np.abs(ref)
    bad = err > bound
    assert not bad.any(), (
        f"{bad.sum()} of {bad.size} bins out of tolerance; worst ratio "
        f"{(err / np.maximum(bound, 1e-30)).max():.3g}")


@pytest.mark.parametrize("T,Tp,D", [
    (64, 16, 1), (64, 64, 64), (256, 64, 7), (1024, 64, 16), (2048, 32, 128),
    (4096, 64, 128), (4096, 64, 1), (8192, 64, 33), (16384, 64, 128), (16384, 64, 16384),
])
def test_beam_spectra_matches_oracle(T, Tp, D):
    rng = np.random.default_rng(T + D)
    C, nb = 3, 3
    plan = _plan_for(T, Tp, C)
    beams = _random_beams(rng, C, nb, T)
    out = torch.full(plan.beam_spectra_shape(nb, D), -1.0, dtype=torch.float32, device="cuda")
    plan.beam_spectra(_dev16(beams), nb, D, out)
    torch.cuda.synchronize()
    plan.close()
    ref = orc.beam_spectra(orc.beams_from_half(beams), D)
    assert out.shape == ref.shape
    _row_close(out.cpu().numpy().astype(np.float64), ref, 2e-5, 1e-6)


def test_beam_spectra_nan_series_gives_zero_and_leaves_others():
    rng = np.random.default_rng(5)
    T, D, C, nb = 4096, 128, 2, 2
    plan = _plan_for(T, 64, C)
    beams = _random_beams(rng, C, nb, T)
    beams[1, 0, 1, 17, 0] = np.float16(np.nan)
    out = torch.empty(plan.beam_spectra_shape(nb, D), dtype=torch.float32, device="cuda")
    plan.beam_spectra(_dev16(beams), nb, D, out)
    torch.cuda.synchronize()
    plan.close()
    got = out.cpu().numpy().astype(np.float64)
    ref = orc.beam_spectra(orc.beams_from_half(beams), D)
    assert np.all(got[1, 0, 1] == 0.0) and np.all(ref[1, 0, 1] == 0.0)
    mask = np.ones(got.shape[:3], bool)
    mask[1, 0, 1] = False
    _row_close(got[mask], ref[mask], 2e-5, 1e-6)


# Tp = 64 with P % 32 == 0 takes the tensor-core path, the rest the SIMT path
@pytest.mark.parametrize("Tp,P,trim,C,nb", [
    (64, 64, 5, 3, 4), (64, 32, 5, 3, 4), (64, 96, 0, 3, 4), (64, 128, 31, 2, 3), (64, 64, 5, 40, 8),
    (64, 1, 5, 3, 4), (64, 33, 0, 3, 4), (64, 100, 31, 3, 4), (32, 5, 5, 3, 4), (32, 64, 0, 3, 4),
    (16, 7, 2, 3, 4), (16, 65, 7, 3, 4),
])
def test_packet_spectra_matches_oracle(Tp, P, trim, C, nb):
    rng = np.random.default_rng(Tp * 1000 + P + C)
    plan = sfgb.Plan(C, 1, Tp, 4, 4, P, 2)
    beams = _random_beams(rng, C, nb, Tp * P)
    out = torch.full(plan.packet_spectra_shape(nb, trim), -1.0, dtype=torch.float32, device="cuda")
    plan.packet_spectra(_dev16(beams), nb, trim, out)
    torch.cuda.synchronize()
    plan.close()
    ref = orc.packet_spectra(orc.beams_from_half(beams), Tp, trim)
    assert out.shape == ref.shape
    _row_close(out.cpu().numpy().astype(np.float64), ref, 2e-5, 1e-6)


def test_spectra_are_deterministic():
    rng = np.random.default_rng(9)
    Tp, P, C, nb = 64, 64, 4, 4
    plan = sfgb.Plan(C, 1, Tp, 4, 4, P, 2)
    b = _dev16(_random_beams(rng, C, nb, Tp * P))
    o1 = torch.empty(plan.packet_spectra_shape(nb, 5), dtype=torch.float32, device="cuda")
    o2 = torch.empty_like(o1)
    w1 = torch.empty(plan.beam_spectra_shape(nb, 128), dtype=torch.float32, device="cuda")
    w2 = torch.empty_like(w1)
    plan.packet_spectra(b, nb, 5, o1)
    plan.packet_spectra(b, nb, 5, o2)
    plan.beam_spectra(b, nb, 128, w1)
    plan.beam_spectra(b, nb, 128, w2)
    torch.cuda.synchronize()
    plan.close()
    assert torch.equal(o1, o2) and torch.equal(w1, w2)


def test_spectra_reject_unsupported_shapes():
    b = torch.zeros(64 * 3 * 2 * 2 * 2 * 2, dtype=torch.float16, device="cuda")
    out = torch.zeros(4096, dtype=torch.float32, device="cuda")
    plan = sfgb.Plan(2, 1, 64, 4, 4, 3, 2)  # T = 192: not a power of two
    with pytest.raises(sfgb.SfError) as e:
        plan.beam_spectra(b, 2, 16, out)
    assert e.value.code == 2
    plan.packet_spectra(b, 2, 5, out)  # Tp = 64 is fine
    with pytest.raises(sfgb.SfError) as e:
        plan.packet_spectra(b, 2, 32, out)  # trim >= Tp / 2
    assert e.value.code == 1
    with pytest.raises(sfgb.SfError) as e:
        plan.packet_spectra(b[1:], 2, 5, out)  # not 16-byte aligned
    assert e.value.code == 1
    plan.close()
    plan = sfgb.Plan(2, 1, 8, 4, 4, 16, 2)  # Tp = 8
    with pytest.raises(sfgb.SfError) as e:
        plan.packet_spectra(b, 2, 1, out)
    assert e.value.code == 2
    with pytest.raises(sfgb.SfError) as e:
        plan.beam_spectra(b, 2, 0, out)
    assert e.value.code == 1
    plan.close()
    torch.cuda.synchronize()


@pytest.fixture(scope="module")
def lambda_chain():
    sh = orc.Shape(6, 4, 64, 36, 9, 64, 4)
    samples, scales, _ = orc.synth_inputs(sh, seed=3, n_interferers=2, frac_channels=0.5)
    weights = orc.synth_weights(sh, seed=4)
    return sh, samples, scales, weights


def test_adaptive_chain_packet_spectra(lambda_chain):
    sh, samples, scales, weights = lambda_chain
    fixed = np.full(sh.C, 2)
    plan = sfgb.Plan(sh.C, sh.F, sh.Tp, sh.R, sh.Rpp, sh.P, sh.B)
    plan.set_weights(weights)
    plan.set_fixed_counts(fixed)
    s = _dev16(samples).view(torch.int8)
    sc = _dev16(scales).view(torch.int16)
    cnt = torch.empty((sh.C, 2), dtype=torch.int32, device="cuda")
    beams = torch.empty(plan.beams_shape(2), dtype=torch.float16, device="cuda")
    spec = torch.empty(plan.packet_spectra_shape(2 * sh.B, 5), dtype=torch.float32, device="cuda")
    plan.run_adaptive(s, sc, sfgb.SF_K_FIXED, 0.0, False, None, None, None, cnt, beams)
    plan.packet_spectra(beams, 2 * sh.B, 5, spec)
    torch.cuda.synchronize()
    rc, bits = plan.status()
    assert rc == 0 and bits == 0
    plan.close()
    got = spec.cpu().numpy().astype(np.float64)
    own = orc.packet_spectra(orc.beams_from_half(beams.cpu().numpy()), sh.Tp, 5)
    _row_close(got, own, 2e-5, 1e-6)
    ref = orc.adaptive_chain(sh, samples, scales, weights, k_fixed=fixed)
    refs = orc.packet_spectra(ref["beams"], sh.Tp, 5)
    _row_close(got[:, :, :sh.B], refs[:, :, :sh.B], 3e-3, 0.0)
    # projected beams carry the fp32 eigensolver's error as well
    _row_close(got[:, :, sh.B:], refs[:, :, sh.B:], 2e-2, 0.0)


def test_lambda_gpu_chain_beam_spectra(lambda_chain):
    sh, samples, scales, weights = lambda_chain
    plan = sfgb.Plan(sh.C, sh.F, sh.Tp, sh.R, sh.Rpp, sh.P, sh.B)
    plan.set_weights(weights)
    s = _dev16(samples).view(torch.int8)
    sc = _dev16(scales).view(torch.int16)
    vis = torch.empty(plan.vis_shape(), dtype=torch.int32, device="cuda")
    beams = torch.empty(plan.beams_shape(1), dtype=torch.float16, device="cuda")
    D = 128
    spec = torch.empty(plan.beam_spectra_shape(sh.B, D), dtype=torch.float32, device="cuda")
    plan.run_lambda_gpu(s, sc, vis, None, None, beams)
    plan.beam_spectra(beams, sh.B, D, spec)
    torch.cuda.synchronize()
    rc, bits = plan.status()
    assert rc == 0 and bits == 0
    plan.close()
    got = spec.cpu().numpy().astype(np.float64)
    ref = orc.lambda_gpu_chain(sh, samples, scales, weights)
    _row_close(got, orc.beam_spectra(ref["beams"], D), 3e-3, 0.0)
