"""Parity at the benchmark's own workload and at the reference's production
integration length (GPU only).

* The 384-channel workload bench.py times (36 antennas, 4096 samples, 8 beams
  x {original, projected}, K = 2, 20 dB interferers in 10 % of the channels,
  fine-delay phasors): visibilities bit-exact for every channel, eigenvalues
  of every whitened covariance within 2e-5 ||A||_2 of LAPACK, the counts, and
  both beam slots within the fp16 bound on every interfered channel plus a
  sample of the others (the C oracle's float64 beams of all 384 channels would
  take 0.8 GB of host memory).
* The reference's production integration, NR_OBSERVING_PACKETS_FOR_CORRELATION
  = 256 packets of 64 samples (T = 16384), through the same chain.
* The explicit fp16 projector output of sf_covariance_eig (the layout of the
  reference's buildIdentityMinusProjection, spatial.cuh:993-1022) against the
  oracle's I - U U^H rounded to fp16.

Tolerances:
  beams slot 0  |y - y_ref| <= 2^-9 |y_ref| + 2^-6 + 2^-10 sum_r |w_r| |x_r(t)|
                (fp16 output rounding, plus the fp16 rounding of the effective
                weights W diag(d) the tensor cores multiply -- at most
                sqrt(2) 2^-11 |w_r| per complex weight: with fine-delay
                phasors they are not fp16-exact)
  beams slot 1  the same + 1e-3 max_t |y_ref| (the projected weights carry the
                fp32 eigenvectors' error)
  eigenvalues   |lambda - lambda_lapack| <= 2e-5 ||A||_2
  projector     |P - P_ref| <= 2e-3 + 2^-11 |P_ref| (fp16 rounding of an fp32
                projector built from separated eigenvectors)
"""
import os

import numpy as np
import pytest
import torch

import sf_oracle as orc
import sf_oracle_c as sfc
import sfgb

pytestmark = pytest.mark.gpu


def _dev(x, dtype):
    return torch.as_tensor(np.ascontiguousarray(x)).to(device="cuda").view(dtype)


def _bench():
    import importlib.util
    from pathlib import Path
    path = Path(__file__).resolve().parents[1] / "bench.py"
    spec = importlib.util.spec_from_file_location("sf_bench_module", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _run(sh, samples, scales, weights, fixed, tau=None, bw=781250.0, min_ch=64):
    plan = sfgb.Plan(sh.C, sh.F, sh.Tp, sh.R, sh.Rpp, sh.P, sh.B)
    plan.set_weights(weights)
    plan.set_fixed_counts(fixed)
    if tau is not None:
        plan.set_fine_delays(tau, 0.0, bw, min_ch)
    s = _dev(samples, torch.int8)
    sc = _dev(scales, torch.int16)
    vis = torch.empty(plan.vis_shape(), dtype=torch.int32, device="cuda")
    ev = torch.empty((sh.C, 2, sh.R), dtype=torch.float32, device="cuda")
    cnt = torch.empty((sh.C, 2), dtype=torch.int32, device="cuda")
    beams = torch.empty(plan.beams_shape(2), dtype=torch.float16, device="cuda")
    plan.run_adaptive(s, sc, sfgb.SF_K_FIXED, 0.0, False, vis, ev, None, cnt, beams)
    torch.cuda.synchronize()
    rc, bits = plan.status()
    assert rc == 0 and bits == 0, f"device status 0x{bits:x}"
    out = {"vis": vis.cpu().numpy(), "evals": ev.cpu().numpy(), "counts": cnt.cpu().numpy(),
           "beams": beams.cpu().numpy()}
    plan.close()
    return out


def _lapack_whitened(sh, vis, d):
    """LAPACK eigenvalues and 2-norms of every whitened same-pol covariance."""
    vc = orc.scaled_visibilities(sh, vis, d)
    lam = np.zeros((sh.C, 2, sh.R))
    nrm = np.zeros((sh.C, 2))
    for p in range(2):
        m = orc.unpack_hermitian(sh, vc, p, p)
        for c in range(sh.C):
            a, _ = orc.whiten(m[c])
            w = np.linalg.eigvalsh(a)
            lam[c, p] = w
            nrm[c, p] = np.abs(w).max()
    return lam, nrm


def _check_beams(got_f16, ref, B):
    """ref: the numpy oracle's adaptive_chain output (beams, w_eff, re, im)."""
    ref_c = ref["beams"]
    y = got_f16.astype(np.float32)
    yb = y[..., 0] + 1j * y[..., 1]
    err = np.abs(yb - ref_c)
    ax = np.sqrt(ref["re"].astype(np.float64) ** 2 + ref["im"].astype(np.float64) ** 2)  # [C][Pol][R][T]
    wsum = np.einsum("cpmr,cprt->cpmt", np.abs(ref["w_eff"]), ax)
    tol0 = 2.0 ** -9 * np.abs(ref_c) + 2.0 ** -6 + 2.0 ** -10 * wsum
    tol1 = tol0 + 1e-3 * np.abs(ref_c).max(axis=-1, keepdims=True)
    assert np.all(err[:, :, :B] <= tol0[:, :, :B]), "slot 0 beams outside the fp16 bound"
    assert np.all(err[:, :, B:] <= tol1[:, :, B:]), "slot 1 beams outside the fp16 bound"


def test_headline_workload_full_parity():
    bench = _bench()
    sh, samples, scales, weights, tau, rfi = bench.make_inputs(seed=0)
    assert (sh.C, sh.R, sh.T, sh.B) == (384, 36, 4096, 8)
    fixed = np.full(sh.C, bench.K_NULL, np.int32)
    got = _run(sh, samples, scales, weights, fixed, tau, bench.CHANNEL_BW, bench.MIN_FREQ_CH)
    nthreads = os.cpu_count() or 1
    # visibilities of all 384 channels, bit-exact against the exact-integer C oracle
    ref_vis = sfc.correlate(sh, samples, scales, orc.sample_offsets(sh), nthreads=nthreads)
    assert np.array_equal(got["vis"], ref_vis)
    assert np.array_equal(got["counts"], np.full((sh.C, 2), bench.K_NULL, np.int32))
    # eigenvalues of all 768 whitened covariances against LAPACK
    d = orc.receiver_factors(sh, phasors=orc.fine_delay_phasors(sh, tau, 0.0, bench.CHANNEL_BW,
                                                                  bench.MIN_FREQ_CH))
    lam, nrm = _lapack_whitened(sh, ref_vis, d)
    assert np.all(np.abs(got["evals"] - lam) <= 2e-5 * nrm[..., None])
    # both beam slots on every interfered channel and a sample of the others
    rng = np.random.default_rng(5)
    quiet = np.flatnonzero(~rfi)
    chans = np.sort(np.concatenate([np.flatnonzero(rfi), rng.choice(quiet, size=10, replace=False)]))
    sub = orc.Shape(len(chans), sh.F, sh.Tp, sh.R, sh.Rpp, sh.P, sh.B)
    ref = orc.adaptive_chain(sub, samples[chans], scales[chans], weights[chans], k_fixed=fixed[chans], d=d[chans])
    assert np.array_equal(ref["vis"], ref_vis[chans])
    _check_beams(got["beams"][chans], ref, sh.B)


def test_reference_production_integration_length():
    """T = 256 packets x 64 samples = 16384 (the reference's default
    NR_OBSERVING_PACKETS_FOR_CORRELATION), 8 channels, 8 beams, K = 2."""
    sh = orc.Shape(8, 4, 64, 36, 9, 256, 8)
    samples, scales, rfi = orc.synth_inputs(sh, seed=3, n_interferers=2, inr_db=20.0, frac_channels=0.5)
    weights = orc.synth_weights(sh, seed=4)
    tau = np.random.default_rng(6).uniform(-5.0, 5.0, sh.R).astype(np.float32)
    fixed = np.full(sh.C, 2, np.int32)
    got = _run(sh, samples, scales, weights, fixed, tau)
    d = orc.receiver_factors(sh, phasors=orc.fine_delay_phasors(sh, tau, 0.0, 781250.0, 64))
    ref = orc.adaptive_chain(sh, samples, scales, weights, k_fixed=fixed, d=d)
    assert np.array_equal(got["vis"], ref["vis"])
    assert np.abs(ref["vis"]).max() > 2 ** 24  # partial sums past fp32's exact range
    lam, nrm = _lapack_whitened(sh, ref["vis"], d)
    assert np.all(np.abs(got["evals"] - lam) <= 2e-5 * nrm[..., None])
    assert np.array_equal(got["counts"], np.full((sh.C, 2), 2, np.int32))
    _check_beams(got["beams"], ref, sh.B)


def test_projector_fp16_output():
    sh = orc.Shape(12, 4, 64, 36, 9, 16, 4)
    samples, scales, rfi = orc.synth_inputs(sh, seed=8, n_interferers=2, inr_db=20.0, frac_channels=0.5)
    weights = orc.synth_weights(sh, seed=9)
    fixed = np.where(rfi, 2, 0).astype(np.int32)
    ref = orc.adaptive_chain(sh, samples, scales, weights, k_fixed=fixed)
    plan = sfgb.Plan(sh.C, sh.F, sh.Tp, sh.R, sh.Rpp, sh.P, sh.B)
    plan.set_weights(weights)
    plan.set_fixed_counts(fixed)
    vis = _dev(ref["vis"].astype(np.int32), torch.int32)
    proj = torch.empty((sh.C, 2, sh.R, sh.R, 2), dtype=torch.float16, device="cuda")
    cnt = torch.empty((sh.C, 2), dtype=torch.int32, device="cuda")
    plan.covariance_eig(vis, sfgb.SF_EIG_SAME_POL_WHITENED, sfgb.SF_K_FIXED, 0.0, False, None, None, cnt, proj)
    torch.cuda.synchronize()
    rc, bits = plan.status()
    assert rc == 0 and bits == 0
    plan.close()
    pf = proj.cpu().numpy().astype(np.float32)
    P = (pf[..., 0] + 1j * pf[..., 1]).transpose(0, 1, 3, 2)  # stored column-major: [col][row]
    Pref = ref["proj"]
    for c in range(sh.C):
        for p in range(2):
            if not rfi[c]:
                # K = 0: the identity, exact in fp16
                assert np.array_equal(P[c, p], np.eye(sh.R))
                continue
            err = np.abs(P[c, p] - Pref[c, p])
            assert np.all(err <= 2e-3 + 2.0 ** -11 * np.abs(Pref[c, p]))
    assert np.array_equal(cnt.cpu().numpy(), np.stack([fixed, fixed], axis=1))
