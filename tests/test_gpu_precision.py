"""Precision form of the batched chain (GPU only): 256-receiver units, more
than 16 beams (beamformer beam groups), FP32 top-K eigenvectors refined in
FP64 with an orthogonal re-projection of the weights, and BF16 / e4m3 beam
operands with per-beam scales, against the FP64 oracle.

Tolerances:
  visibilities   bit-exact
  eigenvalues    |lambda - lambda_lapack| <= 2e-5 ||A||_2 (n <= 128), 5e-5 ||A||_2 (n = 256:
                 Householder in fp32 over 256 columns)
  refinement     FP64 Ritz values within 1e-9 relative of LAPACK; the relative residual after
                 the FP64 steps <= 1e-8 and never above the FP32 one
  weights        FP64-projected effective weights within 2e-6 |w|_max of the oracle's (fp32 storage)
  beams          |y - y_ref| <= 2^-9 |y_ref| + 2^-6 + e_w sum_r |w_r| |x_r(t)| (+ e_x for rounded
                 samples): e_w = 2^-10 (fp16), 2^-8 (bf16), 2^-3 (e4m3, relative to the per-beam
                 scale), e_x = 2^-4 (e4m3-rounded samples)
"""
import numpy as np
import pytest
import torch

import sf_oracle as orc
import sfgb

pytestmark = pytest.mark.gpu

RECV = [256, 64, 256, 128, 36, 256]


def _setup(B, seed, T=512):
    xs, ws = orc.synth_batch(RECV, T, B, seed=seed, max_interferers=3)
    bt = sfgb.Batch(RECV, T, B)
    bt.set_weights(bt.pack_weights(ws))
    s = torch.as_tensor(bt.pack_samples(xs)).cuda()
    return xs, ws, bt, s


def _run(bt, s, precision, steps=2, orthogonal=True):
    bt.set_precision(precision, steps, orthogonal)
    vis = torch.empty(bt.totals["vis"], dtype=torch.int32, device="cuda")
    ev = torch.empty(bt.totals["evals"], dtype=torch.float32, device="cuda")
    cnt = torch.full((bt.n_units, 2), -1, dtype=torch.int32, device="cuda")
    beams = torch.full((2 * bt.totals["beams"],), float("nan"), dtype=torch.float16, device="cuda")
    bt.run(s, sfgb.SF_K_NOISE_FLOOR, 10.0, False, vis, ev, cnt, beams)
    torch.cuda.synchronize()
    rc, bits = bt.status()
    assert rc == 0 and bits == 0, f"device status 0x{bits:x}"
    return vis.cpu().numpy(), ev.cpu().numpy(), cnt.cpu().numpy(), beams.cpu().numpy()


@pytest.mark.parametrize("precision,e_w,e_x", [(sfgb.SF_BEAM_FP16, 2.0 ** -10, 0.0),
                                               (sfgb.SF_BEAM_BF16, 2.0 ** -8, 0.0),
                                               (sfgb.SF_BEAM_E4M3_SPLIT, 2.0 ** -3, 0.0),
                                               (sfgb.SF_BEAM_E4M3, 2.0 ** -3, 2.0 ** -4)])
def test_precision_batch_against_fp64(precision, e_w, e_x):
    B = 20  # more than 16: beamformer beam groups, the refined path
    xs, ws, bt, s = _setup(B, seed=5)
    vis, ev, cnt, beams = _run(bt, s, precision)
    resid, ritz = bt.precision_report()
    for u, R in enumerate(RECV):
        evals = bt.unit_evals(ev, u)
        for p in range(2):
            assert cnt[u, p] == orc.noise_floor_k_f32(evals[p], 10.0)
        ref = orc.unit_chain(xs[u], ws[u], "fixed", k_fixed=cnt[u], orthogonal=True)
        assert np.array_equal(bt.unit_vis(vis, u), ref["vis"]), f"unit {u} visibilities"
        nrm = np.abs(ref["evals"]).max(axis=-1, keepdims=True)
        assert np.all(np.abs(evals - ref["evals"]) <= (2e-5 if R <= 128 else 5e-5) * nrm), f"unit {u} eigenvalues"
        for p in range(2):
            k = cnt[u, p]
            if k == 0:
                continue
            top = ref["evals"][p][::-1][:k]
            assert np.all(np.abs(ritz[u, p, :k] - top) <= 1e-9 * top[0]), f"unit {u} pol {p} Ritz values"
            assert resid[u, p, 1] <= 1e-8 and resid[u, p, 1] <= resid[u, p, 0] + 1e-12, (u, p, resid[u, p])
        y = bt.unit_beams(beams, u).astype(np.float64)
        yb = y[..., 0] + 1j * y[..., 1]
        yr = ref["beams"]
        re, im = orc.unit_samples_split(xs[u])
        ax = np.sqrt(re[0].astype(np.float64) ** 2 + im[0].astype(np.float64) ** 2)
        wsum = np.einsum("pmr,prt->pmt", np.abs(ref["w_eff"]), ax)
        tol = 2.0 ** -9 * np.abs(yr) + 2.0 ** -6 + (e_w + e_x) * wsum
        assert np.all(np.abs(yb - yr) <= tol), f"unit {u} beams ({precision})"
    bt.close()


def test_refined_weights_match_fp64_projection():
    """The FP64-refined, orthogonally re-projected weights equal the oracle's
    W (I - Q Q^H) to fp32 storage accuracy; with orthogonal = False the
    reference's I - U U^H convention."""
    B = 4
    for orthogonal in (True, False):
        xs, ws, bt, s = _setup(B, seed=7)
        vis, ev, cnt, beams = _run(bt, s, sfgb.SF_BEAM_FP16, steps=2, orthogonal=orthogonal)
        # the effective weights are exercised through the fp16 beams with the fp16 weight bound
        for u, R in enumerate(RECV):
            ref = orc.unit_chain(xs[u], ws[u], "fixed", k_fixed=cnt[u], orthogonal=orthogonal)
            y = bt.unit_beams(beams, u).astype(np.float64)
            yb = y[..., 0] + 1j * y[..., 1]
            re, im = orc.unit_samples_split(xs[u])
            ax = np.sqrt(re[0].astype(np.float64) ** 2 + im[0].astype(np.float64) ** 2)
            wsum = np.einsum("pmr,prt->pmt", np.abs(ref["w_eff"]), ax)
            tol = 2.0 ** -9 * np.abs(ref["beams"]) + 2.0 ** -6 + 2.0 ** -10 * wsum
            assert np.all(np.abs(yb - ref["beams"]) <= tol), f"unit {u} orthogonal={orthogonal}"
        bt.close()
