"""Learned subspace proposer (GPU only): the hand-written BF16 tcgen05 GEMM
against a PyTorch fp32 reference, training on pipeline-generated covariances,
and the learned adaptive chain (warm-started Rayleigh-Ritz + residual-gated
fallback) against the plain chain and the FP64 oracle.

Tolerances:
  GEMM fp32 out    |C - C_ref| <= 1e-5 sum_k |a_mk b_nk| + 1e-6 (bf16 inputs exact, fp32 sums)
  GEMM bf16 out    the same + 2^-8 |C_ref| (bf16 rounding of the output)
  learned chain    with tol = 0 every matrix falls back: beams equal the plain chain's bit for bit;
                   with tol = 1e-3: null depth within 0.5 dB of the FP64 full eigensolve
"""
import numpy as np
import pytest
import torch

import sf_oracle as orc
import sfgb
from sfgb import proposer as prop

pytestmark = pytest.mark.gpu


def _bf16(rng, shape):
    return torch.as_tensor(rng.standard_normal(shape).astype(np.float32)).cuda().to(torch.bfloat16)


@pytest.mark.parametrize("a_mn,b_mn", [(0, 0), (1, 0), (0, 1), (1, 1)])
@pytest.mark.parametrize("mode", [0, 1, 2, 3])
def test_gemm_bf16_against_fp32_reference(a_mn, b_mn, mode):
    rng = np.random.default_rng(17 + 4 * a_mn + 2 * b_mn + 8 * mode)
    M, N, K = 296, 200, 264
    A = _bf16(rng, (K, M) if a_mn else (M, K))
    B = _bf16(rng, (K, N) if b_mn else (N, K))
    Af = A.float().T if a_mn else A.float()  # [M][K]
    Bf = B.float().T if b_mn else B.float()  # [N][K]
    ref = Af @ Bf.T
    bound = (Af.abs() @ Bf.abs().T) * 1e-5 + 1e-6
    bias = torch.as_tensor(rng.standard_normal(N).astype(np.float32)).cuda()
    lda = M if a_mn else K
    ldb = N if b_mn else K
    if mode == 1:
        out = torch.empty((M, N), dtype=torch.float32, device="cuda")
        st = sfgb.gemm_bf16(M, N, K, A, lda, a_mn, B, ldb, b_mn, 1, out, N, bias=bias)
        want = ref + bias[None]
        torch.cuda.synchronize()
        assert int(st.item()) == 0
        assert torch.all((out - want).abs() <= bound)
    elif mode == 3:
        out = torch.full((M, N), 0.5, dtype=torch.float32, device="cuda")
        st = sfgb.gemm_bf16(M, N, K, A, lda, a_mn, B, ldb, b_mn, 3, out, N, k_splits=3)
        torch.cuda.synchronize()
        assert int(st.item()) == 0
        assert torch.all((out - (ref + 0.5)).abs() <= bound + 1e-5 * ref.abs())
    else:
        out = torch.empty((M, N), dtype=torch.bfloat16, device="cuda")
        mask = _bf16(rng, (M, N))
        if mode == 0:
            st = sfgb.gemm_bf16(M, N, K, A, lda, a_mn, B, ldb, b_mn, 0, out, N, bias=bias)
            want = torch.relu(ref + bias[None])
        else:
            st = sfgb.gemm_bf16(M, N, K, A, lda, a_mn, B, ldb, b_mn, 2, out, N, mask=mask, ldm=N)
            want = torch.where(mask.float() > 0, ref, torch.zeros_like(ref))
        torch.cuda.synchronize()
        assert int(st.item()) == 0
        assert torch.all((out.float() - want).abs() <= bound + 2.0 ** -8 * want.abs())


def test_training_reduces_loss():
    q = prop.Proposer(36, 512, 8192)
    q.init_params(seed=0)
    x, t, w = prop.make_training_set(8 * 8192, q, P=16, chunk_channels=4096, seed=1)
    hist = prop.train(q, x, t, w, epochs=10, batch=8192, lr=2e-3)
    assert all(np.isfinite(hist))
    # the loss falls steadily (2.74 -> 2.15 in one measured run of these ten epochs)
    assert hist[-1] < 0.85 * hist[0] and hist[-1] < hist[len(hist) // 2] < hist[0], hist
    q.close()


def _chain_inputs(C=64, P=16, seed=4):
    sh = orc.Shape(C, 4, 64, 36, 9, P, 8)
    samples, scales, rfi, steering = orc.synth_inputs(sh, seed=seed, n_interferers=2, inr_db=20.0,
                                                      frac_channels=0.5, return_steering=True)
    weights = orc.synth_weights(sh, seed=seed + 1)
    return sh, samples, scales, weights, rfi, steering


def _run_plain(sh, samples, scales, weights, fixed):
    plan = sfgb.Plan(sh.C, sh.F, sh.Tp, sh.R, sh.Rpp, sh.P, sh.B)
    plan.set_weights(weights)
    plan.set_fixed_counts(fixed)
    s, sc = torch.as_tensor(samples).cuda(), torch.as_tensor(scales).cuda()
    vis = torch.empty(plan.vis_shape(), dtype=torch.int32, device="cuda")
    cnt = torch.empty((sh.C, 2), dtype=torch.int32, device="cuda")
    beams = torch.empty(plan.beams_shape(2), dtype=torch.float16, device="cuda")
    plan.run_adaptive(s, sc, sfgb.SF_K_FIXED, 0.0, False, vis, None, None, cnt, beams)
    weff = torch.empty((sh.C, 2, 2 * sh.B, sh.R, 2), dtype=torch.float32, device="cuda")
    plan.effective_weights(weff)
    torch.cuda.synchronize()
    assert plan.status()[0] == 0
    plan.close()
    return beams.cpu().numpy(), cnt.cpu().numpy(), weff.cpu().numpy()


def _run_learned(q, sh, samples, scales, weights, fixed, n_iter, tol):
    plan = sfgb.Plan(sh.C, sh.F, sh.Tp, sh.R, sh.Rpp, sh.P, sh.B)
    plan.set_weights(weights)
    plan.set_fixed_counts(fixed)
    s, sc = torch.as_tensor(samples).cuda(), torch.as_tensor(scales).cuda()
    vis = torch.empty(plan.vis_shape(), dtype=torch.int32, device="cuda")
    cnt = torch.full((sh.C, 2), -1, dtype=torch.int32, device="cuda")
    beams = torch.empty(plan.beams_shape(2), dtype=torch.float16, device="cuda")
    fb = torch.zeros(1, dtype=torch.int32, device="cuda")
    plan.run_adaptive_learned(q, s, sc, sfgb.SF_K_FIXED, 0.0, n_iter, tol, vis, cnt, beams, fallback_count=fb)
    weff = torch.empty((sh.C, 2, 2 * sh.B, sh.R, 2), dtype=torch.float32, device="cuda")
    plan.effective_weights(weff)
    torch.cuda.synchronize()
    assert plan.status()[0] == 0
    plan.close()
    return beams.cpu().numpy(), cnt.cpu().numpy(), weff.cpu().numpy(), int(fb.item())


def _depth(weff, steering, B):
    w = weff[..., 0].astype(np.float64) + 1j * weff[..., 1].astype(np.float64)
    r0, r1 = [], []
    for c, vecs in steering.items():
        for a in vecs:
            for p in range(2):
                r0.append(np.abs(w[c, p, :B] @ a[:, p]) ** 2)
                r1.append(np.abs(w[c, p, B:2 * B] @ a[:, p]) ** 2)
    return 10 * np.log10(np.sum(r1) / np.sum(r0))


def test_learned_chain_full_fallback_equals_plain_chain():
    """tol = 0 sends every matrix to the full eigensolver: the learned chain
    must then reproduce the plain chain exactly."""
    sh, samples, scales, weights, rfi, steering = _chain_inputs()
    fixed = np.full(sh.C, 2, np.int32)
    q = prop.Proposer(36, 512, 2 * sh.C)
    q.init_params(seed=0)
    plain = _run_plain(sh, samples, scales, weights, fixed)
    got = _run_learned(q, sh, samples, scales, weights, fixed, n_iter=2, tol=0.0)
    assert got[3] == 2 * sh.C
    assert np.array_equal(got[1], plain[1])
    assert np.array_equal(got[0], plain[0])
    q.close()


def test_learned_chain_null_depth_matches_fp64():
    """A briefly trained proposer, three subspace iterations, residual gate
    1e-3 ||A||: most matrices are accepted, the counts equal the plain
    chain's, and the null depth on the known interferers is within 0.5 dB of
    the FP64 full eigensolve's."""
    sh, samples, scales, weights, rfi, steering = _chain_inputs(C=128, seed=6)
    fixed = np.full(sh.C, 2, np.int32)
    q = prop.Proposer(36, 512, 8192)
    q.init_params(seed=0)
    x, t, w = prop.make_training_set(8 * 8192, q, P=16, chunk_channels=4096, seed=2)
    prop.train(q, x, t, w, epochs=10, batch=8192, lr=2e-3)
    beams, cnt, weff, nfb = _run_learned(q, sh, samples, scales, weights, fixed, n_iter=3, tol=1e-3)
    assert np.array_equal(cnt, np.full((sh.C, 2), 2, np.int32))
    assert nfb < 2 * sh.C  # the proposer is used
    ref = orc.adaptive_chain(sh, samples, scales, weights, k_fixed=fixed)
    d_learned = _depth(weff, steering, sh.B)
    wr = np.stack([ref["w_eff"].real, ref["w_eff"].imag], axis=-1)
    d_fp64 = _depth(wr, steering, sh.B)
    assert abs(d_learned - d_fp64) <= 0.5, (d_learned, d_fp64, nfb)
    q.close()
