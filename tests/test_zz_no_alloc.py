"""Allocation-free adaptive chain: sf_run_adaptive_noalloc against sf_run_adaptive.

Some callers of this library cannot call cudaMalloc: a real-time thread or a
CUDA host callback that must never block on the device allocator, or a plugin
running inside a host application that owns all device memory and hands it
pre-allocated buffers.  sf_run_adaptive_noalloc serves them: it takes only
caller-owned inputs and outputs and keeps its intermediates in a fixed 16 MiB
static device array.  These tests call it through the C ABI and check it
against the plan-based entry point, twice in a row (the array keeps the
previous call's contents, which must not leak into the next result).

This file is collected last on purpose, so a run that stops at the first
failure has already run every other test.
"""
import numpy as np
import pytest
import torch

import sf_oracle as orc
import sfgb

pytestmark = pytest.mark.gpu

SHAPE = (24, 4, 64, 36, 9, 16, 4)  # C, F, Tp, R, Rpp, P, B


def _inputs(seed):
    sh = orc.Shape(*SHAPE)
    samples, scales, _ = orc.synth_inputs(sh, seed=seed, n_interferers=2, frac_channels=0.5)
    weights = orc.synth_weights(sh, seed=seed + 10)
    rng = np.random.default_rng(seed)
    gains = (rng.normal(1, 0.1, (sh.C, 2, sh.R)) + 1j * rng.normal(0, 0.1, (sh.C, 2, sh.R))).astype(np.complex64)
    delays = rng.integers(-sh.Tp, sh.Tp + 1, size=sh.F).astype(np.int32)
    fixed = rng.integers(0, 3, size=sh.C).astype(np.int32)
    return sh, samples, scales, weights, gains, delays, fixed


def _plan_path(sh, samples, scales, weights, gains, delays, fixed, k_rule, delta):
    plan = sfgb.Plan(*SHAPE)
    plan.set_weights(weights)
    plan.set_antenna_gains(gains)
    plan.set_subpacket_delays(delays)
    plan.set_fixed_counts(fixed)
    s = torch.as_tensor(samples).cuda()
    sc = torch.as_tensor(scales).cuda()
    beams = torch.empty(plan.beams_shape(2), dtype=torch.float16, device="cuda")
    cnt = torch.empty((sh.C, 2), dtype=torch.int32, device="cuda")
    plan.run_adaptive(s, sc, k_rule, delta, False, None, None, None, cnt, beams)
    torch.cuda.synchronize()
    assert plan.status()[0] == 0
    plan.close()
    return beams.cpu().numpy().astype(np.float32), cnt.cpu().numpy()


def _noalloc_path(sh, samples, scales, weights, gains, delays, fixed, k_rule, delta):
    s = torch.as_tensor(samples).cuda()
    sc = torch.as_tensor(scales).cuda()
    w = torch.as_tensor(np.ascontiguousarray(weights)).cuda()
    fac = torch.as_tensor(np.ascontiguousarray(np.stack([gains.real, gains.imag], -1).astype(np.float32))).cuda()
    dl = torch.as_tensor(delays).cuda()
    fx = torch.as_tensor(fixed).cuda()
    beams = torch.full((sh.C, 2, 2 * sh.B, sh.T, 2), float("nan"), dtype=torch.float16, device="cuda")
    cnt = torch.full((sh.C, 2), -1, dtype=torch.int32, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    sfgb.run_adaptive_noalloc(SHAPE, s, sc, w, k_rule, delta, False, beams, factors=fac, delays=dl,
                              fixed_counts=fx, counts=cnt, status=status)
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    return beams.cpu().numpy().astype(np.float32), cnt.cpu().numpy()


def _close(a, b):
    ya = a[..., 0] + 1j * a[..., 1]
    yb = b[..., 0] + 1j * b[..., 1]
    tol = 2.0 ** -9 * np.abs(yb) + 2.0 ** -6
    return bool(np.all(np.abs(ya - yb) <= tol))


def test_noalloc_matches_plan_entry_point_on_two_calls_in_a_row():
    for seed, k_rule, delta in ((0, sfgb.SF_K_FIXED, 0.0), (1, sfgb.SF_K_DETECT, 3.0)):
        args = _inputs(seed)
        ref_beams, ref_counts = _plan_path(*args, k_rule, delta)
        got_beams, got_counts = _noalloc_path(*args, k_rule, delta)
        assert np.array_equal(got_counts, ref_counts)
        assert _close(got_beams, ref_beams)


def test_noalloc_rejects_shapes_beyond_its_scratch():
    big = (4096, 4, 64, 36, 9, 16, 4)
    s = torch.zeros(16, dtype=torch.int8, device="cuda")
    sc = torch.zeros(16, dtype=torch.int16, device="cuda")
    w = torch.zeros(16, dtype=torch.float16, device="cuda")
    beams = torch.zeros(16, dtype=torch.float16, device="cuda")
    with pytest.raises(sfgb.SfError) as ei:
        sfgb.run_adaptive_noalloc(big, s, sc, w, sfgb.SF_K_FIXED, 0.0, False, beams)
    assert ei.value.code == 2 and "scratch" in str(ei.value)


def test_noalloc_second_call_allocates_nothing():
    # The first call on a device is the set-up call (it resolves the static
    # array's address); after it, a call must leave both the device's free
    # memory and torch's allocator untouched.
    args = _inputs(3)
    sh, samples, scales, weights, gains, delays, fixed = args
    s = torch.as_tensor(samples).cuda()
    sc = torch.as_tensor(scales).cuda()
    w = torch.as_tensor(np.ascontiguousarray(weights)).cuda()
    beams = torch.empty((sh.C, 2, 2 * sh.B, sh.T, 2), dtype=torch.float16, device="cuda")
    cnt = torch.empty((sh.C, 2), dtype=torch.int32, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    call = lambda: sfgb.run_adaptive_noalloc(SHAPE, s, sc, w, sfgb.SF_K_FIXED, 0.0, False, beams,
                                             counts=cnt, status=status)
    call()
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    alloc0 = torch.cuda.memory_allocated()
    call()
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert torch.cuda.memory_allocated() == alloc0
    assert free1 == free0
    assert int(status.item()) == 0


def test_noalloc_out_of_range_delay_is_replaced_and_reported():
    # A delay outside [-Tp, Tp] would move the sample window outside the
    # caller's buffer: the entry point replaces it by 0 and raises the
    # SF_DEV_BAD_DELAY bit, and the beams equal those of a zero delay.
    sh, samples, scales, weights, gains, delays, fixed = _inputs(4)
    bad = np.zeros(sh.F, np.int32)
    bad[1] = 3 * sh.Tp
    bad[2] = -2 * sh.Tp - 5
    got_beams, got_counts, bits = _noalloc_with_delays(sh, samples, scales, weights, bad)
    assert bits & sfgb.SF_DEV_BAD_DELAY
    ref_beams, ref_counts, ref_bits = _noalloc_with_delays(sh, samples, scales, weights, np.zeros(sh.F, np.int32))
    assert ref_bits == 0
    assert np.all(np.isfinite(got_beams))
    assert np.array_equal(got_counts, ref_counts)
    assert np.array_equal(got_beams, ref_beams)


def _noalloc_with_delays(sh, samples, scales, weights, delays):
    s = torch.as_tensor(samples).cuda()
    sc = torch.as_tensor(scales).cuda()
    w = torch.as_tensor(np.ascontiguousarray(weights)).cuda()
    dl = torch.as_tensor(delays).cuda()
    fx = torch.ones(sh.C, dtype=torch.int32, device="cuda")
    beams = torch.full((sh.C, 2, 2 * sh.B, sh.T, 2), float("nan"), dtype=torch.float16, device="cuda")
    cnt = torch.full((sh.C, 2), -1, dtype=torch.int32, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    sfgb.run_adaptive_noalloc(SHAPE, s, sc, w, sfgb.SF_K_FIXED, 0.0, False, beams, delays=dl,
                              fixed_counts=fx, counts=cnt, status=status)
    torch.cuda.synchronize()
    return beams.cpu().numpy().astype(np.float32), cnt.cpu().numpy(), int(status.item())


def test_noalloc_status_word_is_only_or_ed():
    # The caller's status word is only OR-ed into, never cleared: a bit left from
    # an earlier call stays set after a clean call, and the results are unchanged.
    sh, samples, scales, weights, gains, delays, fixed = _inputs(5)
    s = torch.as_tensor(samples).cuda()
    sc = torch.as_tensor(scales).cuda()
    w = torch.as_tensor(np.ascontiguousarray(weights)).cuda()
    fac = torch.as_tensor(np.ascontiguousarray(np.stack([gains.real, gains.imag], -1).astype(np.float32))).cuda()
    dl = torch.as_tensor(delays).cuda()
    fx = torch.as_tensor(fixed).cuda()
    beams = torch.full((sh.C, 2, 2 * sh.B, sh.T, 2), float("nan"), dtype=torch.float16, device="cuda")
    cnt = torch.full((sh.C, 2), -1, dtype=torch.int32, device="cuda")
    stale = sfgb.SF_DEV_BAD_DELAY
    status = torch.full((1,), stale, dtype=torch.int32, device="cuda")
    sfgb.run_adaptive_noalloc(SHAPE, s, sc, w, sfgb.SF_K_FIXED, 0.0, False, beams, factors=fac, delays=dl,
                              fixed_counts=fx, counts=cnt, status=status)
    torch.cuda.synchronize()
    assert int(status.item()) == stale
    ref_beams, ref_counts = _plan_path(sh, samples, scales, weights, gains, delays, fixed, sfgb.SF_K_FIXED, 0.0)
    assert np.array_equal(cnt.cpu().numpy(), ref_counts)
    assert _close(beams.cpu().numpy().astype(np.float32), ref_beams)
