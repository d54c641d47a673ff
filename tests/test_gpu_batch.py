"""Batched sub-arrays of uneven size (sf_batch_*) against the oracle (GPU only).

One mixed batch of units with 4..128 receivers runs through the persistent
correlator, the eigensolver size classes and the persistent beamformer.

Tolerances:
  visibilities  bit-exact (int32 vs the exact-integer oracle)
  eigenvalues   |lambda - lambda_lapack| <= 2e-5 ||A||_2 (whitened covariance)
  K             the device's noise-floor rule applied to its own eigenvalues
                (fp32), and equal to the oracle's for all but near-threshold cases
  beams slot 0  |y - y_ref| <= 2^-9 |y_ref| + 2^-6 + 2^-10 sum_r |w_r| |x_r(t)|
                (fp16 output and fp16 weight operands)
  beams slot 1  the same + 2e-3 max_t |y_ref| (projected weights from fp32
                eigenvectors)
"""
import numpy as np
import pytest
import torch

import sf_oracle as orc
import sfgb

pytestmark = pytest.mark.gpu

MIXED = [16, 36, 64, 128, 36, 16, 64, 4, 8, 48, 128, 16, 36, 20]


def _run(receivers, T, B, seed, k_rule, delta, fixed=None, autotune=False, graph=False):
    xs, ws = orc.synth_batch(receivers, T, B, seed=seed)
    bt = sfgb.Batch(receivers, T, B)
    bt.set_weights(bt.pack_weights(ws))
    if fixed is not None:
        bt.set_fixed_counts(fixed)
    s = torch.as_tensor(bt.pack_samples(xs)).cuda()
    vis = torch.full((bt.totals["vis"],), -7, dtype=torch.int32, device="cuda")
    ev = torch.zeros(bt.totals["evals"], dtype=torch.float32, device="cuda")
    cnt = torch.full((bt.n_units, 2), -1, dtype=torch.int32, device="cuda")
    beams = torch.full((2 * bt.totals["beams"],), float("nan"), dtype=torch.float16, device="cuda")
    report = None
    if autotune:
        report = bt.autotune(s, k_rule, delta, vis, ev, cnt, beams)
    if graph:
        stream = torch.cuda.Stream()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=stream):
            bt.run(s, k_rule, delta, False, vis, ev, cnt, beams, stream=stream)
        vis.fill_(-7)
        beams.fill_(float("nan"))
        g.replay()
    else:
        bt.run(s, k_rule, delta, False, vis, ev, cnt, beams)
    torch.cuda.synchronize()
    rc, bits = bt.status()
    assert rc == 0 and bits == 0, f"device status 0x{bits:x}"
    out = {"vis": vis.cpu().numpy(), "evals": ev.cpu().numpy(), "counts": cnt.cpu().numpy(),
           "beams": beams.cpu().numpy(), "xs": xs, "ws": ws, "batch": bt, "report": report}
    return out


def _check(out, receivers, B, k_rule, delta, fixed=None):
    bt = out["batch"]
    for u, R in enumerate(receivers):
        evals = bt.unit_evals(out["evals"], u)
        cnt = out["counts"][u]
        if k_rule == sfgb.SF_K_NOISE_FLOOR:
            for p in range(2):
                assert cnt[p] == orc.noise_floor_k_f32(evals[p], delta), f"unit {u}: K rule"
            ref = orc.unit_chain(out["xs"][u], out["ws"][u], "fixed", k_fixed=cnt)
        else:
            k = 0 if fixed is None else int(fixed[u])
            assert np.array_equal(cnt, [k, k])
            ref = orc.unit_chain(out["xs"][u], out["ws"][u], "fixed", k_fixed=k)
        assert np.array_equal(bt.unit_vis(out["vis"], u), ref["vis"]), f"unit {u} (R={R}): visibilities"
        nrm = np.abs(ref["evals"]).max(axis=-1, keepdims=True)
        assert np.all(np.abs(evals - ref["evals"]) <= 2e-5 * nrm), f"unit {u}: eigenvalues"
        y = bt.unit_beams(out["beams"], u).astype(np.float64)
        yb = y[..., 0] + 1j * y[..., 1]
        yr = ref["beams"]
        re, im = orc.unit_samples_split(out["xs"][u])
        ax = np.sqrt(re[0].astype(np.float64) ** 2 + im[0].astype(np.float64) ** 2)
        wsum = np.einsum("pmr,prt->pmt", np.abs(ref["w_eff"]), ax)
        tol0 = 2.0 ** -9 * np.abs(yr) + 2.0 ** -6 + 2.0 ** -10 * wsum
        tol1 = tol0 + 2e-3 * np.abs(yr).max(axis=-1, keepdims=True)
        err = np.abs(yb - yr)
        assert np.all(err[:, :B] <= tol0[:, :B]), f"unit {u}: slot 0 beams"
        assert np.all(err[:, B:] <= tol1[:, B:]), f"unit {u}: slot 1 beams"


def test_batch_mixed_fixed_k():
    fixed = np.array([(u % 3) for u in range(len(MIXED))], np.int32)
    out = _run(MIXED, 512, 4, seed=1, k_rule=sfgb.SF_K_FIXED, delta=0.0, fixed=fixed)
    _check(out, MIXED, 4, sfgb.SF_K_FIXED, 0.0, fixed)
    out["batch"].close()


def test_batch_noise_floor_rule_eight_beams():
    out = _run(MIXED, 1024, 8, seed=2, k_rule=sfgb.SF_K_NOISE_FLOOR, delta=10.0)
    _check(out, MIXED, 8, sfgb.SF_K_NOISE_FLOOR, 10.0)
    # units with strong interferers null something
    assert out["counts"].max() >= 1
    out["batch"].close()


def test_batch_autotune_and_graph_replay():
    """The autotuner's choice gives the same results, and the whole batch
    replays from one captured CUDA graph."""
    recv = [128, 16, 64, 36] * 6
    out = _run(recv, 512, 8, seed=3, k_rule=sfgb.SF_K_NOISE_FLOOR, delta=10.0, autotune=True, graph=True)
    rep = out["report"]
    assert "choice" in rep and rep["corr"] and rep["beam"] and rep["eig"]
    _check(out, recv, 8, sfgb.SF_K_NOISE_FLOOR, 10.0)
    out["batch"].close()


def test_batch_many_units_persistent_lists():
    """More work items than SMs, several per CTA, long integration (T = 4096,
    the 1024-sample chunks drained four times)."""
    rng = np.random.default_rng(9)
    recv = list(rng.choice([16, 36, 64, 128], size=300, p=[0.4, 0.3, 0.2, 0.1]))
    xs, ws = orc.synth_batch(recv, 4096, 8, seed=4, max_interferers=2)
    bt = sfgb.Batch(recv, 4096, 8)
    bt.set_weights(bt.pack_weights(ws))
    s = torch.as_tensor(bt.pack_samples(xs)).cuda()
    vis = torch.empty(bt.totals["vis"], dtype=torch.int32, device="cuda")
    bt.correlate(s, vis)
    torch.cuda.synchronize()
    assert bt.status()[0] == 0
    v = vis.cpu().numpy()
    for u in list(range(0, 300, 7)):
        ref = orc.correlate(orc.Shape(1, 1, 4096, recv[u], recv[u], 1, 1), *orc.unit_samples_split(xs[u]))[0]
        assert np.array_equal(bt.unit_vis(v, u), ref), f"unit {u}"
    bt.close()


def test_batch_rejects_unsupported_shapes():
    with pytest.raises(sfgb.SfError) as ei:
        sfgb.Batch([16, 30], 512, 4)  # not a multiple of 4
    assert ei.value.code == 2
    with pytest.raises(sfgb.SfError) as ei:
        sfgb.Batch([16], 500, 4)  # T not a multiple of 128
    assert ei.value.code == 2


def test_batch_k_beyond_kept_eigenvectors_is_clamped_and_reported():
    """A 128-receiver unit keeps 32 eigenvectors of its tridiagonal: a fixed K
    of 40 nulls the top 32, returns K = 32 and raises the bad-shape bit; a
    36-receiver unit in the same batch takes its K of 20 in full."""
    recv = [128, 36]
    fixed = np.array([40, 20], np.int32)
    xs, ws = orc.synth_batch(recv, 512, 4, seed=11)
    bt = sfgb.Batch(recv, 512, 4)
    bt.set_weights(bt.pack_weights(ws))
    bt.set_fixed_counts(fixed)
    s = torch.as_tensor(bt.pack_samples(xs)).cuda()
    vis = torch.empty(bt.totals["vis"], dtype=torch.int32, device="cuda")
    ev = torch.empty(bt.totals["evals"], dtype=torch.float32, device="cuda")
    cnt = torch.full((bt.n_units, 2), -1, dtype=torch.int32, device="cuda")
    beams = torch.empty(2 * bt.totals["beams"], dtype=torch.float16, device="cuda")
    bt.run(s, sfgb.SF_K_FIXED, 0.0, False, vis, ev, cnt, beams)
    torch.cuda.synchronize()
    rc, bits = bt.status()
    assert rc == sfgb.SF_ERR_DEVICE and bits & sfgb.SF_DEV_BAD_SHAPE
    c = cnt.cpu().numpy()
    assert np.array_equal(c[0], [32, 32]) and np.array_equal(c[1], [20, 20])
    # the 36-receiver unit's result is still the oracle's
    ref = orc.unit_chain(xs[1], ws[1], "fixed", k_fixed=20)
    e = bt.unit_evals(ev.cpu().numpy(), 1)
    assert np.all(np.abs(e - ref["evals"]) <= 2e-5 * np.abs(ref["evals"]).max(axis=-1, keepdims=True))
    assert np.all(np.isfinite(beams.cpu().numpy().astype(np.float32)))
    bt.close()


def test_batch_sizes_between_64_and_128_receivers():
    """Units of 68, 100 and 124 receivers (the sixteen-warp eigensolver with
    partly filled lanes and row slots) beside 4 and 60, against the oracle."""
    recv = [68, 100, 124, 4, 60, 100]
    out = _run(recv, 512, 6, seed=13, k_rule=sfgb.SF_K_NOISE_FLOOR, delta=10.0)
    _check(out, recv, 6, sfgb.SF_K_NOISE_FLOOR, 10.0)
    out["batch"].close()
