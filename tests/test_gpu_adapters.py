"""C++ GPUPipeline adapters (include/sf_pipeline.hpp) driven like the
reference's ProcessorState drives its pipelines (GPU only).

The harness (tests/cpp/adapter_harness.cpp) runs two buffers through each
adapter with two-deep buffering and one visibility dump; its landed outputs
must equal the direct C-ABI chains on the same inputs bit for bit, and the
hand-off protocol (buffer release, transfer-complete calls, missing-packet
bookkeeping) must follow the reference's.
"""
import os
import subprocess

import numpy as np
import pytest
import torch

import sf_oracle as orc
import sfgb

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
# TestConfig of the harness
C, F, TP, R, RPP, P, B = 6, 2, 16, 10, 5, 8, 3
FFT_DOWNSAMPLE, FFT_TRIM = 16, 5
DELAYS = [3, -5]
K_MAP = [c % 3 for c in range(C)]


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    libdir = os.path.dirname(os.path.abspath(sfgb.__file__))
    exe = str(tmp_path_factory.mktemp("adapter") / "adapter_harness")
    cmd = ["nvcc", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", "adapter_harness.cpp"), "-L", libdir, "-lsfgb",
           "-Xlinker", "-rpath," + libdir, "-o", exe]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


@pytest.fixture(scope="module")
def inputs():
    sh = orc.Shape(C, F, TP, R, RPP, P, B)
    s0, sc0, _ = orc.synth_inputs(sh, seed=21, n_interferers=1, inr_db=15.0, frac_channels=0.5)
    s1, sc1, _ = orc.synth_inputs(sh, seed=22, n_interferers=1, inr_db=15.0, frac_channels=0.5)
    w = orc.synth_weights(sh, seed=3).astype(np.float16)
    return sh, [s0, s1], [sc0, sc1], w


def _run(harness, mode, inputs, tmp_path, steer=False):
    """steer: False, True (an SfBeamSteering) or "refsteer" (reference-style steering)."""
    sh, samples, scales, w = inputs
    np.concatenate([s.reshape(-1) for s in samples]).astype(np.int8).tofile(tmp_path / "samples.bin")
    np.concatenate([s.reshape(-1) for s in scales]).astype(np.int16).tofile(tmp_path / "scales.bin")
    np.ascontiguousarray(w).tofile(tmp_path / "weights.bin")
    flag = [] if not steer else (["refsteer"] if steer == "refsteer" else ["steer"])
    cmd = [harness, str(mode), str(tmp_path)] + flag
    res = subprocess.run(cmd, capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stderr
    proto = {}
    for line in (tmp_path / "protocol.txt").read_text().splitlines():
        k, *v = line.split()
        proto[k] = v if k == "order" else [int(x) for x in v]
    return proto


def _dev(x, dtype):
    return torch.as_tensor(np.ascontiguousarray(x)).to(device="cuda").view(dtype)


# the harness's steering geometry (adapter_harness.cpp, "steer")
STEER_ENU = [(3.0 * r, -2.0 * r, 0.5 * r + r % 3) for r in range(R)]
STEER_CONNECTED = [0 if r == 4 else 1 for r in range(R)]


def _direct(mode, inputs, steer=False):
    """The same two integrations through the C ABI directly."""
    sh, samples, scales, w = inputs
    plan = sfgb.Plan(C, F, TP, R, RPP, P, B)
    plan.set_weights(w)
    if steer:
        plan.set_steering_weights([(0.0, 0.0, 1.0)] * B, STEER_ENU, STEER_CONNECTED, 1.0e9, 1.0e5, 50)
    if mode != 0:
        plan.set_subpacket_delays(DELAYS)
    if mode == 2:
        plan.set_fixed_counts(np.array(K_MAP, np.int32))
    slots = 2 if mode == 2 else 1
    accum = torch.zeros(plan.vis_shape(), dtype=torch.int64, device="cuda")
    out = {"beams": [], "evals": [], "counts": [], "fft": []}
    for run in range(2):
        s, sc = _dev(samples[run], torch.int8), _dev(scales[run], torch.int16)
        vis = torch.empty(plan.vis_shape(), dtype=torch.int32, device="cuda")
        beams = torch.empty(plan.beams_shape(slots), dtype=torch.float16, device="cuda")
        if mode == 0:
            plan.run_corr_beam(s, sc, vis, beams)
        elif mode == 1:
            ev = torch.empty((C, 2, 2, R), dtype=torch.float32, device="cuda")
            evec = torch.empty((C, 2, 2, R, R, 2), dtype=torch.float32, device="cuda")
            plan.run_lambda_gpu(s, sc, vis, ev, evec, beams)
            out["evals"].append(ev.cpu().numpy())
        else:
            ev = torch.empty((C, 2, R), dtype=torch.float32, device="cuda")
            cnt = torch.empty((C, 2), dtype=torch.int32, device="cuda")
            plan.run_adaptive(s, sc, sfgb.SF_K_FIXED, 3.0, False, vis, ev, None, cnt, beams)
            out["evals"].append(ev.cpu().numpy())
            out["counts"].append(cnt.cpu().numpy())
        plan.accumulate_visibilities(vis, accum)
        out["beams"].append(beams.cpu().numpy())
        if mode == 1:
            spec = torch.empty(plan.beam_spectra_shape(B, FFT_DOWNSAMPLE), dtype=torch.float32, device="cuda")
            plan.beam_spectra(beams, B, FFT_DOWNSAMPLE, spec)
            out["fft"].append(spec.cpu().numpy())
        elif mode == 2:
            spec = torch.empty(plan.packet_spectra_shape(2 * B, FFT_TRIM), dtype=torch.float32, device="cuda")
            plan.packet_spectra(beams, 2 * B, FFT_TRIM, spec)
            out["fft"].append(spec.cpu().numpy())
    vis_f = torch.empty(plan.vis_shape(), dtype=torch.float32, device="cuda")
    plan.visibilities_to_float(accum, vis_f)
    out["vis"] = vis_f.cpu().numpy()
    rc, bits = plan.status()
    assert rc == 0 and bits == 0
    plan.close()
    return out


@pytest.mark.parametrize("mode", [0, 1, 2], ids=["corr_beam_only", "lambda_gpu", "adaptive"])
def test_adapter_matches_direct_chain(harness, inputs, tmp_path, mode):
    proto = _run(harness, mode, inputs, tmp_path)
    ref = _direct(mode, inputs)
    slots = 2 if mode == 2 else 1
    for run in range(2):
        got = np.fromfile(tmp_path / f"beams_{run}.bin", dtype=np.float16).reshape(C, 2, slots * B, P * TP, 2)
        assert np.array_equal(got, ref["beams"][run]), f"beams of run {run}"
        if mode != 0:
            ev = np.fromfile(tmp_path / f"evals_{run}.bin", dtype=np.float32).reshape(ref["evals"][run].shape)
            assert np.array_equal(ev, ref["evals"][run])
        if mode != 0:
            fft = np.fromfile(tmp_path / f"fft_{run}.bin", dtype=np.float32).reshape(ref["fft"][run].shape)
            assert np.array_equal(fft, ref["fft"][run]), f"spectra of run {run}"
        if mode == 2:
            cnt = np.fromfile(tmp_path / f"counts_{run}.bin", dtype=np.int32).reshape(C, 2)
            assert np.array_equal(cnt, ref["counts"][run])
            assert np.array_equal(cnt[:, 0], np.array(K_MAP))
    vis = np.fromfile(tmp_path / "vis.bin", dtype=np.float32).reshape(ref["vis"].shape)
    assert np.array_equal(vis, ref["vis"])
    # hand-off protocol of the reference's pipelines
    assert sorted(proto["released"]) == [10, 11]
    assert proto["beam_done"] == [2] and proto["arrivals_done"] == [2] and proto["vis_done"] == [1]
    assert proto["eig_done"] == [0 if mode == 0 else 2]
    assert proto["vis_missing"] == [1] and proto["vis_total"] == [2 * C * P * F]
    assert proto["vis_start"] == [1000] and proto["vis_end"] == [2999]
    assert proto["status"] == [0]
    # spectra tails land once per run, in each reference pipeline's order
    assert proto["fft_done"] == [0 if mode == 0 else 2]
    run_order = {0: ["beam"], 1: ["beam", "eig", "fft"], 2: ["beam", "fft", "eig"]}[mode]
    assert proto["order"] == run_order * 2


def test_adapter_spectra_match_oracle(harness, inputs, tmp_path):
    """The landed spectra of both tails against the oracle's transforms of
    the landed fp16 beams."""
    for mode in (1, 2):
        _run(harness, mode, inputs, tmp_path)
        slots = 2 if mode == 2 else 1
        for run in range(2):
            beams = np.fromfile(tmp_path / f"beams_{run}.bin", dtype=np.float16).reshape(
                C, 2, slots * B, P * TP, 2)
            bc = orc.beams_from_half(beams)
            ref = orc.beam_spectra(bc, FFT_DOWNSAMPLE) if mode == 1 else orc.packet_spectra(bc, TP, FFT_TRIM)
            got = np.fromfile(tmp_path / f"fft_{run}.bin", dtype=np.float32).reshape(ref.shape)
            m = np.abs(ref).mean(axis=-1, keepdims=True)
            assert np.all(np.abs(got - ref) <= 2e-5 * m + 1e-6 * np.abs(ref))


def test_adapter_visibilities_match_oracle(harness, inputs, tmp_path):
    """The dumped visibilities of two corr+beam integrations are the oracle's
    int64 sum of both, exactly (|x s| <= 128 keeps every chunk exact)."""
    sh, samples, scales, w = inputs
    _run(harness, 0, inputs, tmp_path)
    total = None
    for run in range(2):
        off = orc.sample_offsets(sh, None, mode="packet")
        re, im = orc.aligned_samples(sh, samples[run], scales[run], off)
        v = orc.correlate(sh, re, im)
        total = v if total is None else total + v
    vis = np.fromfile(tmp_path / "vis.bin", dtype=np.float32).reshape(total.shape)
    assert np.array_equal(vis.astype(np.int64), total)


@pytest.mark.parametrize("mode", [0, 2], ids=["corr_beam_only", "adaptive"])
def test_adapter_beam_steering(harness, inputs, tmp_path, mode):
    """An attached SfBeamSteering refreshes the plans' weights before the first
    run: the landed beams equal a direct chain whose plan was steered with the
    same geometry, and differ from the unsteered ones."""
    _run(harness, mode, inputs, tmp_path, steer=True)
    ref = _direct(mode, inputs, steer=True)
    plain = _direct(mode, inputs)
    slots = 2 if mode == 2 else 1
    for run in range(2):
        got = np.fromfile(tmp_path / f"beams_{run}.bin", dtype=np.float16).reshape(C, 2, slots * B, P * TP, 2)
        assert np.array_equal(got, ref["beams"][run])
        assert not np.array_equal(got, plain["beams"][run])


@pytest.mark.parametrize("mode", [0, 1, 2], ids=["corr_beam_only", "lambda_gpu", "adaptive"])
def test_adapter_reference_style_steering(harness, inputs, tmp_path, mode):
    """A steering object with the reference BeamSteering<T>'s interface
    (register_buffer + maybe_refresh) passed as the constructor's third
    argument: its asynchronous weight copies land in every buffer's plan, so
    the landed beams equal a direct chain run with those weights."""
    sh, samples, scales, w = inputs
    w2 = orc.synth_weights(sh, seed=17).astype(np.float16)
    np.ascontiguousarray(w2).tofile(tmp_path / "weights2.bin")
    _run(harness, mode, inputs, tmp_path, steer="refsteer")
    ref = _direct(mode, (sh, samples, scales, w2))
    slots = 2 if mode == 2 else 1
    for run in range(2):
        got = np.fromfile(tmp_path / f"beams_{run}.bin", dtype=np.float16).reshape(C, 2, slots * B, P * TP, 2)
        assert np.array_equal(got, ref["beams"][run])
