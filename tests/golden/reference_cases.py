"""Exact-value golden cases from the reference's own GPU test-suite.

Each case rebuilds the inputs one reference test feeds its pipeline and
records the values that test asserts, read from the test sources:

  tests/test_pipeline.cu            LambdaGPUPipeline goldens
  tests/test_corr_beam_pipeline.cu  LambdaCorrBeamOnlyGPUPipeline goldens
  tests/test_adaptive_pipeline.cu   adaptive null/shrink/detect goldens

Shapes follow the reference's LambdaConfig (channels, FPGAs, samples per
packet, receivers, receivers per packet, packets, beams); padded-receiver
counts are a TCC detail and do not appear.  Layouts: samples
int8[C][P+2][F][Tp][Rpp][Pol][2], scales int16[C][P+2][R][Pol], weights
float16 pairs [C][Pol][B][R][2], gains complex [C][Pol][R].
"""
from __future__ import annotations

import numpy as np

NPOL = 2


class Case:
    def __init__(self, name, cite, path, shape, samples, scales, weights,
                 gains=None, delays=None, adaptive=None, expect=None):
        self.name = name
        self.cite = cite
        self.path = path          # "lambda_gpu" | "corr_beam" | "adaptive"
        self.shape = shape        # (C, F, Tp, R, Rpp, P, B)
        self.samples = samples
        self.scales = scales
        self.weights = weights
        self.gains = gains
        self.delays = delays
        self.adaptive = adaptive or {}
        self.expect = expect or {}

    def __repr__(self):
        return f"Case({self.name})"


def _arrays(shape):
    C, F, Tp, R, Rpp, P, B = shape
    s = np.zeros((C, P + 2, F, Tp, Rpp, NPOL, 2), np.int8)
    sc = np.zeros((C, P + 2, R, NPOL), np.int16)
    w = np.zeros((C, NPOL, B, R, 2), np.float16)
    return s, sc, w


def _unity(shape):
    s, sc, w = _arrays(shape)
    w[..., 0] = 1.0
    return s, sc, w


SMALL = (1, 1, 8, 4, 4, 1, 1)       # test_pipeline.cu:72-88 Config
MULTI_FPGA = (1, 3, 8, 6, 2, 1, 1)  # test_pipeline.cu:90-96 MultiFPGAConfig
ADAPTIVE = (1, 1, 64, 4, 4, 1, 1)   # test_adaptive_pipeline.cu:37-50


def build_cases():
    cases = []

    # ---------------- LambdaGPUPipeline (test_pipeline.cu) ----------------
    s, sc, w = _unity(SMALL)
    s[..., 0], s[..., 1], sc[...] = 2, -2, 1
    cases.append(Case("Ex1", "tests/test_pipeline.cu:98-184", "lambda_gpu", SMALL, s, sc, w,
                      expect={"beam": lambda c, p, m, t: (8.0, -8.0),
                              "vis_re": lambda c, b, p, q: 64.0, "vis_im": 0.0}))

    s, sc, w = _unity(SMALL)
    s[:, :, 0, :, :, 0, 0], s[:, :, 0, :, :, 0, 1] = 2, -2
    sc[...] = 1
    cases.append(Case("PolarizationBlank", "tests/test_pipeline.cu:186-284", "lambda_gpu", SMALL, s, sc, w,
                      expect={"beam": lambda c, p, m, t: (0.0, 0.0) if p == 1 else (8.0, -8.0),
                              "vis_re": lambda c, b, p, q: 0.0 if (p == 1 or q == 1) else 64.0}))

    shp = (6, 1, 8, 4, 4, 1, 1)
    s, sc, w = _unity(shp)
    s[:, :, 0, :, :, 1, 0], s[:, :, 0, :, :, 1, 1] = 2, -2
    sc[...] = 1
    cases.append(Case("PolarizationBlank2", "tests/test_pipeline.cu:286-395", "lambda_gpu", shp, s, sc, w,
                      expect={"beam": lambda c, p, m, t: (0.0, 0.0) if p == 0 else (8.0, -8.0),
                              "vis_re": lambda c, b, p, q: 0.0 if (p == 0 or q == 0) else 64.0}))

    shp = (1, 1, 8, 4, 4, 1, 2)
    s, sc, w = _arrays(shp)
    s[..., 0], s[..., 1], sc[...] = 2, -2, 1
    w[:, :, 0, :, 0] = 1.0
    cases.append(Case("BeamBlank", "tests/test_pipeline.cu:397-482", "lambda_gpu", shp, s, sc, w,
                      expect={"beam": lambda c, p, m, t: (0.0, 0.0) if m == 1 else (8.0, -8.0)}))

    shp = (2, 1, 8, 4, 4, 1, 1)
    s, sc, w = _arrays(shp)
    s[..., 0], s[..., 1], sc[...] = 2, -2, 1
    w[0, ..., 0] = 1.0
    cases.append(Case("ChannelWeightBlank", "tests/test_pipeline.cu:484-568", "lambda_gpu", shp, s, sc, w,
                      expect={"beam": lambda c, p, m, t: (0.0, 0.0) if c == 1 else (8.0, -8.0)}))

    s, sc, w = _unity(shp)
    s[0, ..., 0], s[0, ..., 1], sc[...] = 2, -2, 1
    cases.append(Case("ChannelSamplesBlank", "tests/test_pipeline.cu:570-658", "lambda_gpu", shp, s, sc, w,
                      expect={"beam": lambda c, p, m, t: (0.0, 0.0) if c == 1 else (8.0, -8.0)}))

    s, sc, w = _unity(SMALL)
    s[..., 0], s[..., 1], sc[...] = 2, -2, 2
    cases.append(Case("Scales", "tests/test_pipeline.cu:660-747", "lambda_gpu", SMALL, s, sc, w,
                      expect={"beam": lambda c, p, m, t: (16.0, -16.0),
                              "vis_re": lambda c, b, p, q: 256.0}))

    shp = (1, 1, 8, 4, 4, 2, 1)
    s, sc, w = _unity(shp)
    s[..., 0], s[..., 1] = 2, -2
    for j in range(-1, shp[5] + 1):
        sc[:, j + 1] = j
    cases.append(Case("ScalesMultiplePackets", "tests/test_pipeline.cu:749-847", "lambda_gpu", shp, s, sc, w,
                      expect={"beam": lambda c, p, m, t: (0.0, 0.0) if t // 8 == 0 else (8.0, -8.0),
                              "vis_re": lambda c, b, p, q: 64.0}))

    s, sc, w = _unity(SMALL)
    for l in range(4):
        s[:, :, 0, :, l, :, 0] = l
        s[:, :, 0, :, l, :, 1] = -l
        sc[:, :, l, :] = l
    spr = {2: 16.0, 4: 64.0, 5: 256.0, 7: 144.0, 8: 576.0, 9: 1296.0}
    cases.append(Case("ScalesPerReceiver", "tests/test_pipeline.cu:849-954", "lambda_gpu", SMALL, s, sc, w,
                      expect={"beam": lambda c, p, m, t: (14.0, -14.0),
                              "vis_re": lambda c, b, p, q: spr.get(b, 0.0)}))

    s, sc, w = _unity(SMALL)
    s[..., 0], s[..., 1], sc[...] = 2, -2, 1
    cases.append(Case("EigenvalueBasic", "tests/test_pipeline.cu:956-1052", "lambda_gpu", SMALL, s, sc, w,
                      expect={"evals": [0.0, 0.0, 0.0, 256.0], "evals_tol": 1e-4,
                              "principal_evec": 0.5, "evec_tol": 1e-4}))

    delays = [0, 3, -4]
    s, sc, w = _unity(MULTI_FPGA)
    P, Tp = MULTI_FPGA[5], MULTI_FPGA[2]
    sc[...] = 1
    for f in range(3):
        for j in range(-1, P + 1):
            for k in range(Tp):
                on = ((f == 0 and j not in (-1, P))
                      or (f == 1 and ((j == P and k < delays[1]) or (j == 0 and k >= delays[1])))
                      or (f == 2 and ((j == 0 and k < -delays[2]) or (j == -1 and k >= Tp + delays[2]))))
                if on:
                    s[:, j + 1, f, k, :, :, 0] = 2
                    s[:, j + 1, f, k, :, :, 1] = -2
    cases.append(Case("DelayBeam", "tests/test_pipeline.cu:1054-1155", "lambda_gpu", MULTI_FPGA, s, sc, w,
                      delays=delays, expect={"beam": lambda c, p, m, t: (12.0, -12.0)}))

    s, sc, w = _unity(MULTI_FPGA)
    s[..., 0], s[..., 1], sc[...] = 2, -2, 1
    g = np.zeros((1, NPOL, 6), np.complex64)
    for pol in range(NPOL):
        for r in range(6):
            v = float(r * NPOL + pol)
            g[0, pol, r] = v + 1j * v
    cases.append(Case("Gains", "tests/test_pipeline.cu:1157-1256", "lambda_gpu", MULTI_FPGA, s, sc, w,
                      gains=g, delays=[0, 0, 0],
                      expect={"beam": lambda c, p, m, t: (120.0, 0.0) if p == 0 else (144.0, 0.0)}))

    s, sc, w = _unity(MULTI_FPGA)
    s[:, :, 2, ..., 0], s[:, :, 2, ..., 1], sc[...] = 2, -2, 1
    cases.append(Case("GainsOnlyOneFPGAPresent", "tests/test_pipeline.cu:1258-1360", "lambda_gpu", MULTI_FPGA,
                      s, sc, w, gains=g, delays=[0, 0, 0],
                      expect={"beam": lambda c, p, m, t: (72.0, 0.0) if p == 0 else (80.0, 0.0)}))

    # ---------- LambdaCorrBeamOnlyGPUPipeline (test_corr_beam_pipeline.cu) ----------
    s, sc, w = _unity(SMALL)
    s[..., 0], s[..., 1], sc[...] = 2, -2, 1
    cases.append(Case("CorrBeamExact", "tests/test_corr_beam_pipeline.cu:107-143", "corr_beam", SMALL, s, sc, w,
                      expect={"beam": lambda c, p, m, t: (8.0, -8.0),
                              "vis_re": lambda c, b, p, q: 64.0, "vis_im": 0.0}))

    s, sc, w = _unity(SMALL)
    sc[...] = 1
    cases.append(Case("CorrBeamZeroInput", "tests/test_corr_beam_pipeline.cu:156-181", "corr_beam", SMALL, s, sc, w,
                      expect={"beam": lambda c, p, m, t: (0.0, 0.0),
                              "vis_re": lambda c, b, p, q: 0.0, "vis_im": 0.0}))

    s, sc, w = _arrays(SMALL)
    s[..., 0], s[..., 1], sc[...] = 2, -2, 1
    cases.append(Case("CorrBeamZeroWeights", "tests/test_corr_beam_pipeline.cu:183-211", "corr_beam", SMALL,
                      s, sc, w, expect={"beam": lambda c, p, m, t: (0.0, 0.0),
                                        "vis_re": lambda c, b, p, q: 64.0}))

    s, sc, w = _arrays(SMALL)
    s[..., 0], s[..., 1], sc[...] = 2, -2, 1
    w[..., 0] = 2.0
    cases.append(Case("CorrBeamDoubleWeights", "tests/test_corr_beam_pipeline.cu:213-252", "corr_beam", SMALL,
                      s, sc, w, expect={"beam": lambda c, p, m, t: (16.0, -16.0),
                                        "vis_re": lambda c, b, p, q: 64.0, "vis_im": 0.0}))

    shp = (2, 1, 8, 4, 4, 1, 1)
    s, sc, w = _unity(shp)
    s[0, ..., 0], s[0, ..., 1] = 2, -2
    s[1, ..., 0], s[1, ..., 1] = 3, 1
    sc[...] = 1
    cases.append(Case("CorrBeamTwoChannel", "tests/test_corr_beam_pipeline.cu:254-304", "corr_beam", shp, s, sc, w,
                      expect={"beam": lambda c, p, m, t: ((8.0, -8.0), (12.0, 4.0))[c],
                              "auto_re": lambda c, r, p: (64.0, 80.0)[c]}))

    s, sc, w = _unity(SMALL)
    s[..., 0] = 1
    for r in range(4):
        for p in range(NPOL):
            sc[:, :, r, p] = (r + 1) * (p + 1)
    cases.append(Case("CorrBeamNonUnitScales", "tests/test_corr_beam_pipeline.cu:306-346", "corr_beam", SMALL,
                      s, sc, w, expect={"beam": lambda c, p, m, t: (10.0 * (p + 1), 0.0),
                                        "auto_re": lambda c, r, p: 8.0 * ((r + 1) * (p + 1)) ** 2}))

    shp = (1, 1, 8, 4, 4, 2, 1)
    s, sc, w = _unity(shp)
    s[..., 0], s[..., 1], sc[...] = 2, -2, 1
    cases.append(Case("CorrBeamTwoPacket", "tests/test_corr_beam_pipeline.cu:348-392", "corr_beam", shp, s, sc, w,
                      expect={"beam": lambda c, p, m, t: (8.0, -8.0),
                              "auto_re": lambda c, r, p: 128.0}))

    # ---------- Adaptive pipeline (test_adaptive_pipeline.cu) ----------
    def adaptive_inputs(fn):
        s, sc, w = _unity(ADAPTIVE)
        C, F, Tp, R, Rpp, P, B = ADAPTIVE
        for j in range(P + 2):
            for t in range(Tp):
                for r in range(R):
                    for p in range(NPOL):
                        v = fn(0, t, r, p)
                        s[0, j, 0, t, r, p] = v
        sc[...] = 1
        return s, sc, w

    const = adaptive_inputs(lambda c, t, r, p: (2, -2))
    cases.append(Case("AdaptiveNullK1RankOne", "tests/test_adaptive_pipeline.cu:414-423,491-511", "adaptive",
                      ADAPTIVE, *const, adaptive={"k": 1},
                      expect={"beam_slot0": (8.0, -8.0), "beam_slot1_abs_max": 0.25,
                              "slot1_power_max": 1.0}))
    cases.append(Case("AdaptiveNullK0", "tests/test_adaptive_pipeline.cu:375-409", "adaptive",
                      ADAPTIVE, *const, adaptive={"k": 0},
                      expect={"slots_identical": True, "slot1_power_min": 1e-9}))

    def tagged(c, t, r, p):
        if r != 0:
            return (0, 0)
        return (t + 1, -(1 + 10 * p + 20 * c))
    tag = adaptive_inputs(tagged)
    cases.append(Case("AdaptiveTaggedLayoutK0", "tests/test_adaptive_pipeline.cu:425-452", "adaptive",
                      ADAPTIVE, *tag, adaptive={"k": 0},
                      expect={"beam_all_slots": lambda c, p, t: (float(t + 1), float(-(1 + 10 * p + 20 * c)))}))

    def multimode(c, t, r, p):
        if p == 1:
            return (0, 0)
        a = 20 if (t // 8) % 2 == 0 else -20
        b = 18 if (t // 4) % 2 == 0 else -18
        sgn = 1 if r % 2 == 0 else -1
        return (a + sgn * b, 0)
    mm = adaptive_inputs(multimode)
    cases.append(Case("AdaptiveDetection", "tests/test_adaptive_pipeline.cu:659-674", "adaptive",
                      ADAPTIVE, *mm, adaptive={"detect": True, "delta": 0.5},
                      expect={"counts": [[2, 0]], "pol_power_max": {0: 1.0}, "pol_power_eq": {1: 0.0}}))

    def rank2(c, t, r, p):
        if t < 32:
            return (2, -2)
        return (4, 0) if r == 0 else (0, 0)
    r2 = adaptive_inputs(rank2)
    cases.append(Case("AdaptiveShrinkRankTwo", "tests/test_adaptive_pipeline.cu:636-657", "adaptive",
                      ADAPTIVE, *r2, adaptive={"k": 1, "shrink": True},
                      expect={"shrink_power_gt_null": True}))
    cases.append(Case("AdaptiveShrinkRankOne", "tests/test_adaptive_pipeline.cu:622-634", "adaptive",
                      ADAPTIVE, *const, adaptive={"k": 1, "shrink": True},
                      expect={"slot1_power_max": 1.0}))
    return cases
