"""Shared runners/checkers for the reference golden cases.

``oracle_outputs`` produces the outputs of a case with the CPU oracle;
``check_case`` asserts a set of outputs (from the oracle or from the CUDA
path) against the values the reference's tests assert.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parents[1]
if str(REPO / "oracle") not in sys.path:
    sys.path.insert(0, str(REPO / "oracle"))
if str(REPO / "tests" / "golden") not in sys.path:
    sys.path.insert(0, str(REPO / "tests" / "golden"))

import sf_oracle as orc  # noqa: E402


def oracle_shape(case):
    C, F, Tp, R, Rpp, P, B = case.shape
    return orc.Shape(C, F, Tp, R, Rpp, P, B)


def oracle_outputs(case):
    sh = oracle_shape(case)
    d = orc.receiver_factors(sh, gains=case.gains)
    if case.path == "corr_beam":
        r = orc.corr_beam_chain(sh, case.samples, case.scales, case.weights, d=d)
        r["vis_scaled"] = orc.scaled_visibilities(sh, r["vis"], d)
    elif case.path == "lambda_gpu":
        r = orc.lambda_gpu_chain(sh, case.samples, case.scales, case.weights,
                                 delays=case.delays, d=d)
    else:
        a = case.adaptive
        k = a.get("k", 0)
        r = orc.adaptive_chain(sh, case.samples, case.scales, case.weights,
                               k_fixed=np.full(sh.C, k), detect=a.get("detect", False),
                               delta=a.get("delta", 3.0), shrink=a.get("shrink", False),
                               delays=case.delays, d=d)
    vs = r["vis_scaled"]
    out = {
        "beam_half": orc.half_output(r["beams"]).astype(np.float32),
        "vis": np.stack([np.real(vs), np.imag(vs)], axis=-1).astype(np.float32),
    }
    for key in ("evals", "evecs", "counts"):
        if key in r:
            out[key] = r[key]
    return out


def _power(beam_half, c=None, p=None, slot=1):
    b = beam_half
    sel = b[:, :, slot] if c is None else b[c:c + 1, :, slot]
    if p is not None:
        sel = sel[:, p]
    return float(np.sum(sel.astype(np.float64) ** 2))


def check_case(case, out, beam_tol=0.0):
    """Assert the reference test's expectations on ``out``.  ``beam_tol`` is an
    absolute tolerance on fp16 beam values (0 = exact, like EXPECT_EQ)."""
    e = case.expect
    C, F, Tp, R, Rpp, P, B = case.shape
    T = P * Tp
    beam = out["beam_half"]
    if "beam" in e:
        for c in range(C):
            for p in range(2):
                for m in range(B):
                    for t in range(T):
                        want = e["beam"](c, p, m, t)
                        got = beam[c, p, m, t]
                        assert abs(got[0] - want[0]) <= beam_tol and abs(got[1] - want[1]) <= beam_tol, \
                            f"{case.name}: beam[{c},{p},{m},{t}]={tuple(got)} want {want}"
    vis = out.get("vis")
    if "vis_re" in e:
        nbl = R * (R + 1) // 2
        for c in range(C):
            for b in range(nbl):
                for p in range(2):
                    for q in range(2):
                        want = e["vis_re"](c, b, p, q)
                        assert vis[c, b, p, q, 0] == want, \
                            f"{case.name}: vis[{c},{b},{p},{q}].re={vis[c, b, p, q, 0]} want {want}"
    if "vis_im" in e:
        assert np.all(vis[..., 1] == e["vis_im"]), f"{case.name}: vis imag not {e['vis_im']}"
    if "auto_re" in e:
        for c in range(C):
            for r in range(R):
                bl = r * (r + 1) // 2 + r
                for p in range(2):
                    want = e["auto_re"](c, r, p)
                    assert vis[c, bl, p, p, 0] == want, \
                        f"{case.name}: auto[{c},{r},{p}]={vis[c, bl, p, p, 0]} want {want}"
    if "evals" in e:
        ev = np.asarray(out["evals"])
        want = np.asarray(e["evals"])
        assert np.allclose(ev[..., :], want, atol=e.get("evals_tol", 1e-4)), f"{case.name}: evals {ev}"
    if "principal_evec" in e:
        vec = np.asarray(out["evecs"])[..., -1, :]  # [..., component]
        assert np.allclose(np.real(vec), e["principal_evec"], atol=e["evec_tol"]), f"{case.name}: {vec}"
        assert np.allclose(np.imag(vec), 0.0, atol=e["evec_tol"]), f"{case.name}: {vec}"
    if "beam_slot0" in e:
        want = e["beam_slot0"]
        assert np.all(beam[:, :, 0, :, 0] == want[0]) and np.all(beam[:, :, 0, :, 1] == want[1]), \
            f"{case.name}: slot0 {beam[:, :, 0, :4]}"
    if "beam_slot1_abs_max" in e:
        assert np.max(np.abs(beam[:, :, 1])) <= e["beam_slot1_abs_max"], f"{case.name}: slot1 not nulled"
    if "slot1_power_max" in e:
        assert _power(beam) < e["slot1_power_max"], f"{case.name}: slot1 power {_power(beam)}"
    if "slot1_power_min" in e:
        assert _power(beam) > e["slot1_power_min"], f"{case.name}: slot1 power {_power(beam)}"
    if e.get("slots_identical"):
        assert np.array_equal(beam[:, :, 0], beam[:, :, 1]), f"{case.name}: slots differ"
    if "beam_all_slots" in e:
        for c in range(C):
            for p in range(2):
                for t in range(T):
                    want = e["beam_all_slots"](c, p, t)
                    for m in range(2 * B):
                        got = beam[c, p, m, t]
                        assert got[0] == want[0] and got[1] == want[1], \
                            f"{case.name}: beam[{c},{p},{m},{t}]={tuple(got)} want {want}"
    if "counts" in e:
        assert np.array_equal(np.asarray(out["counts"]), np.asarray(e["counts"])), \
            f"{case.name}: counts {out['counts']}"
    if "pol_power_max" in e:
        for p, lim in e["pol_power_max"].items():
            assert _power(beam, p=p) < lim, f"{case.name}: pol {p} power {_power(beam, p=p)}"
    if "pol_power_eq" in e:
        for p, val in e["pol_power_eq"].items():
            assert _power(beam, p=p) == val, f"{case.name}: pol {p} power {_power(beam, p=p)}"
