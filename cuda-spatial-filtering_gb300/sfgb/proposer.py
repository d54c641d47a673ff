"""Learned subspace proposer: host driver of the sf_proposer_* C ABI.

The network (1344 -> 512 -> 512 -> 288 for 36 receivers, ReLU) maps a
whitened, trace-normalised covariance (packed upper triangle, bf16) to four
complex 36-vectors that warm-start the Rayleigh-Ritz refinement of the
learned adaptive chain (Plan.run_adaptive_learned).  Every arithmetic step --
feature extraction, the forward and backward GEMMs (hand-written BF16
tcgen05 kernels), the loss, the bias gradients and Adam -- runs in
libsfgb.so; this module only sequences the calls and owns device buffers
through PyTorch.

Training data are covariances the pipeline itself produces: seeded synthetic
int8 integrations with 0-4 narrowband interferers (INR uniform in [5, 30] dB)
go through the correlator; the full eigensolver's top-four eigenvectors of
each whitened covariance are the targets, weighted by how far each eigenvalue
stands above the noise floor.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import Plan, SfError, _check, _ptr, _stream, lib, SF_EIG_SAME_POL_WHITENED, SF_K_FIXED, SF_WINDOW_ALIGNED

_P = ctypes.c_void_p


class Proposer:
    def __init__(self, n_receivers=36, hidden=512, max_rows=8192):
        import torch
        if not torch.cuda.is_available():
            raise RuntimeError("no CUDA device: the proposer kernels need an sm_103 GPU")
        h = ctypes.c_void_p()
        _check(lib().sf_proposer_create(int(n_receivers), int(hidden), int(max_rows), ctypes.byref(h)))
        self._h = h
        dims = np.zeros(6, np.int32)
        _check(lib().sf_proposer_dims(self._h, dims.ctypes.data_as(_P)))
        self.n_in, self.in_ld, self.hidden, self.n_out, self.out_ld, self.max_rows = (int(x) for x in dims)
        self.R = int(n_receivers)
        self.shapes = [(self.hidden, self.in_ld), (self.hidden, self.hidden), (self.n_out, self.hidden)]

    def close(self):
        if getattr(self, "_h", None):
            lib().sf_proposer_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def init_params(self, seed=0):
        """He-uniform weights (fan-in of the real features), zero biases."""
        rng = np.random.default_rng(seed)
        params = []
        fan_in = [self.n_in, self.hidden, self.hidden]
        for (o, i), fi in zip(self.shapes, fan_in):
            lim = np.sqrt(6.0 / fi)
            w = rng.uniform(-lim, lim, size=(o, i)).astype(np.float32)
            if i > fi:
                w[:, fi:] = 0.0  # feature padding
            params += [w, np.zeros(o, np.float32)]
        self.set_params(params)

    def set_params(self, params, stream=None):
        arrs = [np.ascontiguousarray(p, np.float32) for p in params]
        _check(lib().sf_proposer_set_params(self._h, *[a.ctypes.data_as(_P) for a in arrs], _stream(stream)))

    def get_params(self, stream=None):
        arrs = []
        for o, i in self.shapes:
            arrs += [np.zeros((o, i), np.float32), np.zeros(o, np.float32)]
        _check(lib().sf_proposer_get_params(self._h, *[a.ctypes.data_as(_P) for a in arrs], _stream(stream)))
        return arrs

    def train_step(self, x, targets, weights, rows, lr, loss, stream=None):
        _check(lib().sf_proposer_train_step(self._h, _ptr(x), _ptr(targets), _ptr(weights), int(rows), float(lr),
                                            _ptr(loss), _stream(stream)))

    def infer(self, x, rows, y, stream=None):
        _check(lib().sf_proposer_infer(self._h, _ptr(x), int(rows), _ptr(y), _stream(stream)))

    def status(self, stream=None):
        bits = ctypes.c_uint32(0)
        rc = lib().sf_proposer_status(self._h, _stream(stream), ctypes.byref(bits))
        return rc, bits.value


def synth_packets_on_device(C, F, Tp, Rpp, P, gen, dev, sigma=16.0, max_interferers=4, inr_db=(5.0, 30.0)):
    """Seeded synthetic integration in the packet layout [C][P+2][F][Tp][Rpp][Pol][2]
    (int8) made on the device: noise clip(round(N(0, sigma^2))) plus
    0..max_interferers narrowband interferers per channel at INR uniform in
    inr_db (interferer eigenvalue over noise eigenvalue), unit-norm random
    steering per pol.  Returns (samples, steering [C][max_interferers][R][Pol]
    complex with zero rows for absent interferers)."""
    import torch
    R = F * Rpp
    tt = (P + 2) * Tp
    x = torch.randn((C, tt, R, 2, 2), generator=gen, device=dev) * sigma
    n_int = torch.randint(0, max_interferers + 1, (C,), generator=gen, device=dev)
    t = torch.arange(tt, device=dev, dtype=torch.float32)
    steer = torch.zeros((C, max_interferers, R, 2), dtype=torch.complex64, device=dev)
    lo, hi = inr_db
    for k in range(max_interferers):
        inr = 10.0 ** ((torch.rand(C, generator=gen, device=dev) * (hi - lo) + lo) / 10.0)
        on = (n_int > k).float()
        amp = torch.sqrt(inr * 2.0 * sigma ** 2) * on
        a = torch.complex(torch.randn((C, R, 2), generator=gen, device=dev),
                          torch.randn((C, R, 2), generator=gen, device=dev))
        a = a / torch.linalg.vector_norm(a, dim=1, keepdim=True)
        steer[:, k] = a * on[:, None, None]
        f0 = torch.rand(C, generator=gen, device=dev) * 0.9 - 0.45
        ph = torch.rand(C, generator=gen, device=dev) * 2 * np.pi
        ang = 2 * np.pi * f0[:, None] * t[None] + ph[:, None]
        s_re = (amp[:, None] * torch.cos(ang))[:, :, None, None]
        s_im = (amp[:, None] * torch.sin(ang))[:, :, None, None]
        a_re, a_im = a.real[:, None], a.imag[:, None]
        x[..., 0] += s_re * a_re - s_im * a_im
        x[..., 1] += s_re * a_im + s_im * a_re
    x = torch.clamp(torch.round(x), -127, 127).to(torch.int8)
    # [C][tt][R][Pol][2] -> [C][P+2][F][Tp][Rpp][Pol][2]
    x = x.view(C, P + 2, Tp, F, Rpp, 2, 2).permute(0, 1, 3, 2, 4, 5, 6).contiguous()
    return x, steer


def make_training_set(n_covariances, proposer, F=4, Rpp=9, Tp=64, P=16, chunk_channels=4096, seed=0, dev="cuda"):
    """Features, targets and weights of n_covariances (channel, pol) matrices
    produced by the pipeline: correlator -> whitened covariance -> full
    eigensolver -> top-four eigenvectors.  Returns device tensors (x bf16
    [N][in_ld], t fp32 [N][n_out], w fp32 [N][4])."""
    import torch
    R = F * Rpp
    assert R == proposer.R
    n_ch = (n_covariances + 1) // 2
    N = 2 * n_ch
    x = torch.zeros((N, proposer.in_ld), dtype=torch.bfloat16, device=dev)
    t = torch.zeros((N, proposer.n_out), dtype=torch.float32, device=dev)
    w = torch.zeros((N, 4), dtype=torch.float32, device=dev)
    gen = torch.Generator(device=dev)
    gen.manual_seed(seed)
    plan = Plan(chunk_channels, F, Tp, R, Rpp, P, 1)
    vis = torch.empty(plan.vis_shape(), dtype=torch.int32, device=dev)
    ev = torch.empty((chunk_channels, 2, R), dtype=torch.float32, device=dev)
    vec = torch.empty((chunk_channels, 2, R, R, 2), dtype=torch.float32, device=dev)
    scales = torch.ones((chunk_channels, P + 2, R, 2), dtype=torch.int16, device=dev)
    done = 0
    while done < n_ch:
        samples, _ = synth_packets_on_device(chunk_channels, F, Tp, Rpp, P, gen, dev)
        plan.correlate(samples, scales, SF_WINDOW_ALIGNED, vis)
        plan.covariance_eig(vis, SF_EIG_SAME_POL_WHITENED, SF_K_FIXED, 0.0, False, ev, vec)
        take = min(chunk_channels, n_ch - done)
        xc = torch.empty((2 * chunk_channels, proposer.in_ld), dtype=torch.bfloat16, device=dev)
        tc = torch.empty((2 * chunk_channels, proposer.n_out), dtype=torch.float32, device=dev)
        wc = torch.empty((2 * chunk_channels, 4), dtype=torch.float32, device=dev)
        plan.proposer_features(vis, xc, proposer.in_ld)
        plan.proposer_targets(vis, ev, vec, tc, wc)
        x[2 * done:2 * (done + take)] = xc[:2 * take]
        t[2 * done:2 * (done + take)] = tc[:2 * take]
        w[2 * done:2 * (done + take)] = wc[:2 * take]
        done += take
    torch.cuda.synchronize()
    rc, bits = plan.status()
    plan.close()
    if rc != 0:
        raise SfError(rc, f"training-set generation: device status 0x{bits:x}")
    return x, t, w


def train(proposer, x, t, w, epochs=10, batch=8192, lr=1e-3, seed=0, stream=None):
    """Adam over shuffled batches; returns the mean loss of every epoch."""
    import torch
    N = x.shape[0]
    gen = torch.Generator(device=x.device)
    gen.manual_seed(seed)
    loss = torch.zeros(1, dtype=torch.float32, device=x.device)
    history = []
    for ep in range(epochs):
        perm = torch.randperm(N, generator=gen, device=x.device)
        loss.zero_()
        nb = 0
        for b0 in range(0, N - batch + 1, batch):
            idx = perm[b0:b0 + batch]
            xb, tb, wb = x[idx].contiguous(), t[idx].contiguous(), w[idx].contiguous()
            proposer.train_step(xb, tb, wb, batch, lr, loss, stream=stream)
            nb += 1
        torch.cuda.synchronize()
        history.append(float(loss.item()) / max(1, nb))
    rc, bits = proposer.status()
    if rc != 0:
        raise SfError(rc, f"training: device status 0x{bits:x}")
    return history
