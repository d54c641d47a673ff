"""CPU oracle for the spatial-filtering hot path.

TEST INFRASTRUCTURE ONLY.  This module is the checker: only ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` may import
it.  The product path (the CUDA kernels behind ``include/sf_capi.h``) never
calls into it and fails loudly when its extension is missing.

It restates, in plain numpy (int64 for the integer work, float64/complex128 for
the floating-point work), the reference's per-channel chain:

  ingest + alignment   include/spatial/spatial.cuh:423-486 (scale_and_convert),
                       include/spatial/spatial.cuh:1420-1506 (apply_delays),
                       include/spatial/pipeline/lambda_corr_beam_only_gpu_pipeline.hpp:305-316
                       (packet_to_corr_input: packets 0..P-1, no delay)
  correlation          TCC launch, include/spatial/pipeline/lambda_gpu_pipeline.hpp:649-651;
                       packed triangle baseline(i,j)=j(j+1)/2+i, i<=j
                       (tests/support/assertions.hpp:35-37); the value convention
                       V(i,p;j,q)=sum_t x_ip conj(x_jq) follows tests/test_beamforming.cpp:49-79
  trim                 src/spatial.cu:176-200 (keep baselines a < R(R+1)/2)
  unpack               include/spatial/spatial.cuh:672-713 (upper triangle, column-major)
  whitening            include/spatial/spatial.cuh:1068-1148
  eigendecomposition   cusolverDnXsyevBatched (ascending, vectors in columns); restated
                       here with LAPACK (numpy.linalg.eigh) in complex128
  K detection          include/spatial/spatial.cuh:900-950 (float32 arithmetic) and
                       scripts/adaptive_detection_reference.py:11-35 (float64)
  projector            include/spatial/spatial.cuh:993-1034 (P = I - U_K U_K^H),
                       shrink form spatial.cuh:952-1063 / adaptive_detection_reference.py:50-63
  weight projection    lambda_adaptive_beamformed_spectra_pipeline.hpp:773-794 (W' = W P)
  beamforming          lambda_gpu_pipeline.hpp:731-733 (Y = W X, no conjugation)
  half output          include/spatial/spatial.cuh:376-418

Gains and fine-delay phasors are folded as a per-(channel, pol, receiver)
complex factor d: the covariance becomes d_i conj(d_j) V and the beam weights
become W diag(d).  This equals the reference's ingest (which multiplies each
sample by its gain before correlating and beamforming) up to the reference's
fp16 rounding of the scaled sample.
"""
from __future__ import annotations

import numpy as np

COMPLEX = 2
NPOL = 2


# --------------------------------------------------------------------------
# Shapes and index helpers
# --------------------------------------------------------------------------
class Shape:
    """Runtime shape of one integration (the reference's LambdaConfig,
    include/spatial/packet_formats.hpp:265-407)."""

    def __init__(self, n_channels, n_fpgas, n_time_per_packet, n_receivers,
                 n_receivers_per_packet, n_packets, n_beams, n_pol=2):
        if n_pol != 2:
            raise ValueError("only 2 polarisations are supported")
        if n_receivers != n_fpgas * n_receivers_per_packet:
            raise ValueError("n_receivers must equal n_fpgas * n_receivers_per_packet")
        self.C = int(n_channels)
        self.F = int(n_fpgas)
        self.Tp = int(n_time_per_packet)
        self.R = int(n_receivers)
        self.Rpp = int(n_receivers_per_packet)
        self.P = int(n_packets)
        self.B = int(n_beams)
        self.T = self.P * self.Tp
        self.NBL = self.R * (self.R + 1) // 2

    def samples_shape(self):
        return (self.C, self.P + 2, self.F, self.Tp, self.Rpp, NPOL, COMPLEX)

    def scales_shape(self):
        return (self.C, self.P + 2, self.R, NPOL)


def baseline_index(i, j):
    """Packed index of baseline (i, j), i <= j (tests/support/assertions.hpp:35-37)."""
    return j * (j + 1) // 2 + i


def baseline_pairs(R):
    """(i, j) arrays in packed order."""
    ii, jj = [], []
    for j in range(R):
        for i in range(j + 1):
            ii.append(i)
            jj.append(j)
    return np.array(ii), np.array(jj)


# --------------------------------------------------------------------------
# Ingest: packet layout -> aligned, scaled integer samples
# --------------------------------------------------------------------------
def sample_offsets(shape, delays=None, mode="aligned"):
    """Per-FPGA offset (in samples) of the integration window inside the
    (P+2)-packet buffer.

    mode "aligned": the LambdaGPUPipeline/adaptive path; window starts one
        packet in, shifted by the sub-packet delay (spatial.cuh:1436-1442).
    mode "packet": the LambdaCorrBeamOnlyGPUPipeline path; window is packets
        0..P-1 with no delay (spatial.cuh:215-279).
    """
    if mode == "packet":
        return np.zeros(shape.F, dtype=np.int64)
    d = np.zeros(shape.F, dtype=np.int64) if delays is None else np.asarray(delays, np.int64)
    if np.any(np.abs(d) > shape.Tp):
        raise ValueError("sub-packet delays must lie in [-Tp, Tp]")
    return shape.Tp + d


def aligned_samples(shape, samples, scales, offsets):
    """Scaled integer samples x[c][p][r][t] (re, im as int64 arrays).

    x = int(sample) * int(scale), as scale_and_convert_to_half_kernel
    (spatial.cuh:464-476) computes before its float conversion.
    """
    s = np.asarray(samples).reshape(shape.samples_shape()).astype(np.int64)
    sc = np.asarray(scales).reshape(shape.scales_shape()).astype(np.int64)
    re = np.zeros((shape.C, NPOL, shape.R, shape.T), dtype=np.int64)
    im = np.zeros_like(re)
    t_al = np.arange(shape.T)
    for f in range(shape.F):
        q = t_al + int(offsets[f])
        pkt = q // shape.Tp
        tin = q % shape.Tp
        # [C][T][Rpp][Pol][2]
        blk = s[:, pkt, f, tin, :, :, :]
        scl = sc[:, pkt, f * shape.Rpp:(f + 1) * shape.Rpp, :]  # [C][T][Rpp][Pol]
        r0 = f * shape.Rpp
        re[:, :, r0:r0 + shape.Rpp, :] = np.transpose(blk[..., 0] * scl, (0, 3, 2, 1))
        im[:, :, r0:r0 + shape.Rpp, :] = np.transpose(blk[..., 1] * scl, (0, 3, 2, 1))
    return re, im


def permute_streams(shape, re, im, recv_perm, pol_perm):
    """Canonical streams from the packet-order ones, after alignment
    (reorder_streams_kernel, spatial.cuh:596-636; set_stream_permutation,
    lambda_gpu_pipeline.hpp:1139-1150): output stream (receiver r, pol p),
    index k = 2 r + p, is source receiver recv_perm[k] (flat f * Rpp + n) at
    source pol pol_perm[k]; recv_perm[k] = -1 gives zeros."""
    rp = np.asarray(recv_perm, np.int64).reshape(shape.R, NPOL)
    pp = np.asarray(pol_perm, np.int64).reshape(shape.R, NPOL)
    ore = np.zeros_like(re)
    oim = np.zeros_like(im)
    for r in range(shape.R):
        for p in range(NPOL):
            src = rp[r, p]
            if src < 0:
                continue
            ore[:, p, r, :] = re[:, pp[r, p], src, :]
            oim[:, p, r, :] = im[:, pp[r, p], src, :]
    return ore, oim


def permuted_factors(shape, recv_perm, pol_perm, gains=None, phasors=None):
    """Per-output-stream factor d: the gain is applied at ingest to the source
    stream (spatial.cuh:464-476), the fine-delay phasor after the reorder to the
    output receiver (lambda_gpu_pipeline.hpp:680-701)."""
    g = np.ones((shape.C, NPOL, shape.R), dtype=np.complex128)
    if gains is not None:
        g = np.asarray(gains, np.complex128).reshape(shape.C, NPOL, shape.R)
    rp = np.asarray(recv_perm, np.int64).reshape(shape.R, NPOL)
    pp = np.asarray(pol_perm, np.int64).reshape(shape.R, NPOL)
    d = np.zeros((shape.C, NPOL, shape.R), dtype=np.complex128)
    for r in range(shape.R):
        for p in range(NPOL):
            if rp[r, p] >= 0:
                d[:, p, r] = g[:, pp[r, p], rp[r, p]]
    if phasors is not None:
        d = d * np.asarray(phasors, np.complex128).reshape(shape.C, 1, shape.R)
    return d


# --------------------------------------------------------------------------
# Correlation (exact integers)
# --------------------------------------------------------------------------
def correlate(shape, re, im):
    """Exact visibilities vis[c][b][p][q][2] (int64), b = baseline(i, j), i <= j,
    value sum_t x_{i,p}(t) conj(x_{j,q}(t))."""
    C, R = shape.C, shape.R
    ii, jj = baseline_pairs(R)
    out = np.zeros((C, shape.NBL, NPOL, NPOL, COMPLEX), dtype=np.int64)
    for c in range(C):
        a = re[c].reshape(NPOL * R, shape.T)  # rows (p, r)
        b = im[c].reshape(NPOL * R, shape.T)
        rr = a @ a.T + b @ b.T               # Re sum x_u conj(x_v)
        ri = b @ a.T - a @ b.T               # Im
        rr = rr.reshape(NPOL, R, NPOL, R)
        ri = ri.reshape(NPOL, R, NPOL, R)
        # out[c, bl, p, q] = V(i,p ; j,q)
        # advanced indexing puts the baseline axis first: [b][p][q]
        out[c, :, :, :, 0] = rr[:, ii, :, jj]
        out[c, :, :, :, 1] = ri[:, ii, :, jj]
    return out


def vis_complex(vis):
    v = np.asarray(vis)
    return v[..., 0].astype(np.float64) + 1j * v[..., 1].astype(np.float64)


# --------------------------------------------------------------------------
# Per-receiver complex factors (gains x fine-delay phasors)
# --------------------------------------------------------------------------
def fine_delay_phasors(shape, delays_ns, base_freq_hz, channel_bw_hz, min_freq_ch):
    """Channel-centre phasor exp(-2 pi i f_c tau_r), f_c = base + (min_ch + c) bw.

    The reference corrects every fine bin k with f_fine = f_c + (k_signed/N) bw
    (lambda_gpu_pipeline.hpp:1100-1131); folding the channel-centre phasor into
    the weights is the narrowband approximation (exact for the k = 0 bin).
    """
    tau = np.asarray(delays_ns, np.float64) * 1e-9
    fc = base_freq_hz + (min_freq_ch + np.arange(shape.C, dtype=np.float64)) * channel_bw_hz
    phi = -2.0 * np.pi * fc[:, None] * tau[None, :]
    return np.exp(1j * phi)  # [C][R]


def receiver_factors(shape, gains=None, phasors=None):
    """d[c][p][r] complex128; gains [C][Pol][R] complex (AntennaGains layout,
    packet_formats.hpp:387-390), phasors [C][R]."""
    d = np.ones((shape.C, NPOL, shape.R), dtype=np.complex128)
    if gains is not None:
        d = d * np.asarray(gains, np.complex128).reshape(shape.C, NPOL, shape.R)
    if phasors is not None:
        d = d * np.asarray(phasors, np.complex128).reshape(shape.C, 1, shape.R)
    return d


def scaled_visibilities(shape, vis, d):
    """Float visibilities as the reference reports them: d_{i,p} conj(d_{j,q}) V."""
    ii, jj = baseline_pairs(shape.R)
    v = vis_complex(vis)
    di = np.transpose(d[:, :, ii], (0, 2, 1))  # [C][NBL][Pol]
    dj = np.transpose(d[:, :, jj], (0, 2, 1))
    return v * di[:, :, :, None] * np.conj(dj[:, :, None, :])


# --------------------------------------------------------------------------
# Covariance matrices
# --------------------------------------------------------------------------
def unpack_hermitian(shape, vis_c, p, q):
    """Dense Hermitian matrices [C][R][R] built the way cuSOLVER reads the
    reference's unpack output (spatial.cuh:672-713 writes the upper triangle
    row=i, col=j, i<=j; uplo=UPPER; the diagonal's imaginary part is ignored)."""
    ii, jj = baseline_pairs(shape.R)
    C, R = shape.C, shape.R
    m = np.zeros((C, R, R), dtype=np.complex128)
    m[:, ii, jj] = vis_c[:, :, p, q]
    lower = np.conj(np.transpose(m, (0, 2, 1)))
    m = m + lower
    diag = np.arange(R)
    m[:, diag, diag] = np.real(vis_c[:, baseline_index(diag, diag), p, q])
    return m


def whiten(m):
    """spatial.cuh:1068-1093: s_i = sqrt(max(Re m_ii, 1e-10)); m_ij / (s_i s_j)."""
    dg = np.real(np.diagonal(m, axis1=-2, axis2=-1))
    s = np.sqrt(np.maximum(dg, 1e-10))
    return m / (s[..., :, None] * s[..., None, :]), s


def unwhiten_normalize(v, s):
    """spatial.cuh:1098-1126: u_ik = s_i v_ik, then each column to unit norm."""
    u = v * s[..., :, None]
    nrm = np.sqrt(np.sum(np.abs(u) ** 2, axis=-2, keepdims=True))
    inv = np.where(nrm > 0, 1.0 / np.where(nrm > 0, nrm, 1.0), 0.0)
    return u * inv


def eigh_ascending(m):
    """FP64 LAPACK eigendecomposition: ascending eigenvalues, vectors in columns."""
    w, v = np.linalg.eigh(m)
    return w, v


def normalize_phase(v):
    """Make each column's largest-magnitude component real and positive (ties:
    lowest index).  Eigenvectors are unique only up to a unit phase; this is
    the convention the CUDA eigensolver applies to its output."""
    v = np.array(v, dtype=np.complex128, copy=True)
    mag = np.abs(v)
    idx = np.argmax(mag, axis=-2)  # [..., k]
    piv = np.take_along_axis(v, idx[..., None, :], axis=-2)
    ph = np.where(np.abs(piv) > 0, np.conj(piv) / np.where(np.abs(piv) > 0, np.abs(piv), 1.0), 1.0)
    return v * ph


# --------------------------------------------------------------------------
# K detection
# --------------------------------------------------------------------------
def _percentile_f32(vals, quant):
    n = len(vals)
    if n <= 0:
        return np.float32(0.0)
    if n == 1:
        return np.float32(vals[0])
    q = np.float32(min(1.0, max(0.0, quant)))
    pos = np.float32(q * np.float32(n - 1))
    lo = int(np.floor(pos))
    hi = int(np.ceil(pos))
    if lo == hi:
        return np.float32(vals[lo])
    frac = np.float32(pos - np.float32(lo))
    return np.float32(vals[lo] + frac * np.float32(vals[hi] - vals[lo]))


def detect_k_f32(evals, delta):
    """detectSignalEigenmodeCountsKernel (spatial.cuh:900-943), float32."""
    e = np.asarray(evals, dtype=np.float32)
    p20 = _percentile_f32(e, 0.2)
    p50 = _percentile_f32(e, 0.5)
    p80 = _percentile_f32(e, 0.8)
    sigma = np.float32(np.float32(p80 - p20) / np.float32(2.0 * 0.8416))
    thr = np.float32(p50 + np.float32(delta) * sigma)
    return int(np.count_nonzero(e > thr))


def detect_k_f64(evals, delta):
    """scripts/adaptive_detection_reference.py:28-35, float64."""
    e = np.asarray(evals, dtype=np.float64)

    def pct(q):
        n = e.size
        if n == 0:
            return 0.0
        if n == 1:
            return float(e[0])
        pos = float(np.clip(q, 0.0, 1.0)) * (n - 1)
        lo, hi = int(np.floor(pos)), int(np.ceil(pos))
        if lo == hi:
            return float(e[lo])
        return float(e[lo] + (pos - lo) * (e[hi] - e[lo]))

    sigma = (pct(0.8) - pct(0.2)) / (2.0 * 0.8416)
    thr = pct(0.5) + delta * sigma
    return int(np.count_nonzero(e > thr))


def detect_k_noise_floor(evals, factor=10.0, floor=None):
    """K = #{lambda > factor x noise floor}; the noise floor defaults to the
    median eigenvalue (the uneven-batching configuration's rule)."""
    e = np.asarray(evals, dtype=np.float64)
    nf = float(np.median(e)) if floor is None else float(floor)
    return int(np.count_nonzero(e > factor * nf))


# --------------------------------------------------------------------------
# Projectors and weights
# --------------------------------------------------------------------------
def null_projection(u, k):
    """P = I - U_K U_K^H over the last k columns (spatial.cuh:993-1022)."""
    n = u.shape[-1]
    eye = np.eye(n, dtype=np.complex128)
    if k <= 0:
        return eye
    rfi = u[:, n - k:]
    return eye - rfi @ np.conj(rfi.T)


def shrink_projection(v, evals, k):
    """M = V diag(d) V^H, d = 1 for kept modes, lambda_bar/lambda for the last k
    (spatial.cuh:952-984, adaptive_detection_reference.py:50-63)."""
    vals = np.asarray(evals, np.float64)
    n = vals.shape[0]
    d = np.ones(n)
    kk = max(0, min(n, int(k)))
    if kk > 0:
        keep = n - kk
        lam_bar = float(np.mean(vals[:keep])) if keep > 0 else 0.0
        for idx in range(keep, n):
            d[idx] = lam_bar / vals[idx] if vals[idx] > 0.0 else 0.0
    return (v * d[None, :]) @ np.conj(v.T)


SPEED_OF_LIGHT = 299792458.0


def steering_weights(shape, dircos, enu, connected=None, base_freq_hz=0.0, channel_bw_hz=0.0,
                     min_freq_ch=0, cal_gains=None):
    """compute_steering_weights (include/spatial/pipeline/common.hpp:97-185) as
    fp16 pairs [C][Pol][B][R][2]: w = (1/R) G exp(i phase),
    phase = -2 pi f_c / c (l e + m n + n u), f_c = base + (min_ch + c) bw, in
    float64, rounded to float32 and then fp16; null inputs (connected == 0)
    exactly zero.  dircos [B][3], enu [R][3], cal_gains complex [C][Pol][R]."""
    C, B, R = shape.C, shape.B, shape.R
    dc = np.asarray(dircos, dtype=np.float64).reshape(B, 3)
    pos = np.asarray(enu, dtype=np.float64).reshape(R, 3)
    path = (dc[:, 0, None] * pos[None, :, 0] + dc[:, 1, None] * pos[None, :, 1]) + dc[:, 2, None] * pos[None, :, 2]
    f = base_freq_hz + (min_freq_ch + np.arange(C)).astype(np.float64) * channel_bw_hz
    phase = (-2.0 * np.pi * f / SPEED_OF_LIGHT)[:, None, None] * path[None]  # [C][B][R]
    ph = np.cos(phase) + 1j * np.sin(phase)
    if cal_gains is None:
        g = np.ones((C, NPOL, R), dtype=np.complex128)
    else:
        g = np.asarray(cal_gains).reshape(C, NPOL, R).astype(np.complex64).astype(np.complex128)
    w = ((1.0 / R) * g)[:, :, None, :] * ph[:, None, :, :]  # [C][Pol][B][R]
    if connected is not None:  # null inputs stay at the zero the result was initialised with
        w = np.where((np.asarray(connected).reshape(R) != 0)[None, None, None, :], w, 0.0)
    out = np.empty(w.shape + (2,), dtype=np.float16)
    out[..., 0] = w.real.astype(np.float32).astype(np.float16)
    out[..., 1] = w.imag.astype(np.float32).astype(np.float16)
    return out


def weights_complex(weights):
    """BeamWeightsT layout complex<__half>[C][Pol][B][R] (pipeline/common.hpp:52-55)
    given as float pairs [..., 2] or complex."""
    w = np.asarray(weights)
    if np.iscomplexobj(w):
        return w.astype(np.complex128)
    return w[..., 0].astype(np.float64) + 1j * w[..., 1].astype(np.float64)


# --------------------------------------------------------------------------
# Beamforming
# --------------------------------------------------------------------------
def beamform(shape, re, im, w_eff):
    """Y[c][p][m][t] = sum_r W_eff[c][p][m][r] x[c][p][r][t] (no conjugation)."""
    x = re.astype(np.float64) + 1j * im.astype(np.float64)
    return np.einsum("cpmr,cprt->cpmt", w_eff, x)


def half_output(y):
    """__half[C][Pol][NB][T][2] as beam_ccglib_to_half_output writes it
    (spatial.cuh:376-404): round-to-nearest fp16 of each component."""
    out = np.empty(y.shape + (2,), dtype=np.float16)
    out[..., 0] = np.real(y).astype(np.float32).astype(np.float16)
    out[..., 1] = np.imag(y).astype(np.float32).astype(np.float16)
    return out


# --------------------------------------------------------------------------
# Beam spectra tail
# --------------------------------------------------------------------------
# The reference transforms its beams with cuFFT (CUDA toolkit library, not part
# of the reference tree): cufftXtMakePlanMany(1-D, C2C, fp32) executed with
# CUFFT_FORWARD, i.e. the unnormalised DFT X[k] = sum_n x[n] exp(-2 pi i n k / N).
# numpy.fft.fft computes the same definition; dft_direct below pins that by the
# O(N^2) sum.
def dft_direct(x):
    """Forward DFT along the last axis by the definition (small N only)."""
    x = np.asarray(x, dtype=np.complex128)
    n = x.shape[-1]
    k = np.arange(n)
    w = np.exp(-2j * np.pi * np.outer(k, k) / n)
    return x @ w.T


def beams_from_half(beams_f16):
    """fp16 pairs [..., T, 2] -> complex128 [..., T]."""
    b = np.asarray(beams_f16).astype(np.float64)
    return b[..., 0] + 1j * b[..., 1]


def beam_spectra(beams_c, downsample):
    """LambdaGPUPipeline spectra tail: one forward FFT of each (channel, pol,
    beam) series over the whole integration (lambda_gpu_pipeline.hpp:522-524;
    plan of length T = P Tp with C Pol B batches, :814-817 and :944-947), then
    detect_and_downsample_fft (spatial.cuh:795-848): output bin g is the mean of
    |X|^2 over bins g D .. g D + D - 1, NaN bins skipped, 0 when every bin of the
    group is NaN; T // D bins ([C][Pol][B][T/D] floats)."""
    beams_c = np.asarray(beams_c, dtype=np.complex128)
    T = beams_c.shape[-1]
    n_out = T // downsample
    with np.errstate(invalid="ignore", over="ignore"):
        x = np.fft.fft(beams_c, axis=-1)
        pw = x.real * x.real + x.imag * x.imag
    pw = pw[..., : n_out * downsample].reshape(beams_c.shape[:-1] + (n_out, downsample))
    ok = ~np.isnan(pw)
    s = np.where(ok, pw, 0.0).sum(axis=-1)
    cnt = ok.sum(axis=-1)
    return np.where(cnt > 0, s / np.maximum(cnt, 1), 0.0)


def fine_channel_order(Tp, trim):
    """FFT bins kept by the adaptive tail, in output order: the upper half
    without its first `trim` bins, then the lower half without its last `trim`
    (the two half-copies of lambda_adaptive_beamformed_spectra_pipeline.hpp:821-833
    over the frequency-major tensor of :816-819)."""
    return np.concatenate([np.arange(Tp // 2 + trim, Tp), np.arange(0, Tp // 2 - trim)])


def packet_spectra(beams_c, Tp, trim):
    """Adaptive pipeline spectra tail
    (lambda_adaptive_beamformed_spectra_pipeline.hpp:808-848): a Tp-point FFT of
    each packet of each (channel, pol, beam) series (plan :1046-1050, batch
    2B C Pol P), the fine-channel trim/reorder, then sum_fft_over_packets
    (spatial.cuh:1508-1567): sum over the P packets of the magnitude |X|
    ([C][Pol][NB][Tp - 2 trim] floats)."""
    beams_c = np.asarray(beams_c, dtype=np.complex128)
    T = beams_c.shape[-1]
    P = T // Tp
    x = np.fft.fft(beams_c.reshape(beams_c.shape[:-1] + (P, Tp)), axis=-1)
    mag = np.abs(x)[..., fine_channel_order(Tp, trim)]
    return mag.sum(axis=-2)


# --------------------------------------------------------------------------
# Whole chains
# --------------------------------------------------------------------------
def corr_beam_chain(shape, samples, scales, weights, d=None, offsets=None):
    """LambdaCorrBeamOnlyGPUPipeline (lambda_corr_beam_only_gpu_pipeline.hpp:305-344):
    exact visibilities + beams with the unprojected weights."""
    if offsets is None:
        offsets = sample_offsets(shape, mode="packet")
    if d is None:
        d = receiver_factors(shape)
    re, im = aligned_samples(shape, samples, scales, offsets)
    vis = correlate(shape, re, im)
    w = weights_complex(weights) * d[:, :, None, :]
    y = beamform(shape, re, im, w)
    return {"vis": vis, "beams": y, "re": re, "im": im}


def lambda_gpu_chain(shape, samples, scales, weights, delays=None, d=None):
    """LambdaGPUPipeline (lambda_gpu_pipeline.hpp:445-743): aligned window,
    eigendecomposition of all C*Pol*Pol blocks, beams with unprojected weights."""
    offsets = sample_offsets(shape, delays, mode="aligned")
    if d is None:
        d = receiver_factors(shape)
    re, im = aligned_samples(shape, samples, scales, offsets)
    vis = correlate(shape, re, im)
    vc = scaled_visibilities(shape, vis, d)
    evals = np.zeros((shape.C, NPOL, NPOL, shape.R))
    evecs = np.zeros((shape.C, NPOL, NPOL, shape.R, shape.R), dtype=np.complex128)
    for p in range(NPOL):
        for q in range(NPOL):
            m = unpack_hermitian(shape, vc, p, q)
            for c in range(shape.C):
                w, v = eigh_ascending(m[c])
                evals[c, p, q] = w
                evecs[c, p, q] = normalize_phase(v).T  # [k][l] = component l of vector k
    w = weights_complex(weights) * d[:, :, None, :]
    y = beamform(shape, re, im, w)
    return {"vis": vis, "vis_scaled": vc, "evals": evals, "evecs": evecs,
            "beams": y, "re": re, "im": im}


def adaptive_chain(shape, samples, scales, weights, k_fixed=None, detect=False,
                   delta=3.0, shrink=False, delays=None, d=None, k_rule=None, perm=None):
    """Adaptive null/shrink chain
    (lambda_adaptive_beamformed_spectra_pipeline.hpp:563-798): per (c, p)
    same-polarisation covariance, diagonal whitening, eigendecomposition, K,
    un-whitened I - U U^H (or shrink V diag(d) V^H), W' = W P; beams for the
    original (slot 0) and projected (slot 1) weights."""
    offsets = sample_offsets(shape, delays, mode="aligned")
    if d is None:
        d = receiver_factors(shape)
    re, im = aligned_samples(shape, samples, scales, offsets)
    if perm is not None:  # (recv_perm, pol_perm): reorder after the alignment
        re, im = permute_streams(shape, re, im, perm[0], perm[1])
    vis = correlate(shape, re, im)
    vc = scaled_visibilities(shape, vis, d)
    C, R, B = shape.C, shape.R, shape.B
    evals = np.zeros((C, NPOL, R))
    evecs = np.zeros((C, NPOL, R, R), dtype=np.complex128)
    counts = np.zeros((C, NPOL), dtype=np.int32)
    proj = np.zeros((C, NPOL, R, R), dtype=np.complex128)
    wc = weights_complex(weights)
    w_eff = np.zeros((C, NPOL, 2 * B, R), dtype=np.complex128)
    for p in range(NPOL):
        m = unpack_hermitian(shape, vc, p, p)
        for c in range(C):
            mw, s = whiten(m[c])
            lam, v = eigh_ascending(mw)
            if k_rule is not None:
                k = int(k_rule(lam))
            elif detect:
                k = detect_k_f32(lam, delta)
            else:
                k = 0 if k_fixed is None else int(np.asarray(k_fixed).reshape(C)[c])
            k = max(0, min(R, k))
            if shrink:
                pm = shrink_projection(v, lam, k)
                vout = v
            else:
                u = unwhiten_normalize(v, s)
                pm = null_projection(u, k)
                vout = u
            evals[c, p] = lam
            evecs[c, p] = normalize_phase(vout).T
            counts[c, p] = k
            proj[c, p] = pm
            w_eff[c, p, :B] = wc[c, p] * d[c, p][None, :]
            w_eff[c, p, B:] = (wc[c, p] @ pm) * d[c, p][None, :]
    y = beamform(shape, re, im, w_eff)
    return {"vis": vis, "vis_scaled": vc, "evals": evals, "evecs": evecs,
            "counts": counts, "proj": proj, "w_eff": w_eff, "beams": y,
            "re": re, "im": im}


# --------------------------------------------------------------------------
# Synthetic LAMBDA-shaped inputs (seeded)
# --------------------------------------------------------------------------
def synth_inputs(shape, seed=0, sigma=16.0, n_interferers=0, inr_db=20.0,
                 frac_channels=0.1, scale_value=1, return_steering=False):
    """Seeded synthetic integration in the packet layout.

    Noise: I, Q = clip(round(N(0, sigma^2)), -127, 127).  Interferers (in a
    random `frac_channels` of the channels) add sqrt(INR * 2 sigma^2) s(t) a
    with unit-norm random complex steering a and unit-power narrowband s(t);
    INR is the interferer eigenvalue over the per-receiver noise eigenvalue.
    With return_steering, a fourth value maps each interfered channel to the
    list of its interferers' steering vectors a [R][Pol] (unit norm per pol).
    """
    rng = np.random.Generator(np.random.PCG64(seed))
    C, R, T = shape.C, shape.R, shape.T
    npk = shape.P + 2
    tt = npk * shape.Tp
    re = rng.normal(0.0, sigma, size=(C, tt, R, NPOL))
    im = rng.normal(0.0, sigma, size=(C, tt, R, NPOL))
    rfi_ch = np.zeros(C, dtype=bool)
    steering = {}
    if n_interferers > 0:
        nsel = max(1, int(round(frac_channels * C)))
        rfi_ch[rng.choice(C, size=nsel, replace=False)] = True
        amp = np.sqrt(10.0 ** (inr_db / 10.0) * 2.0 * sigma ** 2)
        t = np.arange(tt)
        for c in np.nonzero(rfi_ch)[0]:
            for _ in range(n_interferers):
                a = rng.normal(size=(R, NPOL)) + 1j * rng.normal(size=(R, NPOL))
                a /= np.linalg.norm(a, axis=0, keepdims=True)
                steering.setdefault(int(c), []).append(a.copy())
                f0 = rng.uniform(-0.45, 0.45)
                ph0 = rng.uniform(0, 2 * np.pi)
                s = np.exp(1j * (2 * np.pi * f0 * t + ph0))
                sig = amp * s[:, None, None] * a[None, :, :]
                re[c] += np.real(sig)
                im[c] += np.imag(sig)
    re = np.clip(np.round(re), -127, 127).astype(np.int8)
    im = np.clip(np.round(im), -127, 127).astype(np.int8)
    # [C][tt][R][Pol] -> [C][P+2][F][Tp][Rpp][Pol][2]
    x = np.stack([re, im], axis=-1).reshape(C, npk, shape.Tp, shape.F, shape.Rpp, NPOL, 2)
    samples = np.ascontiguousarray(np.transpose(x, (0, 1, 3, 2, 4, 5, 6)))
    scales = np.full(shape.scales_shape(), scale_value, dtype=np.int16)
    if return_steering:
        return samples, scales, rfi_ch, steering
    return samples, scales, rfi_ch


def null_depth_db(w_eff, steering, n_beams):
    """Null depth of the projected weights on known interferers: per
    interfered channel, pol, beam and interferer, 10 log10(|w' a|^2 / |w a|^2)
    with w = slot 0 (original) and w' = slot 1 (projected) of the effective
    weights [C][Pol][2B][R] (complex) and a the interferer's steering vector.
    The beam is sum_r w_r x_r (no conjugation), so the response is w . a."""
    out = []
    for c, vecs in steering.items():
        for a in vecs:
            for p in range(NPOL):
                w0 = w_eff[c, p, :n_beams]
                w1 = w_eff[c, p, n_beams:2 * n_beams]
                r0 = np.abs(w0 @ a[:, p]) ** 2
                r1 = np.abs(w1 @ a[:, p]) ** 2
                out.append(10.0 * np.log10(np.maximum(r1, 1e-30) / np.maximum(r0, 1e-30)))
    return np.concatenate(out) if out else np.zeros(0)


def synth_weights(shape, seed=1, n_beams=None):
    """Unit-modulus weights with uniform random phase, as fp16 pairs
    [C][Pol][B][R][2] (the BeamWeightsT payload)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    B = shape.B if n_beams is None else n_beams
    ph = rng.uniform(0, 2 * np.pi, size=(shape.C, NPOL, B, shape.R))
    w = np.stack([np.cos(ph), np.sin(ph)], axis=-1).astype(np.float16)
    return w


# --------------------------------------------------------------------------
# Batched sub-arrays of uneven size: one unit = one channel-integration of a
# sub-array, int8 samples [T][R][Pol][2] (no packet padding, unit scales),
# through the adaptive chain with unit receiver factors.
# --------------------------------------------------------------------------
def unit_samples_split(x):
    """int8 [T][R][Pol][2] -> re, im int64 [1][Pol][R][T] (the layout correlate() takes)."""
    x = np.asarray(x).astype(np.int64)
    re = np.transpose(x[..., 0], (2, 1, 0))[None]
    im = np.transpose(x[..., 1], (2, 1, 0))[None]
    return re, im


def unit_chain(x, weights, k_rule="fixed", k_fixed=0, delta=10.0, orthogonal=False, beam_samples=None):
    """The adaptive chain of one unit.  weights fp16 pairs [Pol][B][R][2].
    k_rule: "fixed" (k_fixed, an int or a per-pol pair), "noise" (K =
    #{lambda > delta x median}) or "detect" (detect_k_f32).  orthogonal: null
    with the orthogonal projector onto the complement of span(U) (U = the
    un-whitened top-K vectors, orthonormalised) instead of I - U U^H.
    Returns vis (int64 [NBL][Pol][Pol][2]), evals [Pol][R] (whitened, LAPACK),
    counts [Pol], w_eff [Pol][2B][R] and beams [Pol][2B][T] (complex)."""
    T, R = x.shape[0], x.shape[1]
    sh = Shape(1, 1, T, R, R, 1, 1)
    re, im = unit_samples_split(x)
    vis = correlate(sh, re, im)
    vc = scaled_visibilities(sh, vis, receiver_factors(sh))
    w = np.asarray(weights, np.float64)
    wc = w[..., 0] + 1j * w[..., 1]  # [Pol][B][R]
    B = wc.shape[1]
    evals = np.zeros((NPOL, R))
    counts = np.zeros(NPOL, np.int32)
    w_eff = np.zeros((NPOL, 2 * B, R), np.complex128)
    for p in range(NPOL):
        m = unpack_hermitian(sh, vc, p, p)[0]
        mw, s = whiten(m)
        lam, v = eigh_ascending(mw)
        if k_rule == "noise":
            k = detect_k_noise_floor(lam, delta)
        elif k_rule == "detect":
            k = detect_k_f32(lam, delta)
        else:
            kf = np.atleast_1d(k_fixed)
            k = int(kf[p] if kf.size > 1 else kf[0])
        k = max(0, min(R, k))
        u = unwhiten_normalize(v, s)
        if orthogonal and k > 0:
            q, _ = np.linalg.qr(u[:, R - k:])
            pm = np.eye(R, dtype=np.complex128) - q @ np.conj(q.T)
        else:
            pm = null_projection(u, k)
        evals[p] = lam
        counts[p] = k
        w_eff[p, :B] = wc[p]
        w_eff[p, B:] = wc[p] @ pm
    ts = T if beam_samples is None else int(beam_samples)  # beams of the first ts samples
    beams = np.einsum("pmr,prt->pmt", w_eff, re[0][..., :ts] + 1j * im[0][..., :ts])
    return {"vis": vis[0], "evals": evals, "counts": counts, "w_eff": w_eff, "beams": beams}


def synth_unit(R, T, rng, sigma=16.0, n_interferers=0, inr_db=(5.0, 30.0)):
    """int8 [T][R][Pol][2]: noise clip(round(N(0, sigma^2))) plus n_interferers
    narrowband interferers sqrt(INR 2 sigma^2) s(t) a, ||a|| = 1 per pol, INR
    drawn uniformly in dB from inr_db."""
    re = rng.normal(0.0, sigma, size=(T, R, NPOL))
    im = rng.normal(0.0, sigma, size=(T, R, NPOL))
    t = np.arange(T)
    for _ in range(n_interferers):
        inr = 10.0 ** (rng.uniform(*inr_db) / 10.0)
        a = rng.normal(size=(R, NPOL)) + 1j * rng.normal(size=(R, NPOL))
        a /= np.linalg.norm(a, axis=0, keepdims=True)
        s = np.exp(1j * (2 * np.pi * rng.uniform(-0.45, 0.45) * t + rng.uniform(0, 2 * np.pi)))
        sig = np.sqrt(inr * 2.0 * sigma ** 2) * s[:, None, None] * a[None]
        re += np.real(sig)
        im += np.imag(sig)
    x = np.stack([np.clip(np.round(re), -127, 127), np.clip(np.round(im), -127, 127)], axis=-1)
    return x.astype(np.int8)


def synth_batch(receivers, T, B, seed=0, max_interferers=4):
    """Units of the given receiver counts with 0..max_interferers interferers
    each (INR uniform in [5, 30] dB) and unit-modulus random-phase weights
    [Pol][B][R][2] fp16."""
    rng = np.random.Generator(np.random.PCG64(seed))
    xs, ws = [], []
    for R in receivers:
        xs.append(synth_unit(int(R), T, rng, n_interferers=int(rng.integers(0, max_interferers + 1))))
        ph = rng.uniform(0, 2 * np.pi, size=(NPOL, B, int(R)))
        ws.append(np.stack([np.cos(ph), np.sin(ph)], axis=-1).astype(np.float16))
    return xs, ws


def noise_floor_k_f32(evals, delta):
    """The device's noise-floor rule in float32: K = #{lambda > delta x median},
    median = (lambda[(n-1)/2] + lambda[n/2]) / 2 of the ascending eigenvalues."""
    e = np.asarray(evals, dtype=np.float32)
    n = e.size
    med = np.float32(0.5) * (e[(n - 1) // 2] + e[n // 2])
    return int(np.count_nonzero(e > np.float32(delta) * med))
