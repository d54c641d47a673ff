"""The spectra oracle pinned to its definitions (CPU).

The reference's tests only assert that its FFT output is finite
(tests/test_adaptive_pipeline.cu:369-370), so there are no golden spectra.  The
oracle is pinned instead to (a) the DFT definition cuFFT's CUFFT_FORWARD
computes, by the O(N^2) sum, and (b) the reference's own sequence of buffer
operations for the adaptive tail, replayed literally below: the
frequency-major permutation, the two half copies and the per-packet sum of
magnitudes (lambda_adaptive_beamformed_spectra_pipeline.hpp:808-848,
spatial.cuh:1508-1567), and detect_and_downsample_fft's loop
(spatial.cuh:795-835).
"""
import numpy as np

import sf_oracle as orc


def test_numpy_fft_is_the_forward_dft():
    rng = np.random.default_rng(0)
    for n in (16, 64, 256):
        x = rng.standard_normal((3, n)) + 1j * rng.standard_normal((3, n))
        assert np.abs(np.fft.fft(x) - orc.dft_direct(x)).max() < 1e-9 * n


def _reference_adaptive_tail(beams_c, Tp, P, trim):
    """The adaptive tail's buffer operations, step by step."""
    C, NP, NB, T = beams_c.shape
    fft = np.fft.fft(beams_c.reshape(C, NP, NB, P, Tp), axis=-1)        # [c][p][e][o][u]
    fine = np.transpose(fft, (4, 0, 1, 2, 3)).reshape(Tp, -1)             # [u][c p e o]
    kept = Tp - 2 * trim
    removed = np.empty((kept, fine.shape[1]), dtype=fine.dtype)           # [g][c p e o]
    half = kept // 2                                                      # FineChannelCopyType
    seek = Tp // 2 + trim                                                 # FineChannelSeekType
    removed[half:half + half] = fine[0:half]         # first half -> second half of destination
    removed[0:half] = fine[seek:seek + half]         # from the seek point -> start
    down = np.transpose(removed.reshape(kept, C, NP, NB, P), (1, 2, 3, 4, 0))  # [c][p][e][o][g]
    out = np.zeros((C, NP, NB, kept))
    for o in range(P):                               # sum_fft_over_packets
        out += np.sqrt(down[:, :, :, o].real ** 2 + down[:, :, :, o].imag ** 2)
    return out


def test_packet_spectra_replays_reference_buffer_steps():
    rng = np.random.default_rng(1)
    for Tp, P, trim in ((64, 4, 5), (64, 1, 0), (32, 3, 5), (16, 2, 7)):
        b = rng.standard_normal((2, 2, 3, Tp * P)) + 1j * rng.standard_normal((2, 2, 3, Tp * P))
        got = orc.packet_spectra(b, Tp, trim)
        ref = _reference_adaptive_tail(b, Tp, P, trim)
        assert np.allclose(got, ref, rtol=1e-12, atol=1e-12)


def _reference_detect(fft, D):
    """detect_and_downsample_fft's per-thread loop."""
    S, T = fft.shape
    n_out = T // D
    out = np.zeros((S, n_out))
    for s in range(S):
        for g in range(n_out):
            acc, cnt = 0.0, 0
            for j in range(D):
                v = fft[s, g * D + j]
                val = v.real * v.real + v.imag * v.imag
                if not np.isnan(val):
                    acc += val
                    cnt += 1
            out[s, g] = acc / cnt if cnt > 0 else 0.0
    return out


def test_beam_spectra_replays_detect_and_downsample():
    rng = np.random.default_rng(2)
    for T, D in ((64, 1), (64, 7), (128, 16), (256, 256)):
        b = rng.standard_normal((2, 2, 2, T)) + 1j * rng.standard_normal((2, 2, 2, T))
        b[1, 1, 0, 5] = np.nan
        got = orc.beam_spectra(b, D)
        ref = _reference_detect(np.fft.fft(b.reshape(-1, T), axis=-1), D).reshape(got.shape)
        assert np.allclose(got, ref, rtol=1e-12, atol=0)
        assert np.all(got[1, 1, 0] == 0.0)


def test_fine_channel_order_lambda_shape():
    order = orc.fine_channel_order(64, 5)
    assert len(order) == 54
    assert list(order[:27]) == list(range(37, 64)) and list(order[27:]) == list(range(0, 27))
