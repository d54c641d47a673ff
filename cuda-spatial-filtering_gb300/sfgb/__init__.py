"""Python host side of the GB300 spatial-filtering hot path.

Thin ctypes binding of ``include/sf_capi.h`` plus Python mirrors of the
reference's GPU stage interface (``GPUPipeline``,
include/spatial/pipeline_base.hpp:9-40): ``execute_pipeline`` /
``dump_visibilities`` / ``set_subpacket_delays`` / ``set_antenna_gains`` /
``set_fine_delays`` over host packet buffers, writing into an ``Output``
object with the reference's output layouts.  PyTorch only supplies device
memory and streams; every computation runs in the sm_103a kernels of
``libsfgb.so``.  There is no CPU fallback: without the library (or without an
sm_103 GPU) every call raises.
"""
from __future__ import annotations

import ctypes
import os
import re
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "libsfgb.so"
HEADER = PKG.parent.parent / "include" / "sf_capi.h"

SF_OK = 0
# sf_status codes
SF_ERR_INVALID_ARGUMENT = 1
SF_ERR_UNSUPPORTED = 2
SF_ERR_CUDA = 3
SF_ERR_DEVICE = 4
SF_ERR_NO_DEVICE = 5
SF_WINDOW_PACKET = 0
SF_WINDOW_ALIGNED = 1
SF_EIG_ALL_BLOCKS = 0
SF_EIG_SAME_POL_WHITENED = 1
SF_K_FIXED = 0
SF_K_DETECT = 1
SF_K_NOISE_FLOOR = 2
SF_BEAM_FP16 = 0
SF_BEAM_BF16 = 1
SF_BEAM_E4M3 = 2
SF_BEAM_E4M3_SPLIT = 3
# device status bits (sf_device_bits)
SF_DEV_TIMEOUT_TMA = 1 << 0
SF_DEV_TIMEOUT_CONVERT = 1 << 1
SF_DEV_TIMEOUT_MMA = 1 << 2
SF_DEV_TIMEOUT_EPILOGUE = 1 << 3
SF_DEV_EIG_NOT_CONVERGED = 1 << 4
SF_DEV_BAD_SHAPE = 1 << 5
SF_DEV_BAD_DELAY = 1 << 6


class SfError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"sf error {code}: {msg}")
        self.code = code


class ShapeStruct(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int32) for n in (
        "n_channels", "n_fpgas", "n_time_per_packet", "n_receivers",
        "n_polarizations", "n_receivers_per_packet", "n_packets", "n_beams")]


_lib = None

_P = ctypes.c_void_p
_I32 = ctypes.c_int32
_SIGS = {
    "sf_plan_create": ([ctypes.POINTER(ShapeStruct), ctypes.POINTER(_P)], ctypes.c_int),
    "sf_plan_destroy": ([_P], ctypes.c_int),
    "sf_plan_get_shape": ([_P, ctypes.POINTER(ShapeStruct)], ctypes.c_int),
    "sf_last_error": ([], ctypes.c_char_p),
    "sf_plan_status": ([_P, _P, ctypes.POINTER(ctypes.c_uint32)], ctypes.c_int),
    "sf_set_subpacket_delays": ([_P, _P, _P], ctypes.c_int),
    "sf_set_antenna_gains": ([_P, _P, _P], ctypes.c_int),
    "sf_set_fine_delays": ([_P, _P, ctypes.c_double, ctypes.c_double, _I32, _P], ctypes.c_int),
    "sf_set_weights": ([_P, _P, _P], ctypes.c_int),
    "sf_set_fixed_counts": ([_P, _P, _P], ctypes.c_int),
    "sf_plan_weights_buffer": ([_P, ctypes.POINTER(_P)], ctypes.c_int),
    "sf_set_steering_weights": ([_P, _P, _P, _P, ctypes.c_double, ctypes.c_double, _I32, _P, _P], ctypes.c_int),
    "sf_set_stream_permutation": ([_P, _P, _P, _P], ctypes.c_int),
    "sf_correlate": ([_P, _P, _P, _I32, _P, _P], ctypes.c_int),
    "sf_covariance_eig": ([_P, _P, _I32, _I32, ctypes.c_float, _I32, _P, _P, _P, _P, _P], ctypes.c_int),
    "sf_beamform": ([_P, _P, _P, _I32, _I32, _P, _P], ctypes.c_int),
    "sf_get_effective_weights": ([_P, _P, _P], ctypes.c_int),
    "sf_accumulate_visibilities": ([_P, _P, _P, _P], ctypes.c_int),
    "sf_visibilities_to_float": ([_P, _P, _P, _P], ctypes.c_int),
    "sf_beam_spectra": ([_P, _P, _I32, _I32, _P, _P], ctypes.c_int),
    "sf_packet_spectra": ([_P, _P, _I32, _I32, _P, _P], ctypes.c_int),
    "sf_run_corr_beam": ([_P, _P, _P, _P, _P, _P], ctypes.c_int),
    "sf_run_lambda_gpu": ([_P, _P, _P, _P, _P, _P, _P, _P], ctypes.c_int),
    "sf_run_adaptive": ([_P, _P, _P, _I32, ctypes.c_float, _I32, _P, _P, _P, _P, _P, _P], ctypes.c_int),
    "sf_batch_create": ([_I32, _P, _I32, _I32, ctypes.POINTER(_P)], ctypes.c_int),
    "sf_batch_destroy": ([_P], ctypes.c_int),
    "sf_batch_get_layout": ([_P, _P, _P, _P, _P, _P, _P], ctypes.c_int),
    "sf_batch_set_weights": ([_P, _P, _P], ctypes.c_int),
    "sf_batch_set_fixed_counts": ([_P, _P, _P], ctypes.c_int),
    "sf_batch_correlate": ([_P, _P, _P, _P], ctypes.c_int),
    "sf_batch_covariance_eig": ([_P, _P, _I32, ctypes.c_float, _I32, _P, _P, _P], ctypes.c_int),
    "sf_batch_beamform": ([_P, _P, _P, _P], ctypes.c_int),
    "sf_batch_run": ([_P, _P, _I32, ctypes.c_float, _I32, _P, _P, _P, _P, _P], ctypes.c_int),
    "sf_batch_status": ([_P, _P, ctypes.POINTER(ctypes.c_uint32)], ctypes.c_int),
    "sf_batch_set_precision": ([_P, _I32, _I32, _I32], ctypes.c_int),
    "sf_batch_precision_report": ([_P, _P, _P, _P], ctypes.c_int),
    "sf_batch_effective_weights": ([_P, _P, _P], ctypes.c_int),
    "sf_batch_autotune": ([_P, _P, _I32, ctypes.c_float, _P, _P, _P, _P, _P, ctypes.c_char_p, _I32], ctypes.c_int),
    "sf_proposer_create": ([_I32, _I32, _I32, ctypes.POINTER(_P)], ctypes.c_int),
    "sf_proposer_destroy": ([_P], ctypes.c_int),
    "sf_proposer_dims": ([_P, _P], ctypes.c_int),
    "sf_proposer_set_params": ([_P, _P, _P, _P, _P, _P, _P, _P], ctypes.c_int),
    "sf_proposer_get_params": ([_P, _P, _P, _P, _P, _P, _P, _P], ctypes.c_int),
    "sf_proposer_features": ([_P, _P, _P, _I32, _P], ctypes.c_int),
    "sf_proposer_targets": ([_P, _P, _P, _P, _P, _P, _P], ctypes.c_int),
    "sf_proposer_infer": ([_P, _P, _I32, _P, _P], ctypes.c_int),
    "sf_proposer_train_step": ([_P, _P, _P, _P, _I32, ctypes.c_float, _P, _P], ctypes.c_int),
    "sf_proposer_status": ([_P, _P, ctypes.POINTER(ctypes.c_uint32)], ctypes.c_int),
    "sf_covariance_eig_learned": ([_P, _P, _P, _I32, ctypes.c_float, _I32, ctypes.c_float, _P, _P, _P, _P],
                                  ctypes.c_int),
    "sf_run_adaptive_learned": ([_P, _P, _P, _P, _I32, ctypes.c_float, _I32, ctypes.c_float, _P, _P, _P, _P, _P],
                                ctypes.c_int),
    "sf_gemm_bf16": ([_I32, _I32, _I32, _P, _I32, _I32, _P, _I32, _I32, _I32, _P, _P, _I32, _P, _I32, _I32, _P, _P],
                     ctypes.c_int),
    "sf_run_adaptive_noalloc": ([ctypes.POINTER(ShapeStruct), _P, _P, _P, _P, _P, _P, _I32, ctypes.c_float,
                                 _I32, _P, _P, _P, _P], ctypes.c_int),
}


def header_symbols():
    """Function names declared in include/sf_capi.h."""
    text = HEADER.read_text()
    return sorted(set(re.findall(r"^\s*(?:int|const char \*)\s*(sf_\w+)\s*\(", text, re.M)))


def run_adaptive_noalloc(shape, samples, scales, weights, k_rule, delta, shrink, beams, factors=None,
                         delays=None, fixed_counts=None, counts=None, status=None, stream=None):
    """sf_run_adaptive_noalloc over caller-owned device tensors (no plan).
    ``shape`` is (C, F, Tp, R, Rpp, P, B)."""
    C, F, Tp, R, Rpp, P, B = shape
    st = ShapeStruct(C, F, Tp, R, 2, Rpp, P, B)
    _check(lib().sf_run_adaptive_noalloc(ctypes.byref(st), _ptr(samples), _ptr(scales), _ptr(weights),
                                         _ptr(factors), _ptr(delays), _ptr(fixed_counts), int(k_rule),
                                         float(delta), int(bool(shrink)), _ptr(counts), _ptr(beams),
                                         _ptr(status), _stream(stream)))


def lib():
    """Load libsfgb.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} is missing: run __graft_entry__.build() first")
        L = ctypes.CDLL(str(LIB_PATH))
        for name, (args, res) in _SIGS.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _lib = L
    return _lib


def _check(rc):
    if rc != SF_OK:
        raise SfError(rc, lib().sf_last_error().decode())


def _ptr(t):
    if t is None:
        return None
    return ctypes.c_void_p(t.data_ptr())


def _stream(stream=None):
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


class Plan:
    """Owns one sf_plan (device state for one integration shape)."""

    def __init__(self, n_channels, n_fpgas, n_time_per_packet, n_receivers,
                 n_receivers_per_packet, n_packets, n_beams):
        import torch
        if not torch.cuda.is_available():
            raise RuntimeError("no CUDA device: the spatial-filtering kernels need an sm_103 GPU")
        self.C, self.F, self.Tp = n_channels, n_fpgas, n_time_per_packet
        self.R, self.Rpp, self.P, self.B = n_receivers, n_receivers_per_packet, n_packets, n_beams
        self.T = self.P * self.Tp
        self.NBL = self.R * (self.R + 1) // 2
        shape = ShapeStruct(n_channels, n_fpgas, n_time_per_packet, n_receivers, 2,
                            n_receivers_per_packet, n_packets, n_beams)
        h = ctypes.c_void_p()
        _check(lib().sf_plan_create(ctypes.byref(shape), ctypes.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            lib().sf_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- shapes ----
    def samples_shape(self):
        return (self.C, self.P + 2, self.F, self.Tp, self.Rpp, 2, 2)

    def scales_shape(self):
        return (self.C, self.P + 2, self.R, 2)

    def vis_shape(self):
        return (self.C, self.NBL, 2, 2, 2)

    def beams_shape(self, n_slots=1):
        return (self.C, 2, n_slots * self.B, self.T, 2)

    # ---- configuration ----
    def set_subpacket_delays(self, delays=None, stream=None):
        arr = None if delays is None else np.ascontiguousarray(delays, dtype=np.int32)
        _check(lib().sf_set_subpacket_delays(self._h, None if arr is None else arr.ctypes.data_as(_P),
                                             _stream(stream)))

    def set_antenna_gains(self, gains=None, stream=None):
        arr = None
        if gains is not None:
            g = np.asarray(gains).reshape(self.C, 2, self.R)
            arr = np.ascontiguousarray(np.stack([g.real, g.imag], axis=-1).astype(np.float32))
        _check(lib().sf_set_antenna_gains(self._h, None if arr is None else arr.ctypes.data_as(_P),
                                          _stream(stream)))

    def set_fine_delays(self, delays_ns, base_freq_hz, channel_bw_hz, min_freq_ch, stream=None):
        arr = np.ascontiguousarray(delays_ns, dtype=np.float32)
        _check(lib().sf_set_fine_delays(self._h, arr.ctypes.data_as(_P), float(base_freq_hz),
                                        float(channel_bw_hz), int(min_freq_ch), _stream(stream)))

    def set_weights(self, weights_f16, stream=None):
        arr = np.ascontiguousarray(weights_f16, dtype=np.float16).reshape(self.C, 2, self.B, self.R, 2)
        _check(lib().sf_set_weights(self._h, arr.ctypes.data_as(_P), _stream(stream)))

    def set_stream_permutation(self, recv_perm=None, pol_perm=None, stream=None):
        """Canonical stream k = 2 r + p <- source receiver recv_perm[k] at pol
        pol_perm[k] (-1 = zero); both None restores the identity."""
        if recv_perm is None and pol_perm is None:
            _check(lib().sf_set_stream_permutation(self._h, None, None, _stream(stream)))
            return
        rp = np.ascontiguousarray(recv_perm, dtype=np.int32).reshape(-1)
        pp = np.ascontiguousarray(pol_perm, dtype=np.int32).reshape(-1)
        if rp.size != 2 * self.R or pp.size != 2 * self.R:
            raise ValueError("set_stream_permutation: size must equal 2 x receivers")
        _check(lib().sf_set_stream_permutation(self._h, rp.ctypes.data_as(_P), pp.ctypes.data_as(_P),
                                               _stream(stream)))

    def set_steering_weights(self, dircos, enu, connected=None, base_freq_hz=0.0, channel_bw_hz=0.0,
                             min_freq_ch=0, calibration_gains=None, stream=None):
        """Weights synthesised on the device from direction cosines [B][3] and
        antenna positions [R][3] (ENU metres); connected[r] == 0 marks a null
        input; calibration_gains complex [C][Pol][R] or None."""
        dc = np.ascontiguousarray(dircos, dtype=np.float64).reshape(self.B, 3)
        pos = np.ascontiguousarray(enu, dtype=np.float64).reshape(self.R, 3)
        conn = None if connected is None else np.ascontiguousarray(connected, dtype=np.int32).reshape(self.R)
        cal = None
        if calibration_gains is not None:
            g = np.asarray(calibration_gains).reshape(self.C, 2, self.R)
            cal = np.ascontiguousarray(np.stack([g.real, g.imag], axis=-1).astype(np.float32))
        _check(lib().sf_set_steering_weights(
            self._h, dc.ctypes.data_as(_P), pos.ctypes.data_as(_P), None if conn is None else conn.ctypes.data_as(_P),
            float(base_freq_hz), float(channel_bw_hz), int(min_freq_ch),
            None if cal is None else cal.ctypes.data_as(_P), _stream(stream)))

    def set_fixed_counts(self, counts=None, stream=None):
        arr = None if counts is None else np.ascontiguousarray(counts, dtype=np.int32)
        _check(lib().sf_set_fixed_counts(self._h, None if arr is None else arr.ctypes.data_as(_P),
                                         _stream(stream)))

    def status(self, stream=None):
        bits = ctypes.c_uint32(0)
        rc = lib().sf_plan_status(self._h, _stream(stream), ctypes.byref(bits))
        return rc, bits.value

    # ---- stages (device tensors) ----
    def correlate(self, samples, scales, window, vis, stream=None):
        _check(lib().sf_correlate(self._h, _ptr(samples), _ptr(scales), int(window), _ptr(vis),
                                  _stream(stream)))

    def covariance_eig(self, vis, eig_mode, k_rule=SF_K_FIXED, delta=0.0, shrink=False, evals=None,
                       evecs=None, counts=None, proj=None, stream=None):
        _check(lib().sf_covariance_eig(self._h, _ptr(vis), int(eig_mode), int(k_rule), float(delta),
                                       int(bool(shrink)), _ptr(evals), _ptr(evecs), _ptr(counts),
                                       _ptr(proj), _stream(stream)))

    def effective_weights(self, out, stream=None):
        """Copy the plan's (original, projected) effective weights into ``out``
        (float32 [C][2][2B][R][2] device tensor)."""
        _check(lib().sf_get_effective_weights(self._h, _ptr(out), _stream(stream)))

    def beamform(self, samples, scales, window, n_slots, beams, stream=None):
        _check(lib().sf_beamform(self._h, _ptr(samples), _ptr(scales), int(window), int(n_slots),
                                 _ptr(beams), _stream(stream)))

    def accumulate_visibilities(self, vis, accum, stream=None):
        _check(lib().sf_accumulate_visibilities(self._h, _ptr(vis), _ptr(accum), _stream(stream)))

    def visibilities_to_float(self, accum, out, stream=None):
        _check(lib().sf_visibilities_to_float(self._h, _ptr(accum), _ptr(out), _stream(stream)))

    def beam_spectra(self, beams, n_beams_out, downsample, spectra, stream=None):
        """Whole-integration |FFT|^2 spectra, downsampled by `downsample` bins."""
        _check(lib().sf_beam_spectra(self._h, _ptr(beams), int(n_beams_out), int(downsample),
                                     _ptr(spectra), _stream(stream)))

    def packet_spectra(self, beams, n_beams_out, trim, spectra, stream=None):
        """Per-packet |FFT| summed over packets, `trim` edge bins dropped each side."""
        _check(lib().sf_packet_spectra(self._h, _ptr(beams), int(n_beams_out), int(trim),
                                       _ptr(spectra), _stream(stream)))

    def beam_spectra_shape(self, n_beams_out, downsample):
        return (self.C, 2, n_beams_out, self.T // downsample)

    def packet_spectra_shape(self, n_beams_out, trim):
        return (self.C, 2, n_beams_out, self.Tp - 2 * trim)

    # ---- whole chains ----
    def run_corr_beam(self, samples, scales, vis, beams, stream=None):
        _check(lib().sf_run_corr_beam(self._h, _ptr(samples), _ptr(scales), _ptr(vis), _ptr(beams),
                                      _stream(stream)))

    def run_lambda_gpu(self, samples, scales, vis, evals, evecs, beams, stream=None):
        _check(lib().sf_run_lambda_gpu(self._h, _ptr(samples), _ptr(scales), _ptr(vis), _ptr(evals),
                                       _ptr(evecs), _ptr(beams), _stream(stream)))

    def proposer_features(self, vis, x, ld, stream=None):
        _check(lib().sf_proposer_features(self._h, _ptr(vis), _ptr(x), int(ld), _stream(stream)))

    def proposer_targets(self, vis, evals, evecs, targets, weights, stream=None):
        _check(lib().sf_proposer_targets(self._h, _ptr(vis), _ptr(evals), _ptr(evecs), _ptr(targets), _ptr(weights),
                                         _stream(stream)))

    def covariance_eig_learned(self, proposer, vis, k_rule, delta, n_iter, tol, counts=None, ritz=None,
                               fallback_count=None, stream=None):
        _check(lib().sf_covariance_eig_learned(self._h, proposer._h, _ptr(vis), int(k_rule), float(delta), int(n_iter),
                                               float(tol), _ptr(counts), _ptr(ritz), _ptr(fallback_count),
                                               _stream(stream)))

    def run_adaptive_learned(self, proposer, samples, scales, k_rule, delta, n_iter, tol, vis, counts, beams,
                             fallback_count=None, stream=None):
        _check(lib().sf_run_adaptive_learned(self._h, proposer._h, _ptr(samples), _ptr(scales), int(k_rule),
                                             float(delta), int(n_iter), float(tol), _ptr(vis), _ptr(counts),
                                             _ptr(beams), _ptr(fallback_count), _stream(stream)))

    def run_adaptive(self, samples, scales, k_rule, delta, shrink, vis, evals, evecs, counts, beams,
                     stream=None):
        _check(lib().sf_run_adaptive(self._h, _ptr(samples), _ptr(scales), int(k_rule), float(delta),
                                     int(bool(shrink)), _ptr(vis), _ptr(evals), _ptr(evecs),
                                     _ptr(counts), _ptr(beams), _stream(stream)))


from .pipelines import (  # noqa: E402
    GPUPipeline, LambdaAdaptiveBeamformedSpectraPipeline, LambdaCorrBeamOnlyGPUPipeline,
    LambdaGPUPipeline, PacketData, SingleHostMemoryOutput)

__all__ = ["Plan", "SfError", "lib", "header_symbols", "GPUPipeline", "LambdaGPUPipeline",
           "LambdaCorrBeamOnlyGPUPipeline", "LambdaAdaptiveBeamformedSpectraPipeline",
           "PacketData", "SingleHostMemoryOutput"]


class Batch:
    """A batch of sub-array units of uneven receiver counts (sf_batch_*).

    ``receivers``: receiver count per unit; every unit has ``n_samples``
    samples and ``n_beams`` beams.  ``layout`` holds the per-unit offsets of
    every buffer (sample bytes, vis int32 elements, weight fp16 pairs, eval
    floats, beam fp16 pairs) and ``totals`` the buffer sizes."""

    def __init__(self, receivers, n_samples, n_beams):
        import torch
        if not torch.cuda.is_available():
            raise RuntimeError("no CUDA device: the spatial-filtering kernels need an sm_103 GPU")
        self.receivers = np.ascontiguousarray(receivers, dtype=np.int32)
        self.n_units = int(self.receivers.size)
        self.T, self.B = int(n_samples), int(n_beams)
        h = ctypes.c_void_p()
        _check(lib().sf_batch_create(self.n_units, self.receivers.ctypes.data_as(_P), self.T, self.B,
                                     ctypes.byref(h)))
        self._h = h
        tot = np.zeros(5, np.int64)
        offs = [np.zeros(self.n_units, np.int64) for _ in range(5)]
        _check(lib().sf_batch_get_layout(self._h, tot.ctypes.data_as(_P), *[o.ctypes.data_as(_P) for o in offs]))
        self.totals = {k: int(v) for k, v in zip(("samples", "vis", "weights", "evals", "beams"), tot)}
        self.layout = dict(zip(("samples", "vis", "weights", "evals", "beams"), offs))

    def close(self):
        if getattr(self, "_h", None):
            lib().sf_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- host-side packing helpers (layout only; no arithmetic) ----
    def pack_samples(self, units):
        """List of int8 [T][R][Pol][2] -> one int8 array in the batch layout."""
        out = np.zeros(self.totals["samples"], np.int8)
        for u, x in enumerate(units):
            o = int(self.layout["samples"][u])
            out[o:o + x.size] = np.ascontiguousarray(x, np.int8).reshape(-1)
        return out

    def pack_weights(self, weights):
        """List of fp16 [Pol][B][R][2] -> one fp16 array (pairs at the layout's offsets)."""
        out = np.zeros(2 * self.totals["weights"], np.float16)
        for u, w in enumerate(weights):
            o = 2 * int(self.layout["weights"][u])
            out[o:o + w.size] = np.ascontiguousarray(w, np.float16).reshape(-1)
        return out

    def unit_vis(self, vis, u):
        R = int(self.receivers[u])
        o = int(self.layout["vis"][u])
        return vis[o:o + R * (R + 1) // 2 * 8].reshape(R * (R + 1) // 2, 2, 2, 2)

    def unit_evals(self, evals, u):
        R = int(self.receivers[u])
        o = int(self.layout["evals"][u])
        return evals[o:o + 2 * R].reshape(2, R)

    def unit_beams(self, beams, u):
        """fp16 [Pol][2B][T][2] of unit u from the flat beam buffer (fp16 elements)."""
        o = 2 * int(self.layout["beams"][u])
        n = 2 * 2 * self.B * self.T * 2
        return beams[o:o + n].reshape(2, 2 * self.B, self.T, 2)

    # ---- device calls ----
    def set_weights(self, packed_f16, stream=None):
        arr = np.ascontiguousarray(packed_f16, dtype=np.float16)
        _check(lib().sf_batch_set_weights(self._h, arr.ctypes.data_as(_P), _stream(stream)))

    def set_fixed_counts(self, counts=None, stream=None):
        arr = None if counts is None else np.ascontiguousarray(counts, dtype=np.int32)
        _check(lib().sf_batch_set_fixed_counts(self._h, None if arr is None else arr.ctypes.data_as(_P),
                                               _stream(stream)))

    def correlate(self, samples, vis, stream=None):
        _check(lib().sf_batch_correlate(self._h, _ptr(samples), _ptr(vis), _stream(stream)))

    def covariance_eig(self, vis, k_rule, delta, shrink, evals, counts, stream=None):
        _check(lib().sf_batch_covariance_eig(self._h, _ptr(vis), int(k_rule), float(delta), int(bool(shrink)),
                                             _ptr(evals), _ptr(counts), _stream(stream)))

    def beamform(self, samples, beams, stream=None):
        _check(lib().sf_batch_beamform(self._h, _ptr(samples), _ptr(beams), _stream(stream)))

    def run(self, samples, k_rule, delta, shrink, vis, evals, counts, beams, stream=None):
        _check(lib().sf_batch_run(self._h, _ptr(samples), int(k_rule), float(delta), int(bool(shrink)), _ptr(vis),
                                  _ptr(evals), _ptr(counts), _ptr(beams), _stream(stream)))

    def status(self, stream=None):
        bits = ctypes.c_uint32(0)
        rc = lib().sf_batch_status(self._h, _stream(stream), ctypes.byref(bits))
        return rc, bits.value

    def set_precision(self, beam_precision, refine_steps=2, orthogonal=True):
        _check(lib().sf_batch_set_precision(self._h, int(beam_precision), int(refine_steps), int(bool(orthogonal))))

    def effective_weights(self, stream=None):
        """Per unit complex128 [Pol][2B][R] effective weights of the last eigen stage."""
        import torch
        w = torch.empty(4 * self.totals["weights"], dtype=torch.float32, device="cuda")
        _check(lib().sf_batch_effective_weights(self._h, _ptr(w), _stream(stream)))
        torch.cuda.synchronize()
        h = w.cpu().numpy().astype(np.float64)
        out = []
        for u, R in enumerate(self.receivers):
            o = 4 * int(self.layout["weights"][u])
            blk = h[o:o + 2 * 2 * self.B * int(R) * 2].reshape(2, 2 * self.B, int(R), 2)
            out.append(blk[..., 0] + 1j * blk[..., 1])
        return out

    def precision_report(self, stream=None):
        """(residuals [u][Pol][2] before/after, FP64 Ritz values [u][Pol][8]) of the last refined run."""
        r = np.zeros((self.n_units, 2, 2), np.float32)
        t = np.zeros((self.n_units, 2, 8), np.float64)
        _check(lib().sf_batch_precision_report(self._h, r.ctypes.data_as(_P), t.ctypes.data_as(_P), _stream(stream)))
        return r, t

    def autotune(self, samples, k_rule, delta, vis, evals, counts, beams, stream=None):
        """Runs the autotuner; returns its JSON record (dict)."""
        import json
        buf = ctypes.create_string_buffer(8192)
        _check(lib().sf_batch_autotune(self._h, _ptr(samples), int(k_rule), float(delta), _ptr(vis), _ptr(evals),
                                       _ptr(counts), _ptr(beams), _stream(stream), buf, len(buf)))
        return json.loads(buf.value.decode())


def gemm_bf16(M, N, K, A, lda, a_mn, B, ldb, b_mn, epilogue, out, ldo, bias=None, mask=None, ldm=0, k_splits=1,
              status=None, stream=None):
    """sf_gemm_bf16 on device tensors (A, B, mask bf16; out bf16 or fp32)."""
    import torch
    st = status if status is not None else torch.zeros(1, dtype=torch.int32, device=A.device)
    _check(lib().sf_gemm_bf16(int(M), int(N), int(K), _ptr(A), int(lda), int(a_mn), _ptr(B), int(ldb), int(b_mn),
                              int(epilogue), _ptr(bias), _ptr(mask), int(ldm), _ptr(out), int(ldo), int(k_splits),
                              _ptr(st), _stream(stream)))
    return st
