"""Python mirrors of the reference's GPU stage interface over sf_capi.

``GPUPipeline`` mirrors include/spatial/pipeline_base.hpp:9-40 (same method
names and argument meaning; ``set_stream_permutation`` as LambdaGPUPipeline's,
lambda_gpu_pipeline.hpp:1139-1150); the three subclasses mirror the drop-in
targets:

  LambdaCorrBeamOnlyGPUPipeline   lambda_corr_beam_only_gpu_pipeline.hpp:202-344
  LambdaGPUPipeline               lambda_gpu_pipeline.hpp:445-608
  LambdaAdaptiveBeamformedSpectraPipeline
                                  lambda_adaptive_beamformed_spectra_pipeline.hpp:563-957

``execute_pipeline`` takes a ``PacketData`` (the FinalPacketData payload:
host samples/scales in the packet layout), copies it to the device, runs the
chain, accumulates visibilities and lands the beams (and eigen outputs) in
the ``Output`` object, as the reference does with cudaMemcpyAsync into
landing pointers.  LambdaGPUPipeline and the adaptive pipeline also land their
spectra tails (``fft_output``): whole-integration |FFT|^2 downsampled by
``fft_downsample_factor`` (lambda_gpu_pipeline.hpp:522-531), and per-packet |FFT|
summed over packets with 5 edge bins trimmed each side
(lambda_adaptive_beamformed_spectra_pipeline.hpp:808-848); shapes the spectra
kernels do not cover (T not a power of two in [64, 16384]; Tp not 16, 32 or
64) skip the tail and leave ``fft_output`` None.  ``dump_visibilities`` converts the accumulator to the
reference's float layout and resets it.
"""
from __future__ import annotations

import numpy as np

from . import (SF_K_DETECT, SF_K_FIXED, Plan)


class PacketData:
    """FinalPacketData payload (packet_formats.hpp:50-66)."""

    def __init__(self, samples, scales, start_seq_id=0, end_seq_id=0, arrivals=None,
                 buffer_index=0):
        self.samples = samples
        self.scales = scales
        self.start_seq_id = start_seq_id
        self.end_seq_id = end_seq_id
        self.arrivals = arrivals
        self.buffer_index = buffer_index

    def get_num_missing_packets(self):
        if self.arrivals is None:
            return 0
        a = np.asarray(self.arrivals)
        return int(np.count_nonzero(a[:, 1:-1] == 0))


class SingleHostMemoryOutput:
    """Host landing buffers (output.hpp:60-169)."""

    def __init__(self):
        self.beam_data = None
        self.visibilities = None
        self.eigenvalues = None
        self.eigenvectors = None
        self.nulled_eigenmode_counts = None
        self.fft_output = None
        self.blocks = 0
        self.fft_blocks = 0

    def register_beam_data_block(self, start_seq, end_seq):
        self.blocks += 1
        return 1

    def register_visibilities_block(self, start_seq, end_seq, missing, total):
        return 1

    def register_fft_block(self, start_seq, end_seq):
        self.fft_blocks += 1
        return 1


class BeamSteering:
    """BeamSteering mirror (include/spatial/pipeline/common.hpp:187-327): keeps
    every registered plan's weights pointed at the targets, recomputed on the
    device (Plan.set_steering_weights) at most once per update interval.
    Inert without targets.  targets: list of dicts {"mode": "zenith"|"radec",
    "ra_deg", "dec_deg"}; antenna_positions: {antenna id: (east, north, up)};
    antenna_mapping: {receiver index: antenna id} (negative = null input);
    calibration_gains: complex [C][Pol][R] or None."""

    def __init__(self, targets, antenna_positions, antenna_mapping, base_frequency_hz, channel_bandwidth_hz,
                 min_freq_channel, latitude_deg=0.0, longitude_deg=0.0, height_m=0.0,
                 update_interval_seconds=180.0, calibration_gains=None, clock=None):
        import time
        self.targets = list(targets or [])
        self.positions = dict(antenna_positions or {})
        self.mapping = dict(antenna_mapping or {})
        self.base, self.bw, self.min_ch = float(base_frequency_hz), float(channel_bandwidth_hz), int(min_freq_channel)
        self.site = (float(latitude_deg), float(longitude_deg), float(height_m))
        self.interval = float(update_interval_seconds)
        self.cal = calibration_gains
        self.clock = clock or time.time
        self.plans = []
        self.last_update = None

    def active(self):
        return bool(self.targets)

    def register_plan(self, plan, stream=None):
        self.plans.append((plan, stream))

    def refresh(self, unix_seconds):
        from . import pointing
        for plan, stream in self.plans:
            dircos, enu, conn = pointing.steering_geometry(plan.B, plan.R, self.targets, self.positions,
                                                           self.mapping, unix_seconds, *self.site)
            plan.set_steering_weights(dircos, enu, conn, self.base, self.bw, self.min_ch, self.cal, stream=stream)
        self.last_update = unix_seconds

    def maybe_refresh(self):
        if not self.active() or not self.plans:
            return False
        now = self.clock()
        if self.last_update is not None and now - self.last_update < self.interval:
            return False
        self.refresh(now)
        return True


class GPUPipeline:
    def __init__(self):
        self.state_ = None
        self.output_ = None
        self.steering_ = None

    def set_state(self, state):
        self.state_ = state

    def set_output(self, output):
        self.output_ = output

    def set_subpacket_delays(self, delays):
        self.plan.set_subpacket_delays(delays)

    def set_antenna_gains(self, gains):
        self.plan.set_antenna_gains(gains)

    def set_fine_delays(self, delays_ns, base_freq_hz, channel_bw_hz, min_freq_ch):
        self.plan.set_fine_delays(delays_ns, base_freq_hz, channel_bw_hz, min_freq_ch)

    def set_stream_permutation(self, recv_perm, pol_perm):
        # lambda_gpu_pipeline.hpp:1139-1150: sizes must be F * Rpp * Pol
        if len(recv_perm) != 2 * self.plan.R or len(pol_perm) != 2 * self.plan.R:
            raise RuntimeError("set_stream_permutation: size must equal NR_FPGA_SOURCES * "
                               "NR_RECEIVERS_PER_PACKET * NR_POLARIZATIONS")
        self.plan.set_stream_permutation(recv_perm, pol_perm)

    def set_beam_steering(self, steering):
        self.steering_ = steering
        steering.register_plan(self.plan, getattr(self, "stream", None))

    def execute_pipeline(self, packet_data, dummy_run=False):
        raise NotImplementedError

    def dump_visibilities(self, end_seq_num=0):
        raise NotImplementedError


class _Base(GPUPipeline):
    n_slots = 1

    def __init__(self, shape, weights, nr_blocks_to_accumulate=1 << 30):
        import torch
        super().__init__()
        C, F, Tp, R, Rpp, P, B = shape
        self.plan = Plan(C, F, Tp, R, Rpp, P, B)
        self.plan.set_weights(weights)
        self.nr_blocks = int(nr_blocks_to_accumulate)
        dev = torch.device("cuda")
        self.stream = torch.cuda.Stream()
        p = self.plan
        self.d_samples = torch.empty(p.samples_shape(), dtype=torch.int8, device=dev)
        self.d_scales = torch.empty(p.scales_shape(), dtype=torch.int16, device=dev)
        self.d_vis = torch.empty(p.vis_shape(), dtype=torch.int32, device=dev)
        self.d_accum = torch.zeros(p.vis_shape(), dtype=torch.int64, device=dev)
        self.d_vis_f = torch.empty(p.vis_shape(), dtype=torch.float32, device=dev)
        self.d_beams = torch.empty(p.beams_shape(self.n_slots), dtype=torch.float16, device=dev)
        self.integrated = 0

    def _ingest(self, packet_data):
        import torch
        if self.steering_ is not None:
            self.steering_.maybe_refresh()  # first, as the reference's execute_pipeline
        with torch.cuda.stream(self.stream):
            s = torch.as_tensor(np.ascontiguousarray(packet_data.samples)).view(torch.int8)
            sc = torch.as_tensor(np.ascontiguousarray(packet_data.scales)).view(torch.int16)
            self.d_samples.copy_(s.reshape(self.d_samples.shape), non_blocking=False)
            self.d_scales.copy_(sc.reshape(self.d_scales.shape), non_blocking=False)

    def _finish(self, packet_data, dummy_run, extra, spectra=None):
        import torch
        self.plan.accumulate_visibilities(self.d_vis, self.d_accum, stream=self.stream)
        if self.output_ is not None and not dummy_run:
            self.output_.register_beam_data_block(packet_data.start_seq_id, packet_data.end_seq_id)
            with torch.cuda.stream(self.stream):
                self.output_.beam_data = self.d_beams.cpu().numpy()
                for k, v in extra.items():
                    setattr(self.output_, k, v.cpu().numpy())
            if spectra is not None:
                self.output_.register_fft_block(packet_data.start_seq_id, packet_data.end_seq_id)
                with torch.cuda.stream(self.stream):
                    self.output_.fft_output = spectra.cpu().numpy()
            self.integrated += 1
            if self.integrated >= self.nr_blocks:
                self.dump_visibilities()
        self.stream.synchronize()

    def dump_visibilities(self, end_seq_num=0):
        import torch
        self.plan.visibilities_to_float(self.d_accum, self.d_vis_f, stream=self.stream)
        if self.output_ is not None:
            self.output_.register_visibilities_block(0, end_seq_num, 0, 0)
            with torch.cuda.stream(self.stream):
                self.output_.visibilities = self.d_vis_f.cpu().numpy()
        with torch.cuda.stream(self.stream):
            self.d_accum.zero_()
        self.integrated = 0
        self.stream.synchronize()


class LambdaCorrBeamOnlyGPUPipeline(_Base):
    def execute_pipeline(self, packet_data, dummy_run=False):
        self._ingest(packet_data)
        self.plan.run_corr_beam(self.d_samples, self.d_scales, self.d_vis, self.d_beams, stream=self.stream)
        self._finish(packet_data, dummy_run, {})


def whole_spectra_supported(T):
    return 64 <= T <= 16384 and (T & (T - 1)) == 0


def packet_spectra_supported(Tp):
    return Tp in (16, 32, 64)


FINE_CHANNELS_TO_REMOVE_EACH_SIDE = 5  # lambda_adaptive_beamformed_spectra_pipeline.hpp:23


class LambdaGPUPipeline(_Base):
    def __init__(self, shape, weights, nr_blocks_to_accumulate=1 << 30, fft_downsample_factor=128):
        import torch
        super().__init__(shape, weights, nr_blocks_to_accumulate)
        p = self.plan
        self.d_evals = torch.empty((p.C, 2, 2, p.R), dtype=torch.float32, device="cuda")
        self.d_evecs = torch.empty((p.C, 2, 2, p.R, p.R, 2), dtype=torch.float32, device="cuda")
        self.fft_downsample = int(fft_downsample_factor)
        self.d_spectra = None
        if whole_spectra_supported(p.T) and 1 <= self.fft_downsample <= p.T:
            self.d_spectra = torch.empty(p.beam_spectra_shape(p.B, self.fft_downsample), dtype=torch.float32,
                                         device="cuda")

    def execute_pipeline(self, packet_data, dummy_run=False):
        self._ingest(packet_data)
        self.plan.run_lambda_gpu(self.d_samples, self.d_scales, self.d_vis, self.d_evals, self.d_evecs,
                                 self.d_beams, stream=self.stream)
        if self.d_spectra is not None:
            self.plan.beam_spectra(self.d_beams, self.plan.B, self.fft_downsample, self.d_spectra,
                                   stream=self.stream)
        self._finish(packet_data, dummy_run, {"eigenvalues": self.d_evals, "eigenvectors": self.d_evecs},
                     spectra=self.d_spectra)


class LambdaAdaptiveBeamformedSpectraPipeline(_Base):
    n_slots = 2

    def __init__(self, shape, weights, nr_signal_eigenvectors=None, min_freq_channel=0,
                 shrink_eigenvalues=False, detect_signal_eigenmodes=False,
                 detection_threshold_delta=3.0, nr_blocks_to_accumulate=1 << 30):
        import torch
        super().__init__(shape, weights, nr_blocks_to_accumulate)
        p = self.plan
        counts = np.zeros(p.C, dtype=np.int32)
        for c in range(p.C):
            counts[c] = int((nr_signal_eigenvectors or {}).get(min_freq_channel + c, 0))
        p.set_fixed_counts(counts)
        self.shrink = bool(shrink_eigenvalues)
        self.k_rule = SF_K_DETECT if detect_signal_eigenmodes else SF_K_FIXED
        self.delta = float(detection_threshold_delta)
        self.d_evals = torch.empty((p.C, 2, p.R), dtype=torch.float32, device="cuda")
        self.d_evecs = torch.empty((p.C, 2, p.R, p.R, 2), dtype=torch.float32, device="cuda")
        self.d_counts = torch.empty((p.C, 2), dtype=torch.int32, device="cuda")
        self.d_spectra = None
        if packet_spectra_supported(p.Tp):
            self.d_spectra = torch.empty(p.packet_spectra_shape(2 * p.B, FINE_CHANNELS_TO_REMOVE_EACH_SIDE),
                                         dtype=torch.float32, device="cuda")

    def execute_pipeline(self, packet_data, dummy_run=False):
        self._ingest(packet_data)
        self.plan.run_adaptive(self.d_samples, self.d_scales, self.k_rule, self.delta, self.shrink,
                               self.d_vis, self.d_evals, self.d_evecs, self.d_counts, self.d_beams,
                               stream=self.stream)
        if self.d_spectra is not None:
            self.plan.packet_spectra(self.d_beams, 2 * self.plan.B, FINE_CHANNELS_TO_REMOVE_EACH_SIDE,
                                     self.d_spectra, stream=self.stream)
        self._finish(packet_data, dummy_run, {"eigenvalues": self.d_evals, "eigenvectors": self.d_evecs,
                                              "nulled_eigenmode_counts": self.d_counts},
                     spectra=self.d_spectra)
