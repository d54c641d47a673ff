/*
 * sf_pipeline.hpp - GPUPipeline-shaped C++ adapters over the C ABI (sf_capi.h).
 *
 * Drop-in replacements for the three GPU stages of the reference's LAMBDA
 * pipelines, for a host framework that drives them through the
 * GPUPipeline interface (reference include/spatial/pipeline_base.hpp:9-40):
 *
 *   sfgb::SfLambdaCorrBeamOnlyGPUPipeline<Config>  for LambdaCorrBeamOnlyGPUPipeline<Config>
 *       (reference include/spatial/pipeline/lambda_corr_beam_only_gpu_pipeline.hpp:202-403)
 *   sfgb::SfLambdaGPUPipeline<Config>              for LambdaGPUPipeline<Config>
 *       (reference include/spatial/pipeline/lambda_gpu_pipeline.hpp:445-797, 1153-1194)
 *   sfgb::SfLambdaAdaptivePipeline<Config>         for the projection and beam stage of
 *       LambdaAdaptiveBeamformedSpectraPipeline<Config>
 *       (reference lambda_adaptive_beamformed_spectra_pipeline.hpp:563-798, 1014-1036)
 *
 * Include it after the host framework's declarations of GPUPipeline,
 * FinalPacketData, Output and ProcessorStateBase (in the reference:
 * pipeline_base.hpp, packet_formats.hpp, output.hpp, spatial.hpp).  The
 * adapters use only their public / protected interface:
 *   GPUPipeline        state_, output_, the virtual set_* (including
 *                      set_stream_permutation) / execute_pipeline / dump_visibilities
 *   FinalPacketData    start_seq_id, end_seq_id, buffer_index, get_samples_ptr,
 *                      get_samples_elements_size, get_scales_ptr,
 *                      get_scales_element_size, get_arrivals_ptr,
 *                      get_arrivals_size, get_num_missing_packets
 *   ProcessorStateBase release_buffer(int)
 *   Output             register_*_block, get_*_landing_pointer,
 *                      register_*_transfer_complete
 * Config supplies the compile-time sizes the reference's LambdaConfig has:
 * NR_CHANNELS, NR_FPGA_SOURCES, NR_TIME_STEPS_PER_PACKET, NR_RECEIVERS,
 * NR_RECEIVERS_PER_PACKET, NR_POLARIZATIONS (2), NR_PACKETS_FOR_CORRELATION,
 * NR_BEAMS, NR_CORRELATED_BLOCKS_TO_ACCUMULATE (and optionally
 * FFT_DOWNSAMPLE_FACTOR); LambdaConfig itself serves.
 *
 * Behaviour as the reference: execute_pipeline copies the buffer's samples and
 * scales to the device, releases the ring buffer back to the state once the
 * copies have landed, runs the chain on the buffer's stream, integrates the
 * visibilities, lands beams (and eigen outputs) in the Output's landing
 * pointers with transfer-complete callbacks, and dumps the visibilities every
 * nr_blocks_to_accumulate runs.  Errors throw std::runtime_error carrying
 * sf_last_error() (the reference exits through CUDA_CHECK).
 *
 * Spectra tails: SfLambdaGPUPipeline lands |FFT|^2 of each beam over the whole
 * integration downsampled by Config::FFT_DOWNSAMPLE_FACTOR (128 when Config has
 * none; float [C][Pol][B][T/D], lambda_gpu_pipeline.hpp:522-531, 585-595), and
 * SfLambdaAdaptivePipeline lands the per-packet |FFT| summed over packets with
 * 5 bins trimmed each side (float [C][Pol][2B][Tp-10],
 * lambda_adaptive_beamformed_spectra_pipeline.hpp:808-848, 899-911), through
 * Output::register_fft_block / get_fft_landing_pointer /
 * register_fft_transfer_complete.  Shapes the spectra kernels do not cover
 * (T not a power of two in [64, 16384]; Tp not 16, 32 or 64) skip the tail and
 * register no FFT block.
 *
 * Constructors take the reference's arguments in the reference's order, so a
 * host framework swaps only the class name:
 *   SfLambdaCorrBeamOnlyGPUPipeline(num_buffers, h_weights, beam_steering,
 *                                   nr_blocks_to_accumulate = Config::NR_CORRELATED_BLOCKS_TO_ACCUMULATE)
 *       (lambda_corr_beam_only_gpu_pipeline.hpp:385-388)
 *   SfLambdaGPUPipeline(num_buffers, h_weights, beam_steering,
 *                       nr_blocks_to_accumulate = Config::NR_CORRELATED_BLOCKS_TO_ACCUMULATE)
 *       (lambda_gpu_pipeline.hpp:784-786)
 *   SfLambdaAdaptivePipeline(num_buffers, h_weights, nr_signal_eigenvectors, min_freq_channel,
 *                            beam_steering, shrink_eigenvalues = false,
 *                            detect_signal_eigenmodes = false, detection_threshold_delta = 3.0f,
 *                            eigenmode_stats_interval_seconds = 10.0)
 *       (lambda_adaptive_beamformed_spectra_pipeline.hpp:1014-1019)
 *
 * Beam steering: beam_steering is either the reference's BeamSteering<T>
 * (anything with register_buffer(BeamWeights *device_weights, cudaStream_t)
 * and maybe_refresh(), common.hpp:245-303) -- every buffer's plan weights are
 * registered with it and its asynchronous copies land in them -- or this
 * library's SfBeamSteering<Config> (sf_pointing.hpp), which synthesises the
 * weights on the device.  Either is inert without targets.  execute_pipeline
 * calls maybe_refresh() first, before any work of the run is enqueued, as the
 * reference's pipelines do (lambda_gpu_pipeline.hpp:454-456, 973); neither
 * form synchronises with the GPU.  set_beam_steering() attaches one later.
 */
#ifndef SF_PIPELINE_HPP
#define SF_PIPELINE_HPP

#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <complex>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <functional>
#include <iostream>
#include <limits>
#include <mutex>
#include <memory>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <unordered_map>
#include <vector>

#include "sf_capi.h"
#include "sf_pointing.hpp"

namespace sfgb {

namespace detail {

inline void check(int status, const char *what) {
  if (status != SF_OK) throw std::runtime_error(std::string(what) + ": " + sf_last_error());
}

inline void check_cuda(cudaError_t e, const char *what) {
  if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

template <typename T> struct DeviceArray {
  T *ptr = nullptr;
  size_t count = 0;
  void allocate(size_t n) {
    count = n;
    check_cuda(cudaMalloc(reinterpret_cast<void **>(&ptr), n * sizeof(T)), "cudaMalloc");
  }
  size_t bytes() const { return count * sizeof(T); }
  ~DeviceArray() {
    if (ptr) cudaFree(ptr);
  }
};

// Host callbacks: the same hand-off the reference performs from its streams.
template <typename State> struct ReleaseContext {
  State *state;
  int buffer_index;
};
template <typename State> void release_buffer_cb(void *data) {
  auto *ctx = static_cast<ReleaseContext<State> *>(data);
  ctx->state->release_buffer(ctx->buffer_index);
  delete ctx;
}

template <typename Out> struct TransferContext {
  std::shared_ptr<Out> output;
  size_t block;
  int kind;  // 0 beams, 1 visibilities, 2 eigendecomposition, 3 spectra
};
template <typename Out> void transfer_complete_cb(void *data) {
  auto *ctx = static_cast<TransferContext<Out> *>(data);
  if (ctx->kind == 0) ctx->output->register_beam_data_transfer_complete(ctx->block);
  else if (ctx->kind == 1) ctx->output->register_visibilities_transfer_complete(ctx->block);
  else if (ctx->kind == 2) ctx->output->register_eigendecomposition_data_transfer_complete(ctx->block);
  else ctx->output->register_fft_transfer_complete(ctx->block);
  delete ctx;
}

// Config::FFT_DOWNSAMPLE_FACTOR, or LambdaConfig's default of 128.
template <typename Cfg, typename = void> struct FftDownsample {
  static constexpr int value = 128;
};
template <typename Cfg>
struct FftDownsample<Cfg, std::void_t<decltype(Cfg::FFT_DOWNSAMPLE_FACTOR)>> {
  static constexpr int value = static_cast<int>(Cfg::FFT_DOWNSAMPLE_FACTOR);
};

constexpr bool pow2_in(int n, int lo, int hi) { return n >= lo && n <= hi && (n & (n - 1)) == 0; }

// Steering objects: this library's SfBeamSteering (register_plan) or the
// reference's BeamSteering<T> (register_buffer on the device weights).
template <typename S, typename = void> struct HasRegisterPlan : std::false_type {};
template <typename S>
struct HasRegisterPlan<S, std::void_t<decltype(std::declval<S &>().register_plan(
                              static_cast<sf_plan *>(nullptr), static_cast<cudaStream_t>(nullptr)))>>
    : std::true_type {};
template <typename S, typename = void> struct HasRegisterBuffer : std::false_type {};
template <typename S>
struct HasRegisterBuffer<S, std::void_t<typename S::BeamWeights,
                                        decltype(std::declval<S &>().register_buffer(
                                            static_cast<typename S::BeamWeights *>(nullptr),
                                            static_cast<cudaStream_t>(nullptr)))>> : std::true_type {};

}  // namespace detail

// Shared machinery of the three adapters.  Base is the host framework's
// GPUPipeline; Mode selects the chain run per buffer.
template <typename Config, typename Base, int Mode> class SfPipelineBase : public Base {
 public:
  static constexpr int kCorrBeam = 0, kLambdaGpu = 1, kAdaptive = 2;
  static constexpr int C = Config::NR_CHANNELS;
  static constexpr int F = Config::NR_FPGA_SOURCES;
  static constexpr int TP = Config::NR_TIME_STEPS_PER_PACKET;
  static constexpr int R = Config::NR_RECEIVERS;
  static constexpr int RPP = Config::NR_RECEIVERS_PER_PACKET;
  static constexpr int P = Config::NR_PACKETS_FOR_CORRELATION;
  static constexpr int B = Config::NR_BEAMS;
  static constexpr int POL = Config::NR_POLARIZATIONS;
  static constexpr int T = P * TP;
  static constexpr int NBL = R * (R + 1) / 2;
  static constexpr int SLOTS = Mode == kAdaptive ? 2 : 1;  // adaptive: original + projected beams
  // Spectra tails (see the file comment): bins per (channel, pol, beam) row.
  static constexpr int FFT_TRIM = 5;  // NR_FINE_CHANNELS_TO_REMOVE_EACH_SIDE
  static constexpr int FFT_DOWNSAMPLE = detail::FftDownsample<Config>::value;
  static constexpr bool SPECTRA =
      (Mode == kLambdaGpu && detail::pow2_in(T, 64, 16384) && FFT_DOWNSAMPLE >= 1 && FFT_DOWNSAMPLE <= T) ||
      (Mode == kAdaptive && detail::pow2_in(TP, 16, 64));
  static constexpr int FFT_BINS = Mode == kAdaptive ? TP - 2 * FFT_TRIM : T / (FFT_DOWNSAMPLE > 0 ? FFT_DOWNSAMPLE : 1);
  static_assert(POL == 2, "the GB300 path handles two polarisations");
  static_assert(F * RPP == R, "NR_RECEIVERS must equal NR_FPGA_SOURCES x NR_RECEIVERS_PER_PACKET");

  // weights: the BeamWeightsT<Config> payload, std::complex<__half>[C][Pol][B][R]
  template <typename Weights>
  SfPipelineBase(int num_buffers, Weights *h_weights, int nr_blocks_to_accumulate)
      : nr_blocks_(nr_blocks_to_accumulate > 0 ? nr_blocks_to_accumulate : 1) {
    static_assert(sizeof(Weights) == sizeof(uint16_t) * 2 * C * POL * B * R,
                  "weights must be [C][Pol][B][R] complex fp16");
    if (num_buffers < 1) throw std::invalid_argument("num_buffers must be at least 1");
    const sf_shape shape = {C, F, TP, R, POL, RPP, P, B};
    buffers_.resize(num_buffers);
    for (auto &b : buffers_) {
      b.reset(new Buffer);
      detail::check(sf_plan_create(&shape, &b->plan), "sf_plan_create");
      detail::check_cuda(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking), "cudaStreamCreate");
      detail::check_cuda(cudaStreamCreateWithFlags(&b->host_stream, cudaStreamNonBlocking), "cudaStreamCreate");
      detail::check_cuda(cudaEventCreateWithFlags(&b->copied, cudaEventDisableTiming), "cudaEventCreate");
      detail::check_cuda(cudaEventCreateWithFlags(&b->accumulated, cudaEventDisableTiming), "cudaEventCreate");
      b->samples.allocate((size_t)C * (P + 2) * F * TP * RPP * POL * 2);
      b->scales.allocate((size_t)C * (P + 2) * R * POL);
      b->vis.allocate((size_t)C * NBL * POL * POL * 2);
      b->beams.allocate((size_t)C * POL * SLOTS * B * T * 2);
      if (Mode == kLambdaGpu) {
        b->evals.allocate((size_t)C * POL * POL * R);
        b->evecs.allocate((size_t)C * POL * POL * R * R * 2);
      } else if (Mode == kAdaptive) {
        b->evals.allocate((size_t)C * POL * R);
        b->counts.allocate((size_t)C * POL);
      }
      if (SPECTRA) b->spectra.allocate((size_t)C * POL * SLOTS * B * FFT_BINS);
      detail::check(sf_set_weights(b->plan, reinterpret_cast<const uint16_t *>(h_weights), b->stream),
                    "sf_set_weights");
    }
    accum_.allocate((size_t)C * NBL * POL * POL * 2);
    vis_f32_.allocate((size_t)C * NBL * POL * POL * 2);
    detail::check_cuda(cudaMemset(accum_.ptr, 0, accum_.bytes()), "cudaMemset");
    detail::check_cuda(cudaEventCreateWithFlags(&last_accumulate_, cudaEventDisableTiming), "cudaEventCreate");
    detail::check_cuda(cudaEventRecord(last_accumulate_, buffers_[0]->stream), "cudaEventRecord");
  }

  ~SfPipelineBase() {
    for (auto &b : buffers_) {
      if (b->stream) cudaStreamSynchronize(b->stream);
      if (b->host_stream) cudaStreamSynchronize(b->host_stream);
      if (b->copied) cudaEventDestroy(b->copied);
      if (b->accumulated) cudaEventDestroy(b->accumulated);
      if (b->stream) cudaStreamDestroy(b->stream);
      if (b->host_stream) cudaStreamDestroy(b->host_stream);
      if (b->plan) sf_plan_destroy(b->plan);
    }
    if (last_accumulate_) cudaEventDestroy(last_accumulate_);
  }

  SfPipelineBase(const SfPipelineBase &) = delete;
  SfPipelineBase &operator=(const SfPipelineBase &) = delete;

  // GPUPipeline::set_subpacket_delays: int [F] in [-Tp, Tp]
  void set_subpacket_delays(int *delays_subpacket) override {
    this->subpacket_delays_ = delays_subpacket;
    std::vector<int32_t> d(delays_subpacket, delays_subpacket + F);
    for (auto &b : buffers_)
      detail::check(sf_set_subpacket_delays(b->plan, d.data(), b->stream), "sf_set_subpacket_delays");
  }

  // GPUPipeline::set_antenna_gains: complex<float> [C][Pol][R]
  void set_antenna_gains(std::complex<float> *gains) override {
    this->gains_ = gains;
    for (auto &b : buffers_)
      detail::check(sf_set_antenna_gains(b->plan, reinterpret_cast<const float *>(gains), b->stream),
                    "sf_set_antenna_gains");
  }

  // GPUPipeline::set_fine_delays: per-receiver delays in ns
  void set_fine_delays(const float *delays_ns, double base_freq_hz, double channel_bw_hz,
                       int min_freq_ch) override {
    for (auto &b : buffers_)
      detail::check(sf_set_fine_delays(b->plan, delays_ns, base_freq_hz, channel_bw_hz, min_freq_ch, b->stream),
                    "sf_set_fine_delays");
  }

  // LambdaGPUPipeline::set_stream_permutation: both vectors F * Rpp * Pol long
  void set_stream_permutation(const std::vector<int> &recv_perm, const std::vector<int> &pol_perm) override {
    if ((int)recv_perm.size() != 2 * R || (int)pol_perm.size() != 2 * R)
      throw std::runtime_error(
          "set_stream_permutation: size must equal NR_FPGA_SOURCES * NR_RECEIVERS_PER_PACKET * NR_POLARIZATIONS");
    std::vector<int32_t> rp(recv_perm.begin(), recv_perm.end()), pp(pol_perm.begin(), pol_perm.end());
    for (auto &b : buffers_)
      detail::check(sf_set_stream_permutation(b->plan, rp.data(), pp.data(), b->stream), "sf_set_stream_permutation");
  }

  // Keep the beams pointed at the steering's targets (inert without targets):
  // an SfBeamSteering<Config> or the reference's BeamSteering<T>.
  template <typename Steering> void set_beam_steering(Steering steering) {
    static_assert(detail::HasRegisterPlan<Steering>::value || detail::HasRegisterBuffer<Steering>::value,
                  "beam_steering needs register_plan(sf_plan*, cudaStream_t) or "
                  "register_buffer(BeamWeights*, cudaStream_t)");
    auto held = std::make_shared<Steering>(std::move(steering));
    for (auto &b : buffers_) {
      if constexpr (detail::HasRegisterPlan<Steering>::value) {
        held->register_plan(b->plan, b->stream);
      } else {
        void *dw = nullptr;
        detail::check(sf_plan_weights_buffer(b->plan, &dw), "sf_plan_weights_buffer");
        held->register_buffer(static_cast<typename Steering::BeamWeights *>(dw), b->stream);
      }
    }
    refresh_steering_ = [held]() { held->maybe_refresh(); };
  }

  void execute_pipeline(FinalPacketData *packet_data, const bool dummy_run = false) override {
    if (!dummy_run && this->state_ == nullptr)
      throw std::logic_error("State has not been set on GPUPipeline object!");
    if (refresh_steering_) refresh_steering_();
    Buffer &b = *buffers_[current_];
    if (packet_data->get_samples_elements_size() != b.samples.bytes() ||
        packet_data->get_scales_element_size() != b.scales.bytes())
      throw std::invalid_argument("packet buffer sizes do not match Config");
    const size_t start_seq = packet_data->start_seq_id, end_seq = packet_data->end_seq_id;
    if (vis_start_seq_ == std::numeric_limits<size_t>::max()) vis_start_seq_ = start_seq;
    vis_missing_ += packet_data->get_num_missing_packets();

    // ingest; the ring buffer goes back to the state once the copies landed
    detail::check_cuda(cudaMemcpyAsync(b.samples.ptr, packet_data->get_samples_ptr(), b.samples.bytes(),
                                       cudaMemcpyDefault, b.stream),
                       "cudaMemcpyAsync");
    detail::check_cuda(cudaMemcpyAsync(b.scales.ptr, packet_data->get_scales_ptr(), b.scales.bytes(),
                                       cudaMemcpyDefault, b.stream),
                       "cudaMemcpyAsync");
    detail::check_cuda(cudaEventRecord(b.copied, b.stream), "cudaEventRecord");
    if (!dummy_run) {
      detail::check_cuda(cudaStreamWaitEvent(b.host_stream, b.copied, 0), "cudaStreamWaitEvent");
      auto *ctx = new detail::ReleaseContext<ProcessorStateBase>{this->state_,
                                                                 static_cast<int>(packet_data->buffer_index)};
      detail::check_cuda(cudaLaunchHostFunc(b.host_stream, detail::release_buffer_cb<ProcessorStateBase>, ctx),
                         "cudaLaunchHostFunc");
    }

    run_chain(b);
    if (SPECTRA) run_spectra(b);

    // integrate: accumulations of successive buffers are chained in order
    detail::check_cuda(cudaStreamWaitEvent(b.stream, last_accumulate_, 0), "cudaStreamWaitEvent");
    detail::check(sf_accumulate_visibilities(b.plan, b.vis.ptr, accum_.ptr, b.stream), "sf_accumulate_visibilities");
    detail::check_cuda(cudaEventRecord(last_accumulate_, b.stream), "cudaEventRecord");
    detail::check_cuda(cudaEventRecord(b.accumulated, b.stream), "cudaEventRecord");

    if (this->output_ != nullptr && !dummy_run) {
      land_outputs(b, packet_data, start_seq, end_seq);
      if (++integrated_ >= nr_blocks_) dump_visibilities(end_seq);
    }
    if (!dummy_run) current_ = (current_ + 1) % static_cast<int>(buffers_.size());
  }

  void dump_visibilities(const uint64_t end_seq_num = 0) override {
    Buffer &b0 = *buffers_[0];
    detail::check_cuda(cudaStreamWaitEvent(b0.stream, last_accumulate_, 0), "cudaStreamWaitEvent");
    detail::check(sf_visibilities_to_float(b0.plan, accum_.ptr, vis_f32_.ptr, b0.stream), "sf_visibilities_to_float");
    if (this->output_ != nullptr) {
      const size_t block = this->output_->register_visibilities_block(
          vis_start_seq_ == std::numeric_limits<size_t>::max() ? 0 : vis_start_seq_, end_seq_num, vis_missing_,
          integrated_ * C * P * F);  // packets 0..P-1 of every channel and FPGA, as get_num_missing_packets counts
      if (block != std::numeric_limits<size_t>::max()) {
        detail::check_cuda(cudaMemcpyAsync(this->output_->get_visibilities_landing_pointer(block), vis_f32_.ptr,
                                           vis_f32_.bytes(), cudaMemcpyDefault, b0.stream),
                           "cudaMemcpyAsync");
        launch_transfer_done(b0.stream, block, 1);
      }
    }
    detail::check_cuda(cudaMemsetAsync(accum_.ptr, 0, accum_.bytes(), b0.stream), "cudaMemsetAsync");
    detail::check_cuda(cudaEventRecord(last_accumulate_, b0.stream), "cudaEventRecord");
    vis_start_seq_ = std::numeric_limits<size_t>::max();
    vis_missing_ = 0;
    integrated_ = 0;
  }

  // Wait for every queued run and transfer, ignoring errors (destructors).
  void synchronize_quietly() {
    for (auto &b : buffers_) {
      if (b->stream) cudaStreamSynchronize(b->stream);
      if (b->host_stream) cudaStreamSynchronize(b->host_stream);
    }
  }

  // Wait for every queued run and transfer (the reference's destructor syncs).
  void synchronize() {
    for (auto &b : buffers_) {
      detail::check_cuda(cudaStreamSynchronize(b->stream), "cudaStreamSynchronize");
      detail::check_cuda(cudaStreamSynchronize(b->host_stream), "cudaStreamSynchronize");
    }
  }

  // Device error bits reported by the kernels of every buffer (0 = none).
  uint32_t device_status() {
    uint32_t all = 0;
    for (auto &b : buffers_) {
      uint32_t bits = 0;
      sf_plan_status(b->plan, b->stream, &bits);
      all |= bits;
    }
    return all;
  }

 protected:
  struct Buffer {
    sf_plan *plan = nullptr;
    cudaStream_t stream = nullptr, host_stream = nullptr;
    cudaEvent_t copied = nullptr, accumulated = nullptr;
    detail::DeviceArray<int8_t> samples;
    detail::DeviceArray<int16_t> scales;
    detail::DeviceArray<int32_t> vis;
    detail::DeviceArray<uint16_t> beams;
    detail::DeviceArray<float> evals, evecs;
    detail::DeviceArray<int32_t> counts;
    detail::DeviceArray<float> spectra;
  };

  virtual void run_chain(Buffer &b) = 0;

  void run_spectra(Buffer &b) {
    if (Mode == kAdaptive)
      detail::check(sf_packet_spectra(b.plan, b.beams.ptr, SLOTS * B, FFT_TRIM, b.spectra.ptr, b.stream),
                    "sf_packet_spectra");
    else
      detail::check(sf_beam_spectra(b.plan, b.beams.ptr, SLOTS * B, FFT_DOWNSAMPLE, b.spectra.ptr, b.stream),
                    "sf_beam_spectra");
  }

  void land_spectra(Buffer &b, size_t start_seq, size_t end_seq) {
    if (!SPECTRA) return;
    Output &out = *this->output_;
    const size_t block = out.register_fft_block(start_seq, end_seq);
    if (block == std::numeric_limits<size_t>::max()) return;
    detail::check_cuda(cudaMemcpyAsync(out.get_fft_landing_pointer(block), b.spectra.ptr, b.spectra.bytes(),
                                       cudaMemcpyDefault, b.stream),
                       "cudaMemcpyAsync");
    launch_transfer_done(b.stream, block, 3);
  }

  void launch_transfer_done(cudaStream_t s, size_t block, int kind) {
    auto *ctx = new detail::TransferContext<Output>{this->output_, block, kind};
    detail::check_cuda(cudaLaunchHostFunc(s, detail::transfer_complete_cb<Output>, ctx), "cudaLaunchHostFunc");
  }

  void land_outputs(Buffer &b, FinalPacketData *packet_data, size_t start_seq, size_t end_seq) {
    Output &out = *this->output_;
    const size_t block = out.register_beam_data_block(start_seq, end_seq);
    if (block != std::numeric_limits<size_t>::max()) {
      detail::check_cuda(cudaMemcpyAsync(out.get_beam_data_landing_pointer(block), b.beams.ptr, b.beams.bytes(),
                                         cudaMemcpyDefault, b.stream),
                         "cudaMemcpyAsync");
      launch_transfer_done(b.stream, block, 0);
      std::memcpy(out.get_arrivals_data_landing_pointer(block), packet_data->get_arrivals_ptr(),
                  packet_data->get_arrivals_size());
      out.register_arrivals_transfer_complete(block);
    }
    if (Mode == kCorrBeam) return;
    if (Mode == kAdaptive) land_spectra(b, start_seq, end_seq);  // beams, spectra, eigen (reference order)
    land_eigen(b, start_seq, end_seq);
    if (Mode == kLambdaGpu) land_spectra(b, start_seq, end_seq);  // beams, eigen, spectra
  }

  void land_eigen(Buffer &b, size_t start_seq, size_t end_seq) {
    Output &out = *this->output_;
    const size_t eblock = out.register_eigendecomposition_data_block(start_seq, end_seq);
    if (eblock == std::numeric_limits<size_t>::max()) return;
    detail::check_cuda(cudaMemcpyAsync(out.get_eigenvalues_data_landing_pointer(eblock), b.evals.ptr,
                                       b.evals.bytes(), cudaMemcpyDefault, b.stream),
                       "cudaMemcpyAsync");
    if (Mode == kLambdaGpu)
      detail::check_cuda(cudaMemcpyAsync(out.get_eigenvectors_data_landing_pointer(eblock), b.evecs.ptr,
                                         b.evecs.bytes(), cudaMemcpyDefault, b.stream),
                         "cudaMemcpyAsync");
    else
      detail::check_cuda(cudaMemcpyAsync(out.get_nulled_eigenmode_counts_landing_pointer(eblock), b.counts.ptr,
                                         b.counts.bytes(), cudaMemcpyDefault, b.stream),
                         "cudaMemcpyAsync");
    launch_transfer_done(b.stream, eblock, 2);
  }

  std::vector<std::unique_ptr<Buffer>> buffers_;
  std::function<void()> refresh_steering_;
  detail::DeviceArray<int64_t> accum_;
  detail::DeviceArray<float> vis_f32_;
  cudaEvent_t last_accumulate_ = nullptr;
  int current_ = 0;
  int nr_blocks_;
  int integrated_ = 0;
  int vis_missing_ = 0;
  size_t vis_start_seq_ = std::numeric_limits<size_t>::max();
};

// LambdaCorrBeamOnlyGPUPipeline: packet-window correlation + beams with W diag(d).
template <typename Config, typename Base = GPUPipeline>
class SfLambdaCorrBeamOnlyGPUPipeline : public SfPipelineBase<Config, Base, 0> {
  using Super = SfPipelineBase<Config, Base, 0>;

 public:
  template <typename Weights, typename Steering>
  SfLambdaCorrBeamOnlyGPUPipeline(const int num_buffers, Weights *h_weights, Steering beam_steering,
                                  int nr_blocks_to_accumulate = Config::NR_CORRELATED_BLOCKS_TO_ACCUMULATE)
      : Super(num_buffers, h_weights, nr_blocks_to_accumulate) {
    this->set_beam_steering(std::move(beam_steering));
  }

 protected:
  void run_chain(typename Super::Buffer &b) override {
    detail::check(sf_run_corr_beam(b.plan, b.samples.ptr, b.scales.ptr, b.vis.ptr, b.beams.ptr, b.stream),
                  "sf_run_corr_beam");
  }
};

// LambdaGPUPipeline: aligned window, all-blocks eigendecomposition, beams.
template <typename Config, typename Base = GPUPipeline>
class SfLambdaGPUPipeline : public SfPipelineBase<Config, Base, 1> {
  using Super = SfPipelineBase<Config, Base, 1>;

 public:
  template <typename Weights, typename Steering>
  SfLambdaGPUPipeline(const int num_buffers, Weights *h_weights, Steering beam_steering,
                      int nr_blocks_to_accumulate = Config::NR_CORRELATED_BLOCKS_TO_ACCUMULATE)
      : Super(num_buffers, h_weights, nr_blocks_to_accumulate) {
    this->set_beam_steering(std::move(beam_steering));
  }

 protected:
  void run_chain(typename Super::Buffer &b) override {
    detail::check(sf_run_lambda_gpu(b.plan, b.samples.ptr, b.scales.ptr, b.vis.ptr, b.evals.ptr, b.evecs.ptr,
                                    b.beams.ptr, b.stream),
                  "sf_run_lambda_gpu");
  }
};

// Projection and beam stage of LambdaAdaptiveBeamformedSpectraPipeline:
// whitened eigendecomposition, K (fixed map, detection or shrink), W P, and
// 2B beams (original, projected).  nr_signal_eigenvectors maps absolute
// frequency channel -> K (the reference's -e map); channels absent get 0.
// Like the reference, visibilities are dumped only on an explicit
// dump_visibilities() (the reference's is a no-op; this one lands the
// integrated visibilities), and every run's nulled-mode counts are kept for
// print_eigenmode_stats() (reference ..._pipeline.hpp:930-1000).
template <typename Config, typename Base = GPUPipeline>
class SfLambdaAdaptivePipeline : public SfPipelineBase<Config, Base, 2> {
  using Super = SfPipelineBase<Config, Base, 2>;

 public:
  template <typename Weights, typename Steering>
  SfLambdaAdaptivePipeline(const int num_buffers, Weights *h_weights,
                           const std::unordered_map<int, int> nr_signal_eigenvectors, const int min_freq_channel,
                           Steering beam_steering, bool shrink_eigenvalues = false,
                           bool detect_signal_eigenmodes = false, float detection_threshold_delta = 3.0f,
                           double eigenmode_stats_interval_seconds = 10.0)
      : Super(num_buffers, h_weights, std::numeric_limits<int>::max()),
        shrink_(shrink_eigenvalues),
        k_rule_(detect_signal_eigenmodes ? SF_K_DETECT : SF_K_FIXED),
        delta_(detection_threshold_delta),
        eigenmode_stats_interval_seconds_(eigenmode_stats_interval_seconds),
        stats_(std::make_shared<Stats>()) {
    std::vector<int32_t> counts(Config::NR_CHANNELS, 0);
    for (int c = 0; c < Config::NR_CHANNELS; ++c) {
      const auto it = nr_signal_eigenvectors.find(min_freq_channel + c);
      if (it != nr_signal_eigenvectors.end()) counts[c] = it->second;
    }
    for (auto &b : this->buffers_)
      detail::check(sf_set_fixed_counts(b->plan, counts.data(), b->stream), "sf_set_fixed_counts");
    staging_.resize(this->buffers_.size(), nullptr);
    for (auto &h : staging_)
      detail::check_cuda(cudaMallocHost(reinterpret_cast<void **>(&h), sizeof(int32_t) * Config::NR_CHANNELS * 2),
                         "cudaMallocHost");
    this->set_beam_steering(std::move(beam_steering));
  }

  ~SfLambdaAdaptivePipeline() {
    this->synchronize_quietly();
    for (auto h : staging_)
      if (h) cudaFreeHost(h);
  }

  // The interval the host framework prints eigenmode statistics at (stored as
  // the reference stores it; print_eigenmode_stats() does the printing).
  double eigenmode_stats_interval_seconds() const { return eigenmode_stats_interval_seconds_; }

  // Per (channel, pol): min / max / median / mean of the nulled-mode count over
  // the runs since the last call, then the history is cleared.
  void print_eigenmode_stats() {
    std::vector<int32_t> samples;
    {
      std::lock_guard<std::mutex> lock(stats_->mu);
      samples.swap(stats_->history);
    }
    const size_t per = static_cast<size_t>(Config::NR_CHANNELS) * 2;
    if (samples.empty() || samples.size() % per != 0) return;
    const size_t n = samples.size() / per;
    std::cout << "Eigenmode nulling stats over last " << n << " samples" << std::endl;
    for (int c = 0; c < Config::NR_CHANNELS; ++c)
      for (int pol = 0; pol < 2; ++pol) {
        std::vector<int32_t> series(n);
        double sum = 0.0;
        for (size_t i = 0; i < n; ++i) {
          series[i] = samples[i * per + c * 2 + pol];
          sum += series[i];
        }
        std::sort(series.begin(), series.end());
        const double median = n % 2 == 0 ? 0.5 * (series[n / 2 - 1] + series[n / 2]) : series[n / 2];
        std::cout << "  ch=" << c << " pol=" << pol << " min=" << series.front() << " max=" << series.back()
                  << " median=" << median << " mean=" << sum / static_cast<double>(n) << std::endl;
      }
    std::fflush(stdout);
  }

 protected:
  struct Stats {
    std::mutex mu;
    std::vector<int32_t> history;
  };
  struct StatsContext {
    std::shared_ptr<Stats> stats;
    const int32_t *counts;
  };
  static void record_counts_cb(void *data) {
    auto *ctx = static_cast<StatsContext *>(data);
    {
      std::lock_guard<std::mutex> lock(ctx->stats->mu);
      ctx->stats->history.insert(ctx->stats->history.end(), ctx->counts, ctx->counts + Config::NR_CHANNELS * 2);
    }
    delete ctx;
  }

  void run_chain(typename Super::Buffer &b) override {
    detail::check(sf_run_adaptive(b.plan, b.samples.ptr, b.scales.ptr, k_rule_, delta_, shrink_ ? 1 : 0, b.vis.ptr,
                                  b.evals.ptr, nullptr, b.counts.ptr, b.beams.ptr, b.stream),
                  "sf_run_adaptive");
    // the run's counts into the statistics history, off the GPU's path
    size_t i = 0;
    while (this->buffers_[i].get() != &b) ++i;
    detail::check_cuda(cudaMemcpyAsync(staging_[i], b.counts.ptr, sizeof(int32_t) * Config::NR_CHANNELS * 2,
                                       cudaMemcpyDeviceToHost, b.stream),
                       "cudaMemcpyAsync");
    auto *ctx = new StatsContext{stats_, staging_[i]};
    detail::check_cuda(cudaLaunchHostFunc(b.stream, record_counts_cb, ctx), "cudaLaunchHostFunc");
  }

 private:
  bool shrink_;
  int32_t k_rule_;
  float delta_;
  double eigenmode_stats_interval_seconds_;
  std::shared_ptr<Stats> stats_;
  std::vector<int32_t *> staging_;
};

}  // namespace sfgb

#endif  // SF_PIPELINE_HPP
