// Drives the C++ GPUPipeline adapters (include/sf_pipeline.hpp) the way the
// reference's ProcessorState does: execute_pipeline per filled buffer, with a
// state that takes buffers back and an Output with host landing buffers.
//
// The host-framework interfaces below restate, in this test's own code, the
// member functions the adapters use from the reference's declarations
// (include/spatial/pipeline_base.hpp:9-40, packet_formats.hpp:50-66,
// output.hpp:22-58, spatial.hpp:149-247).
//
// With -DSF_REFERENCE_PIPELINE_BASE the GPUPipeline base class comes from the
// reference's own include/spatial/pipeline_base.hpp (self-contained; add
// -I <reference>/include) instead of the restatement below.
//
// usage: adapter_harness <mode 0|1|2> <dir> [steer|refsteer]
//   steer:    pass an SfBeamSteering (zenith targets; receiver r at antenna 200 + r,
//             ENU (3 r, -2 r, 0.5 r + r % 3); receiver 4 a null input; 1.0 GHz + ch x 100 kHz
//             from channel 50) as the constructor's beam_steering
//   refsteer: pass a steering object with the reference BeamSteering<T>'s interface
//             (register_buffer + maybe_refresh) whose first refresh copies
//             dir/weights2.bin into every registered buffer's device weights
//   otherwise an inert SfBeamSteering (no targets)
//   reads  dir/samples.bin (int8, two integrations), dir/scales.bin (int16, two),
//          dir/weights.bin (fp16 pairs)
//   writes dir/beams_<run>.bin, dir/vis.bin (float, after one dump of both runs),
//          dir/evals_<run>.bin, dir/counts_<run>.bin, dir/fft_<run>.bin, dir/protocol.txt
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <atomic>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <functional>
#include <limits>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>

// ---- host-framework interfaces (as the reference declares them) ----
class ProcessorStateBase {
 public:
  virtual ~ProcessorStateBase() = default;
  virtual void release_buffer(const int buffer_index) = 0;
};

class Output {
 public:
  virtual ~Output() = default;
  virtual size_t register_beam_data_block(const size_t start_seq_num, const size_t end_seq_num) = 0;
  virtual size_t register_visibilities_block(const size_t start_seq_num, const size_t end_seq_num,
                                             const int num_missing_packets, const int num_total_packets) = 0;
  virtual size_t register_eigendecomposition_data_block(const size_t start_seq_num, const size_t end_seq_num) = 0;
  virtual size_t register_fft_block(const size_t start_seq_num, const size_t end_seq_num) = 0;
  virtual void *get_beam_data_landing_pointer(const size_t block_num) = 0;
  virtual void *get_visibilities_landing_pointer(const size_t block_num) = 0;
  virtual void *get_arrivals_data_landing_pointer(const size_t block_num) = 0;
  virtual void *get_eigenvalues_data_landing_pointer(const size_t block_num) = 0;
  virtual void *get_eigenvectors_data_landing_pointer(const size_t block_num) = 0;
  virtual void *get_nulled_eigenmode_counts_landing_pointer(const size_t block_num) = 0;
  virtual void *get_fft_landing_pointer(const size_t block_num) = 0;
  virtual void register_beam_data_transfer_complete(const size_t block_num) = 0;
  virtual void register_visibilities_transfer_complete(const size_t block_num) = 0;
  virtual void register_arrivals_transfer_complete(const size_t block_num) = 0;
  virtual void register_eigendecomposition_data_transfer_complete(const size_t block_num) = 0;
  virtual void register_fft_transfer_complete(const size_t block_num) = 0;
};

struct FinalPacketData {
  uint64_t start_seq_id = 0;
  uint64_t end_seq_id = 0;
  size_t buffer_index = 0;
  virtual ~FinalPacketData() = default;
  virtual void *get_samples_ptr() = 0;
  virtual size_t get_samples_elements_size() = 0;
  virtual void *get_scales_ptr() = 0;
  virtual size_t get_scales_element_size() = 0;
  virtual bool *get_arrivals_ptr() = 0;
  virtual size_t get_arrivals_size() = 0;
  virtual int get_num_missing_packets() = 0;
};

#ifdef SF_REFERENCE_PIPELINE_BASE
#include <spatial/pipeline_base.hpp>
#else
class GPUPipeline {
 public:
  virtual ~GPUPipeline() = default;
  void set_state(ProcessorStateBase *state) { state_ = state; }
  void set_output(std::shared_ptr<Output> output) { output_ = output; }
  virtual void set_subpacket_delays(int *delays_subpacket) { subpacket_delays_ = delays_subpacket; }
  virtual void set_antenna_gains(std::complex<float> *gains) { gains_ = gains; }
  virtual void set_fine_delays(const float *, double, double, int) {}
  virtual void set_stream_permutation(const std::vector<int> &, const std::vector<int> &) {
    throw std::runtime_error("set_stream_permutation not supported by this pipeline type");
  }
  virtual void execute_pipeline(FinalPacketData *packet_data, const bool dummy_run = false) = 0;
  virtual void dump_visibilities(const uint64_t end_seq_num = 0) = 0;

 protected:
  ProcessorStateBase *state_ = nullptr;
  std::shared_ptr<Output> output_;
  int *subpacket_delays_ = nullptr;
  std::complex<float> *gains_ = nullptr;
};
#endif

#include "sf_pipeline.hpp"

// ---- a small LAMBDA-shaped configuration ----
struct TestConfig {
  static constexpr int NR_CHANNELS = 6;
  static constexpr int NR_FPGA_SOURCES = 2;
  static constexpr int NR_TIME_STEPS_PER_PACKET = 16;
  static constexpr int NR_RECEIVERS_PER_PACKET = 5;
  static constexpr int NR_RECEIVERS = 10;
  static constexpr int NR_POLARIZATIONS = 2;
  static constexpr int NR_PACKETS_FOR_CORRELATION = 8;
  static constexpr int NR_BEAMS = 3;
  static constexpr int NR_CORRELATED_BLOCKS_TO_ACCUMULATE = 2;
  static constexpr int FFT_DOWNSAMPLE_FACTOR = 16;
};
using Cfg = TestConfig;
constexpr size_t kSamples = (size_t)Cfg::NR_CHANNELS * (Cfg::NR_PACKETS_FOR_CORRELATION + 2) *
                            Cfg::NR_FPGA_SOURCES * Cfg::NR_TIME_STEPS_PER_PACKET * Cfg::NR_RECEIVERS_PER_PACKET * 4;
constexpr size_t kScales = (size_t)Cfg::NR_CHANNELS * (Cfg::NR_PACKETS_FOR_CORRELATION + 2) * Cfg::NR_RECEIVERS * 2;
constexpr size_t kArrivals = (size_t)Cfg::NR_CHANNELS * (Cfg::NR_PACKETS_FOR_CORRELATION + 2) * Cfg::NR_FPGA_SOURCES;

struct Weights {
  std::complex<__half> weights[Cfg::NR_CHANNELS][Cfg::NR_POLARIZATIONS][Cfg::NR_BEAMS][Cfg::NR_RECEIVERS];
};

struct PinnedPacketData : FinalPacketData {
  int8_t *samples = nullptr;
  int16_t *scales = nullptr;
  bool *arrivals = nullptr;
  int missing = 0;
  PinnedPacketData() {
    cudaHostAlloc(reinterpret_cast<void **>(&samples), kSamples, cudaHostAllocDefault);
    cudaHostAlloc(reinterpret_cast<void **>(&scales), kScales * 2, cudaHostAllocDefault);
    cudaHostAlloc(reinterpret_cast<void **>(&arrivals), kArrivals, cudaHostAllocDefault);
    std::memset(arrivals, 1, kArrivals);
  }
  ~PinnedPacketData() override {
    cudaFreeHost(samples);
    cudaFreeHost(scales);
    cudaFreeHost(arrivals);
  }
  void *get_samples_ptr() override { return samples; }
  size_t get_samples_elements_size() override { return kSamples; }
  void *get_scales_ptr() override { return scales; }
  size_t get_scales_element_size() override { return kScales * 2; }
  bool *get_arrivals_ptr() override { return arrivals; }
  size_t get_arrivals_size() override { return kArrivals; }
  int get_num_missing_packets() override { return missing; }
};

// The reference BeamSteering<T>'s interface (common.hpp:245-303): buffers
// register their device weights and stream; a due refresh enqueues one
// asynchronous copy per buffer.  Here the first refresh is due at once and
// copies a second weight set.
struct ReferenceStyleSteering {
  using BeamWeights = Weights;
  std::shared_ptr<Weights> next;
  std::vector<std::pair<BeamWeights *, cudaStream_t>> buffers;
  bool done = false;
  void register_buffer(BeamWeights *device_weights, cudaStream_t stream) { buffers.push_back({device_weights, stream}); }
  bool maybe_refresh() {
    if (done || !next) return false;
    for (auto &b : buffers) cudaMemcpyAsync(b.first, next.get(), sizeof(BeamWeights), cudaMemcpyDefault, b.second);
    done = true;
    return true;
  }
};

class RecordingState : public ProcessorStateBase {
 public:
  std::mutex mu;
  std::vector<int> released;
  void release_buffer(const int buffer_index) override {
    std::lock_guard<std::mutex> lock(mu);
    released.push_back(buffer_index);
  }
};

class HostOutput : public Output {
 public:
  static constexpr size_t kBlocks = 4;
  std::vector<std::vector<char>> beams, vis, evals, evecs, counts, arrivals, fft;
  std::atomic<int> beam_done{0}, vis_done{0}, eig_done{0}, arrivals_done{0}, fft_done{0};
  size_t next_beam = 0, next_eig = 0, next_fft = 0;
  std::vector<std::string> order;  // block registrations in call order
  int vis_missing = -1, vis_total = -1;
  uint64_t vis_start = 0, vis_end = 0;
  HostOutput(size_t beam_bytes, size_t vis_bytes, size_t eval_bytes, size_t evec_bytes, size_t count_bytes,
             size_t fft_bytes)
      : beams(kBlocks, std::vector<char>(beam_bytes)),
        vis(1, std::vector<char>(vis_bytes)),
        evals(kBlocks, std::vector<char>(eval_bytes)),
        evecs(kBlocks, std::vector<char>(evec_bytes)),
        counts(kBlocks, std::vector<char>(count_bytes)),
        arrivals(kBlocks, std::vector<char>(kArrivals)),
        fft(kBlocks, std::vector<char>(fft_bytes)) {}
  size_t register_beam_data_block(const size_t, const size_t) override {
    order.push_back("beam");
    return next_beam++ % kBlocks;
  }
  size_t register_fft_block(const size_t, const size_t) override {
    order.push_back("fft");
    return next_fft++ % kBlocks;
  }
  size_t register_visibilities_block(const size_t s, const size_t e, const int missing, const int total) override {
    vis_start = s;
    vis_end = e;
    vis_missing = missing;
    vis_total = total;
    return 0;
  }
  size_t register_eigendecomposition_data_block(const size_t, const size_t) override {
    order.push_back("eig");
    return next_eig++ % kBlocks;
  }
  void *get_beam_data_landing_pointer(const size_t b) override { return beams[b].data(); }
  void *get_visibilities_landing_pointer(const size_t) override { return vis[0].data(); }
  void *get_arrivals_data_landing_pointer(const size_t b) override { return arrivals[b].data(); }
  void *get_eigenvalues_data_landing_pointer(const size_t b) override { return evals[b].data(); }
  void *get_eigenvectors_data_landing_pointer(const size_t b) override { return evecs[b].data(); }
  void *get_nulled_eigenmode_counts_landing_pointer(const size_t b) override { return counts[b].data(); }
  void *get_fft_landing_pointer(const size_t b) override { return fft[b].data(); }
  void register_beam_data_transfer_complete(const size_t) override { ++beam_done; }
  void register_visibilities_transfer_complete(const size_t) override { ++vis_done; }
  void register_arrivals_transfer_complete(const size_t) override { ++arrivals_done; }
  void register_eigendecomposition_data_transfer_complete(const size_t) override { ++eig_done; }
  void register_fft_transfer_complete(const size_t) override { ++fft_done; }
};

static std::vector<char> read_file(const std::string &path, size_t bytes) {
  std::vector<char> v(bytes);
  std::ifstream f(path, std::ios::binary);
  if (!f.read(v.data(), bytes)) throw std::runtime_error("cannot read " + path);
  return v;
}

static void write_file(const std::string &path, const void *p, size_t bytes) {
  std::ofstream f(path, std::ios::binary);
  f.write(static_cast<const char *>(p), bytes);
}

int main(int argc, char **argv) {
  if (argc < 3) {
    std::fprintf(stderr, "usage: %s <mode 0|1|2> <dir>\n", argv[0]);
    return 2;
  }
  const int mode = std::atoi(argv[1]);
  const std::string dir = argv[2];
  try {
    const auto samples = read_file(dir + "/samples.bin", 2 * kSamples);
    const auto scales = read_file(dir + "/scales.bin", 2 * kScales * 2);
    auto wbytes = read_file(dir + "/weights.bin", sizeof(Weights));
    auto weights = std::make_unique<Weights>();
    std::memcpy(weights.get(), wbytes.data(), sizeof(Weights));

    constexpr int C = Cfg::NR_CHANNELS, R = Cfg::NR_RECEIVERS, B = Cfg::NR_BEAMS;
    constexpr int T = Cfg::NR_PACKETS_FOR_CORRELATION * Cfg::NR_TIME_STEPS_PER_PACKET;
    const int slots = mode == 2 ? 2 : 1;
    const size_t beam_bytes = (size_t)C * 2 * slots * B * T * 4;
    const size_t vis_bytes = (size_t)C * (R * (R + 1) / 2) * 8 * 4;
    const size_t eval_bytes = mode == 1 ? (size_t)C * 4 * R * 4 : (size_t)C * 2 * R * 4;
    const size_t evec_bytes = mode == 1 ? (size_t)C * 4 * R * R * 8 : 8;
    const size_t count_bytes = (size_t)C * 2 * 4;
    const size_t fft_bytes = mode == 2 ? (size_t)C * 2 * 2 * B * (Cfg::NR_TIME_STEPS_PER_PACKET - 10) * 4
                                       : (size_t)C * 2 * B * (T / Cfg::FFT_DOWNSAMPLE_FACTOR) * 4;
    auto output =
        std::make_shared<HostOutput>(beam_bytes, vis_bytes, eval_bytes, evec_bytes, count_bytes, fft_bytes);
    RecordingState state;

    GPUPipeline *pipeline = nullptr;
    std::function<void()> destroy;      // deletes through the concrete type
    std::function<uint32_t()> status;   // device_status() of the concrete type
    int delays[Cfg::NR_FPGA_SOURCES] = {3, -5};
    const bool steer = argc > 3 && std::string(argv[3]) == "steer";
    const bool refsteer = argc > 3 && std::string(argv[3]) == "refsteer";
    sfgb::SfBeamSteering<Cfg> steering;
    if (steer) {
      std::unordered_map<int, sfgb::ENUPosition> positions;
      std::unordered_map<int, int> mapping;
      for (int r = 0; r < R; ++r) {
        positions[200 + r] = sfgb::ENUPosition{3.0 * r, -2.0 * r, 0.5 * r + r % 3};
        mapping[r] = r == 4 ? -100 : 200 + r;
      }
      steering = sfgb::SfBeamSteering<Cfg>({sfgb::BeamTarget{}}, positions, mapping,
                                           sfgb::FrequencyPlan{1.0e9, 1.0e5}, 50,
                                           sfgb::ArrayLocation{52.9, 6.87, 30.0}, 1.0e6);
    }
    ReferenceStyleSteering ref_steering;
    if (refsteer) {
      auto w2 = read_file(dir + "/weights2.bin", sizeof(Weights));
      ref_steering.next = std::make_shared<Weights>();
      std::memcpy(ref_steering.next.get(), w2.data(), sizeof(Weights));
    }
    // constructed exactly as the reference's pipelines are (argument order and defaults)
    auto adopt = [&](auto *p) {
      pipeline = p;
      destroy = [p]() { delete p; };
      status = [p]() { return p->device_status(); };
    };
    std::unordered_map<int, int> k_map;
    for (int c = 0; c < C; ++c) k_map[100 + c] = c % 3;  // absolute channel -> K
    if (mode == 0) {
      if (refsteer) adopt(new sfgb::SfLambdaCorrBeamOnlyGPUPipeline<Cfg>(2, weights.get(), ref_steering));
      else adopt(new sfgb::SfLambdaCorrBeamOnlyGPUPipeline<Cfg>(2, weights.get(), steering));
    } else if (mode == 1) {
      if (refsteer) adopt(new sfgb::SfLambdaGPUPipeline<Cfg>(2, weights.get(), ref_steering));
      else adopt(new sfgb::SfLambdaGPUPipeline<Cfg>(2, weights.get(), steering));
    } else {
      if (refsteer)
        adopt(new sfgb::SfLambdaAdaptivePipeline<Cfg>(2, weights.get(), k_map, 100, ref_steering, false, false, 3.0f,
                                                      10.0));
      else
        adopt(new sfgb::SfLambdaAdaptivePipeline<Cfg>(2, weights.get(), k_map, 100, steering));
    }
    pipeline->set_state(&state);
    pipeline->set_output(output);
    if (mode != 0) pipeline->set_subpacket_delays(delays);

    PinnedPacketData packets[2];
    for (int run = 0; run < 2; ++run) {
      std::memcpy(packets[run].samples, samples.data() + run * kSamples, kSamples);
      std::memcpy(packets[run].scales, scales.data() + run * kScales * 2, kScales * 2);
      packets[run].buffer_index = 10 + run;
      packets[run].start_seq_id = 1000 * (run + 1);
      packets[run].end_seq_id = 1000 * (run + 1) + 999;
      packets[run].missing = run;
      pipeline->execute_pipeline(&packets[run]);  // the second run dumps the visibilities
    }
    // the adaptive pipeline dumps only when asked (its reference counterpart's dump is a no-op)
    if (mode == 2) pipeline->dump_visibilities(packets[1].end_seq_id);
    cudaDeviceSynchronize();
    const uint32_t bits = status();
    destroy();  // the destructor waits for every stream

    for (int run = 0; run < 2; ++run) {
      write_file(dir + "/beams_" + std::to_string(run) + ".bin", output->beams[run].data(), beam_bytes);
      write_file(dir + "/evals_" + std::to_string(run) + ".bin", output->evals[run].data(), eval_bytes);
      write_file(dir + "/counts_" + std::to_string(run) + ".bin", output->counts[run].data(), count_bytes);
      write_file(dir + "/fft_" + std::to_string(run) + ".bin", output->fft[run].data(), fft_bytes);
    }
    write_file(dir + "/vis.bin", output->vis[0].data(), vis_bytes);
    std::ofstream proto(dir + "/protocol.txt");
    proto << "released";
    for (int r : state.released) proto << " " << r;
    proto << "\nbeam_done " << output->beam_done << "\nvis_done " << output->vis_done << "\neig_done "
          << output->eig_done << "\narrivals_done " << output->arrivals_done << "\nvis_missing "
          << output->vis_missing << "\nvis_total " << output->vis_total << "\nvis_start " << output->vis_start
          << "\nvis_end " << output->vis_end << "\nfft_done " << output->fft_done << "\nstatus " << bits << "\n";
    proto << "order";
    for (const auto &o : output->order) proto << " " << o;
    proto << "\n";
  } catch (const std::exception &e) {
    std::fprintf(stderr, "error: %s\n", e.what());
    return 1;
  }
  return 0;
}
