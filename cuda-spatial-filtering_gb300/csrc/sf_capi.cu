// C ABI entry points (include/sf_capi.h): plan lifetime, configuration,
// stage kernels and whole chains.  Plain pointers, runtime shapes, status
// codes; every call is asynchronous on the caller's stream.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

#include "sf_common.cuh"
#include "sf_plan.cuh"

namespace {

thread_local char g_err[512] = "";

int set_err(int code, const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
  return code;
}

int cuda_err(cudaError_t e, const char *what) {
  return set_err(SF_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define SF_TRY(call, what)                       \
  do {                                           \
    cudaError_t e_ = (call);                     \
    if (e_ != cudaSuccess) return cuda_err(e_, what); \
  } while (0)

cudaStream_t as_stream(void *s) { return reinterpret_cast<cudaStream_t>(s); }

int check_plan(const sf_plan *p) {
  if (!p) return set_err(SF_ERR_INVALID_ARGUMENT, "plan is NULL");
  return SF_OK;
}

void free_plan(sf_plan *p) {
  if (!p) return;
  cudaFree(p->d_off_aligned);
  cudaFree(p->d_off_packet);
  cudaFree(p->d_factors);
  cudaFree(p->d_perm);
  cudaFree(p->d_weights);
  cudaFree(p->d_weff);
  cudaFree(p->d_spec_tw);
  cudaFree(p->d_packet_dft);
  cudaFree(p->d_steer);
  cudaFree(p->d_steer_conn);
  cudaFree(p->d_steer_cal);
  if (p->steer_uploaded) {
    cudaEventSynchronize(p->steer_uploaded);
    cudaEventDestroy(p->steer_uploaded);
  }
  cudaFreeHost(p->h_steer);
  cudaFreeHost(p->h_steer_conn);
  cudaFreeHost(p->h_steer_cal);
  cudaFree(p->d_fixed_counts);
  cudaFree(p->d_vis);
  cudaFree(p->d_evals);
  cudaFree(p->d_counts);
  cudaFree(p->d_status);
  free(p->h_delays);
  free(p->h_gains);
  free(p->h_phasors);
  free(p->h_factors);
  free(p->h_perm);
  free(p->h_fixed_counts);
  delete p;
}

int upload_factors(sf_plan *p, cudaStream_t s) {
  for (int c = 0; c < p->C; ++c)
    for (int pol = 0; pol < 2; ++pol)
      for (int r = 0; r < p->R; ++r) {
        // the gain belongs to the source stream (applied at ingest), the
        // phasor to the output receiver (applied after the reorder)
        float2 g = p->h_gains[((size_t)c * 2 + pol) * p->R + r];
        if (p->h_perm) {
          const int32_t src = p->h_perm[2 * r + pol];
          g = src < 0 ? make_float2(0.f, 0.f) : p->h_gains[((size_t)c * 2 + (src & 1)) * p->R + (src >> 1)];
        }
        const float2 ph = p->h_phasors[(size_t)c * p->R + r];
        p->h_factors[((size_t)c * 2 + pol) * p->R + r] =
            make_float2(g.x * ph.x - g.y * ph.y, g.x * ph.y + g.y * ph.x);
      }
  SF_TRY(cudaMemcpyAsync(p->d_factors, p->h_factors, sizeof(float2) * p->C * 2 * p->R,
                         cudaMemcpyHostToDevice, s),
         "upload receiver factors");
  return SF_OK;
}

int upload_offsets(sf_plan *p, cudaStream_t s) {
  int32_t *tmp = static_cast<int32_t *>(malloc(sizeof(int32_t) * p->F));
  if (!tmp) return set_err(SF_ERR_INVALID_ARGUMENT, "out of host memory");
  for (int f = 0; f < p->F; ++f) tmp[f] = p->Tp + p->h_delays[f];
  cudaError_t e = cudaMemcpyAsync(p->d_off_aligned, tmp, sizeof(int32_t) * p->F,
                                  cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);  // tmp is released below
  free(tmp);
  if (e != cudaSuccess) return cuda_err(e, "upload window offsets");
  return SF_OK;
}

}  // namespace

namespace {
struct SmemOptin {
  int device;
  const void *func;
  size_t bytes;
};
std::mutex g_optin_mu;
std::vector<SmemOptin> g_optin;
constexpr int MAX_DEVICES = 64;
int g_max_smem[MAX_DEVICES];
}  // namespace

cudaError_t sf_smem_optin(const void *func, size_t bytes) {
  if (bytes <= 48 * 1024) return cudaSuccess;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lock(g_optin_mu);
  for (SmemOptin &o : g_optin)
    if (o.device == dev && o.func == func) {
      if (o.bytes >= bytes) return cudaSuccess;
      e = cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(bytes));
      if (e == cudaSuccess) o.bytes = bytes;
      return e;
    }
  e = cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(bytes));
  if (e == cudaSuccess) g_optin.push_back({dev, func, bytes});
  return e;
}

int sf_device_max_smem() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEVICES) return 0;
  std::lock_guard<std::mutex> lock(g_optin_mu);
  if (!g_max_smem[dev]) cudaDeviceGetAttribute(&g_max_smem[dev], cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  return g_max_smem[dev];
}

// Lets other translation units of the library report through sf_last_error.
int sf_internal_set_error(int code, const char *msg) { return set_err(code, "%s", msg); }

extern "C" {

const char *sf_last_error(void) { return g_err; }

int sf_plan_create(const sf_shape *shape, sf_plan **out_plan) {
  if (!shape || !out_plan) return set_err(SF_ERR_INVALID_ARGUMENT, "shape/out_plan is NULL");
  *out_plan = nullptr;
  const sf_shape &s = *shape;
  if (s.n_polarizations != 2) return set_err(SF_ERR_UNSUPPORTED, "n_polarizations must be 2");
  if (s.n_channels < 1 || s.n_fpgas < 1 || s.n_time_per_packet < 1 || s.n_receivers < 1 ||
      s.n_receivers_per_packet < 1 || s.n_packets < 1 || s.n_beams < 1)
    return set_err(SF_ERR_INVALID_ARGUMENT, "every shape field must be >= 1");
  if (s.n_receivers != s.n_fpgas * s.n_receivers_per_packet)
    return set_err(SF_ERR_INVALID_ARGUMENT, "n_receivers (%d) != n_fpgas * n_receivers_per_packet (%d)",
                   s.n_receivers, s.n_fpgas * s.n_receivers_per_packet);
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return set_err(SF_ERR_NO_DEVICE, "no CUDA device: %s", cudaGetErrorString(e));
  int major = 0, minor = 0, sms = 0;
  cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
  cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (major != 10 || minor != 3)
    return set_err(SF_ERR_NO_DEVICE, "device %d is sm_%d%d; this library is built for sm_103a", dev,
                   major, minor);

  sf_plan *p = new (std::nothrow) sf_plan();
  if (!p) return set_err(SF_ERR_INVALID_ARGUMENT, "out of host memory");
  memset(p, 0, sizeof(*p));
  p->shape = s;
  p->C = s.n_channels;
  p->F = s.n_fpgas;
  p->Tp = s.n_time_per_packet;
  p->R = s.n_receivers;
  p->Rpp = s.n_receivers_per_packet;
  p->P = s.n_packets;
  p->B = s.n_beams;
  p->T = s.n_packets * s.n_time_per_packet;
  p->NBL = p->R * (p->R + 1) / 2;
  p->device = dev;
  p->num_sms = sms;

  const size_t C = p->C, R = p->R, B = p->B;
  p->h_delays = static_cast<int32_t *>(calloc(p->F, sizeof(int32_t)));
  p->h_gains = static_cast<float2 *>(malloc(sizeof(float2) * C * 2 * R));
  p->h_phasors = static_cast<float2 *>(malloc(sizeof(float2) * C * R));
  p->h_factors = static_cast<float2 *>(malloc(sizeof(float2) * C * 2 * R));
  p->h_fixed_counts = static_cast<int32_t *>(calloc(C, sizeof(int32_t)));
  if (!p->h_delays || !p->h_gains || !p->h_phasors || !p->h_factors || !p->h_fixed_counts) {
    free_plan(p);
    return set_err(SF_ERR_INVALID_ARGUMENT, "out of host memory");
  }
  for (size_t i = 0; i < C * 2 * R; ++i) p->h_gains[i] = make_float2(1.f, 0.f);
  for (size_t i = 0; i < C * R; ++i) p->h_phasors[i] = make_float2(1.f, 0.f);

#define SF_ALLOC(ptr, bytes)                                   \
  do {                                                         \
    cudaError_t ea = cudaMalloc((void **)&(ptr), (bytes));     \
    if (ea != cudaSuccess) {                                   \
      free_plan(p);                                            \
      return cuda_err(ea, "cudaMalloc " #ptr);                 \
    }                                                          \
  } while (0)
  SF_ALLOC(p->d_off_aligned, sizeof(int32_t) * p->F);
  SF_ALLOC(p->d_off_packet, sizeof(int32_t) * p->F);
  SF_ALLOC(p->d_factors, sizeof(float2) * C * 2 * R);
  SF_ALLOC(p->d_weights, sizeof(__half2) * C * 2 * B * R);
  SF_ALLOC(p->d_weff, sizeof(float2) * C * 2 * 2 * B * R);
  SF_ALLOC(p->d_fixed_counts, sizeof(int32_t) * C);
  SF_ALLOC(p->d_vis, sizeof(int32_t) * C * p->NBL * 8);
  SF_ALLOC(p->d_evals, sizeof(float) * C * 4 * R);
  SF_ALLOC(p->d_counts, sizeof(int32_t) * C * 2);
  SF_ALLOC(p->d_status, sizeof(uint32_t));
  if (sf_beam_spectra_supported(p->T)) SF_ALLOC(p->d_spec_tw, sizeof(float2) * p->T);
  if (p->Tp == 64) SF_ALLOC(p->d_packet_dft, sf_packet_dft_bytes());
  SF_ALLOC(p->d_steer, sizeof(double) * 3 * (B + R));
  SF_ALLOC(p->d_steer_conn, sizeof(int32_t) * R);
  SF_ALLOC(p->d_steer_cal, sizeof(float2) * C * 2 * R);
#undef SF_ALLOC
  {
    cudaError_t eh = cudaMallocHost(reinterpret_cast<void **>(&p->h_steer), sizeof(double) * 3 * (B + R));
    if (eh == cudaSuccess) eh = cudaMallocHost(reinterpret_cast<void **>(&p->h_steer_conn), sizeof(int32_t) * R);
    if (eh == cudaSuccess) eh = cudaMallocHost(reinterpret_cast<void **>(&p->h_steer_cal), sizeof(float2) * C * 2 * R);
    if (eh == cudaSuccess) eh = cudaEventCreateWithFlags(&p->steer_uploaded, cudaEventDisableTiming);
    if (eh != cudaSuccess) {
      free_plan(p);
      return cuda_err(eh, "pinned steering staging");
    }
  }
  cudaError_t ez = cudaSuccess;
  ez = ez != cudaSuccess ? ez : cudaMemset(p->d_off_packet, 0, sizeof(int32_t) * p->F);
  ez = ez != cudaSuccess ? ez : cudaMemset(p->d_weights, 0, sizeof(__half2) * C * 2 * B * R);
  ez = ez != cudaSuccess ? ez : cudaMemset(p->d_weff, 0, sizeof(float2) * C * 4 * B * R);
  ez = ez != cudaSuccess ? ez : cudaMemset(p->d_fixed_counts, 0, sizeof(int32_t) * C);
  ez = ez != cudaSuccess ? ez : cudaMemset(p->d_status, 0, sizeof(uint32_t));
  if (p->d_spec_tw) ez = ez != cudaSuccess ? ez : sf_fill_spectra_twiddles(p->d_spec_tw, p->T);
  if (p->d_packet_dft) ez = ez != cudaSuccess ? ez : sf_fill_packet_dft(p->d_packet_dft);
  if (ez != cudaSuccess) {
    free_plan(p);
    return cuda_err(ez, "initialise plan memory");
  }
  int rc = upload_offsets(p, 0);
  if (rc == SF_OK) rc = upload_factors(p, 0);
  if (rc == SF_OK && cudaDeviceSynchronize() != cudaSuccess) rc = cuda_err(cudaGetLastError(), "plan init");
  if (rc != SF_OK) {
    free_plan(p);
    return rc;
  }
  *out_plan = p;
  return SF_OK;
}

int sf_plan_destroy(sf_plan *plan) {
  if (!plan) return SF_OK;
  free_plan(plan);
  return SF_OK;
}

int sf_plan_get_shape(const sf_plan *plan, sf_shape *out_shape) {
  if (int rc = check_plan(plan)) return rc;
  if (!out_shape) return set_err(SF_ERR_INVALID_ARGUMENT, "out_shape is NULL");
  *out_shape = plan->shape;
  return SF_OK;
}

int sf_plan_status(sf_plan *plan, void *stream, uint32_t *out_bits) {
  if (int rc = check_plan(plan)) return rc;
  uint32_t bits = 0;
  cudaStream_t s = as_stream(stream);
  SF_TRY(cudaMemcpyAsync(&bits, plan->d_status, sizeof(bits), cudaMemcpyDeviceToHost, s), "read status");
  SF_TRY(cudaMemsetAsync(plan->d_status, 0, sizeof(uint32_t), s), "clear status");
  SF_TRY(cudaStreamSynchronize(s), "status sync");
  if (out_bits) *out_bits = bits;
  if (bits) return set_err(SF_ERR_DEVICE, "device error bits 0x%x", bits);
  return SF_OK;
}

int sf_set_subpacket_delays(sf_plan *plan, const int32_t *h_delays, void *stream) {
  if (int rc = check_plan(plan)) return rc;
  for (int f = 0; f < plan->F; ++f) {
    const int d = h_delays ? h_delays[f] : 0;
    if (d < -plan->Tp || d > plan->Tp)
      return set_err(SF_ERR_INVALID_ARGUMENT, "delay %d of FPGA %d outside [-%d, %d]", d, f, plan->Tp,
                     plan->Tp);
  }
  for (int f = 0; f < plan->F; ++f) plan->h_delays[f] = h_delays ? h_delays[f] : 0;
  return upload_offsets(plan, as_stream(stream));
}

int sf_set_antenna_gains(sf_plan *plan, const float *h_gains, void *stream) {
  if (int rc = check_plan(plan)) return rc;
  const size_t n = (size_t)plan->C * 2 * plan->R;
  for (size_t i = 0; i < n; ++i)
    plan->h_gains[i] = h_gains ? make_float2(h_gains[2 * i], h_gains[2 * i + 1]) : make_float2(1.f, 0.f);
  cudaStream_t s = as_stream(stream);
  if (int rc = upload_factors(plan, s)) return rc;
  SF_TRY(cudaStreamSynchronize(s), "gains upload");
  return SF_OK;
}

int sf_set_fine_delays(sf_plan *plan, const float *h_delays_ns, double base_freq_hz,
                       double channel_bw_hz, int32_t min_freq_ch, void *stream) {
  if (int rc = check_plan(plan)) return rc;
  for (int c = 0; c < plan->C; ++c) {
    const double fc = base_freq_hz + static_cast<double>(min_freq_ch + c) * channel_bw_hz;
    for (int r = 0; r < plan->R; ++r) {
      const double tau = h_delays_ns ? static_cast<double>(h_delays_ns[r]) * 1e-9 : 0.0;
      const double phi = -2.0 * M_PI * fc * tau;
      plan->h_phasors[(size_t)c * plan->R + r] =
          make_float2(static_cast<float>(cos(phi)), static_cast<float>(sin(phi)));
    }
  }
  cudaStream_t s = as_stream(stream);
  if (int rc = upload_factors(plan, s)) return rc;
  SF_TRY(cudaStreamSynchronize(s), "fine delay upload");
  return SF_OK;
}

int sf_set_stream_permutation(sf_plan *plan, const int32_t *h_recv_perm, const int32_t *h_pol_perm,
                              void *stream) {
  if (int rc = check_plan(plan)) return rc;
  const int R = plan->R;
  cudaStream_t s = as_stream(stream);
  if (!h_recv_perm && !h_pol_perm) {  // back to the identity
    if (plan->d_perm) {
      SF_TRY(cudaStreamSynchronize(s), "permutation reset");
      cudaFree(plan->d_perm);
      plan->d_perm = nullptr;
    }
    free(plan->h_perm);
    plan->h_perm = nullptr;
    if (int rc = upload_factors(plan, s)) return rc;
    SF_TRY(cudaStreamSynchronize(s), "permutation reset");
    return SF_OK;
  }
  if (!h_recv_perm || !h_pol_perm)
    return set_err(SF_ERR_INVALID_ARGUMENT, "both permutation arrays are needed (or neither)");
  for (int k = 0; k < 2 * R; ++k) {
    if (h_recv_perm[k] < -1 || h_recv_perm[k] >= R)
      return set_err(SF_ERR_INVALID_ARGUMENT, "recv_perm[%d] = %d outside [-1, %d)", k, h_recv_perm[k], R);
    if (h_recv_perm[k] >= 0 && (h_pol_perm[k] < 0 || h_pol_perm[k] > 1))
      return set_err(SF_ERR_INVALID_ARGUMENT, "pol_perm[%d] = %d is not 0 or 1", k, h_pol_perm[k]);
  }
  if (!plan->h_perm) {
    plan->h_perm = static_cast<int32_t *>(malloc(sizeof(int32_t) * 2 * R));
    if (!plan->h_perm) return set_err(SF_ERR_INVALID_ARGUMENT, "out of host memory");
  }
  for (int k = 0; k < 2 * R; ++k)
    plan->h_perm[k] = h_recv_perm[k] < 0 ? -1 : ((h_recv_perm[k] << 1) | h_pol_perm[k]);
  if (!plan->d_perm) SF_TRY(cudaMalloc(&plan->d_perm, sizeof(int32_t) * 2 * R), "cudaMalloc permutation");
  SF_TRY(cudaMemcpyAsync(plan->d_perm, plan->h_perm, sizeof(int32_t) * 2 * R, cudaMemcpyHostToDevice, s),
         "upload permutation");
  if (int rc = upload_factors(plan, s)) return rc;
  SF_TRY(cudaStreamSynchronize(s), "permutation upload");
  return SF_OK;
}

int sf_set_weights(sf_plan *plan, const uint16_t *h_weights_f16, void *stream) {
  if (int rc = check_plan(plan)) return rc;
  if (!h_weights_f16) return set_err(SF_ERR_INVALID_ARGUMENT, "weights are NULL");
  const size_t bytes = sizeof(__half2) * plan->C * 2 * plan->B * plan->R;
  cudaStream_t s = as_stream(stream);
  SF_TRY(cudaMemcpyAsync(plan->d_weights, h_weights_f16, bytes, cudaMemcpyHostToDevice, s),
         "weights upload");
  SF_TRY(cudaStreamSynchronize(s), "weights upload");
  return SF_OK;
}

int sf_set_steering_weights(sf_plan *plan, const double *h_dircos, const double *h_enu, const int32_t *h_connected,
                            double base_freq_hz, double channel_bw_hz, int32_t min_freq_ch, const float *h_cal_gains,
                            void *stream) {
  if (int rc = check_plan(plan)) return rc;
  if (!h_dircos || !h_enu) return set_err(SF_ERR_INVALID_ARGUMENT, "direction cosines / antenna positions are NULL");
  const int B = plan->B, R = plan->R;
  for (int i = 0; i < 3 * B; ++i)
    if (!std::isfinite(h_dircos[i])) return set_err(SF_ERR_INVALID_ARGUMENT, "direction cosine %d is not finite", i);
  for (int i = 0; i < 3 * R; ++i)
    if (!std::isfinite(h_enu[i])) return set_err(SF_ERR_INVALID_ARGUMENT, "antenna coordinate %d is not finite", i);
  if (!std::isfinite(base_freq_hz) || !std::isfinite(channel_bw_hz))
    return set_err(SF_ERR_INVALID_ARGUMENT, "frequency plan is not finite");
  // Stage in the plan's pinned buffers (the caller's arrays are free on
  // return) once the previous refresh's copies out of them have landed --
  // that waits for those copies only, never for the runs queued on `stream`.
  SF_TRY(cudaEventSynchronize(plan->steer_uploaded), "previous steering upload");
  memcpy(plan->h_steer, h_dircos, sizeof(double) * 3 * B);
  memcpy(plan->h_steer + 3 * B, h_enu, sizeof(double) * 3 * R);
  for (int r = 0; r < R; ++r) plan->h_steer_conn[r] = h_connected ? (h_connected[r] != 0) : 1;
  if (h_cal_gains) memcpy(plan->h_steer_cal, h_cal_gains, sizeof(float2) * plan->C * 2 * R);
  cudaStream_t s = as_stream(stream);
  SF_TRY(cudaMemcpyAsync(plan->d_steer, plan->h_steer, sizeof(double) * 3 * (B + R), cudaMemcpyHostToDevice, s),
         "steering upload");
  SF_TRY(cudaMemcpyAsync(plan->d_steer_conn, plan->h_steer_conn, sizeof(int32_t) * R, cudaMemcpyHostToDevice, s),
         "steering upload");
  if (h_cal_gains)
    SF_TRY(cudaMemcpyAsync(plan->d_steer_cal, plan->h_steer_cal, sizeof(float2) * plan->C * 2 * R,
                           cudaMemcpyHostToDevice, s),
           "calibration upload");
  SF_TRY(cudaEventRecord(plan->steer_uploaded, s), "steering upload event");
  // the synthesis writes the weights in stream order: runs queued before it
  // finish on the old weights, runs queued after it read the new ones
  SF_TRY(sf_launch_steering(plan, plan->d_steer, plan->d_steer + 3 * B, plan->d_steer_conn,
                            h_cal_gains ? plan->d_steer_cal : nullptr, base_freq_hz, channel_bw_hz, min_freq_ch, s),
         "steering launch");
  return SF_OK;
}

int sf_plan_weights_buffer(sf_plan *plan, void **out_device_weights) {
  if (int rc = check_plan(plan)) return rc;
  if (!out_device_weights) return set_err(SF_ERR_INVALID_ARGUMENT, "out pointer is NULL");
  *out_device_weights = plan->d_weights;
  return SF_OK;
}

int sf_set_fixed_counts(sf_plan *plan, const int32_t *h_counts, void *stream) {
  if (int rc = check_plan(plan)) return rc;
  for (int c = 0; c < plan->C; ++c) {
    const int k = h_counts ? h_counts[c] : 0;
    if (k < 0 || k > plan->R)
      return set_err(SF_ERR_INVALID_ARGUMENT, "count %d of channel %d outside [0, %d]", k, c, plan->R);
    plan->h_fixed_counts[c] = k;
  }
  cudaStream_t s = as_stream(stream);
  SF_TRY(cudaMemcpyAsync(plan->d_fixed_counts, plan->h_fixed_counts, sizeof(int32_t) * plan->C,
                         cudaMemcpyHostToDevice, s),
         "counts upload");
  SF_TRY(cudaStreamSynchronize(s), "counts upload");
  return SF_OK;
}

int sf_correlate(sf_plan *plan, const int8_t *d_samples, const int16_t *d_scales, int32_t window,
                 int32_t *d_vis, void *stream) {
  if (int rc = check_plan(plan)) return rc;
  if (!d_samples || !d_scales || !d_vis) return set_err(SF_ERR_INVALID_ARGUMENT, "NULL buffer");
  if (window != SF_WINDOW_PACKET && window != SF_WINDOW_ALIGNED)
    return set_err(SF_ERR_INVALID_ARGUMENT, "unknown window %d", window);
  if (reinterpret_cast<uintptr_t>(d_samples) % 16 != 0)
    return set_err(SF_ERR_INVALID_ARGUMENT, "samples must be 16-byte aligned");
  char why[160];
  if (!sf_correlate_supported(plan, why, sizeof(why))) return set_err(SF_ERR_UNSUPPORTED, "%s", why);
  const int32_t *off = window == SF_WINDOW_PACKET ? plan->d_off_packet : plan->d_off_aligned;
  cudaError_t e = sf_launch_correlate(plan, d_samples, d_scales, off, d_vis, as_stream(stream));
  if (e == cudaErrorInvalidConfiguration)
    return set_err(SF_ERR_UNSUPPORTED, "packet ring does not fit shared memory for this shape");
  SF_TRY(e, "correlate launch");
  return SF_OK;
}

int sf_covariance_eig(sf_plan *plan, const int32_t *d_vis, int32_t eig_mode, int32_t k_rule,
                      float delta, int32_t shrink, float *d_evals, float *d_evecs,
                      int32_t *d_counts, uint16_t *d_proj_f16, void *stream) {
  if (int rc = check_plan(plan)) return rc;
  if (!d_vis) return set_err(SF_ERR_INVALID_ARGUMENT, "vis is NULL");
  if (eig_mode != SF_EIG_ALL_BLOCKS && eig_mode != SF_EIG_SAME_POL_WHITENED)
    return set_err(SF_ERR_INVALID_ARGUMENT, "unknown eig mode %d", eig_mode);
  if (k_rule < SF_K_FIXED || k_rule > SF_K_NOISE_FLOOR)
    return set_err(SF_ERR_INVALID_ARGUMENT, "unknown K rule %d", k_rule);
  char why[160];
  if (!sf_eig_supported(plan, why, sizeof(why))) return set_err(SF_ERR_UNSUPPORTED, "%s", why);
  SF_TRY(sf_launch_eig(plan, d_vis, eig_mode, k_rule, delta, shrink ? 1 : 0, d_evals,
                       reinterpret_cast<float2 *>(d_evecs), d_counts,
                       reinterpret_cast<__half2 *>(d_proj_f16), as_stream(stream)),
         "eig launch");
  return SF_OK;
}

int sf_get_effective_weights(sf_plan *plan, float *d_weff, void *stream) {
  if (int rc = check_plan(plan)) return rc;
  if (!d_weff) return set_err(SF_ERR_INVALID_ARGUMENT, "weff is NULL");
  SF_TRY(cudaMemcpyAsync(d_weff, plan->d_weff, sizeof(float2) * plan->C * 2 * 2 * plan->B * plan->R,
                         cudaMemcpyDeviceToDevice, as_stream(stream)),
         "effective weights copy");
  return SF_OK;
}

int sf_beamform(sf_plan *plan, const int8_t *d_samples, const int16_t *d_scales, int32_t window,
                int32_t n_slots, uint16_t *d_beams_f16, void *stream) {
  if (int rc = check_plan(plan)) return rc;
  if (!d_samples || !d_scales || !d_beams_f16) return set_err(SF_ERR_INVALID_ARGUMENT, "NULL buffer");
  if (n_slots != 1 && n_slots != 2) return set_err(SF_ERR_INVALID_ARGUMENT, "n_slots must be 1 or 2");
  if (window != SF_WINDOW_PACKET && window != SF_WINDOW_ALIGNED)
    return set_err(SF_ERR_INVALID_ARGUMENT, "unknown window %d", window);
  if (n_slots * plan->B > 32) return set_err(SF_ERR_UNSUPPORTED, "at most 32 output beams");
  if (plan->d_perm && !sf_beam_tc_supported(plan, n_slots * plan->B))
    return set_err(SF_ERR_UNSUPPORTED, "stream permutation with more than 16 output beams per pol");
  cudaStream_t s = as_stream(stream);
  if (n_slots == 1) SF_TRY(sf_launch_weights_plain(plan, s), "weights launch");
  const int32_t *off = window == SF_WINDOW_PACKET ? plan->d_off_packet : plan->d_off_aligned;
  SF_TRY(sf_launch_beam(plan, d_samples, d_scales, off, n_slots,
                        reinterpret_cast<__half2 *>(d_beams_f16), s),
         "beam launch");
  return SF_OK;
}

int sf_beam_spectra(sf_plan *plan, const uint16_t *d_beams_f16, int32_t n_beams_out,
                    int32_t downsample, float *d_spectra, void *stream) {
  if (int rc = check_plan(plan)) return rc;
  if (!d_beams_f16 || !d_spectra) return set_err(SF_ERR_INVALID_ARGUMENT, "NULL buffer");
  if (n_beams_out < 1) return set_err(SF_ERR_INVALID_ARGUMENT, "n_beams_out must be >= 1");
  if (downsample < 1 || downsample > plan->T)
    return set_err(SF_ERR_INVALID_ARGUMENT, "downsample %d outside [1, T = %d]", downsample, plan->T);
  if (!plan->d_spec_tw)
    return set_err(SF_ERR_UNSUPPORTED,
                   "whole-integration spectra need T = P * Tp a power of two in [64, 16384] (T = %d)",
                   plan->T);
  SF_TRY(sf_launch_beam_spectra(plan, reinterpret_cast<const __half2 *>(d_beams_f16), n_beams_out,
                                downsample, d_spectra, as_stream(stream)),
         "beam spectra launch");
  return SF_OK;
}

int sf_packet_spectra(sf_plan *plan, const uint16_t *d_beams_f16, int32_t n_beams_out, int32_t trim,
                      float *d_spectra, void *stream) {
  if (int rc = check_plan(plan)) return rc;
  if (!d_beams_f16 || !d_spectra) return set_err(SF_ERR_INVALID_ARGUMENT, "NULL buffer");
  if (n_beams_out < 1) return set_err(SF_ERR_INVALID_ARGUMENT, "n_beams_out must be >= 1");
  if (reinterpret_cast<uintptr_t>(d_beams_f16) % 16 != 0)
    return set_err(SF_ERR_INVALID_ARGUMENT, "beams must be 16-byte aligned");
  if (!sf_packet_spectra_supported(plan->Tp))
    return set_err(SF_ERR_UNSUPPORTED, "packet spectra need Tp in {16, 32, 64} (Tp = %d)", plan->Tp);
  if (trim < 0 || 2 * trim >= plan->Tp)
    return set_err(SF_ERR_INVALID_ARGUMENT, "trim %d outside [0, Tp/2)", trim);
  SF_TRY(sf_launch_packet_spectra(plan, reinterpret_cast<const __half2 *>(d_beams_f16), n_beams_out,
                                  trim, d_spectra, as_stream(stream)),
         "packet spectra launch");
  return SF_OK;
}

int sf_accumulate_visibilities(sf_plan *plan, const int32_t *d_vis, int64_t *d_accum, void *stream) {
  if (int rc = check_plan(plan)) return rc;
  if (!d_vis || !d_accum) return set_err(SF_ERR_INVALID_ARGUMENT, "NULL buffer");
  SF_TRY(sf_launch_vis_accumulate(plan, d_vis, d_accum, as_stream(stream)), "accumulate launch");
  return SF_OK;
}

int sf_visibilities_to_float(sf_plan *plan, const int64_t *d_accum, float *d_vis_f32, void *stream) {
  if (int rc = check_plan(plan)) return rc;
  if (!d_accum || !d_vis_f32) return set_err(SF_ERR_INVALID_ARGUMENT, "NULL buffer");
  SF_TRY(sf_launch_vis_to_float(plan, d_accum, d_vis_f32, as_stream(stream)), "vis float launch");
  return SF_OK;
}

int sf_run_corr_beam(sf_plan *plan, const int8_t *d_samples, const int16_t *d_scales,
                     int32_t *d_vis, uint16_t *d_beams_f16, void *stream) {
  if (int rc = check_plan(plan)) return rc;
  int32_t *vis = d_vis ? d_vis : plan->d_vis;
  if (!d_samples || !d_scales || !d_beams_f16) return set_err(SF_ERR_INVALID_ARGUMENT, "NULL buffer");
  char why[160];
  if (sf_correlate_supported(plan, why, sizeof(why)) && sf_corrbeam_fused_supported(plan, plan->B) &&
      reinterpret_cast<uintptr_t>(d_samples) % 16 == 0) {
    // one pass over the samples: correlation and beams from the same tiles
    cudaStream_t s = as_stream(stream);
    SF_TRY(sf_launch_weights_plain(plan, s), "weights launch");
    SF_TRY(sf_launch_corrbeam(plan, d_samples, d_scales, plan->d_off_packet, vis, plan->B,
                              reinterpret_cast<__half2 *>(d_beams_f16), 3, s),
           "correlate+beamform launch");
    return SF_OK;
  }
  if (int rc = sf_correlate(plan, d_samples, d_scales, SF_WINDOW_PACKET, vis, stream)) return rc;
  return sf_beamform(plan, d_samples, d_scales, SF_WINDOW_PACKET, 1, d_beams_f16, stream);
}

int sf_run_lambda_gpu(sf_plan *plan, const int8_t *d_samples, const int16_t *d_scales,
                      int32_t *d_vis, float *d_evals, float *d_evecs, uint16_t *d_beams_f16,
                      void *stream) {
  if (int rc = check_plan(plan)) return rc;
  int32_t *vis = d_vis ? d_vis : plan->d_vis;
  float *evals = d_evals ? d_evals : plan->d_evals;
  if (!d_samples || !d_scales || !d_beams_f16) return set_err(SF_ERR_INVALID_ARGUMENT, "NULL buffer");
  char why[160];
  if (sf_correlate_supported(plan, why, sizeof(why)) && sf_corrbeam_fused_supported(plan, plan->B) &&
      reinterpret_cast<uintptr_t>(d_samples) % 16 == 0) {
    cudaStream_t s = as_stream(stream);
    SF_TRY(sf_launch_weights_plain(plan, s), "weights launch");
    SF_TRY(sf_launch_corrbeam(plan, d_samples, d_scales, plan->d_off_aligned, vis, plan->B,
                              reinterpret_cast<__half2 *>(d_beams_f16), 3, s),
           "correlate+beamform launch");
    return sf_covariance_eig(plan, vis, SF_EIG_ALL_BLOCKS, SF_K_FIXED, 0.f, 0, evals, d_evecs, nullptr,
                             nullptr, stream);
  }
  if (int rc = sf_correlate(plan, d_samples, d_scales, SF_WINDOW_ALIGNED, vis, stream)) return rc;
  if (int rc = sf_covariance_eig(plan, vis, SF_EIG_ALL_BLOCKS, SF_K_FIXED, 0.f, 0, evals, d_evecs,
                                 nullptr, nullptr, stream))
    return rc;
  return sf_beamform(plan, d_samples, d_scales, SF_WINDOW_ALIGNED, 1, d_beams_f16, stream);
}

int sf_run_adaptive(sf_plan *plan, const int8_t *d_samples, const int16_t *d_scales, int32_t k_rule,
                    float delta, int32_t shrink, int32_t *d_vis, float *d_evals, float *d_evecs,
                    int32_t *d_counts, uint16_t *d_beams_f16, void *stream) {
  if (int rc = check_plan(plan)) return rc;
  int32_t *vis = d_vis ? d_vis : plan->d_vis;
  float *evals = d_evals ? d_evals : plan->d_evals;
  int32_t *counts = d_counts ? d_counts : plan->d_counts;
  if (int rc = sf_correlate(plan, d_samples, d_scales, SF_WINDOW_ALIGNED, vis, stream)) return rc;
  if (int rc = sf_covariance_eig(plan, vis, SF_EIG_SAME_POL_WHITENED, k_rule, delta, shrink, evals,
                                 d_evecs, counts, nullptr, stream))
    return rc;
  return sf_beamform(plan, d_samples, d_scales, SF_WINDOW_ALIGNED, 2, d_beams_f16, stream);
}

}  // extern "C"
