// sf_run_adaptive_noalloc: the adaptive chain (correlate -> whitened
// eigendecomposition -> K -> I - U U^H -> W P -> beams) for callers that may
// not allocate device memory.
//
// Who needs it: code that runs where cudaMalloc is off limits -- inside a
// host callback or a real-time thread that must never block on the
// allocator, in a process whose device memory is carved up up-front by
// another framework's pool, or in a plugin host that forbids its plugins
// from allocating.  Such a caller owns its input and output buffers but
// cannot create a plan (sf_plan_create allocates).
//
// Where the intermediates live: one file-scope __device__ array of
// SF_NOALLOC_SCRATCH_BYTES (16 MiB), which every GPU that loads this library
// holds until the process exits.  It stores the window offsets, the
// per-receiver factors, the fixed counts, the visibilities, the effective
// weights, the counts (when the caller passes none) and the status word.
// The first call on each device is the set-up call: it looks the array's
// device address up with cudaGetSymbolAddress (with that device current) and
// caches it.  That lookup may load the library's device code and commit the
// 16 MiB, so make the first call outside the real-time path and before any
// stream capture; later calls allocate nothing.  All calls on a device share
// its one array, which keeps the last call's contents: calls that overlap on
// the same GPU (for example on two streams) race with each other, so the
// caller must serialise them (one stream, or events between streams).
#include <cstdio>
#include <cstring>
#include <mutex>

#include "sf_common.cuh"
#include "sf_plan.cuh"

namespace {

constexpr size_t SF_NOALLOC_SCRATCH_BYTES = size_t(16) << 20;
constexpr int MAX_DEVICES = 64;

__device__ __align__(256) unsigned char sf_noalloc_scratch[SF_NOALLOC_SCRATCH_BYTES];

unsigned char *g_scratch[MAX_DEVICES];
std::mutex g_scratch_mu;

size_t round256(size_t x) { return (x + 255) & ~size_t(255); }

// Per-call state that must start fresh: window offsets, factors, fixed
// counts and the scratch status word.  Visibilities and effective weights are
// fully rewritten by the kernels of every call.  The correlator's packet ring
// and the beamformer's sample index assume window offsets in [0, 2 Tp], so a
// delay outside [-Tp, Tp] is replaced by 0 and reported (SF_DEVERR_BAD_DELAY)
// instead of letting a kernel read outside the caller's samples.  Thread 0
// clears the scratch status before it reports, so the two cannot race when
// the report goes to the scratch word.
__global__ void sf_noalloc_init_kernel(int32_t *offsets, const int32_t *delays, int F, int Tp,
                                       float2 *factors, const float2 *factors_in, int nfactors,
                                       int32_t *fixed, const int32_t *fixed_in, int C,
                                       uint32_t *scratch_status, uint32_t *report_status) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int stride = gridDim.x * blockDim.x;
  if (tid == 0) {
    *scratch_status = 0;
    bool bad = false;
    for (int f = 0; f < F; ++f) {
      int d = delays ? delays[f] : 0;
      if (d < -Tp || d > Tp) {
        bad = true;
        d = 0;
      }
      offsets[f] = Tp + d;
    }
    if (bad) atomicOr(report_status, SF_DEVERR_BAD_DELAY);
  }
  for (int i = tid; i < nfactors; i += stride)
    factors[i] = factors_in ? factors_in[i] : make_float2(1.0f, 0.0f);
  for (int c = tid; c < C; c += stride) fixed[c] = fixed_in ? fixed_in[c] : 0;
}

}  // namespace

int sf_internal_set_error(int code, const char *msg);

extern "C" int sf_run_adaptive_noalloc(const sf_shape *shape, const int8_t *d_samples,
                                       const int16_t *d_scales, const uint16_t *d_weights_f16,
                                       const float *d_factors, const int32_t *d_delays,
                                       const int32_t *d_fixed_counts, int32_t k_rule, float delta,
                                       int32_t shrink, int32_t *d_counts, uint16_t *d_beams_f16,
                                       uint32_t *d_status, void *stream) {
  char msg[256];
  if (!shape || !d_samples || !d_scales || !d_weights_f16 || !d_beams_f16)
    return sf_internal_set_error(SF_ERR_INVALID_ARGUMENT, "shape, samples, scales, weights or beams is NULL");
  const sf_shape &s = *shape;
  if (s.n_polarizations != 2)
    return sf_internal_set_error(SF_ERR_UNSUPPORTED, "n_polarizations must be 2");
  if (s.n_channels < 1 || s.n_fpgas < 1 || s.n_time_per_packet < 1 || s.n_receivers < 1 ||
      s.n_receivers_per_packet < 1 || s.n_packets < 1 || s.n_beams < 1 ||
      s.n_receivers != s.n_fpgas * s.n_receivers_per_packet)
    return sf_internal_set_error(SF_ERR_INVALID_ARGUMENT, "inconsistent shape");
  if (k_rule < SF_K_FIXED || k_rule > SF_K_NOISE_FLOOR)
    return sf_internal_set_error(SF_ERR_INVALID_ARGUMENT, "unknown K rule");
  if (reinterpret_cast<uintptr_t>(d_samples) % 16 != 0)
    return sf_internal_set_error(SF_ERR_INVALID_ARGUMENT, "samples must be 16-byte aligned");
  if (reinterpret_cast<uintptr_t>(d_factors) % 8 != 0)
    return sf_internal_set_error(SF_ERR_INVALID_ARGUMENT, "factors must be 8-byte aligned");
  if (reinterpret_cast<uintptr_t>(d_weights_f16) % 4 != 0 || reinterpret_cast<uintptr_t>(d_beams_f16) % 4 != 0)
    return sf_internal_set_error(SF_ERR_INVALID_ARGUMENT, "weights and beams must be 4-byte aligned");

  // A plan-shaped view over the caller's buffers and the static scratch:
  // built on the stack, nothing allocated.
  sf_plan p;
  memset(&p, 0, sizeof(p));
  p.shape = s;
  p.C = s.n_channels;
  p.F = s.n_fpgas;
  p.Tp = s.n_time_per_packet;
  p.R = s.n_receivers;
  p.Rpp = s.n_receivers_per_packet;
  p.P = s.n_packets;
  p.B = s.n_beams;
  p.T = p.P * p.Tp;
  p.NBL = p.R * (p.R + 1) / 2;
  if (!sf_correlate_supported(&p, msg, sizeof(msg)) || !sf_eig_supported(&p, msg, sizeof(msg)))
    return sf_internal_set_error(SF_ERR_UNSUPPORTED, msg);
  if (2 * p.B > 32) return sf_internal_set_error(SF_ERR_UNSUPPORTED, "at most 16 beams (32 outputs)");

  const size_t C = p.C, R = p.R, B = p.B;
  const size_t off_offsets = 0;
  const size_t off_factors = off_offsets + round256(sizeof(int32_t) * p.F);
  const size_t off_fixed = off_factors + round256(sizeof(float2) * C * 2 * R);
  const size_t off_vis = off_fixed + round256(sizeof(int32_t) * C);
  const size_t off_weff = off_vis + round256(sizeof(int32_t) * C * p.NBL * 8);
  const size_t off_counts = off_weff + round256(sizeof(float2) * C * 2 * 2 * B * R);
  const size_t off_status = off_counts + round256(sizeof(int32_t) * C * 2);
  const size_t need = off_status + 256;
  if (need > SF_NOALLOC_SCRATCH_BYTES) {
    snprintf(msg, sizeof(msg),
             "shape needs %zu bytes of scratch; the allocation-free entry point holds %zu "
             "(use sf_plan_create + sf_run_adaptive)",
             need, SF_NOALLOC_SCRATCH_BYTES);
    return sf_internal_set_error(SF_ERR_UNSUPPORTED, msg);
  }

  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= MAX_DEVICES)
    return sf_internal_set_error(SF_ERR_NO_DEVICE, "no usable current device");
  int major = 0, minor = 0;
  cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
  cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
  if (major != 10 || minor != 3)
    return sf_internal_set_error(SF_ERR_NO_DEVICE, "this library is built for sm_103a");
  unsigned char *base = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch[dev]) {
      // Set-up, once per device, with that device current: the host-side
      // name of the array is not a device address.
      void *ptr = nullptr;
      e = cudaGetSymbolAddress(&ptr, sf_noalloc_scratch);
      if (e != cudaSuccess || !ptr) {
        snprintf(msg, sizeof(msg), "cudaGetSymbolAddress(scratch): %s", cudaGetErrorString(e));
        return sf_internal_set_error(SF_ERR_CUDA, msg);
      }
      g_scratch[dev] = static_cast<unsigned char *>(ptr);
    }
    base = g_scratch[dev];
  }
  cudaDeviceGetAttribute(&p.num_sms, cudaDevAttrMultiProcessorCount, dev);
  p.device = dev;
  p.d_off_aligned = reinterpret_cast<int32_t *>(base + off_offsets);
  p.d_factors = reinterpret_cast<float2 *>(base + off_factors);
  p.d_fixed_counts = reinterpret_cast<int32_t *>(base + off_fixed);
  p.d_vis = reinterpret_cast<int32_t *>(base + off_vis);
  p.d_weff = reinterpret_cast<float2 *>(base + off_weff);
  p.d_counts = d_counts ? d_counts : reinterpret_cast<int32_t *>(base + off_counts);
  p.d_status = d_status ? d_status : reinterpret_cast<uint32_t *>(base + off_status);
  p.d_weights = reinterpret_cast<__half2 *>(const_cast<uint16_t *>(d_weights_f16));

  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  // With a caller-provided status word the caller owns (and clears) it.
  sf_noalloc_init_kernel<<<8, 256, 0, st>>>(p.d_off_aligned, d_delays, p.F, p.Tp, p.d_factors,
                                            reinterpret_cast<const float2 *>(d_factors),
                                            static_cast<int>(C * 2 * R), p.d_fixed_counts,
                                            d_fixed_counts, p.C,
                                            reinterpret_cast<uint32_t *>(base + off_status), p.d_status);
  e = cudaGetLastError();
  if (e == cudaSuccess) e = sf_launch_correlate(&p, d_samples, d_scales, p.d_off_aligned, p.d_vis, st);
  if (e == cudaSuccess)
    e = sf_launch_eig(&p, p.d_vis, SF_EIG_SAME_POL_WHITENED, k_rule, delta, shrink ? 1 : 0, nullptr,
                      nullptr, p.d_counts, nullptr, st);
  if (e == cudaSuccess)
    e = sf_launch_beam(&p, d_samples, d_scales, p.d_off_aligned, 2,
                       reinterpret_cast<__half2 *>(d_beams_f16), st);
  if (e == cudaErrorInvalidConfiguration)
    return sf_internal_set_error(SF_ERR_UNSUPPORTED, "packet ring does not fit shared memory for this shape");
  if (e != cudaSuccess) {
    snprintf(msg, sizeof(msg), "allocation-free chain launch: %s", cudaGetErrorString(e));
    return sf_internal_set_error(SF_ERR_CUDA, msg);
  }
  return SF_OK;
}
