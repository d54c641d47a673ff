// Steering-weight synthesis on the device: the weights payload (BeamWeightsT,
// fp16 pairs [C][Pol][B][R]) computed from per-beam direction cosines and
// per-receiver antenna positions, replacing the host loop of
// compute_steering_weights (include/spatial/pipeline/common.hpp:97-185) and
// the host->device copy BeamSteering::maybe_refresh enqueues per buffer
// (common.hpp:255-300).  Per element, in double precision as the reference:
//   f     = base + (min_ch + c) bw                   (channel_to_frequency_hz)
//   phase = -2 pi f / c_light * (l east + m north + n up)
//   w     = (1 / R) * G[c][pol][r] * exp(i phase)   (G = 1 without calibration)
// rounded to float and then to fp16; receivers that are null inputs get
// exactly zero.  The fine-delay phasors and antenna gains of the plan stay
// separate and are applied when the effective weights are formed, as before.
#include <cmath>

#include "sf_common.cuh"
#include "sf_plan.cuh"

namespace {

constexpr double kSpeedOfLight = 299792458.0;  // m/s
constexpr double kPi = 3.14159265358979323846;

struct SteerArgs {
  const double *dircos;    // [B][3] l, m, n
  const double *enu;       // [R][3] east, north, up (metres)
  const int32_t *connected;  // [R], 0 = null input
  const float2 *cal;       // [C][2][R] or nullptr
  __half2 *weights;        // [C][2][B][R]
  double base_hz, bw_hz;
  int min_ch, C, B, R;
};

__global__ void sf_steering_kernel(const SteerArgs a) {
  const int total = a.C * 2 * a.B * a.R;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
    const int r = e % a.R;
    const int b = (e / a.R) % a.B;
    const int pol = (e / (a.R * a.B)) % 2;
    const int c = e / (a.R * a.B * 2);
    if (!a.connected[r]) {
      a.weights[e] = __floats2half2_rn(0.f, 0.f);
      continue;
    }
    const double f = a.base_hz + (double)(a.min_ch + c) * a.bw_hz;
    const double phase_scale = -2.0 * kPi * f / kSpeedOfLight;
    const double *dc = a.dircos + 3 * b;
    const double *p = a.enu + 3 * r;
    const double phase = phase_scale * (dc[0] * p[0] + dc[1] * p[1] + dc[2] * p[2]);
    double s, co;
    sincos(phase, &s, &co);
    double gr = 1.0, gi = 0.0;
    if (a.cal) {
      const float2 g = a.cal[((size_t)c * 2 + pol) * a.R + r];
      gr = g.x;
      gi = g.y;
    }
    const double inv = 1.0 / (double)a.R;
    // ((1/R) G) * phasor, the reference's evaluation order
    const double ar = inv * gr, ai = inv * gi;
    const double wr = ar * co - ai * s, wi = ar * s + ai * co;
    a.weights[e] = __halves2half2(__float2half_rn((float)wr), __float2half_rn((float)wi));
  }
}

}  // namespace

cudaError_t sf_launch_steering(const sf_plan *p, const double *d_dircos, const double *d_enu,
                               const int32_t *d_connected, const float2 *d_cal, double base_hz, double bw_hz,
                               int min_ch, cudaStream_t stream) {
  SteerArgs a;
  a.dircos = d_dircos;
  a.enu = d_enu;
  a.connected = d_connected;
  a.cal = d_cal;
  a.weights = p->d_weights;
  a.base_hz = base_hz;
  a.bw_hz = bw_hz;
  a.min_ch = min_ch;
  a.C = p->C;
  a.B = p->B;
  a.R = p->R;
  const int total = p->C * 2 * p->B * p->R;
  int grid = (total + 255) / 256;
  if (grid > 8 * p->num_sms) grid = 8 * p->num_sms;
  sf_steering_kernel<<<grid, 256, 0, stream>>>(a);
  return cudaGetLastError();
}
