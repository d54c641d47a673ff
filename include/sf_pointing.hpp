/*
 * sf_pointing.hpp - beam pointing and steering for the GB300 path (host side).
 *
 * Replaces, for a host framework that drives the adapters of sf_pipeline.hpp:
 *   pointing helpers       reference include/spatial/pointing.hpp:1-95
 *   BeamSteering<T>        reference include/spatial/pipeline/common.hpp:187-327
 *   compute_steering_weights  common.hpp:97-185 (the weight loop itself runs on the
 *                          device: sf_set_steering_weights in sf_capi.h)
 *
 * The reference converts J2000 RA/Dec to azimuth/elevation through casacore's
 * MeasConvert (reference src/pointing.cpp; casacore is a system library, not
 * part of the reference tree).  topocentric_direction below restates the
 * published algorithms instead:
 *   - precession J2000 -> date, IAU 1976 angles zeta, z, theta (Lieske et al. 1977),
 *   - Greenwich mean sidereal time, IAU 1982 polynomial as in Meeus,
 *     Astronomical Algorithms eq. 12.4 (UT1 taken as UTC),
 *   - hour angle H -> ENU direction cosines
 *       east = -cos(dec) sin(H), north = cos(lat) sin(dec) - sin(lat) cos(dec) cos(H),
 *       up   =  sin(lat) sin(dec) + cos(lat) cos(dec) cos(H).
 * Nutation, annual aberration and the site height are left out (well under
 * 0.01 degree for a sidereal source).  sfgb/pointing.py is the same code in
 * Python.  Everything lives in namespace sfgb, so it can sit beside the
 * reference's own declarations.
 */
#ifndef SF_POINTING_HPP
#define SF_POINTING_HPP

#include <chrono>
#include <cmath>
#include <complex>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <utility>
#include <vector>

namespace sfgb {

constexpr double kSpeedOfLightMetresPerSecond = 299792458.0;

struct ENUPosition {
  double east = 0.0;
  double north = 0.0;
  double up = 0.0;
};

struct ArrayLocation {
  double latitude_deg = 0.0;
  double longitude_deg = 0.0;
  double height_m = 0.0;
};

struct FrequencyPlan {
  double base_frequency_hz = 0.0;
  double channel_bandwidth_hz = 0.0;
};

struct BeamTarget {
  std::string mode = "zenith";  // "radec" or "zenith"
  double ra_deg = 0.0;
  double dec_deg = 0.0;
};

struct DirectionCosines {
  double l = 0.0;
  double m = 0.0;
  double n = 1.0;
};

inline double channel_to_frequency_hz(int absolute_channel_index, const FrequencyPlan &plan) {
  return plan.base_frequency_hz + static_cast<double>(absolute_channel_index) * plan.channel_bandwidth_hz;
}

inline double to_mjd_utc(std::chrono::system_clock::time_point utc_time) {
  using namespace std::chrono;
  const double unix_seconds = duration_cast<duration<double>>(utc_time.time_since_epoch()).count();
  return 40587.0 + unix_seconds / 86400.0;
}

inline DirectionCosines zenith_direction() { return DirectionCosines{0.0, 0.0, 1.0}; }

namespace detail_pointing {
constexpr double kPi = 3.14159265358979323846;
constexpr double kJdJ2000 = 2451545.0;

// Mean place of date from a J2000 mean place (IAU 1976 precession).
inline void precess_from_j2000(double ra, double dec, double t, double *ra_out, double *dec_out) {
  const double asec = kPi / (180.0 * 3600.0);
  const double zeta = (2306.2181 * t + 0.30188 * t * t + 0.017998 * t * t * t) * asec;
  const double z = (2306.2181 * t + 1.09468 * t * t + 0.018203 * t * t * t) * asec;
  const double theta = (2004.3109 * t - 0.42665 * t * t - 0.041833 * t * t * t) * asec;
  const double a = std::cos(dec) * std::sin(ra + zeta);
  const double b = std::cos(theta) * std::cos(dec) * std::cos(ra + zeta) - std::sin(theta) * std::sin(dec);
  double c = std::sin(theta) * std::cos(dec) * std::cos(ra + zeta) + std::cos(theta) * std::sin(dec);
  c = c > 1.0 ? 1.0 : (c < -1.0 ? -1.0 : c);
  *ra_out = std::atan2(a, b) + z;
  *dec_out = std::asin(c);
}

// Greenwich mean sidereal time (IAU 1982), radians in [0, 2 pi).
inline double gmst_rad(double jd_ut) {
  const double d = jd_ut - kJdJ2000;
  const double t = d / 36525.0;
  double deg = 280.46061837 + 360.98564736629 * d + 0.000387933 * t * t - t * t * t / 38710000.0;
  deg = std::fmod(deg, 360.0);
  if (deg < 0.0) deg += 360.0;
  return deg * kPi / 180.0;
}
}  // namespace detail_pointing

// J2000 RA/Dec -> local ENU direction cosines for an observer at
// (latitude, east longitude) at `utc_time`.
inline DirectionCosines topocentric_direction(double ra_deg, double dec_deg,
                                              std::chrono::system_clock::time_point utc_time,
                                              double latitude_deg, double longitude_deg, double /*height_m*/) {
  using namespace detail_pointing;
  const double jd = to_mjd_utc(utc_time) + 2400000.5;
  double ra, dec;
  precess_from_j2000(ra_deg * kPi / 180.0, dec_deg * kPi / 180.0, (jd - kJdJ2000) / 36525.0, &ra, &dec);
  const double h = gmst_rad(jd) + longitude_deg * kPi / 180.0 - ra;
  const double phi = latitude_deg * kPi / 180.0;
  DirectionCosines dc;
  dc.l = -std::cos(dec) * std::sin(h);
  dc.m = std::cos(phi) * std::sin(dec) - std::sin(phi) * std::cos(dec) * std::cos(h);
  dc.n = std::sin(phi) * std::sin(dec) + std::cos(phi) * std::cos(dec) * std::cos(h);
  return dc;
}

inline DirectionCosines target_direction(const BeamTarget &target, std::chrono::system_clock::time_point utc_time,
                                         const ArrayLocation &site) {
  if (target.mode == "zenith") return zenith_direction();
  return topocentric_direction(target.ra_deg, target.dec_deg, utc_time, site.latitude_deg, site.longitude_deg,
                               site.height_m);
}

// Receiver-ordered inputs of sf_set_steering_weights, resolved as
// compute_steering_weights does (common.hpp:109-160): receiver r takes the
// position of antenna antenna_mapping[r], ENU 0 when either lookup misses; a
// negative antenna ID marks a null input.
struct SteeringGeometry {
  std::vector<double> enu;         // [R][3]
  std::vector<int32_t> connected;  // [R]
};

inline SteeringGeometry steering_geometry(int n_receivers,
                                          const std::unordered_map<int, ENUPosition> &antenna_positions,
                                          const std::unordered_map<int, int> &antenna_mapping) {
  SteeringGeometry g;
  g.enu.assign(3 * static_cast<size_t>(n_receivers), 0.0);
  g.connected.assign(n_receivers, 1);
  for (int r = 0; r < n_receivers; ++r) {
    const auto it = antenna_mapping.find(r);
    if (it == antenna_mapping.end()) continue;
    if (it->second < 0) {
      g.connected[r] = 0;
      continue;
    }
    const auto pos = antenna_positions.find(it->second);
    if (pos == antenna_positions.end()) continue;
    g.enu[3 * r + 0] = pos->second.east;
    g.enu[3 * r + 1] = pos->second.north;
    g.enu[3 * r + 2] = pos->second.up;
  }
  return g;
}

}  // namespace sfgb

// ---- steering of the adapters' plans (needs the C ABI) -----------------------
#ifdef SF_CAPI_H
#include <cuda_runtime.h>

namespace sfgb {

// BeamSteering for the GB300 adapters: keeps every registered plan's weights
// pointed at the targets, recomputing at most once per `update_interval`
// (reference common.hpp:187-327).  With no targets it is inert and the plans
// keep their constructor weights.  maybe_refresh() runs the synthesis kernel
// on every registered plan in one call, so all buffers always beamform with
// weights of the same instant; call it from the thread that enqueues the
// pipeline's work, before the run that should see the new weights (the
// adapters do so at the top of execute_pipeline).
// calibration_gains: complex<float> [C][Pol][R] (AntennaGains layout) or nullptr.
template <typename Config> class SfBeamSteering {
 public:
  SfBeamSteering() = default;
  SfBeamSteering(std::vector<BeamTarget> targets, std::unordered_map<int, ENUPosition> antenna_positions,
                 std::unordered_map<int, int> antenna_mapping, FrequencyPlan frequency_plan, int min_freq_channel,
                 ArrayLocation array_location, double update_interval_seconds,
                 const std::complex<float> *calibration_gains = nullptr)
      : targets_(std::move(targets)),
        geometry_(steering_geometry(Config::NR_RECEIVERS, antenna_positions, antenna_mapping)),
        frequency_plan_(frequency_plan),
        min_freq_channel_(min_freq_channel),
        array_location_(array_location),
        update_interval_(update_interval_seconds),
        calibration_gains_(calibration_gains) {}

  bool active() const { return !targets_.empty(); }

  void register_plan(sf_plan *plan, cudaStream_t stream) { plans_.push_back({plan, stream}); }

  // Direction cosines of every beam at `utc_time` ([B][3]; beams past the
  // end of the target list point at the zenith).
  std::vector<double> direction_cosines(std::chrono::system_clock::time_point utc_time) const {
    std::vector<double> dc(3 * static_cast<size_t>(Config::NR_BEAMS));
    for (int b = 0; b < Config::NR_BEAMS; ++b) {
      const BeamTarget target = b < static_cast<int>(targets_.size()) ? targets_[b] : BeamTarget{};
      const DirectionCosines d = target_direction(target, utc_time, array_location_);
      dc[3 * b] = d.l;
      dc[3 * b + 1] = d.m;
      dc[3 * b + 2] = d.n;
    }
    return dc;
  }

  // Recompute every registered plan's weights for `utc_time` now.
  void refresh(std::chrono::system_clock::time_point utc_time) {
    const std::vector<double> dc = direction_cosines(utc_time);
    for (const auto &p : plans_) {
      const int rc = sf_set_steering_weights(p.plan, dc.data(), geometry_.enu.data(), geometry_.connected.data(),
                                             frequency_plan_.base_frequency_hz,
                                             frequency_plan_.channel_bandwidth_hz, min_freq_channel_,
                                             reinterpret_cast<const float *>(calibration_gains_), p.stream);
      if (rc != SF_OK) throw std::runtime_error(std::string("sf_set_steering_weights: ") + sf_last_error());
    }
    last_update_ = utc_time;
  }

  // True when the weights were recomputed (the first call always is).
  bool maybe_refresh() {
    if (!active() || plans_.empty()) return false;
    const auto now = std::chrono::system_clock::now();
    if (now - last_update_ < update_interval_) return false;
    refresh(now);
    return true;
  }

 private:
  struct Registered {
    sf_plan *plan;
    cudaStream_t stream;
  };
  std::vector<BeamTarget> targets_;
  SteeringGeometry geometry_;
  FrequencyPlan frequency_plan_;
  int min_freq_channel_ = 0;
  ArrayLocation array_location_;
  std::chrono::duration<double> update_interval_{0.0};
  const std::complex<float> *calibration_gains_ = nullptr;
  std::vector<Registered> plans_;
  std::chrono::system_clock::time_point last_update_{};
};

}  // namespace sfgb
#endif  // SF_CAPI_H

#endif  // SF_POINTING_HPP
