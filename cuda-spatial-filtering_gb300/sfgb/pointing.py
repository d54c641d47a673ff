"""Beam pointing on the host: target -> direction cosines in the array's
local East-North-Up frame, the geometric input of steering-weight synthesis
(Plan.set_steering_weights).

Mirrors include/sf_pointing.hpp (same functions, same arithmetic) and the
reference's pointing helpers (include/spatial/pointing.hpp:1-95).  The
reference converts J2000 RA/Dec to azimuth/elevation through casacore's
MeasConvert (src/pointing.cpp; casacore is a system library, not part of the
reference tree).  Restated here from the published algorithms:

  * precession J2000 -> date with the IAU 1976 angles zeta, z, theta
    (Lieske et al. 1977, A&A 58, 1),
  * Greenwich mean sidereal time from the IAU 1982 polynomial in the form of
    Meeus, Astronomical Algorithms, eq. 12.4 (UT1 taken as UTC),
  * hour angle -> ENU direction cosines
      east  = -cos(dec) sin(H)
      north =  cos(lat) sin(dec) - sin(lat) cos(dec) cos(H)
      up    =  sin(lat) sin(dec) + cos(lat) cos(dec) cos(H)
    (l = sin(az) cos(el), m = cos(az) cos(el), n = sin(el), azimuth from north
    through east).

Nutation (< 20 arcsec), annual aberration (< 21 arcsec) and the site height
(parallax of a sidereal source) are left out: the direction differs from a
full reduction by well under 0.01 degree, far inside the 0.01 tolerance the
reference's pointing tests allow on direction cosines
(tests/test_pointing.cpp:14-19).
"""
from __future__ import annotations

import math

SPEED_OF_LIGHT = 299792458.0  # m/s, include/spatial/pipeline/common.hpp:62
MJD_UNIX_EPOCH = 40587.0
JD_J2000 = 2451545.0


def channel_to_frequency_hz(absolute_channel, base_frequency_hz, channel_bandwidth_hz):
    """Linear channel plan (pointing.hpp:57-61)."""
    return base_frequency_hz + float(absolute_channel) * channel_bandwidth_hz


def to_mjd_utc(unix_seconds):
    """MJD (UTC) of a Unix time (pointing.hpp:71-77)."""
    return MJD_UNIX_EPOCH + unix_seconds / 86400.0


def zenith_direction():
    """(l, m, n) of the zenith (pointing.hpp:80-83)."""
    return (0.0, 0.0, 1.0)


def precess_from_j2000(ra_rad, dec_rad, centuries):
    """Mean place of date from a J2000 mean place (IAU 1976 precession)."""
    t = centuries
    asec = math.pi / (180.0 * 3600.0)
    zeta = (2306.2181 * t + 0.30188 * t * t + 0.017998 * t * t * t) * asec
    z = (2306.2181 * t + 1.09468 * t * t + 0.018203 * t * t * t) * asec
    theta = (2004.3109 * t - 0.42665 * t * t - 0.041833 * t * t * t) * asec
    a = math.cos(dec_rad) * math.sin(ra_rad + zeta)
    b = math.cos(theta) * math.cos(dec_rad) * math.cos(ra_rad + zeta) - math.sin(theta) * math.sin(dec_rad)
    c = math.sin(theta) * math.cos(dec_rad) * math.cos(ra_rad + zeta) + math.cos(theta) * math.sin(dec_rad)
    return math.atan2(a, b) + z, math.asin(max(-1.0, min(1.0, c)))


def gmst_rad(jd_ut):
    """Greenwich mean sidereal time (IAU 1982), radians in [0, 2 pi)."""
    d = jd_ut - JD_J2000
    t = d / 36525.0
    deg = 280.46061837 + 360.98564736629 * d + 0.000387933 * t * t - t * t * t / 38710000.0
    return math.radians(math.fmod(deg, 360.0) % 360.0)


def topocentric_direction(ra_deg, dec_deg, unix_seconds, latitude_deg, longitude_deg, height_m=0.0):
    """J2000 RA/Dec -> (l, m, n) for an observer at (latitude, east
    longitude) at a UTC time given in Unix seconds."""
    del height_m  # parallax of a sidereal source: negligible
    jd = to_mjd_utc(unix_seconds) + 2400000.5
    ra, dec = precess_from_j2000(math.radians(ra_deg), math.radians(dec_deg), (jd - JD_J2000) / 36525.0)
    h = gmst_rad(jd) + math.radians(longitude_deg) - ra
    phi = math.radians(latitude_deg)
    east = -math.cos(dec) * math.sin(h)
    north = math.cos(phi) * math.sin(dec) - math.sin(phi) * math.cos(dec) * math.cos(h)
    up = math.sin(phi) * math.sin(dec) + math.cos(phi) * math.cos(dec) * math.cos(h)
    return (east, north, up)


def target_direction(target, unix_seconds, latitude_deg, longitude_deg, height_m=0.0):
    """A BeamTarget (dict or object with mode, ra_deg, dec_deg): "zenith" or
    "radec" (common.hpp:113-119)."""
    get = target.get if isinstance(target, dict) else (lambda k, d=None: getattr(target, k, d))
    if get("mode", "zenith") == "zenith":
        return zenith_direction()
    return topocentric_direction(get("ra_deg", 0.0), get("dec_deg", 0.0), unix_seconds, latitude_deg,
                                 longitude_deg, height_m)


def steering_geometry(n_beams, n_receivers, targets, antenna_positions, antenna_mapping, unix_seconds,
                      latitude_deg=0.0, longitude_deg=0.0, height_m=0.0):
    """Receiver-ordered inputs of Plan.set_steering_weights, resolved as
    compute_steering_weights does (common.hpp:109-160): beams past the end of
    `targets` point at the zenith; receiver r takes the position of antenna
    antenna_mapping[r] (ENU 0 when either lookup misses); a negative antenna
    ID marks a null input.  Returns (dircos [B][3], enu [R][3], connected [R])."""
    dircos = []
    for b in range(n_beams):
        t = targets[b] if b < len(targets) else {"mode": "zenith"}
        dircos.append(target_direction(t, unix_seconds, latitude_deg, longitude_deg, height_m))
    enu, connected = [], []
    for r in range(n_receivers):
        pos = (0.0, 0.0, 0.0)
        ok = 1
        if r in antenna_mapping:
            aid = antenna_mapping[r]
            if aid < 0:
                ok = 0
            elif aid in antenna_positions:
                pos = tuple(float(x) for x in antenna_positions[aid])
        enu.append(pos)
        connected.append(ok)
    return dircos, enu, connected
