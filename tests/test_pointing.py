"""Host pointing (sfgb/pointing.py, include/sf_pointing.hpp) and the steering
oracle, on the CPU.

The cases restate the reference's own pointing tests
(tests/test_pointing.cpp:23-93): zenith, linear channel plan, the MJD of the
Unix and J2000 epochs, unit direction vectors over a grid of targets, and the
north celestial pole at the observer's latitude (tolerance 0.01 on direction
cosines there, as in the reference).  The C++ header is compiled with g++ and
must agree with the Python mirror to 1e-12.
"""
import math
import os
import subprocess
import tempfile

import numpy as np
import pytest

import sf_oracle as orc
from sfgb import pointing as pt

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
NOW = 1.7648e9  # a fixed UTC instant (Unix seconds, late 2025)


def test_zenith_and_channel_plan():
    assert pt.zenith_direction() == (0.0, 0.0, 1.0)
    assert pt.channel_to_frequency_hz(0, 1.0e9, 1.0e5) == 1.0e9
    assert pt.channel_to_frequency_hz(10, 1.0e9, 1.0e5) == 1.0e9 + 10 * 1.0e5
    assert pt.channel_to_frequency_hz(-3, 1.0e9, 1.0e5) == 1.0e9 - 3 * 1.0e5


def test_mjd_epochs():
    assert pt.to_mjd_utc(0.0) == 40587.0
    assert abs(pt.to_mjd_utc(946684800 + 12 * 3600) - 51544.5) < 1e-9


def test_topocentric_unit_vector():
    for ra in (0.0, 83.633, 180.0, 279.23):
        for dec in (-60.0, -16.7, 0.0, 38.78, 89.0):
            l, m, n = pt.topocentric_direction(ra, dec, NOW, 52.91, 6.87, 30.0)
            assert abs(l * l + m * m + n * n - 1.0) < 1e-9


@pytest.mark.parametrize("hours", [0, 6, 12, 18])
def test_north_celestial_pole_at_latitude(hours):
    lat = 40.0
    l, m, n = pt.topocentric_direction(123.45, 90.0, NOW + 3600 * hours, lat, -71.06, 0.0)
    assert abs(l - 0.0) < 0.01
    assert abs(m - math.cos(math.radians(lat))) < 0.01
    assert abs(n - math.sin(math.radians(lat))) < 0.01


def test_sidereal_rotation_and_transit():
    # GMST advances 360.9856 degrees per solar day
    d = pt.gmst_rad(2451545.0 + 1.0) - pt.gmst_rad(2451545.0)
    assert abs(math.degrees(d) % 360.0 - 0.98564736629) < 1e-9
    # at J2000.0 the polynomial's constant term
    assert abs(math.degrees(pt.gmst_rad(2451545.0)) - 280.46061837) < 1e-9
    # a source on the local meridian is due south (or north), at el = 90 - |lat - dec|
    t = NOW
    jd = pt.to_mjd_utc(t) + 2400000.5
    lon = 6.87
    ra_date = math.degrees(pt.gmst_rad(jd)) + lon  # H = 0 for a source at this RA of date
    # invert the precession approximately by precessing back with -T (small error)
    ra0, dec0 = pt.precess_from_j2000(math.radians(ra_date), math.radians(20.0), -(jd - 2451545.0) / 36525.0)
    l, m, n = pt.topocentric_direction(math.degrees(ra0), math.degrees(dec0), t, 52.91, lon)
    assert abs(l) < 1e-4
    assert abs(math.degrees(math.asin(n)) - (90.0 - (52.91 - 20.0))) < 1e-3


def test_steering_geometry_resolves_maps():
    pos = {100: (0.0, 0.0, 0.0), 101: (25.0, -10.0, 1.5)}
    mapping = {0: -100, 1: 100, 2: -100, 3: 101}
    dircos, enu, conn = pt.steering_geometry(2, 5, [{"mode": "zenith"}], pos, mapping, NOW)
    assert dircos == [(0.0, 0.0, 1.0), (0.0, 0.0, 1.0)]
    assert conn == [0, 1, 0, 1, 1]  # receiver 4 unmapped: connected at ENU 0
    assert enu[3] == (25.0, -10.0, 1.5) and enu[4] == (0.0, 0.0, 0.0)


def test_steering_oracle_matches_reference_formula():
    """The reference's ComputeSteeringWeightsMatchesGeometricPhaseFormula
    (tests/test_pipeline.cu:1362-1433) on the oracle."""
    sh = orc.Shape(4, 1, 16, 4, 4, 1, 2)
    pos = {100: (0.0, 0.0, 0.0), 101: (25.0, -10.0, 1.5), 102: (-12.5, 30.0, -2.0), 103: (8.0, 8.0, 0.5)}
    mapping = {0: 100, 1: 101, 2: 102, 3: 103}
    targets = [{"mode": "radec", "ra_deg": 83.633, "dec_deg": 22.014}]
    dircos, enu, conn = pt.steering_geometry(sh.B, sh.R, targets, pos, mapping, NOW, 52.91, 6.87, 30.0)
    w = orc.steering_weights(sh, dircos, enu, conn, 1.4e9, 1.0e5, 64)
    dc = pt.topocentric_direction(83.633, 22.014, NOW, 52.91, 6.87, 30.0)
    for c in range(sh.C):
        f = pt.channel_to_frequency_hz(64 + c, 1.4e9, 1.0e5)
        for r in range(sh.R):
            e = pos[mapping[r]]
            ph = -2.0 * math.pi * f / pt.SPEED_OF_LIGHT * (dc[0] * e[0] + dc[1] * e[1] + dc[2] * e[2])
            exp = (1.0 / sh.R) * complex(math.cos(ph), math.sin(ph))
            for p in range(2):
                got = complex(float(w[c, p, 0, r, 0]), float(w[c, p, 0, r, 1]))
                assert abs(got.real - exp.real) < 2e-3 and abs(got.imag - exp.imag) < 2e-3
    # beam 1 has no target: zenith
    wz = orc.steering_weights(sh, [(0, 0, 1)] * 2, enu, conn, 1.4e9, 1.0e5, 64)
    assert np.array_equal(w[:, :, 1], wz[:, :, 1])


def test_steering_oracle_zeroes_null_inputs():
    sh = orc.Shape(3, 1, 16, 4, 4, 1, 2)
    pos = {100: (0.0, 0.0, 0.0), 101: (25.0, -10.0, 1.5)}
    mapping = {0: -100, 1: 100, 2: -100, 3: 101}
    dircos, enu, conn = pt.steering_geometry(sh.B, sh.R, [{"mode": "zenith"}], pos, mapping, NOW)
    w = orc.steering_weights(sh, dircos, enu, conn, 1.4e9, 1.0e5, 0).astype(np.float32)
    amp = np.hypot(w[..., 0], w[..., 1])
    assert np.all(w[:, :, :, [0, 2]] == 0.0)
    assert np.all(np.abs(amp[:, :, :, [1, 3]] - 1.0 / sh.R) < 2e-3)


CPP_TEST = r'''
#include <cstdio>
#include "sf_pointing.hpp"
int main() {
  using namespace std::chrono;
  const double ras[] = {0.0, 83.633, 180.0, 279.23, 123.45};
  const double decs[] = {-60.0, -16.7, 0.0, 38.78, 89.0, 90.0};
  for (double t : {1.7648e9, 1.7648e9 + 21600.0, 1.0e9}) {
    const auto tp = system_clock::time_point{} + duration_cast<system_clock::duration>(duration<double>(t));
    for (double ra : ras)
      for (double dec : decs) {
        sfgb::DirectionCosines d = sfgb::topocentric_direction(ra, dec, tp, 52.91, 6.87, 30.0);
        std::printf("%.17g %.17g %.17g %.17g %.17g %.17g\n", t, ra, dec, d.l, d.m, d.n);
      }
  }
  return 0;
}
'''


def test_cpp_pointing_matches_python():
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "t.cpp")
        exe = os.path.join(d, "t")
        with open(src, "w") as f:
            f.write(CPP_TEST)
        subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), src, "-o", exe],
                       check=True, capture_output=True)
        out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout.split("\n")
    n = 0
    for line in out:
        if not line.strip():
            continue
        t, ra, dec, l, m, nn = (float(x) for x in line.split())
        ref = pt.topocentric_direction(ra, dec, t, 52.91, 6.87, 30.0)
        assert max(abs(l - ref[0]), abs(m - ref[1]), abs(nn - ref[2])) < 1e-9, (t, ra, dec)
        n += 1
    assert n == 3 * 5 * 6
