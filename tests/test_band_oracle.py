"""The oracle's random band forcing (CPU, no GPU).

* Philox4x32-10 against the known-answer vectors published with the
  generator (Random123's kat_vectors for philox4x32_10);
* the Gaussian lattice band: its mode count and every mode's contribution
  restated here from the Philox words, so the C restatement and this one agree;
* bandForcing (src/cpu/solver.js:179-217): the increment is the curl of the
  streamfunction, so its discrete divergence is second order small.
"""
from __future__ import annotations

import math

import numpy as np
import pytest


@pytest.mark.parametrize("ctr,key,expected", [
    ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
    ((0xFFFFFFFF,) * 4, (0xFFFFFFFF,) * 2, (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
    ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
     (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
])
def test_philox_known_answers(O, ctr, key, expected):
    assert O.philox4x32_10(ctr, key) == expected


def _lattice(kf, width):
    K = math.ceil(kf + width)
    lo, hi = kf - width, kf + width
    return [(kx, ky) for ky in range(-K, K + 1) for kx in range(-K, K + 1)
            if kx * kx + ky * ky != 0 and lo * lo <= kx * kx + ky * ky <= hi * hi]


def test_gauss_band_matches_its_definition(O):
    n, kf, width, amp, key, counter, dt = 32, 3.0, 1.0, 2.0, (7 << 32) | 11, 5, 0.01
    lat = _lattice(kf, width)
    assert len(lat) == 40
    assert len(_lattice(9.0, 1.0)) == 124  # the forced-turbulence band 8 <= |k| <= 10
    g = O.grid(n)
    u = np.zeros(n * n)
    v = np.zeros(n * n)
    O.gauss_band_forcing(g, u, v, kf, width, amp, key, counter, dt)
    h = 2 * math.pi / n
    i = np.arange(n)
    X, Y = np.meshgrid(i * h, i * h)  # [j, i]
    eu = np.zeros((n, n))
    ev = np.zeros((n, n))
    s = amp * dt / math.sqrt(len(lat))
    for m, (kx, ky) in enumerate(lat):
        r = O.philox4x32_10((counter, m, 0, 0), (key & 0xFFFFFFFF, key >> 32))
        A = math.sqrt(-2 * math.log((r[0] + 0.5) / 2 ** 32))
        phi = 2 * math.pi * (r[1] + 0.5) / 2 ** 32
        k = math.hypot(kx, ky)
        eu += s * A * (ky / k) * np.cos(kx * X + ky * (Y + h / 2) + phi)
        ev += s * A * (-kx / k) * np.cos(kx * (X + h / 2) + ky * Y + phi)
    assert np.abs(u - eu.ravel()).max() <= 1e-14
    assert np.abs(v - ev.ravel()).max() <= 1e-14


def test_band_forcing_is_nearly_solenoidal(O):
    n = 128
    g = O.grid(n)
    for fn, args in ((O.band_forcing, (28.0, 2.0, 0.4, 3, 0.01)),
                     (O.gauss_band_forcing, (9.0, 1.0, 3.0, 1, 0, 0.01))):
        u = np.zeros(n * n)
        v = np.zeros(n * n)
        fn(g, u, v, *args)
        f = max(np.abs(u).max(), np.abs(v).max())
        assert f > 0
        # the discrete divergence of the sampled curl is O((k h)^2) of |k| |F|
        assert O.max_divergence(g, u, v) < 0.5 * f * 30
