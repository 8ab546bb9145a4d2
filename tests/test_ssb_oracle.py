"""The single-sideband oracle (oracle.ssb_encode) against a literal,
loop-by-loop restatement of the reference's code on small fields (CPU, no
GPU).

The reference's own SSB runs cannot pin it: its FFTW plans take the array
being shifted as their input buffer, so the in-place fftShift overwrites
half of it before it is read. The loops below follow the code line by line
instead — Openholo::fftShift (Openholo/src/Openholo.cpp:749-767), FFTW's
unnormalised DFT in both directions written out as sums, circShift over the
x-major view (Openholo/src/function.h:273-283), the memsets of
ophGen::singleSideBand (ophgen/src/ophGen.cpp:1023-1077), minOfArr /
maxOfArr and oph::normalize (function.h:79-99, 188-196), and the pixel
coordinates of ophPointCloud::encodeHologram
(ophgen/src/ophPointCloud.cpp:191-240) — and the numpy oracle must agree
with them to rounding.

ophGen::encodeSideBand (ophgen/src/ophGen.cpp:1607-1695) transforms through
FFTW's own buffer, so the reference's output is well defined: its oracle
(oracle.sideband_encode) is pinned to the reference run itself
(tests/golden/sideband.npz).
"""
import math
import os

import numpy as np
import pytest


def _shift(a, nx, ny):
    out = [0j] * (nx * ny)
    hnx, hny = nx >> 1, ny >> 1
    for i in range(nx):
        for j in range(ny):
            ti, tj = i - hnx, j - hny
            if ti < 0:
                ti += nx
            if tj < 0:
                tj += ny
            out[ti + tj * nx] = a[i + j * nx]
    return out


def _dft2(a, nx, ny, sign):
    out = []
    for v in range(ny):
        for u in range(nx):
            s = 0j
            for y in range(ny):
                for x in range(nx):
                    s += a[x + y * nx] * complex(math.cos(sign * 2 * math.pi * (u * x / nx + v * y / ny)),
                                                 math.sin(sign * 2 * math.pi * (u * x / nx + v * y / ny)))
            out.append(s)
    return out


def _fft2(a, nx, ny, sign):
    return _shift(_dft2(_shift(a, nx, ny), nx, ny, sign), nx, ny)


def _literal_ssb(h, nx, ny, ppx, ppy, shift):
    t = _fft2(_fft2(h, nx, ny, -1), nx, ny, +1)
    ssx, ssy = nx * ppx, ny * ppy
    out = []
    for i in range(nx * ny):
        w, hh = i % nx, i // nx
        y = (ssy - ppy) - (ppy * hh)
        Y = (math.pi * y * shift[1]) / ppy
        x = -(ssx / 2) + ppx * w + ppx / 2
        X = (math.pi * x * shift[0]) / ppx
        c = math.cos(X) * math.cos(Y) - math.sin(X) * math.sin(Y)
        out.append(t[i].real * c)
    return out


def _literal_offssb(h, nx, ny, passband):
    a = _fft2(h, nx, ny, -1)
    shifted = [0j] * (nx * ny)
    for i in range(nx):
        for j in range(ny):
            tj = (j + 100) % ny
            shifted[i * ny + tj] = a[i * ny + j]
    tmp = _fft2(shifted, nx, ny, +1)
    spec = _fft2(tmp, nx, ny, -1)
    n, half_n, half_nx = nx * ny, (nx * ny) >> 1, nx >> 1
    if passband == 0:
        for r in range(ny):
            for k in range(half_nx):
                spec[r * nx + half_nx + k] = 0j
    elif passband == 1:
        for r in range(ny):
            for k in range(half_nx):
                spec[r * nx + k] = 0j
    elif passband == 2:
        for k in range(half_n):
            spec[half_n + k] = 0j
    else:
        for k in range(half_n):
            spec[k] = 0j
    re = [v.real for v in _fft2(spec, nx, ny, +1)]
    mn, mx = 1.7976931348623158e+308, 2.2250738585072014e-308
    for v in re:
        if v < mn:
            mn = v
        if v > mx:
            mx = v
    return [(v - mn) / (mx - mn) for v in re]


SIZES = [(6, 4), (5, 3), (4, 7)]


@pytest.mark.parametrize("nx,ny", SIZES)
def test_ssb_point_cloud_matches_the_code(oracle_mod, nx, ny):
    rng = np.random.default_rng(nx * 10 + ny)
    h = rng.normal(size=(2, ny, nx)) + 1j * rng.normal(size=(2, ny, nx))
    for shift in ((0.0, 0.5), (0.25, 0.75)):
        got = oracle_mod.ssb_encode(h, 8e-6, 6.4e-6, 7, spectrum_shift=shift)
        for ch in range(2):
            want = np.array(_literal_ssb(list(h[ch].reshape(-1)), nx, ny, 8e-6, 6.4e-6, shift)).reshape(ny, nx)
            assert np.allclose(got[ch], want, rtol=0, atol=1e-12 * np.abs(want).max())


@pytest.mark.parametrize("nx,ny", SIZES)
@pytest.mark.parametrize("passband", [0, 1, 2, 3])
def test_off_axis_ssb_matches_the_code(oracle_mod, nx, ny, passband):
    rng = np.random.default_rng(nx * 100 + ny * 10 + passband)
    h = rng.normal(size=(3, ny, nx)) + 1j * rng.normal(size=(3, ny, nx))
    got = oracle_mod.ssb_encode(h, 8e-6, 8e-6, 8, passband)
    want = np.array(_literal_offssb(list(h[0].reshape(-1)), nx, ny, passband)).reshape(ny, nx)
    for ch in range(3):   # channel 0's field, every channel
        assert np.allclose(got[ch], want, rtol=0, atol=1e-12)
    assert got.min() == 0.0 and got.max() == 1.0


def test_ssb_round_trip_is_the_field_times_n_for_even_sizes(oracle_mod):
    """For even sizes the two shifted transforms compose to N times the
    identity, so the SSB encoding is N Re(H) cos(X + Y)."""
    rng = np.random.default_rng(5)
    ny, nx = 24, 40
    h = rng.normal(size=(1, ny, nx)) + 1j * rng.normal(size=(1, ny, nx))
    got = oracle_mod.ssb_encode(h, 8e-6, 8e-6, 7)[0]
    y = (ny * 8e-6 - 8e-6) - 8e-6 * np.arange(ny)
    c = np.cos(np.pi * y * 0.5 / 8e-6)
    assert np.allclose(got, nx * ny * h[0].real * c[:, None], rtol=0, atol=1e-12 * np.abs(got).max())


GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _sideband_cases():
    z = np.load(os.path.join(GOLD, "sideband.npz"))
    names = sorted({k[:-len("_field")] for k in z.files if k.endswith("_field")})
    return z, names


def test_sideband_oracle_matches_reference(oracle_mod):
    """oracle.sideband_encode against the reference's own encodeSideBand
    (tests/golden/sideband.npz: ophGen.cpp:1607-1695 run from the reference
    build, FFTW replaced by an FP64 DFT), every passband, even, odd and
    mixed sizes."""
    z, names = _sideband_cases()
    assert len(names) == 3
    for name in names:
        pnx, pny, ppx, ppy = z[name + "_geom"]
        field = z[name + "_field"]
        for pb in range(4):
            want = z[f"{name}_enc{pb}"]
            got = oracle_mod.sideband_encode(field, float(ppx), float(ppy), pb)
            assert np.abs(got - want).max() <= 1e-13 * np.abs(want).max(), (name, pb)
