"""The phase encoder's FP64 values (m_lpEncoded = (atan2(im, re) + pi) / (2 pi),
ophgen/src/ophGen.cpp:1843-1853) against numpy's arctan2 on inputs chosen to
stress the table-driven atan2 of pc_encode.cu: every tabulated angle and the
midpoints between them, values just either side of the axes and of the
negative real axis (where the result jumps from 1 to 0), signed zeros,
subnormal, tiny and huge magnitudes (the inputs that take CUDA's atan2), and
random fields over twelve decades.

Bar: within 4 eps of numpy's value (the encoded value lies in [0, 1]; the
other encoder tests allow 8 eps), inside [0, 1], and the exact special
values of atan2 where the result is exactly 0, 0.5 or 1."""
import numpy as np
import pytest

from tests._util import code_agreement, run_encode

pytestmark = pytest.mark.gpu

EPS = np.finfo(np.float64).eps


def _want(z):
    return (np.arctan2(z.imag, z.real) + np.pi) / (2 * np.pi)


def _inputs():
    rng = np.random.default_rng(2024)
    parts = []
    k = np.arange(-128, 129)
    for off in (0.0, 0.5, 0.4999, -0.4999, 1e-9, -1e-9):
        th = (k + off) * np.pi / 128
        for r in (1.0, 3.7e-5, 2.9e4):
            parts.append(r * np.exp(1j * th))
    for s in (1e-17, 1e-12, 1e-6):
        for x in (-1.0, 1.0):
            parts.append(np.array([complex(x, s), complex(x, -s), complex(s, x), complex(-s, x)]))
    parts.append(np.array([complex(-2.0, 0.0), complex(-2.0, -0.0), complex(2.0, 0.0), complex(2.0, -0.0),
                           complex(0.0, 3.0), complex(-0.0, -3.0), complex(0.0, 0.0), complex(-0.0, 0.0),
                           complex(-0.0, -0.0), complex(5e-310, -7e-310), complex(-1e-300, 2e-300),
                           complex(3e300, -1e300), complex(1e19, 1e19), complex(-4.7e18, 1.0),
                           complex(1.0, -4.7e18), complex(2.2e-19, -2.2e-19)]))
    mag = 10.0 ** rng.uniform(-6, 6, 200_000)
    parts.append(mag * np.exp(1j * rng.uniform(-np.pi, np.pi, mag.size)))
    parts.append(rng.normal(size=100_000) + 1j * rng.normal(size=100_000))
    return np.concatenate([np.ravel(p) for p in parts])


def test_phase_values_match_atan2(gpu_ctx):
    z = _inputs()
    enc, codes = run_encode(gpu_ctx, z[None, :], 0)
    want = _want(z)
    err = np.abs(enc[0] - want)
    assert err.max() <= 4 * EPS, (err.max() / EPS, z[np.argmax(err)])
    assert enc.min() >= 0.0 and enc.max() <= 1.0
    # signed zeros and the axes, exactly
    special = ((complex(-2.0, 0.0), 1.0), (complex(-2.0, -0.0), 0.0), (complex(2.0, 0.0), 0.5),
               (complex(2.0, -0.0), 0.5), (complex(0.0, 0.0), 0.5), (complex(-0.0, 0.0), 1.0),
               (complex(-0.0, -0.0), 0.0))   # pairs, not a dict: -0.0 == 0.0 as a key
    for zz, v in special:
        i = np.flatnonzero((z.real == zz.real) & (z.imag == zz.imag)
                           & (np.signbit(z.real) == np.signbit(zz.real))
                           & (np.signbit(z.imag) == np.signbit(zz.imag)))
        assert i.size and np.all(enc[0, i] == v), zz
    # the codes follow from these values as the reference's normalize does
    mn, mx = want.min(), want.max()
    ref = (((want - mn) / (mx - mn)) * 255 + 0.5).astype(np.uint8)
    exact, maxd = code_agreement(codes, ref[None, :], circular=False)
    assert exact >= 0.9999 and maxd <= 1


def test_codes_of_normalize_match_the_division(gpu_ctx):
    """normalize's codes (a product with 255 / gap, the division where that
    product lies within 1e-12 of a code boundary) equal the reference's
    (uchar)(((v - min) / gap) * 255 + 0.5) on values that sit exactly on and
    just beside every code boundary."""
    import ctypes

    import torch

    import openholo_gb300 as oph
    lib = oph.lib()
    lib.ophpc_normalize.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint64,
                                    ctypes.c_void_p, ctypes.c_void_p]
    lib.ophpc_normalize.restype = ctypes.c_int
    rng = np.random.default_rng(5)
    for mn, mx in ((0.0, 1.0), (-3.25, 7.5), (1e-3, 1e-3 + 1e-9), (-1e200, 1e200)):
        gap = mx - mn
        b = (np.arange(256) - 0.5) / 255.0 * gap + mn           # (v - mn) / gap * 255 + 0.5 = integer
        vals = np.concatenate([[mn, mx], b, np.nextafter(b, np.inf), np.nextafter(b, -np.inf),
                               rng.uniform(mn, mx, 50_000)])
        vals = np.clip(vals, mn, mx)
        d = torch.from_numpy(vals).cuda()
        out = torch.empty(vals.size, dtype=torch.uint8, device="cuda")
        assert lib.ophpc_normalize(gpu_ctx._h, d.data_ptr(), 1, vals.size, out.data_ptr(), None) == 0
        torch.cuda.synchronize()
        with np.errstate(all="ignore"):
            v = ((vals - mn) / gap) * 255.0 + 0.5
        want = np.where((v >= 0) & (v < 256), np.floor(np.nan_to_num(v, nan=0.0)), 0).astype(np.uint8)
        assert np.array_equal(out.cpu().numpy(), want), (mn, mx)
