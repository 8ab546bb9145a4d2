"""Python bindings for the CPU oracle (test infrastructure only).

Two checkers live here:

* ``libophpc_oracle.so`` (built from ``ophpc_oracle.c``): the C restatement
  of Openholo's point-cloud CPU path. It always builds (gcc + OpenMP) and is
  what the GPU parity tests, ``smoke()`` and the CPU arm of ``bench.py`` use.
* ``_ref/libophref.so``: the reference's own CPU path compiled from the
  reference sources (``make -C oracle ref``). It exists only where the
  reference tree is present; it pins the restatement through the fixtures in
  ``tests/golden/`` that ``tests/golden/make_golden.py`` writes.

Nothing in the product package imports this module.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading
from dataclasses import dataclass, field
from typing import Optional, Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_LIB = os.path.join(HERE, "lib", "libophpc_oracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libophref.so")
# The reference's source tree: $OPHPC_REFERENCE_TREE, else a directory named
# "reference" beside this repository's checkout (where it is absent, e.g. on
# a machine that only runs the tests, the reference build is skipped).
REFERENCE_TREE = os.environ.get("OPHPC_REFERENCE_TREE") or \
    os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")

_lock = threading.Lock()
_ora = None
_ref = None


def build(with_reference: Optional[bool] = None, quiet: bool = True) -> None:
    """Compile the restatement (always) and the reference build (when the
    reference tree is present, or when ``with_reference`` is True)."""
    if with_reference is None:
        with_reference = os.path.isdir(os.path.join(REFERENCE_TREE, "ophgen", "src"))
    target = "ref" if with_reference else "all"
    cmd = ["make", "-C", HERE, "-j8", target, f"REF={REFERENCE_TREE}"]
    out = subprocess.run(cmd, capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{out.stdout}\n{out.stderr}")
    if not quiet:
        print(out.stdout)


class OracleConfig(ctypes.Structure):
    _fields_ = [
        ("pixel_number", ctypes.c_int32 * 2),
        ("offset", ctypes.c_int32 * 2),
        ("pixel_pitch", ctypes.c_double * 2),
        ("scale", ctypes.c_double * 3),
        ("distance", ctypes.c_double),
        ("field_length", ctypes.c_double),
        ("viewing_window", ctypes.c_int32),
        ("n_channels", ctypes.c_int32),
        ("wave_length", ctypes.c_double * 3),
    ]


@dataclass
class Geometry:
    """One hologram job's geometry: the OphConfig/OphPointCloudConfig fields
    the point-cloud path reads."""
    pnx: int
    pny: int
    ppx: float
    ppy: float
    wavelengths: Sequence[float]
    scale: Sequence[float] = (1.0, 1.0, 1.0)
    distance: float = 0.0
    offset: Sequence[int] = (0, 0)
    field_length: float = 0.0
    viewing_window: bool = False
    extra_xml: dict = field(default_factory=dict)

    @property
    def n_channels(self) -> int:
        return len(self.wavelengths)

    def to_c(self) -> OracleConfig:
        c = OracleConfig()
        c.pixel_number[0], c.pixel_number[1] = self.pnx, self.pny
        c.offset[0], c.offset[1] = int(self.offset[0]), int(self.offset[1])
        c.pixel_pitch[0], c.pixel_pitch[1] = self.ppx, self.ppy
        for i in range(3):
            c.scale[i] = float(self.scale[i])
        c.distance = float(self.distance)
        c.field_length = float(self.field_length)
        c.viewing_window = 1 if self.viewing_window else 0
        c.n_channels = len(self.wavelengths)
        for i, w in enumerate(self.wavelengths):
            c.wave_length[i] = float(w)
        return c

    def xml(self) -> str:
        """The flat <PointCloud> config the reference's readConfig parses
        (ophgen/src/ophGen.cpp:221-358, ophgen/src/ophPointCloud.cpp:83-149)."""
        lines = ["<PointCloud>"]
        lines.append(f"  <ScaleX>{self.scale[0]!r}</ScaleX>")
        lines.append(f"  <ScaleY>{self.scale[1]!r}</ScaleY>")
        lines.append(f"  <ScaleZ>{self.scale[2]!r}</ScaleZ>")
        lines.append(f"  <Distance>{self.distance!r}</Distance>")
        lines.append(f"  <FieldLength>{self.field_length!r}</FieldLength>")
        lines.append(f"  <SLM_PixelPitchX>{self.ppx!r}</SLM_PixelPitchX>")
        lines.append(f"  <SLM_PixelPitchY>{self.ppy!r}</SLM_PixelPitchY>")
        lines.append(f"  <SLM_PixelNumX>{self.pnx}</SLM_PixelNumX>")
        lines.append(f"  <SLM_PixelNumY>{self.pny}</SLM_PixelNumY>")
        lines.append(f"  <SLM_WaveNum>{len(self.wavelengths)}</SLM_WaveNum>")
        for i, w in enumerate(self.wavelengths):
            lines.append(f"  <SLM_WaveLength_{i + 1}>{float(w)!r}</SLM_WaveLength_{i + 1}>")
        for k, v in self.extra_xml.items():
            lines.append(f"  <{k}>{v}</{k}>")
        lines.append("</PointCloud>")
        return "\n".join(lines) + "\n"


def _p(a: np.ndarray, t=ctypes.c_double):
    return a.ctypes.data_as(ctypes.POINTER(t))


def _load_oracle():
    global _ora
    with _lock:
        if _ora is None:
            if not os.path.exists(ORACLE_LIB):
                build(with_reference=False)
            lib = ctypes.CDLL(ORACLE_LIB)
            lib.oracle_generate.argtypes = [ctypes.POINTER(OracleConfig), ctypes.POINTER(ctypes.c_double),
                                            ctypes.c_int64, ctypes.c_int32, ctypes.POINTER(ctypes.c_double)]
            lib.oracle_generate.restype = ctypes.c_int
            lib.oracle_field_at.argtypes = [ctypes.POINTER(OracleConfig), ctypes.POINTER(ctypes.c_double),
                                            ctypes.c_int64, ctypes.c_int32, ctypes.c_int32,
                                            ctypes.POINTER(ctypes.c_int64), ctypes.c_int64,
                                            ctypes.POINTER(ctypes.c_double)]
            lib.oracle_field_at.restype = ctypes.c_int
            lib.oracle_encode.argtypes = [ctypes.POINTER(ctypes.c_double), ctypes.c_int64, ctypes.c_int32,
                                          ctypes.POINTER(ctypes.c_double)]
            lib.oracle_encode.restype = ctypes.c_int
            lib.oracle_normalize.argtypes = [ctypes.POINTER(ctypes.c_double), ctypes.c_int32, ctypes.c_int64,
                                             ctypes.POINTER(ctypes.c_uint8), ctypes.POINTER(ctypes.c_double),
                                             ctypes.POINTER(ctypes.c_double)]
            lib.oracle_normalize.restype = None
            lib.oracle_wrp_zmax.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.c_int64]
            lib.oracle_wrp_zmax.restype = ctypes.c_double
            lib.oracle_wrp_plane.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.c_int64,
                                             ctypes.c_int32, ctypes.POINTER(ctypes.c_double)]
            lib.oracle_wrp_plane.restype = ctypes.c_int
            _ora = lib
    return _ora


def _vertices(v: np.ndarray) -> np.ndarray:
    v = np.ascontiguousarray(v, dtype=np.float64)
    if v.ndim != 2 or v.shape[1] != 7:
        raise ValueError("vertices must be an (n, 7) float64 array: pos[3], color[3], phase")
    return v


def generate(geom: Geometry, vertices: np.ndarray, diff_flag: int) -> np.ndarray:
    """Full complex field [n_channels, pny, pnx] (complex128)."""
    lib = _load_oracle()
    v = _vertices(vertices)
    out = np.empty((geom.n_channels, geom.pny, geom.pnx, 2), dtype=np.float64)
    c = geom.to_c()
    rc = lib.oracle_generate(ctypes.byref(c), _p(v), v.shape[0], diff_flag, _p(out))
    if rc != 0:
        raise ValueError("oracle_generate rejected its arguments")
    return out[..., 0] + 1j * out[..., 1]


def field_at(geom: Geometry, vertices: np.ndarray, diff_flag: int, channel: int,
             pixel_index: np.ndarray) -> np.ndarray:
    """Complex field of one channel at flat pixel indices (y*pnx + x)."""
    lib = _load_oracle()
    v = _vertices(vertices)
    idx = np.ascontiguousarray(pixel_index, dtype=np.int64)
    out = np.empty((idx.shape[0], 2), dtype=np.float64)
    c = geom.to_c()
    rc = lib.oracle_field_at(ctypes.byref(c), _p(v), v.shape[0], diff_flag, channel,
                             _p(idx, ctypes.c_int64), idx.shape[0], _p(out))
    if rc != 0:
        raise ValueError("oracle_field_at rejected its arguments")
    return out[:, 0] + 1j * out[:, 1]


def encode(field: np.ndarray, encode_flag: int, prior: Optional[np.ndarray] = None) -> np.ndarray:
    """field: [n_channels, ...] complex (or one channel). Each channel is
    encoded on its own, as ophGen::encoding does; entries an encoder leaves
    alone (Burckhardt, TwoPhase) keep `prior` (zeros by default)."""
    lib = _load_oracle()
    f = np.ascontiguousarray(field, dtype=np.complex128)
    chans = f.reshape(f.shape[0], -1) if f.ndim > 2 else f.reshape(1, -1)
    out = np.zeros(chans.shape, dtype=np.float64) if prior is None else \
        np.ascontiguousarray(prior, dtype=np.float64).reshape(chans.shape).copy()
    for c in range(chans.shape[0]):
        flat = np.ascontiguousarray(chans[c]).view(np.float64)
        oc = np.ascontiguousarray(out[c])
        if lib.oracle_encode(_p(flat), chans.shape[1], encode_flag, _p(oc)) != 0:
            raise ValueError("oracle_encode rejected its arguments")
        out[c] = oc
    return out.reshape(f.shape)


def normalize(encoded: np.ndarray):
    """encoded: [n_channels, ...]; returns (uint8 codes, min, max)."""
    lib = _load_oracle()
    e = np.ascontiguousarray(encoded, dtype=np.float64)
    nch = e.shape[0]
    per = e.size // nch
    out = np.empty(e.shape, dtype=np.uint8)
    mn, mx = ctypes.c_double(), ctypes.c_double()
    lib.oracle_normalize(_p(e), nch, per, _p(out, ctypes.c_uint8), ctypes.byref(mn), ctypes.byref(mx))
    return out, mn.value, mx.value


# ---------------------------------------------------------------- WRP

class OracleWrpConfig(ctypes.Structure):
    _fields_ = [
        ("pixel_number", ctypes.c_int32 * 2),
        ("pixel_pitch", ctypes.c_double * 2),
        ("scale", ctypes.c_double * 3),
        ("wrp_location", ctypes.c_double),
        ("propagation_distance", ctypes.c_double),
        ("n_channels", ctypes.c_int32),
        ("wave_length", ctypes.c_double * 3),
    ]


@dataclass
class WrpGeometry:
    """ophWRP's configuration (ophgen/src/ophGen.h:643-660 + the SLM keys of
    OphConfig): the <WRP> config file's fields the generator reads."""
    pnx: int
    pny: int
    ppx: float
    ppy: float
    wavelengths: Sequence[float]
    scale: Sequence[float] = (1.0, 1.0, 1.0)
    wrp_location: float = 0.0
    distance: float = 0.0

    def to_c(self) -> OracleWrpConfig:
        c = OracleWrpConfig()
        c.pixel_number[0], c.pixel_number[1] = self.pnx, self.pny
        c.pixel_pitch[0], c.pixel_pitch[1] = self.ppx, self.ppy
        for i in range(3):
            c.scale[i] = float(self.scale[i])
        c.wrp_location = float(self.wrp_location)
        c.propagation_distance = float(self.distance)
        c.n_channels = len(self.wavelengths)
        for i, w in enumerate(self.wavelengths):
            c.wave_length[i] = float(w)
        return c

    def xml(self) -> str:
        """The <WRP> config file ophWRP::readConfig parses
        (ophgen/src/ophWRP.cpp:137-213 and ophGen::readConfig)."""
        keys = [("FieldLength", 1.0), ("ScaleX", self.scale[0]), ("ScaleY", self.scale[1]),
                ("ScaleZ", self.scale[2]), ("Distance", self.distance), ("LocationOfWRP", self.wrp_location),
                ("NumOfWRP", 1), ("SLM_PixelPitchX", self.ppx), ("SLM_PixelPitchY", self.ppy),
                ("SLM_PixelNumX", self.pnx), ("SLM_PixelNumY", self.pny), ("SLM_WaveNum", len(self.wavelengths))]
        keys += [(f"SLM_WaveLength_{i + 1}", float(w)) for i, w in enumerate(self.wavelengths)]
        return "<WRP>\n" + "".join(f"  <{k}>{v!r}</{k}>\n" for k, v in keys) + "</WRP>\n"


def wrp_zmax(geom: WrpGeometry, vertices: np.ndarray) -> float:
    lib = _load_oracle()
    v = _vertices(vertices)
    c = geom.to_c()
    return float(lib.oracle_wrp_zmax(ctypes.byref(c), _p(v), v.shape[0]))


def wrp_plane(geom: WrpGeometry, vertices: np.ndarray, channel: int) -> np.ndarray:
    """One channel's WRP plane (calculateWRPCPU's splat, RandomPhase off),
    complex128 [pnY, pnX] (oracle/ophpc_oracle_wrp.c)."""
    lib = _load_oracle()
    v = _vertices(vertices)
    out = np.empty((geom.pny, geom.pnx, 2), dtype=np.float64)
    c = geom.to_c()
    if lib.oracle_wrp_plane(ctypes.byref(c), _p(v), v.shape[0], channel, _p(out)) != 0:
        raise ValueError("oracle_wrp_plane rejected its arguments")
    return out[..., 0] + 1j * out[..., 1]


def wrp_propagate(plane: np.ndarray, geom: WrpGeometry, wavelength: float) -> np.ndarray:
    """Angular-spectrum propagation of a WRP plane by geom.distance, the
    transform ophGen::Fresnel_FFT (ophgen/src/ophGen.cpp:516-580) intends:
    the plane at the centre (pnY/2, pnX/2) of a zero (2 pnY) x (2 pnX)
    buffer; F = fftshift(FFT2(fftshift(buffer))) (Openholo::fft2 with its
    fftShift, Openholo/src/Openholo.cpp:698-774; fftShift equals numpy's
    fftshift for even sizes); F *= exp(i 2 pi d sqrt(1/lambda^2 - fx^2 -
    fy^2)) with fx = (j - pnX) / (2 ssX), fy = (i - pnY) / (2 ssY);
    buffer = fftshift(IFFT2(fftshift(F))) unnormalised (FFTW's backward
    transform: numpy's ifft2 times the size); the centre block is the
    hologram. The reference runs the shifts in place on an aliased buffer,
    which scrambles its result; this restatement computes what its code
    describes, in FP64 (numpy.fft, pocketfft)."""
    pny, pnx = plane.shape
    hy, hx = pny >> 1, pnx >> 1
    buf = np.zeros((2 * pny, 2 * pnx), dtype=np.complex128)
    buf[hy:hy + pny, hx:hx + pnx] = plane
    f = np.fft.fftshift(np.fft.fft2(np.fft.fftshift(buf)))
    ssx, ssy = pnx * geom.ppx, pny * geom.ppy
    fx = ((np.arange(2 * pnx) - pnx) / (2 * ssx)) ** 2
    fy = ((np.arange(2 * pny) - pny) / (2 * ssy)) ** 2
    sq = np.sqrt(1.0 / (wavelength * wavelength) - fx[None, :] - fy[:, None])
    f *= np.exp(1j * (2 * np.pi * geom.distance) * sq)
    out = np.fft.fftshift(np.fft.ifft2(np.fft.fftshift(f))) * (4 * pnx * pny)
    return out[hy:hy + pny, hx:hx + pnx]


def oph_shift(a: np.ndarray) -> np.ndarray:
    """Openholo::fftShift (Openholo/src/Openholo.cpp:749-767) of a [ny][nx]
    array: out[(i - nx/2) mod nx, (j - ny/2) mod ny] = in[i, j] (numpy's
    ifftshift; fftshift too for even sizes)."""
    ny, nx = a.shape
    return np.roll(a, (-(ny >> 1), -(nx >> 1)), axis=(0, 1))


def oph_fft2(a: np.ndarray, inverse: bool) -> np.ndarray:
    """Openholo::fft2(src, dst, nx, ny, type) with its default shift
    (Openholo/src/Openholo.cpp:698-745): shift, FFTW's unnormalised forward
    (e^-) or backward (e^+) transform, shift."""
    s = oph_shift(a)
    t = np.fft.ifft2(s) * s.size if inverse else np.fft.fft2(s)
    return oph_shift(t)


_MAX_DOUBLE = 1.7976931348623158e+308
_MIN_DOUBLE = 2.2250738585072014e-308


def ssb_encode(field: np.ndarray, ppx: float, ppy: float, encode_flag: int, passband: int = 0,
               spectrum_shift=(0.0, 0.5)) -> np.ndarray:
    """m_lpEncoded of ophPointCloud::encoding(ENCODE_SSB | ENCODE_OFFSSB,
    passband) for field [n_channels, pnY, pnX] complex, FP64, as the
    reference's code describes (its FFTW input aliases the array it shifts,
    so its own runs cannot pin this):

    * ENCODE_SSB (7): ophPointCloud::encodeHologram
      (ophgen/src/ophPointCloud.cpp:191-240) per channel: T = B(F(H)), then
      Re(T) cos(X + Y) at x = -ssX/2 + ppX w + ppX/2, y = (ssY - ppY) - ppY h,
      X = pi x sx / ppX, Y = pi y sy / ppY, in the reference's order of
      operations;
    * ENCODE_OFFSSB (8): ophGen::encoding(flag, passband)
      (ophgen/src/ophGen.cpp:882-921) on complex_H[0] for every channel:
      freqShift(0, 100) (:1079-1098; circShift over the x-major view,
      Openholo/src/function.h:273-283), singleSideBand (:1023-1077: one half
      of the shifted spectrum zeroed), the real part and oph::normalize to
      [0, 1] (function.h:79-99, 188-196).
    """
    nch, pny, pnx = field.shape
    if encode_flag == 7:
        w = np.arange(pnx, dtype=np.float64)
        h = np.arange(pny, dtype=np.float64)
        ssx, ssy = pnx * ppx, pny * ppy
        y = (ssy - ppy) - ppy * h
        Y = (np.pi * y * spectrum_shift[1]) / ppy
        x = (-(ssx / 2) + ppx * w) + ppx / 2
        X = (np.pi * x * spectrum_shift[0]) / ppx
        c = np.cos(X)[None, :] * np.cos(Y)[:, None] - np.sin(X)[None, :] * np.sin(Y)[:, None]
        out = np.empty((nch, pny, pnx))
        for ch in range(nch):
            t = oph_fft2(oph_fft2(field[ch], False), True)
            out[ch] = t.real * c - t.imag * 0.0
        return out
    if encode_flag != 8:
        raise ValueError("encode_flag must be 7 (SSB) or 8 (OFFSSB)")
    a = oph_fft2(field[0], False)
    shifted = np.roll(a.reshape(pnx, pny), 100, axis=1).reshape(pny, pnx)
    tmp = oph_fft2(shifted, True)
    spec = oph_fft2(tmp, False)
    flat = spec.reshape(-1)
    hx, half = pnx >> 1, flat.size >> 1
    if passband == 0:
        spec[:, hx:2 * hx] = 0
    elif passband == 1:
        spec[:, :hx] = 0
    elif passband == 2:
        flat[half:2 * half] = 0
    else:
        flat[:half] = 0
    re = oph_fft2(spec, True).real
    ok = re[~np.isnan(re)]
    mn = min(_MAX_DOUBLE, ok.min()) if ok.size else _MAX_DOUBLE
    mx = max(_MIN_DOUBLE, ok.max()) if ok.size else _MIN_DOUBLE
    enc = (re - mn) / (mx - mn)
    return np.stack([enc] * nch)


def sideband_encode(field: np.ndarray, ppx: float, ppy: float, passband: int) -> np.ndarray:
    """m_lpEncoded of ophGen::encodeSideBand(passband)
    (ophgen/src/ophGen.cpp:1607-1653 with encodeSideBand_CPU, :1655-1695,
    and getShiftPhaseValue, :1741-1781) for field [n_channels, pnY, pnX]:
    per channel the field cropped to the central half along one axis
    (1-based bounds c1 = h - floor(h/2), c2 = c1 + h - 1, h = floor(n/2),
    made 0-based), B = S IFFT S normalised by N, times the carrier
    e^{i theta} — TOP / BOTTOM: theta = +-2 pi yy / (4 ppY), yy = ssY/2 -
    ppY r - ppY; LEFT / RIGHT: theta = -+2 pi xx / (4 ppX), xx = -ssX/2 -
    ppX c - ppX — and the real part. Pinned to the reference's own output
    (tests/golden/sideband.npz)."""
    nch, pny, pnx = field.shape
    if passband in (2, 3):
        h = pny // 2
        y1 = h - h // 2 - 1
        rows, cols = slice(y1, y1 + h), slice(0, pnx)
    else:
        h = pnx // 2
        x1 = h - h // 2 - 1
        rows, cols = slice(0, pny), slice(x1, x1 + h)
    ssx, ssy = pnx * ppx, pny * ppy
    r = np.arange(pny, dtype=np.float64)[:, None]
    c = np.arange(pnx, dtype=np.float64)[None, :]
    if passband in (2, 3):
        yy = (ssy / 2.0) - ppy * r - ppy
        theta = 2 * np.pi * ((yy if passband == 2 else -yy) / (4 * ppy)) + 0.0 * c
    else:
        xx = (-ssx / 2.0) - ppx * c - ppx
        theta = 2 * np.pi * ((-xx if passband == 0 else xx) / (4 * ppx)) + 0.0 * r
    cs, sn = np.cos(theta), np.sin(theta)
    out = np.empty((nch, pny, pnx))
    n = pnx * pny
    for ch in range(nch):
        crop = np.zeros((pny, pnx), dtype=np.complex128)
        crop[rows, cols] = field[ch][rows, cols]
        s = oph_shift(crop)
        t = oph_shift((np.fft.ifft2(s) * n) / n)
        out[ch] = t.real * cs - t.imag * sn
    return out


def wrp_generate(geom: WrpGeometry, vertices: np.ndarray) -> np.ndarray:
    """ophWRP::generateHologram restated: per channel the splat, then the
    propagation; complex128 [n_channels, pnY, pnX]."""
    return np.stack([wrp_propagate(wrp_plane(geom, vertices, c), geom, w) for c, w in enumerate(geom.wavelengths)])


REF_WRP_LIB = os.path.join(HERE, "_ref", "libophref_wrp.so")
REF_SIDEBAND_LIB = os.path.join(HERE, "_ref", "libophref_sideband.so")


def ref_sideband_available() -> bool:
    return os.path.exists(REF_SIDEBAND_LIB)


def ref_sideband(xml_path: str, field: np.ndarray, passband: int) -> np.ndarray:
    """The reference's own ophGen::encodeSideBand on field [n_channels,
    pnY, pnX] (oracle/ref_sideband_driver.cpp; FFTW replaced by the FP64 DFT
    of oracle/ref_dft_stubs.c): m_lpEncoded, float64 [n_channels, pnY, pnX]."""
    lib = ctypes.CDLL(REF_SIDEBAND_LIB)
    lib.ophref_sideband.argtypes = [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_uint, ctypes.c_void_p, ctypes.c_int]
    lib.ophref_sideband.restype = ctypes.c_int
    nch = field.shape[0]
    f = np.ascontiguousarray(field, dtype=np.complex128)
    out = np.zeros(field.shape, dtype=np.float64)
    with _QuietStdout():
        rc = lib.ophref_sideband(xml_path.encode(), f.ctypes.data, passband, out.ctypes.data, nch)
    if rc != nch:
        raise RuntimeError(f"ophref_sideband failed ({rc})")
    return out


def ref_wrp_available() -> bool:
    return os.path.exists(REF_WRP_LIB)


def ref_wrp_planes(xml_path: str, vertices: np.ndarray, n_channels: int, pnx: int, pny: int) -> np.ndarray:
    """The reference's own WRP splat planes (oracle/ref_wrp_driver.cpp),
    complex128 [n_channels, pnY, pnX]."""
    lib = ctypes.CDLL(REF_WRP_LIB)
    lib.ophref_wrp_planes.argtypes = [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_ulonglong, ctypes.c_void_p,
                                      ctypes.c_int]
    lib.ophref_wrp_planes.restype = ctypes.c_int
    v = _vertices(vertices)
    out = np.zeros((n_channels, pny, pnx, 2), dtype=np.float64)
    with _QuietStdout():
        rc = lib.ophref_wrp_planes(xml_path.encode(), v.ctypes.data, v.shape[0], out.ctypes.data, n_channels)
    if rc != n_channels:
        raise RuntimeError(f"ophref_wrp_planes failed ({rc})")
    return out[..., 0] + 1j * out[..., 1]


# ---------------------------------------------------------------- reference

def ref_available() -> bool:
    return os.path.exists(REF_LIB)


def _load_ref():
    global _ref
    with _lock:
        if _ref is None:
            if not os.path.exists(REF_LIB):
                raise FileNotFoundError("oracle/_ref/libophref.so is not built (make -C oracle ref)")
            lib = ctypes.CDLL(REF_LIB)
            lib.ophref_run.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_void_p, ctypes.c_ulonglong,
                                       ctypes.c_int, ctypes.c_uint, ctypes.c_uint,
                                       ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
            lib.ophref_run.restype = ctypes.c_int
            lib.ophref_query.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_int),
                                         ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]
            lib.ophref_query.restype = ctypes.c_int
            lib.ophref_run_save.argtypes = [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_ulonglong, ctypes.c_uint,
                                            ctypes.c_uint, ctypes.c_char_p, ctypes.c_int]
            lib.ophref_run_save.restype = ctypes.c_int
            lib.ophref_run_save_ohc.argtypes = [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_ulonglong, ctypes.c_uint,
                                                ctypes.c_char_p]
            lib.ophref_run_save_ohc.restype = ctypes.c_int
            lib.ophref_load_ohc.argtypes = [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                            ctypes.c_void_p, ctypes.c_ulonglong]
            lib.ophref_load_ohc.restype = ctypes.c_int
            lib.ophref_encode_field.argtypes = [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_uint,
                                                ctypes.c_void_p, ctypes.c_void_p]
            lib.ophref_encode_field.restype = ctypes.c_int
            lib.ophref_load_ply.argtypes = [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_ulonglong]
            lib.ophref_load_ply.restype = ctypes.c_longlong
            _ref = lib
    return _ref


class _QuietStdout:
    """Silences the reference's printf logging (LOG, Openholo/src/sys.h) by
    pointing file descriptor 1 at /dev/null for the duration of a call."""

    def __enter__(self):
        import sys
        sys.stdout.flush()
        self._libc = ctypes.CDLL(None)
        self._saved = os.dup(1)
        self._null = os.open(os.devnull, os.O_WRONLY)
        os.dup2(self._null, 1)
        return self

    def __exit__(self, *a):
        self._libc.fflush(None)
        os.dup2(self._saved, 1)
        os.close(self._saved)
        os.close(self._null)


def ref_load_ply(path: str) -> np.ndarray:
    lib = _load_ref()
    with _QuietStdout():
        n = lib.ophref_load_ply(path.encode(), None, 0)
    if n < 0:
        raise ValueError(f"reference PLYparser failed on {path}")
    out = np.zeros((n, 7), dtype=np.float64)
    with _QuietStdout():
        lib.ophref_load_ply(path.encode(), out.ctypes.data, n)
    return out


def ref_run_save(xml_path: str, vertices: np.ndarray, diff_flag: int, encode_flag: int, bmp_path: str,
                 bits_per_pixel: int = 8) -> None:
    """Reference generate -> encoding -> normalize -> save(bmp_path)."""
    lib = _load_ref()
    v = _vertices(vertices)
    with _QuietStdout():
        rc = lib.ophref_run_save(xml_path.encode(), v.ctypes.data, v.shape[0], diff_flag, encode_flag,
                                 bmp_path.encode(), bits_per_pixel)
    if rc != 0:
        raise RuntimeError(f"ophref_run_save failed ({rc})")


def ref_run_save_ohc(xml_path: str, vertices: np.ndarray, diff_flag: int, ohc_path: str) -> None:
    """Reference generate -> saveAsOhc(ohc_path)."""
    lib = _load_ref()
    v = _vertices(vertices)
    with _QuietStdout():
        rc = lib.ophref_run_save_ohc(xml_path.encode(), v.ctypes.data, v.shape[0], diff_flag, ohc_path.encode())
    if rc != 0:
        raise RuntimeError(f"ophref_run_save_ohc failed ({rc})")


def ref_encode_field(xml_path: str, field: np.ndarray, encode_flag: int, pre_flag: int = -1):
    """Reference encoding(encode_flag) + normalize of a given field
    ([n_channels, pnY, pnX] complex; shape from the config) ->
    (encoded [n_channels, pnY, pnX], codes uint8)."""
    lib = _load_ref()
    f = np.ascontiguousarray(field, dtype=np.complex128)
    enc = np.zeros(f.shape, dtype=np.float64)
    codes = np.zeros(f.shape, dtype=np.uint8)
    with _QuietStdout():
        rc = lib.ophref_encode_field(xml_path.encode(), f.ctypes.data, pre_flag, encode_flag, enc.ctypes.data,
                                     codes.ctypes.data)
    if rc != 0:
        raise RuntimeError(f"ophref_encode_field failed ({rc})")
    return enc, codes


def ref_load_ohc(ohc_path: str):
    """Reference loadAsOhc -> (field [ch, pnY, pnX] complex, pitch[2], wavelengths[ch])."""
    lib = _load_ref()
    shape = np.zeros(3, dtype=np.int32)
    pitch = np.zeros(2)
    wl = np.zeros(3)
    with _QuietStdout():
        rc = lib.ophref_load_ohc(ohc_path.encode(), shape.ctypes.data, pitch.ctypes.data, wl.ctypes.data, None, 0)
    if rc != 0:
        raise RuntimeError(f"ophref_load_ohc failed ({rc})")
    pnx, pny, nch = (int(x) for x in shape)
    buf = np.zeros(2 * pnx * pny * nch)
    with _QuietStdout():
        rc = lib.ophref_load_ohc(ohc_path.encode(), shape.ctypes.data, pitch.ctypes.data, wl.ctypes.data,
                                 buf.ctypes.data, buf.size)
    if rc != 0:
        raise RuntimeError(f"ophref_load_ohc failed ({rc})")
    f = buf.reshape(nch, pny, pnx, 2)
    return f[..., 0] + 1j * f[..., 1], pitch, wl[:nch]


def ref_run(xml_path: str, vertices: Optional[np.ndarray] = None, ply_path: Optional[str] = None,
            diff_flag: int = 0, encode_flag: int = 0, viewing_window: bool = False):
    """Run the reference CPU path; returns (field, encoded, normalized, seconds).
    encode_flag 2 encodes the same field as phase and then amplitude and
    returns both stacked on a leading axis."""
    lib = _load_ref()
    pnx, pny, nch = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    with _QuietStdout():
        q = lib.ophref_query(xml_path.encode(), ctypes.byref(pnx), ctypes.byref(pny), ctypes.byref(nch))
    if q != 0:
        raise ValueError(f"reference readConfig failed on {xml_path}")
    shape = (nch.value, pny.value, pnx.value)
    field = np.zeros(shape + (2,), dtype=np.float64)
    n_enc = 2 if encode_flag == 2 else 1
    enc = np.zeros((n_enc,) + shape, dtype=np.float64)
    nrm = np.zeros((n_enc,) + shape, dtype=np.uint8)
    secs = ctypes.c_double()
    v = None
    n = 0
    if ply_path is None:
        v = _vertices(vertices)
        n = v.shape[0]
    with _QuietStdout():
        rc = lib.ophref_run(xml_path.encode(), ply_path.encode() if ply_path else None,
                            v.ctypes.data if v is not None else None, n, 1 if viewing_window else 0,
                            diff_flag, encode_flag, field.ctypes.data, enc.ctypes.data, nrm.ctypes.data,
                            ctypes.byref(secs))
    if rc != 0:
        raise RuntimeError(f"ophref_run failed ({rc})")
    if n_enc == 1:
        enc, nrm = enc[0], nrm[0]
    return field[..., 0] + 1j * field[..., 1], enc, nrm, secs.value
