"""Python mirror of the reference's ophPointCloud API over libophpc.

``PointCloud`` wraps one ophPointCloud façade object (include/ophPointCloud.h)
through its C ABI (include/ophpc_pointcloud.h); method names and argument
meanings are the reference's (ophgen/src/ophPointCloud.h:547-698):

    h = PointCloud()
    h.readConfig("PointCloud.xml")
    h.loadPointCloud("cloud.ply")          # or h.setPointCloudModel(vertices)
    h.SetMode(MODE_GPU)
    h.generateHologram(PC_DIFF_RS)
    h.encoding(ENCODE_PHASE)
    h.normalize()
    h.save("hologram.bmp")
    h.release()

The file helpers read_config / load_ply / save_bmp / save_ohc / load_ohc bind
include/ophpc_io.h.
"""
from __future__ import annotations

import ctypes
from typing import Optional, Tuple

import numpy as np

from ._abi import OphpcConfig, OphpcError, lib

PC_DIFF_RS = 0
PC_DIFF_FRESNEL = 1
ENCODE_PHASE, ENCODE_AMPLITUDE, ENCODE_REAL, ENCODE_IMAGINARY = 0, 1, 2, 3
ENCODE_SIMPLENI, ENCODE_BURCKHARDT, ENCODE_TWOPHASE = 4, 5, 6


class ImageConfig(ctypes.Structure):
    _fields_ = [
        ("rotate", ctypes.c_int32), ("merge", ctypes.c_int32), ("flip", ctypes.c_int32),
        ("double_precision", ctypes.c_int32), ("shift", ctypes.c_double * 3),
        ("random_phase", ctypes.c_int32), ("num_of_stream", ctypes.c_int32),
    ]


_declared = False


def _L():
    global _declared
    L = lib()
    if not _declared:
        vp, u32, u64, i32, d = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int32, ctypes.c_double
        L.ophpc_read_config.argtypes = [ctypes.c_char_p, ctypes.POINTER(OphpcConfig), ctypes.POINTER(ImageConfig)]
        L.ophpc_read_config.restype = ctypes.c_int
        L.ophpc_load_ply.argtypes = [ctypes.c_char_p, vp, u64]
        L.ophpc_load_ply.restype = ctypes.c_int64
        L.ophpc_save_bmp.argtypes = [ctypes.c_char_p, vp, i32, i32, i32, i32, i32]
        L.ophpc_save_bmp.restype = ctypes.c_int
        L.ophpc_save_ohc.argtypes = [ctypes.c_char_p, vp, i32, i32, d, d, u32, vp]
        L.ophpc_save_ohc.restype = ctypes.c_int
        L.ophpc_load_ohc.argtypes = [ctypes.c_char_p, vp, vp, vp, vp, vp, vp, vp, u64]
        L.ophpc_load_ohc.restype = ctypes.c_int
        L.ophpc_pc_save_ohc.argtypes = [vp, ctypes.c_char_p]
        L.ophpc_pc_save_ohc.restype = i32
        L.ophpc_pc_load_ohc.argtypes = [vp, ctypes.c_char_p]
        L.ophpc_pc_load_ohc.restype = i32
        L.ophpc_normalize.argtypes = [vp, vp, u32, u64, vp, vp]
        L.ophpc_normalize.restype = ctypes.c_int
        L.ophpc_pc_create.restype = vp
        L.ophpc_pc_release.argtypes = [vp]
        L.ophpc_pc_read_config.argtypes = [vp, ctypes.c_char_p]
        L.ophpc_pc_read_config.restype = i32
        L.ophpc_pc_load_point_cloud.argtypes = [vp, ctypes.c_char_p]
        L.ophpc_pc_load_point_cloud.restype = ctypes.c_int64
        L.ophpc_pc_set_point_cloud.argtypes = [vp, vp, u64]
        L.ophpc_pc_set_mode.argtypes = [vp, u32]
        L.ophpc_pc_set_viewing_window.argtypes = [vp, i32]
        L.ophpc_pc_set_scale.argtypes = [vp, d, d, d]
        L.ophpc_pc_set_distance.argtypes = [vp, d]
        L.ophpc_pc_set_offset.argtypes = [vp, i32, i32]
        L.ophpc_pc_generate_hologram.argtypes = [vp, u32]
        L.ophpc_pc_generate_hologram.restype = d
        L.ophpc_pc_encoding.argtypes = [vp, u32]
        L.ophpc_pc_encoding_passband.argtypes = [vp, u32, u32]
        L.ophpc_pc_normalize.argtypes = [vp]
        L.ophpc_pc_save.argtypes = [vp, ctypes.c_char_p, ctypes.c_uint8]
        L.ophpc_pc_save.restype = i32
        L.ophpc_pc_get_config.argtypes = [vp, ctypes.POINTER(OphpcConfig)]
        L.ophpc_pc_get_config.restype = i32
        L.ophpc_pc_number_of_points.argtypes = [vp]
        L.ophpc_pc_number_of_points.restype = u64
        L.ophpc_pc_point_cloud.argtypes = [vp]
        L.ophpc_pc_point_cloud.restype = vp
        L.ophpc_pc_complex_field.argtypes = [vp, u32]
        L.ophpc_pc_complex_field.restype = vp
        L.ophpc_pc_encoded.argtypes = [vp, u32]
        L.ophpc_pc_encoded.restype = vp
        L.ophpc_pc_normalized.argtypes = [vp, u32]
        L.ophpc_pc_normalized.restype = vp
        L.ophpc_pc_last_error.argtypes = [vp]
        L.ophpc_pc_last_error.restype = ctypes.c_char_p
        _declared = True
    return L


# ------------------------------------------------------------------ files

def read_config(path: str) -> Tuple[int, OphpcConfig, ImageConfig]:
    """Returns (status, config, image_config); status 0 = success."""
    cfg, img = OphpcConfig(), ImageConfig()
    st = _L().ophpc_read_config(path.encode(), ctypes.byref(cfg), ctypes.byref(img))
    return st, cfg, img


def load_ply(path: str, pinned: bool = False):
    """(n, 7) float64 vertices (pos[3], color[3], phase); raises on error.
    pinned=True returns a page-locked torch tensor, decoded straight into
    it, ready for an asynchronous host-to-device copy."""
    L = _L()
    n = L.ophpc_load_ply(path.encode(), None, 0)   # header only
    if n < 0:
        raise OphpcError(4, f"cannot load {path}")
    if pinned:
        import torch
        t = torch.empty((n, 7), dtype=torch.float64).pin_memory()
        ptr = t.data_ptr()
    else:
        t = np.zeros((n, 7), dtype=np.float64)
        ptr = t.ctypes.data
    if n and L.ophpc_load_ply(path.encode(), ptr, n) != n:
        raise OphpcError(4, f"cannot load {path}")
    return t


def save_bmp(path: str, pixels: np.ndarray, bits_per_pixel: int = 8, flip: int = 0, rotate: bool = False) -> None:
    p = np.ascontiguousarray(pixels, dtype=np.uint8)
    h, w = p.shape[0], p.shape[1]
    st = _L().ophpc_save_bmp(path.encode(), p.ctypes.data, w, h, bits_per_pixel, flip, 1 if rotate else 0)
    if st != 0:
        raise OphpcError(st, f"cannot save {path}")


def save_ohc(path: str, field: np.ndarray, pitch, wavelengths) -> None:
    """field: complex [n_channels, pnY, pnX] (or [pnY, pnX]); written as the
    reference's saveAsOhc writes it."""
    f = np.asarray(field)
    if f.ndim == 2:
        f = f[None]
    nch, pny, pnx = f.shape
    buf = np.ascontiguousarray(np.stack([f.real, f.imag], axis=-1), dtype=np.float64)
    wl = np.ascontiguousarray(np.asarray(wavelengths, dtype=np.float64).reshape(-1))
    if wl.size != nch:
        raise ValueError("one wavelength per channel")
    st = _L().ophpc_save_ohc(path.encode(), buf.ctypes.data, pnx, pny, float(pitch[0]), float(pitch[1]), nch,
                             wl.ctypes.data)
    if st != 0:
        raise OphpcError(st, f"cannot save {path}")


def load_ohc(path: str):
    """Returns (field complex [n_channels, pnY, pnX], pitch (x, y), wavelengths)."""
    L = _L()
    pnx, pny, nch = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_uint32()
    ppx, ppy = ctypes.c_double(), ctypes.c_double()
    wl = np.zeros(3)
    args = [ctypes.byref(pnx), ctypes.byref(pny), ctypes.byref(ppx), ctypes.byref(ppy), ctypes.byref(nch),
            wl.ctypes.data]
    st = L.ophpc_load_ohc(path.encode(), *args, None, 0)
    if st != 0:
        raise OphpcError(st, f"cannot load {path}")
    buf = np.zeros((nch.value, pny.value, pnx.value, 2))
    st = L.ophpc_load_ohc(path.encode(), *args, buf.ctypes.data, buf.size)
    if st != 0:
        raise OphpcError(st, f"cannot load {path}")
    return buf[..., 0] + 1j * buf[..., 1], (ppx.value, ppy.value), wl[:nch.value].copy()


# ------------------------------------------------------------------ façade

class PointCloud:
    """ophPointCloud with the reference's method names."""
    PC_DIFF_RS = PC_DIFF_RS
    PC_DIFF_FRESNEL = PC_DIFF_FRESNEL
    ENCODE_PHASE = ENCODE_PHASE
    ENCODE_AMPLITUDE = ENCODE_AMPLITUDE
    ENCODE_REAL = ENCODE_REAL
    ENCODE_IMAGINARY = ENCODE_IMAGINARY
    ENCODE_SIMPLENI = ENCODE_SIMPLENI
    ENCODE_BURCKHARDT = ENCODE_BURCKHARDT
    ENCODE_TWOPHASE = ENCODE_TWOPHASE

    def __init__(self, pc_file: Optional[str] = None, cfg_file: Optional[str] = None):
        self._L = _L()
        self._h = self._L.ophpc_pc_create()
        if not self._h:
            raise MemoryError("ophpc_pc_create failed")
        if pc_file is not None:
            self.loadPointCloud(pc_file)
        if cfg_file is not None:
            self.readConfig(cfg_file)

    def release(self) -> None:
        if self._h:
            self._L.ophpc_pc_release(self._h)
            self._h = None

    def __del__(self):  # pragma: no cover
        try:
            self.release()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.release()

    # config and input
    def readConfig(self, path: str) -> bool:
        return bool(self._L.ophpc_pc_read_config(self._h, path.encode()))

    def loadPointCloud(self, path: str) -> int:
        return int(self._L.ophpc_pc_load_point_cloud(self._h, path.encode()))

    def setPointCloudModel(self, vertices: np.ndarray) -> None:
        v = np.ascontiguousarray(vertices, dtype=np.float64)
        if v.ndim != 2 or v.shape[1] != 7:
            raise ValueError("vertices must be (n, 7) float64")
        self._L.ophpc_pc_set_point_cloud(self._h, v.ctypes.data if v.size else None, v.shape[0])

    def getNumberOfPoints(self) -> int:
        return int(self._L.ophpc_pc_number_of_points(self._h))

    def getPointCloudModel(self) -> np.ndarray:
        n = self.getNumberOfPoints()
        p = self._L.ophpc_pc_point_cloud(self._h)
        if not p or n == 0:
            return np.zeros((0, 7))
        return np.ctypeslib.as_array((ctypes.c_double * (7 * n)).from_address(p)).reshape(n, 7).copy()

    def SetMode(self, mode: int) -> None:
        self._L.ophpc_pc_set_mode(self._h, mode)

    def setViewingWindow(self, on: bool) -> None:
        self._L.ophpc_pc_set_viewing_window(self._h, 1 if on else 0)

    def setScale(self, sx: float, sy: float, sz: float) -> None:
        self._L.ophpc_pc_set_scale(self._h, sx, sy, sz)

    def setDistance(self, d: float) -> None:
        self._L.ophpc_pc_set_distance(self._h, d)

    def setOffset(self, ox: int, oy: int) -> None:
        self._L.ophpc_pc_set_offset(self._h, ox, oy)

    def getConfig(self) -> OphpcConfig:
        c = OphpcConfig()
        self._L.ophpc_pc_get_config(self._h, ctypes.byref(c))
        return c

    # the path
    def generateHologram(self, diff_flag: int = PC_DIFF_RS) -> float:
        return float(self._L.ophpc_pc_generate_hologram(self._h, diff_flag))

    def encoding(self, flag: int, passband: Optional[int] = None) -> None:
        """encoding(flag), or encoding(flag, passband) for ENCODE_SSB /
        ENCODE_OFFSSB (ophPointCloud.cpp:242-251)."""
        if passband is None:
            self._L.ophpc_pc_encoding(self._h, flag)
        else:
            self._L.ophpc_pc_encoding_passband(self._h, flag, passband)

    def normalize(self) -> None:
        self._L.ophpc_pc_normalize(self._h)

    def save(self, path: str, bits_per_pixel: int = 8) -> bool:
        return bool(self._L.ophpc_pc_save(self._h, path.encode(), bits_per_pixel))

    def saveAsOhc(self, path: str) -> bool:
        return bool(self._L.ophpc_pc_save_ohc(self._h, path.encode()))

    def loadAsOhc(self, path: str) -> bool:
        return bool(self._L.ophpc_pc_load_ohc(self._h, path.encode()))

    def lastError(self) -> str:
        e = self._L.ophpc_pc_last_error(self._h)
        return e.decode() if e else ""

    # buffers (copies)
    def _shape(self):
        c = self.getConfig()
        return int(c.n_channels), int(c.pixel_number[1]), int(c.pixel_number[0])

    def getComplexField(self) -> np.ndarray:
        nch, pny, pnx = self._shape()
        out = np.zeros((nch, pny, pnx), dtype=np.complex128)
        for ch in range(nch):
            p = self._L.ophpc_pc_complex_field(self._h, ch)
            if p:
                a = np.ctypeslib.as_array((ctypes.c_double * (2 * pnx * pny)).from_address(p))
                out[ch] = (a[0::2] + 1j * a[1::2]).reshape(pny, pnx)
        return out

    def getEncodedBuffer(self) -> np.ndarray:
        nch, pny, pnx = self._shape()
        out = np.zeros((nch, pny, pnx), dtype=np.float64)
        for ch in range(nch):
            p = self._L.ophpc_pc_encoded(self._h, ch)
            if p:
                out[ch] = np.ctypeslib.as_array((ctypes.c_double * (pnx * pny)).from_address(p)).reshape(pny, pnx)
        return out

    def getNormalizedBuffer(self) -> np.ndarray:
        nch, pny, pnx = self._shape()
        out = np.zeros((nch, pny, pnx), dtype=np.uint8)
        for ch in range(nch):
            p = self._L.ophpc_pc_normalized(self._h, ch)
            if p:
                out[ch] = np.ctypeslib.as_array((ctypes.c_uint8 * (pnx * pny)).from_address(p)).reshape(pny, pnx)
        return out
