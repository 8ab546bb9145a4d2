"""ctypes declarations of include/ophpc.h (and the façade entry points)."""
from __future__ import annotations

import ctypes
import os
import threading
from typing import Sequence

PKG = os.path.dirname(os.path.abspath(__file__))

DIFF_RS = 0
DIFF_FRESNEL = 1
MODE_CPU = 0
MODE_GPU = 1
MODE_DOUBLE = 0
MODE_FLOAT = 2
MODE_FASTMATH = 4
MODE_TENSOR_FP16 = 0x100
MODE_TENSOR_BF16X3 = 0x200
ENCODE_PHASE = 0
ENCODE_AMPLITUDE = 1
ENCODE_REAL = 2
ENCODE_IMAGINARY = 3
ENCODE_SIMPLENI = 4
ENCODE_BURCKHARDT = 5
ENCODE_TWOPHASE = 6
ENCODE_SSB = 7
ENCODE_OFFSSB = 8
SSB_LEFT, SSB_RIGHT, SSB_TOP, SSB_BOTTOM = 0, 1, 2, 3

STATUS = {
    0: "success", 1: "invalid argument", 2: "CUDA error", 3: "out of device memory", 4: "I/O error",
    5: "invalid configuration", 6: "unsupported", 7: "queue full", 8: "timeout", 9: "not ready",
    10: "no CUDA device",
}


class OphpcError(RuntimeError):
    def __init__(self, status: int, msg: str = ""):
        self.status = status
        super().__init__(f"[{STATUS.get(status, status)}] {msg}")


class OphpcConfig(ctypes.Structure):
    """struct ophpc_config."""
    _fields_ = [
        ("pixel_number", ctypes.c_int32 * 2),
        ("offset", ctypes.c_int32 * 2),
        ("pixel_pitch", ctypes.c_double * 2),
        ("scale", ctypes.c_double * 3),
        ("distance", ctypes.c_double),
        ("field_length", ctypes.c_double),
        ("viewing_window", ctypes.c_int32),
        ("n_channels", ctypes.c_uint32),
        ("wave_length", ctypes.c_double * 3),
    ]


def make_config(pnx: int, pny: int, ppx: float, ppy: float, wavelengths: Sequence[float],
                scale=(1.0, 1.0, 1.0), distance: float = 0.0, offset=(0, 0), field_length: float = 0.0,
                viewing_window: bool = False) -> OphpcConfig:
    c = OphpcConfig()
    c.pixel_number[0], c.pixel_number[1] = int(pnx), int(pny)
    c.offset[0], c.offset[1] = int(offset[0]), int(offset[1])
    c.pixel_pitch[0], c.pixel_pitch[1] = float(ppx), float(ppy)
    for i in range(3):
        c.scale[i] = float(scale[i])
    c.distance = float(distance)
    c.field_length = float(field_length)
    c.viewing_window = 1 if viewing_window else 0
    c.n_channels = len(wavelengths)
    for i, w in enumerate(wavelengths):
        c.wave_length[i] = float(w)
    return c


class OphpcWrpConfig(ctypes.Structure):
    """struct ophpc_wrp_config (include/ophpc_wrp.h)."""
    _fields_ = [
        ("pixel_number", ctypes.c_int32 * 2),
        ("pixel_pitch", ctypes.c_double * 2),
        ("scale", ctypes.c_double * 3),
        ("wrp_location", ctypes.c_double),
        ("propagation_distance", ctypes.c_double),
        ("n_channels", ctypes.c_uint32),
        ("wave_length", ctypes.c_double * 3),
        ("random_phase", ctypes.c_int32),
    ]


def make_wrp_config(pnx: int, pny: int, ppx: float, ppy: float, wavelengths: Sequence[float],
                    scale=(1.0, 1.0, 1.0), wrp_location: float = 0.0, distance: float = 0.0,
                    random_phase: bool = False) -> OphpcWrpConfig:
    c = OphpcWrpConfig()
    c.pixel_number[0], c.pixel_number[1] = int(pnx), int(pny)
    c.pixel_pitch[0], c.pixel_pitch[1] = float(ppx), float(ppy)
    for i in range(3):
        c.scale[i] = float(scale[i])
    c.wrp_location = float(wrp_location)
    c.propagation_distance = float(distance)
    c.n_channels = len(wavelengths)
    for i, w in enumerate(wavelengths):
        c.wave_length[i] = float(w)
    c.random_phase = 1 if random_phase else 0
    return c


_lock = threading.Lock()
_lib = None


def lib_path() -> str:
    return os.environ.get("OPHPC_LIBRARY", os.path.join(PKG, "lib", "libophpc.so"))


def _declare(L: ctypes.CDLL) -> None:
    vp, u32, u64, i32 = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int32
    L.ophpc_api_version.restype = i32
    L.ophpc_kernel_launches.restype = u64
    L.ophpc_status_string.argtypes = [ctypes.c_int]
    L.ophpc_status_string.restype = ctypes.c_char_p
    L.ophpc_last_error.argtypes = [vp]
    L.ophpc_last_error.restype = ctypes.c_char_p
    L.ophpc_create.argtypes = [i32, ctypes.POINTER(vp)]
    L.ophpc_create.restype = ctypes.c_int
    L.ophpc_destroy.argtypes = [vp]
    L.ophpc_destroy.restype = ctypes.c_int
    L.ophpc_generate.argtypes = [vp, ctypes.POINTER(OphpcConfig), vp, u64, u32, u32, vp, vp]
    L.ophpc_generate.restype = ctypes.c_int
    L.ophpc_generate_host.argtypes = [vp, ctypes.POINTER(OphpcConfig), vp, u64, u32, u32,
                                      ctypes.POINTER(vp), ctypes.POINTER(ctypes.c_double)]
    L.ophpc_generate_host.restype = ctypes.c_int
    L.ophpc_encode.argtypes = [vp, vp, u32, u64, u32, vp, vp, vp]
    L.ophpc_encode.restype = ctypes.c_int
    L.ophpc_plan_create.argtypes = [vp, ctypes.POINTER(OphpcConfig), vp, u64, u32, u32, vp, u32, vp, vp,
                                    ctypes.POINTER(vp)]
    L.ophpc_plan_create.restype = ctypes.c_int
    for fn in ("ophpc_plan_launch", "ophpc_plan_wait"):
        getattr(L, fn).argtypes = [vp, vp]
        getattr(L, fn).restype = ctypes.c_int
    L.ophpc_plan_destroy.argtypes = [vp]
    L.ophpc_plan_destroy.restype = ctypes.c_int
    W = ctypes.POINTER(OphpcWrpConfig)
    L.ophpc_wrp_generate.argtypes = [vp, W, vp, u64, vp, vp]
    L.ophpc_wrp_generate.restype = ctypes.c_int
    L.ophpc_wrp_plane.argtypes = [vp, W, vp, u64, u32, vp, vp]
    L.ophpc_wrp_plane.restype = ctypes.c_int
    L.ophpc_wrp_generate_host.argtypes = [vp, W, vp, u64, ctypes.POINTER(vp), ctypes.POINTER(ctypes.c_double)]
    L.ophpc_wrp_generate_host.restype = ctypes.c_int
    d = ctypes.c_double
    L.ophpc_fresnel_fft.argtypes = [vp, i32, i32, d, d, d, d, vp, vp, vp]
    L.ophpc_fresnel_fft.restype = ctypes.c_int
    L.ophpc_encode_ssb.argtypes = [vp, vp, u32, i32, i32, d, d, u32, u32, d, d, vp, vp, vp]
    L.ophpc_encode_ssb.restype = ctypes.c_int
    L.ophpc_encode_sideband.argtypes = [vp, vp, u32, i32, i32, d, d, u32, vp, vp, vp]
    L.ophpc_encode_sideband.restype = ctypes.c_int


def lib() -> ctypes.CDLL:
    """Loads libophpc.so; raises if it has not been built. No fallback."""
    global _lib
    with _lock:
        if _lib is None:
            p = lib_path()
            if not os.path.exists(p):
                raise RuntimeError(f"libophpc.so is not built ({p}); run openholo_gb300.build() "
                                   "or __graft_entry__.build()")
            L = ctypes.CDLL(p)
            _declare(L)
            _lib = L
    return _lib
