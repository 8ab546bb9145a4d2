"""openholo_gb300 — GB300-native point-cloud hologram generation.

Python view of the C ABI in ``include/ophpc.h`` (``lib/libophpc.so``, built
by ``_build.py``). The hot path is entirely in the CUDA library; this module
only binds it with ctypes. There is no CPU fallback: importing works without
a GPU (for the host-side tests), but every compute call goes to the library
and fails loudly when it or the GPU is missing.
"""
from __future__ import annotations

import ctypes
import os
from typing import Optional, Sequence

from ._abi import (  # noqa: F401
    DIFF_FRESNEL, DIFF_RS, ENCODE_AMPLITUDE, ENCODE_BURCKHARDT, ENCODE_IMAGINARY, ENCODE_PHASE, ENCODE_REAL,
    ENCODE_OFFSSB, ENCODE_SIMPLENI, ENCODE_SSB, ENCODE_TWOPHASE, MODE_CPU, SSB_BOTTOM, SSB_LEFT, SSB_RIGHT, SSB_TOP,
    MODE_DOUBLE, MODE_FASTMATH, MODE_FLOAT, MODE_GPU, MODE_TENSOR_BF16X3, MODE_TENSOR_FP16, OphpcConfig,
    OphpcError, OphpcWrpConfig, STATUS, lib, lib_path, make_config, make_wrp_config,
)

__all__ = [
    "Context", "OphpcConfig", "OphpcError", "make_config", "lib", "lib_path", "OphpcWrpConfig", "make_wrp_config",
    "DIFF_RS", "DIFF_FRESNEL", "MODE_CPU", "MODE_GPU", "MODE_DOUBLE", "MODE_FLOAT", "MODE_FASTMATH",
    "MODE_TENSOR_FP16", "MODE_TENSOR_BF16X3", "ENCODE_PHASE", "ENCODE_AMPLITUDE", "ENCODE_REAL",
    "ENCODE_IMAGINARY", "ENCODE_SIMPLENI", "ENCODE_BURCKHARDT", "ENCODE_TWOPHASE", "ENCODE_SSB", "ENCODE_OFFSSB",
    "SSB_LEFT", "SSB_RIGHT", "SSB_TOP", "SSB_BOTTOM", "Plan", "PLAN_NO_ENCODE",
]

PLAN_NO_ENCODE = 0xFFFFFFFF


class Context:
    """One ophpc_context (one GPU). Thin wrapper; pointers are ints."""

    def __init__(self, device: int = 0):
        self._lib = lib()
        self._h = ctypes.c_void_p()
        st = self._lib.ophpc_create(int(device), ctypes.byref(self._h))
        if st != 0:
            raise OphpcError(st, "ophpc_create failed")
        self.device = device

    def close(self) -> None:
        if self._h:
            self._lib.ophpc_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):  # pragma: no cover - interpreter shutdown order
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def handle(self) -> ctypes.c_void_p:
        return self._h

    def _check(self, st: int, what: str) -> None:
        if st != 0:
            detail = self._lib.ophpc_last_error(self._h)
            raise OphpcError(st, f"{what}: {detail.decode() if detail else ''}")

    def generate(self, cfg: OphpcConfig, d_vertices: int, n_points: int, diff_flag: int, mode: int,
                 d_field: int, stream: int = 0) -> None:
        st = self._lib.ophpc_generate(self._h, ctypes.byref(cfg), ctypes.c_void_p(d_vertices),
                                      ctypes.c_uint64(n_points), diff_flag, mode, ctypes.c_void_p(d_field),
                                      ctypes.c_void_p(stream))
        self._check(st, "ophpc_generate")

    def generate_host(self, cfg: OphpcConfig, h_vertices: int, n_points: int, diff_flag: int, mode: int,
                      h_fields: Sequence[int]) -> float:
        arr = (ctypes.c_void_p * len(h_fields))(*h_fields)
        secs = ctypes.c_double()
        st = self._lib.ophpc_generate_host(self._h, ctypes.byref(cfg), ctypes.c_void_p(h_vertices),
                                           ctypes.c_uint64(n_points), diff_flag, mode, arr, ctypes.byref(secs))
        self._check(st, "ophpc_generate_host")
        return secs.value

    # WRP generator (include/ophpc_wrp.h)
    def wrp_generate(self, cfg: OphpcWrpConfig, d_vertices: int, n_points: int, d_field: int,
                     stream: int = 0) -> None:
        st = self._lib.ophpc_wrp_generate(self._h, ctypes.byref(cfg), ctypes.c_void_p(d_vertices),
                                          ctypes.c_uint64(n_points), ctypes.c_void_p(d_field), ctypes.c_void_p(stream))
        self._check(st, "ophpc_wrp_generate")

    def wrp_plane(self, cfg: OphpcWrpConfig, d_vertices: int, n_points: int, channel: int, d_plane: int,
                  stream: int = 0) -> None:
        st = self._lib.ophpc_wrp_plane(self._h, ctypes.byref(cfg), ctypes.c_void_p(d_vertices),
                                       ctypes.c_uint64(n_points), channel, ctypes.c_void_p(d_plane),
                                       ctypes.c_void_p(stream))
        self._check(st, "ophpc_wrp_plane")

    def wrp_generate_host(self, cfg: OphpcWrpConfig, h_vertices: int, n_points: int,
                          h_fields: Sequence[int]) -> float:
        arr = (ctypes.c_void_p * len(h_fields))(*h_fields)
        secs = ctypes.c_double()
        st = self._lib.ophpc_wrp_generate_host(self._h, ctypes.byref(cfg), ctypes.c_void_p(h_vertices),
                                               ctypes.c_uint64(n_points), arr, ctypes.byref(secs))
        self._check(st, "ophpc_wrp_generate_host")
        return secs.value

    def fresnel_fft(self, pnx: int, pny: int, ppx: float, ppy: float, wavelength: float, distance: float,
                    d_src: int, d_dst: int, stream: int = 0) -> None:
        st = self._lib.ophpc_fresnel_fft(self._h, pnx, pny, ppx, ppy, wavelength, distance, ctypes.c_void_p(d_src),
                                         ctypes.c_void_p(d_dst), ctypes.c_void_p(stream))
        self._check(st, "ophpc_fresnel_fft")

    def encode_ssb(self, d_field: int, n_channels: int, pnx: int, pny: int, ppx: float, ppy: float,
                   encode_flag: int, passband: int = SSB_LEFT, spectrum_shift=(0.0, 0.5),
                   d_encoded: Optional[int] = None, d_normalized: Optional[int] = None, stream: int = 0) -> None:
        """ophPointCloud::encoding(ENCODE_SSB | ENCODE_OFFSSB, passband) (ophpc_encode_ssb)."""
        st = self._lib.ophpc_encode_ssb(self._h, ctypes.c_void_p(d_field), n_channels, pnx, pny, ppx, ppy,
                                        encode_flag, passband, float(spectrum_shift[0]), float(spectrum_shift[1]),
                                        ctypes.c_void_p(d_encoded or 0), ctypes.c_void_p(d_normalized or 0),
                                        ctypes.c_void_p(stream))
        self._check(st, "ophpc_encode_ssb")

    def encode_sideband(self, d_field: int, n_channels: int, pnx: int, pny: int, ppx: float, ppy: float,
                        passband: int, d_encoded: Optional[int] = None, d_normalized: Optional[int] = None,
                        stream: int = 0) -> None:
        """ophGen::encodeSideBand(passband) (ophpc_encode_sideband)."""
        st = self._lib.ophpc_encode_sideband(self._h, ctypes.c_void_p(d_field), n_channels, pnx, pny, ppx, ppy,
                                             passband, ctypes.c_void_p(d_encoded or 0),
                                             ctypes.c_void_p(d_normalized or 0), ctypes.c_void_p(stream))
        self._check(st, "ophpc_encode_sideband")

    def encode(self, d_field: int, n_channels: int, n_pixels: int, encode_flag: int,
               d_encoded: Optional[int], d_normalized: Optional[int], stream: int = 0) -> None:
        st = self._lib.ophpc_encode(self._h, ctypes.c_void_p(d_field), n_channels, ctypes.c_uint64(n_pixels),
                                    encode_flag, ctypes.c_void_p(d_encoded or 0), ctypes.c_void_p(d_normalized or 0),
                                    ctypes.c_void_p(stream))
        self._check(st, "ophpc_encode")

    def plan(self, cfg: OphpcConfig, d_vertices: int, n_points: int, diff_flag: int, mode: int, d_field: int,
             encode_flag: int = PLAN_NO_ENCODE, d_encoded: Optional[int] = None,
             d_normalized: Optional[int] = None) -> "Plan":
        """generate (+ encode) captured once into a CUDA graph (ophpc_plan_create)."""
        h = ctypes.c_void_p()
        st = self._lib.ophpc_plan_create(self._h, ctypes.byref(cfg), ctypes.c_void_p(d_vertices),
                                         ctypes.c_uint64(n_points), diff_flag, mode, ctypes.c_void_p(d_field),
                                         encode_flag, ctypes.c_void_p(d_encoded or 0),
                                         ctypes.c_void_p(d_normalized or 0), ctypes.byref(h))
        self._check(st, "ophpc_plan_create")
        return Plan(self, h)


class Plan:
    """A captured generate (+ encode); launch() replays it, wait() synchronises
    the stream and raises on a kernel timeout."""

    def __init__(self, ctx: Context, handle: ctypes.c_void_p):
        self._ctx = ctx
        self._h = handle

    def launch(self, stream: int = 0) -> None:
        self._ctx._check(self._ctx._lib.ophpc_plan_launch(self._h, ctypes.c_void_p(stream)), "ophpc_plan_launch")

    def wait(self, stream: int = 0) -> None:
        self._ctx._check(self._ctx._lib.ophpc_plan_wait(self._h, ctypes.c_void_p(stream)), "ophpc_plan_wait")

    def close(self) -> None:
        if self._h:
            self._ctx._lib.ophpc_plan_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):  # pragma: no cover - interpreter shutdown order
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def build(force: bool = False) -> str:
    """Compile libophpc.so in-tree (nvcc, sm_103a)."""
    from . import _build
    return _build.build(force=force)


def library_loaded_path() -> str:
    return os.path.realpath(lib_path())
