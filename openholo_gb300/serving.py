"""Python binding of the serving engine (include/ophpc_serve.h)."""
from __future__ import annotations

import ctypes
from dataclasses import dataclass
from typing import Dict, Optional

import numpy as np

from ._abi import OphpcConfig, OphpcError, lib, make_config

POLICY_EARLIEST_DEADLINE = 0   # default
POLICY_SHORTEST_REMAINING = 1
POLICY_DEADLINE = 2            # short jobs first, then earliest deadline


class ServerOptions(ctypes.Structure):
    _fields_ = [("max_in_flight", ctypes.c_uint32), ("policy", ctypes.c_uint32),
                ("memory_budget", ctypes.c_uint64), ("reserve_bytes", ctypes.c_uint64),
                ("step_ms", ctypes.c_double)]


class JobDesc(ctypes.Structure):
    _fields_ = [("cfg", OphpcConfig), ("h_vertices", ctypes.c_void_p), ("n_points", ctypes.c_uint64),
                ("diff_flag", ctypes.c_uint32), ("mode", ctypes.c_uint32), ("h_field", ctypes.c_void_p),
                ("h_codes", ctypes.c_void_p), ("encode_flag", ctypes.c_uint32), ("pad", ctypes.c_uint32)]


class JobStats(ctypes.Structure):
    _fields_ = [("t_submit", ctypes.c_double), ("t_admit", ctypes.c_double), ("t_done", ctypes.c_double)]


_declared = False


def _L():
    global _declared
    L = lib()
    if not _declared:
        vp = ctypes.c_void_p
        L.ophpc_server_create.argtypes = [ctypes.c_int32, ctypes.POINTER(ServerOptions), ctypes.POINTER(vp)]
        L.ophpc_server_create.restype = ctypes.c_int
        L.ophpc_server_submit.argtypes = [vp, ctypes.POINTER(JobDesc), ctypes.POINTER(ctypes.c_uint64)]
        L.ophpc_server_submit.restype = ctypes.c_int
        L.ophpc_server_wait.argtypes = [vp, ctypes.c_uint64, ctypes.c_double, ctypes.POINTER(JobStats)]
        L.ophpc_server_wait.restype = ctypes.c_int
        L.ophpc_server_destroy.argtypes = [vp]
        L.ophpc_server_destroy.restype = ctypes.c_int
        _declared = True
    return L


@dataclass
class Result:
    status: int
    t_submit: float
    t_admit: float
    t_done: float
    field: Optional[np.ndarray]
    codes: Optional[np.ndarray]

    @property
    def latency(self) -> float:
        return self.t_done - self.t_submit


class Server:
    """Continuous-batching hologram server on one GPU."""

    def __init__(self, device: int = 0, max_in_flight: int = 16, memory_budget: int = 0, step_ms: float = 2.0,
                 reserve_bytes: int = 0, policy: int = POLICY_EARLIEST_DEADLINE):
        self._L = _L()
        o = ServerOptions(max_in_flight=max_in_flight, policy=policy, memory_budget=memory_budget,
                          reserve_bytes=reserve_bytes, step_ms=step_ms)
        self._h = ctypes.c_void_p()
        st = self._L.ophpc_server_create(device, ctypes.byref(o), ctypes.byref(self._h))
        if st != 0:
            raise OphpcError(st, "ophpc_server_create failed")
        self._keep: Dict[int, tuple] = {}

    def submit(self, geometry: dict, vertices: np.ndarray, diff_flag: int, want_field: bool = True,
               want_codes: bool = False, encode_flag: int = 0, pinned: bool = False, mode: int = 0) -> int:
        """geometry: make_config keyword arguments. Returns a ticket."""
        v = np.ascontiguousarray(vertices, dtype=np.float64)
        cfg = make_config(**geometry)
        nch, pny, pnx = cfg.n_channels, cfg.pixel_number[1], cfg.pixel_number[0]
        field = np.empty((nch, pny, pnx, 2), dtype=np.float64) if want_field else None
        codes = np.empty((nch, pny, pnx), dtype=np.uint8) if want_codes else None
        bufs = [v, field, codes]
        if pinned:
            import torch
            tv = torch.from_numpy(v).pin_memory()
            tf = torch.empty(field.shape, dtype=torch.float64).pin_memory() if field is not None else None
            tc = torch.empty(codes.shape, dtype=torch.uint8).pin_memory() if codes is not None else None
            bufs = [tv, tf, tc]
            vptr = tv.data_ptr()
            fptr = tf.data_ptr() if tf is not None else None
            cptr = tc.data_ptr() if tc is not None else None
        else:
            vptr = v.ctypes.data if v.size else None
            fptr = field.ctypes.data if field is not None else None
            cptr = codes.ctypes.data if codes is not None else None
        j = JobDesc(cfg=cfg, h_vertices=vptr, n_points=v.shape[0], diff_flag=diff_flag, mode=mode,
                    h_field=fptr, h_codes=cptr, encode_flag=encode_flag)
        t = ctypes.c_uint64()
        st = self._L.ophpc_server_submit(self._h, ctypes.byref(j), ctypes.byref(t))
        if st != 0:
            raise OphpcError(st, "ophpc_server_submit rejected the job")
        self._keep[t.value] = (bufs, pinned)
        return t.value

    def submit_raw(self, cfg: OphpcConfig, h_vertices: int, n_points: int, diff_flag: int,
                   h_field: Optional[int] = None, h_codes: Optional[int] = None, encode_flag: int = 0,
                   mode: int = 0) -> int:
        """Submit with caller-owned (ideally page-locked) host buffers given as
        addresses; the caller keeps them alive until the job is waited for."""
        j = JobDesc(cfg=cfg, h_vertices=h_vertices or None, n_points=n_points, diff_flag=diff_flag, mode=mode,
                    h_field=h_field or None, h_codes=h_codes or None, encode_flag=encode_flag)
        t = ctypes.c_uint64()
        st = self._L.ophpc_server_submit(self._h, ctypes.byref(j), ctypes.byref(t))
        if st != 0:
            raise OphpcError(st, "ophpc_server_submit rejected the job")
        return t.value

    def wait_stats(self, ticket: int, timeout_s: float = -1.0) -> Result:
        """Wait for a job submitted with submit_raw (no buffers returned)."""
        s = JobStats()
        st = self._L.ophpc_server_wait(self._h, ticket, timeout_s, ctypes.byref(s))
        if st == 8:
            raise OphpcError(st, f"job {ticket} not finished within {timeout_s} s")
        return Result(st, s.t_submit, s.t_admit, s.t_done, None, None)

    def wait(self, ticket: int, timeout_s: float = -1.0) -> Result:
        s = JobStats()
        st = self._L.ophpc_server_wait(self._h, ticket, timeout_s, ctypes.byref(s))
        if st == 8:   # OPHPC_ERROR_TIMEOUT: the job is still running and keeps its buffers
            raise OphpcError(st, f"job {ticket} not finished within {timeout_s} s")
        bufs, pinned = self._keep.pop(ticket, ([None, None, None], False))
        field = codes = None
        f, c = bufs[1], bufs[2]
        if f is not None:
            f = f.numpy() if pinned else f
            field = f[..., 0] + 1j * f[..., 1]
        if c is not None:
            codes = c.numpy().copy() if pinned else c
        return Result(st, s.t_submit, s.t_admit, s.t_done, field, codes)

    def poll(self, ticket: int) -> Optional[Result]:
        """The job's result if it has finished (the ticket is then spent), else
        None without blocking (ophpc_server_wait with timeout 0)."""
        try:
            return self.wait(ticket, 0.0)
        except OphpcError as e:
            if e.status == 8:
                return None
            raise

    def close(self) -> None:
        if self._h:
            self._L.ophpc_server_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
