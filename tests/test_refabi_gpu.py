"""Reference-signature launchers (include/ophpc_refabi.h) driven the way the
reference's genCghPointCloudGPU drives its own kernels
(ophgen/src/ophPointCloud_GPU.cpp:218-279): config structs filled as its
constructors fill them and copied to device memory, one launch per colour
into a zeroed cuDoubleComplex buffer, sum_Kernel for the multi-buffer sum.
Fields are compared with the reference's own CPU fields (tests/golden/)
at the parity bar relL2 <= 1e-4 and with ophpc_generate's."""
import ctypes
import os

import numpy as np
import pytest

from tests._util import rel_l2, run_generate

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FIELD_TOL = 1e-4


class RefConfig(ctypes.Structure):
    _fields_ = [("n_points", ctypes.c_int32), ("pad0", ctypes.c_int32),
                ("scale_X", ctypes.c_double), ("scale_Y", ctypes.c_double), ("scale_Z", ctypes.c_double),
                ("offset_depth", ctypes.c_double), ("pn_X", ctypes.c_int32), ("pn_Y", ctypes.c_int32),
                ("offset_X", ctypes.c_int32), ("offset_Y", ctypes.c_int32), ("pp_X", ctypes.c_double),
                ("pp_Y", ctypes.c_double), ("half_ss_X", ctypes.c_double), ("half_ss_Y", ctypes.c_double),
                ("k", ctypes.c_double), ("lambda_", ctypes.c_double), ("d0", ctypes.c_double),
                ("d1", ctypes.c_double)]


def _lib():
    import openholo_gb300 as oph
    L = oph.lib()
    ip = ctypes.POINTER(ctypes.c_int)
    up = ctypes.POINTER(ctypes.c_uint)
    vp = ctypes.c_void_p
    for fn in ("cudaPointCloud_RS", "cudaPointCloud_Fresnel"):
        getattr(L, fn).argtypes = [ip, ip, vp, vp, vp, up, up]
        getattr(L, fn).restype = None
    L.sum_Kernel.argtypes = [ip, ip, vp, vp, ctypes.c_int]
    L.sum_Kernel.restype = None
    L.ophpc_refabi_last_status.restype = ctypes.c_int
    return L


def _config(g: dict, n_points: int, ch: int, diff: int) -> RefConfig:
    """What CudaPointCloudConfig{RS,Fresnel}(...) holds for channel ch."""
    pnx, pny, ppx, ppy = g["pnx"], g["pny"], g["ppx"], g["ppy"]
    lam = g["wavelengths"][ch]
    sc = g.get("scale", (1.0, 1.0, 1.0))
    c = RefConfig(n_points=n_points, scale_X=sc[0], scale_Y=sc[1], scale_Z=sc[2],
                  offset_depth=g.get("distance", 0.0), pn_X=pnx, pn_Y=pny, offset_X=0, offset_Y=0, pp_X=ppx,
                  pp_Y=ppy, half_ss_X=pnx * ppx / 2, half_ss_Y=pny * ppy / 2, k=2 * np.pi / lam, lambda_=lam)
    tx, ty = lam / (2 * ppx), lam / (2 * ppy)
    if diff == 0:
        c.d0, c.d1 = tx / np.sqrt(1 - tx * tx), ty / np.sqrt(1 - ty * ty)
    else:
        c.d0, c.d1 = tx, ty
    return c


def _geometry(xml: str) -> dict:
    import re
    def num(tag):
        return float(re.search(rf"<{tag}>([^<]+)</{tag}>", xml).group(1))
    nch = int(num("SLM_WaveNum")) if "<SLM_WaveNum>" in xml else 1
    return dict(pnx=int(num("SLM_PixelNumX")), pny=int(num("SLM_PixelNumY")), ppx=num("SLM_PixelPitchX"),
                ppy=num("SLM_PixelPitchY"), wavelengths=[num(f"SLM_WaveLength_{i + 1}") for i in range(nch)],
                scale=(num("ScaleX"), num("ScaleY"), num("ScaleZ")), distance=num("Distance"))


def _launch(L, diff, d_v, d_dst, d_cfg, ch, mode=0):
    nb, nt = ctypes.c_int(1), ctypes.c_int(1)
    fn = L.cudaPointCloud_RS if diff == 0 else L.cudaPointCloud_Fresnel
    fn(ctypes.byref(nb), ctypes.byref(nt), ctypes.c_void_p(d_v), ctypes.c_void_p(d_dst), ctypes.c_void_p(d_cfg),
       ctypes.byref(ctypes.c_uint(ch)), ctypes.byref(ctypes.c_uint(mode)))
    return L.ophpc_refabi_last_status()


def _run(L, g, v, diff, mode=0):
    """The reference driver's single-GPU loop; returns [nch, pny, pnx] complex."""
    import torch
    nch = len(g["wavelengths"])
    d_v = torch.from_numpy(np.ascontiguousarray(v, dtype=np.float64)).cuda()
    d_dst = torch.zeros((g["pny"] * g["pnx"], 2), dtype=torch.float64, device="cuda")
    out = []
    for ch in range(nch):
        c = _config(g, v.shape[0], ch, diff)
        d_cfg = torch.frombuffer(bytearray(bytes(c)), dtype=torch.uint8).cuda()
        assert _launch(L, diff, d_v.data_ptr(), d_dst.data_ptr(), d_cfg.data_ptr(), ch, mode) == 0
        h = d_dst.cpu().numpy()
        out.append((h[:, 0] + 1j * h[:, 1]).reshape(g["pny"], g["pnx"]))
        d_dst.zero_()
    return np.stack(out)


@pytest.mark.parametrize("name", ["rs_window_1ch", "fresnel_window_1ch", "fresnel_3ch"])
def test_launchers_match_reference_fields(gpu_ctx, name):
    d = np.load(os.path.join(GOLD, name + ".npz"))
    assert not bool(d["viewing_window"])
    g = _geometry(str(d["xml"]))
    diff = int(d["diff_flag"])
    got = _run(_lib(), g, d["vertices"], diff)
    assert rel_l2(got, d["field"]) <= FIELD_TOL
    mine = run_generate(gpu_ctx, g, d["vertices"], diff)
    assert rel_l2(got, mine) <= 1e-12


@pytest.mark.parametrize("name", ["rs_window_1ch", "fresnel_window_1ch", "fresnel_3ch"])
def test_launchers_reach_the_tensor_cores(gpu_ctx, name):
    """mode = OPHPC_MODE_TENSOR_BF16X3 (with the reference's MODE_GPU bit):
    the tensor-core tile kernels behind the same launchers, against the
    reference's fields and ophpc_generate's tensor-core result; adding into a
    field that already holds one result doubles it."""
    import openholo_gb300 as oph
    d = np.load(os.path.join(GOLD, name + ".npz"))
    g = _geometry(str(d["xml"]))
    diff = int(d["diff_flag"])
    L = _lib()
    before = oph.lib().ophpc_kernel_launches()
    got = _run(L, g, d["vertices"], diff, mode=0x200 | 1)
    assert oph.lib().ophpc_kernel_launches() - before >= 3 * len(g["wavelengths"])
    assert rel_l2(got, d["field"]) <= FIELD_TOL
    mine = run_generate(gpu_ctx, g, d["vertices"], diff, 0x200)
    assert rel_l2(got, mine) <= 5e-5
    plain = _run(L, g, d["vertices"], diff)
    assert rel_l2(got, plain) <= FIELD_TOL


def test_launchers_accumulate_and_sum_kernel(gpu_ctx):
    import torch
    L = _lib()
    d = np.load(os.path.join(GOLD, "rs_window_1ch.npz"))
    g = _geometry(str(d["xml"]))
    v = d["vertices"]
    d_v = torch.from_numpy(np.ascontiguousarray(v)).cuda()
    npx = g["pnx"] * g["pny"]
    d_dst = torch.zeros((npx, 2), dtype=torch.float64, device="cuda")
    d_cfg = torch.frombuffer(bytearray(bytes(_config(g, v.shape[0], 0, 0))), dtype=torch.uint8).cuda()
    assert _launch(L, 0, d_v.data_ptr(), d_dst.data_ptr(), d_cfg.data_ptr(), 0) == 0
    once = d_dst.clone()
    assert _launch(L, 0, d_v.data_ptr(), d_dst.data_ptr(), d_cfg.data_ptr(), 0) == 0
    torch.testing.assert_close(d_dst, 2 * once, rtol=1e-15, atol=0)
    # sum_Kernel: dst += src
    src = torch.randn((npx, 2), dtype=torch.float64, device="cuda")
    before = d_dst.clone()
    nb, nt = ctypes.c_int(1), ctypes.c_int(1)
    L.sum_Kernel(ctypes.byref(nb), ctypes.byref(nt), ctypes.c_void_p(d_dst.data_ptr()),
                 ctypes.c_void_p(src.data_ptr()), npx)
    torch.cuda.synchronize()
    assert L.ophpc_refabi_last_status() == 0
    assert torch.equal(d_dst, before + src)


def test_launchers_reject_bad_arguments(gpu_ctx):
    import torch
    L = _lib()
    d_v = torch.zeros((4, 7), dtype=torch.float64, device="cuda")
    d_dst = torch.zeros((64, 2), dtype=torch.float64, device="cuda")
    g = dict(pnx=8, pny=8, ppx=8e-6, ppy=8e-6, wavelengths=[532e-9])
    c = _config(g, 4, 0, 0)
    d_cfg = torch.frombuffer(bytearray(bytes(c)), dtype=torch.uint8).cuda()
    assert _launch(L, 0, d_v.data_ptr(), d_dst.data_ptr(), d_cfg.data_ptr(), 3) == 1   # colour 3
    assert _launch(L, 0, d_v.data_ptr(), d_dst.data_ptr(), 0, 0) == 1                  # no config
    c.n_points = -1
    d_cfg = torch.frombuffer(bytearray(bytes(c)), dtype=torch.uint8).cuda()
    assert _launch(L, 1, d_v.data_ptr(), d_dst.data_ptr(), d_cfg.data_ptr(), 0) == 1
    torch.cuda.synchronize()
    assert not torch.any(d_dst)


def test_launcher_returns_before_its_kernel_completes(gpu_ctx):
    """The reference's launchers only enqueue (ophgen/src/ophPCKernel.cu:
    893-933); so do these: with the config uploaded the way the reference's
    driver uploads it (a blocking cudaMemcpy right before the call,
    ophgen/src/ophPointCloud_GPU.cpp:249-251), the call returns while its
    kernel is still running, and the field is complete after a synchronise."""
    import time

    import torch
    L = _lib()
    rng = np.random.default_rng(12)
    n = 40_000
    v = np.zeros((n, 7))
    v[:, 0:2] = rng.uniform(-1e-3, 1e-3, (n, 2))
    v[:, 2] = rng.uniform(0.4, 0.5, n)
    v[:, 3:6] = 1.0 - rng.uniform(0.0, 1.0, (n, 3))
    g = dict(pnx=2048, pny=2048, ppx=8e-6, ppy=8e-6, wavelengths=[532e-9])
    d_v = torch.from_numpy(v).cuda()
    d_dst = torch.zeros((g["pnx"] * g["pny"], 2), dtype=torch.float64, device="cuda")
    # warm-up: the first call on a device creates the launchers' context
    d_cfg = torch.frombuffer(bytearray(bytes(_config(g, 1, 0, 0))), dtype=torch.uint8).cuda()
    assert _launch(L, 0, d_v.data_ptr(), d_dst.data_ptr(), d_cfg.data_ptr(), 0) == 0
    d_dst.zero_()
    d_cfg = torch.frombuffer(bytearray(bytes(_config(g, n, 0, 0))), dtype=torch.uint8).cuda()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    assert _launch(L, 0, d_v.data_ptr(), d_dst.data_ptr(), d_cfg.data_ptr(), 0) == 0
    t_call = time.perf_counter() - t0
    pending = not torch.cuda.default_stream().query()   # the launcher's work is on the legacy stream
    torch.cuda.synchronize()
    t_total = time.perf_counter() - t0
    assert pending, "the launcher waited for its own kernel"
    assert t_call < 0.5 * t_total, (t_call, t_total)
    h = d_dst.cpu().numpy()
    mine = run_generate(gpu_ctx, g, v, 0)
    assert rel_l2((h[:, 0] + 1j * h[:, 1]).reshape(1, g["pny"], g["pnx"]), mine) <= 1e-12
