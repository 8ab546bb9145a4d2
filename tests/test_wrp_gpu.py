"""WRP generator on the GPU (include/ophpc_wrp.h) against the oracle.

* The splat plane (ophpc_wrp_plane) against the reference's own planes
  (tests/golden/wrp_*.npz): FP64 with 64-bit fixed-point amplitude sums, so
  within relL2 1e-12.
* The propagation (ophpc_fresnel_fft) against the numpy FP64 restatement of
  ophGen::Fresnel_FFT (oracle.wrp_propagate): relL2 1e-10.
* The whole generate (ophpc_wrp_generate) against oracle.wrp_generate on the
  synthetic three-colour case and on the reference's WRP example (Dice,
  1920x1080): relL2 1e-10, 8-bit phase codes >= 99.9 % exact within +-1 LSB.
"""
import os
import re

import numpy as np
import pytest

from tests._util import code_agreement, rel_l2

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _cfgs(z, oracle_mod):
    import openholo_gb300 as oph
    kw = dict(pnx=int(z["pnx"]), pny=int(z["pny"]), ppx=float(z["ppx"]), ppy=float(z["ppy"]),
              wavelengths=list(z["wavelengths"]), scale=tuple(z["scale"]), wrp_location=float(z["wrp_location"]),
              distance=float(z["distance"]))
    return oph.make_wrp_config(**kw), oracle_mod.WrpGeometry(**kw)


def _dice(oracle_mod):
    import openholo_gb300 as oph
    z = np.load(os.path.join(GOLD, "wrp_dice.npz"))
    xml = str(z["xml"])

    def num(tag):
        return float(re.search(rf"<{tag}>([^<]+)</{tag}>", xml).group(1))
    kw = dict(pnx=int(num("SLM_PixelNumX")), pny=int(num("SLM_PixelNumY")), ppx=num("SLM_PixelPitchX"),
              ppy=num("SLM_PixelPitchY"), wavelengths=[num("SLM_WaveLength_1")],
              scale=(num("ScaleX"), num("ScaleY"), num("ScaleZ")), wrp_location=num("LocationOfWRP"),
              distance=num("Distance"))
    return z, oph.make_wrp_config(**kw), oracle_mod.WrpGeometry(**kw)


def _plane(ctx, cfg, v, channel):
    import torch
    dv = torch.from_numpy(np.ascontiguousarray(v)).cuda()
    out = torch.full((cfg.pixel_number[1], cfg.pixel_number[0], 2), float("nan"), dtype=torch.float64,
                     device="cuda")
    ctx.wrp_plane(cfg, dv.data_ptr(), v.shape[0], channel, out.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    h = out.cpu().numpy()
    return h[..., 0] + 1j * h[..., 1]


def _generate(ctx, cfg, v):
    import torch
    dv = torch.from_numpy(np.ascontiguousarray(v)).cuda()
    out = torch.full((cfg.n_channels, cfg.pixel_number[1], cfg.pixel_number[0], 2), float("nan"),
                     dtype=torch.float64, device="cuda")
    ctx.wrp_generate(cfg, dv.data_ptr() if v.shape[0] else 0, v.shape[0], out.data_ptr(),
                     torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    h = out.cpu().numpy()
    return h[..., 0] + 1j * h[..., 1]


@pytest.mark.parametrize("name", ["wrp_3ch", "wrp_negdz_edges"])
def test_wrp_plane_matches_reference(gpu_ctx, oracle_mod, name):
    z = np.load(os.path.join(GOLD, name + ".npz"))
    cfg, _ = _cfgs(z, oracle_mod)
    got = np.stack([_plane(gpu_ctx, cfg, z["vertices"], c) for c in range(cfg.n_channels)])
    assert rel_l2(got, z["planes"]) <= 1e-12


def test_wrp_dice_plane_matches_reference(gpu_ctx, oracle_mod):
    z, cfg, _ = _dice(oracle_mod)
    p = _plane(gpu_ctx, cfg, z["vertices"], 0)
    assert np.count_nonzero(p) == int(z["nonzero"])
    at = p.reshape(-1)[z["pixel_index"]]
    assert rel_l2(at, z["plane_at"]) <= 1e-12
    assert abs(np.linalg.norm(p) - float(z["plane_norm"])) <= 1e-12 * float(z["plane_norm"])


@pytest.mark.parametrize("pnx,pny", [(40, 24), (96, 72), (105, 49), (128, 36)])
def test_fresnel_fft_matches_oracle(gpu_ctx, oracle_mod, pnx, pny):
    """Transform lengths 2*pn with radices 8, 4, 2, 3, 5 and 7."""
    import torch
    rng = np.random.default_rng(pnx * 1000 + pny)
    plane = rng.normal(size=(pny, pnx)) + 1j * rng.normal(size=(pny, pnx))
    g = oracle_mod.WrpGeometry(pnx=pnx, pny=pny, ppx=6.4e-6, ppy=7.1e-6, wavelengths=[532e-9], distance=0.02)
    want = oracle_mod.wrp_propagate(plane, g, 532e-9)
    src = torch.from_numpy(np.ascontiguousarray(plane).view(np.float64).reshape(pny, pnx, 2)).cuda()
    dst = torch.full_like(src, float("nan"))
    gpu_ctx.fresnel_fft(pnx, pny, g.ppx, g.ppy, 532e-9, g.distance, src.data_ptr(), dst.data_ptr(),
                        torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    h = dst.cpu().numpy()
    assert rel_l2(h[..., 0] + 1j * h[..., 1], want) <= 1e-10
    # in place
    gpu_ctx.fresnel_fft(pnx, pny, g.ppx, g.ppy, 532e-9, g.distance, src.data_ptr(), src.data_ptr(),
                        torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert torch.equal(src, dst)


def test_wrp_generate_three_colours(gpu_ctx, oracle_mod):
    z = np.load(os.path.join(GOLD, "wrp_3ch.npz"))
    cfg, g = _cfgs(z, oracle_mod)
    got = _generate(gpu_ctx, cfg, z["vertices"])
    want = oracle_mod.wrp_generate(g, z["vertices"])
    assert rel_l2(got, want) <= 1e-10
    # deterministic: the fixed-point anchor sums do not depend on the order of the atomics
    assert np.array_equal(got, _generate(gpu_ctx, cfg, z["vertices"]))


def test_wrp_generate_dice_example(gpu_ctx, oracle_mod):
    """The reference's WRP example, 1920x1080: field and 8-bit phase codes."""
    import torch
    z, cfg, g = _dice(oracle_mod)
    got = _generate(gpu_ctx, cfg, z["vertices"])
    want = oracle_mod.wrp_generate(g, z["vertices"])
    assert rel_l2(got, want) <= 1e-10
    npx = cfg.pixel_number[0] * cfg.pixel_number[1]
    f = torch.from_numpy(np.ascontiguousarray(got).view(np.float64).reshape(1, npx, 2)).cuda()
    codes = torch.empty((1, npx), dtype=torch.uint8, device="cuda")
    gpu_ctx.encode(f.data_ptr(), 1, npx, 0, None, codes.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    codes_ref, _, _ = oracle_mod.normalize(oracle_mod.encode(want, 0))
    exact, maxd = code_agreement(codes.cpu().numpy(), codes_ref.reshape(1, -1), True)
    assert exact >= 0.999 and maxd <= 1


def test_wrp_host_path_and_edge_cases(gpu_ctx, oracle_mod):
    import openholo_gb300 as oph
    z = np.load(os.path.join(GOLD, "wrp_3ch.npz"))
    cfg, _ = _cfgs(z, oracle_mod)
    v = np.ascontiguousarray(z["vertices"])
    dev = _generate(gpu_ctx, cfg, v)
    fields = [np.full((cfg.pixel_number[1], cfg.pixel_number[0], 2), np.nan) for _ in range(cfg.n_channels)]
    secs = gpu_ctx.wrp_generate_host(cfg, v.ctypes.data, v.shape[0], [f.ctypes.data for f in fields])
    assert secs > 0
    host = np.stack([f[..., 0] + 1j * f[..., 1] for f in fields])
    assert np.array_equal(host, dev)
    # no points: a zero field
    assert not np.any(_generate(gpu_ctx, cfg, np.zeros((0, 7))))
    # sizes the transform does not support, and random phase, are refused
    bad = oph.make_wrp_config(67, 45, 8e-6, 8e-6, [532e-9], wrp_location=1e-3, distance=0.01)
    with pytest.raises(oph.OphpcError) as e:
        _generate(gpu_ctx, bad, v)
    assert e.value.status == 6   # OPHPC_ERROR_UNSUPPORTED
    rp = oph.make_wrp_config(96, 72, 8e-6, 8e-6, [532e-9], wrp_location=1e-3, distance=0.01, random_phase=True)
    with pytest.raises(oph.OphpcError) as e:
        _generate(gpu_ctx, rp, v)
    assert e.value.status == 6
