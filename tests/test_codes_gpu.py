"""8-bit phase / amplitude codes without the FP64 encoded values (ophpc_encode
with d_encoded NULL): FP32 estimates decide most codes, FP64 the rest. The
codes must equal the FP64 path's bit for bit (the FP64 path runs when
d_encoded is given), on random fields, a generated hologram, fields with
exact zeros (pixels no window reaches) and degenerate ones. Fields up to
~7.8 million pixels take the single-pass kernel (estimates cached in shared
memory across a cooperative grid); the 9.4-million-pixel case takes the
three-pass kernels."""
import functools

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _codes(ctx, field, flag, with_fp64):
    import torch
    f = torch.from_numpy(np.ascontiguousarray(field)).cuda()
    nch, npx = field.shape[0], field.shape[1] * field.shape[2]
    codes = torch.empty((nch, npx), dtype=torch.uint8, device="cuda")
    enc = torch.empty((nch, npx), dtype=torch.float64, device="cuda") if with_fp64 else None
    ctx.encode(f.data_ptr(), nch, npx, flag, enc.data_ptr() if enc is not None else None, codes.data_ptr())
    torch.cuda.synchronize()
    return codes.cpu().numpy()


@functools.lru_cache(maxsize=1)
def _fields():
    rng = np.random.default_rng(7)
    out = {}
    out["large_3ch_three_pass"] = rng.normal(size=(3, 1536, 2048, 2))
    g = rng.normal(size=(3, 300, 401, 2))
    out["gaussian_3ch"] = g
    w = rng.normal(size=(1, 256, 256, 2)) * np.exp(rng.uniform(-6, 6, size=(1, 256, 256, 1)))
    out["wide_dynamic_range"] = w
    z = rng.normal(size=(2, 128, 160, 2))
    z[:, 40:90, 50:120, :] = 0.0
    z[:, 10:20, :, 1] = -0.0
    out["with_zeros"] = z
    c = np.zeros((1, 64, 64, 2))
    c[..., 0] = 1.0
    out["constant"] = c
    # a pixel count that is no multiple of 4: the single-pass kernel's last
    # group of four pixels is partial
    out["odd_size"] = rng.normal(size=(1, 123, 457, 2))
    return out


@pytest.mark.parametrize("flag", [0, 1])
@pytest.mark.parametrize("name", sorted(_fields()))
def test_codes_equal_fp64_path(gpu_ctx, name, flag):
    field = _fields()[name]
    fast = _codes(gpu_ctx, field, flag, False)
    exact = _codes(gpu_ctx, field, flag, True)
    assert np.array_equal(fast, exact), (name, flag, int(np.sum(fast != exact)))


def test_codes_of_a_generated_hologram(gpu_ctx):
    import torch

    import openholo_gb300 as oph
    rng = np.random.default_rng(8)
    n = 3000
    v = np.zeros((n, 7))
    v[:, 0:2] = rng.uniform(-1e-3, 1e-3, (n, 2))
    v[:, 2] = rng.uniform(0.3, 0.5, n)
    v[:, 3:6] = 1.0 - rng.uniform(0.0, 1.0, (n, 3))
    cfg = oph.make_config(pnx=512, pny=384, ppx=8e-6, ppy=8e-6, wavelengths=[638e-9, 532e-9, 473e-9])
    dv = torch.from_numpy(v).cuda()
    f = torch.empty((3, 384, 512, 2), dtype=torch.float64, device="cuda")
    gpu_ctx.generate(cfg, dv.data_ptr(), n, 0, 0x200, f.data_ptr(), 0)
    torch.cuda.synchronize()
    field = f.cpu().numpy()
    for flag in (0, 1):
        assert np.array_equal(_codes(gpu_ctx, field, flag, False), _codes(gpu_ctx, field, flag, True)), flag


def test_codes_into_unaligned_buffer(gpu_ctx):
    """A codes buffer that is not 4-byte aligned takes the three-pass
    kernels (the single-pass kernel stores four codes at a time): same
    codes."""
    import torch
    field = _fields()["gaussian_3ch"]
    want = _codes(gpu_ctx, field, 0, True)
    f = torch.from_numpy(np.ascontiguousarray(field)).cuda()
    nch, npx = field.shape[0], field.shape[1] * field.shape[2]
    raw = torch.zeros(nch * npx + 16, dtype=torch.uint8, device="cuda")
    for off in (1, 2, 3):
        gpu_ctx.encode(f.data_ptr(), nch, npx, 0, None, raw.data_ptr() + off)
        torch.cuda.synchronize()
        got = raw[off:off + nch * npx].cpu().numpy().reshape(nch, npx)
        assert np.array_equal(got, want), off
