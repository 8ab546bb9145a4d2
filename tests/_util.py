"""Shared comparison helpers for the parity tests."""
from __future__ import annotations

import numpy as np


def rel_l2(a: np.ndarray, ref: np.ndarray) -> float:
    den = float(np.linalg.norm(ref))
    return float(np.linalg.norm(a - ref)) / (den if den > 0 else 1.0)


def code_agreement(codes: np.ndarray, ref: np.ndarray, circular: bool):
    """(fraction exact, max |difference| in LSB); phase codes wrap 255 <-> 0."""
    d = codes.astype(np.int32) - ref.astype(np.int32)
    if circular:
        d = (d + 128) % 256 - 128
    ad = np.abs(d)
    return float(np.mean(ad == 0)), int(ad.max()) if ad.size else 0


def run_generate(ctx, geom_kwargs: dict, vertices: np.ndarray, diff_flag: int, mode: int = 0,
                 offset=(0, 0), viewing_window=False, field_length=0.0):
    """Device path through the C ABI; returns complex128 [nch, pny, pnx]."""
    import torch

    import openholo_gb300 as oph
    cfg = oph.make_config(offset=offset, viewing_window=viewing_window, field_length=field_length,
                          **geom_kwargs)
    nch = len(geom_kwargs["wavelengths"])
    pnx, pny = geom_kwargs["pnx"], geom_kwargs["pny"]
    dv = torch.from_numpy(np.ascontiguousarray(vertices, dtype=np.float64)).cuda()
    field = torch.empty((nch, pny, pnx, 2), dtype=torch.float64, device="cuda")
    ctx.generate(cfg, dv.data_ptr() if dv.numel() else 0, vertices.shape[0], diff_flag, mode,
                 field.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    f = field.cpu().numpy()
    return f[..., 0] + 1j * f[..., 1]


def run_encode(ctx, field: np.ndarray, encode_flag: int, prior=None):
    """Device encode + normalise of a complex128 [nch, ...] field; `prior`
    (default zeros) is what the encoded buffer holds before the call."""
    import torch
    nch = field.shape[0]
    npx = field[0].size
    f = np.ascontiguousarray(field, dtype=np.complex128)
    df = torch.from_numpy(f.view(np.float64).reshape(nch, npx, 2)).cuda()
    enc = torch.zeros((nch, npx), dtype=torch.float64, device="cuda")
    if prior is not None:
        enc.copy_(torch.from_numpy(np.ascontiguousarray(prior, dtype=np.float64).reshape(nch, npx)))
    nrm = torch.empty((nch, npx), dtype=torch.uint8, device="cuda")
    ctx.encode(df.data_ptr(), nch, npx, encode_flag, enc.data_ptr(), nrm.data_ptr(),
               torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return enc.cpu().numpy().reshape(field.shape), nrm.cpu().numpy().reshape(field.shape)
