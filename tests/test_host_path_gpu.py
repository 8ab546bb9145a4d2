"""The host-buffer entry points against the CPU oracle.

ophpc_generate_host is what genCghPointCloudGPU does end to end
(ophgen/src/ophPointCloud_GPU.cpp:218-286): host Vertex records in, one host
Complex<double> buffer per channel out (complex_H[ch]). The façade sequence
generateHologram -> encoding -> normalize (ophgen/src/ophPointCloud.cpp:151-191,
ophgen/src/ophGen.cpp:816-849, 654-687) is what a reference caller sees. Both
are checked here against the FP64 oracle: fields within relL2 1e-4, 8-bit
codes >= 99.9 % exact and within +-1 LSB (phase codes wrap around)."""
import ctypes

import numpy as np
import pytest

from tests._util import code_agreement, rel_l2

pytestmark = pytest.mark.gpu

FIELD_TOL = 1e-4


def _points(n, seed, nch=3, z=(0.2, 0.3)):
    rng = np.random.default_rng(seed)
    v = np.zeros((n, 7))
    v[:, 0] = rng.uniform(-1e-3, 1e-3, n)
    v[:, 1] = rng.uniform(-1e-3, 1e-3, n)
    v[:, 2] = rng.uniform(z[0], z[1], n)
    v[:, 3:6] = 1.0 - rng.uniform(0.0, 1.0, (n, 3))
    return v


GEOM = dict(pnx=200, pny=136, ppx=8e-6, ppy=8e-6, wavelengths=[638e-9, 532e-9, 473e-9])


@pytest.mark.parametrize("diff,mode", [(0, 0), (0, 0x200), (1, 0), (1, 0x200)])
def test_generate_host_matches_oracle(gpu_ctx, oracle_mod, diff, mode):
    import openholo_gb300 as oph
    v = _points(700, 11 + diff)
    cfg = oph.make_config(**GEOM)
    nch, pnx, pny = 3, GEOM["pnx"], GEOM["pny"]
    # one separate host buffer per channel, filled with NaN: every entry must be written
    fields = [np.full((pny, pnx, 2), np.nan) for _ in range(nch)]
    hv = np.ascontiguousarray(v)
    secs = gpu_ctx.generate_host(cfg, hv.ctypes.data, v.shape[0], diff, mode, [f.ctypes.data for f in fields])
    assert secs > 0.0
    got = np.stack([f[..., 0] + 1j * f[..., 1] for f in fields])
    want = oracle_mod.generate(oracle_mod.Geometry(**GEOM), v, diff)
    err = rel_l2(got, want)
    assert err <= FIELD_TOL, f"diff={diff} mode={mode:#x}: relL2 {err:.3e}"


def test_generate_host_without_points_writes_zeros(gpu_ctx):
    import openholo_gb300 as oph
    cfg = oph.make_config(**GEOM)
    fields = [np.full((GEOM["pny"], GEOM["pnx"], 2), np.nan) for _ in range(3)]
    gpu_ctx.generate_host(cfg, 0, 0, 0, 0, [f.ctypes.data for f in fields])
    assert all(bool((f == 0).all()) for f in fields)


def test_generate_host_rejects_missing_channel_buffer(gpu_ctx):
    import openholo_gb300 as oph
    cfg = oph.make_config(**GEOM)
    v = np.ascontiguousarray(_points(10, 3))
    f0 = np.zeros((GEOM["pny"], GEOM["pnx"], 2))
    with pytest.raises(oph.OphpcError) as e:
        gpu_ctx.generate_host(cfg, v.ctypes.data, 10, 0, 0, [f0.ctypes.data, 0, 0])
    assert e.value.status == 1   # OPHPC_ERROR_INVALID_ARGUMENT


@pytest.mark.parametrize("encode_flag", [0, 1])
def test_facade_sequence_matches_oracle(tmp_path, gpu_ctx, oracle_mod, encode_flag):
    """generateHologram (tensor-core RS) -> encoding -> normalize through the
    façade's C ABI, host buffers throughout, against the oracle's field,
    encoding and 8-bit codes."""
    from openholo_gb300.pointcloud import PointCloud
    v = _points(600, 21)
    g = oracle_mod.Geometry(**GEOM)
    xml = tmp_path / "cfg.xml"
    xml.write_text(g.xml())
    with PointCloud() as h:
        assert h.readConfig(str(xml))
        h.setPointCloudModel(v)
        h.SetMode(1 | 0x200)
        assert h.generateHologram(0) > 0.0, h.lastError()
        h.encoding(encode_flag)
        h.normalize()
        field, enc, codes = h.getComplexField(), h.getEncodedBuffer(), h.getNormalizedBuffer()
    want = oracle_mod.generate(g, v, 0)
    assert rel_l2(field, want) <= FIELD_TOL
    enc_ref = oracle_mod.encode(want, encode_flag)
    codes_ref, _, _ = oracle_mod.normalize(enc_ref)
    exact, maxd = code_agreement(codes, codes_ref.reshape(codes.shape), encode_flag == 0)
    assert exact >= 0.999 and maxd <= 1, (exact, maxd)
