"""Single-sideband encodings on the GPU (ophpc_encode_ssb) against the FP64
oracle (oracle.ssb_encode, itself checked against a loop-by-loop restatement
of the reference's code in tests/test_ssb_oracle.py).

FP64 FFTs on both sides (this library's Stockham passes, numpy's pocketfft):
m_lpEncoded within relL2 1e-10, 8-bit codes >= 99.99 % exact, at most
1 LSB apart.
"""
import numpy as np
import pytest

from tests._util import code_agreement, rel_l2

pytestmark = pytest.mark.gpu

SSB, OFFSSB = 7, 8


def _run(ctx, field, ppx, ppy, flag, passband=0, shift=(0.0, 0.5)):
    import torch
    nch, pny, pnx = field.shape
    f = torch.from_numpy(np.ascontiguousarray(field).view(np.float64).reshape(nch, pny, pnx, 2)).cuda()
    enc = torch.full((nch, pny * pnx), float("nan"), dtype=torch.float64, device="cuda")
    codes = torch.empty((nch, pny * pnx), dtype=torch.uint8, device="cuda")
    ctx.encode_ssb(f.data_ptr(), nch, pnx, pny, ppx, ppy, flag, passband, shift, enc.data_ptr(), codes.data_ptr(),
                   torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return enc.cpu().numpy().reshape(nch, pny, pnx), codes.cpu().numpy()


def _field(nch, pny, pnx, seed):
    rng = np.random.default_rng(seed)
    return rng.normal(size=(nch, pny, pnx)) + 1j * rng.normal(size=(nch, pny, pnx))


# even, odd, radix-7 and mixed sizes (every length factors into 2, 3, 5, 7)
SIZES = [(40, 24), (45, 27), (105, 49), (128, 36), (64, 63)]


@pytest.mark.parametrize("pnx,pny", SIZES)
@pytest.mark.parametrize("shift", [(0.0, 0.5), (0.25, -0.5)])
def test_ssb_matches_oracle(gpu_ctx, oracle_mod, pnx, pny, shift):
    field = _field(3, pny, pnx, pnx * 1000 + pny)
    enc, codes = _run(gpu_ctx, field, 8e-6, 6.4e-6, SSB, shift=shift)
    want = oracle_mod.ssb_encode(field, 8e-6, 6.4e-6, SSB, spectrum_shift=shift)
    assert rel_l2(enc, want) <= 1e-10
    codes_ref, _, _ = oracle_mod.normalize(want.reshape(3, -1))
    exact, maxd = code_agreement(codes, codes_ref.reshape(3, -1), False)
    assert exact >= 0.9999 and maxd <= 1


@pytest.mark.parametrize("pnx,pny", SIZES)
@pytest.mark.parametrize("passband", [0, 1, 2, 3])
def test_off_axis_ssb_matches_oracle(gpu_ctx, oracle_mod, pnx, pny, passband):
    field = _field(2, pny, pnx, pnx * 100 + pny * 10 + passband)
    enc, codes = _run(gpu_ctx, field, 8e-6, 8e-6, OFFSSB, passband)
    want = oracle_mod.ssb_encode(field, 8e-6, 8e-6, OFFSSB, passband)
    assert rel_l2(enc, want) <= 1e-10
    assert np.array_equal(enc[0], enc[1])          # channel 0's field into every channel
    assert enc.min() == 0.0 and enc.max() == 1.0
    codes_ref, _, _ = oracle_mod.normalize(want.reshape(2, -1))
    exact, maxd = code_agreement(codes, codes_ref.reshape(2, -1), False)
    assert exact >= 0.9999 and maxd <= 1


def test_ssb_of_a_generated_hologram(gpu_ctx, oracle_mod):
    """A 3-channel tensor-core RS hologram of 1920x1080 (the sphere_fhd
    geometry) through both encoders."""
    import torch

    import openholo_gb300 as oph
    from openholo_gb300 import workloads
    w = workloads.sphere_fhd().subset(2000)
    cfg = oph.make_config(**w.geometry_kwargs())
    dv = torch.from_numpy(w.vertices).cuda()
    f = torch.empty((3, w.pny, w.pnx, 2), dtype=torch.float64, device="cuda")
    gpu_ctx.generate(cfg, dv.data_ptr(), w.n_points, 0, oph.MODE_TENSOR_BF16X3, f.data_ptr(), 0)
    torch.cuda.synchronize()
    h = f.cpu().numpy()
    field = h[..., 0] + 1j * h[..., 1]
    for flag, pb in ((SSB, 0), (OFFSSB, 2)):
        enc, codes = _run(gpu_ctx, field, w.pp, w.pp, flag, pb)
        want = oracle_mod.ssb_encode(field, w.pp, w.pp, flag, pb)
        assert rel_l2(enc, want) <= 1e-10, flag
        codes_ref, _, _ = oracle_mod.normalize(want.reshape(3, -1))
        exact, maxd = code_agreement(codes, codes_ref.reshape(3, -1), False)
        assert exact >= 0.9999 and maxd <= 1, flag


def test_ssb_refuses_what_it_cannot_do(gpu_ctx):
    import openholo_gb300 as oph
    field = _field(1, 45, 67, 3)   # 67 is prime
    with pytest.raises(oph.OphpcError) as e:
        _run(gpu_ctx, field, 8e-6, 8e-6, SSB)
    assert e.value.status == 6
    field = _field(1, 24, 40, 3)
    with pytest.raises(oph.OphpcError) as e:
        _run(gpu_ctx, field, 8e-6, 8e-6, OFFSSB, 4)   # no such passband
    assert e.value.status == 1
    with pytest.raises(oph.OphpcError) as e:
        _run(gpu_ctx, field, 8e-6, 8e-6, 5)           # not an SSB flag
    assert e.value.status == 6


def test_facade_ssb_encoding(tmp_path, gpu_ctx, oracle_mod):
    """ophPointCloud::encoding(flag, passband) through the façade's C ABI,
    host buffers throughout: m_lpEncoded against the oracle on the façade's
    own complex_H, then normalize's 8-bit codes."""
    from openholo_gb300.pointcloud import PointCloud
    rng = np.random.default_rng(11)
    n = 300
    v = np.zeros((n, 7))
    v[:, 0:2] = rng.uniform(-1e-3, 1e-3, (n, 2))
    v[:, 2] = rng.uniform(0.3, 0.4, n)
    v[:, 3:6] = 1.0 - rng.uniform(0.0, 1.0, (n, 3))
    g = oracle_mod.Geometry(pnx=160, pny=96, ppx=8e-6, ppy=8e-6, wavelengths=[532e-9, 638e-9])
    xml = tmp_path / "cfg.xml"
    xml.write_text(g.xml())
    with PointCloud() as h:
        assert h.readConfig(str(xml))
        h.setPointCloudModel(v)
        h.SetMode(1)
        assert h.generateHologram(0) > 0.0, h.lastError()
        field = h.getComplexField()
        for flag, pb in ((SSB, 3), (OFFSSB, 1)):
            h.encoding(flag, pb)
            h.normalize()
            enc, codes = h.getEncodedBuffer(), h.getNormalizedBuffer()
            want = oracle_mod.ssb_encode(field, 8e-6, 8e-6, flag, pb)
            assert rel_l2(enc, want) <= 1e-10, flag
            codes_ref, _, _ = oracle_mod.normalize(want.reshape(2, -1))
            exact, maxd = code_agreement(codes.reshape(2, -1), codes_ref.reshape(2, -1), False)
            assert exact >= 0.9999 and maxd <= 1, flag


def _sideband(ctx, field, ppx, ppy, passband):
    import torch
    nch, pny, pnx = field.shape
    f = torch.from_numpy(np.ascontiguousarray(field).view(np.float64).reshape(nch, pny, pnx, 2)).cuda()
    enc = torch.full((nch, pny * pnx), float("nan"), dtype=torch.float64, device="cuda")
    codes = torch.empty((nch, pny * pnx), dtype=torch.uint8, device="cuda")
    ctx.encode_sideband(f.data_ptr(), nch, pnx, pny, ppx, ppy, passband, enc.data_ptr(), codes.data_ptr(),
                        torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return enc.cpu().numpy().reshape(nch, pny, pnx), codes.cpu().numpy()


def test_sideband_matches_reference_fixtures(gpu_ctx):
    """ophpc_encode_sideband against the reference's own encodeSideBand
    (tests/golden/sideband.npz), every passband."""
    import os
    z = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "sideband.npz"))
    names = sorted({k[:-len("_field")] for k in z.files if k.endswith("_field")})
    for name in names:
        pnx, pny, ppx, ppy = z[name + "_geom"]
        for pb in range(4):
            want = z[f"{name}_enc{pb}"]
            got, _ = _sideband(gpu_ctx, z[name + "_field"], float(ppx), float(ppy), pb)
            assert rel_l2(got, want) <= 1e-12, (name, pb)


@pytest.mark.parametrize("pnx,pny", [(128, 36), (105, 49), (1920, 1080)])
@pytest.mark.parametrize("passband", [0, 1, 2, 3])
def test_sideband_matches_oracle(gpu_ctx, oracle_mod, pnx, pny, passband):
    field = _field(2, pny, pnx, pnx + pny + passband)
    enc, codes = _sideband(gpu_ctx, field, 8e-6, 8e-6, passband)
    want = oracle_mod.sideband_encode(field, 8e-6, 8e-6, passband)
    assert rel_l2(enc, want) <= 1e-10
    codes_ref, _, _ = oracle_mod.normalize(want.reshape(2, -1))
    exact, maxd = code_agreement(codes, codes_ref.reshape(2, -1), False)
    assert exact >= 0.9999 and maxd <= 1


def test_ssb_encoders_on_an_empty_field(gpu_ctx, oracle_mod):
    """A field of zeros (no point reached the SLM): every encoder returns
    what the oracle returns, all finite (oph::normalize's max starts at
    MIN_DOUBLE, so a constant field normalises to 0, not NaN)."""
    field = np.zeros((2, 27, 40), dtype=np.complex128)
    for flag, pb in ((SSB, 0), (OFFSSB, 1), (OFFSSB, 3)):
        enc, codes = _run(gpu_ctx, field, 8e-6, 8e-6, flag, pb)
        want = oracle_mod.ssb_encode(field, 8e-6, 8e-6, flag, pb)
        assert np.all(np.isfinite(enc)) and np.array_equal(enc, want), (flag, pb)
        assert not np.any(codes)
    for pb in range(4):
        enc, _ = _sideband(gpu_ctx, field, 8e-6, 8e-6, pb)
        assert not np.any(enc)
