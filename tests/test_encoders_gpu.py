"""Device encoders beyond phase/amplitude (ophGen.cpp:1821-1974) against the
reference's own output on the same fields (tests/golden/encoders_*.npz):
Real, Imaginary, SimpleNI, Burckhardt and TwoPhase, then normalize.

Encoded values may differ from the reference's in the last bits where a
device sin / cos / atan2 / acos rounds differently from the host libm
(tolerance below); the 8-bit codes must match on >= 99.9% of pixels and
within 1 LSB elsewhere."""
import os

import numpy as np
import pytest

from tests._util import code_agreement, run_encode

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FLAGS = (2, 3, 4, 5, 6)
# a few ulps of the value: libm-vs-device differences of the transcendental
# functions, carried through at most a multiply and an add
ENC_TOL = 8 * np.finfo(np.float64).eps


def _cases():
    f3 = np.load(os.path.join(GOLD, "fresnel_3ch.npz"))["field"]
    g3 = np.load(os.path.join(GOLD, "encoders_3ch.npz"))
    g1 = np.load(os.path.join(GOLD, "encoders_odd_1ch.npz"))
    return (("3ch_80x48", f3, g3), ("1ch_41x23", g1["field"], g1))


def _check(enc, codes, enc_ref, codes_ref, what):
    scale = np.maximum(1.0, np.abs(enc_ref))
    assert np.all(np.abs(enc - enc_ref) <= ENC_TOL * scale), what
    exact, maxd = code_agreement(codes, codes_ref, circular=False)
    assert exact >= 0.999 and maxd <= 1, (what, exact, maxd)


@pytest.mark.parametrize("flag", FLAGS)
def test_device_encoders_match_reference(gpu_ctx, flag):
    for name, field, gold in _cases():
        enc, codes = run_encode(gpu_ctx, field, flag)
        _check(enc, codes, gold[f"enc_{flag}"], gold[f"codes_{flag}"], f"{name} flag {flag}")


def test_partial_encoders_keep_earlier_entries(gpu_ctx, oracle_mod):
    """Burckhardt after Phase and TwoPhase after Amplitude on a 943-pixel
    field: the entries they skip keep the earlier encoding."""
    g1 = np.load(os.path.join(GOLD, "encoders_odd_1ch.npz"))
    for flag, pre in ((5, 0), (6, 1)):
        prior, _ = run_encode(gpu_ctx, g1["field"], pre)
        enc, codes = run_encode(gpu_ctx, g1["field"], flag, prior=prior)
        _check(enc, codes, g1[f"enc_{flag}_after_{pre}"], g1[f"codes_{flag}_after_{pre}"], f"{flag} after {pre}")


def test_partial_encoder_without_encoded_buffer(gpu_ctx):
    """d_encoded NULL: skipped entries count as 0 (the state right after
    generateHologram) and the codes match the reference's."""
    import torch
    g1 = np.load(os.path.join(GOLD, "encoders_odd_1ch.npz"))
    f = np.ascontiguousarray(g1["field"])
    npx = f[0].size
    df = torch.from_numpy(f.view(np.float64).reshape(1, npx, 2)).cuda()
    nrm = torch.empty((1, npx), dtype=torch.uint8, device="cuda")
    for flag in (4, 5, 6):
        gpu_ctx.encode(df.data_ptr(), 1, npx, flag, None, nrm.data_ptr(), torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        exact, maxd = code_agreement(nrm.cpu().numpy().reshape(f.shape), g1[f"codes_{flag}"], circular=False)
        assert exact >= 0.999 and maxd <= 1


def test_facade_encoders_through_ohc(tmp_path, gpu_ctx):
    """The ophPointCloud façade: loadAsOhc a field, encoding(flag),
    normalize, compare with the reference; Burckhardt after Phase keeps the
    phase values where it writes nothing."""
    from openholo_gb300 import pointcloud as P
    g1 = np.load(os.path.join(GOLD, "encoders_odd_1ch.npz"))
    path = str(tmp_path / "f.ohc")
    P.save_ohc(path, g1["field"], (8e-6, 8e-6), [532e-9])
    for flag in (4, 5, 6):
        with P.PointCloud() as h:
            assert h.loadAsOhc(path)
            h.encoding(flag)
            h.normalize()
            _check(h.getEncodedBuffer(), h.getNormalizedBuffer(), g1[f"enc_{flag}"], g1[f"codes_{flag}"],
                   f"facade {flag}")
    with P.PointCloud() as h:
        assert h.loadAsOhc(path)
        h.encoding(0)
        h.normalize()
        h.encoding(5)
        h.normalize()
        _check(h.getEncodedBuffer(), h.getNormalizedBuffer(), g1["enc_5_after_0"], g1["codes_5_after_0"],
               "facade 5 after 0")


def test_unsupported_encoder_flags(gpu_ctx):
    import torch

    from openholo_gb300 import OphpcError
    df = torch.zeros((1, 16, 2), dtype=torch.float64, device="cuda")
    enc = torch.zeros((1, 16), dtype=torch.float64, device="cuda")
    for flag in (7, 8, 9, 10):   # SSB, off-axis SSB, binary, error-diffusion binary
        with pytest.raises(OphpcError):
            gpu_ctx.encode(df.data_ptr(), 1, 16, flag, enc.data_ptr(), None, 0)
