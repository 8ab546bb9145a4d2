"""GPU parity on the reference's own example fixtures
(Example/dataset/Dice/PointCloud: Dice_PointCloud.xml + dice_100000.ply,
7,493 points on a 1920x1080, 4.3 um SLM; Openholo_python/test/
PointCloud_Dice_RGB.ply, 1,461 points, in three colours), against the
reference CPU path's output stored in tests/golden/dice*.npz: the complex
field at 16,384 seeded pixels (relL2 <= 1e-4), the 8-bit phase and
amplitude codes there (>= 99.9% exact, +-1 LSB elsewhere, phase circular)
and the normalisation range. The config goes through the XML reader and the
field through both the C ABI and the ophPointCloud facade."""
import os

import numpy as np
import pytest

from openholo_gb300 import pointcloud as P
from tests._util import code_agreement, rel_l2, run_encode

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FIELD_TOL = 1e-4
CODE_EXACT = 0.999


def _config(tmp_path, xml):
    p = tmp_path / "dice.xml"
    p.write_text(xml)
    st, cfg, _ = P.read_config(str(p))
    assert st == 0
    return cfg, str(p)


def _device_field(ctx, cfg, vertices, diff, mode=0):
    import torch
    nch, pny, pnx = cfg.n_channels, cfg.pixel_number[1], cfg.pixel_number[0]
    dv = torch.from_numpy(np.ascontiguousarray(vertices)).cuda()
    f = torch.empty((nch, pny, pnx, 2), dtype=torch.float64, device="cuda")
    ctx.generate(cfg, dv.data_ptr(), vertices.shape[0], diff, mode, f.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    h = f.cpu().numpy()
    return h[..., 0] + 1j * h[..., 1]


def _check(ctx, field, d, pre):
    idx = d[pre + "pixel_index"]
    nch = field.shape[0]
    flat = field.reshape(nch, -1)
    assert rel_l2(flat[:, idx], d[pre + "field_at"]) <= FIELD_TOL
    for flag, name, circ in ((0, "phase", True), (1, "amp", False)):
        enc, codes = run_encode(ctx, field, flag)
        lo, hi = d[f"{pre}enc_{name}_range"]
        assert abs(enc.min() - lo) <= 1e-6 * max(1.0, abs(lo)) + 1e-3 * (hi - lo)
        assert abs(enc.max() - hi) <= 1e-3 * (hi - lo)
        exact, maxd = code_agreement(codes.reshape(nch, -1)[:, idx], d[f"{pre}codes_{name}_at"], circ)
        assert exact >= CODE_EXACT and maxd <= 1, (pre, name, exact, maxd)


# mode 0x200 (OPHPC_MODE_TENSOR_BF16X3): RS and Fresnel on the tensor cores.
# The Dice's anti-aliasing windows cut most 128x128 tiles, so for RS most
# pairs go to the FP32-core complement and the two kernels' split is tested
# against the reference's own output.
@pytest.mark.parametrize("diff,tag,mode", [(0, "rs", 0), (1, "fresnel", 0), (0, "rs", 0x200), (1, "fresnel", 0x200)])
def test_dice_through_c_abi(tmp_path, gpu_ctx, diff, tag, mode):
    d = np.load(os.path.join(GOLD, "dice.npz"))
    cfg, _ = _config(tmp_path, str(d["xml"]))
    assert (cfg.pixel_number[0], cfg.pixel_number[1], cfg.n_channels) == (1920, 1080, 1)
    _check(gpu_ctx, _device_field(gpu_ctx, cfg, d["vertices"], diff, mode), d, tag + "_")


@pytest.mark.parametrize("mode", [1, 1 | 0x200])
def test_dice_rgb_through_facade(tmp_path, gpu_ctx, mode):
    d = np.load(os.path.join(GOLD, "dice_rgb.npz"))
    _, xml = _config(tmp_path, str(d["xml"]))
    with P.PointCloud() as h:
        assert h.readConfig(xml)
        h.setPointCloudModel(d["vertices"])
        h.SetMode(mode)
        assert h.generateHologram(0) > 0.0, h.lastError()
        field = h.getComplexField()
        assert field.shape == (3, 1080, 1920)
        _check(gpu_ctx, field, d, "")
        # the facade's own encode + normalise give the same codes
        h.encoding(0)
        h.normalize()
        idx = d["pixel_index"]
        exact, maxd = code_agreement(h.getNormalizedBuffer().reshape(3, -1)[:, idx], d["codes_phase_at"], True)
        assert exact >= CODE_EXACT and maxd <= 1
