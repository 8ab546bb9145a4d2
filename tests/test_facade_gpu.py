"""The ophPointCloud façade driven with the reference's own call sequence
(Example/examPointCloud/examPointCloud.cpp:54-132) against the goldens the
reference produced (tests/golden/make_golden.py). Same tolerances as
tests/test_gpu_parity.py: field relL2 <= 1e-4, 8-bit codes exact on >= 99.9%
of pixels and within +-1 LSB (phase circular)."""
import os

import numpy as np
import pytest

from openholo_gb300 import pointcloud as P
from tests._util import code_agreement, rel_l2

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _xml(tmp_path, text, name="cfg.xml"):
    p = tmp_path / name
    p.write_text(text)
    return str(p)


@pytest.mark.parametrize("name", ["rs_window_1ch", "fresnel_window_1ch", "rs_3ch_vw", "fresnel_3ch"])
def test_facade_reference_sequence(tmp_path, gpu_ctx, name):
    d = np.load(os.path.join(GOLD, name + ".npz"))
    with P.PointCloud() as h:
        assert h.readConfig(_xml(tmp_path, str(d["xml"])))
        h.setPointCloudModel(d["vertices"])
        h.setViewingWindow(bool(d["viewing_window"]))
        h.SetMode(1)
        secs = h.generateHologram(int(d["diff_flag"]))
        assert secs > 0.0, h.lastError()
        f = h.getComplexField()
        assert rel_l2(f, d["field"]) <= 1e-4
        for flag, enc_key, codes_key, circ in ((0, "enc_phase", "codes_phase", True),
                                              (1, "enc_amp", "codes_amp", False)):
            h.encoding(flag)
            h.normalize()
            exact, maxd = code_agreement(h.getNormalizedBuffer(), d[codes_key], circ)
            assert exact >= 0.999 and maxd <= 1, (flag, exact, maxd)


def test_facade_encoding_reads_host_buffer(tmp_path, gpu_ctx):
    """encoding() encodes what getComplexField() holds, like the reference."""
    d = np.load(os.path.join(GOLD, "rs_window_1ch.npz"))
    with P.PointCloud() as h:
        assert h.readConfig(_xml(tmp_path, str(d["xml"])))
        h.setPointCloudModel(d["vertices"])
        h.generateHologram(0)
        h.encoding(1)
        a = h.getEncodedBuffer()
        f = h.getComplexField()
        assert rel_l2(a, np.abs(f)) < 1e-15


def test_facade_ply_path(tmp_path, gpu_ctx):
    d = np.load(os.path.join(GOLD, "ply_generate_rs.npz"))
    with P.PointCloud() as h:
        assert h.readConfig(_xml(tmp_path, str(d["xml"])))
        assert h.loadPointCloud(os.path.join(GOLD, "ply_ascii_channel.ply")) == 64
        h.generateHologram(0)
        assert rel_l2(h.getComplexField(), d["field"]) <= 1e-4
        h.encoding(0)
        h.normalize()
        exact, maxd = code_agreement(h.getNormalizedBuffer(), d["codes_phase"], True)
        assert exact >= 0.999 and maxd <= 1


@pytest.mark.parametrize("name", ["bmp_1ch_w96", "bmp_1ch_w90", "bmp_3ch_merge"])
def test_facade_save_bmp(tmp_path, gpu_ctx, name):
    d = np.load(os.path.join(GOLD, name + ".npz"))
    ref = open(os.path.join(GOLD, name + ".bmp"), "rb").read()
    with P.PointCloud() as h:
        assert h.readConfig(_xml(tmp_path, str(d["xml"])))
        h.setPointCloudModel(d["vertices"])
        h.generateHologram(0)
        h.encoding(0)
        h.normalize()
        out = str(tmp_path / "holo")       # no extension: ".bmp" appended
        assert h.save(out, int(d["bpp"]))
        got = open(out + ".bmp", "rb").read()
    assert len(got) == len(ref)
    hdr = 54 + (1024 if int(d["bpp"]) == 8 else 0)
    assert got[:hdr] == ref[:hdr]
    a = np.frombuffer(got[hdr:], np.uint8).astype(int)
    b = np.frombuffer(ref[hdr:], np.uint8).astype(int)
    dd = np.abs((a - b + 128) % 256 - 128)
    assert np.mean(dd == 0) >= 0.999 and dd.max() <= 1
