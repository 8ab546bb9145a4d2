"""Pins the CPU oracle (oracle/ophpc_oracle.c) to the reference itself.

The fixtures in tests/golden/ were produced by the reference's own CPU path
compiled from its sources (tests/golden/make_golden.py). The oracle must
reproduce them to double-precision summation-order noise, which is what makes
it a valid checker for the GPU parity tests.
"""
import os
import xml.etree.ElementTree as ET

import numpy as np
import pytest

from tests._util import code_agreement, rel_l2

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FIELD_CASES = ["rs_window_1ch", "fresnel_window_1ch", "rs_3ch_vw", "fresnel_3ch"]


def geometry_from_xml(oracle_mod, text, viewing_window=False):
    root = ET.fromstring(text)
    f = lambda k, d=None: float(root.find(k).text) if root.find(k) is not None else d  # noqa: E731
    nw = int(root.find("SLM_WaveNum").text)
    return oracle_mod.Geometry(
        pnx=int(root.find("SLM_PixelNumX").text), pny=int(root.find("SLM_PixelNumY").text),
        ppx=f("SLM_PixelPitchX"), ppy=f("SLM_PixelPitchY"),
        wavelengths=[f(f"SLM_WaveLength_{i + 1}") for i in range(nw)],
        scale=(f("ScaleX"), f("ScaleY"), f("ScaleZ")), distance=f("Distance"),
        field_length=f("FieldLength", 0.0), viewing_window=viewing_window)


@pytest.mark.parametrize("name", FIELD_CASES)
def test_oracle_matches_reference_field(oracle_mod, name):
    d = np.load(os.path.join(GOLD, name + ".npz"))
    g = geometry_from_xml(oracle_mod, str(d["xml"]), bool(d["viewing_window"]))
    got = oracle_mod.generate(g, d["vertices"], int(d["diff_flag"]))
    assert got.shape == d["field"].shape
    assert rel_l2(got, d["field"]) < 1e-13


@pytest.mark.parametrize("name", FIELD_CASES)
def test_oracle_encode_normalize_bit_exact(oracle_mod, name):
    d = np.load(os.path.join(GOLD, name + ".npz"))
    for flag, enc_key, codes_key in ((0, "enc_phase", "codes_phase"), (1, "enc_amp", "codes_amp")):
        enc = oracle_mod.encode(d["field"], flag)
        assert np.array_equal(enc, d[enc_key])
        codes, _, _ = oracle_mod.normalize(enc)
        assert np.array_equal(codes, d[codes_key])


@pytest.mark.parametrize("name", FIELD_CASES)
def test_oracle_codes_from_own_field(oracle_mod, name):
    """Codes from the oracle's own field (summation order differs from the
    reference's OpenMP atomics) agree on all but boundary-straddling pixels."""
    d = np.load(os.path.join(GOLD, name + ".npz"))
    g = geometry_from_xml(oracle_mod, str(d["xml"]), bool(d["viewing_window"]))
    f = oracle_mod.generate(g, d["vertices"], int(d["diff_flag"]))
    codes, _, _ = oracle_mod.normalize(oracle_mod.encode(f, 0))
    exact, maxd = code_agreement(codes, d["codes_phase"], circular=True)
    assert exact >= 0.9999 and maxd <= 1


@pytest.mark.parametrize("name", FIELD_CASES)
def test_pixel_gather_matches_reference(oracle_mod, name):
    d = np.load(os.path.join(GOLD, name + ".npz"))
    g = geometry_from_xml(oracle_mod, str(d["xml"]), bool(d["viewing_window"]))
    ref = d["field"]
    rng = np.random.default_rng(3)
    idx = rng.choice(g.pnx * g.pny, 200, replace=False)
    for ch in range(g.n_channels):
        got = oracle_mod.field_at(g, d["vertices"], int(d["diff_flag"]), ch, idx)
        assert rel_l2(got, ref[ch].reshape(-1)[idx]) < 1e-13


def test_rs_1k_crop(oracle_mod):
    d = np.load(os.path.join(GOLD, "rs_1k_crop.npz"))
    g = geometry_from_xml(oracle_mod, str(d["xml"]))
    got = oracle_mod.field_at(g, d["vertices"], 0, 0, d["pixel_index"])
    assert rel_l2(got, d["field_at"]) < 1e-13


def test_ply_generate(oracle_mod):
    """The reference's loadPointCloud -> generate chain on a PLY fixture."""
    d = np.load(os.path.join(GOLD, "ply_generate_rs.npz"))
    verts = np.load(os.path.join(GOLD, "ply_vertices.npz"))["ply_ascii_channel"]
    g = geometry_from_xml(oracle_mod, str(d["xml"]))
    got = oracle_mod.generate(g, verts, 0)
    assert rel_l2(got, d["field"]) < 1e-13


def test_window_is_exercised(oracle_mod):
    """The window fixtures really clip: a single point's field is zero outside
    its window rectangle."""
    d = np.load(os.path.join(GOLD, "rs_window_1ch.npz"))
    g = geometry_from_xml(oracle_mod, str(d["xml"]))
    f = oracle_mod.generate(g, d["vertices"][:1], 0)
    frac = np.mean(f == 0)
    assert 0.2 < frac < 1.0


def test_normalize_edge_cases(oracle_mod):
    # all-zero encoded values: max stays MIN_DOUBLE, gap = MIN_DOUBLE -> code 0
    codes, mn, mx = oracle_mod.normalize(np.zeros((1, 10)))
    assert mn == 0.0 and mx == 2.2250738585072014e-308 and not codes.any()
    # negative values never raise the max above MIN_DOUBLE (maxOfArr semantics)
    codes, mn, mx = oracle_mod.normalize(-np.arange(1.0, 5.0).reshape(1, 4))
    assert mx == 2.2250738585072014e-308 and mn == -4.0
    assert codes.tolist() == [[191, 128, 64, 0]]


ENCODER_FLAGS = (2, 3, 4, 5, 6)


def test_oracle_encoders_match_reference(oracle_mod):
    """Real, Imaginary, SimpleNI, Burckhardt and TwoPhase + normalize,
    bit-exact against the reference's own output on the same fields."""
    f3 = np.load(os.path.join(GOLD, "fresnel_3ch.npz"))["field"]
    g3 = np.load(os.path.join(GOLD, "encoders_3ch.npz"))
    g1 = np.load(os.path.join(GOLD, "encoders_odd_1ch.npz"))
    for field, gold in ((f3, g3), (g1["field"], g1)):
        for flag in ENCODER_FLAGS:
            enc = oracle_mod.encode(field, flag)
            assert np.array_equal(enc, gold[f"enc_{flag}"], equal_nan=True), flag
            codes, _, _ = oracle_mod.normalize(enc)
            assert np.array_equal(codes, gold[f"codes_{flag}"]), flag
    # Burckhardt after Phase, TwoPhase after Amplitude: skipped entries keep
    # the earlier encoding (943 pixels: neither 2 nor 3 divides the count)
    for flag, pre in ((5, 0), (6, 1)):
        enc = oracle_mod.encode(g1["field"], flag, prior=oracle_mod.encode(g1["field"], pre))
        assert np.array_equal(enc, g1[f"enc_{flag}_after_{pre}"])
        codes, _, _ = oracle_mod.normalize(enc)
        assert np.array_equal(codes, g1[f"codes_{flag}_after_{pre}"])


@pytest.mark.parametrize("name,tags", [("dice", ("rs", "fresnel")), ("dice_rgb", ("",))])
def test_oracle_matches_reference_on_dice_fixtures(oracle_mod, name, tags):
    """The reference's own example fixtures (Dice 1920x1080, 7,493 points;
    Dice RGB, 1,461 points in three colours): the oracle's pixel gather at
    16,384 seeded pixels against the reference's CPU field there."""
    d = np.load(os.path.join(GOLD, name + ".npz"))
    g = geometry_from_xml(oracle_mod, str(d["xml"]))
    for tag in tags:
        pre = f"{tag}_" if tag else ""
        diff = 1 if tag == "fresnel" else 0
        want = d[pre + "field_at"]
        for ch in range(want.shape[0]):
            got = oracle_mod.field_at(g, d["vertices"], diff, ch, d[pre + "pixel_index"])
            assert rel_l2(got, want[ch]) < 1e-12, (tag, ch)


def test_dice_ply_files_parse_as_reference(oracle_mod):
    """Our PLY loader on the reference's example files gives the vertices
    its parser gave (needs the reference tree; skipped elsewhere)."""
    from openholo_gb300 import pointcloud as P
    paths = {"dice": ("Example", "dataset", "Dice", "PointCloud", "dice_100000.ply"),
             "dice_rgb": ("Openholo_python", "test", "PointCloud_Dice_RGB.ply")}
    for name, parts in paths.items():
        path = os.path.join(oracle_mod.REFERENCE_TREE, *parts)
        if not os.path.exists(path):
            pytest.skip("reference tree not present")
        assert np.array_equal(P.load_ply(path), np.load(os.path.join(GOLD, name + ".npz"))["vertices"])
