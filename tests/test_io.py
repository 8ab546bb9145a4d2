"""Host-side files of the path (no GPU): PLY loader, XML config reader, BMP
writer, each against what the reference itself produced (tests/golden/)."""
import os
import struct

import numpy as np
import pytest

from openholo_gb300 import pointcloud as P

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.mark.parametrize("name", ["ply_ascii_channel", "ply_ascii_nochannel", "ply_binary_channel"])
def test_ply_matches_reference_parser(name):
    want = np.load(os.path.join(GOLD, "ply_vertices.npz"))[name]
    got = P.load_ply(os.path.join(GOLD, name + ".ply"))
    assert got.shape == want.shape
    assert np.array_equal(got, want)


def test_ply_faces_match_reference_parser():
    """Face colours (a list property before them) land on the vertices."""
    want = np.load(os.path.join(GOLD, "ply_faces.npz"))["ply_binary_faces"]
    assert np.array_equal(P.load_ply(os.path.join(GOLD, "ply_binary_faces.ply")), want)


def _binary_ply(path, xyz, rgb, extra_double=False, truncate=0):
    """binary_little_endian vertices: float x y z, [double nx unused],
    uchar red green blue, float phase; optionally cut short."""
    n = xyz.shape[0]
    props = "property float x\nproperty float y\nproperty float z\n"
    if extra_double:
        props += "property double nx\n"
    props += "property uchar red\nproperty uchar green\nproperty uchar blue\nproperty float phase\n"
    hdr = (f"ply\nformat binary_little_endian 1.0\nelement color 1\nproperty int channel\n"
           f"element vertex {n}\n{props}end_header\n").encode()
    fields = [("x", "<f4"), ("y", "<f4"), ("z", "<f4")] + ([("nx", "<f8")] if extra_double else []) + \
             [("r", "u1"), ("g", "u1"), ("b", "u1"), ("p", "<f4")]
    rec = np.zeros(n, dtype=fields)
    rec["x"], rec["y"], rec["z"] = xyz[:, 0], xyz[:, 1], xyz[:, 2]
    rec["r"], rec["g"], rec["b"] = rgb[:, 0], rgb[:, 1], rgb[:, 2]
    rec["p"] = np.linspace(0, 6, n, dtype=np.float32)
    body = struct.pack("<i", 3) + rec.tobytes()
    with open(path, "wb") as f:
        f.write(hdr + body[:len(body) - truncate])
    return rec


@pytest.mark.parametrize("extra_double", [False, True])
def test_ply_binary_bulk_decode(tmp_path, extra_double):
    """200,000 records (decoded in parallel ranges), with and without a
    property the vertex does not use between the coordinates and colours."""
    rng = np.random.default_rng(21)
    n = 200_000
    xyz = rng.uniform(-1, 1, (n, 3)).astype(np.float32)
    rgb = rng.integers(0, 256, (n, 3)).astype(np.uint8)
    rec = _binary_ply(tmp_path / "b.ply", xyz, rgb, extra_double)
    got = P.load_ply(str(tmp_path / "b.ply"))
    assert got.shape == (n, 7)
    assert np.array_equal(got[:, :3], xyz.astype(np.float64))
    assert np.array_equal(got[:, 3:6], (rgb.astype(np.float32) / np.float32(255.0)).astype(np.float64))
    assert np.array_equal(got[:, 6], rec["p"].astype(np.float64))


def test_ply_truncated_data_fails(tmp_path):
    rng = np.random.default_rng(22)
    xyz = rng.uniform(-1, 1, (100, 3)).astype(np.float32)
    rgb = rng.integers(0, 256, (100, 3)).astype(np.uint8)
    _binary_ply(tmp_path / "t.ply", xyz, rgb, truncate=5)
    with pytest.raises(Exception):
        P.load_ply(str(tmp_path / "t.ply"))
    with P.PointCloud() as h:
        assert h.loadPointCloud(str(tmp_path / "t.ply")) == -1
    # ASCII with a missing last line
    txt = "ply\nformat ascii 1.0\nelement vertex 3\nproperty float x\nproperty float y\nproperty float z\n" \
          "end_header\n1 2 3\n4 5 6\n"
    (tmp_path / "a.ply").write_text(txt)
    with pytest.raises(Exception):
        P.load_ply(str(tmp_path / "a.ply"))


def test_ply_count_reads_header_only(tmp_path):
    """ophpc_load_ply(path, NULL, 0) answers from the header alone."""
    import ctypes
    from openholo_gb300 import lib
    rng = np.random.default_rng(23)
    _binary_ply(tmp_path / "c.ply", rng.uniform(-1, 1, (50, 3)).astype(np.float32),
                rng.integers(0, 256, (50, 3)).astype(np.uint8), truncate=20)
    L = lib()
    L.ophpc_load_ply.restype = ctypes.c_int64
    assert L.ophpc_load_ply(str(tmp_path / "c.ply").encode(), None, ctypes.c_uint64(0)) == 50


def test_ply_appends_extension_and_fails_cleanly(tmp_path):
    got = P.load_ply(os.path.join(GOLD, "ply_ascii_channel"))   # ".ply" appended
    assert got.shape[0] == 64
    with pytest.raises(Exception):
        P.load_ply(str(tmp_path / "missing.ply"))
    bad = tmp_path / "bad.ply"
    bad.write_text("not a ply\n")
    with pytest.raises(Exception):
        P.load_ply(str(bad))


def test_ply_big_endian_roundtrip(tmp_path):
    """binary_big_endian is byte-swapped (the reference reads it unswapped)."""
    n = 5
    rng = np.random.default_rng(0)
    xyz = rng.uniform(-1, 1, (n, 3)).astype(np.float32)
    rgb = rng.integers(0, 256, (n, 3))
    hdr = ("ply\nformat binary_big_endian 1.0\nelement color 1\nproperty int channel\n"
           f"element vertex {n}\nproperty float x\nproperty float y\nproperty float z\n"
           "property uchar red\nproperty uchar green\nproperty uchar blue\nend_header\n")
    p = tmp_path / "be.ply"
    with open(p, "wb") as f:
        f.write(hdr.encode())
        f.write(struct.pack(">i", 3))
        for i in range(n):
            f.write(struct.pack(">fffBBB", *xyz[i], *[int(c) for c in rgb[i]]))
    got = P.load_ply(str(p))
    assert np.array_equal(got[:, :3], xyz.astype(np.float64))
    assert np.array_equal(got[:, 3:6], (rgb.astype(np.float32) / np.float32(255.0)).astype(np.float64))


def _write(tmp_path, name, text):
    p = tmp_path / name
    p.write_text(text)
    return str(p)


DICE_STYLE = """<PointCloud>
  <!-- About points -->
  <FieldLength>1000e-3</FieldLength> <!-- Double Type -->
  <ScaleX>0.01</ScaleX> <!-- Double Type -->
  <ScaleY>0.01</ScaleY>
  <ScaleZ>0.01</ScaleZ>
  <Distance>0.1</Distance>
  <IMG_Rotation>0</IMG_Rotation>
  <IMG_Merge>1</IMG_Merge>
  <DoublePrecision>1</DoublePrecision>
  <SLM_PixelPitchX>4.3e-6</SLM_PixelPitchX>
  <SLM_PixelPitchY> 4.3e-6</SLM_PixelPitchY>
  <SLM_PixelNumX>1920</SLM_PixelNumX>
  <SLM_PixelNumY>1080</SLM_PixelNumY>
  <SLM_WaveNum>3</SLM_WaveNum>
  <SLM_WaveLength_1>638e-9</SLM_WaveLength_1>
  <SLM_WaveLength_2>520e-9</SLM_WaveLength_2>
  <SLM_WaveLength_3>450e-9</SLM_WaveLength_3>
  <NumOfStream>0</NumOfStream>
</PointCloud>
"""


def test_config_reader_dice_style(tmp_path):
    st, c, img = P.read_config(_write(tmp_path, "a.xml", DICE_STYLE))
    assert st == 0
    assert (c.pixel_number[0], c.pixel_number[1]) == (1920, 1080)
    assert (c.pixel_pitch[0], c.pixel_pitch[1]) == (4.3e-6, 4.3e-6)
    assert c.n_channels == 3 and list(c.wave_length) == [638e-9, 520e-9, 450e-9]
    assert list(c.scale) == [0.01, 0.01, 0.01] and c.distance == 0.1 and c.field_length == 1.0
    assert img.merge == 1 and img.rotate == 0 and img.flip == 0 and img.double_precision == 1
    assert img.num_of_stream == 0 and list(img.shift) == [0, 0, 0]


def test_config_reader_golden_xml(tmp_path):
    for name in ["rs_window_1ch", "rs_3ch_vw", "fresnel_3ch"]:
        d = np.load(os.path.join(GOLD, name + ".npz"))
        st, c, _ = P.read_config(_write(tmp_path, name + ".xml", str(d["xml"])))
        assert st == 0


def test_config_reader_errors(tmp_path):
    # wrong extension / unreadable -> I/O error
    assert P.read_config(_write(tmp_path, "a.txt", DICE_STYLE))[0] == 4
    assert P.read_config(str(tmp_path / "missing.xml"))[0] == 4
    # the reference reads keys under xml_doc.FirstChild(): a declaration
    # first makes every key missing -> no usable document
    assert P.read_config(_write(tmp_path, "b.xml", '<?xml version="1.0"?>\n' + DICE_STYLE))[0] == 4
    # missing required key -> config error, other keys still read
    st, c, _ = P.read_config(_write(tmp_path, "c.xml", DICE_STYLE.replace("<SLM_PixelNumY>1080</SLM_PixelNumY>", "")))
    assert st == 5 and c.pixel_number[0] == 1920
    # malformed number -> config error
    st, _, _ = P.read_config(_write(tmp_path, "d.xml", DICE_STYLE.replace("0.01</ScaleX>", "abc</ScaleX>")))
    assert st == 5
    # more than three wavelengths: Vertex carries three colours
    st, _, _ = P.read_config(_write(tmp_path, "e.xml", DICE_STYLE.replace("<SLM_WaveNum>3", "<SLM_WaveNum>4")))
    assert st == 5


def test_config_reader_tinyxml_value_rules(tmp_path):
    x = DICE_STYLE.replace("<IMG_Rotation>0</IMG_Rotation>", "<IMG_Rotation>true</IMG_Rotation>")
    x = x.replace("<SLM_PixelNumX>1920</SLM_PixelNumX>", "<SLM_PixelNumX>0x780</SLM_PixelNumX>")
    st, c, img = P.read_config(_write(tmp_path, "f.xml", x))
    assert st == 0 and img.rotate == 1 and c.pixel_number[0] == 1920


def _bmp_pixels(raw: bytes):
    off = struct.unpack_from("<I", raw, 10)[0]
    w, h = struct.unpack_from("<ii", raw, 18)
    bpp = struct.unpack_from("<H", raw, 28)[0]
    ch = bpp // 8
    stride = (w * ch + 3) & ~3
    rows = [raw[off + y * stride: off + y * stride + w * ch] for y in range(h)]
    return np.frombuffer(b"".join(rows), dtype=np.uint8).reshape(h, w * ch), w, h, bpp


@pytest.mark.parametrize("name", ["bmp_1ch_w96", "bmp_1ch_w90", "bmp_3ch_merge"])
def test_bmp_writer_byte_identical(tmp_path, name):
    ref = open(os.path.join(GOLD, name + ".bmp"), "rb").read()
    pix, w, h, bpp = _bmp_pixels(ref)
    out = tmp_path / "o.bmp"
    P.save_bmp(str(out), pix.reshape(h, w, bpp // 8) if bpp == 24 else pix, bits_per_pixel=bpp)
    assert open(out, "rb").read() == ref


def test_bmp_flip_and_rotate(tmp_path):
    pix = np.arange(12, dtype=np.uint8).reshape(3, 4)
    for flip, want in ((1, pix[::-1]), (2, pix[:, ::-1]), (3, pix[::-1, ::-1])):
        P.save_bmp(str(tmp_path / "f.bmp"), pix, 8, flip=flip)
        got, _, _, _ = _bmp_pixels(open(tmp_path / "f.bmp", "rb").read())
        assert np.array_equal(got, want)
    P.save_bmp(str(tmp_path / "r.bmp"), pix, 8, rotate=True)
    got, _, _, _ = _bmp_pixels(open(tmp_path / "r.bmp", "rb").read())
    assert np.array_equal(got, pix[::-1, ::-1])


# ------------------------------------------------------------------ OHC

@pytest.mark.parametrize("name", ["ohc_1ch_fresnel", "ohc_3ch_rs"])
def test_ohc_reader_matches_reference(name):
    want = np.load(os.path.join(GOLD, name + ".npz"))
    field, pitch, wl = P.load_ohc(os.path.join(GOLD, name + ".ohc"))
    assert np.array_equal(field, want["field"])
    assert np.array_equal(np.asarray(pitch), want["pitch"])
    assert np.array_equal(wl, want["wavelengths"])


@pytest.mark.parametrize("name", ["ohc_1ch_fresnel", "ohc_3ch_rs"])
def test_ohc_writer_byte_identical(tmp_path, name):
    """The reference's saveAsOhc file, rewritten from the field it holds."""
    ref = open(os.path.join(GOLD, name + ".ohc"), "rb").read()
    want = np.load(os.path.join(GOLD, name + ".npz"))
    out = tmp_path / "o"                      # ".ohc" appended
    P.save_ohc(str(out), want["field"], want["pitch"], want["wavelengths"])
    assert open(str(out) + ".ohc", "rb").read() == ref


@pytest.mark.parametrize("variant", ["seqt_f64", "each_f32", "seqt_f32"])
def test_ohc_reader_layouts(variant):
    """Channels interleaved per pixel and float32 data, read as the
    reference's decoder reads them."""
    z = np.load(os.path.join(GOLD, "ohc_variants.npz"))
    field, pitch, wl = P.load_ohc(os.path.join(GOLD, f"ohc_{variant}.ohc"))
    assert np.array_equal(field, z[variant])
    assert pitch == (4e-6, 5e-6)
    assert np.array_equal(wl, [638e-9, 532e-9, 473e-9])


def _ohc_bytes(field, arrange=2, dtype=10, code=2, nwl=None):
    nch = field.shape[0] if nwl is None else nwl
    a, b = (field.real, field.imag) if code == 2 else (np.abs(field), np.angle(field))
    data = np.concatenate([a.reshape(-1), b.reshape(-1)]).astype(np.float64 if dtype == 10 else np.float32)
    info = struct.pack("<IIIddBIBBBBBBBddQB", 65 + 8 * nch, field.shape[2], field.shape[1], 1e-6, 1e-6, 1, nch, 2,
                       arrange, 1, dtype, 1, code, 0, -1.0, 1.0, data.nbytes, 0)
    head = struct.pack("<2sQBBIII", b"OH", 24 + len(info) + 8 * nch + data.nbytes, 3, 0, 0, 0,
                       24 + len(info) + 8 * nch)
    return head + info + np.full(nch, 5e-7).tobytes() + data.tobytes()


def test_ohc_amplitude_phase_and_errors(tmp_path):
    rng = np.random.default_rng(3)
    f = rng.normal(size=(1, 4, 5)) + 1j * rng.normal(size=(1, 4, 5))
    p = tmp_path / "ap.ohc"
    p.write_bytes(_ohc_bytes(f, code=1))
    got, _, _ = P.load_ohc(str(p))
    assert np.allclose(got, f, rtol=0, atol=1e-12)
    # amplitude-only coding, truncated data, bad signature, too many channels
    bad = {"ae.ohc": _ohc_bytes(f, code=3), "short.ohc": _ohc_bytes(f)[:-8],
           "sig.ohc": b"XX" + _ohc_bytes(f)[2:], "nch.ohc": _ohc_bytes(np.zeros((4, 2, 2)))}
    for name, raw in bad.items():
        (tmp_path / name).write_bytes(raw)
        with pytest.raises(Exception):
            P.load_ohc(str(tmp_path / name))
    with pytest.raises(Exception):
        P.load_ohc(str(tmp_path / "missing.ohc"))
    with pytest.raises(Exception):
        P.save_ohc(str(tmp_path / "x.ohc"), np.zeros((4, 2, 2)), (1e-6, 1e-6), [5e-7] * 4)


def test_facade_ohc_roundtrip(tmp_path):
    """PointCloud.loadAsOhc replaces the context and complex field;
    saveAsOhc writes the reference's bytes back (no GPU needed)."""
    src = os.path.join(GOLD, "ohc_3ch_rs.ohc")
    want = np.load(os.path.join(GOLD, "ohc_3ch_rs.npz"))
    with P.PointCloud() as h:
        assert h.loadAsOhc(src)
        c = h.getConfig()
        assert (c.pixel_number[0], c.pixel_number[1], c.n_channels) == (40, 24, 3)
        assert np.array_equal(list(c.wave_length), want["wavelengths"])
        assert np.array_equal(h.getComplexField(), want["field"])
        assert h.saveAsOhc(str(tmp_path / "back.ohc"))
        assert not h.loadAsOhc(str(tmp_path / "missing"))
    assert open(tmp_path / "back.ohc", "rb").read() == open(src, "rb").read()
