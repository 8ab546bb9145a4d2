"""Generates the golden vectors in tests/golden/ from the reference itself.

Runs the reference's own CPU path (oracle/_ref/libophref.so, compiled from
the reference sources by ``make -C oracle ref``) through its public API
(readConfig -> setPointCloudModel | loadPointCloud -> SetMode(MODE_CPU) ->
generateHologram -> encoding -> normalize; Example/examPointCloud/
examPointCloud.cpp:54-132) on small seeded inputs, and stores the complex
field, the encoded buffer and the 8-bit codes. The PLY cases write PLY files
in the reference's own point-cloud format (ASCII and binary_little_endian,
with and without the `color channel` element) and record the Vertex arrays
the reference PLYparser returns for them.

The reference does not exist where the GPU tests run; only these committed
fixtures travel. Re-run with:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import struct
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402


def box(n, xy, z, seed):
    rng = np.random.default_rng(seed)
    v = np.zeros((n, 7))
    v[:, 0] = rng.uniform(-xy[0], xy[0], n)
    v[:, 1] = rng.uniform(-xy[1], xy[1], n)
    v[:, 2] = rng.uniform(z[0], z[1], n)
    v[:, 3:6] = 1.0 - rng.uniform(0.0, 1.0, (n, 3))
    v[:, 6] = rng.uniform(0, 2 * np.pi, n)
    return v


# name: (geometry, vertices, diff_flag, viewing_window)
FIELD_CASES = {
    "rs_window_1ch": (oracle.Geometry(pnx=96, pny=64, ppx=8e-6, ppy=8e-6, wavelengths=[532e-9]),
                      box(300, (4e-4, 3e-4), (0.002, 0.01), 101), 0, False),
    "fresnel_window_1ch": (oracle.Geometry(pnx=96, pny=64, ppx=8e-6, ppy=8e-6, wavelengths=[532e-9]),
                           box(300, (4e-4, 3e-4), (0.002, 0.01), 102), 1, False),
    "rs_3ch_vw": (oracle.Geometry(pnx=80, pny=48, ppx=6.4e-6, ppy=7.1e-6, wavelengths=[638e-9, 532e-9, 473e-9],
                                  scale=(0.01, 0.01, 0.01), distance=0.1, field_length=1.0,
                                  viewing_window=True),
                  box(250, (0.05, 0.05), (-0.2, 0.2), 103), 0, True),
    "fresnel_3ch": (oracle.Geometry(pnx=80, pny=48, ppx=6.4e-6, ppy=7.1e-6,
                                    wavelengths=[638e-9, 532e-9, 473e-9], scale=(0.5, 0.5, 2.0), distance=0.05),
                    box(250, (1e-3, 1e-3), (0.05, 0.2), 104), 1, False),
}


def rs_1k_crop():
    """The rs_1k distribution (x, y ~ U(+-2 mm), z ~ U[0.45, 0.55] m, amplitude
    U(0, 1], seed 0) on a 256x256 crop of its SLM with 500 points."""
    rng = np.random.default_rng(0)
    n = 500
    v = np.zeros((n, 7))
    v[:, 0] = rng.uniform(-2e-3, 2e-3, n)
    v[:, 1] = rng.uniform(-2e-3, 2e-3, n)
    v[:, 2] = rng.uniform(0.45, 0.55, n)
    amp = 1.0 - rng.uniform(0.0, 1.0, n)
    v[:, 3:6] = amp[:, None]
    return oracle.Geometry(pnx=256, pny=256, ppx=8e-6, ppy=8e-6, wavelengths=[532e-9]), v


def write_ply_ascii(path, xyz, rgb, phase, with_channel=True):
    n = xyz.shape[0]
    with open(path, "w") as f:
        f.write("ply\nformat ascii 1.0\ncomment synthetic point cloud\n")
        if with_channel:
            f.write("element color 1\nproperty int channel\n")
        f.write(f"element vertex {n}\nproperty float x\nproperty float y\nproperty float z\n")
        f.write("property uchar red\nproperty uchar green\nproperty uchar blue\nproperty double phase\n")
        f.write("end_header\n")
        if with_channel:
            f.write("3\n")
        for i in range(n):
            f.write(f"{xyz[i, 0]:.6f} {xyz[i, 1]:.6f} {xyz[i, 2]:.6f} {rgb[i, 0]} {rgb[i, 1]} {rgb[i, 2]} "
                    f"{phase[i]:.6f}\n")


def write_ply_binary(path, xyz, rgb, phase, with_channel=True):
    n = xyz.shape[0]
    hdr = "ply\nformat binary_little_endian 1.0\ncomment synthetic point cloud\n"
    if with_channel:
        hdr += "element color 1\nproperty int channel\n"
    hdr += (f"element vertex {n}\nproperty float x\nproperty float y\nproperty float z\n"
            "property uchar red\nproperty uchar green\nproperty uchar blue\nproperty float phase\nend_header\n")
    with open(path, "wb") as f:
        f.write(hdr.encode())
        if with_channel:
            f.write(struct.pack("<i", 3))
        for i in range(n):
            f.write(struct.pack("<fffBBBf", xyz[i, 0], xyz[i, 1], xyz[i, 2], int(rgb[i, 0]), int(rgb[i, 1]),
                                int(rgb[i, 2]), phase[i]))


def write_ohc(path, field, pitch, wavelengths, arrange=2, dtype=10, code=2):
    """A .ohc in the reference's layout (Openholo/src/ImgCodecDefine.h:53-210):
    24-byte file header, 65-byte field-info header, wavelength table, then the
    first part (real or amplitude) of every pixel of every channel, then the
    second. arrange 2: one plane per channel; 1: channels interleaved per
    pixel. dtype 10: float64, 9: float32. code 2: real/imaginary,
    1: amplitude/phase."""
    nch, pny, pnx = field.shape
    if code == 2:
        a, b = field.real, field.imag
    else:
        a, b = np.abs(field), np.angle(field)
    if arrange == 2:
        a, b = a.reshape(-1), b.reshape(-1)
    else:
        a, b = a.reshape(nch, -1).T.reshape(-1), b.reshape(nch, -1).T.reshape(-1)
    np_t = np.float64 if dtype == 10 else np.float32
    data = np.concatenate([a, b]).astype(np_t).tobytes()
    info_size = 65 + 8 * nch
    info = struct.pack("<IIIddBIBBBBBBBddQB", info_size, pnx, pny, pitch[0], pitch[1], 1, nch, 2 if nch > 1 else 1,
                       arrange, 1, dtype, 1, code, 0, -1.0, 1.0, len(data), 0)
    head = struct.pack("<2sQBBIII", b"OH", 24 + info_size + len(data), 3, 0, 0, 0, 24 + info_size)
    with open(path, "wb") as f:
        f.write(head + info + np.asarray(wavelengths, dtype=np.float64).tobytes() + data)


def make_ohc(xml):
    """OHC fixtures; xml is a scratch path for the config file."""
    out = {}
    # OHC: the reference's saveAsOhc output for a one- and a
    # three-channel field, and what its loadAsOhc reads back from it.
    ohc_cases = {"ohc_1ch_fresnel": "fresnel_window_1ch", "ohc_3ch_rs": "rs_3ch_vw"}
    for name, case in ohc_cases.items():
        g, v, diff, _ = FIELD_CASES[case]
        small = oracle.Geometry(pnx=40, pny=24, ppx=g.ppx, ppy=g.ppy, wavelengths=g.wavelengths,
                                scale=g.scale, distance=g.distance)
        with open(xml, "w") as f:
            f.write(small.xml())
        path = os.path.join(HERE, name + ".ohc")
        oracle.ref_run_save_ohc(xml, v, diff, path)
        field, pitch, wl = oracle.ref_load_ohc(path)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), field=field, pitch=pitch, wavelengths=wl)
        out[name] = os.path.getsize(path)
    # Layouts the reference reads but does not write: channels
    # interleaved per pixel, float32; the reference's reading of each.
    rng = np.random.default_rng(11)
    fld = rng.normal(size=(3, 6, 10)) + 1j * rng.normal(size=(3, 6, 10))
    variants = {}
    for vname, kw in {"seqt_f64": dict(arrange=1), "each_f32": dict(dtype=9),
                      "seqt_f32": dict(arrange=1, dtype=9)}.items():
        path = os.path.join(HERE, f"ohc_{vname}.ohc")
        write_ohc(path, fld, (4e-6, 5e-6), [638e-9, 532e-9, 473e-9], **kw)
        variants[vname] = oracle.ref_load_ohc(path)[0]
    np.savez_compressed(os.path.join(HERE, "ohc_variants.npz"), source=fld, **variants)
    return out


def write_ply_binary_faces(path, xyz, rgb_f):
    """binary_little_endian with a color channel element, colourless
    vertices (float x y z) and one face per vertex (a uchar-counted int list
    of 3 indices, then uchar red green blue): vertex e takes face e's colour.
    (With colours on both elements the reference reads the face records
    with the vertex's property indices and loses its place in the file.)"""
    n = xyz.shape[0]
    hdr = ("ply\nformat binary_little_endian 1.0\nelement color 1\nproperty int channel\n"
           f"element vertex {n}\nproperty float x\nproperty float y\nproperty float z\n"
           f"element face {n}\nproperty list uchar int vertex_indices\n"
           "property uchar red\nproperty uchar green\nproperty uchar blue\nend_header\n")
    with open(path, "wb") as f:
        f.write(hdr.encode())
        f.write(struct.pack("<i", 3))
        for i in range(n):
            f.write(struct.pack("<fff", xyz[i, 0], xyz[i, 1], xyz[i, 2]))
        for i in range(n):
            f.write(struct.pack("<Biii", 3, i, (i + 1) % n, (i + 2) % n))
            f.write(struct.pack("<BBB", *(int(c) for c in rgb_f[i])))


def make_ply_faces():
    """PLY with a face element: what the reference's PLYparser returns."""
    rng = np.random.default_rng(13)
    n = 48
    xyz = np.round(rng.uniform(-0.5, 0.5, (n, 3)), 6)
    path = os.path.join(HERE, "ply_binary_faces.ply")
    write_ply_binary_faces(path, xyz, rng.integers(0, 256, (n, 3)))
    np.savez_compressed(os.path.join(HERE, "ply_faces.npz"), ply_binary_faces=oracle.ref_load_ply(path))
    return {"ply_faces": n}


REFERENCE = oracle.REFERENCE_TREE
DICE_DIR = os.path.join(REFERENCE, "Example", "dataset", "Dice", "PointCloud")
DICE_RGB = os.path.join(REFERENCE, "Openholo_python", "test", "PointCloud_Dice_RGB.ply")


def _sampled(field, enc, codes, n_sample, seed):
    """Field, encodings and codes at seeded pixels of every channel, plus the
    normalisation range (min, max of the encoded buffer over all channels)."""
    nch, pny, pnx = field.shape
    rng = np.random.default_rng(seed)
    idx = np.sort(rng.choice(pny * pnx, n_sample, replace=False))
    out = {"pixel_index": idx, "field_at": field.reshape(nch, -1)[:, idx]}
    for k, name in enumerate(("phase", "amp")):
        out[f"codes_{name}_at"] = codes[k].reshape(nch, -1)[:, idx]
        out[f"enc_{name}_range"] = np.array([enc[k].min(), enc[k].max()])
    return out


def make_dice(xml):
    """The reference's own example fixtures through its CPU path:
    Example/dataset/Dice/PointCloud (Dice_PointCloud.xml + dice_100000.ply,
    7,493 points, 1920x1080, RS and Fresnel) and
    Openholo_python/test/PointCloud_Dice_RGB.ply (1,461 points) with the Dice
    geometry in three colours. Stored: the vertices the reference's PLY
    parser returns, the config, and the field / codes at 16,384 seeded
    pixels with the normalisation range (the full 1920x1080 field is 33 MB
    per channel)."""
    out = {}
    dice_xml = open(os.path.join(DICE_DIR, "Dice_PointCloud.xml")).read()
    ply = os.path.join(DICE_DIR, "dice_100000.ply")
    verts = oracle.ref_load_ply(ply)
    with open(xml, "w") as f:
        f.write(dice_xml)
    res = {"vertices": verts, "xml": dice_xml}
    for diff, tag in ((0, "rs"), (1, "fresnel")):
        field, enc, codes, secs = oracle.ref_run(xml, ply_path=ply, diff_flag=diff, encode_flag=2)
        for k, v in _sampled(field, enc, codes, 16384, 31 + diff).items():
            res[f"{tag}_{k}"] = v
        out[f"dice_{tag}"] = round(secs, 1)
    np.savez_compressed(os.path.join(HERE, "dice.npz"), **res)
    rgb_xml = dice_xml.replace("<SLM_WaveNum>1</SLM_WaveNum>", "<SLM_WaveNum>3</SLM_WaveNum>").replace(
        "<SLM_WaveLength_1>532e-9</SLM_WaveLength_1>",
        "<SLM_WaveLength_1>638e-9</SLM_WaveLength_1> <SLM_WaveLength_2>532e-9</SLM_WaveLength_2> "
        "<SLM_WaveLength_3>473e-9</SLM_WaveLength_3>")
    with open(xml, "w") as f:
        f.write(rgb_xml)
    field, enc, codes, secs = oracle.ref_run(xml, ply_path=DICE_RGB, diff_flag=0, encode_flag=2)
    res = {"vertices": oracle.ref_load_ply(DICE_RGB), "xml": rgb_xml}
    res.update(_sampled(field, enc, codes, 16384, 33))
    np.savez_compressed(os.path.join(HERE, "dice_rgb.npz"), **res)
    out["dice_rgb_rs"] = round(secs, 1)
    return out


ENCODER_FLAGS = (2, 3, 4, 5, 6)   # Real, Imaginary, SimpleNI, Burckhardt, TwoPhase


def make_encoders(xml):
    """The reference's encoding + normalize of given fields: the fresnel_3ch
    golden field (3 channels, 80x48) and a seeded 41x23 one-channel field
    whose pixel count divides by neither 2 nor 3; on the latter also
    Burckhardt after Phase and TwoPhase after Amplitude on the same object
    (the entries they skip keep the earlier encoding)."""
    out = {}
    z = np.load(os.path.join(HERE, "fresnel_3ch.npz"))
    with open(xml, "w") as f:
        f.write(str(z["xml"]))
    res = {}
    for flag in ENCODER_FLAGS:
        res[f"enc_{flag}"], res[f"codes_{flag}"] = oracle.ref_encode_field(xml, z["field"], flag)
    np.savez_compressed(os.path.join(HERE, "encoders_3ch.npz"), **res)
    out["encoders_3ch"] = len(res)
    rng = np.random.default_rng(5)
    g = oracle.Geometry(pnx=41, pny=23, ppx=8e-6, ppy=8e-6, wavelengths=[532e-9])
    with open(xml, "w") as f:
        f.write(g.xml())
    fld = rng.normal(size=(1, 23, 41)) + 1j * rng.normal(size=(1, 23, 41))
    res = {"field": fld, "xml": g.xml()}
    for flag in ENCODER_FLAGS:
        res[f"enc_{flag}"], res[f"codes_{flag}"] = oracle.ref_encode_field(xml, fld, flag)
    for flag, pre in ((5, 0), (6, 1)):
        res[f"enc_{flag}_after_{pre}"], res[f"codes_{flag}_after_{pre}"] = oracle.ref_encode_field(xml, fld, flag,
                                                                                                   pre)
    np.savez_compressed(os.path.join(HERE, "encoders_odd_1ch.npz"), **res)
    out["encoders_odd_1ch"] = len(res)
    return out


WRP_CASES = {
    # three colours, positive depth difference: w = 16 (32 x 32 splats)
    "wrp_3ch": (oracle.WrpGeometry(pnx=96, pny=72, ppx=8e-6, ppy=8e-6, wavelengths=[638e-9, 532e-9, 473e-9],
                                   scale=(1.0, 1.0, 1.0), wrp_location=2e-3, distance=0.05),
                box(120, (3.5e-4, 2.6e-4), (-1e-3, 0.0), 201)),
    # negative depth difference (the WRP in front of the points), odd size,
    # points reaching past the plane's edges
    "wrp_negdz_edges": (oracle.WrpGeometry(pnx=67, pny=45, ppx=6.4e-6, ppy=7.1e-6, wavelengths=[532e-9],
                                           scale=(2.0, 2.0, 0.5), wrp_location=-1.5e-3, distance=0.02),
                        box(80, (2.4e-4, 1.8e-4), (-1e-3, 1e-3), 202)),
}


def make_wrp(xml):
    """The reference's own WRP splat planes (ophWRP::calculateWRPCPU,
    ophgen/src/ophWRP.cpp:321-420; captured by oracle/ref_wrp_driver.cpp):
    two small synthetic cases in full, and the reference's WRP example
    (Example/dataset/Dice/WRP/Dice_WRP.xml with the Dice point cloud,
    1920x1080) at 16,384 seeded pixels among those the splat reaches, with
    the plane's count of nonzero pixels, sum and L2 norm."""
    out = {}
    for name, (g, v) in WRP_CASES.items():
        with open(xml, "w") as f:
            f.write(g.xml())
        planes = oracle.ref_wrp_planes(xml, v, len(g.wavelengths), g.pnx, g.pny)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), vertices=v, planes=planes, xml=g.xml(),
                            pnx=g.pnx, pny=g.pny, ppx=g.ppx, ppy=g.ppy, wavelengths=np.array(g.wavelengths),
                            scale=np.array(g.scale), wrp_location=g.wrp_location, distance=g.distance)
        out[name] = planes.shape
    wrp_dir = os.path.join(os.path.dirname(DICE_DIR), "WRP")
    dice_xml = open(os.path.join(wrp_dir, "Dice_WRP.xml")).read()
    verts = oracle.ref_load_ply(os.path.join(wrp_dir, "dice_100000.ply"))
    with open(xml, "w") as f:
        f.write(dice_xml)
    plane = oracle.ref_wrp_planes(xml, verts, 1, 1920, 1080)[0]
    nz = np.flatnonzero(plane)
    rng = np.random.default_rng(41)
    idx = np.sort(rng.choice(nz, min(16384, nz.size), replace=False))
    np.savez_compressed(os.path.join(HERE, "wrp_dice.npz"), vertices=verts, xml=dice_xml, pixel_index=idx,
                        plane_at=plane.reshape(-1)[idx], nonzero=nz.size, plane_sum=plane.sum(),
                        plane_norm=np.linalg.norm(plane))
    out["wrp_dice"] = nz.size
    return out


SIDEBAND_CASES = {   # (pnx, pny, ppx, ppy, wavelengths, seed)
    "even_2ch": (24, 16, 8e-6, 6.4e-6, [532e-9, 638e-9], 61),
    "odd_1ch": (15, 9, 8e-6, 8e-6, [532e-9], 62),
    "mixed_3ch": (20, 21, 6.4e-6, 7.1e-6, [638e-9, 532e-9, 473e-9], 63),
}


def make_sideband(xml):
    """The reference's own ophGen::encodeSideBand (ophgen/src/ophGen.cpp:
    1607-1695) on seeded random fields, every passband (oracle/
    ref_sideband_driver.cpp; FFTW replaced by the FP64 DFT of
    oracle/ref_dft_stubs.c)."""
    arrays = {}
    for name, (pnx, pny, ppx, ppy, wl, seed) in SIDEBAND_CASES.items():
        g = oracle.Geometry(pnx=pnx, pny=pny, ppx=ppx, ppy=ppy, wavelengths=wl)
        with open(xml, "w") as f:
            f.write(g.xml())
        rng = np.random.default_rng(seed)
        field = rng.normal(size=(len(wl), pny, pnx)) + 1j * rng.normal(size=(len(wl), pny, pnx))
        arrays[name + "_field"] = field
        arrays[name + "_geom"] = np.array([pnx, pny, ppx, ppy])
        for pb in range(4):
            arrays[f"{name}_enc{pb}"] = oracle.ref_sideband(xml, field, pb)
    np.savez_compressed(os.path.join(HERE, "sideband.npz"), **arrays)
    return {"sideband": len(arrays)}


def main():
    if not oracle.ref_available():
        oracle.build(with_reference=True)
    out = {}
    with tempfile.TemporaryDirectory() as d:
        xml = os.path.join(d, "cfg.xml")
        for name, (g, v, diff, vw) in FIELD_CASES.items():
            with open(xml, "w") as f:
                f.write(g.xml())
            field, enc, codes, _ = oracle.ref_run(xml, vertices=v, diff_flag=diff, encode_flag=2,
                                                  viewing_window=vw)
            enc_p, enc_a, codes_p, codes_a = enc[0], enc[1], codes[0], codes[1]
            np.savez_compressed(os.path.join(HERE, f"{name}.npz"), vertices=v, field=field, enc_phase=enc_p,
                                codes_phase=codes_p, enc_amp=enc_a, codes_amp=codes_a, diff_flag=diff,
                                xml=g.xml(), viewing_window=vw)
            out[name] = field.shape
        # rs_1k crop: codes in full, the field at sampled pixels
        g, v = rs_1k_crop()
        with open(xml, "w") as f:
            f.write(g.xml())
        field, _, codes, _ = oracle.ref_run(xml, vertices=v, diff_flag=0, encode_flag=2)
        codes_p, codes_a = codes[0], codes[1]
        rng = np.random.default_rng(7)
        idx = np.sort(rng.choice(256 * 256, 2048, replace=False))
        np.savez_compressed(os.path.join(HERE, "rs_1k_crop.npz"), vertices=v, pixel_index=idx,
                            field_at=field[0].reshape(-1)[idx], codes_phase=codes_p, codes_amp=codes_a,
                            xml=g.xml())
        out["rs_1k_crop"] = codes_p.shape

        # PLY: files in the reference's format + what PLYparser makes of them
        rng = np.random.default_rng(9)
        n = 64
        xyz = np.round(rng.uniform(-0.5, 0.5, (n, 3)), 6)
        rgb = rng.integers(0, 256, (n, 3))
        phase = np.round(rng.uniform(0, 6.28, n), 6)
        plys = {
            "ply_ascii_channel.ply": (write_ply_ascii, True),
            "ply_ascii_nochannel.ply": (write_ply_ascii, False),
            "ply_binary_channel.ply": (write_ply_binary, True),
        }
        ply_vertices = {}
        for fname, (writer, ch) in plys.items():
            path = os.path.join(HERE, fname)
            writer(path, xyz, rgb, phase, ch)
            ply_vertices[fname.replace(".ply", "")] = oracle.ref_load_ply(path)
        np.savez_compressed(os.path.join(HERE, "ply_vertices.npz"), **ply_vertices)

        # A PLY-driven generate: the reference's loadPointCloud path end to end
        g = oracle.Geometry(pnx=72, pny=40, ppx=4.3e-6, ppy=4.3e-6, wavelengths=[638e-9, 532e-9, 473e-9],
                            scale=(0.01, 0.01, 0.01), distance=0.1)
        with open(xml, "w") as f:
            f.write(g.xml())
        field, _, codes_p, _ = oracle.ref_run(xml, ply_path=os.path.join(HERE, "ply_ascii_channel.ply"),
                                             diff_flag=0, encode_flag=0)
        np.savez_compressed(os.path.join(HERE, "ply_generate_rs.npz"), field=field, codes_phase=codes_p,
                            xml=g.xml())
        # BMP output of ophGen::save: one channel (row width a multiple of 4
        # and not), and three channels merged into 24-bit BGR.
        bmp_cases = {
            "bmp_1ch_w96": (FIELD_CASES["rs_window_1ch"][0], FIELD_CASES["rs_window_1ch"][1], 8, {}),
            "bmp_1ch_w90": (oracle.Geometry(pnx=90, pny=50, ppx=8e-6, ppy=8e-6, wavelengths=[532e-9]),
                            box(120, (3e-4, 2e-4), (0.01, 0.03), 105), 8, {}),
            "bmp_3ch_merge": (oracle.Geometry(pnx=80, pny=48, ppx=6.4e-6, ppy=7.1e-6,
                                              wavelengths=[638e-9, 532e-9, 473e-9], scale=(0.5, 0.5, 2.0),
                                              distance=0.05, extra_xml={"IMG_Merge": 1}),
                              box(150, (1e-3, 1e-3), (0.05, 0.2), 106), 24, {}),
        }
        for name, (g, v, bpp, _) in bmp_cases.items():
            with open(xml, "w") as f:
                f.write(g.xml())
            bmp = os.path.join(HERE, name + ".bmp")
            oracle.ref_run_save(xml, v, 0, 0, bmp, bpp)
            field, _, codes, _ = oracle.ref_run(xml, vertices=v, diff_flag=0, encode_flag=0)
            np.savez_compressed(os.path.join(HERE, name + ".npz"), vertices=v, xml=g.xml(), bpp=bpp)
            out[name] = os.path.getsize(bmp)

        out.update(make_ohc(xml))
        out.update(make_encoders(xml))
        out.update(make_ply_faces())
        out.update(make_dice(xml))
        out.update(make_wrp(xml))
        out.update(make_sideband(xml))
    for k, v in out.items():
        print(k, v)


if __name__ == "__main__":
    only = {"ohc": make_ohc, "encoders": make_encoders, "ply_faces": lambda xml: make_ply_faces(),
            "dice": make_dice, "wrp": make_wrp, "sideband": make_sideband}
    if len(sys.argv) == 2 and sys.argv[1] in only:   # one group of fixtures
        if not oracle.ref_available() or not oracle.ref_wrp_available() or not oracle.ref_sideband_available():
            oracle.build(with_reference=True)
        with tempfile.TemporaryDirectory() as d:
            print(only[sys.argv[1]](os.path.join(d, "cfg.xml")))
    else:
        main()
