"""C++ drop-in: tests/cpp/exam_pointcloud.cpp, the reference's example
program (Example/examPointCloud/examPointCloud.cpp:54-132) with the same
call sequence, compiled with g++ against include/ophPointCloud.h and linked
to libophpc.so, run on a PLY / XML fixture the reference itself produced a
field and phase codes for (tests/golden/ply_generate_rs.npz). Checks: the
.ohc it writes holds the reference's field within relL2 1e-4, and the three
8-bit BMPs together hold the reference's phase codes (>= 99.9% exact, +-1
LSB, circular)."""
import os
import shutil
import struct
import subprocess

import numpy as np
import pytest

from openholo_gb300 import lib_path
from openholo_gb300 import pointcloud as P
from tests._util import code_agreement, rel_l2

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
GOLD = os.path.join(HERE, "golden")


def _bmp_pixels(raw: bytes):
    off = struct.unpack_from("<I", raw, 10)[0]
    w, h = struct.unpack_from("<ii", raw, 18)
    stride = (w + 3) & ~3
    return np.frombuffer(b"".join(raw[off + y * stride: off + y * stride + w] for y in range(h)),
                         dtype=np.uint8).reshape(h, w)


def test_reference_example_program(tmp_path, gpu_ctx):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no C++ compiler")
    libdir = os.path.dirname(lib_path())
    exe = str(tmp_path / "exam_pointcloud")
    r = subprocess.run([gxx, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                        os.path.join(HERE, "cpp", "exam_pointcloud.cpp"), "-L", libdir, "-lophpc",
                        "-Wl,-rpath," + libdir, "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    d = np.load(os.path.join(GOLD, "ply_generate_rs.npz"))
    xml = tmp_path / "cfg.xml"
    xml.write_text(str(d["xml"]))
    out = tmp_path / "result"
    out.mkdir()
    r = subprocess.run([exe, str(xml), os.path.join(GOLD, "ply_ascii_channel.ply"), str(out)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    field, _, wl = P.load_ohc(str(out / "pc_sample.ohc"))
    assert field.shape == d["field"].shape
    assert rel_l2(field, d["field"]) <= 1e-4
    assert np.allclose(wl, [638e-9, 532e-9, 473e-9])
    # three colours, not merged: one file per channel; the bar holds over
    # the hologram (8,640 codes), as in the other facade tests
    codes = np.stack([_bmp_pixels(open(out / f"{ch}_pc_sample.bmp", "rb").read()) for ch in range(3)])
    exact, maxd = code_agreement(codes, d["codes_phase"], circular=True)
    assert exact >= 0.999 and maxd <= 1, (exact, maxd)
