"""Host-side checks of the C ABI library (no compute calls, no GPU needed)."""
import ctypes
import glob
import os
import re
import subprocess

import numpy as np
import pytest

import openholo_gb300 as oph
from openholo_gb300 import pointcloud as P

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_c_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        # C declarations only: skip the C++ façade class header
        if "class ophPointCloud" in text:
            continue
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w\s\*]*?\b((?:ophpc|cudaPointCloud|sum)_?\w*)\s*\(", text, re.M):
            if not m.group(0).lstrip().startswith("#"):
                names.add(m.group(1))
    return sorted(names)


def test_library_exports_every_declared_symbol():
    decl = _declared_c_functions()
    assert len(decl) >= 20
    out = subprocess.run(["nm", "-D", "--defined-only", oph.lib_path()], capture_output=True, text=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if ln.strip()}
    missing = [d for d in decl if d not in exported]
    assert not missing, f"declared but not exported: {missing}"
    L = oph.lib()
    for d in decl:
        getattr(L, d)   # resolvable through the loader too


def test_abi_basics_without_compute():
    L = oph.lib()
    assert L.ophpc_api_version() == 1
    assert L.ophpc_status_string(0) == b"success"
    assert L.ophpc_status_string(10) == b"no CUDA device"
    assert ctypes.sizeof(oph.OphpcConfig) == 2 * 4 + 2 * 4 + 2 * 8 + 3 * 8 + 8 + 8 + 4 + 4 + 3 * 8


def test_null_context_is_rejected():
    L = oph.lib()
    cfg = oph.make_config(64, 64, 8e-6, 8e-6, [532e-9])
    assert L.ophpc_generate(None, ctypes.byref(cfg), None, 0, 0, 0, None, None) == 1
    assert L.ophpc_encode(None, None, 1, 1, 0, None, None, None) == 1
    assert L.ophpc_destroy(None) == 1


def _gpu_visible():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_gpu_visible(), reason="checks the no-GPU error path")
def test_create_without_gpu_reports_no_device():
    L = oph.lib()
    h = ctypes.c_void_p()
    assert L.ophpc_create(0, ctypes.byref(h)) == 10
    with pytest.raises(oph.OphpcError):
        oph.Context(0)


@pytest.mark.skipif(_gpu_visible(), reason="checks the no-GPU error path")
def test_facade_without_gpu_fails_loudly(tmp_path):
    """No CPU fallback: generateHologram returns 0.0 and says why."""
    x = tmp_path / "c.xml"
    x.write_text("<PointCloud><ScaleX>1</ScaleX><ScaleY>1</ScaleY><ScaleZ>1</ScaleZ><Distance>0</Distance>"
                 "<SLM_PixelPitchX>8e-6</SLM_PixelPitchX><SLM_PixelPitchY>8e-6</SLM_PixelPitchY>"
                 "<SLM_PixelNumX>32</SLM_PixelNumX><SLM_PixelNumY>16</SLM_PixelNumY>"
                 "<SLM_WaveNum>1</SLM_WaveNum><SLM_WaveLength_1>532e-9</SLM_WaveLength_1></PointCloud>")
    with P.PointCloud() as h:
        assert h.readConfig(str(x))
        h.setPointCloudModel(np.array([[0, 0, 0.3, 1, 1, 1, 0]], dtype=np.float64))
        assert h.getNumberOfPoints() == 1
        assert h.generateHologram(0) == 0.0
        assert "GPU" in h.lastError()


def test_facade_config_and_model_state(tmp_path):
    x = tmp_path / "c.xml"
    x.write_text("<PointCloud><ScaleX>0.5</ScaleX><ScaleY>0.25</ScaleY><ScaleZ>2</ScaleZ><Distance>0.1</Distance>"
                 "<SLM_PixelPitchX>8e-6</SLM_PixelPitchX><SLM_PixelPitchY>6e-6</SLM_PixelPitchY>"
                 "<SLM_PixelNumX>40</SLM_PixelNumX><SLM_PixelNumY>24</SLM_PixelNumY>"
                 "<SLM_WaveNum>2</SLM_WaveNum><SLM_WaveLength_1>532e-9</SLM_WaveLength_1>"
                 "<SLM_WaveLength_2>638e-9</SLM_WaveLength_2></PointCloud>")
    with P.PointCloud() as h:
        assert h.readConfig(str(x))
        c = h.getConfig()
        assert (c.pixel_number[0], c.pixel_number[1], c.n_channels) == (40, 24, 2)
        assert list(c.scale) == [0.5, 0.25, 2.0] and c.distance == 0.1
        h.setScale(1, 2, 3)
        h.setDistance(0.2)
        h.setOffset(3, -1)
        c = h.getConfig()
        assert list(c.scale) == [1, 2, 3] and c.distance == 0.2 and list(c.offset) == [3, -1]
        v = np.random.default_rng(0).normal(size=(10, 7))
        h.setPointCloudModel(v)
        assert np.array_equal(h.getPointCloudModel(), v)
        assert h.getComplexField().shape == (2, 24, 40)
        assert h.generateHologram(7) == 0.0    # bad flag -> 0.0, as the reference
        assert not h.readConfig(str(tmp_path / "missing.xml"))


@pytest.mark.parametrize("n", [74_897, 74_899, 149_796, 149_797, 200_001])
def test_facade_keeps_large_models_whole(n):
    """setPointCloudModel copies the caller's records (ophPointCloud.h:577-586)
    in one part below 4 MiB, two from 4 MiB and four from 8 MiB: every record
    arrives, at sizes either side of those steps and off the 64-byte part
    boundaries, and a second model of the same size reuses the buffer."""
    rng = np.random.default_rng(n)
    with P.PointCloud() as h:
        for _ in range(2):
            v = rng.normal(size=(n, 7))
            h.setPointCloudModel(v)
            assert h.getNumberOfPoints() == n
            assert np.array_equal(h.getPointCloudModel(), v)


@pytest.mark.parametrize("lang", ["c", "c++"])
def test_public_headers_compile(tmp_path, lang):
    """Every include/*.h compiles on its own as C11 and as C++17."""
    import shutil
    cc = shutil.which("gcc" if lang == "c" else "g++")
    if cc is None:
        pytest.skip("no host compiler")
    std = "-std=c11" if lang == "c" else "-std=c++17"
    for h in sorted(glob.glob(os.path.join(ROOT, "include", "*.h"))):
        if lang == "c" and "class ophPointCloud" in open(h).read():
            continue
        src = tmp_path / ("t.c" if lang == "c" else "t.cpp")
        src.write_text(f'#include "{os.path.basename(h)}"\nint main(void) {{ return 0; }}\n')
        r = subprocess.run([cc, std, "-Wall", "-Wextra", "-Werror", "-fsyntax-only", "-I",
                            os.path.join(ROOT, "include"), str(src)], capture_output=True, text=True)
        assert r.returncode == 0, (h, r.stderr)


def test_reference_example_program_builds_unchanged(tmp_path):
    """The reference's own example program (Example/examPointCloud/
    examPointCloud.cpp, read where it lies in the reference's source tree,
    not copied) compiles against include/ophPointCloud.h and links to
    libophpc.so with no edit to it. The one flag it needs on GCC is
    `-include experimental/filesystem`: the file names
    std::experimental::filesystem after including <filesystem>, which MSVC
    declares there and libstdc++ declares in <experimental/filesystem>.
    Running it needs a GPU (tests/test_cpp_dropin_gpu.py runs the same call
    sequence there)."""
    import shutil

    import oracle
    src = os.path.join(oracle.REFERENCE_TREE, "Example", "examPointCloud", "examPointCloud.cpp")
    if not os.path.isfile(src):
        pytest.skip("the reference's source tree is not on this machine")
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no C++ compiler")
    libdir = os.path.dirname(oph.lib_path())
    exe = str(tmp_path / "examPointCloud")
    r = subprocess.run([gxx, "-std=c++17", "-include", "experimental/filesystem", "-I",
                        os.path.join(ROOT, "include"), src, "-L", libdir, "-lophpc", "-Wl,-rpath," + libdir,
                        "-Wl,--no-undefined", "-lstdc++fs", "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    nm = subprocess.run(["nm", "-uC", exe], capture_output=True, text=True)
    if nm.returncode == 0:
        used = [ln for ln in nm.stdout.splitlines() if "ophPointCloud::" in ln]
        assert any("generateHologram" in ln for ln in used), nm.stdout


def test_reference_launcher_reports_status_without_crashing():
    """cudaPointCloud_RS with the reference's signature: no config -> a
    status on the calling thread (no device here: NO_DEVICE; with one:
    INVALID_ARGUMENT), nothing launched."""
    L = oph.lib()
    ip, up = ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_uint)
    L.cudaPointCloud_RS.argtypes = [ip, ip, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, up, up]
    L.cudaPointCloud_RS.restype = None
    L.ophpc_refabi_last_status.restype = ctypes.c_int
    one, zero = ctypes.c_int(1), ctypes.c_uint(0)
    L.cudaPointCloud_RS(ctypes.byref(one), ctypes.byref(one), None, None, None, ctypes.byref(zero),
                        ctypes.byref(zero))
    assert L.ophpc_refabi_last_status() in (1, 10)
