"""The reference's own GPU kernels (ophgen/src/ophPCKernel.cu, compiled from
its sources for sm_103a into oracle/_ref by `make -C oracle ref`) against
this library and the committed reference CPU fields: a second, independent
pin of the device path. Skipped where the cubin was not built (it needs the
reference tree at build time)."""
import os

import numpy as np
import pytest

from tests._util import rel_l2, run_generate

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def ref_kernels():
    from oracle import ref_gpu
    if not ref_gpu.available():
        pytest.skip("reference GPU kernels not built (needs the reference tree at build time)")
    k = ref_gpu.RefGpuKernels()
    yield k
    k.close()


def _geometry(xml: str) -> dict:
    import re

    def num(tag):
        return float(re.search(rf"<{tag}>([^<]+)</{tag}>", xml).group(1))
    nch = int(num("SLM_WaveNum"))
    return dict(pnx=int(num("SLM_PixelNumX")), pny=int(num("SLM_PixelNumY")), ppx=num("SLM_PixelPitchX"),
                ppy=num("SLM_PixelPitchY"), wavelengths=[num(f"SLM_WaveLength_{i + 1}") for i in range(nch)],
                scale=(num("ScaleX"), num("ScaleY"), num("ScaleZ")), distance=num("Distance"))


@pytest.mark.parametrize("name", ["rs_window_1ch", "fresnel_window_1ch", "fresnel_3ch"])
def test_reference_fp64_kernel_agrees(gpu_ctx, ref_kernels, name):
    """Reference FP64 GPU kernel vs the reference CPU field (same maths, FP64
    both, but the GPU build contracts to FMA and phases reach ~1e6 rad, so
    they differ by ~1e6 x 2^-52 relative) and vs ours (FP32 core with FP64
    phase reduction, the 1e-4 parity bar)."""
    d = np.load(os.path.join(GOLD, name + ".npz"))
    g = _geometry(str(d["xml"]))
    diff = int(d["diff_flag"])
    theirs = ref_kernels.generate(g, d["vertices"], diff)
    assert rel_l2(theirs, d["field"]) <= 1e-8
    ours = run_generate(gpu_ctx, g, d["vertices"], diff)
    assert rel_l2(ours, theirs) <= 1e-4
