"""8-bit holograms over whole benchmark fields against the reference's encoding.

ophGen::normalize takes the minimum and maximum over every pixel of every
channel (ophgen/src/ophGen.cpp:654-687, Openholo/src/function.h:79-99), so
the codes of one pixel depend on the whole field: these checks encode full
fields, not samples.

* rs_1k (1024x1024, 8 um, 532 nm, 5,000 points, seed 0): the FP64 field of
  the CPU oracle over every pixel (OpenMP on the host cores, ~20 s per
  method), against the FP32-core RS kernel, the tensor-core RS, the plain
  Fresnel kernel and the split-BF16 tensor-core Fresnel; phase and
  amplitude codes over all 1,048,576 pixels.
* sphere_fhd (1920x1080, three colours, 100,000 points): the FP64 field of
  the reference's own FP64 GPU kernel (ophgen/src/ophPCKernel.cu, compiled
  unchanged for sm_103a; ~3 minutes), pinned here against the CPU oracle's
  codes on rs_1k, against the headline step (tensor-core RS, phase encoding,
  normalisation over the three channels).

Bar: codes equal on >= 99.9 % of pixels and within +-1 LSB elsewhere (phase
codes wrap around: 255 and 0 are neighbours); fields within relL2 1e-4.
"""
import numpy as np
import pytest

from tests._util import code_agreement, rel_l2

pytestmark = pytest.mark.gpu

FIELD_TOL = 1e-4
CODES_EXACT = 0.999


def _device_codes(ctx, field_dev, nch, npx, flag):
    import torch
    codes = torch.empty((nch, npx), dtype=torch.uint8, device="cuda")
    ctx.encode(field_dev.data_ptr(), nch, npx, flag, None, codes.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return codes.cpu().numpy()


def _generate_dev(ctx, w, diff, mode):
    import torch

    import openholo_gb300 as oph
    cfg = oph.make_config(**w.geometry_kwargs())
    dv = torch.from_numpy(w.vertices).cuda()
    f = torch.empty((w.n_channels, w.pny, w.pnx, 2), dtype=torch.float64, device="cuda")
    ctx.generate(cfg, dv.data_ptr(), w.n_points, diff, mode, f.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return f


def _reference_codes(field, flag):
    import oracle
    codes, _, _ = oracle.normalize(oracle.encode(field, flag))
    return codes.reshape(field.shape[0], -1)


@pytest.fixture(scope="module")
def rs_1k_oracle(oracle_mod):
    from openholo_gb300 import workloads
    w = workloads.rs_1k()
    g = oracle_mod.Geometry(pnx=w.pnx, pny=w.pny, ppx=w.pp, ppy=w.pp, wavelengths=list(w.wavelengths))
    fields = {diff: oracle_mod.generate(g, w.vertices, diff) for diff in (0, 1)}
    codes = {(diff, flag): _reference_codes(fields[diff], flag) for diff in (0, 1) for flag in (0, 1)}
    return w, fields, codes


@pytest.mark.parametrize("diff,mode", [(0, 0), (0, 0x200), (1, 0), (1, 0x200)],
                         ids=["rs_plain", "rs_tensor", "fresnel_plain", "fresnel_tensor_bf16x3"])
def test_rs_1k_full_field_codes(gpu_ctx, rs_1k_oracle, diff, mode):
    w, fields, codes = rs_1k_oracle
    f = _generate_dev(gpu_ctx, w, diff, mode)
    h = f.cpu().numpy()
    err = rel_l2(h[..., 0] + 1j * h[..., 1], fields[diff])
    assert err <= FIELD_TOL, f"field relL2 {err:.3e}"
    npx = w.pnx * w.pny
    for flag in (0, 1):
        got = _device_codes(gpu_ctx, f, w.n_channels, npx, flag)
        exact, maxd = code_agreement(got, codes[(diff, flag)], flag == 0)
        assert exact >= CODES_EXACT and maxd <= 1, f"encode {flag}: exact {exact:.5f}, max |d| {maxd}"


@pytest.fixture(scope="module")
def ref_kernels():
    from oracle import ref_gpu
    if not ref_gpu.available():
        pytest.skip("reference GPU kernels not built (needs the reference tree at build time)")
    k = ref_gpu.RefGpuKernels()
    yield k
    k.close()


def test_reference_fp64_kernel_codes_pinned_on_rs_1k(ref_kernels, rs_1k_oracle):
    """The checker of the sphere_fhd test, the reference's FP64 GPU kernel,
    gives the CPU oracle's codes on a whole rs_1k field."""
    w, fields, codes = rs_1k_oracle
    theirs = ref_kernels.generate(w.geometry_kwargs(), w.vertices, 0, chunk_points=1000)
    assert rel_l2(theirs, fields[0]) <= 1e-8
    for flag in (0, 1):
        exact, maxd = code_agreement(_reference_codes(theirs, flag), codes[(0, flag)], flag == 0)
        assert exact >= 0.99999 and maxd <= 1, (flag, exact, maxd)


def test_sphere_fhd_headline_step_codes(gpu_ctx, ref_kernels):
    from openholo_gb300 import workloads
    w = workloads.sphere_fhd()
    ref = ref_kernels.generate(w.geometry_kwargs(), w.vertices, 0, chunk_points=5000)
    f = _generate_dev(gpu_ctx, w, 0, 0x200)
    h = f.cpu().numpy()
    err = rel_l2(h[..., 0] + 1j * h[..., 1], ref)
    assert err <= FIELD_TOL, f"field relL2 {err:.3e}"
    npx = w.pnx * w.pny
    for flag in (0, 1):
        got = _device_codes(gpu_ctx, f, w.n_channels, npx, flag)
        exact, maxd = code_agreement(got, _reference_codes(ref, flag), flag == 0)
        assert exact >= CODES_EXACT and maxd <= 1, f"encode {flag}: exact {exact:.5f}, max |d| {maxd}"
