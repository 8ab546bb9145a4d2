"""Parity at the benchmark's full sizes, where the oracle cannot compute a
whole field in seconds: the device field is checked against the FP64 oracle
at seeded pixels plus a row segment and a column segment that cross tile
boundaries (stripe artefacts would show there), and, for the 1920x1080
case, through additivity over disjoint point sets at full size.

Workloads (openholo_gb300/workloads.py, seeded synthetic inputs with the
benchmark's shapes and distributions): rs_1k 1024x1024 / 5,000 points,
sphere_fhd 1920x1080 x 3 colours / 100,000, box_4k 3840x2160 / 1,000,000,
box_8k 7680x4320 / 2,000,000. Bars: relL2 <= 1e-4 (plain kernels, tensor
cores split-BF16 for Fresnel and RS)."""
import numpy as np
import pytest

from tests._util import rel_l2

pytestmark = [pytest.mark.gpu, pytest.mark.slow]

FIELD_TOL = 1e-4


def _pixels(pnx, pny, n_random, seg, seed):
    rng = np.random.default_rng(seed)
    idx = rng.choice(pnx * pny, n_random, replace=False)
    y0, x0 = pny // 2 - 7, pnx // 2 - seg // 2 + 3          # off-centre, crossing tile edges
    row = y0 * pnx + x0 + np.arange(seg)
    col = (pny // 2 - seg // 2 + 5 + np.arange(seg)) * pnx + pnx // 3
    return np.unique(np.concatenate([idx, row, col]))


def _generate(ctx, w, diff, mode=0):
    import torch

    import openholo_gb300 as oph
    cfg = oph.make_config(**w.geometry_kwargs())
    dv = torch.from_numpy(w.vertices).cuda()
    f = torch.empty((w.n_channels, w.pny, w.pnx, 2), dtype=torch.float64, device="cuda")
    ctx.generate(cfg, dv.data_ptr(), w.n_points, diff, mode, f.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return f


def _check_at(oracle_mod, w, f, diff, idx, channels=None):
    g = oracle_mod.Geometry(pnx=w.pnx, pny=w.pny, ppx=w.pp, ppy=w.pp, wavelengths=list(w.wavelengths),
                            scale=w.scale, distance=w.distance)
    for ch in (channels if channels is not None else range(w.n_channels)):
        want = oracle_mod.field_at(g, w.vertices, diff, ch, idx)
        h = f[ch].reshape(-1, 2)[idx].cpu().numpy()
        got = h[:, 0] + 1j * h[:, 1]
        e = rel_l2(got, want)
        print(f"  {w.name} diff {diff} ch {ch}: relL2 {e:.2e} on {idx.size} pixels")
        assert e <= FIELD_TOL


@pytest.mark.parametrize("diff", [0, 1])
def test_rs_1k(gpu_ctx, oracle_mod, diff):
    from openholo_gb300 import workloads
    w = workloads.rs_1k()
    _check_at(oracle_mod, w, _generate(gpu_ctx, w, diff), diff, _pixels(w.pnx, w.pny, 4096, 256, 1))


@pytest.mark.parametrize("diff", [0, 1])
def test_sphere_fhd(gpu_ctx, oracle_mod, diff):
    from openholo_gb300 import workloads
    w = workloads.sphere_fhd()
    _check_at(oracle_mod, w, _generate(gpu_ctx, w, diff), diff, _pixels(w.pnx, w.pny, 768, 128, 2))


def test_sphere_fhd_tensor_rs(gpu_ctx, oracle_mod):
    """The headline configuration on the tensor-core RS path."""
    import openholo_gb300 as oph
    from openholo_gb300 import workloads
    w = workloads.sphere_fhd()
    _check_at(oracle_mod, w, _generate(gpu_ctx, w, 0, oph.MODE_TENSOR_BF16X3), 0, _pixels(w.pnx, w.pny, 768, 128, 2))


def test_sphere_fhd_additivity(gpu_ctx):
    """Full size: field(A ∪ B) = field(A) + field(B) for disjoint point sets
    (the sum is linear in the points; only rounding differs)."""
    from openholo_gb300 import workloads
    w = workloads.sphere_fhd()
    half = w.n_points // 2
    a = workloads.Workload(w.name, w.pnx, w.pny, w.pp, w.wavelengths, np.ascontiguousarray(w.vertices[:half]),
                           w.distance, w.scale)
    b = workloads.Workload(w.name, w.pnx, w.pny, w.pp, w.wavelengths, np.ascontiguousarray(w.vertices[half:]),
                           w.distance, w.scale)
    for diff in (0, 1):
        whole = _generate(gpu_ctx, w, diff)
        parts = _generate(gpu_ctx, a, diff) + _generate(gpu_ctx, b, diff)
        import torch
        e = float(torch.linalg.vector_norm(whole - parts) / torch.linalg.vector_norm(whole))
        assert e <= 1e-6, (diff, e)


def test_box_4k(gpu_ctx, oracle_mod):
    import openholo_gb300 as oph
    from openholo_gb300 import workloads
    w = workloads.box_4k()
    idx = _pixels(w.pnx, w.pny, 256, 64, 3)
    _check_at(oracle_mod, w, _generate(gpu_ctx, w, 0), 0, idx)                         # plain RS
    _check_at(oracle_mod, w, _generate(gpu_ctx, w, 0, oph.MODE_TENSOR_BF16X3), 0, idx)  # RS, tensor cores
    _check_at(oracle_mod, w, _generate(gpu_ctx, w, 1, oph.MODE_TENSOR_BF16X3), 1, idx)  # Fresnel, tensor cores


def test_box_8k_tensor(gpu_ctx, oracle_mod):
    import openholo_gb300 as oph
    from openholo_gb300 import workloads
    w = workloads.box_8k()
    idx = _pixels(w.pnx, w.pny, 128, 32, 4)
    _check_at(oracle_mod, w, _generate(gpu_ctx, w, 1, oph.MODE_TENSOR_BF16X3), 1, idx)
    # config 5 is an RS workload: the tensor-core RS at full size (6.6e13 interactions)
    _check_at(oracle_mod, w, _generate(gpu_ctx, w, 0, oph.MODE_TENSOR_BF16X3), 0, idx)
