"""Plans (ophpc_plan_*): one generate + encode captured into a CUDA graph and
replayed. Every replay must equal the direct ophpc_generate + ophpc_encode
calls bit for bit, and read the vertices that are in its buffer when it is
launched (successive frames of a moving point cloud)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PNX, PNY = 320, 200


def _box(n, seed):
    rng = np.random.default_rng(seed)
    v = np.zeros((n, 7))
    v[:, 0] = rng.uniform(-8e-4, 8e-4, n)
    v[:, 1] = rng.uniform(-6e-4, 6e-4, n)
    v[:, 2] = rng.uniform(0.3, 0.4, n)
    v[:, 3:6] = 1.0 - rng.uniform(0.0, 1.0, (n, 3))
    return v


@pytest.mark.parametrize("diff,mode", [(0, 0), (1, 0), (0, 0x200), (1, 0x200), (1, 0x100)])
def test_plan_replays_match_direct_calls(gpu_ctx, diff, mode):
    import torch

    import openholo_gb300 as oph
    cfg = oph.make_config(pnx=PNX, pny=PNY, ppx=8e-6, ppy=8e-6, wavelengths=[638e-9, 532e-9])
    n = 1500
    dv = torch.empty((n, 7), dtype=torch.float64, device="cuda")
    f = torch.empty((2, PNY, PNX, 2), dtype=torch.float64, device="cuda")
    codes = torch.empty((2, PNY * PNX), dtype=torch.uint8, device="cuda")
    f_ref, c_ref = torch.empty_like(f), torch.empty_like(codes)
    s = torch.cuda.current_stream().cuda_stream
    before = oph.lib().ophpc_kernel_launches()
    with gpu_ctx.plan(cfg, dv.data_ptr(), n, diff, mode, f.data_ptr(), oph.ENCODE_PHASE, None,
                      codes.data_ptr()) as plan:
        captured = oph.lib().ophpc_kernel_launches() - before
        assert captured >= 3   # prep, the kernels, encode: counted once, at capture
        for seed in (1, 2, 3):
            dv.copy_(torch.from_numpy(_box(n, seed)))
            at = oph.lib().ophpc_kernel_launches()
            plan.launch(s)
            plan.wait(s)
            assert oph.lib().ophpc_kernel_launches() == at   # a replay issues no host-side launches
            gpu_ctx.generate(cfg, dv.data_ptr(), n, diff, mode, f_ref.data_ptr(), s)
            gpu_ctx.encode(f_ref.data_ptr(), 2, PNY * PNX, oph.ENCODE_PHASE, None, c_ref.data_ptr(), s)
            torch.cuda.synchronize()
            assert torch.equal(f, f_ref), (diff, mode, seed)
            assert torch.equal(codes, c_ref), (diff, mode, seed)


def test_plan_without_encode_and_zero_points(gpu_ctx):
    import torch

    import openholo_gb300 as oph
    cfg = oph.make_config(pnx=PNX, pny=PNY, ppx=8e-6, ppy=8e-6, wavelengths=[532e-9])
    f = torch.full((1, PNY, PNX, 2), 7.0, dtype=torch.float64, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    with gpu_ctx.plan(cfg, 0, 0, 0, 0, f.data_ptr()) as plan:
        plan.launch(s)
        plan.wait(s)
    assert not torch.any(f)


def test_plan_rejects_what_generate_rejects(gpu_ctx):
    import torch

    import openholo_gb300 as oph
    cfg = oph.make_config(pnx=PNX, pny=PNY, ppx=8e-6, ppy=8e-6, wavelengths=[532e-9])
    f = torch.empty((1, PNY, PNX, 2), dtype=torch.float64, device="cuda")
    dv = torch.zeros((10, 7), dtype=torch.float64, device="cuda")
    with pytest.raises(oph.OphpcError):
        gpu_ctx.plan(cfg, dv.data_ptr(), 10, 5, 0, f.data_ptr())              # bad diff_flag
    with pytest.raises(oph.OphpcError):
        gpu_ctx.plan(cfg, dv.data_ptr(), 10, 0, 0x300, f.data_ptr())          # both tensor modes
    with pytest.raises(oph.OphpcError):
        gpu_ctx.plan(cfg, dv.data_ptr(), 10, 0, 0, f.data_ptr(), 99)          # unsupported encoder
