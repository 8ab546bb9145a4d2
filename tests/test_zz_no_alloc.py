"""The allocation-free entry point, ophpc_generate_static_scratch.

It serves callers that cannot allocate device memory (a host whose device
memory is owned by its own allocator under a fixed budget, or a real-time loop
that must never enter cudaMalloc/cudaFree): its scratch is a fixed 32 MiB
device array inside the library instead of per-call allocations. These checks
call it through the C ABI, twice in a row with different inputs (the array
keeps the previous call's contents), and compare each result with the
allocating entry point ophpc_generate within the parity tolerance the other
GPU tests use (relative L2 error <= 1e-4). The file is named to run last so
that a stop-at-first-failure run has already run every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIELD_TOL = 1e-4


def _points(n, seed, z=(0.05, 0.3)):
    rng = np.random.default_rng(seed)
    v = np.zeros((n, 7))
    v[:, 0] = rng.uniform(-1e-3, 1e-3, n)
    v[:, 1] = rng.uniform(-1e-3, 1e-3, n)
    v[:, 2] = rng.uniform(z[0], z[1], n)
    v[:, 3:6] = 1.0 - rng.uniform(0.0, 1.0, (n, 3))
    return v


def _entry(lib):
    f = lib.ophpc_generate_static_scratch
    f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32,
                  ctypes.c_void_p, ctypes.c_void_p]
    f.restype = ctypes.c_int
    return f


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_static_scratch_matches_allocating_entry_point():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("GPU test selected but no CUDA device is visible")
    import openholo_gb300 as oph

    lib = oph.lib()
    gen_static = _entry(lib)
    torch.cuda.set_device(0)
    stream = torch.cuda.current_stream()
    with oph.Context(0) as ctx:
        # two calls in a row per method; the second has fewer points and a
        # window-cutting geometry, so leftovers of the first would show
        cases = [
            (oph.make_config(200, 120, 8e-6, 8e-6, [532e-9, 638e-9]), _points(1500, 1)),
            (oph.make_config(96, 80, 8e-6, 8e-6, [473e-9]), _points(300, 2, z=(0.002, 0.01))),
        ]
        for diff in (oph.DIFF_RS, oph.DIFF_FRESNEL):
            for cfg, v in cases:
                nch, pnx, pny = cfg.n_channels, cfg.pixel_number[0], cfg.pixel_number[1]
                dv = torch.from_numpy(v).cuda()
                want = torch.empty((nch, pny, pnx, 2), dtype=torch.float64, device="cuda")
                got = torch.full_like(want, float("nan"))
                ctx.generate(cfg, dv.data_ptr(), v.shape[0], diff, 0, want.data_ptr(), stream.cuda_stream)
                st = gen_static(ctypes.byref(cfg), dv.data_ptr(), v.shape[0], diff, 0, got.data_ptr(),
                                stream.cuda_stream)
                assert st == 0, f"status {st}"
                torch.cuda.synchronize()
                err = _rel(got.cpu().numpy(), want.cpu().numpy())
                assert err <= FIELD_TOL, f"diff={diff}: relL2 {err:.3e}"


def test_static_scratch_full_array_and_empty_call():
    """The largest accepted call fills the array exactly (one channel,
    OPHPC_STATIC_SCRATCH_RECORDS points); a call with no points writes a zero
    field over whatever the buffer held."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("GPU test selected but no CUDA device is visible")
    import openholo_gb300 as oph

    gen_static = _entry(oph.lib())
    torch.cuda.set_device(0)
    stream = torch.cuda.current_stream()
    cfg = oph.make_config(64, 64, 8e-6, 8e-6, [532e-9])
    v = _points(524288, 3, z=(0.2, 0.3))
    dv = torch.from_numpy(v).cuda()
    with oph.Context(0) as ctx:
        for diff in (oph.DIFF_RS, oph.DIFF_FRESNEL):
            want = torch.empty((1, 64, 64, 2), dtype=torch.float64, device="cuda")
            got = torch.full_like(want, float("nan"))
            ctx.generate(cfg, dv.data_ptr(), v.shape[0], diff, 0, want.data_ptr(), stream.cuda_stream)
            st = gen_static(ctypes.byref(cfg), dv.data_ptr(), v.shape[0], diff, 0, got.data_ptr(),
                            stream.cuda_stream)
            assert st == 0, f"status {st}"
            torch.cuda.synchronize()
            err = _rel(got.cpu().numpy(), want.cpu().numpy())
            assert err <= FIELD_TOL, f"diff={diff}, full array: relL2 {err:.3e}"
    empty = torch.full((1, 64, 64, 2), float("nan"), dtype=torch.float64, device="cuda")
    st = gen_static(ctypes.byref(cfg), dv.data_ptr(), 0, oph.DIFF_RS, 0, empty.data_ptr(), stream.cuda_stream)
    assert st == 0, f"status {st}"
    torch.cuda.synchronize()
    assert bool((empty == 0).all())


def test_static_scratch_rejects_sizes_beyond_its_array():
    torch = pytest.importorskip("torch")
    import openholo_gb300 as oph

    gen_static = _entry(oph.lib())
    cfg = oph.make_config(64, 64, 8e-6, 8e-6, [532e-9, 638e-9])
    dv = torch.zeros((4, 7), dtype=torch.float64, device="cuda")
    out = torch.zeros((2, 64, 64, 2), dtype=torch.float64, device="cuda")
    too_many = 524288 // 2 + 1     # n_points * n_channels above OPHPC_STATIC_SCRATCH_RECORDS
    st = gen_static(ctypes.byref(cfg), dv.data_ptr(), too_many, 0, 0, out.data_ptr(), None)
    assert st == 1   # OPHPC_ERROR_INVALID_ARGUMENT, rejected before any work is queued
    torch.cuda.synchronize()
    assert not out.any()
    # a NULL config is an invalid argument, as for ophpc_generate
    st = gen_static(None, dv.data_ptr(), 4, 0, 0, out.data_ptr(), None)
    assert st == 1
