"""Serving engine: continuous batching of mixed hologram jobs.

The bar: a job's result is the same alone and in the mix, and
jobs that arrive while others run are admitted and overlap on the device.
Alone-vs-mix results are compared bit for bit (each job's chunking and FP64
accumulation order are fixed by the job alone); against the single-call
entry point the tolerance is relL2 <= 1e-6 (only the FP64 summation order of
point-range partial sums differs), and against the FP64 oracle the parity
bar relL2 <= 1e-4.
"""
import numpy as np
import pytest

from tests._util import rel_l2, run_generate

pytestmark = pytest.mark.gpu


def _jobs(seed=0, n_jobs=10):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n_jobs):
        pnx = int(rng.choice([96, 160, 256, 384]))
        pny = int(rng.choice([64, 128, 200]))
        nch = int(rng.integers(1, 4))
        n = int(np.exp(rng.uniform(np.log(300), np.log(20000))))
        v = np.zeros((n, 7))
        v[:, 0] = rng.uniform(-5e-4, 5e-4, n)
        v[:, 1] = rng.uniform(-5e-4, 5e-4, n)
        v[:, 2] = rng.uniform(0.05, 0.3, n)
        v[:, 3:6] = 1.0 - rng.uniform(0.0, 1.0, (n, 3))
        geom = dict(pnx=pnx, pny=pny, ppx=8e-6, ppy=8e-6, wavelengths=[638e-9, 532e-9, 473e-9][:nch])
        out.append((geom, v, int(rng.integers(0, 2))))
    return out


def test_same_alone_and_in_mix_and_overlap(gpu_ctx, oracle_mod):
    from openholo_gb300.serving import Server
    jobs = _jobs()
    with Server(0, max_in_flight=4, step_ms=0.5) as srv:
        alone = []
        for g, v, d in jobs:
            r = srv.wait(srv.submit(g, v, d))
            assert r.status == 0
            alone.append(r)
        tickets = [srv.submit(g, v, d) for g, v, d in jobs]
        mix = [srv.wait(t) for t in tickets]
    for (g, v, d), a, m in zip(jobs, alone, mix):
        assert m.status == 0
        assert np.array_equal(a.field, m.field)
        direct = run_generate(gpu_ctx, g, v, d)
        assert rel_l2(m.field, direct) <= 1e-6
    # admitted jobs overlapped in time on the device
    spans = sorted((m.t_admit, m.t_done) for m in mix)
    overlaps = sum(1 for i in range(1, len(spans)) if spans[i][0] < spans[i - 1][1])
    assert overlaps >= 1
    # and the FP64 oracle agrees on two of them
    for k in (0, 3):
        g, v, d = jobs[k]
        og = oracle_mod.Geometry(**{x: g[x] for x in ("pnx", "pny", "ppx", "ppy", "wavelengths")})
        assert rel_l2(mix[k].field, oracle_mod.generate(og, v, d)) <= 1e-4


def test_codes_match_device_encoder(gpu_ctx):
    from openholo_gb300.serving import Server
    from tests._util import run_encode
    g, v, d = _jobs(seed=3, n_jobs=1)[0]
    with Server(0) as srv:
        r = srv.wait(srv.submit(g, v, d, want_field=True, want_codes=True, encode_flag=0))
    _, codes = run_encode(gpu_ctx, r.field, 0)
    assert np.array_equal(r.codes, codes)


def test_memory_admission_serialises_jobs(gpu_ctx):
    from openholo_gb300 import OphpcError
    from openholo_gb300.serving import Server
    g0, v0, d0 = _jobs(seed=5, n_jobs=1)[0]
    jobs = [(g0, v0, d0)] * 4          # equal jobs: exactly one fits the budget
    one = max(  # bytes of the largest job, as the server counts them
        (v.shape[0] * 56 + v.shape[0] * 64 * len(g["wavelengths"]) +
         g["pnx"] * g["pny"] * len(g["wavelengths"]) * 17 + 4 * 256 + 256) for g, v, _ in jobs)
    with Server(0, max_in_flight=4, memory_budget=int(one * 1.5)) as srv:
        res = [srv.wait(t) for t in [srv.submit(g, v, d) for g, v, d in jobs]]
        spans = sorted((r.t_admit, r.t_done) for r in res)
        assert all(spans[i][0] >= spans[i - 1][1] - 1e-6 for i in range(1, len(spans)))
        big = dict(pnx=4096, pny=4096, ppx=8e-6, ppy=8e-6, wavelengths=[532e-9])
        with pytest.raises(OphpcError):
            srv.submit(big, np.zeros((10, 7)), 0)


def test_policies_give_identical_results(gpu_ctx):
    """The three policies (earliest deadline, the default; shortest remaining
    work; short jobs first) reorder steps, not arithmetic: every job's field
    is the same under each."""
    from openholo_gb300 import OphpcError
    from openholo_gb300.serving import POLICY_DEADLINE, POLICY_EARLIEST_DEADLINE, POLICY_SHORTEST_REMAINING, Server
    jobs = _jobs(seed=7)
    fields = {}
    for pol in (POLICY_EARLIEST_DEADLINE, POLICY_SHORTEST_REMAINING, POLICY_DEADLINE):
        with Server(0, max_in_flight=4, step_ms=0.5, policy=pol) as srv:
            tickets = [srv.submit(g, v, d) for g, v, d in jobs]
            fields[pol] = [srv.wait(t).field for t in tickets]
    for other in (POLICY_SHORTEST_REMAINING, POLICY_DEADLINE):
        for a, b in zip(fields[POLICY_EARLIEST_DEADLINE], fields[other]):
            assert np.array_equal(a, b)
    with pytest.raises(OphpcError):
        Server(0, policy=7)


def test_tensor_core_jobs_in_the_mix(gpu_ctx, oracle_mod):
    """Jobs submitted with OPHPC_MODE_TENSOR_BF16X3 run as steps on the tensor
    cores (RS: point ranges of the tensor-core RS; Fresnel: one channel's
    chunk of factor tables + GEMM per step), mixed with FP32-core jobs: alone
    and in the mix bit for bit; against the single-call tensor-core generate
    within relL2 3e-5 (both ~1e-5 from FP64; the tensor core's FP32
    accumulation runs start at other points); against the FP64 oracle
    within the parity bar."""
    from openholo_gb300.serving import Server
    jobs = _jobs(seed=9, n_jobs=8)
    modes = [0x200 if k % 4 != 3 else 0 for k in range(len(jobs))]
    with Server(0, max_in_flight=4, step_ms=0.5) as srv:
        alone = [srv.wait(srv.submit(g, v, d, mode=m)) for (g, v, d), m in zip(jobs, modes)]
        tickets = [srv.submit(g, v, d, mode=m) for (g, v, d), m in zip(jobs, modes)]
        mix = [srv.wait(t) for t in tickets]
    for (g, v, d), m, a, x in zip(jobs, modes, alone, mix):
        assert a.status == 0 and x.status == 0
        assert np.array_equal(a.field, x.field)
        direct = run_generate(gpu_ctx, g, v, d, m)
        e = rel_l2(x.field, direct)
        print(f"diff {d} mode {m:#x} ({v.shape[0]} points): served vs single call relL2 {e:.2e}")
        assert e <= (3e-5 if m else 1e-6)
    for k in (1, 2):   # Fresnel (625 points) and RS (17,070 points) on the tensor cores
        g, v, d = jobs[k]
        og = oracle_mod.Geometry(**{x: g[x] for x in ("pnx", "pny", "ppx", "ppy", "wavelengths")})
        assert rel_l2(mix[k].field, oracle_mod.generate(og, v, d)) <= 1e-4


def test_tensor_fresnel_fp16_served(gpu_ctx):
    """FP16 tensor-core Fresnel (one product, ~2.5e-4 from FP64) through the
    server equals its single-call result within the FP16 tolerance."""
    from openholo_gb300.serving import Server
    g, v, d = [j for j in _jobs(seed=9, n_jobs=8) if j[2] == 1][0]
    with Server(0, step_ms=0.2) as srv:
        r = srv.wait(srv.submit(g, v, d, mode=0x100))
    assert r.status == 0
    assert rel_l2(r.field, run_generate(gpu_ctx, g, v, d, 0)) <= 1e-3


def test_tensor_modes_rejected_where_not_served(gpu_ctx):
    from openholo_gb300 import OphpcError
    from openholo_gb300.serving import Server
    g, v, _ = _jobs(seed=9, n_jobs=1)[0]
    with Server(0) as srv:
        for d, m in ((0, 0x100), (0, 0x300), (1, 0x300)):
            with pytest.raises(OphpcError):
                srv.submit(g, v, d, mode=m)


def test_poll_does_not_block(gpu_ctx):
    """ophpc_server_wait with timeout 0 polls: None while the job runs, then
    the job's result, the same as a blocking wait; the ticket is spent
    after that."""
    import time
    from openholo_gb300.serving import Server
    rng = np.random.default_rng(11)
    n = 20000
    v = np.zeros((n, 7))
    v[:, 0:2] = rng.uniform(-5e-4, 5e-4, (n, 2))
    v[:, 2] = rng.uniform(0.1, 0.3, n)
    v[:, 3:6] = 1.0 - rng.uniform(0.0, 1.0, (n, 3))
    g = dict(pnx=2048, pny=2048, ppx=8e-6, ppy=8e-6, wavelengths=[532e-9])
    with Server(0) as srv:
        blocking = srv.wait(srv.submit(g, v, 0))
        t = srv.submit(g, v, 0)
        assert srv.poll(t) is None      # ~5e10 interactions, polled right after submission
        r, t0 = None, time.monotonic()
        while r is None and time.monotonic() - t0 < 60.0:
            time.sleep(1e-3)
            r = srv.poll(t)
        assert r is not None and r.status == 0
        assert np.array_equal(r.field, blocking.field)
        assert srv.poll(t).status != 0  # spent ticket: OPHPC_ERROR_INVALID_ARGUMENT
