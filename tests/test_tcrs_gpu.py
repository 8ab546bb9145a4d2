"""Tensor-core RS (tcgen05, OPHPC_MODE_TENSOR_BF16X3 with PC_DIFF_RS) against
the FP64 oracle.

Within each 128x128 tile the RS term is expanded into a row factor times a
column factor plus a first-order cross pair, and contracted over the points
on the tensor cores in split-BF16 (the cross pair in FP16) with FP32
accumulation; pairs the expansion does not hold for are added by the
CUDA-core RS kernel. Tolerances: relL2 <= 1e-4 against FP64 (the accuracy
bar), 8-bit phase codes exact on >= 99.9% of pixels and within +-1 LSB.
"""
import numpy as np
import pytest

from tests._util import code_agreement, rel_l2, run_encode, run_generate

pytestmark = pytest.mark.gpu

MODE_BF16X3 = 0x200
RS = 0


def _box(n, xy, z, seed):
    rng = np.random.default_rng(seed)
    v = np.zeros((n, 7))
    v[:, 0] = rng.uniform(-xy[0], xy[0], n)
    v[:, 1] = rng.uniform(-xy[1], xy[1], n)
    v[:, 2] = rng.uniform(z[0], z[1], n)
    v[:, 3:6] = 1.0 - rng.uniform(0.0, 1.0, (n, 3))
    return v


def _mixed(seed):
    """Half the points far (whole-tile windows, tensor cores), half so close
    that their windows cut the tiles (CUDA-core complement)."""
    far = _box(600, (1e-3, 8e-4), (0.25, 0.4), seed)
    near = _box(300, (1e-3, 8e-4), (0.003, 0.02), seed + 1)
    return np.concatenate([far, near])


CASES = {
    "full_aperture": (dict(pnx=384, pny=256, ppx=8e-6, ppy=8e-6, wavelengths=[532e-9]),
                      _box(3000, (1e-3, 1e-3), (0.3, 0.5), 41)),
    "mixed_window_cut_odd": (dict(pnx=300, pny=170, ppx=8e-6, ppy=8e-6, wavelengths=[532e-9]), _mixed(42)),
    "three_channels": (dict(pnx=130, pny=77, ppx=6.4e-6, ppy=7.1e-6, wavelengths=[638e-9, 532e-9, 473e-9],
                            scale=(0.5, 0.5, 2.0), distance=0.05),
                       _box(900, (1e-3, 1e-3), (0.05, 0.2), 43)),
    "fine_pitch": (dict(pnx=512, pny=256, ppx=3.74e-6, ppy=3.74e-6, wavelengths=[532e-9]),
                   _box(2000, (3e-3, 3e-3), (0.29, 0.31), 44)),
    # windows of 830-1250 pixels on a 1536x1024 field: most pairs hold the
    # tile, many cut it (masked factors on the tensor cores) and a few fail
    # the cone test at the window edge (CUDA-core complement)
    "window_cut_tensor": (dict(pnx=1536, pny=1024, ppx=8e-6, ppy=8e-6, wavelengths=[532e-9]),
                          _box(800, (4e-3, 3e-3), (0.1, 0.15), 49)),
}


def _oracle(oracle_mod, gk, v):
    g = oracle_mod.Geometry(**{k: gk[k] for k in ("pnx", "pny", "ppx", "ppy", "wavelengths")},
                            scale=gk.get("scale", (1.0, 1.0, 1.0)), distance=gk.get("distance", 0.0))
    return oracle_mod.generate(g, v, RS)


@pytest.mark.parametrize("name", sorted(CASES))
def test_tensor_rs_meets_the_bar(gpu_ctx, oracle_mod, name):
    import openholo_gb300 as oph
    gk, v = CASES[name]
    ref = _oracle(oracle_mod, gk, v)
    before = oph.lib().ophpc_kernel_launches()
    got = run_generate(gpu_ctx, gk, v, RS, MODE_BF16X3)
    launched = oph.lib().ophpc_kernel_launches() - before
    # prep, one amax reduction per channel, the tensor-core kernel, the
    # complement, and the partial-field sum when the points were split
    assert launched in (3 + len(gk["wavelengths"]), 4 + len(gk["wavelengths"]))
    err = rel_l2(got, ref)
    print(f"{name}: tensor-core RS relL2 = {err:.3e}")
    assert err <= 1e-4
    _, codes = run_encode(gpu_ctx, got, 0)
    codes_ref, _, _ = oracle_mod.normalize(oracle_mod.encode(ref, 0))
    exact, maxd = code_agreement(codes, codes_ref, True)
    print(f"  phase codes exact {exact:.5f} max|d| {maxd}")
    assert exact >= 0.999 and maxd <= 1


def test_tensor_rs_many_points(gpu_ctx):
    """70,000 points: 69 TMEM accumulation runs folded into the TMEM running
    sum, with an FP64 flush every 16 runs. The plain FP32 RS kernel (relL2 ~1e-6 against FP64)
    is the reference here."""
    gk = dict(pnx=640, pny=384, ppx=8e-6, ppy=8e-6, wavelengths=[532e-9])
    v = _box(70000, (2e-3, 2e-3), (0.45, 0.55), 45)
    plain = run_generate(gpu_ctx, gk, v, RS, 0)
    tc = run_generate(gpu_ctx, gk, v, RS, MODE_BF16X3)
    err = rel_l2(tc, plain)
    print(f"tensor-core RS vs plain RS, 70,000 points: relL2 {err:.3e}")
    assert err <= 1e-4


def test_tensor_rs_zero_points_and_determinism(gpu_ctx):
    gk = dict(pnx=150, pny=100, ppx=8e-6, ppy=8e-6, wavelengths=[532e-9])
    z = run_generate(gpu_ctx, gk, np.zeros((0, 7)), RS, MODE_BF16X3)
    assert not np.any(z)
    v = _mixed(46)
    a = run_generate(gpu_ctx, gk, v, RS, MODE_BF16X3)
    b = run_generate(gpu_ctx, gk, v, RS, MODE_BF16X3)
    assert np.array_equal(a, b)


def test_tensor_rs_single_point_known_answer(gpu_ctx):
    """One on-axis point: the field is the analytic RS term at every pixel."""
    gk = dict(pnx=256, pny=128, ppx=8e-6, ppy=8e-6, wavelengths=[532e-9])
    v = np.array([[1.3e-4, -7e-5, 0.4, 0.8, 0.8, 0.8, 0.0]])
    got = run_generate(gpu_ctx, gk, v, RS, MODE_BF16X3)[0]
    lam = 532e-9
    xs = -256 * 8e-6 / 2 + (np.arange(256) - 1) * 8e-6
    ys = -128 * 8e-6 / 2 + (128 - np.arange(128)) * 8e-6
    X, Y = np.meshgrid(xs, ys)
    r = np.sqrt((X - v[0, 0]) ** 2 + (Y - v[0, 1]) ** 2 + v[0, 2] ** 2)
    amp = 0.8 * v[0, 2] / (lam * r * r)
    k = 2 * np.pi / lam
    want = amp * (np.sin(k * r) - 1j * np.cos(k * r))
    err = rel_l2(got, want)
    print(f"single point: relL2 {err:.3e}")
    assert err <= 1e-4


@pytest.mark.parametrize("n", [1, 15, 17, 1024, 1030, 2064, 16400])
def test_tensor_rs_point_counts(gpu_ctx, n):
    """Point counts at the edges of the kernel's pipeline: partial last
    stage, a last stage that opens a new accumulation run (1030, 2064), an
    FP64 flush in the middle (16400 = 17 runs). The plain FP32 RS kernel is
    the reference."""
    gk = dict(pnx=256, pny=200, ppx=8e-6, ppy=8e-6, wavelengths=[638e-9])
    v = _box(n, (1.5e-3, 1.5e-3), (0.35, 0.5), 47 + n)
    plain = run_generate(gpu_ctx, gk, v, RS, 0)
    tc = run_generate(gpu_ctx, gk, v, RS, MODE_BF16X3)
    err = rel_l2(tc, plain)
    print(f"n={n}: tensor-core RS vs plain relL2 {err:.3e}")
    assert err <= 1e-4


def test_tensor_rs_offset_scale_viewing_window(gpu_ctx, oracle_mod):
    """Pixel offsets, per-axis scale, a distance and the viewing-window
    transform (transVW, ophgen/src/ophGen.cpp:1976-1985) reach the tensor-core
    path through the same point preparation as the FP32-core kernels."""
    gk = dict(pnx=320, pny=200, ppx=6e-6, ppy=7e-6, wavelengths=[532e-9, 638e-9],
              scale=(0.8, 1.2, 1.5), distance=0.1)
    v = _box(1500, (1e-3, 1e-3), (0.15, 0.3), 48)
    kw = dict(offset=(5, -3), viewing_window=True, field_length=0.9)
    g = oracle_mod.Geometry(**{k: gk[k] for k in ("pnx", "pny", "ppx", "ppy", "wavelengths")},
                            scale=gk["scale"], distance=gk["distance"], offset=kw["offset"],
                            viewing_window=True, field_length=kw["field_length"])
    ref = oracle_mod.generate(g, v, RS)
    got = run_generate(gpu_ctx, gk, v, RS, MODE_BF16X3, **kw)
    err = rel_l2(got, ref)
    print(f"offset / scale / viewing window: relL2 {err:.3e}")
    assert err <= 1e-4
