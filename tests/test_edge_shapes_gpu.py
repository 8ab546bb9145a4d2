"""Degenerate SLM shapes on every generate path against the FP64 oracle: a
single pixel, a single row, a single column, and a field one pixel wider
than a 128-pixel tensor-core tile. The plain kernels tile the field in 64x32
blocks and the tensor-core kernels in 128x128 tiles; here most of every
tile lies outside the field.

Tolerances: relL2 <= 1e-4 against FP64 for the plain kernels and the
split-BF16 tensor-core paths (the parity bar), 1e-3 for FP16 Fresnel (its
measured error is ~2.5e-4 at full size).
"""
import numpy as np
import pytest

from tests._util import rel_l2, run_generate

pytestmark = pytest.mark.gpu

SHAPES = [(1, 1), (1920, 1), (1, 97), (129, 3)]
PATHS = [("rs", 0, 0, 1e-4), ("rs_tensor", 0, 0x200, 1e-4), ("fresnel", 1, 0, 1e-4),
         ("fresnel_tensor_bf16x3", 1, 0x200, 1e-4), ("fresnel_tensor_fp16", 1, 0x100, 1e-3)]


def _points(n, seed, half):
    rng = np.random.default_rng(seed)
    v = np.zeros((n, 7))
    v[:, 0] = rng.uniform(-half[0], half[0], n)
    v[:, 1] = rng.uniform(-half[1], half[1], n)
    v[:, 2] = rng.uniform(0.2, 0.3, n)
    v[:, 3:6] = 1.0 - rng.uniform(0.0, 1.0, (n, 3))
    return v


@pytest.mark.parametrize("pnx,pny", SHAPES)
@pytest.mark.parametrize("name,diff,mode,tol", PATHS)
def test_degenerate_shapes(gpu_ctx, oracle_mod, pnx, pny, name, diff, mode, tol):
    pp = 8e-6
    gk = dict(pnx=pnx, pny=pny, ppx=pp, ppy=pp, wavelengths=[532e-9, 638e-9])
    v = _points(700, pnx * 31 + pny + diff, (pnx * pp / 2 + 1e-4, pny * pp / 2 + 1e-4))
    g = oracle_mod.Geometry(pnx=pnx, pny=pny, ppx=pp, ppy=pp, wavelengths=[532e-9, 638e-9])
    want = oracle_mod.generate(g, v, diff)
    got = run_generate(gpu_ctx, gk, v, diff, mode)
    assert np.all(np.isfinite(got))
    err = rel_l2(got, want)
    print(f"{name} {pnx}x{pny}: relL2 {err:.3e}")
    assert err <= tol


@pytest.mark.parametrize("name,diff,mode,tol", PATHS)
def test_points_behind_the_slm(gpu_ctx, oracle_mod, name, diff, mode, tol):
    """Negative depths (points behind the SLM, z in [-0.3, -0.2] m) and a
    mix of both signs: the reference's windows use |z| and its amplitudes
    and phases carry the sign (ophGen.cpp:361-514)."""
    pp = 8e-6
    gk = dict(pnx=200, pny=136, ppx=pp, ppy=pp, wavelengths=[532e-9])
    g = oracle_mod.Geometry(pnx=200, pny=136, ppx=pp, ppy=pp, wavelengths=[532e-9])
    v = _points(600, 77 + diff, (1e-3, 1e-3))
    v[:, 2] = -v[:, 2]
    v[::3, 2] = -v[::3, 2]   # every third point in front again
    want = oracle_mod.generate(g, v, diff)
    got = run_generate(gpu_ctx, gk, v, diff, mode)
    err = rel_l2(got, want)
    print(f"{name} behind the SLM: relL2 {err:.3e}")
    assert err <= tol
