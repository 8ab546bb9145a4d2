"""The WRP oracle pinned to the reference's own splat planes (CPU, no GPU).

tests/golden/wrp_*.npz hold the planes ophWRP::calculateWRPCPU
(ophgen/src/ophWRP.cpp:321-420) computed, captured from the reference build
by oracle/ref_wrp_driver.cpp (tests/golden/make_golden.py). The reference
adds the points in OpenMP atomic order and the oracle in index order, so the
two agree to the last few bits; the propagation step has no reference pin
(the reference's buffer is aliased) and is checked here for the properties
the transform must have.
"""
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _geom(oracle_mod, z):
    return oracle_mod.WrpGeometry(pnx=int(z["pnx"]), pny=int(z["pny"]), ppx=float(z["ppx"]), ppy=float(z["ppy"]),
                                  wavelengths=list(z["wavelengths"]), scale=tuple(z["scale"]),
                                  wrp_location=float(z["wrp_location"]), distance=float(z["distance"]))


@pytest.mark.parametrize("name", ["wrp_3ch", "wrp_negdz_edges"])
def test_wrp_plane_matches_reference(oracle_mod, name):
    z = np.load(os.path.join(GOLD, name + ".npz"))
    g = _geom(oracle_mod, z)
    planes = np.stack([oracle_mod.wrp_plane(g, z["vertices"], c) for c in range(len(g.wavelengths))])
    ref = z["planes"]
    assert np.count_nonzero(ref) > 1000
    assert np.array_equal(planes != 0, ref != 0)
    assert np.linalg.norm(planes - ref) <= 1e-13 * np.linalg.norm(ref)


def test_wrp_dice_plane_matches_reference(oracle_mod):
    """The reference's WRP example (Example/dataset/Dice/WRP/Dice_WRP.xml,
    the Dice point cloud): sampled pixels, count, sum and norm."""
    import re
    z = np.load(os.path.join(GOLD, "wrp_dice.npz"))
    xml = str(z["xml"])

    def num(tag):
        return float(re.search(rf"<{tag}>([^<]+)</{tag}>", xml).group(1))
    g = oracle_mod.WrpGeometry(pnx=int(num("SLM_PixelNumX")), pny=int(num("SLM_PixelNumY")),
                               ppx=num("SLM_PixelPitchX"), ppy=num("SLM_PixelPitchY"),
                               wavelengths=[num("SLM_WaveLength_1")],
                               scale=(num("ScaleX"), num("ScaleY"), num("ScaleZ")),
                               wrp_location=num("LocationOfWRP"), distance=num("Distance"))
    p = oracle_mod.wrp_plane(g, z["vertices"], 0)
    assert np.count_nonzero(p) == int(z["nonzero"])
    at = p.reshape(-1)[z["pixel_index"]]
    assert np.linalg.norm(at - z["plane_at"]) <= 1e-13 * np.linalg.norm(z["plane_at"])
    assert abs(p.sum() - complex(z["plane_sum"])) <= 1e-12 * abs(complex(z["plane_sum"]))
    assert abs(np.linalg.norm(p) - float(z["plane_norm"])) <= 1e-13 * float(z["plane_norm"])


def test_wrp_propagation_properties(oracle_mod):
    """Distance 0 returns the plane times the unnormalised transform size;
    propagating forward then back by the same distance returns it (the
    transfer function is unitary where 1/lambda^2 > fx^2 + fy^2)."""
    rng = np.random.default_rng(3)
    pny, pnx = 24, 40
    plane = rng.normal(size=(pny, pnx)) + 1j * rng.normal(size=(pny, pnx))
    g = oracle_mod.WrpGeometry(pnx=pnx, pny=pny, ppx=8e-6, ppy=8e-6, wavelengths=[532e-9], distance=0.0)
    n = 4 * pnx * pny
    assert np.allclose(oracle_mod.wrp_propagate(plane, g, 532e-9), plane * n, rtol=0, atol=1e-10 * n)
    # a plane supported in the centre quarter: no wrap-around within the padding
    small = np.zeros((pny, pnx), complex)
    small[8:16, 14:26] = plane[8:16, 14:26]
    gf = oracle_mod.WrpGeometry(pnx=pnx, pny=pny, ppx=8e-6, ppy=8e-6, wavelengths=[532e-9], distance=1e-4)
    gb = oracle_mod.WrpGeometry(pnx=pnx, pny=pny, ppx=8e-6, ppy=8e-6, wavelengths=[532e-9], distance=-1e-4)
    # forward then backward over the padded buffer is exact only without the
    # crop; check energy conservation of the forward step instead
    f = oracle_mod.wrp_propagate(small, gf, 532e-9) / n
    assert abs(np.linalg.norm(f) - np.linalg.norm(small)) <= 0.05 * np.linalg.norm(small)
    b = oracle_mod.wrp_propagate(f, gb, 532e-9) / n
    assert np.linalg.norm(b - small) <= 0.1 * np.linalg.norm(small)
