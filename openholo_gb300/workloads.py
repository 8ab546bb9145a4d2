"""Seeded synthetic point clouds and SLM geometries of the benchmark workloads.

The reference ships no benchmark data; these generators stand in for it with
the shapes, sizes and value distributions of the five workloads:

  rs_1k        1024x1024 SLM, 8.0 um pitch, 532 nm, 5,000 points,
               x, y ~ U(+-2 mm), z ~ U[0.45, 0.55] m, amplitude U(0, 1], seed 0
  sphere_fhd   1920x1080, 8.0 um, 638/532/473 nm (three channels), 100,000
               points on a sphere of radius 3 mm perturbed by 8 random
               low-order harmonics (l <= 4, eps ~ U(-0.1, 0.1)), centred at
               z = 0.5 m, per-colour amplitude U(0, 1], seed 1
  box_4k       3840x2160, 3.74 um, 532 nm, 1,000,000 points uniform in a
               6x6x20 mm box centred at z = 0.3 m, amplitude log-uniform
               [0.01, 1], seed 3
  box_8k       7680x4320, 3.74 um, 532 nm, 2,000,000 points uniform in a
               10x10x30 mm box centred at z = 0.4 m, amplitude U(0, 1], seed 5
  serving      512 jobs, Poisson arrivals; resolution from {512^2, 1920x1080,
               2048^2, 3840x2160}, N log-uniform [1e3, 5e5], wavelength from
               {473, 532, 638} nm, z-centre U[0.2, 0.8] m, RS/Fresnel 50/50

Vertices are (n, 7) float64 arrays in the reference's Vertex layout
(pos[3], color[3], phase; Openholo/src/struct.h:86-106).
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import List, Sequence, Tuple

import numpy as np


@dataclass
class Workload:
    name: str
    pnx: int
    pny: int
    pp: float
    wavelengths: Tuple[float, ...]
    vertices: np.ndarray
    distance: float = 0.0
    scale: Tuple[float, float, float] = (1.0, 1.0, 1.0)

    @property
    def n_points(self) -> int:
        return int(self.vertices.shape[0])

    @property
    def n_channels(self) -> int:
        return len(self.wavelengths)

    @property
    def interactions(self) -> int:
        """point x pixel pairs over all channels (full-aperture count)."""
        return self.n_points * self.pnx * self.pny * self.n_channels

    def geometry_kwargs(self) -> dict:
        return dict(pnx=self.pnx, pny=self.pny, ppx=self.pp, ppy=self.pp, wavelengths=list(self.wavelengths),
                    scale=self.scale, distance=self.distance)

    def config_xml(self) -> str:
        """The workload's geometry as the flat <PointCloud> config file that
        readConfig parses (ophgen/src/ophGen.cpp:221-358,
        ophgen/src/ophPointCloud.cpp:83-149)."""
        keys = [("ScaleX", self.scale[0]), ("ScaleY", self.scale[1]), ("ScaleZ", self.scale[2]),
                ("Distance", self.distance), ("FieldLength", 0.0), ("SLM_PixelPitchX", self.pp),
                ("SLM_PixelPitchY", self.pp), ("SLM_PixelNumX", self.pnx), ("SLM_PixelNumY", self.pny),
                ("SLM_WaveNum", self.n_channels)]
        keys += [(f"SLM_WaveLength_{i + 1}", float(w)) for i, w in enumerate(self.wavelengths)]
        return "<PointCloud>\n" + "".join(f"  <{k}>{v!r}</{k}>\n" for k, v in keys) + "</PointCloud>\n"

    def subset(self, n: int, name_suffix: str = "") -> "Workload":
        return Workload(self.name + name_suffix, self.pnx, self.pny, self.pp, self.wavelengths,
                        np.ascontiguousarray(self.vertices[:n]), self.distance, self.scale)


def _vertices(xyz: np.ndarray, amp: np.ndarray) -> np.ndarray:
    n = xyz.shape[0]
    v = np.zeros((n, 7), dtype=np.float64)
    v[:, 0:3] = xyz
    if amp.ndim == 1:
        v[:, 3:6] = amp[:, None]
    else:
        v[:, 3:6] = amp
    return v


def rs_1k(n_points: int = 5000, seed: int = 0) -> Workload:
    rng = np.random.default_rng(seed)
    x = rng.uniform(-2e-3, 2e-3, n_points)
    y = rng.uniform(-2e-3, 2e-3, n_points)
    z = rng.uniform(0.45, 0.55, n_points)
    amp = 1.0 - rng.uniform(0.0, 1.0, n_points)          # (0, 1]
    return Workload("rs_1k", 1024, 1024, 8.0e-6, (532e-9,), _vertices(np.stack([x, y, z], 1), amp))


def _real_sph_harm(l: int, m: int, theta: np.ndarray, phi: np.ndarray) -> np.ndarray:
    """Real spherical harmonic (unnormalised): P_l^|m|(cos theta) * cos/sin(m phi)."""
    from scipy.special import lpmv
    p = lpmv(abs(m), l, np.cos(theta))
    return p * (np.cos(m * phi) if m >= 0 else np.sin(-m * phi))


def sphere_fhd(n_points: int = 100_000, seed: int = 1) -> Workload:
    rng = np.random.default_rng(seed)
    d = rng.normal(size=(n_points, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    theta = np.arccos(np.clip(d[:, 2], -1, 1))
    phi = np.arctan2(d[:, 1], d[:, 0])
    radius = np.ones(n_points)
    for _ in range(8):
        l = int(rng.integers(1, 5))
        m = int(rng.integers(-l, l + 1))
        eps = rng.uniform(-0.1, 0.1)
        y = _real_sph_harm(l, m, theta, phi)
        y /= max(1e-12, np.abs(y).max())
        radius += eps * y
    r = 3e-3 * radius
    xyz = d * r[:, None]
    xyz[:, 2] += 0.5
    amp = 1.0 - rng.uniform(0.0, 1.0, (n_points, 3))
    return Workload("sphere_fhd", 1920, 1080, 8.0e-6, (638e-9, 532e-9, 473e-9), _vertices(xyz, amp))


def box_4k(n_points: int = 1_000_000, seed: int = 3) -> Workload:
    rng = np.random.default_rng(seed)
    xyz = np.stack([rng.uniform(-3e-3, 3e-3, n_points), rng.uniform(-3e-3, 3e-3, n_points),
                    rng.uniform(0.3 - 10e-3, 0.3 + 10e-3, n_points)], 1)
    amp = np.exp(rng.uniform(np.log(0.01), 0.0, n_points))
    return Workload("box_4k", 3840, 2160, 3.74e-6, (532e-9,), _vertices(xyz, amp))


def box_8k(n_points: int = 2_000_000, seed: int = 5) -> Workload:
    rng = np.random.default_rng(seed)
    xyz = np.stack([rng.uniform(-5e-3, 5e-3, n_points), rng.uniform(-5e-3, 5e-3, n_points),
                    rng.uniform(0.4 - 15e-3, 0.4 + 15e-3, n_points)], 1)
    amp = 1.0 - rng.uniform(0.0, 1.0, n_points)
    return Workload("box_8k", 7680, 4320, 3.74e-6, (532e-9,), _vertices(xyz, amp))


@dataclass
class ServingJob:
    arrival_s: float
    workload: Workload
    diff_flag: int


def serving_stream(n_jobs: int = 512, rate_per_s: float = 10.0, seed: int = 4,
                   max_points: int = 500_000) -> List[ServingJob]:
    """Mixed hologram jobs with Poisson arrivals at `rate_per_s`."""
    rng = np.random.default_rng(seed)
    resolutions: Sequence[Tuple[int, int]] = [(512, 512), (1920, 1080), (2048, 2048), (3840, 2160)]
    lambdas = [473e-9, 532e-9, 638e-9]
    t = 0.0
    jobs = []
    for j in range(n_jobs):
        t += rng.exponential(1.0 / rate_per_s)
        pnx, pny = resolutions[int(rng.integers(0, len(resolutions)))]
        n = int(np.exp(rng.uniform(np.log(1e3), np.log(max_points))))
        lam = lambdas[int(rng.integers(0, 3))]
        zc = rng.uniform(0.2, 0.8)
        pp = 8.0e-6 if pnx <= 2048 else 3.74e-6
        half = 0.25 * min(pnx * pp, pny * pp)
        xyz = np.stack([rng.uniform(-half, half, n), rng.uniform(-half, half, n),
                        rng.uniform(zc - 5e-3, zc + 5e-3, n)], 1)
        amp = 1.0 - rng.uniform(0.0, 1.0, n)
        w = Workload(f"job{j}", pnx, pny, pp, (lam,), _vertices(xyz, amp))
        jobs.append(ServingJob(t, w, int(rng.integers(0, 2))))
    return jobs


BY_NAME = {"rs_1k": rs_1k, "sphere_fhd": sphere_fhd, "box_4k": box_4k, "box_8k": box_8k}
