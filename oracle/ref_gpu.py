"""The reference's own GPU kernels (ophgen/src/ophPCKernel.cu), compiled from
the reference sources into oracle/_ref/ophPCKernel_sm103a.cubin by
``make -C oracle ref`` and launched here through the CUDA driver API.

TEST INFRASTRUCTURE ONLY: an informational baseline (the reference's GPU
path recompiled for sm_103a, timed on the same GPU) and a second checker for
tests/; the product never loads it. The reference's host driver
(genCghPointCloudGPU, ophgen/src/ophPointCloud_GPU.cpp:179-279) is not used,
because its cudaWrapper divides by zero on sm_10x; this module does what that
driver does for one GPU: config structs filled as their constructors fill
them (ophPointCloud_GPU.h:89-217) and copied to device memory, one thread per
pixel (grid = ceil(pnX*pnY / block)), one launch per colour accumulating into
a zeroed cuDoubleComplex buffer. The kernels write a pixel only inside a
window clamped to [0, pnX) x [0, pnY), so the grid's last partial block
writes nothing out of range.

    python -m oracle.ref_gpu --workload sphere_fhd --points 1000
times the FP64 and FP32 RS/Fresnel kernels on a point subset of the workload
(cost is linear in the point count) and prints one JSON line.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
CUBIN = os.path.join(HERE, "_ref", "ophPCKernel_sm103a.cubin")

# Itanium-mangled names of the reference's __global__ functions
# (uint, Vertex*, const CudaPointCloudConfig{RS,Fresnel}*, cuDoubleComplex*).
KERNELS = {
    (0, False): "_Z32cudaKernel_double_RS_DiffractionjP6VertexPK23_CudaPointCloudConfigRSP7double2",
    (0, True): "_Z32cudaKernel_single_RS_DiffractionjP6VertexPK23_CudaPointCloudConfigRSP7double2",
    (1, False): "_Z37cudaKernel_double_Fresnel_DiffractionjP6VertexPK28_CudaPointCloudConfigFresnelP7double2",
    (1, True): "_Z37cudaKernel_single_Fresnel_DiffractionjP6VertexPK28_CudaPointCloudConfigFresnelP7double2",
}
BLOCK = 256


class RefConfig(ctypes.Structure):
    """_CudaPointCloudConfig + the RS (det_tx, det_ty) or Fresnel (tx, ty)
    pair: 120 bytes."""
    _fields_ = [("n_points", ctypes.c_int32), ("pad0", ctypes.c_int32),
                ("scale_X", ctypes.c_double), ("scale_Y", ctypes.c_double), ("scale_Z", ctypes.c_double),
                ("offset_depth", ctypes.c_double), ("pn_X", ctypes.c_int32), ("pn_Y", ctypes.c_int32),
                ("offset_X", ctypes.c_int32), ("offset_Y", ctypes.c_int32), ("pp_X", ctypes.c_double),
                ("pp_Y", ctypes.c_double), ("half_ss_X", ctypes.c_double), ("half_ss_Y", ctypes.c_double),
                ("k", ctypes.c_double), ("lambda_", ctypes.c_double), ("d0", ctypes.c_double),
                ("d1", ctypes.c_double)]


def make_config(pnx, pny, ppx, ppy, wavelength, n_points, diff_flag, scale=(1.0, 1.0, 1.0), distance=0.0,
                offset=(0, 0)) -> RefConfig:
    c = RefConfig(n_points=n_points, scale_X=scale[0], scale_Y=scale[1], scale_Z=scale[2], offset_depth=distance,
                  pn_X=pnx, pn_Y=pny, offset_X=offset[0], offset_Y=offset[1], pp_X=ppx, pp_Y=ppy,
                  half_ss_X=(pnx * ppx) / 2, half_ss_Y=(pny * ppy) / 2, k=(2 * np.pi) / wavelength,
                  lambda_=wavelength)
    tx, ty = wavelength / (2 * ppx), wavelength / (2 * ppy)
    if diff_flag == 0:
        c.d0, c.d1 = tx / np.sqrt(1 - tx * tx), ty / np.sqrt(1 - ty * ty)
    else:
        c.d0, c.d1 = tx, ty
    return c


def available() -> bool:
    return os.path.exists(CUBIN)


class RefGpuKernels:
    """The cubin loaded into the current (PyTorch primary) context."""

    def __init__(self):
        import torch
        if not available():
            raise FileNotFoundError(f"{CUBIN} not built (make -C oracle ref)")
        torch.cuda.init()
        torch.empty(1, device="cuda")               # make the primary context current
        self.cu = ctypes.CDLL("libcuda.so.1")
        self.cu.cuModuleLoadData.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_void_p]
        self.cu.cuModuleGetFunction.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_void_p, ctypes.c_char_p]
        self.cu.cuLaunchKernel.argtypes = [ctypes.c_void_p] + [ctypes.c_uint] * 6 + \
            [ctypes.c_uint, ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p), ctypes.c_void_p]
        self.cu.cuModuleUnload.argtypes = [ctypes.c_void_p]
        image = open(CUBIN, "rb").read()
        self._image = ctypes.create_string_buffer(image, len(image))
        self.mod = ctypes.c_void_p()
        self._check(self.cu.cuModuleLoadData(ctypes.byref(self.mod), self._image), "cuModuleLoadData")
        self.fn = {}
        for key, name in KERNELS.items():
            f = ctypes.c_void_p()
            self._check(self.cu.cuModuleGetFunction(ctypes.byref(f), self.mod, name.encode()), name)
            self.fn[key] = f

    @staticmethod
    def _check(rc, what):
        if rc != 0:
            raise RuntimeError(f"{what}: CUDA driver error {rc}")

    def launch(self, diff_flag: int, single: bool, channel: int, d_vertices: int, d_config: int, d_dst: int,
               n_pixels: int, stream: int = 0) -> None:
        """One reference launch: dst[pixel] += the channel's field."""
        ch = ctypes.c_uint(channel)
        v, c, d = ctypes.c_void_p(d_vertices), ctypes.c_void_p(d_config), ctypes.c_void_p(d_dst)
        args = (ctypes.c_void_p * 4)(ctypes.cast(ctypes.byref(ch), ctypes.c_void_p),
                                     ctypes.cast(ctypes.byref(v), ctypes.c_void_p),
                                     ctypes.cast(ctypes.byref(c), ctypes.c_void_p),
                                     ctypes.cast(ctypes.byref(d), ctypes.c_void_p))
        grid = (n_pixels + BLOCK - 1) // BLOCK
        self._check(self.cu.cuLaunchKernel(self.fn[(diff_flag, single)], grid, 1, 1, BLOCK, 1, 1, 0,
                                           ctypes.c_void_p(stream), args, None), "cuLaunchKernel")

    def generate(self, geom: dict, vertices: np.ndarray, diff_flag: int, single: bool = False,
                 chunk_points: int = 0):
        """The reference driver's single-GPU loop on one device buffer per
        channel; returns complex128 [n_channels, pnY, pnX]. With
        chunk_points > 0 each channel runs as launches over consecutive
        ranges of that many points accumulating into the same buffer (what
        the reference's multi-GPU driver does per device,
        ophgen/src/ophPointCloud_GPU.cpp:287-410), so that no launch runs
        for more than a few seconds."""
        import torch
        pnx, pny = geom["pnx"], geom["pny"]
        n = vertices.shape[0]
        step = chunk_points if chunk_points > 0 else max(n, 1)
        d_v = torch.from_numpy(np.ascontiguousarray(vertices, dtype=np.float64)).cuda()
        d_dst = torch.zeros((pny * pnx, 2), dtype=torch.float64, device="cuda")
        out = []
        stream = torch.cuda.current_stream().cuda_stream
        for ch, lam in enumerate(geom["wavelengths"]):
            for p0 in range(0, n, step):
                m = min(step, n - p0)
                cfg = make_config(pnx, pny, geom["ppx"], geom["ppy"], lam, m, diff_flag,
                                  geom.get("scale", (1.0, 1.0, 1.0)), geom.get("distance", 0.0))
                d_cfg = torch.frombuffer(bytearray(bytes(cfg)), dtype=torch.uint8).cuda()
                self.launch(diff_flag, single, ch, d_v.data_ptr() + p0 * 56, d_cfg.data_ptr(), d_dst.data_ptr(),
                            pnx * pny, stream)
                torch.cuda.synchronize()
            h = d_dst.cpu().numpy()
            out.append((h[:, 0] + 1j * h[:, 1]).reshape(pny, pnx))
            d_dst.zero_()
        return np.stack(out)

    def close(self) -> None:
        if self.mod:
            self.cu.cuModuleUnload(self.mod)
            self.mod = ctypes.c_void_p()


def time_kernels(workload: str, n_points: int, steps: int = 2) -> dict:
    """Times each reference kernel (FP64 and FP32; RS and Fresnel) over all
    channels of the workload on its first `n_points` points with CUDA events,
    and reports interactions/s at full resolution (cost is linear in points)."""
    import torch

    from openholo_gb300 import workloads
    w = workloads.BY_NAME[workload]()
    sub = w.subset(n_points)
    k = RefGpuKernels()
    pnx, pny = w.pnx, w.pny
    d_v = torch.from_numpy(np.ascontiguousarray(sub.vertices)).cuda()
    d_dst = torch.zeros((pny * pnx, 2), dtype=torch.float64, device="cuda")
    s = torch.cuda.current_stream()
    out = {"workload": workload, "points_sampled": n_points, "of_points": w.n_points, "pnx": pnx, "pny": pny,
           "channels": w.n_channels, "block": BLOCK, "kernels": {}}
    for diff in (0, 1):
        for single in (False, True):
            cfgs = []
            for ch, lam in enumerate(w.wavelengths):
                c = make_config(pnx, pny, w.pp, w.pp, lam, n_points, diff, w.scale, w.distance)
                cfgs.append(torch.frombuffer(bytearray(bytes(c)), dtype=torch.uint8).cuda())

            def run():
                for ch in range(w.n_channels):
                    k.launch(diff, single, ch, d_v.data_ptr(), cfgs[ch].data_ptr(), d_dst.data_ptr(), pnx * pny,
                             s.cuda_stream)

            run()                       # warm-up
            torch.cuda.synchronize()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(s)
            for _ in range(steps):
                run()
            b.record(s)
            torch.cuda.synchronize()
            secs = a.elapsed_time(b) / 1e3 / steps
            inter = n_points * pnx * pny * w.n_channels
            name = ("RS" if diff == 0 else "Fresnel") + ("_fp32" if single else "_fp64")
            out["kernels"][name] = {"interactions_per_s": inter / secs, "ms_per_generate_sample": secs * 1e3,
                                    "ms_per_generate_full_extrapolated": secs * 1e3 * w.n_points / n_points}
    # accuracy of each variant against the FP64 kernel on a smaller sample
    # (50 points at full resolution)
    acc = w.subset(min(50, n_points))
    g = w.geometry_kwargs()
    for diff in (0, 1):
        f64 = k.generate(g, acc.vertices, diff, single=False)
        f32 = k.generate(g, acc.vertices, diff, single=True)
        name = "RS" if diff == 0 else "Fresnel"
        out["kernels"][name + "_fp32"]["relL2_vs_fp64_kernel"] = float(np.linalg.norm(f32 - f64) /
                                                                        np.linalg.norm(f64))
    k.close()
    return out


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="sphere_fhd")
    ap.add_argument("--points", type=int, default=1000)
    ap.add_argument("--steps", type=int, default=2)
    a = ap.parse_args()
    print(json.dumps(time_kernels(a.workload, a.points, a.steps)))


if __name__ == "__main__":
    main()
