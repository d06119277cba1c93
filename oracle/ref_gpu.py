"""The reference's own projector kernels on the GPU (TEST INFRASTRUCTURE).

oracle/build_ref.sh compiles CudaPerformProjection (Projector.cu:227-372)
and CudaPerformBackProjection (Projector.cu:376-785) from the reference
tree into two cubins in oracle/_ref/: one with nvcc's defaults, as the
reference ships them, and one with -fmad=false.  This module loads a cubin
through the CUDA driver API (ctypes on libcuda) into the context PyTorch
made current and launches the kernels exactly as Projector::PerformProjection
and ::PerformBackProjection do (Projector.cu:917-954, 1082-1125): blocks of
32 x 16 threads, per-view float3 detector origins and sources, the volume
origin (unused by the kernels) and the spacings by value.

It is a checker for the engine's RC kernels and the "reference GPU" timing
line, never part of the product path.

Safety.  FindProjectionAlphas_d returns no value for a ray that misses the
volume (Projector.cu:79-85); the count the forward kernel then loops over is
undefined and its local-memory reads could leave the thread's frame.
forward() therefore refuses a geometry unless every ray crosses both the
bottom and the top face of the volume at least one voxel inside its lateral
faces (all_rays_cross_volume, checked in double on the host), and unless
every ray's crossing list stays below the kernel's 2000-entry array
(Projector.cu:128-132).  The backprojector clamps its pixel window to the
detector (Projector.cu:609-645) and needs no such check.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
CUBINS = {"fma": os.path.join(HERE, "_ref", "ref_kernels.cubin"),
          "nofma": os.path.join(HERE, "_ref", "ref_kernels_nofma.cubin")}


def available(variant="fma"):
    return os.path.exists(CUBINS[variant])


class _Dim3(C.Structure):
    _fields_ = [("x", C.c_uint), ("y", C.c_uint), ("z", C.c_uint)]


class _F3(C.Structure):
    _fields_ = [("x", C.c_float), ("y", C.c_float), ("z", C.c_float)]


class _F2(C.Structure):
    _fields_ = [("x", C.c_float), ("y", C.c_float)]


_cuda = None
_modules = {}


def _drv():
    global _cuda
    if _cuda is None:
        _cuda = C.CDLL("libcuda.so.1")
        for name in ("cuInit", "cuCtxGetCurrent", "cuModuleLoad", "cuModuleGetFunction", "cuLaunchKernel"):
            getattr(_cuda, name).restype = C.c_int
    return _cuda


def _check(rc, what):
    if rc != 0:
        raise RuntimeError(f"{what} failed with CUDA driver error {rc}")


def _functions(variant):
    if variant in _modules:
        return _modules[variant]
    import torch
    torch.zeros(1, device="cuda")          # makes torch's primary context current
    d = _drv()
    _check(d.cuInit(0), "cuInit")
    ctx = C.c_void_p()
    _check(d.cuCtxGetCurrent(C.byref(ctx)), "cuCtxGetCurrent")
    if not ctx.value:
        raise RuntimeError("no current CUDA context")
    mod = C.c_void_p()
    _check(d.cuModuleLoad(C.byref(mod), CUBINS[variant].encode()), "cuModuleLoad")
    fns = {}
    for name in ("CudaPerformProjection", "CudaPerformBackProjection"):
        f = C.c_void_p()
        _check(d.cuModuleGetFunction(C.byref(f), mod, name.encode()), f"cuModuleGetFunction({name})")
        fns[name] = f
    _modules[variant] = (mod, fns)
    return _modules[variant]


def all_rays_cross_volume(g, views=None, margin_voxels=1.0, max_list=1900):
    """True when every ray of the given views enters the volume through its
    bottom face and leaves through its top face at least `margin_voxels`
    inside the lateral faces, and every ray's crossing list (x + y + z plane
    spans + 3, Projector.cu:124-127) stays below `max_list`.  Positions on a
    horizontal plane are affine in the pixel indices, so the four corner rays
    bound the rest."""
    src = np.asarray(g.src, np.float64).reshape(-1, 3)
    org = np.asarray(g.det_origin, np.float64).reshape(-1, 3)
    views = range(g.n_views) if views is None else views
    hx, hy, hz = g.nx * g.dx / 2, g.ny * g.dy / 2, g.nz * g.dz / 2
    for p in views:
        s = src[p]
        corners = [(u, v) for u in (0, g.nu - 1) for v in (0, g.nv - 1)]
        for u, v in corners:
            q = np.array([org[p, 0] + (u + 0.5) * g.du, org[p, 1] + (v + 0.5) * g.dv, org[p, 2]])
            d = q - s
            span = 3
            xs, ys = [], []
            for z in (-hz, hz):
                a = (z - s[2]) / d[2]
                if not (0.0 < a < 1.0):
                    return False
                x, y = s[0] + a * d[0], s[1] + a * d[1]
                if abs(x) > hx - margin_voxels * g.dx or abs(y) > hy - margin_voxels * g.dy:
                    return False
                xs.append(x / g.dx)
                ys.append(y / g.dy)
            span += abs(xs[1] - xs[0]) + abs(ys[1] - ys[0]) + g.nz + 2
            if span >= max_list:
                return False
    return True


def _views(g):
    src = np.ascontiguousarray(np.asarray(g.src, np.float32).reshape(-1, 3))
    org = np.ascontiguousarray(np.asarray(g.det_origin, np.float32).reshape(-1, 3))
    return src, org


def _launch(variant, name, in_t, out_t, g, grid, stream):
    import torch
    _, fns = _functions(variant)
    src, org = _views(g)
    d_src = torch.from_numpy(src).cuda()
    d_org = torch.from_numpy(org).cuda()
    args = [C.c_void_p(in_t.data_ptr()), _Dim3(g.nx, g.ny, g.nz), _F3(0.0, 0.0, 0.0),
            _F3(g.dx, g.dy, g.dz), C.c_void_p(out_t.data_ptr()), _Dim3(g.nu, g.nv, g.n_views),
            _F2(g.du, g.dv), C.c_void_p(d_org.data_ptr()), C.c_void_p(d_src.data_ptr())]
    params = (C.c_void_p * len(args))(*[C.cast(C.pointer(a), C.c_void_p) for a in args])
    if stream is None:
        stream = torch.cuda.current_stream().cuda_stream
    _check(_drv().cuLaunchKernel(fns[name], C.c_uint(grid[0]), C.c_uint(grid[1]), C.c_uint(grid[2]),
                                 C.c_uint(32), C.c_uint(16), C.c_uint(1), C.c_uint(0),
                                 C.c_void_p(stream), params, None), f"cuLaunchKernel({name})")
    return d_src, d_org           # keep alive until the caller synchronises


def forward(g, vol, out=None, variant="fma", stream=None):
    """CudaPerformProjection over the whole geometry: vol is a CUDA float32
    tensor [nz][ny][nx]; returns [P][nv][nu] (a mean along each ray)."""
    import torch
    if not all_rays_cross_volume(g):
        raise ValueError("reference forward kernel: some ray misses the volume or its "
                         "crossing list could exceed the kernel's array; refused")
    if out is None:
        out = torch.empty((g.n_views, g.nv, g.nu), dtype=torch.float32, device=vol.device)
    grid = (-(-g.nu // 32), -(-g.nv // 16), g.n_views)
    keep = _launch(variant, "CudaPerformProjection", vol, out, g, grid, stream)
    torch.cuda.synchronize()
    del keep
    return out


def back(g, proj, out=None, variant="fma", stream=None):
    """CudaPerformBackProjection over the whole volume: the reference's
    windowed, normalised backprojection (Projector.cu:376-785)."""
    import torch
    if out is None:
        out = torch.empty((g.nz, g.ny, g.nx), dtype=torch.float32, device=proj.device)
    grid = (-(-g.nx // 32), -(-g.ny // 16), g.nz)
    keep = _launch(variant, "CudaPerformBackProjection", proj, out, g, grid, stream)
    torch.cuda.synchronize()
    del keep
    return out
