"""ctypes binding of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Wraps liboracle.so (kvtomo_oracle.c: the RC restatement in FP32, the FP64
Siddon EXACT operators, the drivers, shift-and-add, the phantom rasteriser)
and, when it was built in this checkout, oracle/_ref/libkvref.so (the
reference's own kernels compiled for the host).  Only tests/, the smoke test
and bench.py's CPU legs use it.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_i64p = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")


class CGeom(C.Structure):
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32),
                ("dx", C.c_float), ("dy", C.c_float), ("dz", C.c_float),
                ("n_views", C.c_int32), ("nu", C.c_int32), ("nv", C.c_int32),
                ("du", C.c_float), ("dv", C.c_float),
                ("src", C.POINTER(C.c_float)), ("det_origin", C.POINTER(C.c_float)),
                ("fulcrum_z", C.c_float)]


def cgeom(g):
    """C struct for a kevernals_gb300.geometry.Geometry (keeps the arrays alive)."""
    src = np.ascontiguousarray(g.src, np.float32)
    det = np.ascontiguousarray(g.det_origin, np.float32)
    s = CGeom(g.nx, g.ny, g.nz, g.dx, g.dy, g.dz, src.shape[0], g.nu, g.nv, g.du, g.dv,
              src.ctypes.data_as(C.POINTER(C.c_float)), det.ctypes.data_as(C.POINTER(C.c_float)),
              g.fulcrum_z)
    s._keep = (src, det)
    return s


_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build_oracle()
        L = C.CDLL(path)
        G = C.POINTER(CGeom)
        sigs = {
            "kvo_rc_forward": [G, _f32p, _f32p],
            "kvo_rc_forward_rays": [G, _f32p, _i64p, C.c_int64, _f32p],
            "kvo_rc_back": [G, _f32p, _f32p],
            "kvo_rc_back_voxels": [G, _f32p, _i64p, C.c_int64, _f32p],
            "kvo_rc_mlem": [G, _f32p, _f32p, C.c_int, C.c_float],
            "kvo_rc_art": [G, _f32p, _f32p, C.c_int, C.c_float],
            "kvo_rc_ray_hits": [G, C.c_int, C.c_int, C.c_int],
            "kvo_saa_shifts": [G, C.c_int, _i32p],
            "kvo_saa": [G, _i32p, _f32p, _f32p],
            "kvo_exact_forward": [G, _f64p, _f64p],
            "kvo_exact_forward_rays": [G, _f64p, _i64p, C.c_int64, _f64p],
            "kvo_exact_back": [G, _f64p, _f64p],
            "kvo_exact_back_rays": [G, _f64p, _i64p, C.c_int64, _f64p],
            "kvo_rc_forward_rays_refcost": [G, _f32p, _i64p, C.c_int64, _f32p],
            "kvo_exact_ray_lengths": [G, _f64p],
            "kvo_exact_mlem": [G, _f64p, _f64p, C.c_int, C.c_double],
            "kvo_exact_sart": [G, _f64p, _f64p, C.c_int, C.c_double],
            "kvo_phantom": [C.c_int, C.c_int, C.c_int, C.c_float, C.c_float, C.c_float,
                            _f32p, C.c_int, _f32p],
            "kvo_rc_mlem_host_loops": [_f32p, _f32p, _i64p, C.c_int64, _f32p, _f32p, _i64p, C.c_int64,
                                       C.c_float],
            "kvo_num_threads": [],
            "kvo_set_threads": [C.c_int],
        }
        for name, args in sigs.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = C.c_int if name in ("kvo_rc_ray_hits", "kvo_saa_shifts",
                                             "kvo_num_threads") else None
        _lib = L
    return _lib


def ref_lib():
    """The reference kernels compiled for the host, or None when unavailable."""
    global _ref
    if _ref is None:
        path = _build.REF_SO if os.path.exists(_build.REF_SO) else _build.build_ref()
        if not path or not os.path.exists(path):
            return None
        L = C.CDLL(path)
        G = C.POINTER(CGeom)
        L.kvref_forward.argtypes = [G, _f32p, _f32p]
        L.kvref_back.argtypes = [G, _f32p, _f32p]
        L.kvref_forward.restype = None
        L.kvref_back.restype = None
        L.kvref_forward_rays.argtypes = [G, _f32p, _i64p, C.c_int64, _f32p]
        L.kvref_back_voxels.argtypes = [G, _f32p, _i64p, C.c_int64, _f32p]
        L.kvref_forward_rays.restype = None
        L.kvref_back_voxels.restype = None
        _ref = L
    return _ref


def _vol(g, x, dt):
    return np.ascontiguousarray(np.asarray(x, dt).reshape(g.volume_shape))


def _proj(g, p, dt):
    return np.ascontiguousarray(np.asarray(p, dt).reshape(g.proj_shape))


# ---- RC family (FP32 restatement of the reference) -------------------------

def rc_forward(g, vol):
    out = np.empty(g.proj_shape, np.float32)
    lib().kvo_rc_forward(C.byref(cgeom(g)), _vol(g, vol, np.float32), out)
    return out


def rc_back(g, proj):
    out = np.empty(g.volume_shape, np.float32)
    lib().kvo_rc_back(C.byref(cgeom(g)), _proj(g, proj, np.float32), out)
    return out


def rc_forward_rays(g, vol, rays):
    rays = np.ascontiguousarray(rays, np.int64)
    out = np.empty(rays.shape[0], np.float32)
    lib().kvo_rc_forward_rays(C.byref(cgeom(g)), _vol(g, vol, np.float32), rays, rays.shape[0], out)
    return out


def rc_forward_rays_refcost(g, vol, rays):
    """RC forward of sampled rays with the reference's selection sort."""
    rays = np.ascontiguousarray(rays, np.int64)
    out = np.empty(rays.shape[0], np.float32)
    lib().kvo_rc_forward_rays_refcost(C.byref(cgeom(g)), _vol(g, vol, np.float32), rays,
                                      rays.shape[0], out)
    return out


def exact_back_rays(g, values, rays, vol):
    """Adds the transpose of the sampled rays into vol (float64, in place)."""
    rays = np.ascontiguousarray(rays, np.int64)
    values = np.ascontiguousarray(values, np.float64)
    assert vol.dtype == np.float64 and vol.flags.c_contiguous and vol.size == g.n_voxels
    lib().kvo_exact_back_rays(C.byref(cgeom(g)), values, rays, rays.shape[0], vol)
    return vol


def rc_back_voxels(g, proj, voxels):
    voxels = np.ascontiguousarray(voxels, np.int64)
    out = np.empty(voxels.shape[0], np.float32)
    lib().kvo_rc_back_voxels(C.byref(cgeom(g)), _proj(g, proj, np.float32), voxels,
                             voxels.shape[0], out)
    return out


def rc_mlem(g, p, x0, iters, relax):
    x = _vol(g, x0, np.float32).copy()
    lib().kvo_rc_mlem(C.byref(cgeom(g)), _proj(g, p, np.float32), x, iters, relax)
    return x


def rc_art(g, p, x0, iters, relax):
    x = _vol(g, x0, np.float32).copy()
    lib().kvo_rc_art(C.byref(cgeom(g)), _proj(g, p, np.float32), x, iters, relax)
    return x


def saa_shifts(g, rule):
    out = np.empty((g.nz, g.n_views), np.int32)
    rc = lib().kvo_saa_shifts(C.byref(cgeom(g)), int(rule), out)
    if rc != 0:
        raise ValueError("shift-and-add geometry rejected")
    return out


def saa(g, proj, rule):
    sh = saa_shifts(g, rule)
    out = np.empty((g.nz, g.nv, g.nu), np.float32)
    lib().kvo_saa(C.byref(cgeom(g)), sh, _proj(g, proj, np.float32), out)
    return out


# ---- EXACT family (FP64 Siddon) -------------------------------------------

def exact_forward(g, vol):
    out = np.empty(g.proj_shape, np.float64)
    lib().kvo_exact_forward(C.byref(cgeom(g)), _vol(g, vol, np.float64), out)
    return out


def exact_forward_rays(g, vol, rays):
    rays = np.ascontiguousarray(rays, np.int64)
    out = np.empty(rays.shape[0], np.float64)
    lib().kvo_exact_forward_rays(C.byref(cgeom(g)), _vol(g, vol, np.float64), rays,
                                 rays.shape[0], out)
    return out


def exact_back(g, proj):
    out = np.empty(g.volume_shape, np.float64)
    lib().kvo_exact_back(C.byref(cgeom(g)), _proj(g, proj, np.float64), out)
    return out


def exact_ray_lengths(g):
    out = np.empty(g.proj_shape, np.float64)
    lib().kvo_exact_ray_lengths(C.byref(cgeom(g)), out)
    return out


def exact_mlem(g, p, x0, iters, relax=1.0):
    x = _vol(g, x0, np.float64).copy()
    lib().kvo_exact_mlem(C.byref(cgeom(g)), _proj(g, p, np.float64), x, iters, relax)
    return x


def exact_sart(g, p, x0, iters, relax):
    x = _vol(g, x0, np.float64).copy()
    lib().kvo_exact_sart(C.byref(cgeom(g)), _proj(g, p, np.float64), x, iters, relax)
    return x


def phantom(g, params):
    params = np.ascontiguousarray(params, np.float32)
    out = np.empty(g.volume_shape, np.float32)
    lib().kvo_phantom(g.nx, g.ny, g.nz, g.dx, g.dy, g.dz, params, params.shape[0], out)
    return out


def num_threads():
    return lib().kvo_num_threads()


def set_threads(n):
    lib().kvo_set_threads(int(n))


# ---- the reference kernels compiled for the host ---------------------------

def ref_forward(g, vol):
    L = ref_lib()
    if L is None:
        raise RuntimeError("reference kernels not built (reference tree absent)")
    out = np.empty(g.proj_shape, np.float32)
    L.kvref_forward(C.byref(cgeom(g)), _vol(g, vol, np.float32), out)
    return out


def ref_back(g, proj):
    L = ref_lib()
    if L is None:
        raise RuntimeError("reference kernels not built (reference tree absent)")
    out = np.empty(g.volume_shape, np.float32)
    L.kvref_back(C.byref(cgeom(g)), _proj(g, proj, np.float32), out)
    return out


def ref_forward_rays(g, vol, rays, proj):
    """The reference's forward kernel on sampled rays, written into the
    full projection stack `proj` (float32, in place)."""
    L = ref_lib()
    if L is None:
        raise RuntimeError("reference kernels not built (reference tree absent)")
    rays = np.ascontiguousarray(rays, np.int64)
    assert proj.dtype == np.float32 and proj.flags.c_contiguous and proj.size == g.n_rays
    L.kvref_forward_rays(C.byref(cgeom(g)), _vol(g, vol, np.float32), rays, rays.shape[0], proj)
    return proj


def ref_back_voxels(g, proj, voxels, vol):
    """The reference's backprojection kernel on sampled voxels, written into
    the full volume `vol` (float32, in place)."""
    L = ref_lib()
    if L is None:
        raise RuntimeError("reference kernels not built (reference tree absent)")
    voxels = np.ascontiguousarray(voxels, np.int64)
    assert vol.dtype == np.float32 and vol.flags.c_contiguous and vol.size == g.n_voxels
    L.kvref_back_voxels(C.byref(cgeom(g)), _proj(g, proj, np.float32), voxels, voxels.shape[0], vol)
    return vol


def rc_mlem_host_loops(p, q, rays, x, b, voxels, relax):
    """The reference MLEM iteration's serial host loops on sampled indices
    (ratio over rays, multiplicative update over voxels), in place."""
    for a in (p, q, x, b):
        assert a.dtype == np.float32 and a.flags.c_contiguous
    rays = np.ascontiguousarray(rays, np.int64)
    voxels = np.ascontiguousarray(voxels, np.int64)
    lib().kvo_rc_mlem_host_loops(p.reshape(-1), q.reshape(-1), rays, rays.shape[0], x.reshape(-1),
                                 b.reshape(-1), voxels, voxels.shape[0], float(relax))


def ramp_taps(half_taps):
    """Shepp-Logan ramp kernel in pixel units, h[n] = -2 / (pi^2 (4n^2 - 1)),
    n = 0..half_taps (L. A. Shepp, B. F. Logan, IEEE Trans. Nucl. Sci. 21, 1974)."""
    n = np.arange(half_taps + 1, dtype=np.float64)
    return -2.0 / (np.pi ** 2 * (4.0 * n * n - 1.0))


def ramp_filter_v(proj, half_taps):
    """FP64 filtering of every detector column along v with the truncated
    Shepp-Logan kernel, zero outside the detector ([P][nv][nu] layout)."""
    p = np.asarray(proj, np.float64)
    h = ramp_taps(half_taps)
    out = h[0] * p
    nv = p.shape[1]
    for k in range(1, min(half_taps, nv - 1) + 1):
        out[:, k:, :] += h[k] * p[:, :-k, :]
        out[:, :-k, :] += h[k] * p[:, k:, :]
    return out


def exact_fbp(g, proj, half_taps):
    """A^T(h * p) / A^T 1 (0 where A^T 1 = 0), the engine's kv_fbp, in FP64."""
    b = exact_back(g, ramp_filter_v(proj, half_taps))
    s = exact_back(g, np.ones(g.proj_shape))
    return np.where(s > 0, b / np.where(s > 0, s, 1.0), 0.0)
