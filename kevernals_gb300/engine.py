"""Python host API over the C ABI: contexts and plans.

A Plan holds one geometry, an operator family ("rc": the reference's own
operators; "exact": Siddon A and its exact transpose) and a storage type.
Buffers may be numpy arrays (host memory: the library copies in and out) or
CUDA torch tensors (device memory: used in place, ordered on the current
torch stream).
"""
from __future__ import annotations

import atexit
import ctypes as C
import sys
import weakref

import numpy as np

from . import _lib
from ._lib import KvError, KvGeometry, lib

try:  # torch is optional: only needed for device-resident buffers
    import torch
except Exception:  # pragma: no cover
    torch = None


_LIVE = weakref.WeakSet()


@atexit.register
def _close_all():
    """Destroys every live plan, then every context, before interpreter
    teardown (a plan must not outlive the CUDA runtime)."""
    objs = list(_LIVE)
    for o in objs:
        if isinstance(o, Plan):
            o.close()
    for o in objs:
        o.close()


def _is_cuda_tensor(x):
    return torch is not None and isinstance(x, torch.Tensor) and x.is_cuda


class Context:
    """A device plus a stream (kv_ctx)."""

    def __init__(self, device: int = 0):
        h = C.c_void_p()
        s = lib().kv_ctx_create(device, C.byref(h))
        if s != _lib.KV_OK:
            raise KvError(s, lib().kv_status_string(s).decode())
        self._h = h
        self.device = device
        _LIVE.add(self)

    @property
    def handle(self):
        return self._h

    def last_error(self) -> str:
        return lib().kv_ctx_last_error(self._h).decode()

    def check(self, status):
        if status != _lib.KV_OK:
            raise KvError(status, self.last_error())

    def set_stream(self, stream_handle):
        self.check(lib().kv_ctx_set_stream(self._h, C.c_void_p(stream_handle or 0)))

    def use_torch_stream(self):
        if torch is not None and torch.cuda.is_available():
            self.set_stream(torch.cuda.current_stream(self.device).cuda_stream)

    def sync(self):
        self.check(lib().kv_sync(self._h))

    def set_timing(self, enable: bool):
        """Brackets every kernel launch with CUDA events (tracing)."""
        self.check(lib().kv_ctx_set_timing(self._h, int(bool(enable))))

    def read_timing(self):
        """{kernel name: (launches, total device ms)} since the last read."""
        buf = C.create_string_buffer(1 << 16)
        self.check(lib().kv_ctx_timing_read(self._h, buf, len(buf)))
        out = {}
        for line in buf.value.decode().splitlines():
            name, n, ms = line.split()
            out[name] = (int(n), float(ms))
        return out

    def close(self):
        if getattr(self, "_h", None):
            lib().kv_ctx_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
        return False

    def __del__(self):
        if sys.is_finalizing():
            return
        try:
            self.close()
        except Exception:
            pass


def make_cgeom(g):
    src = np.ascontiguousarray(g.src, np.float32)
    det = np.ascontiguousarray(g.det_origin, np.float32)
    cg = KvGeometry(g.nx, g.ny, g.nz, g.dx, g.dy, g.dz, src.shape[0], g.nu, g.nv, g.du, g.dv,
                    src.ctypes.data_as(C.POINTER(C.c_float)),
                    det.ctypes.data_as(C.POINTER(C.c_float)), g.fulcrum_z)
    cg._keep = (src, det)
    return cg


class Plan:
    """kv_plan: geometry + operator family + storage type."""

    def __init__(self, ctx: Context, geometry, family: str = "exact", storage: str = "f32"):
        self.ctx = ctx
        self.geometry = geometry
        self.family = family
        self.storage = storage
        h = C.c_void_p()
        cg = make_cgeom(geometry)
        s = lib().kv_plan_create(ctx.handle, C.byref(cg), _lib.FAMILY[family],
                                 _lib.STORAGE[storage], C.byref(h))
        ctx.check(s)
        self._h = h
        _LIVE.add(self)

    @property
    def handle(self):
        return self._h

    def close(self):
        if getattr(self, "_h", None):
            lib().kv_plan_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
        return False

    def __del__(self):
        if sys.is_finalizing():
            return
        try:
            self.close()
        except Exception:
            pass

    # -- buffer helpers --------------------------------------------------
    def _buf(self, x, shape, dtype=np.float32, out=False):
        """Returns (pointer, mem flag, keep-alive)."""
        if _is_cuda_tensor(x):
            want = {np.float32: torch.float32, np.float64: torch.float64}[dtype]
            if x.dtype != want or not x.is_contiguous() or x.numel() != int(np.prod(shape)):
                raise ValueError(f"device buffer must be contiguous {want} with {np.prod(shape)} elements")
            self.ctx.use_torch_stream()
            return C.c_void_p(x.data_ptr()), _lib.MEM_DEVICE, x
        a = np.asarray(x)
        if out:
            if a.dtype != dtype or not a.flags.c_contiguous or a.size != int(np.prod(shape)):
                raise ValueError("output array has the wrong dtype / size / layout")
        else:
            a = np.ascontiguousarray(a, dtype)
            if a.size != int(np.prod(shape)):
                raise ValueError(f"expected {int(np.prod(shape))} elements, got {a.size}")
        return C.c_void_p(a.ctypes.data), _lib.MEM_HOST, a

    def _like(self, x, shape, dtype=np.float32):
        if _is_cuda_tensor(x):
            return torch.empty(shape, dtype={np.float32: torch.float32, np.float64: torch.float64}[dtype],
                               device=x.device)
        return np.empty(shape, dtype)

    # -- operators -------------------------------------------------------
    def forward(self, volume, out=None):
        g = self.geometry
        out = self._like(volume, g.proj_shape) if out is None else out
        pv, mv, kv = self._buf(volume, g.volume_shape)
        po, mo, ko = self._buf(out, g.proj_shape, out=True)
        if mv != mo:
            raise ValueError("input and output must both be host or both be device buffers")
        self.ctx.check(lib().kv_forward(self._h, pv, po, mv))
        return out

    def forward_single(self, volume, src, det_origin, out=None):
        g = self.geometry
        shape = (g.nv, g.nu)
        out = self._like(volume, shape) if out is None else out
        pv, mv, kv = self._buf(volume, g.volume_shape)
        po, mo, ko = self._buf(out, shape, out=True)
        s = (C.c_float * 3)(*[float(t) for t in src])
        d = (C.c_float * 3)(*[float(t) for t in det_origin])
        self.ctx.check(lib().kv_forward_single(self._h, pv, C.cast(s, C.c_void_p),
                                               C.cast(d, C.c_void_p), po, mv))
        return out

    def back(self, proj, out=None):
        g = self.geometry
        out = self._like(proj, g.volume_shape) if out is None else out
        pp, mp, kp = self._buf(proj, g.proj_shape)
        po, mo, ko = self._buf(out, g.volume_shape, out=True)
        self.ctx.check(lib().kv_back(self._h, pp, po, mp))
        return out

    def fbp(self, proj, half_taps=128, out=None):
        """Filtered backprojection: A^T(h * p) / A^T 1 with the Shepp-Logan
        ramp along v truncated at |n| <= half_taps (kv_fbp)."""
        g = self.geometry
        out = self._like(proj, g.volume_shape) if out is None else out
        pp, mp, kp = self._buf(proj, g.proj_shape)
        po, mo, ko = self._buf(out, g.volume_shape, out=True)
        if mp != mo:
            raise ValueError("input and output must both be host or both be device buffers")
        self.ctx.check(lib().kv_fbp(self._h, pp, po, int(half_taps), mp))
        return out

    def sensitivity(self, out=None, device=False):
        g = self.geometry
        if out is None:
            out = (torch.empty(g.volume_shape, dtype=torch.float64, device=f"cuda:{self.ctx.device}")
                   if device else np.empty(g.volume_shape, np.float64))
        po, mo, ko = self._buf(out, g.volume_shape, np.float64, out=True)
        self.ctx.check(lib().kv_sensitivity(self._h, po, mo))
        return out

    def shift_and_add(self, proj, out=None):
        g = self.geometry
        shape = (g.nz, g.nv, g.nu)
        out = self._like(proj, shape) if out is None else out
        pp, mp, kp = self._buf(proj, g.proj_shape)
        po, mo, ko = self._buf(out, shape, out=True)
        self.ctx.check(lib().kv_shift_and_add(self._h, pp, po, mp))
        return out

    def uniform_volume(self, device=False):
        g = self.geometry
        out = (torch.empty(g.volume_shape, dtype=torch.float32, device=f"cuda:{self.ctx.device}")
               if device else np.empty(g.volume_shape, np.float32))
        po, mo, ko = self._buf(out, g.volume_shape, out=True)
        self.ctx.check(lib().kv_uniform_volume(self._h, po, mo))
        return out

    def _iterate(self, fn, proj, volume, iterations, relax, callback):
        g = self.geometry
        pp, mp, kp = self._buf(proj, g.proj_shape)
        if not _is_cuda_tensor(volume):
            if not (isinstance(volume, np.ndarray) and volume.dtype == np.float32
                    and volume.flags.c_contiguous):
                raise ValueError("the iterate must be a C-contiguous float32 array (updated in place)")
        px, mx, kx = self._buf(volume, g.volume_shape, out=True)
        if mp != mx:
            raise ValueError("projections and volume must both be host or both be device buffers")
        history = []

        def _cb(it, res, ll, user):
            history.append((it, res, ll))
            return int(bool(callback(it, res, ll))) if callback else 0
        cb = _lib.ITER_CB(_cb) if callback is not None else _lib.ITER_CB()
        self.ctx.check(fn(self._h, pp, px, int(iterations), float(relax), mp, cb, None))
        return history

    def mlem(self, proj, volume, iterations, relax=1.0, callback=None):
        """In-place MLEM on `volume`; returns the (iteration, residual, loglik)
        history when a callback is given."""
        return self._iterate(lib().kv_mlem, proj, volume, iterations, relax, callback)

    def sart(self, proj, volume, iterations, relax=0.5, callback=None):
        return self._iterate(lib().kv_sart, proj, volume, iterations, relax, callback)

    def residual(self, proj, volume):
        g = self.geometry
        pp, mp, kp = self._buf(proj, g.proj_shape)
        px, mx, kx = self._buf(volume, g.volume_shape)
        r, ll = C.c_double(), C.c_double()
        self.ctx.check(lib().kv_residual(self._h, pp, px, mp, C.byref(r), C.byref(ll)))
        return r.value, ll.value


def shift_and_add_shifts(geometry, family: str = "exact") -> np.ndarray:
    """Row shifts [nz, n_views] of shift-and-add, computed on the host."""
    out = np.empty((geometry.nz, geometry.n_views), np.int32)
    cg = make_cgeom(geometry)
    s = lib().kv_shift_and_add_shifts(C.byref(cg), _lib.FAMILY[family], C.c_void_p(out.ctypes.data))
    if s != _lib.KV_OK:
        raise KvError(s, "shift-and-add geometry rejected")
    return out


def phantom(ctx: Context, geometry, params, device=False):
    """Rasterises ellipsoid parameters (kevernals_gb300.phantom.ellipsoid_params)."""
    g = geometry
    params = np.ascontiguousarray(params, np.float32)
    if device:
        out = torch.empty(g.volume_shape, dtype=torch.float32, device=f"cuda:{ctx.device}")
        ctx.use_torch_stream()
        prm = torch.from_numpy(params).to(out.device)
        ctx.check(lib().kv_phantom_ellipsoids(ctx.handle, g.nx, g.ny, g.nz, g.dx, g.dy, g.dz,
                                              C.c_void_p(prm.data_ptr()), params.shape[0],
                                              C.c_void_p(out.data_ptr()), _lib.MEM_DEVICE))
        return out
    out = np.empty(g.volume_shape, np.float32)
    ctx.check(lib().kv_phantom_ellipsoids(ctx.handle, g.nx, g.ny, g.nz, g.dx, g.dy, g.dz,
                                          C.c_void_p(params.ctypes.data), params.shape[0],
                                          C.c_void_p(out.ctypes.data), _lib.MEM_HOST))
    return out


def _plan_autotune(self):
    """Chooses the forward ray-bundle and backprojector tile shapes by timing."""
    self.ctx.check(lib().kv_plan_autotune(self._h))
    return self.tuning


def _plan_tuning(self):
    f, b = C.c_int(), C.c_int()
    self.ctx.check(lib().kv_plan_get_tuning(self._h, C.byref(f), C.byref(b)))
    return f.value, b.value


def _plan_set_tuning(self, fwd_rows, back_rows):
    self.ctx.check(lib().kv_plan_set_tuning(self._h, int(fwd_rows), int(back_rows)))


def _plan_slab(self):
    """(rays per thread, slices per slab, stages, view group) of the slab
    forward projector; rays per thread 0: the one-thread-per-ray kernel."""
    v = [C.c_int() for _ in range(4)]
    self.ctx.check(lib().kv_plan_get_slab(self._h, *(C.byref(x) for x in v)))
    return tuple(x.value for x in v)


def _plan_set_slab(self, rays_per_thread, slices=4, stages=3, view_group=16):
    self.ctx.check(lib().kv_plan_set_slab(self._h, int(rays_per_thread), int(slices), int(stages),
                                          int(view_group)))


def _plan_back_shape(self):
    """(voxel rows, slices) per thread of the gather backprojector (rows 0:
    one voxel per thread)."""
    r, z = C.c_int(), C.c_int()
    self.ctx.check(lib().kv_plan_get_back_shape(self._h, C.byref(r), C.byref(z)))
    return r.value, z.value


def _plan_set_back_shape(self, rows_per_thread, slices_per_thread=1):
    self.ctx.check(lib().kv_plan_set_back_shape(self._h, int(rows_per_thread), int(slices_per_thread)))


def _plan_back_staging(self):
    """(voxel rows per thread, stages, patch columns, patch rows) of the
    TMA-staged backprojector; rows 0: not used."""
    v = [C.c_int() for _ in range(4)]
    self.ctx.check(lib().kv_plan_get_back_staging(self._h, *[C.byref(x) for x in v]))
    return tuple(x.value for x in v)


def _plan_set_back_staging(self, rows_per_thread, stages=2):
    self.ctx.check(lib().kv_plan_set_back_staging(self._h, int(rows_per_thread), int(stages)))


Plan.back_shape = property(_plan_back_shape)
Plan.set_back_shape = _plan_set_back_shape
Plan.back_staging = property(_plan_back_staging)
Plan.set_back_staging = _plan_set_back_staging
Plan.slab = property(_plan_slab)
Plan.set_slab = _plan_set_slab
Plan.autotune = _plan_autotune
Plan.tuning = property(_plan_tuning)
Plan.set_tuning = _plan_set_tuning


def batch_mlem(ctx: Context, plans, projections, volumes, iterations, relax=1.0):
    """MLEM on many EXACT plans at once (kv_batch_mlem); volumes updated in place.
    Buffers are all numpy (host) or all CUDA tensors (device)."""
    n = len(plans)
    if not (len(projections) == len(volumes) == n) or n == 0:
        raise ValueError("one projection stack and one volume per plan")
    keep, pp, pv, mem = [], [], [], None
    for plan, p, x in zip(plans, projections, volumes):
        a, m1, k1 = plan._buf(p, plan.geometry.proj_shape)
        if not _is_cuda_tensor(x) and not (isinstance(x, np.ndarray) and x.dtype == np.float32
                                           and x.flags.c_contiguous):
            raise ValueError("volumes must be C-contiguous float32 (updated in place)")
        b, m2, k2 = plan._buf(x, plan.geometry.volume_shape, out=True)
        if mem is None:
            mem = m1
        if m1 != mem or m2 != mem:
            raise ValueError("all buffers must be host or all device")
        keep += [k1, k2]
        pp.append(a.value)
        pv.append(b.value)
    hp = (C.c_void_p * n)(*[plan.handle.value for plan in plans])
    ap = (C.c_void_p * n)(*pp)
    av = (C.c_void_p * n)(*pv)
    ctx.check(lib().kv_batch_mlem(ctx.handle, n, hp, ap, av, int(iterations), float(relax), mem))


class UNet:
    """The learned warm start (kv_unet): y = x + f(x) on [D][H][W] volumes."""

    def __init__(self, ctx: Context, seed: int = 0):
        self.ctx = ctx
        h = C.c_void_p()
        ctx.check(lib().kv_unet_create(ctx.handle, C.c_uint64(seed), C.byref(h)))
        self._h = h
        _LIVE.add(self)

    @property
    def num_params(self) -> int:
        return int(lib().kv_unet_num_params(self._h))

    def close(self):
        if getattr(self, "_h", None):
            lib().kv_unet_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
        return False

    def __del__(self):
        if sys.is_finalizing():
            return
        try:
            self.close()
        except Exception:
            pass

    def _io(self, x, out=False):
        if _is_cuda_tensor(x):
            if x.dtype != torch.float32 or not x.is_contiguous():
                raise ValueError("device volumes must be contiguous float32")
            self.ctx.use_torch_stream()
            return C.c_void_p(x.data_ptr()), _lib.MEM_DEVICE, x
        a = x if out else np.ascontiguousarray(x, np.float32)
        if a.dtype != np.float32 or not a.flags.c_contiguous:
            raise ValueError("host volumes must be C-contiguous float32")
        return C.c_void_p(a.ctypes.data), _lib.MEM_HOST, a

    def forward(self, x, out=None):
        D, H, W = x.shape
        if out is None:
            out = torch.empty_like(x) if _is_cuda_tensor(x) else np.empty((D, H, W), np.float32)
        pi, m, k1 = self._io(x)
        po, m2, k2 = self._io(out, out=True)
        self.ctx.check(lib().kv_unet_forward(self._h, pi, po, D, H, W, m))
        return out

    def train_step(self, x, target, lr=1e-3):
        D, H, W = x.shape
        pi, m, k1 = self._io(x)
        pt, m2, k2 = self._io(target)
        loss = C.c_float()
        self.ctx.check(lib().kv_unet_train_step(self._h, pi, pt, D, H, W, float(lr), C.byref(loss), m))
        return loss.value

    def gradients(self, x, target):
        D, H, W = x.shape
        pi, m, k1 = self._io(x)
        pt, m2, k2 = self._io(target)
        g = np.empty(self.num_params, np.float32)
        loss = C.c_float()
        self.ctx.check(lib().kv_unet_gradients(self._h, pi, pt, D, H, W, C.byref(loss),
                                               C.c_void_p(g.ctypes.data), m))
        return loss.value, g

    def get_state(self):
        st = np.empty(3 * self.num_params, np.float32)
        step = C.c_int64()
        self.ctx.check(lib().kv_unet_get_state(self._h, C.c_void_p(st.ctypes.data), C.byref(step)))
        return st, step.value

    def set_state(self, state, step):
        st = np.ascontiguousarray(state, np.float32)
        if st.size != 3 * self.num_params:
            raise ValueError("state size mismatch")
        self.ctx.check(lib().kv_unet_set_state(self._h, C.c_void_p(st.ctypes.data), int(step)))

    @property
    def params(self):
        return self.get_state()[0][: self.num_params]

    def save(self, path):
        """Full training state (parameters and Adam moments)."""
        st, step = self.get_state()
        np.savez(path, state=st, step=step)

    def save_weights(self, path):
        """Parameters only (for inference; training resumes with fresh moments)."""
        st, step = self.get_state()
        np.savez_compressed(path, params=st[: self.num_params], step=step)

    def load(self, path):
        """Loads a file written by save() or save_weights()."""
        z = np.load(path)
        if "state" in z.files:
            self.set_state(z["state"], int(z["step"]))
            return
        n = self.num_params
        params = np.asarray(z["params"], np.float32)
        if params.size != n:
            raise ValueError(f"checkpoint holds {params.size} parameters, the network has {n}")
        self.set_state(np.concatenate([params, np.zeros(2 * n, np.float32)]), int(z["step"]))
