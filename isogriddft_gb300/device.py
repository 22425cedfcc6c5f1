"""Device residency: per-geometry caches and tensor plumbing.

Geometry arrays are uploaded once per geometry object and cached with a
weakref finaliser (the reference keys its JAX caches by ``id(grid)``,
``ks/eigensolver_jax_cache.py:26-35``, which breaks when ids are reused;
a finaliser drops the entry when the geometry object dies).
"""

from __future__ import annotations

import contextlib
import threading

import weakref

import numpy as np
import torch

from . import _lib
from .grid import is_monitor_geometry

_CACHE: dict[int, "DeviceGrid"] = {}


def require_cuda() -> torch.device:
    if not torch.cuda.is_available():
        raise RuntimeError("isogriddft_gb300 operators need a CUDA GPU (no CPU fallback)")
    _lib.load()
    return torch.device("cuda", torch.cuda.current_device())


_HELD = threading.local()  # per thread: the stream fixed by held_stream(), if any


def stream_ptr() -> int:
    """Current torch stream as a raw cudaStream_t (the value fixed by :func:`held_stream`, if any)."""

    fixed = getattr(_HELD, "stream", None)
    if fixed is not None:
        return fixed
    return torch.cuda.current_stream().cuda_stream


@contextlib.contextmanager
def held_stream():
    """Resolve the current stream once for a block of many launches (the lookup costs
    more than a launch); the block must not switch streams.  Per thread, so
    SCFs on several threads (each on its own stream) do not interfere."""

    old = getattr(_HELD, "stream", None)
    _HELD.stream = torch.cuda.current_stream().cuda_stream
    try:
        yield _HELD.stream
    finally:
        _HELD.stream = old


def ptr(t) -> int | None:
    return None if t is None else t.data_ptr()


def torch_dtype(dtype: str):
    return {"fp32": torch.float32, "fp64": torch.float64}[dtype]


def igd_dtype(tdtype) -> int:
    if tdtype == torch.float32:
        return _lib.IGD_F32
    if tdtype == torch.float64:
        return _lib.IGD_F64
    raise ValueError(f"unsupported dtype {tdtype}")


def normalize_precision(precision: str) -> str:
    p = precision.strip().lower()
    if p in ("fp64", "float64", "double"):
        return "fp64"
    if p in ("fp32", "float32", "single", "mixed"):
        return "fp32"
    raise ValueError(f"precision must be `fp64` or `fp32`; received `{precision}`")


def _step(coords, label: str = "x") -> float:
    """Uniform logical spacing (``ops/kinetic.py:76-84``, same message)."""

    d = np.diff(np.asarray(coords, dtype=np.float64))
    if not np.allclose(d, d[0]):
        raise ValueError(f"The current kinetic operator expects a uniform logical {label}-axis.")
    return float(d[0])


def validate_geometry(geom) -> None:
    """The reference operators' geometry checks (``ops/kinetic.py:76-84, 156-162``, same
    messages), on the host before anything is copied to the device: uniform logical axes, and for
    monitor grids a finite, strictly positive Jacobian and a finite inverse metric."""

    names = ("logical_x", "logical_y", "logical_z") if is_monitor_geometry(geom) else \
        ("x_logical", "y_logical", "z_logical")
    for label, name in zip("xyz", names):
        _step(getattr(geom, name), label)
    if is_monitor_geometry(geom):
        j = np.asarray(geom.jacobian, dtype=np.float64)
        if np.any(~np.isfinite(j)):
            raise ValueError("Monitor-grid Jacobian must be finite.")
        if np.any(j <= 0.0):
            raise ValueError("Monitor-grid Jacobian must stay strictly positive.")
        if np.any(~np.isfinite(np.asarray(geom.inverse_metric_tensor, dtype=np.float64))):
            raise ValueError("Monitor-grid inverse metric tensor must be finite.")


def _legacy_axis_coeffs(h_pts, logical):
    """cm, cp of the legacy flux form (``ops/kinetic.py:87-114``)."""

    s = np.asarray(h_pts, dtype=np.float64)
    du = _step(logical)
    face = 0.5 * (s[:-1] + s[1:])
    cm = np.empty_like(s)
    cp = np.empty_like(s)
    cm[0] = 1.0 / (du * s[0] * du * s[0])
    cm[1:] = 1.0 / (du * face * du * s[1:])
    cp[:-1] = 1.0 / (du * face * du * s[:-1])
    cp[-1] = 1.0 / (du * s[-1] * du * s[-1])
    return cm, cp


class DeviceGrid:
    """Device copies of one geometry (FP64 source arrays + per-dtype coefficients)."""

    def __init__(self, geom):
        validate_geometry(geom)
        self.device = require_cuda()
        self.geom_ref = weakref.ref(geom)
        self.monitor = is_monitor_geometry(geom)
        self.shape = tuple(int(s) for s in geom.spec.shape)
        self.n = int(np.prod(self.shape))
        dev = self.device
        f64 = lambda a: torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64), device=dev)  # noqa: E731
        self.cell_volumes = f64(geom.cell_volumes).reshape(-1)
        self.x = f64(geom.x_points).reshape(-1)
        self.y = f64(geom.y_points).reshape(-1)
        self.z = f64(geom.z_points).reshape(-1)
        self._coeffs: dict[str, torch.Tensor] = {}
        self._cache: dict = {}  # per-geometry device data built on first use (solver preconditioners)
        if self.monitor:
            self.h = (_step(geom.logical_x), _step(geom.logical_y), _step(geom.logical_z))
            j = np.asarray(geom.jacobian, dtype=np.float64)
            g = np.asarray(geom.inverse_metric_tensor, dtype=np.float64)
            self.jacobian = f64(j).reshape(-1)
            self.inverse_metric = f64(g).reshape(-1)
            self.box_bounds = geom.spec.box_bounds
        else:
            cx = _legacy_axis_coeffs(geom.x_point_jacobian, geom.x_logical)
            cy = _legacy_axis_coeffs(geom.y_point_jacobian, geom.y_logical)
            cz = _legacy_axis_coeffs(geom.z_point_jacobian, geom.z_logical)
            self.axis_coeffs = f64(np.concatenate([cx[0], cx[1], cy[0], cy[1], cz[0], cz[1]]))
            self.reference_center = tuple(geom.spec.reference_center)
            self.legacy_h = (
                np.asarray(geom.x_point_jacobian, dtype=np.float64),
                np.asarray(geom.y_point_jacobian, dtype=np.float64),
                np.asarray(geom.z_point_jacobian, dtype=np.float64),
            )
            self.legacy_du = (_step(geom.x_logical), _step(geom.y_logical), _step(geom.z_logical))

    def workspace(self, name: str, nbytes: int) -> torch.Tensor:
        """Cached device workspace of at least ``nbytes`` bytes (256-byte aligned)."""

        ws = getattr(self, "_ws", None)
        if ws is None:
            ws = self._ws = {}
        t = ws.get(name)
        if t is None or t.numel() < nbytes:
            t = torch.empty(int(nbytes) + 256, dtype=torch.uint8, device=self.device)
            ws[name] = t
        return t

    def potential(self, v, tdtype) -> torch.Tensor | None:
        """Device copy of a potential field in ``tdtype`` (cached by host-array identity)."""

        if v is None:
            return None
        if isinstance(v, torch.Tensor) and v.is_cuda:
            return v.reshape(-1).to(tdtype).contiguous()
        key = (id(v), tdtype)
        hit = getattr(self, "_pot", None)
        if hit is not None and hit[0] == key and hit[1] is v:
            return hit[2]
        t = to_device(v, tdtype, self.device).reshape(-1)
        if t.numel() != self.n:
            raise ValueError("potential must match the grid shape")
        self._pot = (key, v, t)
        return t

    def coeffs(self, dtype: str) -> torch.Tensor:
        """Seven folded stencil coefficient fields (A~ab and 1/J) in ``dtype``."""

        if not self.monitor:
            raise TypeError("stencil coefficients exist only for monitor geometries")
        c = self._coeffs.get(dtype)
        if c is None:
            c = torch.empty(7 * self.n, dtype=torch_dtype(dtype), device=self.device)
            nx, ny, nz = self.shape
            _lib.check(
                _lib.call("igd_agrid_prepare_geometry", igd_dtype(c.dtype), nx, ny, nz, *self.h,
                          ptr(self.jacobian), ptr(self.inverse_metric), ptr(c), stream_ptr()),
                "igd_agrid_prepare_geometry",
            )
            self._coeffs[dtype] = c
        return c


def device_grid(geom) -> DeviceGrid:
    key = id(geom)
    dg = _CACHE.get(key)
    if dg is not None and dg.geom_ref() is geom:
        return dg
    dg = DeviceGrid(geom)
    _CACHE[key] = dg
    weakref.finalize(geom, _CACHE.pop, key, None)
    return dg


def clear_cache() -> None:
    _CACHE.clear()


def to_device(a, dtype, dev) -> torch.Tensor:
    """Host array or tensor -> contiguous device tensor of ``dtype``."""

    if isinstance(a, torch.Tensor):
        return a.to(device=dev, dtype=dtype).contiguous()
    arr = np.asarray(a)
    if not np.issubdtype(arr.dtype, np.inexact):
        arr = arr.astype(np.float64)
    return torch.as_tensor(np.ascontiguousarray(arr), device=dev).to(dtype)
