"""Drop-in kinetic / Laplacian operators on the GPU.

Names, arguments and errors mirror ``src/isogrid/ops/kinetic.py``
(``validate_orbital_field`` :41-58, ``integrate_field`` :61-66,
``weighted_l2_norm`` :69-74, legacy :117-153, monitor :279-358, dispatch
:361-374).  Host NumPy inputs return NumPy FP64 results; CUDA tensors stay
on the device.  Extra keyword-only argument ``precision`` selects the FP64
parity path (default) or the FP32 stencil.
"""

from __future__ import annotations

import numpy as np
import torch

from . import _lib
from .device import device_grid, igd_dtype, normalize_precision, ptr, require_cuda, stream_ptr, to_device, torch_dtype
from .grid import is_monitor_geometry


def validate_orbital_field(psi, grid_geometry, name: str = "psi"):
    if isinstance(psi, torch.Tensor):
        field = psi
        if field.dim() != 3:
            raise ValueError(f"{name} must be a 3D field; received ndim={field.dim()}.")
        if tuple(field.shape) != tuple(grid_geometry.spec.shape):
            raise ValueError(f"{name} must match the grid shape {grid_geometry.spec.shape}; received {tuple(field.shape)}.")
        return field
    field = np.asarray(psi)
    if field.ndim != 3:
        raise ValueError(f"{name} must be a 3D field; received ndim={field.ndim}.")
    if field.shape != tuple(grid_geometry.spec.shape):
        raise ValueError(f"{name} must match the grid shape {grid_geometry.spec.shape}; received {field.shape}.")
    if not np.issubdtype(field.dtype, np.inexact):
        field = field.astype(np.float64)
    return field


def hpsi_device(dg, psi: torch.Tensor, *, closure: str = "trial_fix", kscale: float = -0.5, veff=None,
                vscale: float = 1.0, out: torch.Tensor | None = None) -> torch.Tensor:
    """GPU-native block apply: ``psi`` is (nb, nx, ny, nz) or (nb, n), contiguous, fp32/fp64."""

    nb = psi.shape[0] if psi.dim() in (2, 4) else 1
    # the kernels address nb orbitals of dg.n points through raw pointers: a tensor of another
    # size, layout or device would be read or written out of bounds, so it is refused here
    if not (psi.is_cuda and psi.is_contiguous() and psi.numel() == nb * dg.n):
        raise ValueError(f"psi must be a contiguous CUDA block of {nb} x {dg.n} points; "
                         f"received shape {tuple(psi.shape)} on {psi.device}.")
    if out is None:
        out = torch.empty_like(psi)
    elif not (out.is_cuda and out.is_contiguous() and out.numel() == psi.numel() and out.dtype == psi.dtype):
        raise ValueError(f"out must be a contiguous CUDA tensor like psi; received shape {tuple(out.shape)}, "
                         f"{out.dtype} on {out.device}.")
    nx, ny, nz = dg.shape
    dt = igd_dtype(psi.dtype)
    if veff is not None and veff.dtype != psi.dtype:
        raise ValueError("veff must have the orbital dtype")
    if veff is not None and not (veff.is_cuda and veff.is_contiguous() and veff.numel() == dg.n):
        raise ValueError(f"veff must be a contiguous CUDA field of {dg.n} points; received shape "
                         f"{tuple(veff.shape)} on {veff.device}.")
    if dg.monitor:
        coeffs = dg.coeffs("fp32" if psi.dtype == torch.float32 else "fp64")
        cl = _lib.IGD_CLOSURE_PRODUCTION if closure == "production" else _lib.IGD_CLOSURE_TRIAL_FIX
        st = _lib.call("igd_hpsi_agrid", dt, cl, nx, ny, nz, ptr(coeffs), ptr(veff), ptr(psi), ptr(out), nb, dg.n,
                       kscale, vscale, stream_ptr())
        _lib.check(st, "igd_hpsi_agrid")
    else:
        st = _lib.call("igd_hpsi_legacy", dt, nx, ny, nz, ptr(dg.axis_coeffs), ptr(veff), ptr(psi), ptr(out), nb,
                       dg.n, kscale, vscale, stream_ptr())
        _lib.check(st, "igd_hpsi_legacy")
    return out


def apply_hamiltonian_block(orbitals, grid_geometry, effective_local_potential, *, kinetic_version: str = "trial_fix",
                            precision: str = "fp32", out=None):
    """H psi_i = T psi_i + v_eff psi_i for an orbital block (k, nx, ny, nz).

    Block form of ``apply_fixed_potential_static_local_block``
    (``ks/eigensolver.py:773-784``).  Host inputs (NumPy or CPU tensors,
    preferably pinned) are copied to the device, applied in one fused launch
    and copied back into ``out`` (a host array/tensor) or a new host tensor;
    pinned tensors of the compute dtype stream through in orbital chunks with
    the copies in, the stencil and the copies out overlapped.  CUDA inputs stay
    on the device.
    """

    dev = require_cuda()
    dg = device_grid(grid_geometry)
    tdt = torch_dtype(normalize_precision(precision))
    host = not (isinstance(orbitals, torch.Tensor) and orbitals.is_cuda)
    if host and _pipelinable(orbitals, out, tdt, dg.shape):
        veff = dg.potential(effective_local_potential, tdt)
        hin = orbitals if orbitals.dim() == 4 else orbitals.unsqueeze(0)
        if out is None:
            out = torch.empty(orbitals.shape, dtype=tdt, pin_memory=True)
        _pipelined_host_apply(dg, hin, out.view(hin.shape), kinetic_version, veff)
        return out
    block = to_device(orbitals, tdt, dev)
    if block.dim() == 3:
        block = block.unsqueeze(0)
    if tuple(block.shape[1:]) != tuple(dg.shape):
        raise ValueError(f"orbitals must have shape (k, {dg.shape}); received {tuple(block.shape)}.")
    veff = dg.potential(effective_local_potential, tdt)
    res = hpsi_device(dg, block.reshape(block.shape[0], -1), closure=kinetic_version, veff=veff).reshape(block.shape)
    if not host:
        if out is not None:
            out.copy_(res)
            return out
        return res
    if out is None:
        out = torch.empty(res.shape, dtype=res.dtype, pin_memory=True)
    if isinstance(out, torch.Tensor):
        out.copy_(res, non_blocking=True)
        torch.cuda.current_stream().synchronize()
        return out
    np.copyto(out, res.cpu().numpy())
    return out


_COPY_STREAMS: dict = {}


def _pipelinable(orbitals, out, tdt, shape) -> bool:
    """Pinned, contiguous host tensors of the compute dtype (and a matching pinned ``out``)."""

    def ok(t):
        return (isinstance(t, torch.Tensor) and not t.is_cuda and t.dtype == tdt and t.is_contiguous()
                and t.is_pinned() and t.dim() in (3, 4) and tuple(t.shape[-3:]) == tuple(shape))

    return ok(orbitals) and (out is None or (ok(out) and out.shape == orbitals.shape))


def _pipelined_host_apply(dg, host_in: torch.Tensor, host_out: torch.Tensor, closure: str, veff,
                          chunk: int | None = None) -> None:
    """Host-to-host block apply in orbital chunks on three streams: the copy in of chunk i+1,
    the fused stencil on chunk i and the copy out of chunk i-1 overlap (the copy engines of
    the two directions run concurrently).  Returns after the last copy out has landed.

    Monitor grids run the whole pipeline in one native call (``igd_hpsi_agrid_host``, eight
    chunks by default); the legacy grid chunks from Python."""

    dev = dg.device
    k = host_in.shape[0]
    if dg.monitor:
        din = torch.empty(host_in.shape, dtype=host_in.dtype, device=dev)
        dout = torch.empty_like(din)
        nx, ny, nz = dg.shape
        coeffs = dg.coeffs("fp32" if host_in.dtype == torch.float32 else "fp64")
        cl = _lib.IGD_CLOSURE_PRODUCTION if closure == "production" else _lib.IGD_CLOSURE_TRIAL_FIX
        sp = stream_ptr()
        st = _lib.call("igd_hpsi_agrid_host", igd_dtype(host_in.dtype), cl, nx, ny, nz, ptr(coeffs), ptr(veff),
                       ptr(host_in), ptr(host_out), k, -0.5, 1.0, ptr(din), ptr(dout), int(chunk or 0), sp)
        _lib.check(st, "igd_hpsi_agrid_host")  # returns once host_out is complete
        return
    chunk = chunk or max(1, -(-k // 8))
    key = torch.cuda.current_device() if dev.index is None else dev.index
    if key not in _COPY_STREAMS:
        _COPY_STREAMS[key] = (torch.cuda.Stream(device=dev), torch.cuda.Stream(device=dev))
    h2d, d2h = _COPY_STREAMS[key]
    comp = torch.cuda.current_stream(dev)
    din = torch.empty(host_in.shape, dtype=host_in.dtype, device=dev)
    dout = torch.empty_like(din)
    h2d.wait_stream(comp)  # the buffers' earlier users on the compute stream are done
    d2h.wait_stream(comp)
    n = dg.n
    for i0 in range(0, k, chunk):
        i1 = min(k, i0 + chunk)
        with torch.cuda.stream(h2d):
            din[i0:i1].copy_(host_in[i0:i1], non_blocking=True)
        comp.wait_stream(h2d)
        hpsi_device(dg, din[i0:i1].view(i1 - i0, n), closure=closure, veff=veff, out=dout[i0:i1].view(i1 - i0, n))
        d2h.wait_stream(comp)
        with torch.cuda.stream(d2h):
            host_out[i0:i1].copy_(dout[i0:i1], non_blocking=True)
    comp.wait_stream(d2h)  # device buffers stay live until the copies out are done
    d2h.synchronize()


def _apply(psi, grid_geometry, closure, kscale, precision):
    field = validate_orbital_field(psi, grid_geometry)
    dev = require_cuda()
    dg = device_grid(grid_geometry)
    if isinstance(field, torch.Tensor):
        t = field.contiguous()
        if not t.is_cuda:
            t = t.to(dev)
        return hpsi_device(dg, t.reshape(1, -1), closure=closure, kscale=kscale).reshape(field.shape)
    t = to_device(field, torch_dtype(normalize_precision(precision)), dev).reshape(1, -1)
    out = hpsi_device(dg, t, closure=closure, kscale=kscale)
    return out.reshape(field.shape).to(torch.float64).cpu().numpy()


def _require_monitor(grid_geometry):
    if not is_monitor_geometry(grid_geometry):
        raise TypeError("This operator requires a MonitorGridGeometry.")


def _require_legacy(grid_geometry):
    if is_monitor_geometry(grid_geometry):
        raise TypeError("This operator requires a StructuredGridGeometry.")


def apply_legacy_laplacian_operator(psi, grid_geometry, *, precision: str = "fp64"):
    _require_legacy(grid_geometry)
    return _apply(psi, grid_geometry, "legacy", 1.0, precision)


def apply_legacy_kinetic_operator(psi, grid_geometry, *, precision: str = "fp64"):
    _require_legacy(grid_geometry)
    return _apply(psi, grid_geometry, "legacy", -0.5, precision)


def apply_monitor_grid_laplacian_operator(psi, grid_geometry, *, precision: str = "fp64"):
    _require_monitor(grid_geometry)
    return _apply(psi, grid_geometry, "production", 1.0, precision)


def apply_monitor_grid_laplacian_operator_trial_boundary_fix(psi, grid_geometry, *, precision: str = "fp64"):
    _require_monitor(grid_geometry)
    return _apply(psi, grid_geometry, "trial_fix", 1.0, precision)


def apply_monitor_grid_kinetic_operator(psi, grid_geometry, *, precision: str = "fp64"):
    _require_monitor(grid_geometry)
    return _apply(psi, grid_geometry, "production", -0.5, precision)


def apply_monitor_grid_kinetic_operator_trial_boundary_fix(psi, grid_geometry, *, precision: str = "fp64"):
    _require_monitor(grid_geometry)
    return _apply(psi, grid_geometry, "trial_fix", -0.5, precision)


def apply_laplacian_operator(psi, grid_geometry, *, precision: str = "fp64"):
    if is_monitor_geometry(grid_geometry):
        return apply_monitor_grid_laplacian_operator(psi, grid_geometry, precision=precision)
    return apply_legacy_laplacian_operator(psi, grid_geometry, precision=precision)


def apply_kinetic_operator(psi, grid_geometry, *, precision: str = "fp64"):
    if is_monitor_geometry(grid_geometry):
        return apply_monitor_grid_kinetic_operator(psi, grid_geometry, precision=precision)
    return apply_legacy_kinetic_operator(psi, grid_geometry, precision=precision)


def integrate_field(field, grid_geometry):
    """sum(field * cell_volumes) in FP64 (host arrays stay on the host)."""

    if isinstance(field, torch.Tensor):
        dg = device_grid(grid_geometry)
        return float(torch.dot(field.reshape(-1).to(torch.float64), dg.cell_volumes))
    values = validate_orbital_field(field, grid_geometry, name="field")
    return np.sum(values * grid_geometry.cell_volumes, dtype=np.result_type(values.dtype, np.float64))


def weighted_l2_norm(field, grid_geometry) -> float:
    if isinstance(field, torch.Tensor):
        dg = device_grid(grid_geometry)
        f = field.reshape(-1).to(torch.float64)
        return float(torch.sqrt(torch.dot(f * f, dg.cell_volumes)))
    values = validate_orbital_field(field, grid_geometry, name="field")
    return float(np.sqrt(np.sum(np.abs(values) ** 2 * grid_geometry.cell_volumes, dtype=np.float64)))


def autotune_report() -> list[str]:
    """The H.Psi autotuner's picks so far, one line per (closure, grid shape, orbital count,
    v_eff present): "closure nx ny nz nb veff -> orbitals per CTA (us per launch)"."""

    import ctypes

    n = int(_lib.call("igd_hpsi_autotune_report", None, 0))
    buf = ctypes.create_string_buffer(n + 1)
    _lib.call("igd_hpsi_autotune_report", buf, n + 1)
    return [line for line in buf.value.decode().splitlines() if line]
