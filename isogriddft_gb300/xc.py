"""Spin-polarised LSDA on the GPU (drop-in for ``src/isogrid/xc/lsda.py``).

``evaluate_lsda_terms`` (:70-121) returns the reference's ``LSDAEvaluation``
fields; the arithmetic is the library's Slater + VWN5 kernel (the functional
the reference obtains from libxc as ``lda,vwn``), FP64 by default or FP32 math
with ``precision="fp32"``.  ``lda,pw92`` selects Slater + PW92 (an addition).
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np
import torch

from . import _lib
from .device import device_grid, ptr, require_cuda, stream_ptr

SUPPORTED_LSDA_FUNCTIONAL = "lda,vwn"
_FUNCTIONALS = {"lda,vwn": 0, "lda,pw92": 1, "lda,pw": 1}


@dataclass(frozen=True)
class LSDAEvaluation:
    functional: str
    backend: str
    rho_up: np.ndarray
    rho_down: np.ndarray
    rho_total: np.ndarray
    eps_xc: np.ndarray
    energy_density: np.ndarray
    v_xc_up: np.ndarray
    v_xc_down: np.ndarray


def _functional_id(functional: str) -> tuple[str, int]:
    f = functional.strip().lower()
    if f not in _FUNCTIONALS:
        raise ValueError("The current IsoGridDFT LSDA layer supports only the PySCF-aligned `lda,vwn` "
                         f"functional (and `lda,pw92`); received `{functional}`.")
    return f, _FUNCTIONALS[f]


def lsda_device(rho_up: torch.Tensor, rho_down: torch.Tensor, *, functional: str = "lda,vwn", math: str = "fp64",
                w: torch.Tensor | None = None, want=("eps", "v_up", "v_down", "edens")):
    """Device LSDA on flat tensors; returns dict of device tensors (+ 'energy' if w given)."""

    _, fid = _functional_id(functional)
    dt = _lib.IGD_F64 if rho_up.dtype == torch.float64 else _lib.IGD_F32
    mt = _lib.IGD_F64 if math == "fp64" else _lib.IGD_F32
    n = rho_up.numel()
    # the kernel reads n points of each input through raw pointers
    for name, t in (("rho_up", rho_up), ("rho_down", rho_down), ("w", w)):
        if t is not None and not (t.is_cuda and t.is_contiguous() and t.numel() == n
                                  and t.dtype == (torch.float64 if name == "w" else rho_up.dtype)):
            raise ValueError(f"{name} must be a contiguous CUDA field of {n} points like rho_up; received shape "
                             f"{tuple(t.shape)}, {t.dtype} on {t.device}.")
    out ={k: (torch.empty_like(rho_up) if k in want else None) for k in ("eps", "v_up", "v_down", "edens")}
    energy = torch.zeros(1, dtype=torch.float64, device=rho_up.device) if w is not None else None
    flags = torch.zeros(1, dtype=torch.int32, device=rho_up.device)
    _lib.check(_lib.call("igd_lsda", dt, mt, fid, n, ptr(rho_up), ptr(rho_down), ptr(out["eps"]), ptr(out["v_up"]),
                         ptr(out["v_down"]), ptr(out["edens"]), ptr(w), ptr(energy), ptr(flags), stream_ptr()),
               "igd_lsda")
    if int(flags.item()):
        _raise_input_error(rho_up, rho_down)
    if energy is not None:
        out["energy"] = energy
    return out


def _raise_input_error(rho_up: torch.Tensor, rho_down: torch.Tensor):
    """Name the offending field once the kernel has flagged bad input, in the reference's order
    (``xc/lsda.py:56-67``: each field checked for finite values, then for non-negativity up to
    roundoff, rho_up first)."""

    tol = 1.0e-14  # the kernel's threshold, on the value converted to FP64
    for name, t in (("rho_up", rho_up), ("rho_down", rho_down)):
        if not bool(torch.isfinite(t).all()):
            raise ValueError(f"{name} must contain only finite values.")
        if bool((t < -tol).any()):
            raise ValueError(f"{name} must be non-negative up to roundoff.")
    raise ValueError("rho_up / rho_down must contain only finite, non-negative values.")


def _host_input(rho, name):
    values = np.asarray(rho, dtype=np.float64)
    if values.ndim != 3:
        raise ValueError(f"{name} must be a 3D field; received ndim={values.ndim}.")
    return values


def evaluate_lsda_terms(rho_up, rho_down, functional: str = SUPPORTED_LSDA_FUNCTIONAL, *,
                        precision: str = "fp64") -> LSDAEvaluation:
    name, _ = _functional_id(functional)
    up = _host_input(rho_up, "rho_up")
    dn = _host_input(rho_down, "rho_down")
    if up.shape != dn.shape:
        raise ValueError(f"rho_up and rho_down must have the same 3D shape; received {up.shape} and {dn.shape}.")
    dev = require_cuda()
    tu = torch.as_tensor(np.ascontiguousarray(up), device=dev).reshape(-1)
    td = torch.as_tensor(np.ascontiguousarray(dn), device=dev).reshape(-1)
    o = lsda_device(tu, td, functional=name, math="fp64" if precision == "fp64" else "fp32")
    host = lambda t: t.cpu().numpy().reshape(up.shape)  # noqa: E731
    upc, dnc = np.maximum(up, 0.0), np.maximum(dn, 0.0)
    return LSDAEvaluation(functional=name, backend="gb300", rho_up=upc, rho_down=dnc, rho_total=upc + dnc,
                          eps_xc=host(o["eps"]), energy_density=host(o["edens"]), v_xc_up=host(o["v_up"]),
                          v_xc_down=host(o["v_down"]))


def evaluate_lsda_energy_density(rho_up, rho_down, functional: str = SUPPORTED_LSDA_FUNCTIONAL):
    return evaluate_lsda_terms(rho_up, rho_down, functional).eps_xc


def evaluate_lsda_potential(rho_up, rho_down, functional: str = SUPPORTED_LSDA_FUNCTIONAL):
    e = evaluate_lsda_terms(rho_up, rho_down, functional)
    return e.v_xc_up, e.v_xc_down


def evaluate_lsda_energy(rho_up, rho_down, grid_geometry, functional: str = SUPPORTED_LSDA_FUNCTIONAL, *,
                         precision: str = "fp64") -> float:
    """E_xc = sum rho eps_xc W (FP64 device reduction)."""

    name, _ = _functional_id(functional)
    dg = device_grid(grid_geometry)
    up = torch.as_tensor(np.ascontiguousarray(_host_input(rho_up, "rho_up")), device=dg.device).reshape(-1)
    dn = torch.as_tensor(np.ascontiguousarray(_host_input(rho_down, "rho_down")), device=dg.device).reshape(-1)
    o = lsda_device(up, dn, functional=name, math="fp64" if precision == "fp64" else "fp32", w=dg.cell_volumes,
                    want=())
    return float(o["energy"].item())
