"""Spin-density build, renormalisation and residual on the GPU.

Device counterparts of ``scf/driver.py``: ``_build_density_from_occupied_orbitals``
(:663-676), ``_renormalize_density`` (:679-690), ``_density_residual``
(:693-702), and ``build_total_density`` (``ks/static_hamiltonian.py:226-235``).
Orbitals may be FP32 or FP64; densities and sums are FP64.
"""

from __future__ import annotations

import numpy as np
import torch

from . import _lib
from .device import device_grid, ptr, stream_ptr
from .ks import validate_orbital_block
from .ops import validate_orbital_field


def build_density_device(dg, orbitals: torch.Tensor, occupations, *, out: torch.Tensor | None = None,
                         accumulate: bool = False, integral: torch.Tensor | None = None) -> torch.Tensor:
    nb = 0 if orbitals is None else orbitals.shape[0]
    occ = torch.as_tensor(np.asarray(occupations, dtype=np.float64), device=dg.device)
    if len(occ) < nb:
        nb = len(occ)
    if out is None:
        out = torch.zeros(dg.n, dtype=torch.float64, device=dg.device)
    dt = _lib.IGD_F32 if (orbitals is not None and orbitals.dtype == torch.float32) else _lib.IGD_F64
    _lib.check(_lib.call("igd_density", dt, dg.n, nb, dg.n, ptr(orbitals) if nb else None, ptr(occ) if nb else None,
                         ptr(dg.cell_volumes), ptr(out), ptr(integral), int(accumulate), stream_ptr()), "igd_density")
    return out


def renormalize_device(dg, rho: torch.Tensor, target: float, integral: torch.Tensor) -> torch.Tensor:
    if target == 0.0:
        rho.zero_()
        return rho
    flags = torch.zeros(1, dtype=torch.int32, device=dg.device)
    _lib.check(_lib.call("igd_density_renormalize", dg.n, ptr(rho), ptr(integral), float(target), ptr(flags),
                         stream_ptr()), "igd_density_renormalize")
    if int(flags.item()) & 4:
        raise ValueError("A positive density integral is required for renormalization.")
    return rho


def residual_device(dg, up_in, dn_in, up_out, dn_out) -> float:
    out = torch.zeros(1, dtype=torch.float64, device=dg.device)
    _lib.check(_lib.call("igd_density_residual2", dg.n, ptr(up_in), ptr(dn_in), ptr(up_out), ptr(dn_out),
                         ptr(dg.cell_volumes), ptr(out), stream_ptr()), "igd_density_residual2")
    return float(np.sqrt(max(float(out.item()), 0.0)))


def build_density_from_occupied_orbitals(orbitals, occupations, grid_geometry) -> np.ndarray:
    if len(occupations) == 0:
        return np.zeros(grid_geometry.spec.shape)
    block = np.asarray(validate_orbital_block(orbitals, grid_geometry, name="orbitals"), dtype=np.float64)
    dg = device_grid(grid_geometry)
    if block.shape[0] < len(occupations):
        raise ValueError("Not enough orbitals were provided for the requested occupations.")
    t = torch.as_tensor(np.ascontiguousarray(block[: len(occupations)]), device=dg.device).reshape(len(occupations), -1)
    return build_density_device(dg, t, occupations).cpu().numpy().reshape(grid_geometry.spec.shape)


def renormalize_density(rho, target_electrons: float, grid_geometry) -> np.ndarray:
    if target_electrons == 0.0:
        return np.zeros(grid_geometry.spec.shape)
    rho = validate_orbital_field(rho, grid_geometry, name="rho")
    dg = device_grid(grid_geometry)
    t = torch.as_tensor(np.ascontiguousarray(rho, dtype=np.float64), device=dg.device).reshape(-1)
    integral = torch.zeros(1, dtype=torch.float64, device=dg.device)
    _lib.check(_lib.call("igd_weighted_sum", _lib.IGD_F64, dg.n, ptr(t), None, ptr(dg.cell_volumes), ptr(integral),
                         stream_ptr()), "igd_weighted_sum")
    return renormalize_device(dg, t, target_electrons, integral).cpu().numpy().reshape(grid_geometry.spec.shape)


def density_residual(rho_up_in, rho_down_in, rho_up_out, rho_down_out, grid_geometry) -> float:
    # the reference takes weighted norms of the two differences (``ops/kinetic.py:69-74``), which
    # checks each difference against the grid shape with the same message
    fields = [np.asarray(a) for a in (rho_up_in, rho_down_in, rho_up_out, rho_down_out)]
    for a, b in ((fields[2], fields[0]), (fields[3], fields[1])):
        validate_orbital_field(a - b, grid_geometry, name="field")
    dg = device_grid(grid_geometry)
    f = lambda a: torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64), device=dg.device).reshape(-1)  # noqa: E731
    return residual_device(dg, *(f(a) for a in fields))


def build_total_density(rho_up, rho_down, grid_geometry) -> np.ndarray:
    return np.asarray(np.asarray(rho_up, dtype=np.float64) + np.asarray(rho_down, dtype=np.float64))
