"""Monitor A-grid generation on the GPU (FP64).

Drives the kernels of ``csrc/grid_gen.cu`` through the outer loop of the
reference generator (``grid/monitor_geometry.py:481-577``): per outer
iteration the monitor field on the current coordinates, smoothing, up to
``harmonic_inner_iterations`` damped-Jacobi sweeps with device-side
convergence detection, the Jacobian-floor backtracking update and the
displacement test; then the final geometry.  Arithmetic is the reference's,
in the same order, but exp/pow/division come from CUDA's libraries and the
3x3 inverse/determinant are closed-form, so results agree with the host
builder to rounding (the tests hold them to 1e-10 relative) rather than bit
for bit.  Host <-> device traffic: one sync per outer iteration and per
backtracking trial.
"""

from __future__ import annotations

import numpy as np
import torch

from . import _lib
from .device import ptr, require_cuda, stream_ptr
from .grid import (
    GlobalMonitorField,
    MonitorGridGeometry,
    _patch_interfaces,
    _quality,
    _uniform_step,
    monitor_box_axes,
)

_JACOBIAN_FLOOR = 1.0e-12


def _atom_table(case, spec, dev) -> torch.Tensor:
    rows = []
    for atom in case.geometry.atoms:
        p = spec.element_parameters[atom.element]
        rows.append([*atom.position, p.kinetic_weight, p.near_core_radius, p.kinetic_exponent, p.local_weight,
                     p.local_radius, p.local_exponent, p.projector_weight, p.projector_radius, p.projector_exponent,
                     p.monitor_cap])
    return torch.tensor(np.asarray(rows, dtype=np.float64).reshape(-1), device=dev)


def _call(name, *args):
    _lib.check(_lib.call(name, *args), name)


def generate_monitor_grid_geometry_device(case, spec, *, return_device: bool = False):
    """Device twin of ``generate_monitor_grid_geometry``; returns a MonitorGridGeometry."""

    if case.geometry.unit.lower() != spec.unit.lower():
        raise ValueError("Benchmark geometry and monitor-grid spec must use the same unit system.")
    dev = require_cuda()
    st = stream_ptr()
    nx, ny, nz = spec.shape
    n = nx * ny * nz
    lx, ly, lz, box = monitor_box_axes(spec)
    hx, hy, hz = _uniform_step(lx), _uniform_step(ly), _uniform_step(lz)
    # SoA coordinates (3, n)
    fixed = torch.as_tensor(np.ascontiguousarray(np.moveaxis(box, -1, 0).reshape(3, n)), device=dev)
    X = fixed.clone()
    buf0 = torch.empty_like(X)
    buf1 = torch.empty_like(X)
    atoms = _atom_table(case, spec, dev)
    mon = torch.empty(n, dtype=torch.float64, device=dev)
    raw = torch.empty(n, dtype=torch.float64, device=dev)
    smoothed = torch.empty_like(mon)
    state = torch.zeros(2, dtype=torch.int64, device=dev)
    scratch = torch.zeros(1, dtype=torch.int64, device=dev)
    scal = torch.zeros(1, dtype=torch.float64, device=dev)
    natoms = len(case.geometry.atoms)
    sweeps = spec.harmonic_inner_iterations
    for _ in range(spec.harmonic_outer_iterations):
        _call("igd_grid_monitor_field", n, ptr(X[0]), ptr(X[1]), ptr(X[2]), natoms, ptr(atoms), ptr(mon), None, st)
        if spec.monitor_smoothing > 0.0:
            _call("igd_grid_smooth", nx, ny, nz, ptr(mon), ptr(smoothed), spec.monitor_smoothing, st)
            coef = smoothed
        else:
            coef = mon
        buf0.copy_(X)  # faces of X are the fixed box faces at every stage
        _call("igd_grid_harmonic_sweeps", nx, ny, nz, ptr(coef), ptr(buf0), ptr(buf1), hx, hy, hz,
              spec.inner_relaxation, spec.harmonic_tolerance, sweeps, ptr(state), st)
        conv = int(state.view(torch.int32)[3].item())
        solved = (buf0, buf1)[(conv + 1) % 2] if conv >= 0 else (buf0, buf1)[sweeps % 2]
        alpha = spec.harmonic_relaxation
        moved = 0.0
        accepted = False
        while alpha >= 1.0e-3:
            _call("igd_grid_min_jacobian", nx, ny, nz, ptr(X), ptr(solved), alpha, hx, hy, hz, ptr(scratch), ptr(scal), st)
            if float(scal.item()) > _JACOBIAN_FLOOR:
                _call("igd_grid_relax_update", 3 * n, ptr(X), ptr(solved), alpha, ptr(scratch), ptr(scal), st)
                moved = float(scal.item())
                accepted = True
                break
            alpha *= 0.5
        if not accepted:
            moved = 0.0
        if moved < spec.harmonic_tolerance:
            break
    _call("igd_grid_monitor_field", n, ptr(X[0]), ptr(X[1]), ptr(X[2]), natoms, ptr(atoms), ptr(mon), ptr(raw), st)
    basis = torch.empty(n * 9, dtype=torch.float64, device=dev)
    metric = torch.empty_like(basis)
    inv = torch.empty_like(basis)
    jac = torch.empty(n, dtype=torch.float64, device=dev)
    vol = torch.empty_like(jac)
    spacing = torch.empty(n * 3, dtype=torch.float64, device=dev)
    _call("igd_grid_geometry", nx, ny, nz, ptr(X), hx, hy, hz, ptr(basis), ptr(metric), ptr(inv), ptr(jac), ptr(vol),
          ptr(spacing), st)
    shape = spec.shape
    host = lambda t, extra=(): t.cpu().numpy().reshape(shape + extra)  # noqa: E731
    Xh = X.cpu().numpy().reshape((3,) + shape)
    sp = host(spacing, (3,))
    measure = np.mean(sp, axis=-1)
    values, raw_h = host(mon), host(raw)
    monitor = GlobalMonitorField(values=values, raw_values=raw_h, atomic_contributions=(),
                                 baseline_value=1.0, minimum_value=float(values.min()), maximum_value=float(values.max()))
    jach, volh = host(jac), host(vol)

    class _Part:  # per-atom record for the quality report
        def __init__(self, atom):
            self.position = atom.position
            self.parameters = spec.element_parameters[atom.element]

    parts = type("M", (), {"atomic_contributions": tuple(_Part(a) for a in case.geometry.atoms)})
    quality = _quality(spec, Xh[0], Xh[1], Xh[2], jach, volh, measure, parts)
    geom = MonitorGridGeometry(
        spec=spec, logical_x=lx, logical_y=ly, logical_z=lz, x_points=Xh[0], y_points=Xh[1], z_points=Xh[2],
        covariant_basis=host(basis, (3, 3)), jacobian=jach, metric_tensor=host(metric, (3, 3)),
        inverse_metric_tensor=host(inv, (3, 3)), cell_volumes=volh, spacing_x=sp[..., 0], spacing_y=sp[..., 1],
        spacing_z=sp[..., 2], spacing_measure=measure, monitor_field=monitor,
        patch_interfaces=_patch_interfaces(case, spec.element_parameters), quality_report=quality,
    )
    return geom
