"""Open-boundary Hartree / Poisson solve on the GPU (drop-in).

Mirrors ``src/isogrid/poisson/open_boundary.py`` and ``poisson/hartree.py``:
result dataclasses (:45-102), ``solve_open_boundary_poisson`` (:1379),
``solve_hartree_potential`` (``hartree.py:47-98``), ``evaluate_hartree_energy``
(:117-129), ``build_hartree_action`` (:132-144), ``evaluate_hartree_terms``
(:147-192).  The whole pipeline runs on the device: multipole moments (with
the monitor-grid corrected moments or the legacy_split correction), face
values, the split right-hand side 4 pi rho + L(b), the interior BiCGSTAB
(FP64, or FP32 inside FP64 iterative refinement with ``precision="mixed"``)
and the composition v = u + b.  ``tolerance`` keeps the SciPy meaning the
reference's default backend uses (relative 2-norm residual); the JAX-route
keyword arguments are accepted and ignored (one GPU solver serves both).
"""

from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib
from .device import DeviceGrid, device_grid, ptr, require_cuda, stream_ptr
from .grid import is_monitor_geometry
from .ops import hpsi_device, validate_orbital_field

_NEGATIVE_DENSITY_TOLERANCE = 1.0e-14
_VALID_MODES = {"corrected_moments", "legacy_split"}


@dataclass(frozen=True)
class OpenBoundaryBoundaryConstructionDiagnostics:
    baseline_total_charge: float
    baseline_dipole_moment: np.ndarray
    baseline_quadrupole_tensor: np.ndarray
    correction_total_charge: float
    correction_dipole_moment: np.ndarray
    correction_quadrupole_tensor: np.ndarray
    boundary_value_correction_rms: float
    boundary_value_correction_max_abs: float
    corrected_moment_boundary_rms_mismatch: float
    corrected_moment_boundary_max_abs_mismatch: float


@dataclass(frozen=True)
class OpenBoundaryPoissonResponseDiagnostics:
    boundary_value_rms: float
    boundary_value_max_abs: float
    boundary_source_laplacian_rms: float
    boundary_source_laplacian_max_abs: float
    rhs_l2_norm: float
    rhs_max_abs: float
    interior_potential_rms: float
    interior_potential_max_abs: float
    interior_poisson_residual_l2_norm: float
    interior_poisson_residual_max_abs: float


@dataclass(frozen=True)
class OpenBoundaryMultipoleBoundary:
    reference_center: tuple[float, float, float]
    multipole_order: int
    total_charge: float
    dipole_moment: np.ndarray
    quadrupole_tensor: np.ndarray
    boundary_values: np.ndarray
    description: str
    diagnostics: OpenBoundaryBoundaryConstructionDiagnostics | None = None


@dataclass(frozen=True)
class OpenBoundaryPoissonResult:
    rho: np.ndarray
    potential: np.ndarray
    boundary_condition: OpenBoundaryMultipoleBoundary
    solver_method: str
    solver_iterations: int
    residual_max: float
    description: str
    response_diagnostics: OpenBoundaryPoissonResponseDiagnostics | None = None


@dataclass(frozen=True)
class HartreeEvaluation:
    rho: np.ndarray
    potential: np.ndarray
    action: np.ndarray
    energy: float
    poisson_result: OpenBoundaryPoissonResult | None


def _check(st, what):
    _lib.check(st, what)


def _moments_to_pq(m: np.ndarray):
    q = float(m[0])
    p = np.array(m[1:4], dtype=np.float64)
    Q = np.array([[m[4], m[5], m[6]], [m[5], m[7], m[8]], [m[6], m[8], m[9]]], dtype=np.float64)
    return q, p, Q


def _face_potential_host(q, p, Q, dx, dy, dz, r, order):
    v = q / r
    if order >= 1:
        v = v + (p[0] * dx + p[1] * dy + p[2] * dz) / r**3
    if order >= 2:
        c = (Q[0, 0] * dx * dx + 2 * Q[0, 1] * dx * dy + 2 * Q[0, 2] * dx * dz + Q[1, 1] * dy * dy
             + 2 * Q[1, 2] * dy * dz + Q[2, 2] * dz * dz)
        v = v + 0.5 * c / r**5
    return v


def _selected_cells(dg: DeviceGrid, geom):
    """Cells with cell-averaged J at or above the 0.9 quantile over interior cells
    (``open_boundary.py:182-203``) and the incident-node fractions (:206-220, :278-285);
    geometry-only, cached per device grid."""

    hit = getattr(dg, "_sel", None)
    if hit is not None:
        return hit
    J = np.asarray(geom.jacobian, dtype=np.float64)
    cj = (J[:-1, :-1, :-1] + J[1:, :-1, :-1] + J[:-1, 1:, :-1] + J[1:, 1:, :-1]
          + J[:-1, :-1, 1:] + J[1:, :-1, 1:] + J[:-1, 1:, 1:] + J[1:, 1:, 1:]) / 8.0
    inner = np.zeros(cj.shape, dtype=bool)
    inner[1:-1, 1:-1, 1:-1] = True
    if not inner.any():
        dg._sel = (None, 0, None)
        return dg._sel
    thr = float(np.quantile(cj[inner], 0.9))
    mask = inner & (cj >= thr)
    cells = np.argwhere(mask).astype(np.int32)

    def incident(cm):
        c = cm.astype(np.float64)
        n = np.zeros(tuple(s + 1 for s in c.shape))
        for a in (0, 1):
            for b in (0, 1):
                for d in (0, 1):
                    n[a:a + c.shape[0], b:b + c.shape[1], d:d + c.shape[2]] += c
        return n

    tot = incident(np.ones_like(mask))
    frac = np.divide(incident(mask), tot, out=np.zeros_like(tot), where=tot > 0.0)
    dev = dg.device
    dg._sel = (torch.as_tensor(cells.reshape(-1), device=dev), int(cells.shape[0]),
               torch.as_tensor(frac.reshape(-1), device=dev))
    return dg._sel


def validate_density_field(rho, grid_geometry=None, name: str = "rho"):
    """``poisson/hartree.py:32-44`` (same messages): the grid shape, finite values, non-negative
    up to roundoff; returns the density clipped at zero.  Device tensors are checked on the
    device (flat tensors of the grid's point count are accepted)."""

    if isinstance(rho, torch.Tensor):
        if grid_geometry is not None and rho.numel() != int(np.prod(grid_geometry.spec.shape)):
            raise ValueError(f"{name} must match the grid shape {grid_geometry.spec.shape}; "
                             f"received {tuple(rho.shape)}.")
        t = rho.to(torch.float64)
        if not bool(torch.isfinite(t).all()):
            raise ValueError(f"{name} must contain only finite values.")
        if bool((t < -_NEGATIVE_DENSITY_TOLERANCE).any()):
            raise ValueError(f"{name} must be non-negative up to roundoff.")
        return torch.clamp_min(t, 0.0)
    if grid_geometry is not None:
        rho = validate_orbital_field(rho, grid_geometry, name=name)
    values = np.asarray(rho, dtype=np.float64)
    if not np.all(np.isfinite(values)):
        raise ValueError(f"{name} must contain only finite values.")
    if np.any(values < -_NEGATIVE_DENSITY_TOLERANCE):
        raise ValueError(f"{name} must be non-negative up to roundoff.")
    return np.maximum(values, 0.0)


class DevicePoissonSolution:
    """Device-side result of one open-boundary solve."""

    def __init__(self, potential, boundary, u, rhs, Lb, moments, baseline, iterations, residual_max, rel, rounds,
                 center, legacy_corr):
        self.potential, self.boundary, self.u, self.rhs, self.Lb = potential, boundary, u, rhs, Lb
        self.moments, self.baseline = moments, baseline
        self.iterations, self.residual_max, self.relative_residual, self.rounds = iterations, residual_max, rel, rounds
        self.center, self.legacy_corr = center, legacy_corr


_PCG_KINDS = {"none": 0, "diag": 1, "separable": 2, "line": 3}


def _uniform_logical_step(coords) -> float:
    """The logical spacing of a uniform axis; the JAX route rejects any other
    (``poisson/poisson_jax.py:236-245``, same message)."""

    d = np.diff(np.asarray(coords, dtype=np.float64))
    if not np.allclose(d, d[0]):
        raise ValueError("The current monitor-grid JAX Poisson kernels expect uniform logical axes.")
    return float(d[0])


def _pcg_preconditioner(geom, kind: str, dev):
    """Device data of the JAX route's preconditioners (``poisson/poisson_jax.py``): ``diag``
    (:248-273) 1 / (2 sum_a g^aa / h_a^2) floored at 1e-10 of its median, as a full field with
    zero faces; ``separable`` (:276-383) the orthonormal Dirichlet sine matrices and the inverse
    constant-stiffness spectrum, FP32; ``line`` (:411-579) the Thomas factorisation (sub-diagonal,
    c', 1/den) along the stiffest axis, three full fields.  Returns (data64, data32, axis)."""

    J = np.asarray(geom.jacobian, dtype=np.float64)
    G = np.asarray(geom.inverse_metric_tensor, dtype=np.float64)
    h = tuple(_uniform_logical_step(c) for c in (geom.logical_x, geom.logical_y, geom.logical_z))
    shape = J.shape
    if kind == "none":
        return None, None, 0
    if kind == "diag":
        d = 2.0 * (G[..., 0, 0] / h[0] ** 2 + G[..., 1, 1] / h[1] ** 2 + G[..., 2, 2] / h[2] ** 2)
        pos = d[np.isfinite(d) & (d > 0.0)]
        if pos.size == 0:
            raise ValueError("The monitor-grid Poisson diagonal surrogate must stay positive to build the very small "
                             "Jacobi preconditioner.")
        full = np.zeros(shape)
        full[1:-1, 1:-1, 1:-1] = (1.0 / np.maximum(d, max(1.0e-12, 1.0e-10 * float(np.median(pos)))))[1:-1, 1:-1,
                                                                                                          1:-1]
        return torch.as_tensor(full.reshape(-1), device=dev), None, 0
    Jc = J[1:-1, 1:-1, 1:-1]
    lows, ups = [], []
    for a in range(3):
        wa = J * G[..., a, a]
        lo, up = [slice(1, -1)] * 3, [slice(1, -1)] * 3
        lo[a], up[a] = slice(0, -2), slice(2, None)
        c = wa[1:-1, 1:-1, 1:-1]
        lows.append(0.5 * (c + wa[tuple(lo)]) / (Jc * h[a] ** 2))
        ups.append(0.5 * (c + wa[tuple(up)]) / (Jc * h[a] ** 2))
    stiff = [0.5 * float(np.mean(lows[a] + ups[a])) * h[a] ** 2 for a in range(3)]
    for k in stiff:
        if not np.isfinite(k) or k <= 0.0:
            raise ValueError("The separable monitor-grid preconditioner requires positive axis stiffness "
                             "coefficients.")
    inner = tuple(n - 2 for n in shape)
    if kind == "separable":
        mats, lam = [], []
        for a in range(3):
            m = inner[a]
            i = np.arange(1, m + 1, dtype=np.float64)
            mats.append(np.sqrt(2.0 / (m + 1)) * np.sin(np.pi * np.outer(i, i) / (m + 1)))
            lam.append(4.0 * np.sin(np.pi * i / (2.0 * (m + 1))) ** 2 / h[a] ** 2)
        ev = stiff[0] * lam[0][:, None, None] + stiff[1] * lam[1][None, :, None] + stiff[2] * lam[2][None, None, :]
        inv = 1.0 / np.maximum(ev, max(1.0e-12, 1.0e-12 * float(np.max(ev))))
        data = np.concatenate([mats[0].ravel(), mats[1].ravel(), mats[2].ravel(), inv.ravel()]).astype(np.float32)
        return None, torch.as_tensor(data, device=dev), 0
    if kind == "line":
        ax = int(np.argmax([2.0 * stiff[a] / h[a] ** 2 for a in range(3)]))
        diag = sum(lows[a] + ups[a] for a in range(3))
        lower, upper = np.zeros_like(diag), np.zeros_like(diag)
        sl_lo, sl_up = [slice(None)] * 3, [slice(None)] * 3
        sl_lo[ax], sl_up[ax] = slice(1, None), slice(None, -1)
        lower[tuple(sl_lo)] = -lows[ax][tuple(sl_lo)]
        upper[tuple(sl_up)] = -ups[ax][tuple(sl_up)]
        dl, ll, ul = (np.moveaxis(x, ax, -1) for x in (diag, lower, upper))
        cp, inv_den = np.zeros_like(dl), np.zeros_like(dl)
        prev_c = np.zeros(dl.shape[:-1])
        for i in range(dl.shape[-1]):  # Thomas factorisation, vectorised over the lines
            den = dl[..., i] - ll[..., i] * prev_c
            inv_den[..., i] = 1.0 / den
            cp[..., i] = ul[..., i] / den
            prev_c = cp[..., i]
        full = np.zeros((3,) + shape)
        for k, arr in enumerate((ll, cp, inv_den)):
            full[k][1:-1, 1:-1, 1:-1] = np.moveaxis(arr, -1, ax)
        return torch.as_tensor(full.reshape(-1), device=dev), None, ax
    raise ValueError(f"cg_preconditioner must be `none`, `diag`, `separable`, or `line`; received `{kind}`.")


def solve_poisson_device(dg: DeviceGrid, geom, rho_dev: torch.Tensor, *, multipole_order: int = 2,
                         tolerance: float = 1.0e-8, max_iterations: int = 400, precision: str = "fp64",
                         mode: str = "corrected_moments", start: torch.Tensor | None = None,
                         route: str = "bicgstab", cg_preconditioner: str = "none") -> DevicePoissonSolution:
    """Open-boundary Poisson for a validated FP64 device density (n,).

    ``start`` (the ``u`` field of an earlier solution on the same grid)
    starts the interior Krylov solve from that field instead of zero: the
    stopping rule is unchanged (||f - A u|| <= tolerance ||f||), the iteration
    count drops when the density has changed little (SCF steps).

    ``route="cg"`` (monitor grids, FP64) is the reference's JAX route instead:
    preconditioned CG from zero stopping at max |r| < ``tolerance``
    (``poisson/poisson_jax.py:675-750``) with ``cg_preconditioner`` none, diag,
    separable or line (``igd_poisson_pcg``)."""

    if multipole_order not in (0, 1, 2):
        raise ValueError("The current open-boundary multipole boundary supports only orders 0, 1, and 2; "
                         f"received {multipole_order}.")
    st = stream_ptr()
    dev = dg.device
    nx, ny, nz = dg.shape
    n = dg.n
    x, y, z, w = dg.x, dg.y, dg.z, dg.cell_volumes
    if dg.monitor:
        b = dg.box_bounds
        center = (0.5 * (b[0][0] + b[0][1]), 0.5 * (b[1][0] + b[1][1]), 0.5 * (b[2][0] + b[2][1]))
    else:
        center = tuple(float(c) for c in dg.reference_center)
    mom = torch.zeros(40, dtype=torch.float64, device=dev)  # base | region | quadrature | correction-pass
    base, region, quad, corr = mom[0:10], mom[10:20], mom[20:30], mom[30:40]
    _check(_lib.call("igd_multipole_nodal_moments", n, ptr(rho_dev), ptr(w), ptr(x), ptr(y), ptr(z), None, *center,
                     ptr(base), st), "nodal moments")
    bfield = torch.empty(n, dtype=torch.float64, device=dev)
    total = base
    legacy_corr = None
    if dg.monitor:
        cells, ncells, frac = _selected_cells(dg, geom)
        fail = torch.zeros(1, dtype=torch.int32, device=dev)
        dvol = float(np.prod(dg.h)) / 8.0
        if ncells > 0:
            _check(_lib.call("igd_multipole_nodal_moments", n, ptr(rho_dev), ptr(w), ptr(x), ptr(y), ptr(z), ptr(frac),
                             *center, ptr(region), st), "region moments")
            _check(_lib.call("igd_multipole_cell_quadrature", nx, ny, nz, ptr(x), ptr(y), ptr(z), ptr(dg.jacobian),
                             ptr(rho_dev), ptr(cells), ncells, dvol, 0, *center, ptr(quad), ptr(fail), st),
                   "corrected moments")
            total = base + (quad - region)
        if mode == "legacy_split":
            _check(_lib.call("igd_multipole_boundary", nx, ny, nz, ptr(x), ptr(y), ptr(z), ptr(base), multipole_order,
                             *center, ptr(bfield), 0, st), "boundary")
            if ncells > 0:
                _check(_lib.call("igd_multipole_cell_quadrature", nx, ny, nz, ptr(x), ptr(y), ptr(z), ptr(dg.jacobian),
                                 ptr(rho_dev), ptr(cells), ncells, dvol, 1, 0.0, 0.0, 0.0, ptr(corr), ptr(fail), st),
                       "legacy_split pass 1")
                s1 = corr.cpu().numpy()
                if s1[0] > 0.0:
                    cc = (float(s1[1] / s1[0]), float(s1[2] / s1[0]), float(s1[3] / s1[0]))
                    _check(_lib.call("igd_multipole_cell_quadrature", nx, ny, nz, ptr(x), ptr(y), ptr(z),
                                     ptr(dg.jacobian), ptr(rho_dev), ptr(cells), ncells, dvol, 2, *cc, ptr(corr),
                                     ptr(fail), st), "legacy_split pass 2")
                    _check(_lib.call("igd_multipole_boundary", nx, ny, nz, ptr(x), ptr(y), ptr(z), ptr(corr),
                                     multipole_order, *cc, ptr(bfield), 1, st), "boundary correction")
                    legacy_corr = (cc, corr.clone())
        else:
            _check(_lib.call("igd_multipole_boundary", nx, ny, nz, ptr(x), ptr(y), ptr(z), ptr(total), multipole_order,
                             *center, ptr(bfield), 0, st), "boundary")
        if int(fail.item()):
            raise RuntimeError("a corrected-moment quadratic fit was singular")
    else:
        _check(_lib.call("igd_multipole_boundary", nx, ny, nz, ptr(x), ptr(y), ptr(z), ptr(total), multipole_order,
                         *center, ptr(bfield), 0, st), "boundary")
    # split: -L u = 4 pi rho + L(b) inside, u = 0 on the faces
    Lb = hpsi_device(dg, bfield.reshape(1, -1), closure="production", kscale=1.0).reshape(-1)
    f = torch.empty_like(bfield)
    _check(_lib.call("igd_poisson_rhs", nx, ny, nz, ptr(rho_dev), ptr(Lb), ptr(f), st), "rhs")
    prec = _lib.IGD_PREC_MIXED if precision == "mixed" else _lib.IGD_PREC_FP64
    wsb = int(_lib.call("igd_poisson_workspace_bytes", prec, n))
    ws = dg.workspace("poisson", wsb)
    if start is not None and (start.numel() != n or start.dtype != torch.float64 or start.device != dev):
        raise ValueError(f"start must be an FP64 device field of {n} values on {dev}.")
    u = torch.zeros(n, dtype=torch.float64, device=dev) if start is None else start.reshape(-1).clone()
    info = (ctypes.c_double * 6)()
    if route == "cg":
        if not dg.monitor:
            raise ValueError("The JAX Hartree backend currently supports only the monitor-grid path.")
        kind = cg_preconditioner.strip().lower()
        kind = "diag" if kind == "jacobi" else kind
        if kind not in _PCG_KINDS:
            raise ValueError("cg_preconditioner must be `none`, `diag`, `jacobi`, `separable`, or `line`; "
                             f"received `{cg_preconditioner}`.")
        key = ("pcg", kind)
        pcd = dg._cache.get(key)
        if pcd is None:
            pcd = dg._cache[key] = _pcg_preconditioner(geom, kind, dev)
        d64, d32, axis = pcd
        wsb = int(_lib.call("igd_poisson_pcg_workspace_bytes", _PCG_KINDS[kind], nx, ny, nz))
        ws = dg.workspace("poisson_pcg", wsb)
        _check(_lib.call("igd_poisson_pcg", nx, ny, nz, ptr(dg.coeffs("fp64")), ptr(f), ptr(u), float(tolerance),
                         int(max_iterations), _PCG_KINDS[kind], ptr(d64), ptr(d32), int(axis), ptr(ws), wsb, info, st),
               "igd_poisson_pcg")
        v = torch.empty_like(u)
        _check(_lib.call("igd_poisson_compose", nx, ny, nz, ptr(bfield), ptr(u), ptr(v), st), "compose")
        return DevicePoissonSolution(v, bfield, u, f, Lb, total, base, int(info[0]), float(info[1]), float("nan"),
                                     1, center, legacy_corr)
    if route != "bicgstab":
        raise ValueError(f"route must be `bicgstab` or `cg`; received `{route}`.")
    if dg.monitor:
        c64, c32 = dg.coeffs("fp64"), (dg.coeffs("fp32") if prec == _lib.IGD_PREC_MIXED else None)
        kind = _lib.IGD_GRID_MONITOR
    else:
        c64, c32, kind = dg.axis_coeffs, dg.axis_coeffs, _lib.IGD_GRID_LEGACY
    stt = _lib.call("igd_poisson_solve" if start is None else "igd_poisson_solve_from", kind, prec, nx, ny, nz,
                    ptr(c64), ptr(c32), ptr(f), ptr(u),
                    float(tolerance), int(max_iterations), ptr(ws), wsb, info, st)
    if stt not in (_lib.IGD_OK, _lib.IGD_ERR_BREAKDOWN):
        _check(stt, "igd_poisson_solve")
    v = torch.empty_like(u)
    _check(_lib.call("igd_poisson_compose", nx, ny, nz, ptr(bfield), ptr(u), ptr(v), st), "compose")
    return DevicePoissonSolution(v, bfield, u, f, Lb, total, base, int(info[0]), float(info[5]), float(info[1]),
                                 int(info[3]), center, legacy_corr)


def _rms(a):
    a = np.asarray(a, dtype=np.float64)
    return 0.0 if a.size == 0 else float(np.sqrt(np.mean(a * a)))


def _normalize_mode(mode: str) -> str:
    m = mode.strip().lower()
    if m not in _VALID_MODES:
        raise ValueError("monitor_boundary_construction_mode must be `corrected_moments` or `legacy_split`; "
                         f"received `{mode}`.")
    return m


def solve_open_boundary_poisson(grid_geometry, rho, multipole_order: int = 2, tolerance: float = 1.0e-8,
                                max_iterations: int = 400, solver: str = "auto",
                                monitor_boundary_construction_mode: str = "corrected_moments", *,
                                precision: str = "fp64", route: str = "bicgstab",
                                cg_preconditioner: str = "none") -> OpenBoundaryPoissonResult:
    """GPU twin of ``open_boundary.py:1379`` (monitor and legacy grids)."""

    if solver not in {"auto", "scipy_bicgstab", "jacobi"}:
        raise ValueError("The current open-boundary Poisson slice supports solver=`auto`, `scipy_bicgstab`, "
                         f"or `jacobi`; received `{solver}`.")
    mode = _normalize_mode(monitor_boundary_construction_mode)
    for label in "xyz":  # monitor geometries name the axes logical_x, the legacy one x_logical
        coords = getattr(grid_geometry, f"logical_{label}", None)
        coords = getattr(grid_geometry, f"{label}_logical") if coords is None else coords
        d = np.diff(np.asarray(coords, dtype=np.float64))
        if not np.allclose(d, d[0]):  # open_boundary.py:112-119, same message
            raise ValueError(f"The current open-boundary Poisson slice expects a uniform logical {label}-axis.")
    require_cuda()
    density = validate_density_field(rho, grid_geometry)
    dg = device_grid(grid_geometry)
    rho_dev = torch.as_tensor(np.ascontiguousarray(density), device=dg.device).reshape(-1)
    sol = solve_poisson_device(dg, grid_geometry, rho_dev, multipole_order=multipole_order, tolerance=tolerance,
                               max_iterations=max_iterations, precision=precision, mode=mode, route=route,
                               cg_preconditioner=cg_preconditioner)
    shape = dg.shape
    potential = sol.potential.cpu().numpy().reshape(shape)
    bvals = sol.boundary.cpu().numpy().reshape(shape)
    q, p, Q = _moments_to_pq(sol.moments.cpu().numpy())
    monitor = is_monitor_geometry(grid_geometry)
    faces = np.ones(shape, dtype=bool)
    faces[1:-1, 1:-1, 1:-1] = False
    desc = ("Finite-domain Dirichlet boundary values from a free-space multipole expansion truncated at order "
            f"{multipole_order} about the grid reference center.")
    bdiag = None
    resp = None
    if monitor:
        desc += f" Monitor boundary construction mode: {mode}."
        bq, bp, bQ = _moments_to_pq(sol.baseline.cpu().numpy())
        c = sol.center
        dx = grid_geometry.x_points[faces] - c[0]
        dy = grid_geometry.y_points[faces] - c[1]
        dz = grid_geometry.z_points[faces] - c[2]
        r = np.sqrt(dx * dx + dy * dy + dz * dz)
        base_b = _face_potential_host(bq, bp, bQ, dx, dy, dz, r, multipole_order)
        corr_b = _face_potential_host(q, p, Q, dx, dy, dz, r, multipole_order)
        actual = bvals[faces]
        bdiag = OpenBoundaryBoundaryConstructionDiagnostics(
            baseline_total_charge=bq, baseline_dipole_moment=bp, baseline_quadrupole_tensor=bQ,
            correction_total_charge=q - bq, correction_dipole_moment=p - bp, correction_quadrupole_tensor=Q - bQ,
            boundary_value_correction_rms=_rms(actual - base_b),
            boundary_value_correction_max_abs=float(np.max(np.abs(actual - base_b), initial=0.0)),
            corrected_moment_boundary_rms_mismatch=_rms(actual - corr_b),
            corrected_moment_boundary_max_abs_mismatch=float(np.max(np.abs(actual - corr_b), initial=0.0)),
        )
        inner = ~faces
        Lb = sol.Lb.cpu().numpy().reshape(shape)
        rhs = sol.rhs.cpu().numpy().reshape(shape)
        Lv = hpsi_device(dg, sol.potential.reshape(1, -1), closure="production", kscale=1.0).cpu().numpy().reshape(shape)
        res = -Lv - 4.0 * math.pi * density
        resp = OpenBoundaryPoissonResponseDiagnostics(
            boundary_value_rms=_rms(actual), boundary_value_max_abs=float(np.max(np.abs(actual), initial=0.0)),
            boundary_source_laplacian_rms=_rms(Lb[inner]),
            boundary_source_laplacian_max_abs=float(np.max(np.abs(Lb[inner]), initial=0.0)),
            rhs_l2_norm=float(np.linalg.norm(rhs[inner])), rhs_max_abs=float(np.max(np.abs(rhs[inner]), initial=0.0)),
            interior_potential_rms=_rms(potential[inner]),
            interior_potential_max_abs=float(np.max(np.abs(potential[inner]), initial=0.0)),
            interior_poisson_residual_l2_norm=float(np.linalg.norm(res[inner])),
            interior_poisson_residual_max_abs=float(np.max(np.abs(res[inner]), initial=0.0)),
        )
    boundary = OpenBoundaryMultipoleBoundary(
        reference_center=sol.center, multipole_order=multipole_order, total_charge=q, dipole_moment=p,
        quadrupole_tensor=Q, boundary_values=bvals, description=desc, diagnostics=bdiag,
    )
    method = ("jax_cg_monitor" if route == "cg" else
              "gb300_bicgstab" + ("_monitor" if monitor else "") + ("_mixed_refinement" if precision == "mixed" else ""))
    return OpenBoundaryPoissonResult(
        rho=density, potential=potential, boundary_condition=boundary, solver_method=method,
        solver_iterations=sol.iterations, residual_max=sol.residual_max,
        description="Finite-domain Poisson solve on the GB300 with free-space multipole Dirichlet boundary data.",
        response_diagnostics=resp,
    )


_VALID_CG_IMPLS = {"baseline", "jax_loop"}
_VALID_CG_PRECONDITIONERS = {"none", "diag", "jacobi", "separable", "line"}
_VALID_LINE_IMPLS = {"baseline", "optimized"}


def validate_hartree_solver_options(*, backend: str = "python", cg_impl: str = "baseline",
                                    cg_preconditioner: str = "none", line_preconditioner_impl: str = "baseline"):
    """Normalised Hartree-solver options, rejecting unknown values with the reference's
    messages (``poisson/hartree.py:66-72``, ``poisson/poisson_jax.py:204-239``); ``jacobi``
    is the ``diag`` preconditioner.  Returns (backend, cg_impl, preconditioner, line_impl).
    Every accepted combination runs the same GPU BiCGSTAB solve (one fixed point)."""

    nb = backend.strip().lower()
    if nb not in {"python", "jax", "gb300"}:
        raise ValueError(f"backend must be `python` or `jax`; received `{backend}`.")
    impl = cg_impl.strip().lower()
    if impl not in _VALID_CG_IMPLS:
        raise ValueError(f"cg_impl must be `baseline` or `jax_loop`; received `{cg_impl}`.")
    pre = cg_preconditioner.strip().lower()
    if pre not in _VALID_CG_PRECONDITIONERS:
        raise ValueError("cg_preconditioner must be `none`, `diag`, `jacobi`, `separable`, or `line`; "
                         f"received `{cg_preconditioner}`.")
    if pre == "jacobi":
        pre = "diag"
    line = line_preconditioner_impl.strip().lower()
    if line not in _VALID_LINE_IMPLS:
        raise ValueError(f"line_preconditioner_impl must be `baseline` or `optimized`; "
                         f"received `{line_preconditioner_impl}`.")
    return nb, impl, pre, line


def solve_hartree_potential(grid_geometry, rho, multipole_order: int = 2, tolerance: float = 1.0e-8,
                            max_iterations: int = 400, solver: str = "auto", backend: str = "python",
                            use_jax_cached_operator: bool = False, cg_impl: str = "baseline",
                            cg_preconditioner: str = "none", line_preconditioner_impl: str = "baseline",
                            monitor_boundary_construction_mode: str = "corrected_moments", *,
                            precision: str = "fp64") -> OpenBoundaryPoissonResult:
    """GPU twin of ``poisson/hartree.py:47-98``.  The python backend runs the GPU BiCGSTAB
    (relative 2-norm rule, FP64 or mixed); the jax backend runs the reference's JAX route on
    the GPU: preconditioned CG from zero to max |r| < ``tolerance`` with ``cg_preconditioner``
    (``poisson/poisson_jax.py:675-750``; both ``cg_impl`` forms are the same iteration)."""

    nb, _, pre, _ = validate_hartree_solver_options(backend=backend, cg_impl=cg_impl,
                                                    cg_preconditioner=cg_preconditioner,
                                                    line_preconditioner_impl=line_preconditioner_impl)
    if nb == "jax" and not is_monitor_geometry(grid_geometry):
        raise ValueError("The JAX Hartree backend currently supports only the monitor-grid path.")
    return solve_open_boundary_poisson(grid_geometry, rho, multipole_order=multipole_order, tolerance=tolerance,
                                       max_iterations=max_iterations, solver=solver,
                                       monitor_boundary_construction_mode=monitor_boundary_construction_mode,
                                       precision=precision, route="cg" if nb == "jax" else "bicgstab",
                                       cg_preconditioner=pre)


def _potential_array(grid_geometry, hartree_potential):
    """``poisson/hartree.py:100-114``: a solve result, or a field checked against the grid."""

    if isinstance(hartree_potential, OpenBoundaryPoissonResult):
        return hartree_potential.potential, hartree_potential
    field = validate_orbital_field(hartree_potential, grid_geometry, name="hartree_potential")
    return np.asarray(field, dtype=np.float64), None


def evaluate_hartree_energy(rho, grid_geometry, hartree_potential) -> float:
    """E_H = 1/2 sum rho v W (FP64 device reduction)."""

    density = validate_density_field(rho, grid_geometry)
    potential, _ = _potential_array(grid_geometry, hartree_potential)
    dg = device_grid(grid_geometry)
    a = torch.as_tensor(np.ascontiguousarray(density), device=dg.device).reshape(-1)
    b = torch.as_tensor(np.ascontiguousarray(potential, dtype=np.float64), device=dg.device).reshape(-1)
    out = torch.zeros(1, dtype=torch.float64, device=dg.device)
    _check(_lib.call("igd_weighted_sum", _lib.IGD_F64, dg.n, ptr(a), ptr(b), ptr(dg.cell_volumes), ptr(out),
                     stream_ptr()), "igd_weighted_sum")
    return 0.5 * float(out.item())


def build_hartree_action(psi, grid_geometry, hartree_potential):
    field = validate_orbital_field(psi, grid_geometry)
    potential, _ = _potential_array(grid_geometry, hartree_potential)
    return potential * field


def evaluate_hartree_terms(psi, grid_geometry, rho, hartree_potential=None, multipole_order: int = 2,
                           tolerance: float = 1.0e-8, max_iterations: int = 400, solver: str = "auto",
                           ) -> HartreeEvaluation:
    density = validate_density_field(rho, grid_geometry)
    if hartree_potential is None:
        res = solve_hartree_potential(grid_geometry, density, multipole_order, tolerance, max_iterations, solver)
        potential = res.potential
    else:
        potential, res = _potential_array(grid_geometry, hartree_potential)
    return HartreeEvaluation(rho=density, potential=potential,
                             action=build_hartree_action(psi, grid_geometry, potential),
                             energy=evaluate_hartree_energy(density, grid_geometry, potential), poisson_result=res)
