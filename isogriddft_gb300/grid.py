"""Host-side grid construction (legacy sinh grid and monitor A-grid).

Grid construction is set-up work, done once per geometry, and the north-star
contract asks for it to be bit-exact with the reference.  Bit-exactness in
IEEE double needs the same elementwise operations in the same order, so the
arithmetic of every step below follows the reference builder one to one:

* legacy separable sinh mapping: ``grid/mapping.py:33-135``,
  ``grid/geometry.py:34-104``, defaults ``grid/__init__.py:39-101``;
* monitor A-grid: monitor field ``grid/monitor_geometry.py:51-113``,
  smoothing ``:116-135``, weighted-harmonic damped Jacobi ``:268-321``,
  covariant basis / metric / Jacobian ``:324-373``, backtracking ``:376-396``,
  quality report ``:425-478``, driver ``:481-577``; specs and element
  parameters ``grid/monitor_builder.py:53-228``.

The dataclasses keep the reference field names so the GB300 operators accept
either a reference geometry object or one built here.  The device-side
generator for large grids lives in :mod:`isogriddft_gb300.grid_device`.
"""

from __future__ import annotations

import os
from dataclasses import dataclass, replace

import numpy as np

from .config import H2_BENCHMARK_CASE, BenchmarkCase

Coordinate3D = tuple[float, float, float]
BoxBounds3D = tuple[tuple[float, float], tuple[float, float], tuple[float, float]]

# --------------------------------------------------------------------------
# Legacy separable sinh grid
# --------------------------------------------------------------------------


@dataclass(frozen=True)
class AxisStretchSpec:
    label: str
    lower_offset: float
    upper_offset: float
    stretch: float

    def __post_init__(self) -> None:
        if self.lower_offset >= self.upper_offset:
            raise ValueError("Axis bounds must satisfy lower_offset < upper_offset.")
        if not (self.lower_offset < 0.0 < self.upper_offset):
            raise ValueError("The reference center must lie inside the axis bounds.")
        if self.stretch < 0.0:
            raise ValueError("Axis stretch must be non-negative.")


@dataclass(frozen=True)
class StructuredGridSpec:
    name: str
    description: str
    nx: int
    ny: int
    nz: int
    reference_center: Coordinate3D
    unit: str
    x_axis: AxisStretchSpec
    y_axis: AxisStretchSpec
    z_axis: AxisStretchSpec

    def __post_init__(self) -> None:
        if min(self.nx, self.ny, self.nz) < 2:
            raise ValueError("Each grid direction must have at least two points.")

    @property
    def shape(self) -> tuple[int, int, int]:
        return (self.nx, self.ny, self.nz)


@dataclass(frozen=True)
class StructuredGridGeometry:
    spec: StructuredGridSpec
    x_logical: np.ndarray
    y_logical: np.ndarray
    z_logical: np.ndarray
    x_coordinates: np.ndarray
    y_coordinates: np.ndarray
    z_coordinates: np.ndarray
    x_points: np.ndarray
    y_points: np.ndarray
    z_points: np.ndarray
    x_point_jacobian: np.ndarray
    y_point_jacobian: np.ndarray
    z_point_jacobian: np.ndarray
    point_jacobian: np.ndarray
    cell_widths_x: np.ndarray
    cell_widths_y: np.ndarray
    cell_widths_z: np.ndarray
    cell_volumes: np.ndarray


H2_DEFAULT_GRID_SHAPE = (51, 51, 51)
H2_DEFAULT_GRID_HALF_EXTENTS_BOHR = (8.0, 8.0, 10.0)
H2_DEFAULT_GRID_STRETCH = (2.5, 2.5, 2.8)


def _sinh_axis(n: int, axis: AxisStretchSpec, center: float):
    """Logical [-1, 1] axis, its sinh-stretched physical image and dx/du."""

    if n < 2:
        raise ValueError("At least two logical points are required per axis.")
    u = np.linspace(-1.0, 1.0, n, dtype=np.float64)
    a = np.abs(u)
    s = axis.stretch
    if s == 0.0:
        frac, dfrac = a, np.ones_like(a)
    else:
        frac = np.sinh(s * a) / np.sinh(s)
        dfrac = s * np.cosh(s * a) / np.sinh(s)
    neg = u < 0.0
    left, right = -axis.lower_offset, axis.upper_offset
    x = np.empty_like(u)
    x[neg] = center - left * frac[neg]
    x[~neg] = center + right * frac[~neg]
    h = np.empty_like(u)
    h[neg] = left * dfrac[neg]
    h[~neg] = right * dfrac[~neg]
    return u, x, h


def _point_centred_widths(points: np.ndarray) -> np.ndarray:
    p = np.asarray(points, dtype=np.float64)
    if p.ndim != 1 or p.size < 2 or not np.all(np.diff(p) > 0.0):
        raise ValueError("Cell edges require a strictly increasing 1D axis.")
    edges = np.empty(p.size + 1, dtype=np.float64)
    edges[1:-1] = 0.5 * (p[1:] + p[:-1])
    edges[0] = p[0] - 0.5 * (p[1] - p[0])
    edges[-1] = p[-1] + 0.5 * (p[-1] - p[-2])
    return np.diff(edges)


def build_grid_geometry(spec: StructuredGridSpec) -> StructuredGridGeometry:
    cx, cy, cz = spec.reference_center
    ux, xc, hx = _sinh_axis(spec.nx, spec.x_axis, cx)
    uy, yc, hy = _sinh_axis(spec.ny, spec.y_axis, cy)
    uz, zc, hz = _sinh_axis(spec.nz, spec.z_axis, cz)
    xp, yp, zp = np.meshgrid(xc, yc, zc, indexing="ij")
    wx, wy, wz = _point_centred_widths(xc), _point_centred_widths(yc), _point_centred_widths(zc)
    return StructuredGridGeometry(
        spec=spec,
        x_logical=ux, y_logical=uy, z_logical=uz,
        x_coordinates=xc, y_coordinates=yc, z_coordinates=zc,
        x_points=xp, y_points=yp, z_points=zp,
        x_point_jacobian=hx, y_point_jacobian=hy, z_point_jacobian=hz,
        point_jacobian=hx[:, None, None] * hy[None, :, None] * hz[None, None, :],
        cell_widths_x=wx, cell_widths_y=wy, cell_widths_z=wz,
        cell_volumes=wx[:, None, None] * wy[None, :, None] * wz[None, None, :],
    )


def compute_geometry_reference_center(case: BenchmarkCase) -> Coordinate3D:
    atoms = case.geometry.atoms
    if not atoms:
        raise ValueError("Benchmark geometry must contain at least one atom.")
    n = float(len(atoms))
    return (
        sum(a.position[0] for a in atoms) / n,
        sum(a.position[1] for a in atoms) / n,
        sum(a.position[2] for a in atoms) / n,
    )


def build_default_h2_grid_spec(
    case: BenchmarkCase = H2_BENCHMARK_CASE,
    shape: tuple[int, int, int] = H2_DEFAULT_GRID_SHAPE,
) -> StructuredGridSpec:
    (hx, hy, hz), (sx, sy, sz) = H2_DEFAULT_GRID_HALF_EXTENTS_BOHR, H2_DEFAULT_GRID_STRETCH
    return StructuredGridSpec(
        name="h2_r1p4_structured_grid",
        description="Separable per-axis sinh-stretched structured grid about the molecular centre.",
        nx=shape[0], ny=shape[1], nz=shape[2],
        reference_center=compute_geometry_reference_center(case),
        unit=case.geometry.unit,
        x_axis=AxisStretchSpec("x", -hx, hx, sx),
        y_axis=AxisStretchSpec("y", -hy, hy, sy),
        z_axis=AxisStretchSpec("z", -hz, hz, sz),
    )


def build_default_h2_grid_geometry(
    case: BenchmarkCase = H2_BENCHMARK_CASE,
    shape: tuple[int, int, int] = H2_DEFAULT_GRID_SHAPE,
) -> StructuredGridGeometry:
    return build_grid_geometry(build_default_h2_grid_spec(case, shape))


# --------------------------------------------------------------------------
# Monitor A-grid
# --------------------------------------------------------------------------


@dataclass(frozen=True)
class NearCoreElementParameters:
    element: str
    near_core_radius: float
    local_radius: float
    projector_radius: float
    patch_radius: float
    kinetic_weight: float
    local_weight: float
    projector_weight: float
    kinetic_exponent: float
    local_exponent: float
    projector_exponent: float
    monitor_cap: float

    def __post_init__(self) -> None:
        for name in ("near_core_radius", "local_radius", "projector_radius", "patch_radius"):
            if getattr(self, name) <= 0.0:
                raise ValueError(f"{name} must be positive.")
        if min(self.kinetic_exponent, self.local_exponent, self.projector_exponent) <= 0.0:
            raise ValueError("All monitor exponents must be positive.")
        if self.monitor_cap <= 1.0:
            raise ValueError("monitor_cap must be larger than 1.")


@dataclass(frozen=True)
class MonitorPatchInterface:
    atom_index: int
    element: str
    center: Coordinate3D
    patch_radius: float
    purposes: tuple[str, ...]
    relation_to_main_grid: str
    implemented_purposes: tuple[str, ...] = ()
    implemented: bool = False


@dataclass(frozen=True)
class AtomicMonitorContribution:
    atom_index: int
    element: str
    position: Coordinate3D
    parameters: NearCoreElementParameters
    kinetic_component: np.ndarray
    local_component: np.ndarray
    projector_component: np.ndarray
    raw_total: np.ndarray
    capped_total: np.ndarray


@dataclass(frozen=True)
class GlobalMonitorField:
    values: np.ndarray
    raw_values: np.ndarray
    atomic_contributions: tuple[AtomicMonitorContribution, ...]
    baseline_value: float
    minimum_value: float
    maximum_value: float


@dataclass(frozen=True)
class MonitorGridSpec:
    name: str
    description: str
    nx: int
    ny: int
    nz: int
    unit: str
    box_bounds: BoxBounds3D
    logical_bounds: BoxBounds3D
    element_parameters: dict
    harmonic_outer_iterations: int
    harmonic_inner_iterations: int
    harmonic_tolerance: float
    harmonic_relaxation: float
    inner_relaxation: float
    monitor_smoothing: float

    def __post_init__(self) -> None:
        if min(self.nx, self.ny, self.nz) < 3:
            raise ValueError("Monitor grids require at least three points per direction.")
        if self.harmonic_outer_iterations <= 0 or self.harmonic_inner_iterations <= 0:
            raise ValueError("Harmonic iteration counts must be positive.")
        if self.harmonic_tolerance <= 0.0:
            raise ValueError("harmonic_tolerance must be positive.")
        if not (0.0 < self.harmonic_relaxation <= 1.0) or not (0.0 < self.inner_relaxation <= 1.0):
            raise ValueError("relaxation factors must satisfy 0 < value <= 1.")
        if not (0.0 <= self.monitor_smoothing < 1.0):
            raise ValueError("monitor_smoothing must satisfy 0 <= value < 1.")
        if not self.element_parameters:
            raise ValueError("element_parameters must not be empty.")

    @property
    def shape(self) -> tuple[int, int, int]:
        return (self.nx, self.ny, self.nz)


@dataclass(frozen=True)
class MonitorGridQualityReport:
    min_jacobian: float
    max_jacobian: float
    has_nonpositive_jacobian: bool
    min_cell_volume: float
    max_cell_volume: float
    mean_near_atom_spacing: float
    mean_far_field_spacing: float
    near_to_far_spacing_ratio: float


@dataclass(frozen=True)
class MonitorGridGeometry:
    spec: MonitorGridSpec
    logical_x: np.ndarray
    logical_y: np.ndarray
    logical_z: np.ndarray
    x_points: np.ndarray
    y_points: np.ndarray
    z_points: np.ndarray
    covariant_basis: np.ndarray
    jacobian: np.ndarray
    metric_tensor: np.ndarray
    inverse_metric_tensor: np.ndarray
    cell_volumes: np.ndarray
    spacing_x: np.ndarray
    spacing_y: np.ndarray
    spacing_z: np.ndarray
    spacing_measure: np.ndarray
    monitor_field: GlobalMonitorField
    patch_interfaces: tuple[MonitorPatchInterface, ...]
    quality_report: MonitorGridQualityReport


_MONITOR_BASELINE = 1.0
_JACOBIAN_FLOOR = 1.0e-12
_UNIT_CUBE = ((0.0, 1.0), (0.0, 1.0), (0.0, 1.0))
H2_MONITOR_LOCAL_PATCH_BASELINE_SHAPE = (83, 83, 101)
H2_MONITOR_LOCAL_PATCH_BASELINE_BOX_HALF_EXTENTS_BOHR = (8.0, 8.0, 10.0)
H2_MONITOR_LOCAL_PATCH_BASELINE_WEIGHT_SCALE = 4.0
H2_MONITOR_LOCAL_PATCH_BASELINE_RADIUS_SCALE = 0.70

# GTH-inspired seeds: (ionic charge, rloc, local coefficients, projector radii).
_GTH_SEEDS = {
    "H": (1, 0.2, (-4.1802368, 0.72507482), ()),
    "C": (4, 0.34883045, (-8.5137711, 1.22843203), (0.30455321,)),
    "N": (5, 0.28917923, (-12.23481988, 1.76640728), (0.25660487,)),
    "O": (6, 0.24762086, (-16.58031797, 2.39570092), (0.22178614,)),
}


def build_default_near_core_element_parameters(case: BenchmarkCase) -> dict:
    """Element parameters derived from GTH seeds (``grid/monitor_builder.py:63-99``)."""

    out: dict = {}
    for atom in case.geometry.atoms:
        el = atom.element
        if el in out:
            continue
        if el not in _GTH_SEEDS:
            raise ValueError(f"The monitor-grid core supports only H/C/N/O seeds; received `{el}`.")
        zion, rloc, coeffs, prad = _GTH_SEEDS[el]
        rnl = max(prad, default=1.5 * rloc)
        out[el] = NearCoreElementParameters(
            element=el,
            near_core_radius=max(0.35, 1.8 * rloc + 0.15),
            local_radius=max(0.45, 2.5 * rloc + 0.15),
            projector_radius=max(0.55, 2.4 * rnl),
            patch_radius=max(1.0, 4.0 * max(rloc, rnl) + 0.25),
            kinetic_weight=1.5 + 0.9 * zion,
            local_weight=2.0 + 1.1 * zion + 0.05 * sum(abs(c) for c in coeffs),
            projector_weight=0.45 * zion if prad else 0.0,
            kinetic_exponent=2.0,
            local_exponent=4.0,
            projector_exponent=2.0,
            monitor_cap=4.0 + 0.8 * zion,
        )
    return out


def build_h2_local_patch_development_element_parameters() -> dict:
    base = build_default_near_core_element_parameters(H2_BENCHMARK_CASE)
    rs, ws = H2_MONITOR_LOCAL_PATCH_BASELINE_RADIUS_SCALE, H2_MONITOR_LOCAL_PATCH_BASELINE_WEIGHT_SCALE
    return {
        el: replace(
            p,
            near_core_radius=p.near_core_radius * rs,
            local_radius=p.local_radius * rs,
            kinetic_weight=p.kinetic_weight * ws,
            local_weight=p.local_weight * ws,
        )
        for el, p in base.items()
    }


def build_two_peak_element_parameters(
    elements=("H",), amplitude: float = 4.0, width: float = 0.5, cap: float = 1.0e6
) -> dict:
    """Monitor parameters with a single Gaussian refinement peak per atom.

    Used for the 128^3 operator benchmark: ``kinetic_weight`` = amplitude,
    ``near_core_radius`` = width, exponent 2, no local/projector terms and a cap
    so large that the capped monitor equals the raw one to first order.
    """

    return {
        el: NearCoreElementParameters(
            element=el, near_core_radius=width, local_radius=1.0, projector_radius=1.0,
            patch_radius=1.0, kinetic_weight=amplitude, local_weight=0.0, projector_weight=0.0,
            kinetic_exponent=2.0, local_exponent=4.0, projector_exponent=2.0, monitor_cap=cap,
        )
        for el in elements
    }


def _default_box_half_extents(case: BenchmarkCase, params: dict) -> Coordinate3D:
    c = compute_geometry_reference_center(case)
    support = max(max(p.patch_radius, p.local_radius, p.projector_radius) for p in params.values())
    reach = [0.0, 0.0, 0.0]
    for atom in case.geometry.atoms:
        for a in range(3):
            reach[a] = max(reach[a], abs(atom.position[a] - c[a]))
    pad = max(6.0, 4.0 * support)
    return (reach[0] + pad, reach[1] + pad, reach[2] + pad)


def build_monitor_grid_spec_for_case(
    case: BenchmarkCase,
    *,
    shape: tuple[int, int, int] | None = None,
    box_half_extents: Coordinate3D | None = None,
    element_parameters: dict | None = None,
    harmonic_outer_iterations: int = 6,
    harmonic_inner_iterations: int = 180,
    harmonic_tolerance: float = 5.0e-5,
    harmonic_relaxation: float = 0.55,
    inner_relaxation: float = 0.82,
    monitor_smoothing: float = 0.18,
) -> MonitorGridSpec:
    params = element_parameters or build_default_near_core_element_parameters(case)
    if shape is None:
        shape = (29, 29, 29) if len(case.geometry.atoms) <= 2 else (31, 31, 31)
    if box_half_extents is None:
        box_half_extents = _default_box_half_extents(case, params)
    c = compute_geometry_reference_center(case)
    hx, hy, hz = box_half_extents
    return MonitorGridSpec(
        name=f"{case.geometry.name.lower()}_monitor_grid",
        description="Atom-centred monitor-function grid from a weighted harmonic map.",
        nx=shape[0], ny=shape[1], nz=shape[2],
        unit=case.geometry.unit,
        box_bounds=((c[0] - hx, c[0] + hx), (c[1] - hy, c[1] + hy), (c[2] - hz, c[2] + hz)),
        logical_bounds=_UNIT_CUBE,
        element_parameters=params,
        harmonic_outer_iterations=harmonic_outer_iterations,
        harmonic_inner_iterations=harmonic_inner_iterations,
        harmonic_tolerance=harmonic_tolerance,
        harmonic_relaxation=harmonic_relaxation,
        inner_relaxation=inner_relaxation,
        monitor_smoothing=monitor_smoothing,
    )


def _uniform_step(coords: np.ndarray) -> float:
    d = np.diff(np.asarray(coords, dtype=np.float64))
    if not np.allclose(d, d[0]):
        raise ValueError("The monitor-grid generator expects uniform logical coordinates.")
    return float(d[0])


def evaluate_global_monitor_field(case, spec, x_points, y_points, z_points) -> GlobalMonitorField:
    """Sum of capped per-atom monitor terms on the current coordinates."""

    raw = np.full(spec.shape, _MONITOR_BASELINE, dtype=np.float64)
    val = np.full(spec.shape, _MONITOR_BASELINE, dtype=np.float64)
    parts = []
    for idx, atom in enumerate(case.geometry.atoms):
        p = spec.element_parameters[atom.element]
        dx = x_points - atom.position[0]
        dy = y_points - atom.position[1]
        dz = z_points - atom.position[2]
        r = np.sqrt(dx * dx + dy * dy + dz * dz, dtype=np.float64)
        kin = p.kinetic_weight * np.exp(-np.power(r / p.near_core_radius, p.kinetic_exponent))
        loc = p.local_weight / (1.0 + np.power(r / p.local_radius, p.local_exponent))
        if p.projector_weight > 0.0:
            prj = p.projector_weight * np.exp(-np.power(r / p.projector_radius, p.projector_exponent))
        else:
            prj = np.zeros(spec.shape, dtype=np.float64)
        atom_raw = kin + loc + prj
        atom_cap = p.monitor_cap * (1.0 - np.exp(-atom_raw / p.monitor_cap))
        raw += atom_raw
        val += atom_cap
        parts.append(AtomicMonitorContribution(idx, atom.element, atom.position, p, kin, loc, prj, atom_raw, atom_cap))
    return GlobalMonitorField(
        values=val, raw_values=raw, atomic_contributions=tuple(parts),
        baseline_value=_MONITOR_BASELINE, minimum_value=float(np.min(val)), maximum_value=float(np.max(val)),
    )


def _smooth(values: np.ndarray, smoothing: float) -> np.ndarray:
    m = np.asarray(values, dtype=np.float64)
    if smoothing <= 0.0:
        return m
    c = (slice(1, -1),) * 3
    avg = (
        m[c] + m[:-2, 1:-1, 1:-1] + m[2:, 1:-1, 1:-1] + m[1:-1, :-2, 1:-1]
        + m[1:-1, 2:, 1:-1] + m[1:-1, 1:-1, :-2] + m[1:-1, 1:-1, 2:]
    ) / 7.0
    out = np.array(m, copy=True)
    out[c] = (1.0 - smoothing) * m[c] + smoothing * avg
    return np.maximum(out, _MONITOR_BASELINE)


def _face_mask(shape) -> np.ndarray:
    mask = np.ones(shape, dtype=bool)
    mask[1:-1, 1:-1, 1:-1] = False
    return mask


def _slab_pool():
    """Thread pool for the slab-parallel host sweeps (NumPy releases the GIL in its loops)."""

    global _POOL
    if _POOL is None:
        from concurrent.futures import ThreadPoolExecutor

        _POOL = ThreadPoolExecutor(max_workers=max(1, min(32, os.cpu_count() or 1)))
    return _POOL


_POOL = None


def _harmonic_solve(monitor, hx, hy, hz, fixed, start, sweeps, tol, relax) -> np.ndarray:
    """Damped-Jacobi sweeps for div(M grad X) = 0 with Dirichlet faces.

    The sweep is the reference's (``grid/monitor_geometry.py:268-321``, same elementwise
    operations in the same order, so the result is bit-identical), run over x-slabs of a
    few planes by a thread pool into a second buffer: every interior value of a sweep
    depends only on the previous sweep, and max|change| is an exact reduction.
    """

    m = np.asarray(monitor, dtype=np.float64)
    X = np.asarray(start, dtype=np.float64).copy()
    faces = _face_mask(m.shape)
    X[faces] = fixed[faces]
    c = (slice(1, -1),) * 3
    mc = m[c]
    wxm = 0.5 * (mc + m[:-2, 1:-1, 1:-1]) / (hx * hx)
    wxp = 0.5 * (mc + m[2:, 1:-1, 1:-1]) / (hx * hx)
    wym = 0.5 * (mc + m[1:-1, :-2, 1:-1]) / (hy * hy)
    wyp = 0.5 * (mc + m[1:-1, 2:, 1:-1]) / (hy * hy)
    wzm = 0.5 * (mc + m[1:-1, 1:-1, :-2]) / (hz * hz)
    wzp = 0.5 * (mc + m[1:-1, 1:-1, 2:]) / (hz * hz)
    wsum = wxm + wxp + wym + wyp + wzm + wzp
    wxm, wxp, wym, wyp, wzm, wzp, wsum = (a[..., None] for a in (wxm, wxp, wym, wyp, wzm, wzp, wsum))
    nxt = X.copy()
    n_int = m.shape[0] - 2
    step = max(1, min(4, n_int // 8 or 1))
    slabs = [(lo, min(lo + step, n_int)) for lo in range(0, n_int, step)]
    keep = 1.0 - relax
    # per-slab scratch, reused every sweep (in-place ufuncs round exactly like the
    # expression form: ((((a + b) + c) + d) + e) + f, then / wsum)
    inner = (X.shape[1] - 2, X.shape[2] - 2, X.shape[3])
    scratch = {b: (np.empty((b[1] - b[0],) + inner), np.empty((b[1] - b[0],) + inner)) for b in slabs}

    def sweep_slab(src, dst, lo, hi):
        s = slice(lo, hi)
        xs = slice(lo + 1, hi + 1)
        cand, t = scratch[(lo, hi)]
        np.multiply(wxm[s], src[lo:hi, 1:-1, 1:-1, :], out=cand)
        for w, v in ((wxp, src[lo + 2:hi + 2, 1:-1, 1:-1, :]), (wym, src[xs, :-2, 1:-1, :]),
                     (wyp, src[xs, 2:, 1:-1, :]), (wzm, src[xs, 1:-1, :-2, :]), (wzp, src[xs, 1:-1, 2:, :])):
            np.multiply(w[s], v, out=t)
            np.add(cand, t, out=cand)
        np.divide(cand, wsum[s], out=cand)
        old = src[xs, 1:-1, 1:-1, :]
        new = dst[xs, 1:-1, 1:-1, :]
        np.multiply(relax, cand, out=cand)
        np.multiply(keep, old, out=new)
        np.add(new, cand, out=new)
        np.subtract(new, old, out=t)
        np.abs(t, out=t)
        return float(np.max(t)) if t.size else 0.0

    pool = _slab_pool()
    for _ in range(sweeps):
        changes = list(pool.map(lambda b: sweep_slab(X, nxt, *b), slabs))
        X, nxt = nxt, X
        if max(changes, default=0.0) < tol:
            break
    return X


def _geometry_from_coordinates(lx, ly, lz, X):
    basis = np.zeros(X.shape[:-1] + (3, 3), dtype=np.float64)
    for comp in range(3):
        basis[..., 0, comp] = np.gradient(X[..., comp], lx, axis=0, edge_order=2)
        basis[..., 1, comp] = np.gradient(X[..., comp], ly, axis=1, edge_order=2)
        basis[..., 2, comp] = np.gradient(X[..., comp], lz, axis=2, edge_order=2)
    hx, hy, hz = _uniform_step(lx), _uniform_step(ly), _uniform_step(lz)
    metric = np.empty_like(basis)
    inv_metric = np.empty_like(basis)
    jac = np.empty(basis.shape[:3], dtype=np.float64)
    spacing = np.empty(basis.shape[:3] + (3,), dtype=np.float64)

    def pointwise(lo, hi):
        # per-point 3x3 algebra: every output point depends on its own basis only, so
        # x-slabs run in parallel with results identical to one whole-array call
        b = basis[lo:hi]
        g = np.einsum("...ai,...bi->...ab", b, b)
        metric[lo:hi] = g
        inv_metric[lo:hi] = np.linalg.inv(g)
        jac[lo:hi] = np.linalg.det(b)
        spacing[lo:hi, ..., 0] = np.linalg.norm(b[..., 0, :], axis=-1) * hx
        spacing[lo:hi, ..., 1] = np.linalg.norm(b[..., 1, :], axis=-1) * hy
        spacing[lo:hi, ..., 2] = np.linalg.norm(b[..., 2, :], axis=-1) * hz

    nx = basis.shape[0]
    list(_slab_pool().map(lambda lo: pointwise(lo, min(lo + 2, nx)), range(0, nx, 2)))
    vol = jac * hx * hy * hz
    return basis, jac, metric, inv_metric, vol, spacing


def _backtrack(cur, solved, lx, ly, lz, relax):
    alpha = relax
    while alpha >= 1.0e-3:
        trial = cur + alpha * (solved - cur)
        _, jac, *_ = _geometry_from_coordinates(lx, ly, lz, trial)
        if float(np.min(jac)) > _JACOBIAN_FLOOR:
            return trial
        alpha *= 0.5
    return np.asarray(cur, dtype=np.float64)


def _patch_interfaces(case, params):
    return tuple(
        MonitorPatchInterface(
            atom_index=i, element=a.element, center=a.position,
            patch_radius=params[a.element].patch_radius,
            purposes=("local_gth", "nonlocal_projector", "near_core_integration"),
            implemented_purposes=("local_gth", "near_core_integration"),
            relation_to_main_grid="Atom-anchored auxiliary patch sampling main-grid fields.",
            implemented=True,
        )
        for i, a in enumerate(case.geometry.atoms)
    )


def _quality(spec, xp, yp, zp, jac, vol, spacing, monitor) -> MonitorGridQualityReport:
    nearest = np.full(spec.shape, np.inf, dtype=np.float64)
    near = np.zeros(spec.shape, dtype=bool)
    max_patch = 0.0
    for part in monitor.atomic_contributions:
        dx = xp - part.position[0]
        dy = yp - part.position[1]
        dz = zp - part.position[2]
        r = np.sqrt(dx * dx + dy * dy + dz * dz, dtype=np.float64)
        nearest = np.minimum(nearest, r)
        thr = max(part.parameters.patch_radius, part.parameters.local_radius, part.parameters.near_core_radius)
        near |= r <= thr
        max_patch = max(max_patch, part.parameters.patch_radius)
    spans = np.array([b[1] - b[0] for b in spec.box_bounds], dtype=np.float64)
    far = nearest >= max(3.0 * max_patch, 0.35 * float(np.min(spans)))
    if not np.any(far):
        far = nearest >= np.quantile(nearest, 0.75)
    mn = float(np.mean(spacing[near])) if np.any(near) else float("nan")
    mf = float(np.mean(spacing[far])) if np.any(far) else float("nan")
    ratio = mn / mf if np.isfinite(mn) and np.isfinite(mf) and mf > 0.0 else float("nan")
    return MonitorGridQualityReport(
        min_jacobian=float(np.min(jac)), max_jacobian=float(np.max(jac)),
        has_nonpositive_jacobian=bool(np.any(jac <= 0.0)),
        min_cell_volume=float(np.min(vol)), max_cell_volume=float(np.max(vol)),
        mean_near_atom_spacing=mn, mean_far_field_spacing=mf, near_to_far_spacing_ratio=float(ratio),
    )


def assemble_monitor_geometry(case, spec, lx, ly, lz, X) -> MonitorGridGeometry:
    """Final geometry record from converged physical coordinates ``X[..., 3]``."""

    monitor = evaluate_global_monitor_field(case, spec, X[..., 0], X[..., 1], X[..., 2])
    basis, jac, metric, inv_metric, vol, spacings = _geometry_from_coordinates(lx, ly, lz, X)
    measure = np.mean(spacings, axis=-1)
    return MonitorGridGeometry(
        spec=spec, logical_x=lx, logical_y=ly, logical_z=lz,
        x_points=np.asarray(X[..., 0], dtype=np.float64),
        y_points=np.asarray(X[..., 1], dtype=np.float64),
        z_points=np.asarray(X[..., 2], dtype=np.float64),
        covariant_basis=basis, jacobian=jac, metric_tensor=metric, inverse_metric_tensor=inv_metric,
        cell_volumes=vol, spacing_x=spacings[..., 0], spacing_y=spacings[..., 1], spacing_z=spacings[..., 2],
        spacing_measure=measure, monitor_field=monitor,
        patch_interfaces=_patch_interfaces(case, spec.element_parameters),
        quality_report=_quality(spec, X[..., 0], X[..., 1], X[..., 2], jac, vol, measure, monitor),
    )


def monitor_box_axes(spec: MonitorGridSpec):
    """Logical axes and the initial (uniform box) physical coordinates."""

    def axis(b, n):
        lo, hi = b
        if hi <= lo:
            raise ValueError("Logical axis bounds must satisfy upper > lower.")
        return np.linspace(lo, hi, n, dtype=np.float64)

    lx, ly, lz = (axis(spec.logical_bounds[a], spec.shape[a]) for a in range(3))
    px, py, pz = (axis(spec.box_bounds[a], spec.shape[a]) for a in range(3))
    xr, yr, zr = np.meshgrid(px, py, pz, indexing="ij")
    return lx, ly, lz, np.stack([xr, yr, zr], axis=-1)


def generate_monitor_grid_geometry(case: BenchmarkCase, spec: MonitorGridSpec) -> MonitorGridGeometry:
    """Host FP64 monitor-grid generator (bit-exact with the reference)."""

    if case.geometry.unit.lower() != spec.unit.lower():
        raise ValueError("Benchmark geometry and monitor-grid spec must use the same unit system.")
    lx, ly, lz, box = monitor_box_axes(spec)
    hx, hy, hz = _uniform_step(lx), _uniform_step(ly), _uniform_step(lz)
    X = np.array(box, copy=True)
    for _ in range(spec.harmonic_outer_iterations):
        mon = evaluate_global_monitor_field(case, spec, X[..., 0], X[..., 1], X[..., 2])
        smoothed = _smooth(mon.values, spec.monitor_smoothing)
        solved = _harmonic_solve(
            smoothed, hx, hy, hz, box, X, spec.harmonic_inner_iterations, spec.harmonic_tolerance,
            spec.inner_relaxation,
        )
        nxt = _backtrack(X, solved, lx, ly, lz, spec.harmonic_relaxation)
        moved = float(np.max(np.abs(nxt - X)))
        X = nxt
        if moved < spec.harmonic_tolerance:
            break
    return assemble_monitor_geometry(case, spec, lx, ly, lz, X)


def build_monitor_grid_for_case(
    case: BenchmarkCase,
    *,
    shape: tuple[int, int, int] | None = None,
    box_half_extents: Coordinate3D | None = None,
    element_parameters: dict | None = None,
    device: bool = False,
) -> MonitorGridGeometry:
    """Build the monitor A-grid; ``device=True`` runs the sweeps on the GPU."""

    spec = build_monitor_grid_spec_for_case(
        case, shape=shape, box_half_extents=box_half_extents, element_parameters=element_parameters
    )
    if device:
        from .grid_device import generate_monitor_grid_geometry_device

        return generate_monitor_grid_geometry_device(case, spec)
    return generate_monitor_grid_geometry(case, spec)


def build_h2_local_patch_development_monitor_grid(shape=H2_MONITOR_LOCAL_PATCH_BASELINE_SHAPE, device=False):
    return build_monitor_grid_for_case(
        H2_BENCHMARK_CASE,
        shape=shape,
        box_half_extents=H2_MONITOR_LOCAL_PATCH_BASELINE_BOX_HALF_EXTENTS_BOHR,
        element_parameters=build_h2_local_patch_development_element_parameters(),
        device=device,
    )


def is_monitor_geometry(geom) -> bool:
    """Duck-typed test: monitor geometries carry an inverse metric tensor."""

    return hasattr(geom, "inverse_metric_tensor")
