"""GTH pseudopotentials on the GPU (drop-in for ``src/isogrid/pseudo``).

* gth-pade data for H/C/N/O (``pseudo/gth_data.py:28-180``);
* ``evaluate_local_ionic_potential`` (``pseudo/local.py:349-357``) through the
  ``igd_gth_local_potential`` kernel;
* ``evaluate_nonlocal_ionic_action`` (``pseudo/nonlocal.py:286-337``) through
  compact projector tables (``igd_gth_nonlocal_apply``).  Projector values are
  tabulated once per (geometry, case) on the points where the radial factor
  exceeds 1e-17 of its peak; the reference evaluates them on the whole grid,
  which differs only in terms below that threshold.

``extra_channels`` adds projector channels the reference data leaves empty
(for example the carbon p channel, ``gth_data.py:58-63``).
"""

from __future__ import annotations

import weakref
from dataclasses import dataclass
from math import gamma, pi, sqrt

import numpy as np
import torch

from . import _lib
from .device import device_grid, ptr, stream_ptr

SUPPORTED_GTH_FAMILY = "gth-pade"
SUPPORTED_GTH_ELEMENTS = ("H", "C", "N", "O")


@dataclass(frozen=True)
class GTHLocalTerm:
    rloc: float
    coefficients: tuple[float, ...]


@dataclass(frozen=True)
class GTHNonlocalChannel:
    angular_momentum: int
    radius: float
    projector_count: int
    h_matrix: tuple[tuple[float, ...], ...]


@dataclass(frozen=True)
class GTHPseudoData:
    family: str
    element: str
    valence_configuration: tuple[int, ...]
    ionic_charge: int
    local: GTHLocalTerm
    nonlocal_channels: tuple[GTHNonlocalChannel, ...]
    source: str
    description: str

    @property
    def valence_electrons(self) -> int:
        return self.ionic_charge


def _pp(el, val, z, rloc, coeffs, channels):
    return GTHPseudoData(SUPPORTED_GTH_FAMILY, el, val, z, GTHLocalTerm(rloc, coeffs), channels,
                         "gth-pade family (CP2K format)", f"GTH-PADE pseudopotential for {el}.")


_GTH = {
    "H": _pp("H", (1,), 1, 0.2, (-4.1802368, 0.72507482), ()),
    "C": _pp("C", (2, 2), 4, 0.34883045, (-8.5137711, 1.22843203),
             (GTHNonlocalChannel(0, 0.30455321, 1, ((9.52284179,),)), GTHNonlocalChannel(1, 0.2326773, 0, ()))),
    "N": _pp("N", (2, 3), 5, 0.28917923, (-12.23481988, 1.76640728),
             (GTHNonlocalChannel(0, 0.25660487, 1, ((13.55224272,),)), GTHNonlocalChannel(1, 0.27013369, 0, ()))),
    "O": _pp("O", (2, 4), 6, 0.24762086, (-16.58031797, 2.39570092),
             (GTHNonlocalChannel(0, 0.22178614, 1, ((18.26691718,),)), GTHNonlocalChannel(1, 0.2568289, 0, ()))),
}


def load_gth_pseudo_data(symbol: str, family: str = SUPPORTED_GTH_FAMILY) -> GTHPseudoData:
    if family.strip().lower() != SUPPORTED_GTH_FAMILY:
        raise ValueError(f"The GTH data layer supports only the `gth-pade` family; received `{family}`.")
    s = "".join(ch for ch in symbol.strip() if ch.isalpha())
    if not s:
        raise ValueError("An element symbol is required to load GTH data.")
    s = s[0].upper() + s[1:].lower()
    if s not in _GTH:
        raise ValueError(f"The GTH data layer supports only H, C, N, O; received `{symbol}`.")
    return _GTH[s]


def load_case_gth_pseudo_data(case) -> dict:
    out = {}
    for atom in case.geometry.atoms:
        if atom.element not in out:
            out[atom.element] = load_gth_pseudo_data(atom.element, case.reference_model.pseudo)
    return out


@dataclass(frozen=True)
class LocalIonicPotentialEvaluation:
    pseudo_family: str
    grid_geometry: object
    atom_contributions: tuple
    total_local_potential: np.ndarray


@dataclass(frozen=True)
class NonlocalIonicActionEvaluation:
    pseudo_family: str
    grid_geometry: object
    atom_contributions: tuple
    total_nonlocal_action: np.ndarray


def _check_units(case, geom, evaluator: str = "local GTH evaluator expects a Bohr-space structured grid"):
    """``pseudo/local.py:190-195, 267-271`` and ``pseudo/nonlocal.py:171-176, 293-297`` (same messages)."""

    if case.geometry.unit.lower() != geom.spec.unit.lower():
        raise ValueError("Benchmark geometry and grid geometry must use the same unit system; "
                         f"received `{case.geometry.unit}` and `{geom.spec.unit}`.")
    if geom.spec.unit.lower() != "bohr":
        raise ValueError(f"The current {evaluator}; received `{geom.spec.unit}`.")


def _local_atom_table(case, dev) -> tuple[int, torch.Tensor]:
    """8 doubles per atom: position, valence charge, r_loc, C1..C3."""

    rows = []
    for atom in case.geometry.atoms:
        d = load_gth_pseudo_data(atom.element, case.reference_model.pseudo)
        c = list(d.local.coefficients) + [0.0] * (3 - len(d.local.coefficients))
        if len(c) > 3:
            raise ValueError("at most three local GTH coefficients are supported")
        rows.append([*atom.position, float(d.ionic_charge), d.local.rloc, *c])
    return len(rows), torch.tensor(np.asarray(rows, dtype=np.float64).reshape(-1), device=dev)


def local_potential_device(case, dg) -> torch.Tensor:
    natoms, atoms = _local_atom_table(case, dg.device)
    out = torch.empty(dg.n, dtype=torch.float64, device=dg.device)
    _lib.check(_lib.call("igd_gth_local_potential", dg.n, ptr(dg.x), ptr(dg.y), ptr(dg.z), natoms, ptr(atoms),
                         ptr(out), stream_ptr()), "igd_gth_local_potential")
    return out


def local_force_device(case, dg, rho: torch.Tensor) -> np.ndarray:
    """Hellmann-Feynman force of the local GTH potential, (natoms, 3), for a device density (n,)."""

    natoms, atoms = _local_atom_table(case, dg.device)
    out = torch.empty(3 * natoms, dtype=torch.float64, device=dg.device)
    rho = rho.reshape(-1).to(torch.float64).contiguous()
    _lib.check(_lib.call("igd_gth_local_force", dg.n, ptr(dg.x), ptr(dg.y), ptr(dg.z), ptr(rho),
                         ptr(dg.cell_volumes), natoms, ptr(atoms), ptr(out), stream_ptr()), "igd_gth_local_force")
    return out.cpu().numpy().reshape(natoms, 3)


def evaluate_local_ionic_potential(case, grid_geometry) -> LocalIonicPotentialEvaluation:
    _check_units(case, grid_geometry)
    dg = device_grid(grid_geometry)
    v = local_potential_device(case, dg).cpu().numpy().reshape(grid_geometry.spec.shape)
    return LocalIonicPotentialEvaluation(SUPPORTED_GTH_FAMILY, grid_geometry, (), v)


def _radial(r, l, i, rl):
    g = l + 0.5 * (4 * (i + 1) - 1)
    return sqrt(2.0) / (rl**g * sqrt(gamma(g))) * r ** (l + 2 * i) * np.exp(-0.5 * (r / rl) ** 2)


def _harmonic(l, m, dx, dy, dz, r):
    if l == 0:
        return np.full(dx.shape, 1.0 / sqrt(4.0 * pi))
    c = sqrt(3.0 / (4.0 * pi))
    comp = {-1: dy, 0: dz, 1: dx}[m]
    out = np.zeros_like(r)
    nz = r > 0.0
    out[nz] = c * comp[nz] / r[nz]
    return out


def _projector_gradient(l, m, i, rl, dx, dy, dz, r):
    """d/dx_k of the projector p = R_i^l(r) Y_lm at offsets (dx, dy, dz) from its atom, as
    three arrays (no reference counterpart: the reference computes no forces).

    With N the radial normalisation and e = exp(-r^2 / 2 rl^2), p = N r^(2i) e / sqrt(4 pi)
    (l = 0) or p = c N u r^(2i) e with u the Cartesian component of m (l = 1), so
    grad p = d q(r) N / sqrt(4 pi) (l = 0) and grad_k p = c N (delta_{k,u} r^(2i) e
    + u d_k q(r)) (l = 1), where q(r) = (2i r^(2i-2) - r^(2i) / rl^2) e is smooth at r = 0."""

    g = l + 0.5 * (4 * (i + 1) - 1)
    N = sqrt(2.0) / (rl**g * sqrt(gamma(g)))
    e = np.exp(-0.5 * (r / rl) ** 2)
    q = -(r ** (2 * i)) / rl**2 * e
    if i > 0:
        q = q + 2 * i * r ** (2 * i - 2) * e
    d = (dx, dy, dz)
    if l == 0:
        s = N / sqrt(4.0 * pi)
        return [s * dk * q for dk in d]
    c = sqrt(3.0 / (4.0 * pi))
    ui = {-1: 1, 0: 2, 1: 0}[m]
    u = d[ui]
    out = [c * N * u * dk * q for dk in d]
    out[ui] = out[ui] + c * N * r ** (2 * i) * e
    return out


class ProjectorTable:
    """Device tables of all projectors of a case on one geometry (and, for forces,
    of their gradients on the same point lists)."""

    def __init__(self, case, geom, dg, extra_channels=None, rel_cut: float = 1.0e-17):
        X = np.asarray(geom.x_points, dtype=np.float64).reshape(-1)
        Y = np.asarray(geom.y_points, dtype=np.float64).reshape(-1)
        Z = np.asarray(geom.z_points, dtype=np.float64).reshape(-1)
        offsets, idx, val, groups, hoff, hmat = [0], [], [], [], [0], []
        grad: list = [[], [], []]
        self.group_atoms: list = []
        self.group_h: list = []
        nproj = 0
        for ia, atom in enumerate(case.geometry.atoms):
            data = load_gth_pseudo_data(atom.element, case.reference_model.pseudo)
            chans = [(c.angular_momentum, c.radius, c.h_matrix) for c in data.nonlocal_channels if c.projector_count]
            if extra_channels and atom.element in extra_channels:
                chans += list(extra_channels[atom.element])
            if not chans:
                continue
            dx, dy, dz = X - atom.position[0], Y - atom.position[1], Z - atom.position[2]
            r = np.sqrt(dx * dx + dy * dy + dz * dz)
            for l, rl, h in chans:
                h = np.asarray(h, dtype=np.float64)
                cnt = h.shape[0]
                # radial support: exp(-r^2/2rl^2) r^(l+2i) above rel_cut of its peak
                rcut = rl * sqrt(2.0 * (-np.log(rel_cut) + (l + 2 * cnt) * np.log(10.0)))
                sel = np.flatnonzero(r <= rcut).astype(np.int32)
                for m in ((0,) if l == 0 else (-1, 0, 1)):
                    groups.append((nproj, cnt))
                    self.group_atoms.append(ia)
                    self.group_h.append(h)
                    for i in range(cnt):
                        v = _radial(r[sel], l, i, rl) * _harmonic(l, m, dx[sel], dy[sel], dz[sel], r[sel])
                        idx.append(sel)
                        val.append(v)
                        for k, gk in enumerate(_projector_gradient(l, m, i, rl, dx[sel], dy[sel], dz[sel], r[sel])):
                            grad[k].append(gk)
                        offsets.append(offsets[-1] + sel.size)
                        nproj += 1
                    hmat.append(h.reshape(-1))
                    hoff.append(hoff[-1] + h.size)
        self.nproj = nproj
        self.ngroups = len(groups)
        dev = dg.device
        if nproj:
            self.offsets = torch.tensor(offsets, dtype=torch.int64, device=dev)
            self.idx = torch.as_tensor(np.concatenate(idx), device=dev)
            self.val = torch.as_tensor(np.concatenate(val), device=dev)
            self.groups = torch.tensor(np.asarray(groups, dtype=np.int32).reshape(-1), device=dev)
            self.hoff = torch.tensor(hoff[:-1], dtype=torch.int64, device=dev)
            self.hmat = torch.as_tensor(np.concatenate(hmat), device=dev)
            self.points = int(offsets[-1])
            self._grad_host = grad
            self._grad = None
        self._groups_host = groups

    def apply(self, dg, psi: torch.Tensor, out: torch.Tensor, scale: float = 1.0) -> torch.Tensor:
        """out += scale * V_nl psi for a (nb, n) block."""

        if self.nproj == 0:
            return out
        nb = psi.shape[0]
        ws = torch.empty(2 * self.nproj * nb, dtype=torch.float64, device=dg.device)
        dt = _lib.IGD_F32 if psi.dtype == torch.float32 else _lib.IGD_F64
        _lib.check(_lib.call("igd_gth_nonlocal_apply", dt, self.nproj, ptr(self.offsets), ptr(self.idx), ptr(self.val),
                             self.ngroups, ptr(self.groups), ptr(self.hoff), ptr(self.hmat), ptr(dg.cell_volumes),
                             ptr(psi), ptr(out), nb, dg.n, float(scale), ptr(ws), stream_ptr()),
                   "igd_gth_nonlocal_apply")
        return out


    def projections(self, dg, psi: torch.Tensor, val: torch.Tensor | None = None) -> np.ndarray:
        """<p_j | psi_o>_W for a (nb, n) block as an (nproj, nb) host array (``val``: another
        table on the same point lists, e.g. a gradient component)."""

        nb = psi.shape[0]
        out = torch.empty((self.nproj, nb), dtype=torch.float64, device=dg.device)
        dt = _lib.IGD_F32 if psi.dtype == torch.float32 else _lib.IGD_F64
        _lib.check(_lib.call("igd_gth_projections", dt, self.nproj, ptr(self.offsets), ptr(self.idx),
                             ptr(self.val if val is None else val), ptr(dg.cell_volumes), ptr(psi), nb,
                             psi.stride(0), ptr(out), stream_ptr()), "igd_gth_projections")
        return out.cpu().numpy()

    def forces(self, dg, psi: torch.Tensor, occupations, natoms: int) -> np.ndarray:
        """Nonlocal Hellmann-Feynman force (natoms, 3) of occupied orbitals at fixed psi:
        E_nl = sum_o f_o sum_ab c_ao h_ab c_bo with c = <p|psi>_W, and since the projectors
        move with their atom, F_k = -dE/dR_k = 2 sum_o f_o sum_ab <d_k p_a|psi_o> h_ab c_bo.
        No reference counterpart (the reference computes no forces)."""

        f = np.zeros((natoms, 3))
        if self.nproj == 0:
            return f
        if self._grad is None:
            self._grad = [torch.as_tensor(np.concatenate(g), device=dg.device) for g in self._grad_host]
        occ = np.asarray(occupations, dtype=np.float64)
        psi = psi[: len(occ)].contiguous()
        c = self.projections(dg, psi)
        gk = [self.projections(dg, psi, self._grad[k]) for k in range(3)]
        for (first, cnt), ia, h in zip(self._groups_host, self.group_atoms, self.group_h):
            cg = c[first:first + cnt]  # (cnt, nb)
            hc = h @ cg
            for k in range(3):
                f[ia, k] += 2.0 * float(np.sum(occ * np.sum(gk[k][first:first + cnt] * hc, axis=0)))
        return f


_TABLES: dict = {}


def projector_table(case, geom, extra_channels=None) -> ProjectorTable:
    key = (id(geom), id(case), id(extra_channels))
    hit = _TABLES.get(key)
    if hit is not None and hit[0]() is geom and hit[1]() is case:
        return hit[2]
    dg = device_grid(geom)
    t = ProjectorTable(case, geom, dg, extra_channels)
    _TABLES[key] = (weakref.ref(geom), weakref.ref(case) if hasattr(case, "__weakref__") else (lambda: case), t)
    weakref.finalize(geom, _TABLES.pop, key, None)
    return t


def evaluate_nonlocal_ionic_action(case, grid_geometry, psi, *, extra_channels=None) -> NonlocalIonicActionEvaluation:
    from .ops import validate_orbital_field

    _check_units(case, grid_geometry, "GTH nonlocal projector evaluator expects a Bohr-space grid")
    field = validate_orbital_field(psi, grid_geometry)
    dg = device_grid(grid_geometry)
    tab = projector_table(case, grid_geometry, extra_channels)
    p = torch.as_tensor(np.ascontiguousarray(field, dtype=np.float64), device=dg.device).reshape(1, -1)
    out = torch.zeros_like(p)
    tab.apply(dg, p, out)
    return NonlocalIonicActionEvaluation(SUPPORTED_GTH_FAMILY, grid_geometry, (),
                                         out.cpu().numpy().reshape(grid_geometry.spec.shape))


# --------------------------------------------------------------- near-core patch
@dataclass(frozen=True)
class LocalPotentialPatchParameters:
    """Atom-centred local-GTH patch parameters (``pseudo/local.py:55-77``)."""

    patch_radius_scale: float = 1.0
    patch_grid_shape: tuple = (25, 25, 25)
    correction_strength: float = 1.0
    interpolation_neighbors: int = 8

    def __post_init__(self) -> None:
        if self.patch_radius_scale <= 0.0:
            raise ValueError("patch_radius_scale must be positive.")
        if self.correction_strength < 0.0:
            raise ValueError("correction_strength must be non-negative.")
        if self.interpolation_neighbors <= 0:
            raise ValueError("interpolation_neighbors must be positive.")
        if len(self.patch_grid_shape) != 3:
            raise ValueError("patch_grid_shape must be a 3-tuple.")
        for n in self.patch_grid_shape:
            if n < 3 or n % 2 == 0:
                raise ValueError("Each patch-grid direction must use an odd number of points >= 3.")


# the parameters every reference A-grid SCF route uses (``scf/driver.py:1018-1024``)
DEFAULT_MONITOR_PATCH_PARAMETERS = LocalPotentialPatchParameters(0.75, (25, 25, 25), 1.30, 8)


@dataclass(frozen=True)
class AtomicLocalPotentialPatchCorrection:
    atom_index: int
    element: str
    position: tuple
    patch_radius_bohr: float
    patch_grid_shape: tuple
    correction_strength: float
    main_grid_patch_energy: float
    patch_integrated_energy: float
    correction_energy: float
    patch_point_count: int


@dataclass(frozen=True)
class LocalIonicPotentialPatchEvaluation:
    base_evaluation: object
    density_field: np.ndarray | None
    patch_parameters: LocalPotentialPatchParameters
    atomic_patch_corrections: tuple
    uncorrected_local_energy: float
    corrected_local_energy: float
    total_patch_correction: float


@dataclass(frozen=True)
class FrozenPatchLocalPotentialEmbedding:
    base_evaluation: object
    patch_evaluation: LocalIonicPotentialPatchEvaluation
    corrected_total_local_potential: np.ndarray
    correction_field: np.ndarray
    atomic_scaling_factors: tuple
    embedded_patch_correction_energy: float
    embedding_energy_mismatch: float


class PatchTables:
    """Device tables of the near-core patch for one (geometry, case, parameters).

    Per atom: the spherical set of patch points of a (2R)^3 Cartesian patch grid
    (``_build_patch_grid``, :379-411), the atom's local potential there, the
    k-nearest-neighbour weights from the main grid (``igd_patch_knn``), and the
    main-grid mask of the same sphere times the atom's potential.  Geometry-only:
    built once; every density then costs one gather and two weighted sums per atom."""

    def __init__(self, case, geom, params: LocalPotentialPatchParameters):
        from .device import device_grid

        dg = device_grid(geom)
        self.dg, self.params = dg, params
        dev = dg.device
        X = np.asarray(geom.x_points, dtype=np.float64)
        Y = np.asarray(geom.y_points, dtype=np.float64)
        Z = np.asarray(geom.z_points, dtype=np.float64)
        self.atoms = []
        for a, atom in enumerate(case.geometry.atoms):
            iface = geom.patch_interfaces[a]
            if "local_gth" not in iface.implemented_purposes:
                raise ValueError("This monitor-grid patch interface does not implement local-GTH correction.")
            R = float(iface.patch_radius) * params.patch_radius_scale
            c = atom.position
            ax = [np.linspace(c[i] - R, c[i] + R, params.patch_grid_shape[i], dtype=np.float64) for i in range(3)]
            vol = float(ax[0][1] - ax[0][0]) * float(ax[1][1] - ax[1][0]) * float(ax[2][1] - ax[2][0])
            px, py, pz = np.meshgrid(*ax, indexing="ij")
            dx, dy, dz = px - c[0], py - c[1], pz - c[2]
            m = np.sqrt(dx * dx + dy * dy + dz * dz, dtype=np.float64) <= R
            q = [torch.as_tensor(np.ascontiguousarray(v[m]), device=dev) for v in (px, py, pz)]
            nq = int(m.sum())
            one = _AtomCase(case, a)
            n1, table = _local_atom_table(one, dev)
            vpatch = torch.empty(nq, dtype=torch.float64, device=dev)
            _lib.check(_lib.call("igd_gth_local_potential", nq, ptr(q[0]), ptr(q[1]), ptr(q[2]), n1, ptr(table),
                                 ptr(vpatch), stream_ptr()), "igd_gth_local_potential")
            vmain = local_potential_device(one, dg)
            rm = np.sqrt((X - c[0]) ** 2 + (Y - c[1]) ** 2 + (Z - c[2]) ** 2, dtype=np.float64) <= R
            mask = torch.as_tensor(rm.reshape(-1).astype(np.float64), device=dev)
            k = params.interpolation_neighbors
            idx = torch.empty(nq * k, dtype=torch.int32, device=dev)
            w = torch.empty(nq * k, dtype=torch.float64, device=dev)
            _lib.check(_lib.call("igd_patch_knn", nq, ptr(q[0]), ptr(q[1]), ptr(q[2]), dg.n, ptr(dg.x), ptr(dg.y),
                                 ptr(dg.z), k, ptr(idx), ptr(w), stream_ptr()), "igd_patch_knn")
            self.atoms.append(dict(index=a, element=atom.element, position=tuple(c), radius=R, volume=vol, nq=nq,
                                   vpatch=vpatch, vmain=vmain, mask=mask, vmask=vmain * mask, idx=idx, w=w,
                                   rho_patch=torch.empty(nq, dtype=torch.float64, device=dev)))

    def corrections(self, rho: torch.Tensor) -> list:
        """Per atom (main_grid_patch_energy, patch_integrated_energy, correction_energy) for a
        device total density (one host read)."""

        dg, k = self.dg, self.params.interpolation_neighbors
        sums = []
        for at in self.atoms:
            _lib.check(_lib.call("igd_patch_gather", at["nq"], k, ptr(at["idx"]), ptr(at["w"]), ptr(rho),
                                 ptr(at["rho_patch"]), stream_ptr()), "igd_patch_gather")
            sums.append(_wsum(dg, rho, at["vmask"], dg.cell_volumes))
            sums.append(_wsum(dg, at["rho_patch"], at["vpatch"], None, n=at["nq"]))
        h = torch.cat(sums).cpu().numpy()
        out = []
        for i, at in enumerate(self.atoms):
            main, patch = float(h[2 * i]), float(h[2 * i + 1]) * at["volume"]
            out.append((main, patch, self.params.correction_strength * (patch - main)))
        return out

    def embedding_field(self, rho: torch.Tensor, corr: list) -> tuple[torch.Tensor, list]:
        """Frozen correction field (``_build_atomic_frozen_patch_correction_field``, :567-600)."""

        field = torch.zeros(self.dg.n, dtype=torch.float64, device=self.dg.device)
        scalings = []
        for at, (main, _, ce) in zip(self.atoms, corr):
            if float(at["mask"].sum()) == 0.0 or abs(ce) <= 1.0e-16:
                scalings.append(0.0)
                continue
            if abs(main) > 1.0e-14:
                s = ce / main
                field += s * at["vmask"]
            else:
                dw = float(_wsum(self.dg, rho, at["mask"], self.dg.cell_volumes).item())
                if dw <= 1.0e-16:
                    scalings.append(0.0)
                    continue
                s = ce / dw
                field += s * at["mask"]
            scalings.append(float(s))
        return field, scalings


class _AtomCase:
    """A one-atom view of a case for the local-potential tables."""

    def __init__(self, case, a):
        self.geometry = type("G", (), {"atoms": (case.geometry.atoms[a],)})()
        self.reference_model = case.reference_model


def _wsum(dg, a, b, w, n=None) -> torch.Tensor:
    out = torch.empty(1, dtype=torch.float64, device=dg.device)
    _lib.check(_lib.call("igd_weighted_sum", _lib.IGD_F64, dg.n if n is None else n, ptr(a), ptr(b), ptr(w),
                         ptr(out), stream_ptr()), "igd_weighted_sum")
    return out


_PATCH_TABLES: dict = {}


def patch_tables(case, geom, params) -> PatchTables:
    key = (id(geom), id(case), params)
    hit = _PATCH_TABLES.get(key)
    if hit is not None and hit[0]() is geom:
        return hit[1]
    t = PatchTables(case, geom, params)
    _PATCH_TABLES[key] = (weakref.ref(geom), t)
    weakref.finalize(geom, _PATCH_TABLES.pop, key, None)
    return t


def evaluate_monitor_grid_local_ionic_potential_with_patch(case, grid_geometry, density_field, *,
                                                           patch_parameters=None, base_evaluation=None):
    """E_loc^patch = E_loc^main + sum_A lambda [I_A^patch - I_A^main(patch)] (``pseudo/local.py:603-660``)."""

    from .device import device_grid

    params = patch_parameters or LocalPotentialPatchParameters()
    dg = device_grid(grid_geometry)
    rho = np.asarray(density_field, dtype=np.float64)
    if rho.shape != tuple(grid_geometry.spec.shape):
        raise ValueError("density_field must match the grid shape.")
    rd = torch.as_tensor(np.ascontiguousarray(rho), device=dg.device).reshape(-1)
    if base_evaluation is None:
        base_evaluation = evaluate_local_ionic_potential(case, grid_geometry)
    vloc = torch.as_tensor(np.ascontiguousarray(base_evaluation.total_local_potential), device=dg.device).reshape(-1)
    unc = float(_wsum(dg, rd, vloc, dg.cell_volumes).item())
    tab = patch_tables(case, grid_geometry, params)
    corr = tab.corrections(rd)
    atoms = tuple(AtomicLocalPotentialPatchCorrection(
        at["index"], at["element"], at["position"], at["radius"], tuple(params.patch_grid_shape),
        float(params.correction_strength), main, patch, ce, at["nq"]) for at, (main, patch, ce) in zip(tab.atoms, corr))
    total = float(sum(c.correction_energy for c in atoms))
    return LocalIonicPotentialPatchEvaluation(base_evaluation, rho, params, atoms, unc, unc + total, total)


def evaluate_monitor_grid_local_ionic_potential_with_frozen_patch_field(case, grid_geometry, density_field, *,
                                                                       patch_parameters=None, patch_evaluation=None,
                                                                       base_evaluation=None):
    """Corrected local potential with the patch correction embedded (``pseudo/local.py:603-703``)."""

    from .device import device_grid

    params = patch_parameters or LocalPotentialPatchParameters()
    if patch_evaluation is None:
        patch_evaluation = evaluate_monitor_grid_local_ionic_potential_with_patch(
            case, grid_geometry, density_field, patch_parameters=params, base_evaluation=base_evaluation)
    dg = device_grid(grid_geometry)
    rd = torch.as_tensor(np.ascontiguousarray(patch_evaluation.density_field), device=dg.device).reshape(-1)
    tab = patch_tables(case, grid_geometry, params)
    corr = [(c.main_grid_patch_energy, c.patch_integrated_energy, c.correction_energy)
            for c in patch_evaluation.atomic_patch_corrections]
    field, scalings = tab.embedding_field(rd, corr)
    shape = tuple(grid_geometry.spec.shape)
    f = field.cpu().numpy().reshape(shape)
    base = patch_evaluation.base_evaluation
    emb = float(_wsum(dg, rd, field, dg.cell_volumes).item())
    return FrozenPatchLocalPotentialEmbedding(base, patch_evaluation,
                                              np.asarray(base.total_local_potential + f, dtype=np.float64), f,
                                              tuple(scalings), emb, emb - patch_evaluation.total_patch_correction)
