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


def _check_units(case, geom):
    if case.geometry.unit.lower() != geom.spec.unit.lower():
        raise ValueError("Benchmark geometry and grid geometry must use the same unit system.")
    if geom.spec.unit.lower() != "bohr":
        raise ValueError("The GTH evaluators expect a Bohr-space grid.")


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


class ProjectorTable:
    """Device tables of all projectors of a case on one geometry."""

    def __init__(self, case, geom, dg, extra_channels=None, rel_cut: float = 1.0e-17):
        X = np.asarray(geom.x_points, dtype=np.float64).reshape(-1)
        Y = np.asarray(geom.y_points, dtype=np.float64).reshape(-1)
        Z = np.asarray(geom.z_points, dtype=np.float64).reshape(-1)
        offsets, idx, val, groups, hoff, hmat = [0], [], [], [], [0], []
        nproj = 0
        for atom in case.geometry.atoms:
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
                    for i in range(cnt):
                        v = _radial(r[sel], l, i, rl) * _harmonic(l, m, dx[sel], dy[sel], dz[sel], r[sel])
                        idx.append(sel)
                        val.append(v)
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
    _check_units(case, grid_geometry)
    dg = device_grid(grid_geometry)
    tab = projector_table(case, grid_geometry, extra_channels)
    p = torch.as_tensor(np.ascontiguousarray(psi, dtype=np.float64), device=dg.device).reshape(1, -1)
    out = torch.zeros_like(p)
    tab.apply(dg, p, out)
    return NonlocalIonicActionEvaluation(SUPPORTED_GTH_FAMILY, grid_geometry, (),
                                         out.cpu().numpy().reshape(grid_geometry.spec.shape))
