"""Kohn-Sham single-point SCF on the GPU (drop-in for ``src/isogrid/scf/driver.py``).

* occupations (``driver.py:593-627``), ion-ion repulsion (:884-902), the
  bonding/antibonding start (:705-769);
* energy assembly E = T_s + E_loc + E_nl + E_H + E_xc + E_II
  (``evaluate_single_point_energy`` :905-1015 and the local-only variant
  ``evaluate_static_local_single_point_energy`` :2668-2810), every term an
  FP64 device reduction;
* the minimal SCF loop ``run_h2_minimal_scf`` (:2953-3159): per step one
  Hartree solve, LSDA, a block eigensolve per spin channel warm-started from
  the previous orbitals, density build, energy, linear mixing; Pulay (DIIS)
  extrapolation of the mixed densities (``_apply_monitor_grid_density_diis``
  :2234-2294) as an option.

Densities, potentials and orbitals stay in device memory for the whole SCF;
the host sees scalars and the small Rayleigh-Ritz matrices.  ``precision``
picks the orbital arithmetic: "fp64" throughout, or "fp32" (alias "mixed")
for the H.Psi stencil, Gram/rotation data and the inner Poisson iterations,
with FP64 Rayleigh-Ritz, FP64 Poisson refinement and FP64 energy reductions.
"""

from __future__ import annotations

import time
from dataclasses import dataclass

import numpy as np
import torch

from .active_subspace import (ActiveSubspaceConfig, MonitorGridActiveSubspaceIterationDiagnostics,
                              initialize_active_subspace, update_active_subspace)
from .config import H2_BENCHMARK_CASE
from .density import build_density_device, renormalize_device, residual_device
from .device import device_grid, normalize_precision, ptr, stream_ptr, torch_dtype
from .grid import is_monitor_geometry
from .ks import BlockLA, DeviceOperator, FixedPotentialEigensolverResult, JacobiPreconditioner, _dev64, block_size, \
    block_subspace_iteration_device, default_guess_device, orthonormalize_device
from .ks import _result as _solve_result
from .ops import hpsi_device
from .mixing import AndersonMixer, BroydenMixer, PulayMixer  # noqa: F401
from .mixing import closed_shell_singlet_baseline_mix, cycle_breaker_mix, detect_singlet_alternation, \
    previous_density_residual_ratio, singlet_hartree_tail_channel_shares
from .poisson import solve_poisson_device
from .pseudo import load_case_gth_pseudo_data, local_potential_device, projector_table
from .xc import lsda_device
from . import _lib


@dataclass(frozen=True)
class SpinOccupations:
    label: str
    spin: int
    total_electrons: int
    n_alpha: int
    n_beta: int
    occupations_up: tuple
    occupations_down: tuple


@dataclass(frozen=True)
class FixedPotentialSolveSummary:
    spin_channel: str
    target_orbitals: int
    solver_backend: str
    use_scipy_fallback: bool
    solver_method: str
    solver_note: str
    converged: bool
    eigenvalues: np.ndarray
    residual_norms: np.ndarray


@dataclass(frozen=True)
class SinglePointEnergyComponents:
    kinetic: float
    local_ionic: float
    nonlocal_ionic: float
    hartree: float
    xc: float
    ion_ion_repulsion: float
    total: float


@dataclass(frozen=True)
class ScfIterationRecord:
    iteration: int
    input_rho_up: np.ndarray | None
    input_rho_down: np.ndarray | None
    output_rho_up: np.ndarray | None
    output_rho_down: np.ndarray | None
    mixed_rho_up: np.ndarray | None
    mixed_rho_down: np.ndarray | None
    density_residual: float
    energy: SinglePointEnergyComponents
    energy_change: float | None
    solve_up: FixedPotentialSolveSummary | None
    solve_down: FixedPotentialSolveSummary | None
    wall_time_seconds: float = 0.0
    eigensolver_iterations: tuple = ()
    poisson_iterations: int = 0


@dataclass(frozen=True)
class H2ScfResult:
    converged: bool
    spin_state_label: str
    spin: int
    occupations: SpinOccupations
    iteration_count: int
    history: tuple
    eigenvalues_up: np.ndarray
    eigenvalues_down: np.ndarray
    orbitals_up: np.ndarray
    orbitals_down: np.ndarray
    rho_up: np.ndarray
    rho_down: np.ndarray
    energy: SinglePointEnergyComponents
    solve_up: FixedPotentialEigensolverResult | None
    solve_down: FixedPotentialEigensolverResult | None
    wall_time_seconds: float = 0.0
    precision: str = "fp64"


def _validate_h2_case(case) -> None:
    """``driver.py:570-590``: the reference drivers accept neutral H2 in Bohr only (same messages).
    The reference also pins the case name to its default benchmark; any neutral H2 case in Bohr is
    accepted here, so bond-length scans run through the same drivers."""

    if case.charge != 0:
        raise ValueError("The current minimal SCF driver supports only neutral H2; "
                         f"received charge={case.charge}.")
    atoms = case.geometry.atoms
    if case.geometry.name.upper() != "H2" or len(atoms) != 2 or any(a.element != "H" for a in atoms):
        raise ValueError("The current minimal SCF driver supports only H2 geometries; "
                         f"received `{case.geometry.name}`.")
    if case.geometry.unit.lower() != "bohr":
        raise ValueError("The current minimal SCF driver expects Bohr geometries; "
                         f"received `{case.geometry.unit}`.")


def resolve_spin_occupations(spin_label: str, case=H2_BENCHMARK_CASE) -> SpinOccupations:
    """Aufbau occupations for a named spin state of any supported molecule."""

    wanted = spin_label.strip().lower()
    state = next((s for s in case.spin_states if s.label.lower() == wanted), None)
    if state is None:  # driver.py:557-567, same message
        available = ", ".join(s.label for s in case.spin_states)
        raise ValueError(f"Spin state `{spin_label}` is not configured for `{case.name}`. "
                         f"Available states: {available}.")
    pseudo = load_case_gth_pseudo_data(case)
    total = sum(pseudo[a.element].ionic_charge for a in case.geometry.atoms) - case.charge
    if total <= 0:
        raise ValueError("The SCF driver expects a positive valence-electron count.")
    if (total + state.spin) % 2 != 0:
        raise ValueError("The requested spin state is inconsistent with the total electron count.")
    na = (total + state.spin) // 2
    nb = total - na
    if na < 0 or nb < 0:
        raise ValueError("Resolved alpha/beta occupations must be non-negative.")
    return SpinOccupations(state.label, state.spin, total, na, nb, (1.0,) * na, (1.0,) * nb)


def resolve_h2_spin_occupations(spin_label: str, case=H2_BENCHMARK_CASE) -> SpinOccupations:
    _validate_h2_case(case)
    return resolve_spin_occupations(spin_label, case)


def evaluate_ion_ion_repulsion(case=H2_BENCHMARK_CASE) -> float:
    """Sum over ion pairs of Z_i Z_j / |R_i - R_j| with GTH valence charges."""

    pseudo = load_case_gth_pseudo_data(case)
    atoms = case.geometry.atoms
    e = 0.0
    for i, a in enumerate(atoms):
        for b in atoms[i + 1:]:
            d = float(np.linalg.norm(np.subtract(a.position, b.position)))
            if d <= 0.0:
                raise ValueError("Distinct ions must not occupy the same position.")
            e += pseudo[a.element].ionic_charge * pseudo[b.element].ionic_charge / d
    return e


def evaluate_ion_ion_forces(case=H2_BENCHMARK_CASE) -> np.ndarray:
    """-dE_II/dR_a = sum_b Z_a Z_b (R_a - R_b) / |R_a - R_b|^3, (natoms, 3)."""

    pseudo = load_case_gth_pseudo_data(case)
    atoms = case.geometry.atoms
    f = np.zeros((len(atoms), 3))
    for i, a in enumerate(atoms):
        for j, b in enumerate(atoms):
            if i != j:
                d = np.subtract(a.position, b.position)
                f[i] += pseudo[a.element].ionic_charge * pseudo[b.element].ionic_charge * d / np.linalg.norm(d) ** 3
    return f


def evaluate_hellmann_feynman_forces(case, grid_geometry, rho_total, orbitals=None) -> np.ndarray:
    """Atomic forces -dE/dR_a of a converged SCF on a fixed grid, (natoms, 3): the local
    GTH term (``igd_gth_local_force``), the nonlocal GTH term (projector gradients,
    ``igd_gth_projections``) and the ion-ion term.

    ``orbitals``: for cases with nonlocal channels, a list of (orbital block (k, nx, ny,
    nz) or (k, n), occupations) per spin channel.  No reference counterpart (the
    reference computes no forces).  Exact for the discrete energy when the grid does
    not move with the atoms and the kinetic operator is self-adjoint in the
    cell-volume metric (trial-fix A-grid)."""

    from .pseudo import local_force_device, projector_table

    dg = device_grid(grid_geometry)
    rho = rho_total if isinstance(rho_total, torch.Tensor) else torch.as_tensor(
        np.ascontiguousarray(rho_total, dtype=np.float64), device=dg.device)
    f = local_force_device(case, dg, rho.reshape(-1)) + evaluate_ion_ion_forces(case)
    tab = projector_table(case, grid_geometry)
    if tab.nproj:
        if orbitals is None:
            raise ValueError("a case with nonlocal GTH channels needs the occupied orbitals for its forces")
        for block, occ in orbitals:
            if block is None or len(occ) == 0:
                continue
            psi = block if isinstance(block, torch.Tensor) else torch.as_tensor(np.ascontiguousarray(block),
                                                                                  device=dg.device)
            psi = psi.reshape(psi.shape[0], -1).to(torch.float64)
            f = f + tab.forces(dg, psi, occ, len(case.geometry.atoms))
    return f


def _is_closed_shell_singlet(occ: SpinOccupations) -> bool:
    return occ.n_alpha == occ.n_beta and occ.spin == 0 and occ.occupations_up == occ.occupations_down


# ----------------------------------------------------------------- device engine
class DeviceScfEngine:
    """Everything one SCF needs on one geometry, resident on the device."""

    def __init__(self, case, grid_geometry, occupations: SpinOccupations, *, precision: str = "fp64",
                 kinetic_version: str = "production", include_nonlocal: bool = True, functional: str | None = None,
                 poisson_tolerance: float = 1.0e-8, poisson_max_iterations: int = 400,
                 poisson_precision: str | None = None, preconditioner: str = "jacobi",
                 use_monitor_patch: bool = False, patch_parameters=None, poisson_warm_start: bool = False):
        if preconditioner not in ("jacobi", "none"):
            raise ValueError(f"preconditioner must be `jacobi` or `none`; received `{preconditioner}`.")
        self.preconditioner = preconditioner
        self.block = None
        # Rayleigh-Ritz of the eigensolver: "symmetric" (the reference's) or "right"
        # (right eigenpairs of an operator that is not self-adjoint in the W inner product)
        self.ritz = "symmetric"
        # start each Hartree solve from the previous one's interior field (the
        # reference starts from zero; the stopping rule is the same)
        self.poisson_warm_start = poisson_warm_start
        self._last_u = None
        self.eigensolver_graphs = True  # CUDA-graph replay of the eigensolver's device stages
        self.case, self.geom, self.occ = case, grid_geometry, occupations
        self.dg = dg = device_grid(grid_geometry)
        self.prec = normalize_precision(precision)
        self.odt = torch_dtype(self.prec)
        self.closure = kinetic_version if is_monitor_geometry(grid_geometry) else "legacy"
        self.functional = case.reference_model.xc if functional is None else functional
        self.poisson_tolerance = float(poisson_tolerance)
        self.poisson_max_iterations = int(poisson_max_iterations)
        self.poisson_precision = poisson_precision or ("mixed" if self.prec == "fp32" else "fp64")
        self.vloc = local_potential_device(case, dg)
        self.table = None
        if include_nonlocal:
            t = projector_table(case, grid_geometry)
            self.table = t if t.nproj else None
        self.e_ii = evaluate_ion_ion_repulsion(case)
        self.patch = None
        if use_monitor_patch:
            if not is_monitor_geometry(grid_geometry):
                raise ValueError("the near-core patch applies to monitor A-grids only")
            from .pseudo import DEFAULT_MONITOR_PATCH_PARAMETERS, patch_tables

            self.patch = patch_tables(case, grid_geometry, patch_parameters or DEFAULT_MONITOR_PATCH_PARAMETERS)
        self.la = BlockLA(dg)
        self._guesses: dict = {}
        self.poisson_iterations = 0
        self.poisson_history: list = []
        self.eigensolver_iterations: list = []

    # -- reductions (FP64 on the device; one host read per scalar)
    def wdot(self, a: torch.Tensor, b: torch.Tensor | None = None) -> torch.Tensor:
        out = torch.empty(1, dtype=torch.float64, device=self.dg.device)
        dt = _lib.IGD_F32 if a.dtype == torch.float32 else _lib.IGD_F64
        _lib.check(_lib.call("igd_weighted_sum", dt, self.dg.n, ptr(a), ptr(b), ptr(self.dg.cell_volumes), ptr(out),
                             stream_ptr()), "igd_weighted_sum")
        return out

    def density(self, orbitals: torch.Tensor | None, occupations, target: float) -> torch.Tensor:
        """Occupation-weighted |psi|^2 renormalised to ``target`` electrons (FP64)."""

        integral = torch.zeros(1, dtype=torch.float64, device=self.dg.device)
        rho = build_density_device(self.dg, orbitals if len(occupations) else None, occupations, integral=integral)
        return renormalize_device(self.dg, rho, float(target), integral)

    def renormalized(self, rho: torch.Tensor, target: float) -> torch.Tensor:
        if target == 0.0:
            return torch.zeros_like(rho)
        integral = self.wdot(rho)
        return renormalize_device(self.dg, rho.clone(), float(target), integral)

    def hartree(self, rho_total: torch.Tensor):
        sol = solve_poisson_device(self.dg, self.geom, rho_total, tolerance=self.poisson_tolerance,
                                   max_iterations=self.poisson_max_iterations, precision=self.poisson_precision,
                                   start=self._last_u if self.poisson_warm_start else None)
        if self.poisson_warm_start:
            self._last_u = sol.u
        self.poisson_iterations += sol.iterations
        self.poisson_history.append(int(sol.iterations))
        return sol

    def xc(self, up: torch.Tensor, dn: torch.Tensor):
        return lsda_device(up, dn, functional=self.functional, w=self.dg.cell_volumes)

    # -- operators and the eigensolve
    def operator(self, veff: torch.Tensor) -> DeviceOperator:
        return DeviceOperator.from_potential(self.geom, self.case, veff, closure=self.closure, dtype=self.odt,
                                             include_nonlocal=self.table is not None)

    def default_guess(self, count: int) -> torch.Tensor:
        g = self._guesses.get(count)
        if g is None:
            g = default_guess_device(self.case, self.geom, self.dg, count)
            self._guesses[count] = g
        return g

    def eigensolve(self, veff: torch.Tensor, k: int, guess, *, tolerance: float, max_iterations: int, ncv=None,
                   stall_iterations: int | None = 30):
        op = self.operator(veff)
        pre = JacobiPreconditioner(op) if self.preconditioner == "jacobi" else None
        # With the preconditioned expansion a small working block is enough (measured
        # on H2: 12 columns for one or two bands, 2k beyond; 12k + 8 costs 2-8x more
        # time per SCF); the unpreconditioned iteration keeps the reference's 12k + 8.
        blk = ((12 if k <= 2 else 2 * k) if self.block is None else self.block) if pre is not None else None
        m = blk if blk else block_size(k, None, ncv)
        res = block_subspace_iteration_device(op, self.case, k, max_iterations=max_iterations, tolerance=tolerance,
                                              initial_guess=guess, ncv=ncv, default_guess=self.default_guess(max(k, m)),
                                              stall_iterations=stall_iterations, preconditioner=pre, block=blk,
                                              graphs=self.eigensolver_graphs, ritz=self.ritz)
        self.eigensolver_iterations.append(int(res["iteration_count"]))
        return res

    # -- energy terms
    def kinetic_energy(self, orbitals: torch.Tensor | None, occupations) -> float:
        if orbitals is None or len(occupations) == 0:
            return 0.0
        psi = orbitals[: len(occupations)].to(torch.float64).contiguous()
        tpsi = hpsi_device(self.dg, psi, closure=self.closure, kscale=-0.5)
        d = torch.diagonal(self.la.gram(psi, tpsi)).cpu().numpy()
        return float(np.dot(np.asarray(occupations, dtype=np.float64), d))

    def nonlocal_energy(self, orbitals: torch.Tensor | None, occupations) -> float:
        if self.table is None or orbitals is None or len(occupations) == 0:
            return 0.0
        psi = orbitals[: len(occupations)].to(torch.float64).contiguous()
        out = torch.zeros_like(psi)
        self.table.apply(self.dg, psi, out)
        d = torch.diagonal(self.la.gram(psi, out)).cpu().numpy()
        return float(np.dot(np.asarray(occupations, dtype=np.float64), d))

    def energy(self, up: torch.Tensor, dn: torch.Tensor, orb_up, orb_dn, *, local_only: bool = False,
               hartree=None, lsda=None) -> tuple[SinglePointEnergyComponents, object, dict]:
        """Energy at renormalised densities (``driver.py:905-1015``); returns (E, hartree, lsda)."""

        occ = self.occ
        rho = up + dn
        if hartree is None:
            hartree = self.hartree(rho)
        if lsda is None:
            lsda = self.xc(up, dn)
        sums = torch.cat([self.wdot(rho, self.vloc), self.wdot(rho, hartree.potential), lsda["energy"]]).cpu().numpy()
        if self.patch is not None:  # E_loc^patch (``pseudo/local.py:603-660``)
            sums[0] += sum(c[2] for c in self.patch.corrections(rho))
        kin = self.kinetic_energy(orb_up, occ.occupations_up) + self.kinetic_energy(orb_dn, occ.occupations_down)
        enl = 0.0 if local_only else (self.nonlocal_energy(orb_up, occ.occupations_up)
                                      + self.nonlocal_energy(orb_dn, occ.occupations_down))
        eloc, eh, exc = float(sums[0]), 0.5 * float(sums[1]), float(sums[2])
        total = kin + eloc + enl + eh + exc + self.e_ii
        return SinglePointEnergyComponents(kin, eloc, enl, eh, exc, self.e_ii, total), hartree, lsda


# ----------------------------------------------------------------- start and mixing
def h2_trial_orbitals_device(case, grid_geometry) -> torch.Tensor:
    """Bonding / antibonding exp(-0.8 r^2) pair, W-orthonormalised (``driver.py:705-734``)."""

    dg = device_grid(grid_geometry)
    x, y, z = dg.x, dg.y, dg.z
    f = [torch.exp(-0.8 * ((x - a.position[0]) ** 2 + (y - a.position[1]) ** 2 + (z - a.position[2]) ** 2))
         for a in case.geometry.atoms]
    bonding, anti = f[0] + f[1], f[0] - f[1]
    la = BlockLA(dg)
    if float(torch.sqrt(torch.clamp(la.gram(anti[None], anti[None]), min=0.0)).item()) < 1.0e-12:
        c = dg.reference_center if not dg.monitor else None
        if c is None:
            b = dg.box_bounds
            c = (0.5 * (b[0][0] + b[0][1]), 0.5 * (b[1][0] + b[1][1]), 0.5 * (b[2][0] + b[2][1]))
        zs = z - c[2]
        anti = zs * torch.exp(-0.6 * ((x - c[0]) ** 2 + (y - c[1]) ** 2 + zs * zs))
    return orthonormalize_device(la, torch.stack([bonding, anti]).contiguous(), require_full_rank=True)


def atomic_gaussian_density_device(case, grid_geometry, electrons: float, exponent: float = 1.0) -> torch.Tensor:
    """Superposition of valence-charge-weighted exp(-a r^2) atomic densities, scaled to ``electrons``."""

    dg = device_grid(grid_geometry)
    pseudo = load_case_gth_pseudo_data(case)
    rho = torch.zeros(dg.n, dtype=torch.float64, device=dg.device)
    for a in case.geometry.atoms:
        r2 = (dg.x - a.position[0]) ** 2 + (dg.y - a.position[1]) ** 2 + (dg.z - a.position[2]) ** 2
        rho += pseudo[a.element].ionic_charge * torch.exp(-exponent * r2)
    if electrons == 0.0:
        return torch.zeros_like(rho)
    integral = torch.sum(rho * dg.cell_volumes).reshape(1)
    return renormalize_device(dg, rho, float(electrons), integral)


# ----------------------------------------------------------------- the SCF loop
_HOST = lambda t, shape: None if t is None else t.to(torch.float64).cpu().numpy().reshape(shape)  # noqa: E731


def _summary(res, channel, k, prec):
    if res is None:
        return None
    return FixedPotentialSolveSummary(channel, k, "gb300", False, "gb300_block_subspace_iteration",
                                      f"block subspace iteration, {prec} orbitals", bool(res["converged"]),
                                      np.asarray(res["eigenvalues"]), np.asarray(res["residual_norms"]))


def run_scf_device(*args, **kwargs) -> H2ScfResult:
    """One single-point SCF with every field on the device (see :func:`_run_scf_device`)."""

    from .device import held_stream

    with held_stream():
        return _run_scf_device(*args, **kwargs)


def _run_scf_device(case, grid_geometry, spin_label: str, *, precision: str = "fp64", max_iterations: int = 8,
                   mixing: float = 0.6, density_tolerance: float = 2.5e-3, energy_tolerance: float = 1.0e-5,
                   eigensolver_tolerance: float = 5.0e-3, eigensolver_ncv: int | None = 20,
                   eigensolver_max_iterations: int = 400, mixer: str = "linear", diis_depth: int = 6,
                   diis_warmup_iterations: int = 3, eigensolver_ritz: str = "symmetric",
                   kinetic_version: str = "production", include_nonlocal: bool = True, local_only_energy: bool = False,
                   poisson_tolerance: float = 1.0e-8, poisson_max_iterations: int = 400,
                   initial_density: str = "h2_trial", record_fields: bool = True, require_h2: bool = True,
                   functional: str | None = None, bands: int = 0,
                   eigensolver_preconditioner: str = "jacobi", use_monitor_patch: bool = False,
                   patch_parameters=None, adaptive_eigensolver_tolerance: float = 0.0,
                   poisson_warm_start: bool = False, eigensolver_graphs: bool = True,
                   mixer_options: dict | None = None, diagnostics: dict | None = None,
                   singlet_controls: bool = False, cycle_breaker_weight: float | None = None) -> H2ScfResult:
    """One single-point SCF with every field on the device (``driver.py:2953-3159``).

    ``bands`` > occupied count solves for that many lowest states per spin
    channel (the extra ones are unoccupied).  ``singlet_controls`` turns on the A-grid dry
    run's default H2 closed-shell singlet path (``driver.py:3437-3447``, ``:3823-3867``,
    ``:4165-4203``): the lowest two orbitals are solved and the occupied one is tracked through
    their span (:mod:`.active_subspace`), and the baseline update mixes the total density with
    the Hartree-aware weight (:func:`.mixing.closed_shell_singlet_baseline_mix`).  Other spin
    states are unaffected.  ``cycle_breaker_weight`` (with the linear mixer only) blends the
    H2 singlet's mixed densities with the previous step's when its outputs alternate
    (``driver.py:4272-4295``)."""

    if max_iterations <= 0:
        raise ValueError("max_iterations must be positive.")
    if not (0.0 < mixing <= 1.0):
        raise ValueError("mixing must satisfy 0 < mixing <= 1.")
    if density_tolerance <= 0.0 or energy_tolerance <= 0.0 or eigensolver_tolerance <= 0.0:
        raise ValueError("SCF tolerances must be positive.")
    mixer = mixer.strip().lower()
    if mixer not in ("linear", "diis", "anderson", "broyden"):
        raise ValueError(f"mixer must be `linear`, `diis`, `anderson` or `broyden`; received `{mixer}`.")
    occ = resolve_h2_spin_occupations(spin_label, case) if require_h2 else resolve_spin_occupations(spin_label, case)
    t_start = time.perf_counter()
    eng = DeviceScfEngine(case, grid_geometry, occ, precision=precision, kinetic_version=kinetic_version,
                          include_nonlocal=include_nonlocal, functional=functional,
                          poisson_tolerance=poisson_tolerance, poisson_max_iterations=poisson_max_iterations,
                          preconditioner=eigensolver_preconditioner, use_monitor_patch=use_monitor_patch,
                          patch_parameters=patch_parameters, poisson_warm_start=poisson_warm_start)
    eng.eigensolver_graphs = eigensolver_graphs
    eng.ritz = eigensolver_ritz
    na, nb = occ.n_alpha, occ.n_beta
    shape = tuple(grid_geometry.spec.shape)
    if initial_density == "h2_trial":
        trial = h2_trial_orbitals_device(case, grid_geometry)
        if na > trial.shape[0] or nb > trial.shape[0]:
            raise ValueError("The H2 initial guess builder provides only two trial orbitals.")
        guess_up, guess_dn = (trial[:na] if na else None), (trial[:nb] if nb else None)
        up = eng.density(guess_up, occ.occupations_up, na)
        dn = eng.density(guess_dn, occ.occupations_down, nb)
    elif initial_density == "atomic_gaussians":
        guess_up = guess_dn = None
        up = atomic_gaussian_density_device(case, grid_geometry, na)
        dn = atomic_gaussian_density_device(case, grid_geometry, nb)
    else:
        raise ValueError("initial_density must be `h2_trial` or `atomic_gaussians`.")
    singlet = nb > 0 and _is_closed_shell_singlet(occ)
    tracking = bool(singlet_controls) and occ.spin == 0 and na == 1 and nb == 1
    as_config, as_state, as_history, prev_raw = ActiveSubspaceConfig.local_only_h2_singlet_default(), None, [], None
    solve_guess = None
    if tracking and initial_density == "h2_trial":  # driver.py:3495-3505: the two trial orbitals
        solve_guess = trial[: as_config.subspace_size]
    h2_singlet = occ.spin == 0 and na == 1 and nb == 1
    cb_on = cycle_breaker_weight is not None and h2_singlet and mixer == "linear"
    cb_prev, cb_last_mixed, cb_triggered = [], None, []
    mopt = dict(mixer_options or {})
    if mixer == "diis":
        pulay = PulayMixer(eng, diis_depth, diis_warmup_iterations)
    elif mixer == "anderson":
        pulay = AndersonMixer(eng, **mopt)
    elif mixer == "broyden":
        pulay = BroydenMixer(eng, mixing=mixing, **mopt)
    else:
        pulay = None
    if diagnostics is not None:
        diagnostics["mixer"] = pulay
        diagnostics["hartree_iterations"] = eng.poisson_history
        if tracking:
            diagnostics["active_subspace"] = (as_config, as_history)
        diagnostics["cycle_breaker_triggered"] = cb_triggered
    history = []
    prev = None
    converged = False
    res_up = res_dn = None
    orb_up, orb_dn = guess_up, guess_dn
    energy = None
    for it in range(1, max_iterations + 1):
        t_it = time.perf_counter()
        p0, e0 = eng.poisson_iterations, len(eng.eigensolver_iterations)
        rho_in = up + dn
        hart = eng.hartree(rho_in)
        lx = eng.xc(up, dn)
        vbase = eng.vloc
        if eng.patch is not None:  # frozen patch embedding of the input density
            vbase = eng.vloc + eng.patch.embedding_field(rho_in, eng.patch.corrections(rho_in))[0]
        # optional adaptive tolerance: orbitals of a density far from self-consistency
        # need not be converged further than that density (max(tol, f * last residual))
        tol_it = eigensolver_tolerance
        if adaptive_eigensolver_tolerance > 0.0 and history:
            tol_it = max(eigensolver_tolerance, adaptive_eigensolver_tolerance * history[-1].density_residual)
        elif adaptive_eigensolver_tolerance > 0.0:
            tol_it = max(eigensolver_tolerance, 1.0e-2)
        kw = dict(tolerance=tol_it, max_iterations=eigensolver_max_iterations, ncv=eigensolver_ncv)
        if tracking:  # driver.py:3739-3745, 3823-3867
            res_up = eng.eigensolve(vbase + hart.potential + lx["v_up"], max(as_config.subspace_size, bands),
                                    solve_guess, **kw)
            raw = res_up["orbitals"][: as_config.subspace_size]
            sel = (initialize_active_subspace(raw_subspace_orbitals=raw, config=as_config) if as_state is None else
                   update_active_subspace(raw_subspace_orbitals=raw, state=as_state, weights=eng.dg.cell_volumes))
            as_state, orb_up = sel.state, sel.occupied_orbitals
            ev = np.asarray(res_up["eigenvalues"], dtype=np.float64)
            gap = float(ev[1] - ev[0]) if prev_raw is not None and ev.size >= 2 else None  # driver.py:1532-1562
            as_history.append(MonitorGridActiveSubspaceIterationDiagnostics(
                it, as_config.subspace_size, as_config.target_occupied_count, sel.raw_occupied_overlap_abs,
                sel.best_in_subspace_occupied_overlap_abs, sel.internal_rotation_angle_deg,
                sel.projector_drift_frobenius_norm, sel.subspace_rotation_max_angle_deg, gap, sel.verdict))
            prev_raw = raw
            solve_guess = res_up["orbitals"][: as_config.subspace_size]  # driver.py:4880-4886
        else:
            res_up = eng.eigensolve(vbase + hart.potential + lx["v_up"], max(na, bands), orb_up, **kw) if na else None
            orb_up = res_up["orbitals"] if na else None
        if singlet:
            res_dn, orb_dn = None, orb_up
        elif nb:
            res_dn = eng.eigensolve(vbase + hart.potential + lx["v_down"], max(nb, bands), orb_dn, **kw)
            orb_dn = res_dn["orbitals"]
        up_out = eng.density(orb_up, occ.occupations_up, na)
        dn_out = eng.density(orb_dn, occ.occupations_down, nb)
        resid = residual_device(eng.dg, up, dn, up_out, dn_out)
        energy, hart_out, lx_out = eng.energy(up_out, dn_out, orb_up, orb_dn, local_only=local_only_energy)
        change = None if prev is None else energy.total - prev
        if tracking:  # driver.py:4165-4203: Hartree-aware mixing of the total density
            vbase_out = eng.vloc
            if eng.patch is not None:
                rho_out = up_out + dn_out
                vbase_out = eng.vloc + eng.patch.embedding_field(rho_out, eng.patch.corrections(rho_out))[0]
            d_h = hart_out.potential - hart.potential
            d_xc = lx_out["v_up"] - lx["v_up"]
            share = singlet_hartree_tail_channel_shares(d_h, d_xc, (vbase_out - vbase) + d_h + d_xc,
                                                        eng.dg.cell_volumes)[0]
            ratio = previous_density_residual_ratio(history, float(resid))
            mixed_up, mixed_dn, _ = closed_shell_singlet_baseline_mix(eng.renormalized, occ, up, dn, up_out, dn_out,
                                                                      mixing, share, ratio)
        else:
            mixed_up = eng.renormalized((1.0 - mixing) * up + mixing * up_out, na)
            mixed_dn = eng.renormalized((1.0 - mixing) * dn + mixing * dn_out, nb)
        if cb_on:  # driver.py:4272-4295, with the alternation test of :1177-1206
            dist = lambda a, b, c, d: residual_device(eng.dg, a, b, c, d)  # noqa: E731
            if detect_singlet_alternation(cb_prev, up_out, dn_out, change, dist):
                mixed_up, mixed_dn = cycle_breaker_mix(eng.renormalized, occ, mixed_up, mixed_dn, *cb_last_mixed,
                                                       float(cycle_breaker_weight))
                cb_triggered.append(it)
            cb_prev = (cb_prev + [(up_out, dn_out, change)])[-2:]
            cb_last_mixed = (mixed_up, mixed_dn)
        if pulay is not None:
            mixed_up, mixed_dn = pulay(mixed_up, mixed_dn, up_out - up, dn_out - dn)
        done = resid < density_tolerance and (change is None or abs(change) < energy_tolerance)
        rec = [_HOST(a, shape) if record_fields else None for a in (up, dn, up_out, dn_out, mixed_up, mixed_dn)]
        history.append(ScfIterationRecord(
            it, *rec, float(resid), energy, None if change is None else float(change),
            _summary(res_up, "up", na, eng.prec),
            _summary(res_up if singlet else res_dn, "down", nb, eng.prec),
            time.perf_counter() - t_it, tuple(eng.eigensolver_iterations[e0:]), eng.poisson_iterations - p0))
        if done:
            up, dn = up_out, dn_out
            converged = True
            break
        up, dn = mixed_up, mixed_dn
        prev = energy.total
    torch.cuda.current_stream().synchronize()
    wall = time.perf_counter() - t_start
    ev_up = np.asarray(res_up["eigenvalues"]) if res_up is not None else np.zeros(0)
    ev_dn = ev_up.copy() if singlet else (np.asarray(res_dn["eigenvalues"]) if res_dn is not None else np.zeros(0))
    empty = np.zeros((0,) + shape)
    # the last step's eigensolver results, shaped as the reference reports them (driver.py:3126,
    # :4792: the singlet's down channel is its up solve); host copies only when fields are recorded
    solve_up = solve_dn = None
    if record_fields:
        def solve(res):
            return _solve_result(res, None, len(res["eigenvalues"]), tol_it, "gb300", None, None, grid_geometry,
                                 eng.prec)

        solve_up = solve(res_up) if res_up is not None else None
        solve_dn = solve_up if singlet else (solve(res_dn) if res_dn is not None else None)
    return H2ScfResult(
        converged, occ.label, occ.spin, occ, len(history), tuple(history), ev_up, ev_dn,
        _HOST(orb_up, (-1,) + shape) if na else empty, _HOST(orb_dn, (-1,) + shape) if nb else empty,
        _HOST(up, shape), _HOST(dn, shape), energy, solve_up, solve_dn, wall, eng.prec)


# ----------------------------------------------------------------- drop-in host API
def _host_orbitals(orbitals, geom, count):
    if count == 0:
        return None
    from .ks import validate_orbital_block

    block = validate_orbital_block(orbitals, geom)
    if block.shape[0] < count:
        raise ValueError("Not enough orbitals were provided for the requested occupations.")
    dg = device_grid(geom)
    return torch.as_tensor(np.ascontiguousarray(block[:count], dtype=np.float64), device=dg.device).reshape(count, -1)


def _energy_host(rho_up, rho_down, orbitals_up, orbitals_down, occupations, grid_geometry, case, *, local_only,
                 kinetic_version, poisson_tolerance, poisson_max_iterations, precision, use_monitor_patch=False,
                 patch_parameters=None):
    from .poisson import validate_density_field

    eng = DeviceScfEngine(case, grid_geometry, occupations, precision=precision, kinetic_version=kinetic_version,
                          include_nonlocal=not local_only, poisson_tolerance=poisson_tolerance,
                          poisson_max_iterations=poisson_max_iterations, use_monitor_patch=use_monitor_patch,
                          patch_parameters=patch_parameters)
    dev = eng.dg.device
    up = torch.as_tensor(validate_density_field(rho_up, grid_geometry, "rho_up").reshape(-1), device=dev)
    dn = torch.as_tensor(validate_density_field(rho_down, grid_geometry, "rho_down").reshape(-1), device=dev)
    up, dn = eng.renormalized(up, occupations.n_alpha), eng.renormalized(dn, occupations.n_beta)
    ou = _host_orbitals(orbitals_up, grid_geometry, occupations.n_alpha)
    od = _host_orbitals(orbitals_down, grid_geometry, occupations.n_beta)
    return eng.energy(up, dn, ou, od, local_only=local_only)[0]


def evaluate_single_point_energy(rho_up, rho_down, orbitals_up, orbitals_down, occupations, grid_geometry,
                                 case=H2_BENCHMARK_CASE, *, poisson_tolerance: float = 1.0e-8,
                                 poisson_max_iterations: int = 400) -> SinglePointEnergyComponents:
    """Full single-point energy (``driver.py:905-1015``) with device kernels."""

    _validate_h2_case(case)
    return _energy_host(rho_up, rho_down, orbitals_up, orbitals_down, occupations, grid_geometry, case,
                        local_only=False, kinetic_version="production", poisson_tolerance=poisson_tolerance,
                        poisson_max_iterations=poisson_max_iterations, precision="fp64")


def evaluate_static_local_single_point_energy(rho_up, rho_down, orbitals_up, orbitals_down, occupations,
                                             grid_geometry, case=H2_BENCHMARK_CASE, *, use_monitor_patch: bool = False,
                                             patch_parameters=None, kinetic_version: str = "production",
                                             hartree_backend: str = "python",
                                             use_jax_hartree_cached_operator: bool = False,
                                             jax_hartree_cg_impl: str = "baseline",
                                             jax_hartree_cg_preconditioner: str = "none",
                                             jax_hartree_line_preconditioner_impl: str = "baseline",
                                             poisson_tolerance: float = 1.0e-8,
                                             poisson_max_iterations: int = 400) -> SinglePointEnergyComponents:
    """Local-only energy T_s + E_loc + E_H + E_xc + E_II (``driver.py:2668-2810``)."""

    _validate_h2_case(case)
    return _energy_host(rho_up, rho_down, orbitals_up, orbitals_down, occupations, grid_geometry, case,
                        local_only=True, kinetic_version=kinetic_version, poisson_tolerance=poisson_tolerance,
                        poisson_max_iterations=poisson_max_iterations, precision="fp64",
                        use_monitor_patch=use_monitor_patch and is_monitor_geometry(grid_geometry),
                        patch_parameters=patch_parameters)


def build_h2_initial_density_guess(occupations: SpinOccupations, case=H2_BENCHMARK_CASE, grid_geometry=None):
    """(rho_up, rho_down, orbitals_up, orbitals_down) of the H2 trial pair (``driver.py:737-769``)."""

    from .grid import build_default_h2_grid_geometry

    _validate_h2_case(case)
    if grid_geometry is None:
        grid_geometry = build_default_h2_grid_geometry(case)
    shape = tuple(grid_geometry.spec.shape)
    trial = h2_trial_orbitals_device(case, grid_geometry)
    na, nb = occupations.n_alpha, occupations.n_beta
    if na > trial.shape[0] or nb > trial.shape[0]:
        raise ValueError("The current H2 initial guess builder provides only two trial orbitals.")
    eng = DeviceScfEngine(case, grid_geometry, occupations, include_nonlocal=False)
    up = eng.density(trial[:na] if na else None, occupations.occupations_up, na)
    dn = eng.density(trial[:nb] if nb else None, occupations.occupations_down, nb)
    empty = np.zeros((0,) + shape)
    return (_HOST(up, shape), _HOST(dn, shape), _HOST(trial[:na], (-1,) + shape) if na else empty,
            _HOST(trial[:nb], (-1,) + shape) if nb else empty)


def run_h2_minimal_scf(spin_label: str, case=H2_BENCHMARK_CASE, grid_geometry=None, max_iterations: int = 8,
                       mixing: float = 0.6, density_tolerance: float = 2.5e-3, energy_tolerance: float = 1.0e-5,
                       eigensolver_tolerance: float = 5.0e-3, eigensolver_ncv: int = 20, *, precision: str = "fp64",
                       mixer: str = "linear", poisson_tolerance: float = 1.0e-8,
                       poisson_max_iterations: int = 400, eigensolver_ritz: str = "symmetric") -> H2ScfResult:
    """Drop-in for ``run_h2_minimal_scf`` (``driver.py:2953``): legacy-grid default, full energy.
    ``eigensolver_ritz="right"`` (no reference counterpart) makes the orbitals right
    eigenvectors of the legacy operator, which is not self-adjoint in the cell-volume inner
    product."""

    from .grid import build_default_h2_grid_geometry

    _validate_h2_case(case)
    if grid_geometry is None:
        grid_geometry = build_default_h2_grid_geometry(case)
    return run_scf_device(case, grid_geometry, spin_label, precision=precision, max_iterations=max_iterations,
                          mixing=mixing, density_tolerance=density_tolerance, energy_tolerance=energy_tolerance,
                          eigensolver_tolerance=eigensolver_tolerance, eigensolver_ncv=eigensolver_ncv, mixer=mixer,
                          poisson_tolerance=poisson_tolerance, poisson_max_iterations=poisson_max_iterations,
                          eigensolver_ritz=eigensolver_ritz)


def _dry_run_hartree_options(backend: str, cg_impl: str, preconditioner: str, line_impl: str,
                             cached_operator: bool) -> tuple:
    """The dry run's Hartree-solver options, checked and normalised as ``driver.py:3380-3429``
    does (same messages, ``jacobi`` read as ``diag``, the JAX-only options rejected with
    another backend).  Every accepted combination runs the same GPU solve."""

    nb = backend.strip().lower()
    if nb not in {"python", "jax"}:
        raise ValueError(f"hartree_backend must be `python` or `jax`; received `{backend}`.")
    if cached_operator and nb != "jax":
        raise ValueError("use_jax_hartree_cached_operator requires hartree_backend='jax'.")
    impl = cg_impl.strip().lower()
    if impl not in {"baseline", "jax_loop"}:
        raise ValueError(f"jax_hartree_cg_impl must be `baseline` or `jax_loop`; received `{cg_impl}`.")
    if nb != "jax" and impl != "baseline":
        raise ValueError("jax_hartree_cg_impl requires hartree_backend='jax'.")
    pre = preconditioner.strip().lower()
    if pre not in {"none", "diag", "jacobi", "separable", "line"}:
        raise ValueError("jax_hartree_cg_preconditioner must be `none`, `diag`, `jacobi`, `separable`, or `line`; "
                         f"received `{preconditioner}`.")
    if pre == "jacobi":
        pre = "diag"
    line = line_impl.strip().lower()
    if line not in {"baseline", "optimized"}:
        raise ValueError("jax_hartree_line_preconditioner_impl must be `baseline` or `optimized`; "
                         f"received `{line_impl}`.")
    if nb != "jax" and pre != "none":
        raise ValueError("jax_hartree_cg_preconditioner requires hartree_backend='jax'.")
    if pre != "none" and impl != "jax_loop":
        raise ValueError("jax_hartree_cg_preconditioner currently requires jax_hartree_cg_impl='jax_loop'.")
    return nb, impl, pre, line


def run_h2_monitor_grid_scf_dry_run(spin_label: str, case=H2_BENCHMARK_CASE, grid_geometry=None, *,
                                    patch_parameters=None, max_iterations: int = 10, mixing: float = 0.35,
                                    density_tolerance: float = 5.0e-3, energy_tolerance: float = 5.0e-5,
                                    eigensolver_tolerance: float = 1.0e-3, eigensolver_ncv: int = 20,
                                    kinetic_version: str = "trial_fix", enable_diis: bool = False,
                                    diis_history_length: int = 4, diis_warmup_iterations: int = 3,
                                    enable_anderson: bool = False, anderson_warmup_iterations: int = 3,
                                    anderson_history_length: int = 4, anderson_regularization: float = 1.0e-8,
                                    anderson_damping: float = 0.5, anderson_step_clip_factor: float | None = None,
                                    anderson_reset_on_growth: bool = False, anderson_reset_growth_factor: float = 1.10,
                                    anderson_adaptive_damping_enabled: bool = False,
                                    anderson_min_damping: float = 0.35, anderson_max_damping: float = 0.75,
                                    anderson_acceptance_residual_ratio_threshold: float = 1.02,
                                    anderson_collinearity_cosine_threshold: float = 0.995,
                                    enable_broyden: bool = False, broyden_warmup_iterations: int = 3,
                                    broyden_history_length: int = 4, broyden_regularization: float = 1.0e-8,
                                    broyden_damping: float = 0.5, hartree_backend: str = "python",
                                    jax_hartree_cg_impl: str = "baseline",
                                    jax_hartree_cg_preconditioner: str = "none",
                                    jax_hartree_line_preconditioner_impl: str = "baseline",
                                    precision: str = "fp64", eigensolver_preconditioner: str = "jacobi",
                                    enable_cycle_breaker: bool = False, cycle_breaker_weight: float = 0.5,
                                    **unsupported):
    """A-grid SCF with the near-core patch (``scf/driver.py:3162``): frozen patch embedding in the
    operator, patched local energy, local-only energy (``driver.py:2668-2810``), linear, DIIS,
    Anderson or Broyden-like mixing with the reference's schedules and checks
    (``driver.py:3240-3350``, ``:4297-4430``).  Returns the reference-shaped
    :class:`~isogriddft_gb300.dryrun.H2StaticLocalScfDryRunResult`.  The default grid is the
    reference's 83 x 83 x 101 A-grid from the bit-exact host builder.  The reference's other
    experimental controllers (cycle breaker, Hartree-tail guards, singlet preconditioners,
    active subspace, projector route) are not built; passing one raises."""

    from .dryrun import build_dry_run_result
    from .grid import build_h2_local_patch_development_element_parameters, build_monitor_grid_for_case
    from .pseudo import DEFAULT_MONITOR_PATCH_PARAMETERS

    _validate_h2_case(case)
    if max_iterations <= 0:
        raise ValueError("max_iterations must be positive.")
    if not (0.0 < mixing <= 1.0):
        raise ValueError("mixing must satisfy 0 < mixing <= 1.")
    if not (0.0 <= cycle_breaker_weight <= 1.0):
        raise ValueError("cycle_breaker_weight must satisfy 0 <= cycle_breaker_weight <= 1.")
    if (int(bool(enable_cycle_breaker)) + int(bool(enable_diis)) + int(bool(enable_anderson))
            + int(bool(enable_broyden))) > 1:
        raise ValueError("The minimal monitor-grid dry-run supports at most one of cycle-breaker, DIIS, Anderson, "
                         "or Broyden-like mixing.")
    checks = [
        (diis_warmup_iterations < 0, "diis_warmup_iterations must be non-negative."),
        (diis_history_length < 2, "diis_history_length must be at least 2."),
        (anderson_warmup_iterations < 0, "anderson_warmup_iterations must be non-negative."),
        (anderson_history_length < 2, "anderson_history_length must be at least 2."),
        (anderson_regularization < 0.0, "anderson_regularization must be non-negative."),
        (not (0.0 < anderson_damping <= 1.0), "anderson_damping must satisfy 0 < anderson_damping <= 1."),
        (anderson_step_clip_factor is not None and (not np.isfinite(anderson_step_clip_factor)
                                                    or anderson_step_clip_factor <= 0.0),
         "anderson_step_clip_factor must be positive when provided."),
        (anderson_reset_growth_factor < 1.0, "anderson_reset_growth_factor must be >= 1."),
        (not (0.0 < anderson_min_damping <= anderson_max_damping <= 1.0),
         "Anderson damping bounds must satisfy 0 < min <= max <= 1."),
        (anderson_acceptance_residual_ratio_threshold < 0.0,
         "anderson_acceptance_residual_ratio_threshold must be non-negative."),
        (not (0.0 <= anderson_collinearity_cosine_threshold < 1.0),
         "anderson_collinearity_cosine_threshold must satisfy 0 <= value < 1."),
        (broyden_warmup_iterations < 0, "broyden_warmup_iterations must be non-negative."),
        (broyden_history_length < 2, "broyden_history_length must be at least 2."),
        (broyden_regularization < 0.0, "broyden_regularization must be non-negative."),
        (not (0.0 < broyden_damping <= 1.0), "broyden_damping must satisfy 0 < broyden_damping <= 1."),
        (density_tolerance <= 0.0 or energy_tolerance <= 0.0 or eigensolver_tolerance <= 0.0,
         "SCF tolerances must be positive."),
    ]
    for bad, msg in checks:
        if bad:
            raise ValueError(msg)
    on = [k for k, v in unsupported.items() if v not in (None, False, "none", "baseline", "baseline_linear",
                                                          "python", "corrected_moments")]
    if on:
        raise NotImplementedError(f"dry-run options not built on the GB300 path: {on}")
    hopts = _dry_run_hartree_options(hartree_backend, jax_hartree_cg_impl, jax_hartree_cg_preconditioner,
                                     jax_hartree_line_preconditioner_impl,
                                     bool(unsupported.get("use_jax_hartree_cached_operator", False)))
    if grid_geometry is None:
        grid_geometry = build_monitor_grid_for_case(
            case, shape=(83, 83, 101), box_half_extents=(8.0, 8.0, 10.0),
            element_parameters=build_h2_local_patch_development_element_parameters(), device=False)
    if enable_anderson:
        mixer, mopt = "anderson", dict(
            history_length=anderson_history_length, warmup=anderson_warmup_iterations,
            regularization=anderson_regularization, damping=anderson_damping,
            step_clip_factor=anderson_step_clip_factor, reset_on_growth=anderson_reset_on_growth,
            reset_growth_factor=anderson_reset_growth_factor, adaptive_damping=anderson_adaptive_damping_enabled,
            min_damping=anderson_min_damping, max_damping=anderson_max_damping,
            acceptance_ratio=anderson_acceptance_residual_ratio_threshold,
            collinearity=anderson_collinearity_cosine_threshold)
    elif enable_broyden:
        mixer, mopt = "broyden", dict(history_length=broyden_history_length, warmup=broyden_warmup_iterations,
                                      regularization=broyden_regularization, damping=broyden_damping)
    else:
        mixer, mopt = ("diis" if enable_diis else "linear"), None
    patch = patch_parameters or DEFAULT_MONITOR_PATCH_PARAMETERS
    diag: dict = {}
    t0 = time.perf_counter()
    res = run_scf_device(case, grid_geometry, spin_label, precision=precision, max_iterations=max_iterations,
                         mixing=mixing, density_tolerance=density_tolerance, energy_tolerance=energy_tolerance,
                         eigensolver_tolerance=eigensolver_tolerance, eigensolver_ncv=eigensolver_ncv,
                         mixer=mixer, diis_depth=diis_history_length, diis_warmup_iterations=diis_warmup_iterations,
                         kinetic_version=kinetic_version, include_nonlocal=False, local_only_energy=True,
                         eigensolver_preconditioner=eigensolver_preconditioner, use_monitor_patch=True,
                         patch_parameters=patch, mixer_options=mopt, diagnostics=diag, singlet_controls=True,
                         cycle_breaker_weight=float(cycle_breaker_weight) if enable_cycle_breaker else None)
    options = dict(diis_warmup_iterations=diis_warmup_iterations, diis_history_length=diis_history_length,
                   anderson_warmup_iterations=anderson_warmup_iterations,
                   anderson_history_length=anderson_history_length, anderson_regularization=anderson_regularization,
                   anderson_damping=anderson_damping, anderson_step_clip_factor=anderson_step_clip_factor,
                   anderson_reset_on_growth=anderson_reset_on_growth,
                   anderson_reset_growth_factor=anderson_reset_growth_factor,
                   anderson_adaptive_damping_enabled=anderson_adaptive_damping_enabled,
                   anderson_min_damping=anderson_min_damping, anderson_max_damping=anderson_max_damping,
                   anderson_acceptance_residual_ratio_threshold=anderson_acceptance_residual_ratio_threshold,
                   anderson_collinearity_cosine_threshold=anderson_collinearity_cosine_threshold,
                   broyden_warmup_iterations=broyden_warmup_iterations, broyden_history_length=broyden_history_length,
                   broyden_regularization=broyden_regularization, broyden_damping=broyden_damping)
    return build_dry_run_result(res, kinetic_version=kinetic_version, mixer=diag.get("mixer"), mixer_name=mixer,
                                options=options, hartree_iterations=diag.get("hartree_iterations", []),
                                hartree_options=(hopts[0], hopts[1], hopts[2], hopts[3]), patch_parameters=patch,
                                total_wall=time.perf_counter() - t0, active_subspace=diag.get("active_subspace"),
                                cycle_breaker=(bool(enable_cycle_breaker), float(cycle_breaker_weight),
                                               tuple(diag.get("cycle_breaker_triggered", ()))))
