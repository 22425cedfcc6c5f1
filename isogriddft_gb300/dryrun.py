"""Reference-shaped result of the A-grid dry-run SCF.

``H2StaticLocalScfDryRunResult`` and ``H2ScfDryRunParameterSummary`` carry the
field names of ``scf/driver.py:174-240`` and ``:357-548`` so that a caller of
the reference's ``run_h2_monitor_grid_scf_dry_run`` reads the same attributes
(``diis_used_iterations``, ``anderson_rejected_iterations``,
``hartree_cg_iterations_history``, ...).  Fields of the reference's
experimental controllers that this path does not build (Hartree-tail guards
and mitigation, singlet preconditioners,
projector route) hold their disabled values; per-phase wall times that the
device path does not split out (its phases overlap on the stream) are None or
empty.  The wall times it does report: the whole run, the average SCF step,
and the Hartree solve count with its iteration history.
"""

from __future__ import annotations

from dataclasses import field, make_dataclass

import numpy as np

_RESIDUAL = "density_fixed_point_residual=rho_out-rho_in"

_SUMMARY_FIELDS = [
    ("grid_shape", tuple), ("box_half_extents_bohr", tuple), ("weight_scale", float), ("radius_scale", float),
    ("patch_radius_scale", float), ("patch_grid_shape", tuple), ("correction_strength", float),
    ("interpolation_neighbors", int), ("kinetic_version", str), ("hartree_backend", str),
    ("use_jax_hartree_cached_operator", bool), ("jax_hartree_cg_impl", str), ("jax_hartree_cg_preconditioner", str),
    ("jax_hartree_line_preconditioner_impl", str), ("use_jax_block_kernels", bool),
    ("use_step_local_static_local_reuse", bool), ("includes_nonlocal", bool), ("cycle_breaker_enabled", bool),
    ("cycle_breaker_weight", float), ("diis_enabled", bool), ("diis_warmup_iterations", int),
    ("diis_history_length", int), ("diis_residual_definition", str), ("anderson_enabled", bool),
    ("anderson_warmup_iterations", int), ("anderson_history_length", int), ("anderson_regularization", float),
    ("anderson_damping", float), ("anderson_step_clip_factor", object), ("anderson_reset_on_growth", bool),
    ("anderson_reset_growth_factor", float), ("anderson_adaptive_damping_enabled", bool),
    ("anderson_min_damping", float), ("anderson_max_damping", float),
    ("anderson_acceptance_residual_ratio_threshold", float), ("anderson_collinearity_cosine_threshold", float),
    ("anderson_residual_definition", str), ("singlet_hartree_tail_mitigation_enabled", bool),
    ("singlet_hartree_tail_mitigation_weight", object), ("singlet_hartree_tail_residual_ratio_trigger", object),
    ("singlet_hartree_tail_projected_ratio_trigger", object), ("singlet_hartree_tail_hartree_share_trigger", object),
    ("broyden_enabled", bool), ("broyden_warmup_iterations", int), ("broyden_history_length", int),
    ("broyden_regularization", float), ("broyden_damping", float), ("broyden_residual_definition", str),
]
_SUMMARY_DEFAULTS = [
    ("hartree_tail_guard_enabled", bool, False), ("hartree_tail_guard_name", object, None),
    ("hartree_tail_guard_strategy", object, None), ("hartree_tail_guard_alpha", object, None),
    ("hartree_tail_guard_residual_ratio_trigger", object, None),
    ("hartree_tail_guard_projected_ratio_trigger", object, None),
    ("hartree_tail_guard_hartree_share_trigger", object, None), ("hartree_tail_guard_hold_steps", object, None),
    ("hartree_tail_guard_exit_residual_ratio", object, None), ("hartree_tail_guard_exit_stable_steps", object, None),
    ("singlet_real_space_preconditioner_enabled", bool, False),
    ("singlet_real_space_preconditioner_strength", object, None),
]
H2ScfDryRunParameterSummary = make_dataclass(
    "H2ScfDryRunParameterSummary", _SUMMARY_FIELDS + _SUMMARY_DEFAULTS, frozen=True,
    namespace={"__doc__": "Fixed parameter summary of the monitor-grid SCF dry run (``driver.py:174-240``)."})

# the result: fields the run fills, then measured-or-absent timing fields, then the
# disabled experimental-controller fields (all with defaults)
_RESULT_FIELDS = [
    ("path_type", str), ("kinetic_version", str), ("includes_nonlocal", bool), ("spin_state_label", str),
    ("spin", int), ("occupations", object), ("parameter_summary", object), ("hartree_backend", str),
    ("use_jax_hartree_cached_operator", bool), ("jax_hartree_cg_impl", str), ("jax_hartree_cg_preconditioner", str),
    ("jax_hartree_line_preconditioner_impl", str), ("use_jax_block_kernels", bool),
    ("use_step_local_static_local_reuse", bool), ("cycle_breaker_enabled", bool), ("cycle_breaker_weight", float),
    ("cycle_breaker_triggered_iterations", tuple), ("diis_enabled", bool), ("diis_warmup_iterations", int),
    ("diis_history_length", int), ("diis_residual_definition", str), ("diis_used_iterations", tuple),
    ("diis_history_sizes", tuple), ("diis_fallback_iterations", tuple), ("anderson_enabled", bool),
    ("anderson_warmup_iterations", int), ("anderson_history_length", int), ("anderson_regularization", float),
    ("anderson_damping", float), ("anderson_step_clip_factor", object), ("anderson_reset_on_growth", bool),
    ("anderson_reset_growth_factor", float), ("anderson_adaptive_damping_enabled", bool),
    ("anderson_min_damping", float), ("anderson_max_damping", float),
    ("anderson_acceptance_residual_ratio_threshold", float), ("anderson_collinearity_cosine_threshold", float),
    ("anderson_residual_definition", str), ("anderson_used_iterations", tuple), ("anderson_history_sizes", tuple),
    ("anderson_filtered_history_sizes", tuple), ("anderson_fallback_iterations", tuple),
    ("anderson_rejected_iterations", tuple), ("anderson_reset_iterations", tuple),
    ("anderson_effective_damping_history", tuple), ("anderson_projected_residual_ratio_history", tuple),
    ("singlet_hartree_tail_mitigation_enabled", bool), ("singlet_hartree_tail_mitigation_weight", object),
    ("singlet_hartree_tail_residual_ratio_trigger", object), ("singlet_hartree_tail_projected_ratio_trigger", object),
    ("singlet_hartree_tail_hartree_share_trigger", object),
    ("singlet_hartree_tail_mitigation_triggered_iterations", tuple),
    ("singlet_hartree_tail_hartree_share_history", tuple), ("singlet_hartree_tail_residual_ratio_history", tuple),
    ("singlet_hartree_tail_projected_ratio_history", tuple), ("broyden_enabled", bool),
    ("broyden_warmup_iterations", int), ("broyden_history_length", int), ("broyden_regularization", float),
    ("broyden_damping", float), ("broyden_residual_definition", str), ("broyden_used_iterations", tuple),
    ("broyden_history_sizes", tuple), ("broyden_fallback_iterations", tuple), ("converged", bool),
    ("iteration_count", int), ("history", tuple), ("energy_history", tuple), ("density_residual_history", tuple),
    ("eigenvalues_up", np.ndarray), ("eigenvalues_down", np.ndarray), ("orbitals_up", np.ndarray),
    ("orbitals_down", np.ndarray), ("rho_up", np.ndarray), ("rho_down", np.ndarray), ("energy", object),
    ("lowest_eigenvalue", object), ("solve_up", object), ("solve_down", object),
    ("total_wall_time_seconds", float), ("average_iteration_wall_time_seconds", object),
]
_NONE_TIMES = [
    "eigensolver_wall_time_seconds", "static_local_prepare_wall_time_seconds", "hartree_solve_wall_time_seconds",
    "local_ionic_resolve_wall_time_seconds", "xc_resolve_wall_time_seconds", "energy_evaluation_wall_time_seconds",
    "kinetic_energy_wall_time_seconds", "local_ionic_energy_wall_time_seconds", "hartree_energy_wall_time_seconds",
    "xc_energy_wall_time_seconds", "ion_ion_energy_wall_time_seconds", "density_update_wall_time_seconds",
    "bookkeeping_wall_time_seconds",
]
_NONE_AVERAGES = [
    "average_hartree_solve_wall_time_seconds", "first_hartree_solve_wall_time_seconds",
    "repeated_hartree_solve_average_wall_time_seconds", "repeated_hartree_solve_min_wall_time_seconds",
    "repeated_hartree_solve_max_wall_time_seconds", "average_hartree_cg_iterations", "first_hartree_cg_iterations",
    "repeated_hartree_cg_iteration_average", "average_hartree_boundary_condition_wall_time_seconds",
    "average_hartree_build_wall_time_seconds", "average_hartree_rhs_assembly_wall_time_seconds",
    "average_hartree_cg_wall_time_seconds", "average_hartree_matvec_call_count",
    "average_hartree_matvec_wall_time_seconds", "average_hartree_matvec_wall_time_per_call_seconds",
    "average_hartree_preconditioner_apply_count", "average_hartree_preconditioner_apply_wall_time_seconds",
    "average_hartree_preconditioner_apply_wall_time_per_call_seconds",
    "average_hartree_preconditioner_setup_wall_time_seconds",
    "average_hartree_preconditioner_axis_reorder_wall_time_seconds",
    "average_hartree_preconditioner_tridiagonal_solve_wall_time_seconds",
    "average_hartree_preconditioner_other_overhead_wall_time_seconds",
]
_EMPTY_HISTORIES = [
    "hartree_solve_wall_time_seconds_history", "hartree_cg_iterations_history",
    "hartree_boundary_condition_wall_time_seconds_history", "hartree_build_wall_time_seconds_history",
    "hartree_rhs_assembly_wall_time_seconds_history", "hartree_cg_wall_time_seconds_history",
    "hartree_matvec_call_count_history", "hartree_matvec_wall_time_seconds_history",
    "hartree_preconditioner_apply_count_history", "hartree_preconditioner_apply_wall_time_seconds_history",
    "hartree_preconditioner_setup_wall_time_seconds_history",
    "hartree_preconditioner_axis_reorder_wall_time_seconds_history",
    "hartree_preconditioner_tridiagonal_solve_wall_time_seconds_history",
    "hartree_preconditioner_other_overhead_wall_time_seconds_history",
]
_NONE_EIGENSOLVER = [
    "eigensolver_subspace_iteration_wall_time_seconds", "eigensolver_orthogonalization_wall_time_seconds",
    "eigensolver_residual_expansion_wall_time_seconds", "eigensolver_rayleigh_ritz_wall_time_seconds",
    "eigensolver_hamiltonian_apply_wall_time_seconds", "eigensolver_projected_matrix_build_wall_time_seconds",
]
_EMPTY_ITERATION_HISTORIES = [
    "solver_backend_iteration_history", "total_step_wall_time_seconds_history",
    "static_local_prepare_iteration_wall_time_seconds", "hartree_solve_iteration_wall_time_seconds",
    "eigensolver_subspace_iteration_iteration_wall_time_seconds",
    "eigensolver_orthogonalization_iteration_wall_time_seconds",
    "eigensolver_residual_expansion_iteration_wall_time_seconds",
    "eigensolver_rayleigh_ritz_iteration_wall_time_seconds", "eigensolver_hamiltonian_apply_iteration_wall_time_seconds",
    "eigensolver_projected_matrix_build_iteration_wall_time_seconds", "eigensolver_iteration_wall_time_seconds",
    "energy_evaluation_iteration_wall_time_seconds", "density_update_iteration_wall_time_seconds",
    "bookkeeping_iteration_wall_time_seconds", "hartree_response_diagnostics_history",
]
_CONTROLLER_DEFAULTS = [
    ("hartree_solve_call_count", int, 0), ("hartree_cached_operator_usage_count", int, 0),
    ("hartree_cached_operator_first_solve_count", int, 0),
    ("hartree_tail_guard_enabled", bool, False), ("hartree_tail_guard_name", object, None),
    ("hartree_tail_guard_strategy", object, None), ("hartree_tail_guard_alpha", object, None),
    ("hartree_tail_guard_residual_ratio_trigger", object, None),
    ("hartree_tail_guard_projected_ratio_trigger", object, None),
    ("hartree_tail_guard_hartree_share_trigger", object, None), ("hartree_tail_guard_hold_steps", object, None),
    ("hartree_tail_guard_exit_residual_ratio", object, None), ("hartree_tail_guard_exit_stable_steps", object, None),
    ("hartree_tail_guard_triggered_iterations", tuple, ()), ("hartree_tail_guard_entry_iterations", tuple, ()),
    ("hartree_tail_guard_exit_iterations", tuple, ()), ("hartree_tail_guard_hold_lengths", tuple, ()),
    ("hartree_tail_guard_active_iteration_history", tuple, ()),
    ("hartree_tail_guard_hartree_share_history", tuple, ()), ("hartree_tail_guard_residual_ratio_history", tuple, ()),
    ("hartree_tail_guard_projected_ratio_history", tuple, ()), ("controller_name", str, "baseline_linear"),
    ("controller_signals_history", tuple, ()), ("controller_charge_mixing_history", tuple, ()),
    ("controller_spin_mixing_history", tuple, ()), ("controller_state_flags_history", tuple, ()),
    ("controller_charge_unbounded_trial_history", tuple, ()), ("controller_charge_trial_history", tuple, ()),
    ("controller_charge_preclip_next_history", tuple, ()), ("controller_charge_postclip_next_history", tuple, ()),
    ("active_subspace_enabled", bool, False), ("active_subspace_size", object, None),
    ("active_subspace_target_occupied_count", object, None), ("active_subspace_diagnostics_history", tuple, ()),
    ("projector_route_enabled", bool, False), ("projector_route_name", object, None),
    ("projector_route_diagnostics_history", tuple, ()), ("projector_route_guard_enabled", bool, False),
    ("projector_route_guard_active_iteration_history", tuple, ()),
    ("projector_route_guard_trigger_iterations", tuple, ()), ("projector_route_guard_reason_history", tuple, ()),
]
H2StaticLocalScfDryRunResult = make_dataclass(
    "H2StaticLocalScfDryRunResult",
    _RESULT_FIELDS
    + [(n, object, None) for n in _NONE_TIMES + _NONE_AVERAGES + _NONE_EIGENSOLVER]
    + [(n, tuple, field(default=())) for n in _EMPTY_HISTORIES + _EMPTY_ITERATION_HISTORIES]
    + _CONTROLLER_DEFAULTS,
    frozen=True,
    namespace={"__doc__": "Result of the A-grid static-local SCF dry run, shaped as ``driver.py:357-548``."})


def build_dry_run_result(res, *, kinetic_version: str, mixer, mixer_name: str, options: dict,
                         hartree_iterations: list, hartree_options: tuple, patch_parameters,
                         total_wall: float, active_subspace=None,
                         cycle_breaker=(False, 0.5, ())) -> "H2StaticLocalScfDryRunResult":
    """Assemble the reference-shaped result from a device SCF result (``scf.H2ScfResult``),
    the mixer object and its options; ``active_subspace`` is the (config, per-step
    diagnostics) pair of the singlet tracking when it ran (``driver.py:5267-5276``);
    ``cycle_breaker`` is (enabled, weight, iterations where it blended)."""

    from .grid import (H2_MONITOR_LOCAL_PATCH_BASELINE_BOX_HALF_EXTENTS_BOHR, H2_MONITOR_LOCAL_PATCH_BASELINE_RADIUS_SCALE,
                       H2_MONITOR_LOCAL_PATCH_BASELINE_SHAPE, H2_MONITOR_LOCAL_PATCH_BASELINE_WEIGHT_SCALE)

    backend, cg_impl, cg_pre, line_impl = hartree_options
    o = options
    diis, anderson, broyden = mixer_name == "diis", mixer_name == "anderson", mixer_name == "broyden"
    n_it = len(res.history)
    blank = tuple(0 for _ in range(n_it))

    def attr(name, default=()):
        return tuple(getattr(mixer, name, default)) if mixer is not None else default

    common = dict(
        kinetic_version=kinetic_version, hartree_backend=backend, use_jax_hartree_cached_operator=False,
        jax_hartree_cg_impl=cg_impl, jax_hartree_cg_preconditioner=cg_pre, jax_hartree_line_preconditioner_impl=line_impl,
        use_jax_block_kernels=False, use_step_local_static_local_reuse=False,
        cycle_breaker_enabled=bool(cycle_breaker[0]), cycle_breaker_weight=float(cycle_breaker[1]), diis_enabled=diis,
        diis_warmup_iterations=o["diis_warmup_iterations"],
        diis_history_length=o["diis_history_length"], diis_residual_definition=_RESIDUAL, anderson_enabled=anderson,
        anderson_warmup_iterations=o["anderson_warmup_iterations"], anderson_history_length=o["anderson_history_length"],
        anderson_regularization=o["anderson_regularization"], anderson_damping=o["anderson_damping"],
        anderson_step_clip_factor=o["anderson_step_clip_factor"],
        anderson_reset_on_growth=o["anderson_reset_on_growth"],
        anderson_reset_growth_factor=o["anderson_reset_growth_factor"],
        anderson_adaptive_damping_enabled=o["anderson_adaptive_damping_enabled"],
        anderson_min_damping=o["anderson_min_damping"], anderson_max_damping=o["anderson_max_damping"],
        anderson_acceptance_residual_ratio_threshold=o["anderson_acceptance_residual_ratio_threshold"],
        anderson_collinearity_cosine_threshold=o["anderson_collinearity_cosine_threshold"],
        anderson_residual_definition=_RESIDUAL, singlet_hartree_tail_mitigation_enabled=False,
        singlet_hartree_tail_mitigation_weight=None, singlet_hartree_tail_residual_ratio_trigger=None,
        singlet_hartree_tail_projected_ratio_trigger=None, singlet_hartree_tail_hartree_share_trigger=None,
        broyden_enabled=broyden, broyden_warmup_iterations=o["broyden_warmup_iterations"],
        broyden_history_length=o["broyden_history_length"], broyden_regularization=o["broyden_regularization"],
        broyden_damping=o["broyden_damping"], broyden_residual_definition=_RESIDUAL,
    )
    summary = H2ScfDryRunParameterSummary(
        grid_shape=H2_MONITOR_LOCAL_PATCH_BASELINE_SHAPE,
        box_half_extents_bohr=H2_MONITOR_LOCAL_PATCH_BASELINE_BOX_HALF_EXTENTS_BOHR,
        weight_scale=H2_MONITOR_LOCAL_PATCH_BASELINE_WEIGHT_SCALE,
        radius_scale=H2_MONITOR_LOCAL_PATCH_BASELINE_RADIUS_SCALE,
        patch_radius_scale=float(patch_parameters.patch_radius_scale),
        patch_grid_shape=tuple(patch_parameters.patch_grid_shape),
        correction_strength=float(patch_parameters.correction_strength),
        interpolation_neighbors=int(patch_parameters.interpolation_neighbors), includes_nonlocal=False, **common)
    ev_up, ev_dn = np.asarray(res.eigenvalues_up), np.asarray(res.eigenvalues_down)
    lows = [float(e[0]) for e in (ev_up, ev_dn) if e.size]
    hart = tuple(int(x) for x in hartree_iterations)
    tracking = {}
    if active_subspace is not None:
        cfg, steps = active_subspace
        tracking = dict(active_subspace_enabled=bool(cfg.enabled), active_subspace_size=int(cfg.subspace_size),
                        active_subspace_target_occupied_count=int(cfg.target_occupied_count),
                        active_subspace_diagnostics_history=tuple(steps))
    return H2StaticLocalScfDryRunResult(
        path_type="monitor_a_grid_plus_patch", includes_nonlocal=False, spin_state_label=res.occupations.label,
        spin=res.occupations.spin, occupations=res.occupations, parameter_summary=summary,
        cycle_breaker_triggered_iterations=tuple(cycle_breaker[2]),
        diis_used_iterations=attr("used") if diis else (),
        diis_history_sizes=attr("history_sizes") if diis else blank,
        diis_fallback_iterations=attr("fallback") if diis else (),
        anderson_used_iterations=attr("used") if anderson else (),
        anderson_history_sizes=attr("history_sizes") if anderson else blank,
        anderson_filtered_history_sizes=attr("filtered_sizes") if anderson else blank,
        anderson_fallback_iterations=attr("fallback") if anderson else (),
        anderson_rejected_iterations=attr("rejected") if anderson else (),
        anderson_reset_iterations=attr("resets") if anderson else (),
        anderson_effective_damping_history=attr("effective_damping") if anderson else (),
        anderson_projected_residual_ratio_history=attr("projected_ratios") if anderson else (),
        singlet_hartree_tail_mitigation_triggered_iterations=(), singlet_hartree_tail_hartree_share_history=(),
        singlet_hartree_tail_residual_ratio_history=(), singlet_hartree_tail_projected_ratio_history=(),
        broyden_used_iterations=attr("used") if broyden else (),
        broyden_history_sizes=attr("history_sizes") if broyden else blank,
        broyden_fallback_iterations=attr("fallback") if broyden else (),
        converged=bool(res.converged), iteration_count=n_it, history=tuple(res.history),
        energy_history=tuple(r.energy.total for r in res.history),
        density_residual_history=tuple(r.density_residual for r in res.history),
        eigenvalues_up=ev_up, eigenvalues_down=ev_dn,
        orbitals_up=np.asarray(res.orbitals_up, dtype=np.float64),
        orbitals_down=np.asarray(res.orbitals_down, dtype=np.float64),
        rho_up=np.asarray(res.rho_up, dtype=np.float64), rho_down=np.asarray(res.rho_down, dtype=np.float64),
        energy=res.energy, lowest_eigenvalue=min(lows) if lows else None,
        solve_up=res.solve_up, solve_down=res.solve_down, total_wall_time_seconds=float(total_wall),
        average_iteration_wall_time_seconds=None if n_it == 0 else float(total_wall / n_it),
        hartree_solve_call_count=len(hart), hartree_cg_iterations_history=hart,
        average_hartree_cg_iterations=float(np.mean(hart)) if hart else None,
        first_hartree_cg_iterations=hart[0] if hart else None,
        repeated_hartree_cg_iteration_average=float(np.mean(hart[1:])) if len(hart) > 1 else None,
        total_step_wall_time_seconds_history=tuple(float(r.wall_time_seconds) for r in res.history),
        solver_backend_iteration_history=tuple("gb300_block_subspace" for _ in res.history),
        **tracking, **common)
