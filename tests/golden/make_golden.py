"""Generate golden fixtures by running the reference IsoGridDFT NumPy path.

Run in a container where the reference source tree is available:

    PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_golden.py <reference checkout>/src

It imports the reference read-only and writes small ``.npz`` files next to
this script.  The fixtures are committed; tests never import the reference.
Reference functions exercised (paths relative to the reference project):
``grid/monitor_builder.py:186`` and ``grid/__init__.py:101`` (grids),
``ops/kinetic.py:147,340,349,279`` (kinetic/Laplacian),
``pseudo/local.py:349`` and ``pseudo/nonlocal.py:286`` (GTH),
``poisson/open_boundary.py:794,1379`` and ``poisson/hartree.py:117`` (Poisson),
``ks/eigensolver.py:818,292,1183`` (guess, orthonormalisation, eigsh route),
``scf/driver.py:663,679,693`` (density helpers).
"""

from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def main(ref_src: str) -> None:
    sys.path.insert(0, ref_src)
    from isogrid.config import H2_BENCHMARK_CASE, N2_AUDIT_CASE
    from isogrid.grid import (build_default_h2_grid_geometry, build_grid_geometry, build_default_h2_grid_spec,
                              build_h2_local_patch_development_element_parameters, build_monitor_grid_for_case)
    from isogrid.ks import eigensolver as eig
    from isogrid.ops import kinetic as kin
    from isogrid.poisson import open_boundary as ob
    from isogrid.poisson.hartree import evaluate_hartree_energy, solve_hartree_potential
    from isogrid.pseudo import evaluate_local_ionic_potential, evaluate_nonlocal_ionic_action
    from isogrid.scf import driver as drv
    from dataclasses import replace

    rng = np.random.default_rng(2024)

    # ------------------------------------------------------------ monitor grid
    shape = (13, 13, 15)
    geom = build_monitor_grid_for_case(
        H2_BENCHMARK_CASE, shape=shape, box_half_extents=(8.0, 8.0, 10.0),
        element_parameters=build_h2_local_patch_development_element_parameters(),
    )
    psi = np.zeros(shape)
    for atom in H2_BENCHMARK_CASE.geometry.atoms:
        d2 = (geom.x_points - atom.position[0]) ** 2 + (geom.y_points - atom.position[1]) ** 2 + (geom.z_points - atom.position[2]) ** 2
        psi += np.exp(-0.8 * d2)
    psi /= np.sqrt(np.sum(psi * psi * geom.cell_volumes))
    rnd = rng.normal(size=(3,) + shape)
    rho = 2.0 * psi * psi
    poisson = solve_hartree_potential(geom, rho)
    legacy_split = ob._compute_multipole_boundary_condition(geom, rho, 2, monitor_boundary_construction_mode="legacy_split")
    vloc = evaluate_local_ionic_potential(H2_BENCHMARK_CASE, geom).total_local_potential
    n2_nl = evaluate_nonlocal_ionic_action(N2_AUDIT_CASE, geom, psi).total_nonlocal_action
    # fixed-potential eigenproblem (trial-fix kinetic, SciPy route) with explicit XC potential
    vxc = -0.7 * np.cbrt(rho)
    res = eig.solve_fixed_potential_static_local_eigenproblem(
        geom, rho / 2, rho / 2, "up", 2, case=H2_BENCHMARK_CASE, xc_potential=vxc,
        hartree_potential=poisson.potential, kinetic_version="trial_fix", tolerance=1e-6, max_iterations=2000,
    )
    ctx = res.operator_context
    guess = eig._build_default_guess_orbitals(ctx, 8)
    dens = drv._build_density_from_occupied_orbitals(res.orbitals, (1.0, 1.0), geom)
    ren = drv._renormalize_density(dens, 2.0, geom)
    resid = drv._density_residual(rho / 2, rho / 2, ren / 2, ren / 2, geom)
    np.savez_compressed(
        os.path.join(HERE, "monitor_h2_13x13x15.npz"),
        shape=np.array(shape), x=geom.x_points, y=geom.y_points, z=geom.z_points, jacobian=geom.jacobian,
        inverse_metric=geom.inverse_metric_tensor, cell_volumes=geom.cell_volumes,
        psi=psi, rnd=rnd,
        kin_prod_psi=kin.apply_monitor_grid_kinetic_operator(psi, geom),
        kin_trial_psi=kin.apply_monitor_grid_kinetic_operator_trial_boundary_fix(psi, geom),
        kin_prod_rnd=np.stack([kin.apply_monitor_grid_kinetic_operator(r, geom) for r in rnd]),
        kin_trial_rnd=np.stack([kin.apply_monitor_grid_kinetic_operator_trial_boundary_fix(r, geom) for r in rnd]),
        lap_prod_rnd0=kin.apply_monitor_grid_laplacian_operator(rnd[0], geom),
        vloc=vloc, n2_nonlocal_psi=n2_nl,
        rho=rho, hartree_potential=poisson.potential, hartree_iterations=poisson.solver_iterations,
        hartree_residual_max=poisson.residual_max,
        boundary_values=poisson.boundary_condition.boundary_values, q=poisson.boundary_condition.total_charge,
        p=poisson.boundary_condition.dipole_moment, Q=poisson.boundary_condition.quadrupole_tensor,
        legacy_split_boundary=legacy_split.boundary_values, hartree_energy=evaluate_hartree_energy(rho, geom, poisson),
        vxc=vxc, eig_values=res.eigenvalues, eig_orbitals=res.orbitals, eig_residuals=res.residual_norms,
        veff=ctx.effective_local_potential, guess8=guess, density=dens, density_renorm=ren, density_residual=resid,
    )

    # ------------------------------------------------------------- legacy grid
    spec = replace(build_default_h2_grid_spec(H2_BENCHMARK_CASE), nx=17, ny=17, nz=19)
    lg = build_grid_geometry(spec)
    lpsi = np.zeros(spec.shape)
    for atom in H2_BENCHMARK_CASE.geometry.atoms:
        d2 = (lg.x_points - atom.position[0]) ** 2 + (lg.y_points - atom.position[1]) ** 2 + (lg.z_points - atom.position[2]) ** 2
        lpsi += np.exp(-0.8 * d2)
    lpsi /= np.sqrt(np.sum(lpsi * lpsi * lg.cell_volumes))
    lrho = 2.0 * lpsi * lpsi
    lpois = solve_hartree_potential(lg, lrho)
    lrnd = rng.normal(size=spec.shape)
    np.savez_compressed(
        os.path.join(HERE, "legacy_h2_17x17x19.npz"),
        shape=np.array(spec.shape), x=lg.x_points, cell_volumes=lg.cell_volumes, psi=lpsi, rnd=lrnd,
        kin_rnd=kin.apply_legacy_kinetic_operator(lrnd, lg), kin_psi=kin.apply_legacy_kinetic_operator(lpsi, lg),
        vloc=evaluate_local_ionic_potential(H2_BENCHMARK_CASE, lg).total_local_potential,
        rho=lrho, hartree_potential=lpois.potential, hartree_iterations=lpois.solver_iterations,
        boundary_values=lpois.boundary_condition.boundary_values, q=lpois.boundary_condition.total_charge,
        p=lpois.boundary_condition.dipole_moment, Q=lpois.boundary_condition.quadrupole_tensor,
        hartree_energy=evaluate_hartree_energy(lrho, lg, lpois),
    )
    default = build_default_h2_grid_geometry(H2_BENCHMARK_CASE)
    np.savez_compressed(os.path.join(HERE, "legacy_default_axes.npz"),
                        x=default.x_coordinates, y=default.y_coordinates, z=default.z_coordinates,
                        wx=default.cell_widths_x, wz=default.cell_widths_z, hx=default.x_point_jacobian,
                        hz=default.z_point_jacobian)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    src = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("ISOGRID_REFERENCE_SRC")
    if not src:
        raise SystemExit(f"usage: python {sys.argv[0]} <reference checkout>/src"
                         " (or set ISOGRID_REFERENCE_SRC)")
    main(src)
