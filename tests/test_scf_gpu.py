"""GPU parity of the energy assembly and the single-point SCF.

Pins: the reference's recorded static-chain energies on the default legacy
51^3 grid; the reference's own legacy-grid H2 SCF run here (golden
``scf_legacy_h2.json``, made by ``tests/golden/make_golden_scf.py``); the
oracle's energy assembly on the small golden grids.
"""

import json
import os

import numpy as np
import pytest

from tests.conftest import GOLDEN, gpu_available

import oracle.scf as OS

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not gpu_available():
        pytest.skip("needs a CUDA GPU")


@pytest.fixture(scope="module")
def scf_golden():
    return json.load(open(os.path.join(GOLDEN, "scf_legacy_h2.json")))


@pytest.fixture(scope="module")
def default_legacy():
    from isogriddft_gb300.config import H2_BENCHMARK_CASE
    from isogriddft_gb300.grid import build_default_h2_grid_geometry

    return build_default_h2_grid_geometry(H2_BENCHMARK_CASE)


def _bonding(case, geom):
    return OS.bonding_trial_orbital(case, geom)


def test_static_chain_matches_recorded_legacy_values(default_legacy):
    """``audit/baselines.py:819-822``: T, E_loc, E_H, E_xc of the singlet trial density on 51^3."""

    from isogriddft_gb300 import scf
    from isogriddft_gb300.config import H2_BENCHMARK_CASE

    psi = _bonding(H2_BENCHMARK_CASE, default_legacy)
    occ = scf.resolve_h2_spin_occupations("singlet")
    rho = psi * psi
    e = scf.evaluate_single_point_energy(rho, rho, psi[None], psi[None], occ, default_legacy,
                                         poisson_tolerance=1e-12, poisson_max_iterations=4000)
    # recorded values are for one electron pair in one orbital: T and E_loc count both spins
    assert abs(e.kinetic - 1.995064629672) < 1e-9
    assert abs(e.local_ionic - -4.347356525602) < 1e-9
    assert abs(e.hartree - 1.748670071699) < 1e-8
    assert abs(e.xc - -0.869107874980) < 1e-9
    assert e.nonlocal_ionic == 0.0
    assert abs(e.ion_ion_repulsion - 1.0 / 1.4) < 1e-15


@pytest.mark.parametrize("grid", ["legacy", "monitor"])
def test_energy_assembly_matches_oracle(grid, legacy_geom, monitor_geom, golden_legacy, golden_monitor):
    from isogriddft_gb300 import scf
    from isogriddft_gb300.config import H2_BENCHMARK_CASE

    geom, g = (legacy_geom, golden_legacy) if grid == "legacy" else (monitor_geom, golden_monitor)
    psi = g["psi"]
    rnd = g["rnd"] if grid == "monitor" else g["rnd"][None]
    second = OS.renormalize(rnd[0] ** 2, 1.0, geom) ** 0.5  # a second, positive orbital-like field
    occ = scf.resolve_h2_spin_occupations("triplet")
    up = psi * psi + second * second
    dn = np.zeros_like(up)
    orbs = np.stack([psi, second])
    if grid == "legacy":
        e = scf.evaluate_single_point_energy(up, dn, orbs, orbs[:0], occ, geom, poisson_tolerance=1e-13,
                                             poisson_max_iterations=4000)
        ref = OS.single_point_energy(up, dn, orbs, orbs[:0], (1.0, 1.0), (), H2_BENCHMARK_CASE, geom, "production")
    else:
        e = scf.evaluate_static_local_single_point_energy(up, dn, orbs, orbs[:0], occ, geom,
                                                         kinetic_version="trial_fix", poisson_tolerance=1e-13,
                                                         poisson_max_iterations=4000)
        ref = OS.single_point_energy(up, dn, orbs, orbs[:0], (1.0, 1.0), (), H2_BENCHMARK_CASE, geom, "trial_fix",
                                     local_only=True)
    for k in ("kinetic", "local_ionic", "nonlocal_ionic", "hartree", "xc", "ion_ion_repulsion", "total"):
        assert abs(getattr(e, k) - ref[k]) < 1e-10, k


@pytest.mark.parametrize("spin", ["singlet", "triplet"])
def test_legacy_scf_matches_reference_run(spin, scf_golden, default_legacy):
    """The reference's own ``run_h2_minimal_scf`` (defaults and tight) on the default 51^3 grid."""

    from isogriddft_gb300 import scf

    tight = scf_golden.get(f"{spin}_tight")
    if tight is None:
        pytest.skip("no tight reference run recorded")
    # the reference's tight triplet stalls at a density residual of 1.5e-5 with
    # its energy wandering by +-3e-9 (history in the fixture): stop there too
    # (its linear mixing had not settled after 40 steps; Pulay mixing reaches the
    # same fixed point in far fewer)
    dtol, etol, mixer = (1e-6, 1e-10, "linear") if spin == "singlet" else (5e-5, 1e-8, "diis")
    r = scf.run_h2_minimal_scf(spin, grid_geometry=default_legacy, max_iterations=40, density_tolerance=dtol,
                               energy_tolerance=etol, eigensolver_tolerance=1e-7, poisson_tolerance=1e-10,
                               poisson_max_iterations=2000, mixer=mixer)
    assert r.converged
    # The legacy kinetic operator is not self-adjoint in the cell-volume inner
    # product (0.6 % asymmetry), so its Rayleigh-Ritz vectors depend on the
    # search space: the reference's ARPACK Lanczos, the plain block iteration
    # and the preconditioned one settle 1e-7 Ha apart on the triplet's sigma_u
    # orbital (-0.76607041 / -0.76607047 / -0.76607057); the singlet agrees to 1e-9.
    etot, ecomp = (2e-8, 2e-5) if spin == "singlet" else (2e-7, 1e-4)
    assert abs(r.energy.total - tight["energy"]["total"]) < etot
    for k, v in tight["energy"].items():
        assert abs(getattr(r.energy, k) - v) < ecomp, k
    # same cause for the sigma_u eigenvalue of the triplet (Ritz values of a non-self-adjoint
    # operator from different search spaces: -0.091812 here, -0.091725 from ARPACK)
    np.testing.assert_allclose(r.eigenvalues_up, tight["eigenvalues_up"], atol=2e-6 if spin == "singlet" else 2e-4)
    if spin == "triplet":
        # right Ritz pairs (true eigenpairs of the legacy operator, see
        # test_legacy_eigenvalue_definitions): sigma_u -0.0918147, and a total energy 1.9e-8 Ha
        # from the reference's tight run (the symmetrised iteration's is 1.6e-7 away)
        rr = scf.run_h2_minimal_scf(spin, grid_geometry=default_legacy, max_iterations=40, density_tolerance=dtol,
                                    energy_tolerance=etol, eigensolver_tolerance=1e-7, poisson_tolerance=1e-10,
                                    poisson_max_iterations=2000, mixer=mixer, eigensolver_ritz="right")
        assert rr.converged
        assert abs(rr.energy.total - tight["energy"]["total"]) < 5e-8
        np.testing.assert_allclose(rr.eigenvalues_up, tight["eigenvalues_up"], atol=2e-4)
    # mixed precision reaches the same fixed point (its FP32 noise floor puts the density
    # residual near 1e-5, so it stops at the bench's 1e-4 criterion)
    m = scf.run_h2_minimal_scf(spin, grid_geometry=default_legacy, max_iterations=60, density_tolerance=1e-4,
                               energy_tolerance=1e-8, eigensolver_tolerance=1e-4, precision="mixed", mixer="diis",
                               poisson_tolerance=1e-10, poisson_max_iterations=2000)
    assert m.converged
    assert abs(m.energy.total - tight["energy"]["total"]) < 1e-6
    assert abs(m.energy.total - r.energy.total) < 5e-7


def test_legacy_scf_defaults_match_reference(scf_golden, default_legacy):
    """Reference defaults (linear mixing 0.6, loose tolerances): same energy to the stopping accuracy."""

    from isogriddft_gb300 import scf

    ref = scf_golden["singlet_default"]
    r = scf.run_h2_minimal_scf("singlet", grid_geometry=default_legacy)
    assert r.converged
    assert abs(r.energy.total - ref["energy"]["total"]) < 5e-5
    assert abs(r.iteration_count - ref["iterations"]) <= 2
    assert r.history[0].input_rho_up.shape == tuple(default_legacy.spec.shape)


def test_monitor_scf_steps_match_oracle(monitor_geom):
    """Two A-grid SCF steps (trial-fix kinetic, local-only energy) from the H2 trial
    density: the step map (Hartree, LSDA, eigensolve, density, energy, mixing)
    against the oracle's restatement on the 13x13x15 grid."""

    from isogriddft_gb300 import scf
    from isogriddft_gb300.config import H2_BENCHMARK_CASE

    r = scf.run_scf_device(H2_BENCHMARK_CASE, monitor_geom, "triplet", max_iterations=2, mixing=0.4,
                           density_tolerance=1e-12, energy_tolerance=1e-12, eigensolver_tolerance=1e-9,
                           eigensolver_max_iterations=3000, kinetic_version="trial_fix", local_only_energy=True,
                           poisson_tolerance=1e-13, poisson_max_iterations=4000)
    ref = OS.minimal_scf(H2_BENCHMARK_CASE, monitor_geom, 2, 0, closure="trial_fix", max_iterations=2, mixing=0.4,
                         eig_tolerance=1e-9, local_only=True)
    assert r.iteration_count == 2
    for h, (res, e) in zip(r.history, ref["history"]):
        assert abs(h.density_residual - res) < 1e-7
        assert abs(h.energy.total - e) < 1e-8
    np.testing.assert_allclose(r.eigenvalues_up, ref["eigenvalues_up"], atol=1e-8)


def test_legacy_eigenvalue_definitions():
    """Which eigenvalues the legacy route computes.  The legacy kinetic operator is not
    self-adjoint in the cell-volume inner product (a W-asymmetry of a few 1e-4), so Ritz
    values depend on the method.  Fixed potential: a 31^3 legacy grid; local GTH + Hartree +
    LSDA up potential of two atomic Gaussians holding 2 spin-up electrons.
    * ritz="right" (Rayleigh-Ritz on the projected matrices as they are) converges to the
      operator's right eigenpairs H x = lambda x.  Both eigenvalues match the oracle's
      (Arnoldi on the FP64 matrix) to 1e-9 Ha, with residuals below 1e-8.
    * The default symmetrised Rayleigh-Ritz (the reference's JAX route) stalls with a
      residual floor.  Its second Ritz value lies between the right eigenvalue and the
      eigenvalue of the W-symmetric part 1/2 (W^1/2 H W^-1/2 + transpose), which differ by
      about 2e-5 Ha here.
    The reference's legacy route is a third answer: ARPACK's symmetric Lanczos on the
    non-symmetric weighted operator (ks/eigensolver.py:993-1133).  That spread is the
    definition gap behind the triplet sigma_u eigenvalue's 8.7e-5 Ha difference from the
    reference's tight SCF run."""

    from dataclasses import replace

    from oracle import kinetic as OK
    from oracle import poisson as OP
    from oracle import pseudo as OPs
    from oracle import xc as OX
    from isogriddft_gb300 import ks
    from isogriddft_gb300.config import H2_BENCHMARK_CASE
    from isogriddft_gb300.grid import build_default_h2_grid_spec, build_grid_geometry

    geom = build_grid_geometry(replace(build_default_h2_grid_spec(H2_BENCHMARK_CASE), nx=31, ny=31, nz=31))
    rho = sum(np.exp(-((geom.x_points - a.position[0]) ** 2 + (geom.y_points - a.position[1]) ** 2
                       + (geom.z_points - a.position[2]) ** 2)) for a in H2_BENCHMARK_CASE.geometry.atoms)
    rho *= 2.0 / np.sum(rho * geom.cell_volumes)
    dn = np.zeros_like(rho)
    veff = (OPs.local_potential(H2_BENCHMARK_CASE, geom) + OP.solve_legacy(geom, rho, solver="direct")["potential"]
            + OX.lsda(rho, dn)["v_xc_up"])
    h = OK.legacy_hamiltonian_matrix(geom, veff)
    sym = OK.weighted_symmetric_eigenvalues(h, geom, 2)
    right = OK.nonsymmetric_eigenvalues(h, 2)
    zero = np.zeros_like(rho)
    kw = dict(case=H2_BENCHMARK_CASE, local_ionic_potential=veff, hartree_potential=zero, xc_potential=zero,
              max_iterations=4000, precision="fp64")
    res = ks.solve_fixed_potential_static_local_eigenproblem(geom, rho, dn, "up", 2, tolerance=1e-9, ritz="right",
                                                             **kw)
    np.testing.assert_allclose(res.operator_context.effective_local_potential, veff, rtol=0, atol=0)
    assert res.converged and np.max(res.residual_norms) < 1e-8
    np.testing.assert_allclose(res.eigenvalues, right, atol=1e-9)
    # the two definitions agree on the bound state and part on the second one
    assert abs(sym[0] - right[0]) < 1e-7 and abs(sym[1] - right[1]) > 1e-6
    # the symmetrised iteration (the default) stops on its residual floor between them
    s = ks.solve_fixed_potential_static_local_eigenproblem(geom, rho, dn, "up", 2, tolerance=1e-9, **kw)
    assert abs(s.eigenvalues[0] - right[0]) < 1e-7
    lo, hi = min(sym[1], right[1]), max(sym[1], right[1])
    assert lo - 1e-6 <= s.eigenvalues[1] <= hi + 1e-6, (s.eigenvalues, sym, right)
    # the reference's route (oracle restatement): its symmetric Lanczos does not converge the
    # second pair of this operator (residual far above ours)
    from oracle import eigensolver as OE

    ref = OE.eigsh_route(lambda b: np.stack([OK.legacy_kinetic(x, geom) + veff * x for x in b]), H2_BENCHMARK_CASE,
                         geom, 2, tolerance=1e-7)
    assert ref["residual_norms"][1] > 1e-6 > 1e-8 > np.max(res.residual_norms)
