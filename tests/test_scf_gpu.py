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
