"""GPU parity of the near-core local-GTH patch (``pseudo/local.py:379-703``) against the
reference's own values (``tests/golden/make_golden_patch.py``), and the A-grid SCF dry run
that uses it against the reference's recorded triplet total."""

import numpy as np
import pytest

from tests.conftest import gpu_available, load_golden

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not gpu_available():
        pytest.skip("needs a CUDA GPU")


@pytest.fixture(scope="module")
def golden_patch():
    return load_golden("patch_h2.npz")


def _params(name):
    from isogriddft_gb300.pseudo import DEFAULT_MONITOR_PATCH_PARAMETERS, LocalPotentialPatchParameters

    return LocalPotentialPatchParameters() if name == "default" else DEFAULT_MONITOR_PATCH_PARAMETERS


@pytest.mark.parametrize("name", ["default", "scf"])
def test_patch_small_grid_matches_reference(name, golden_patch, golden_monitor, monitor_geom):
    from isogriddft_gb300 import pseudo
    from isogriddft_gb300.config import H2_BENCHMARK_CASE

    g, tag = golden_patch, "13x13x15_" + name
    rho = golden_monitor["rho"]
    ev = pseudo.evaluate_monitor_grid_local_ionic_potential_with_patch(H2_BENCHMARK_CASE, monitor_geom, rho,
                                                                      patch_parameters=_params(name))
    assert abs(ev.uncorrected_local_energy - float(g[tag + "_uncorrected"])) < 1e-12
    assert abs(ev.corrected_local_energy - float(g[tag + "_corrected"])) < 1e-11
    got = np.array([[c.patch_radius_bohr, c.main_grid_patch_energy, c.patch_integrated_energy, c.correction_energy,
                     c.patch_point_count] for c in ev.atomic_patch_corrections])
    np.testing.assert_allclose(got, g[tag + "_atoms"], rtol=1e-12, atol=1e-13)
    emb = pseudo.evaluate_monitor_grid_local_ionic_potential_with_frozen_patch_field(
        H2_BENCHMARK_CASE, monitor_geom, rho, patch_parameters=_params(name), patch_evaluation=ev)
    np.testing.assert_allclose(emb.correction_field, g[tag + "_field"], rtol=1e-12, atol=1e-14)
    np.testing.assert_allclose(emb.atomic_scaling_factors, g[tag + "_scalings"], rtol=1e-12)
    assert abs(emb.embedding_energy_mismatch) < 1e-12


@pytest.fixture(scope="module")
def agrid67():
    from isogriddft_gb300.config import H2_BENCHMARK_CASE
    from isogriddft_gb300.grid import build_h2_local_patch_development_element_parameters, build_monitor_grid_for_case

    return build_monitor_grid_for_case(H2_BENCHMARK_CASE, shape=(67, 67, 81), box_half_extents=(8.0, 8.0, 10.0),
                                       element_parameters=build_h2_local_patch_development_element_parameters(),
                                       device=True)


def test_patch_recorded_static_chain_value(golden_patch, agrid67):
    """``audit/baselines.py:834-843``: E_loc with the patch = -4.287134389497 on 67x67x81."""

    import oracle.scf as OS
    from isogriddft_gb300 import pseudo
    from isogriddft_gb300.config import H2_BENCHMARK_CASE

    psi = OS.bonding_trial_orbital(H2_BENCHMARK_CASE, agrid67)
    ev = pseudo.evaluate_monitor_grid_local_ionic_potential_with_patch(
        H2_BENCHMARK_CASE, agrid67, 2.0 * psi * psi, patch_parameters=_params("scf"))
    assert abs(ev.corrected_local_energy - -4.287134389497) < 1e-8
    assert abs(ev.corrected_local_energy - float(golden_patch["67x67x81_scf_corrected"])) < 1e-8
    assert abs(ev.uncorrected_local_energy - -4.364949512790) < 1e-8


def test_dry_run_scf_matches_recorded_triplet(agrid67):
    """``audit/baselines.py:1969-1980``: A-grid triplet dry run, -1.2214418066604806 after 18 steps
    of linear mixing at the reference's loose tolerances; Pulay mixing to a tighter point here."""

    from isogriddft_gb300 import scf

    r = scf.run_h2_monitor_grid_scf_dry_run("triplet", grid_geometry=agrid67, enable_diis=True, max_iterations=40,
                                            density_tolerance=1e-4, energy_tolerance=1e-7,
                                            eigensolver_tolerance=1e-5)
    assert r.converged
    # the recorded run stopped at the reference's loose tolerances (density 5e-3, energy
    # 5e-5, eigensolver 1e-3) with a BiCGSTAB Hartree solve whose E_H is 1.5e-4 off a
    # tight solve on this grid; this run converges tighter: measured gap 6.2e-4 Ha
    assert abs(r.energy.total - -1.2214418066604806) < 1e-3


@pytest.mark.parametrize("name", ["triplet_diis_tight", "triplet_default", "triplet_anderson_tight",
                                  "triplet_broyden_tight"])
def test_dry_run_scf_matches_reference_run(name, agrid67):
    """The reference's own ``run_h2_monitor_grid_scf_dry_run`` on the same 67x67x81 A-grid
    (``tests/golden/make_golden_dryrun.py``): the first three steps (linear mixing from the
    same start), the converged totals of the Pulay and Anderson runs, the Broyden-like run
    that the reference does not converge (its first extrapolated steps and its climb), the
    first iteration each extrapolating mixer was used in, and the unconverged end of the
    default ten-step run."""

    import json
    import os

    from isogriddft_gb300 import scf
    from tests.conftest import GOLDEN

    runs = json.load(open(os.path.join(GOLDEN, "dryrun_agrid_h2.json")))
    if name not in runs:
        pytest.skip(f"{name} is not in the fixture (tests/golden/make_golden_dryrun.py)")
    ref = runs[name]
    r = scf.run_h2_monitor_grid_scf_dry_run(ref["spin"], grid_geometry=agrid67, **ref["params"])
    for key, got_list in (("anderson_used_iterations", r.anderson_used_iterations),
                          ("broyden_used_iterations", r.broyden_used_iterations)):
        # the extrapolating mixer is used in both runs from its warm-up iteration on
        if ref.get("mixer", {}).get(key):
            assert got_list and got_list[0] == ref["mixer"][key][0], (key, got_list, ref["mixer"][key])
    got = [h.energy.total for h in r.history]
    print(name, r.converged, r.iteration_count, repr(r.energy.total), [round(e, 10) for e in got])
    assert r.converged == ref["converged"]
    # the loose eigensolver tolerance of the default run (1e-3) leaves its per-step totals
    # dependent on the Krylov path at the 1e-5 level (measured 1.4e-5 at the first step)
    early = 1e-5 if ref["params"].get("eigensolver_tolerance", 1e-3) <= 1e-5 else 5e-5
    for k in range(3):
        assert abs(got[k] - ref["history"][k][1]) < early, (k, got[k], ref["history"][k][1])
    if ref["converged"]:
        assert abs(r.energy.total - ref["energy"]["total"]) < 1e-5
        np.testing.assert_allclose(r.eigenvalues_up, ref["eigenvalues_up"], atol=1e-4)
    elif ref.get("mixer", {}).get("broyden_used_iterations"):
        # the reference's Broyden-like run does not settle on this grid: after its first
        # extrapolations the energy climbs from -1.22 to about -0.85 Ha and oscillates; the
        # first extrapolated steps follow the reference's, then both runs show the climb
        assert r.iteration_count == ref["iterations"]
        for k in range(3, 6):
            assert abs(got[k] - ref["history"][k][1]) < 1e-3, (k, got[k], ref["history"][k][1])
        assert max(got[8:]) > -1.1 and max(h[1] for h in ref["history"][8:]) > -1.1
    else:
        assert r.iteration_count == ref["iterations"]
        assert abs(r.energy.total - ref["energy"]["total"]) < 1e-3
