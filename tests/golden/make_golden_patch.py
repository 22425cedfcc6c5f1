"""Golden values for the near-core local-GTH patch, from the reference's own code.

    PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_golden_patch.py /path/to/reference/src

Runs ``evaluate_monitor_grid_local_ionic_potential_with_patch`` and
``evaluate_monitor_grid_local_ionic_potential_with_frozen_patch_field``
(``pseudo/local.py:379-703``) on the 13x13x15 A-grid of ``make_golden.py`` (the
H2 trial density, both the default and the SCF-driver patch parameters) and on
the 67x67x81 A-grid of the recorded static-chain baseline.  Writes
``patch_h2.npz`` beside this script.
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def _trial_density(H2, geom):
    psi = np.zeros(geom.spec.shape)
    for atom in H2.geometry.atoms:
        d2 = (geom.x_points - atom.position[0]) ** 2 + (geom.y_points - atom.position[1]) ** 2 + \
            (geom.z_points - atom.position[2]) ** 2
        psi += np.exp(-0.8 * d2)
    psi /= np.sqrt(np.sum(psi * psi * geom.cell_volumes))
    return 2.0 * psi * psi


def main(src):
    sys.path.insert(0, src)
    from isogrid.config import H2_BENCHMARK_CASE as H2
    from isogrid.grid import build_h2_local_patch_development_element_parameters, build_monitor_grid_for_case
    from isogrid.pseudo import LocalPotentialPatchParameters
    from isogrid.pseudo.local import (evaluate_monitor_grid_local_ionic_potential_with_frozen_patch_field,
                                      evaluate_monitor_grid_local_ionic_potential_with_patch)

    params = {"default": LocalPotentialPatchParameters(),
              "scf": LocalPotentialPatchParameters(patch_radius_scale=0.75, patch_grid_shape=(25, 25, 25),
                                                   correction_strength=1.30, interpolation_neighbors=8)}
    out = {}
    for shape in ((13, 13, 15), (67, 67, 81)):
        geom = build_monitor_grid_for_case(H2, shape=shape, box_half_extents=(8.0, 8.0, 10.0),
                                           element_parameters=build_h2_local_patch_development_element_parameters())
        rho = _trial_density(H2, geom)
        tag = "x".join(map(str, shape))
        for name, p in params.items():
            ev = evaluate_monitor_grid_local_ionic_potential_with_patch(H2, geom, rho, patch_parameters=p)
            out[f"{tag}_{name}_uncorrected"] = ev.uncorrected_local_energy
            out[f"{tag}_{name}_corrected"] = ev.corrected_local_energy
            out[f"{tag}_{name}_atoms"] = np.array([[c.patch_radius_bohr, c.main_grid_patch_energy,
                                                    c.patch_integrated_energy, c.correction_energy,
                                                    c.patch_point_count] for c in ev.atomic_patch_corrections])
            if shape == (13, 13, 15):
                emb = evaluate_monitor_grid_local_ionic_potential_with_frozen_patch_field(
                    H2, geom, rho, patch_parameters=p, patch_evaluation=ev)
                out[f"{tag}_{name}_field"] = emb.correction_field
                out[f"{tag}_{name}_scalings"] = np.array(emb.atomic_scaling_factors)
            print(tag, name, ev.corrected_local_energy, flush=True)
    np.savez_compressed(os.path.join(HERE, "patch_h2.npz"), **out)


if __name__ == "__main__":
    src = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("ISOGRID_REFERENCE_SRC")
    if not src:
        raise SystemExit(f"usage: python {sys.argv[0]} <reference checkout>/src"
                         " (or set ISOGRID_REFERENCE_SRC)")
    main(src)
