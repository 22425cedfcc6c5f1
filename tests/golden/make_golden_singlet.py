"""Generate golden vectors for the H2 singlet controls of the dry run with the reference's own
functions: the active-subspace tracking (``scf/active_subspace.py``), the Hartree-aware
singlet mixing weight and baseline update, and the potential-change channel shares
(``scf/driver.py:1565-1583``, ``:1825-1937``).

Run in a checkout that has the reference sources (read-only):

    PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_golden_singlet.py /path/to/reference/src

On the reference's 7 x 7 x 9 H2 A-grid, a seeded sequence of weighted-orthonormal lowest-two
blocks (two smooth states rotating into each other, with sign flips, an order swap and a step
where a third state leaks in) goes through ``initialize_active_subspace`` and
``update_active_subspace``; seeded densities and potential changes go through the mixing
helpers.  Writes ``singlet_h2.npz`` and ``singlet_h2.json`` beside this script.
"""

import json
import os
import sys
from types import SimpleNamespace

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

# (rotation angle in degrees, leak of the third state, sign of each raw orbital, swap the order);
# the 88-degree step rotates the raw basis inside the tracked span, and the last step (angle None)
# keeps only a 0.12 share of the first state in the span
STEPS = [(0.0, 0.0, (1, 1), False), (8.0, 0.02, (1, -1), False), (20.0, 0.05, (-1, 1), False),
         (35.0, 0.0, (1, 1), True), (88.0, 0.0, (1, 1), False), (50.0, 0.1, (-1, -1), False),
         (None, 0.12, (1, 1), False)]
MIX_CASES = [(0.35, None, None), (0.35, 0.40, 0.80), (0.35, 0.70, None), (0.35, 0.95, 1.00), (0.35, None, 1.20),
             (0.05, 0.90, 1.10), (1.00, 0.60, 0.95), (0.20, float("nan"), 0.93)]


def main(src):
    sys.path.insert(0, src)
    from isogrid.config import H2_BENCHMARK_CASE
    from isogrid.grid import build_h2_local_patch_development_element_parameters, build_monitor_grid_for_case
    from isogrid.ks import weighted_orthonormalize_orbitals
    from isogrid.scf import active_subspace as A
    from isogrid.scf import driver as D

    geom = build_monitor_grid_for_case(H2_BENCHMARK_CASE, shape=(7, 7, 9), box_half_extents=(8.0, 8.0, 10.0),
                                       element_parameters=build_h2_local_patch_development_element_parameters())
    shape = geom.spec.shape
    rng = np.random.default_rng(11)
    r2 = geom.x_points ** 2 + geom.y_points ** 2 + geom.z_points ** 2
    base = np.stack([np.exp(-0.3 * r2), geom.z_points * np.exp(-0.3 * r2), geom.x_points * np.exp(-0.25 * r2)])
    base = base + 0.05 * rng.normal(size=base.shape)
    phi = weighted_orthonormalize_orbitals(base, grid_geometry=geom)
    out = {"cell_volumes": np.asarray(geom.cell_volumes, dtype=np.float64)}
    meta = {"verdicts": []}
    config = A.ActiveSubspaceConfig.local_only_h2_singlet_default()
    state = None
    for t, (deg, leak, signs, swap) in enumerate(STEPS):
        if deg is None:
            a, b = phi[1], leak * phi[0] + np.sqrt(1.0 - leak * leak) * phi[2]
        else:
            th = np.radians(deg)
            a = np.cos(th) * phi[0] + np.sin(th) * phi[1]
            b = -np.sin(th) * phi[0] + np.cos(th) * phi[1]
            a = np.sqrt(1.0 - leak * leak) * a + leak * phi[2]
        raw = np.stack([signs[0] * a, signs[1] * b])
        if swap:
            raw = np.ascontiguousarray(raw[::-1])  # rows stay weighted-orthonormal, as eigenvectors are
        sel = (A.initialize_active_subspace(raw_subspace_orbitals=raw, grid_geometry=geom, config=config)
               if state is None else
               A.update_active_subspace(raw_subspace_orbitals=raw, state=state, grid_geometry=geom))
        state = sel.state
        out[f"raw_{t}"] = raw
        out[f"occupied_{t}"] = np.asarray(sel.occupied_orbitals, dtype=np.float64)
        out[f"aligned_{t}"] = np.asarray(sel.aligned_subspace_orbitals, dtype=np.float64)
        out[f"diag_{t}"] = np.asarray([sel.raw_occupied_overlap_abs, sel.best_in_subspace_occupied_overlap_abs,
                                       sel.internal_rotation_angle_deg, sel.projector_drift_frobenius_norm,
                                       sel.subspace_rotation_max_angle_deg, *sel.subspace_overlap_singular_values],
                                      dtype=np.float64)
        meta["verdicts"].append(sel.verdict)

    out["mix_factor"] = np.asarray([D._closed_shell_singlet_hartree_aware_mixing_factor(
        baseline_mixing=m, hartree_share=h, previous_residual_ratio=r) for m, h, r in MIX_CASES])
    meta["mix_cases"] = [[m, None if h is None else (str(h) if not np.isfinite(h) else h), r]
                         for m, h, r in MIX_CASES]

    singlet = D.resolve_h2_spin_occupations("singlet", H2_BENCHMARK_CASE)
    triplet = D.resolve_h2_spin_occupations("triplet", H2_BENCHMARK_CASE)
    dens = np.abs(rng.normal(1.0, 0.3, size=(4,) + shape))
    out["mix_in"] = dens
    for label, occ in (("singlet", singlet), ("triplet", triplet)):
        up, dn = D._renormalize_density(dens[0], occ.n_alpha, geom), D._renormalize_density(dens[1], occ.n_beta, geom)
        uo, do = D._renormalize_density(dens[2], occ.n_alpha, geom), D._renormalize_density(dens[3], occ.n_beta, geom)
        res = D._apply_closed_shell_singlet_hartree_aware_baseline_mixing(
            occupations=occ, rho_up_current=up, rho_down_current=dn, rho_up_output=uo, rho_down_output=do,
            grid_geometry=geom, baseline_mixing=0.35, hartree_share=0.72, previous_residual_ratio=0.97)
        out[f"mix_{label}"] = np.stack([up, dn, uo, do, res[0], res[1]])

    pots = rng.normal(size=(6,) + shape)
    ctx = lambda h, x, e: SimpleNamespace(hartree_potential=h, xc_potential=x,  # noqa: E731
                                          effective_local_potential=e, grid_geometry=geom)
    out["share_in"] = pots
    out["shares"] = np.asarray(D._estimate_singlet_hartree_tail_channel_shares(
        input_context=ctx(pots[0], pots[1], pots[2]), output_context=ctx(pots[3], pots[4], pots[5])),
        dtype=np.float64)
    out["field_norm"] = np.asarray([D._weighted_field_norm(pots[0], grid_geometry=geom)])

    # cycle-breaker alternation test (driver.py:1177-1206) on seeded output densities
    outs = np.abs(rng.normal(1.0, 0.2, size=(4, 2) + shape))
    outs[2] = outs[0] + 0.01 * rng.normal(size=(2,) + shape)  # the new output returns to two steps back
    out["cb_outputs"] = outs
    # (history as (output index, energy change) oldest first, new output index, new energy change)
    specs = [([(0, None), (1, -0.2)], 2, 0.1), ([(0, None), (1, -0.2)], 2, -0.1), ([(0, None), (1, 0.2)], 2, -0.1),
             ([(0, None), (1, -0.2)], 3, 0.1), ([(1, -0.2)], 2, 0.1), ([(0, None), (1, None)], 2, 0.1),
             ([(0, None), (1, -0.2)], 2, None)]
    meta["cb_cases"] = specs
    meta["cb_detect"] = [bool(D._detect_monitor_grid_singlet_alternation(
        [SimpleNamespace(output_rho_up=outs[i][0], output_rho_down=outs[i][1], energy_change=c) for i, c in hist],
        rho_up_out=outs[k][0], rho_down_out=outs[k][1], energy_change=c, grid_geometry=geom))
        for hist, k, c in specs]

    np.savez_compressed(os.path.join(HERE, "singlet_h2.npz"), **out)
    with open(os.path.join(HERE, "singlet_h2.json"), "w") as f:
        json.dump(meta, f, indent=1)
        f.write("\n")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden_singlet.py /path/to/reference/src")
    main(sys.argv[1])
