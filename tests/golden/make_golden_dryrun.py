"""Generate A-grid (monitor-grid) H2 SCF dry-run golden values with the reference itself.

Run in a checkout that has the reference sources (read-only):

    PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_golden_dryrun.py /path/to/reference/src [run ...]

The reference's ``run_h2_monitor_grid_scf_dry_run`` runs unmodified on the
67x67x81 A-grid built by its own ``build_monitor_grid_for_case`` with the
local-patch development element parameters; LSDA goes through the same
stand-in ``pyscf.dft.libxc`` module as ``make_golden_scf.py``.  Writes
``dryrun_agrid_h2.json`` beside this script (runs already present are kept):
per run the parameters, converged flag, iteration count, energy components,
eigenvalues and per-iteration (density residual, total energy); for the singlet also the
active-subspace diagnostics of each step.
"""

import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

from make_golden_scf import _install_libxc_shim  # noqa: E402

RUNS = {
    # the reference defaults (10 steps of linear mixing, loose tolerances)
    "triplet_default": ("triplet", {}),
    # Pulay mixing at tighter tolerances
    "triplet_diis_tight": ("triplet", dict(max_iterations=40, enable_diis=True, density_tolerance=1e-4,
                                           energy_tolerance=1e-7, eigensolver_tolerance=1e-5)),
    # Anderson (adaptive damping, reset on growth) and Broyden-like mixing at the same tolerances
    "triplet_anderson_tight": ("triplet", dict(max_iterations=40, enable_anderson=True,
                                               anderson_adaptive_damping_enabled=True, anderson_reset_on_growth=True,
                                               density_tolerance=1e-4, energy_tolerance=1e-7,
                                               eigensolver_tolerance=1e-5)),
    "triplet_broyden_tight": ("triplet", dict(max_iterations=40, enable_broyden=True, density_tolerance=1e-4,
                                              energy_tolerance=1e-7, eigensolver_tolerance=1e-5)),
    # the singlet's default path: active-subspace tracking and Hartree-aware total-density mixing
    "singlet_default": ("singlet", {}),
}


def main(src, names):
    sys.path.insert(0, src)
    _install_libxc_shim()
    from isogrid.config import H2_BENCHMARK_CASE
    from isogrid.grid import build_h2_local_patch_development_element_parameters, build_monitor_grid_for_case
    from isogrid.scf.driver import run_h2_monitor_grid_scf_dry_run

    geom = build_monitor_grid_for_case(H2_BENCHMARK_CASE, shape=(67, 67, 81), box_half_extents=(8.0, 8.0, 10.0),
                                       element_parameters=build_h2_local_patch_development_element_parameters())
    path = os.path.join(HERE, "dryrun_agrid_h2.json")
    out = json.load(open(path)) if os.path.exists(path) else {}
    for name in names or list(RUNS):
        if name in out:
            continue
        label, kw = RUNS[name]
        t = time.time()
        r = run_h2_monitor_grid_scf_dry_run(label, H2_BENCHMARK_CASE, geom, **kw)
        e = r.energy
        out[name] = {
            "spin": label, "params": kw, "shape": [67, 67, 81], "converged": bool(r.converged),
            "iterations": int(r.iteration_count),
            "energy": {k: float(getattr(e, k)) for k in ("kinetic", "local_ionic", "nonlocal_ionic", "hartree", "xc",
                                                          "ion_ion_repulsion", "total")},
            "eigenvalues_up": [float(v) for v in r.eigenvalues_up],
            "eigenvalues_down": [float(v) for v in r.eigenvalues_down],
            "history": [[float(h.density_residual), float(h.energy.total)] for h in r.history],
            "mixer": {k: list(getattr(r, k)) for k in ("diis_used_iterations", "anderson_used_iterations",
                                                       "anderson_rejected_iterations", "anderson_reset_iterations",
                                                       "broyden_used_iterations", "broyden_fallback_iterations")},
            "cpu_seconds": time.time() - t,
        }
        if r.active_subspace_enabled:
            out[name]["active_subspace"] = [[d.iteration, d.raw_occupied_overlap_abs, d.best_in_subspace_occupied_overlap_abs,
                                             d.internal_rotation_angle_deg, d.lowest_gap_ha, d.verdict]
                                            for d in r.active_subspace_diagnostics_history]
        print(name, out[name]["iterations"], out[name]["energy"]["total"], out[name]["cpu_seconds"], flush=True)
        json.dump(out, open(path, "w"), indent=1)


if __name__ == "__main__":
    src = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("ISOGRID_REFERENCE_SRC")
    if not src:
        raise SystemExit(f"usage: python {sys.argv[0]} <reference checkout>/src"
                         " (or set ISOGRID_REFERENCE_SRC)")
    main(src, sys.argv[2:])
