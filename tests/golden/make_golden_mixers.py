"""Generate density-mixer golden vectors with the reference's own mixer functions.

Run in a checkout that has the reference sources (read-only):

    PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_golden_mixers.py /path/to/reference/src

On the reference's 7 x 7 x 9 H2 A-grid (its own ``build_monitor_grid_for_case``),
seeded synthetic SCF sequences (positive mixed spin densities, residuals that
shrink with an occasional growth) go through the schedule of the reference's
dry-run loop (``scf/driver.py:4297-4430``: history append and truncation, the
warm-up test, Anderson's reset on residual growth), with the reference's
``_apply_monitor_grid_density_diis``, ``_apply_monitor_grid_density_anderson``
and ``_apply_monitor_grid_density_broyden_like`` computing each step.  Writes
``mixers_h2.npz`` beside this script: the cell volumes, the inputs of every
iteration, and per mixer configuration the densities returned and the
diagnostics lists.
"""

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
T = 9  # SCF iterations per sequence
NA, NB = 2, 1

CONFIGS = {
    "diis": ("diis", dict(history_length=4, warmup=3)),
    "anderson_default": ("anderson", dict(history_length=4, warmup=3, regularization=1e-8, damping=0.5,
                                          step_clip_factor=None, reset_on_growth=False, reset_growth_factor=1.10,
                                          adaptive_damping=False, min_damping=0.35, max_damping=0.75,
                                          acceptance_ratio=1.02, collinearity=0.995)),
    "anderson_guarded": ("anderson", dict(history_length=5, warmup=2, regularization=1e-6, damping=0.6,
                                          step_clip_factor=0.8, reset_on_growth=True, reset_growth_factor=1.10,
                                          adaptive_damping=True, min_damping=0.35, max_damping=0.75,
                                          acceptance_ratio=1.5, collinearity=0.9)),
    "anderson_strict": ("anderson", dict(history_length=4, warmup=2, regularization=1e-8, damping=0.3,
                                         step_clip_factor=None, reset_on_growth=False, reset_growth_factor=1.10,
                                         adaptive_damping=False, min_damping=0.1, max_damping=0.95,
                                         acceptance_ratio=0.90, collinearity=0.995)),
    "broyden": ("broyden", dict(mixing=0.35, history_length=4, warmup=3, regularization=1e-8, damping=0.5)),
}


def sequence(shape, seed):
    rng = np.random.default_rng(seed)
    decay = [1.0, 0.6, 0.4, 0.5, 0.25, 0.3, 0.12, 0.08, 0.05]  # grows at iterations 4 and 6 (1-based)
    seq = []
    base_u = rng.uniform(0.2, 1.0, shape)
    base_d = rng.uniform(0.2, 1.0, shape)
    for k in range(T):
        mu = base_u * (1.0 + 0.05 * rng.normal(size=shape))
        md = base_d * (1.0 + 0.05 * rng.normal(size=shape))
        ru = 0.05 * decay[k] * rng.normal(size=shape)
        rd = 0.05 * decay[k] * rng.normal(size=shape)
        seq.append((np.abs(mu), np.abs(md), ru, rd))
    return seq


def main(src):
    sys.path.insert(0, src)
    from isogrid.config import H2_BENCHMARK_CASE
    from isogrid.grid import build_h2_local_patch_development_element_parameters, build_monitor_grid_for_case
    from isogrid.scf import driver as D

    geom = build_monitor_grid_for_case(H2_BENCHMARK_CASE, shape=(7, 7, 9), box_half_extents=(8.0, 8.0, 10.0),
                                       element_parameters=build_h2_local_patch_development_element_parameters())
    shape = geom.spec.shape
    out = {"cell_volumes": np.asarray(geom.cell_volumes, dtype=np.float64)}
    seq = sequence(shape, 7)
    for k, (mu, md, ru, rd) in enumerate(seq):
        out[f"in_{k}"] = np.stack([mu, md, ru, rd])
    meta = {}
    for name, (kind, p) in CONFIGS.items():
        hist, got = [], []
        diag = {"used": [], "fallback": [], "rejected": [], "resets": [], "sizes": [], "filtered": [],
                "damping": [], "ratios": []}
        for k, (mu, md, ru, rd) in enumerate(seq):
            it = k + 1
            res = (mu, md)
            if kind == "diis":
                hist = (hist + [D.MonitorGridDiisHistoryEntry(mu, md, ru, rd)])[-p["history_length"]:]
                if it >= p["warmup"] and len(hist) >= 2:
                    c = D._apply_monitor_grid_density_diis(tuple(hist), grid_geometry=geom, n_alpha=NA, n_beta=NB)
                    if c is not None:
                        res = c
                        diag["used"].append(it)
                    else:
                        diag["fallback"].append(it)
                diag["sizes"].append(len(hist))
            elif kind == "anderson":
                hist = (hist + [D.MonitorGridAndersonHistoryEntry(mu, md, ru, rd)])[-p["history_length"]:]
                if p["reset_on_growth"] and len(hist) >= 2:  # driver.py:4330-4360
                    prev = hist[-2]
                    pn = np.sqrt(D._weighted_spin_density_dot(prev.residual_up, prev.residual_down, prev.residual_up,
                                                              prev.residual_down, grid_geometry=geom))
                    cn = np.sqrt(D._weighted_spin_density_dot(ru, rd, ru, rd, grid_geometry=geom))
                    if not np.isfinite(cn) or (pn > 0.0 and cn > p["reset_growth_factor"] * pn):
                        hist = hist[-1:]
                        diag["resets"].append(it)
                if it >= p["warmup"] and len(hist) >= 2:
                    c = D._apply_monitor_grid_density_anderson(
                        tuple(hist), grid_geometry=geom, n_alpha=NA, n_beta=NB, regularization=p["regularization"],
                        damping=p["damping"], step_clip_factor=p["step_clip_factor"],
                        adaptive_damping_enabled=p["adaptive_damping"], min_damping=p["min_damping"],
                        max_damping=p["max_damping"],
                        acceptance_residual_ratio_threshold=p["acceptance_ratio"],
                        collinearity_cosine_threshold=p["collinearity"])
                    diag["filtered"].append(c.filtered_history_length)
                    diag["damping"].append(c.effective_damping)
                    diag["ratios"].append(np.nan if c.projected_residual_ratio is None
                                          else c.projected_residual_ratio)
                    if c.accepted and c.mixed_rho_up is not None:
                        res = (c.mixed_rho_up, c.mixed_rho_down)
                        diag["used"].append(it)
                    elif c.projected_residual_ratio is None:
                        diag["fallback"].append(it)
                    else:
                        diag["rejected"].append(it)
                else:
                    diag["filtered"].append(len(hist))
                diag["sizes"].append(len(hist))
            else:
                hist = (hist + [D.MonitorGridBroydenHistoryEntry(mu, md, ru, rd)])[-p["history_length"]:]
                if it >= p["warmup"] and len(hist) >= 2:
                    c = D._apply_monitor_grid_density_broyden_like(
                        tuple(hist), grid_geometry=geom, n_alpha=NA, n_beta=NB, mixing=p["mixing"],
                        regularization=p["regularization"], damping=p["damping"])
                    if c is not None:
                        res = c
                        diag["used"].append(it)
                    else:
                        diag["fallback"].append(it)
                diag["sizes"].append(len(hist))
            got.append(np.stack([np.asarray(res[0], dtype=np.float64), np.asarray(res[1], dtype=np.float64)]))
        out[f"{name}_out"] = np.stack(got)
        out[f"{name}_ratios"] = np.asarray(diag.pop("ratios"), dtype=np.float64)
        out[f"{name}_damping"] = np.asarray(diag.pop("damping"), dtype=np.float64)
        meta[name] = {"kind": kind, "params": p, **diag}
        print(name, {k: v for k, v in diag.items()}, flush=True)
    out["meta"] = np.asarray(json.dumps(meta))
    out["occupations"] = np.asarray([NA, NB])
    np.savez_compressed(os.path.join(HERE, "mixers_h2.npz"), **out)


if __name__ == "__main__":
    src = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("ISOGRID_REFERENCE_SRC")
    if not src:
        raise SystemExit(f"usage: python {sys.argv[0]} <reference checkout>/src (or set ISOGRID_REFERENCE_SRC)")
    main(src)
