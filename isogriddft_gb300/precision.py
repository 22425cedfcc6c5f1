"""Mixed-precision vs FP64 study on a benzene-sized molecule (no reference counterpart).

The FP32-stencil / FP32-inner-Poisson / 3xTF32-Gram path (``precision="mixed"``) is run
against the all-FP64 GPU path on the same A-grid and the same input density, and every
energy term, the occupied eigenvalues and the iteration counts are compared:

1. input density: superposition of valence-weighted atomic Gaussians (30 electrons for
   C6H6), split evenly between the spins (closed-shell singlet);
2. Hartree potential of that density (BiCGSTAB, FP64 or FP32 inside FP64 refinement) and
   LSDA potentials (FP64 on both paths);
3. the 15 lowest eigenpairs of the static KS Hamiltonian (kinetic + local GTH + nonlocal
   C s projectors + v_H + v_xc) by the preconditioned block iteration with a working block of
   32 columns (FP32 or FP64 orbitals);
4. the band energy sum_i f_i eps_i and the Harris-Foulkes energy of the input density,
   E_HF = sum f eps - E_H[rho_in] - <rho_in, v_xc> + E_xc[rho_in] + E_II, which is stationary
   in the orbitals (its error is second order in the orbital error, like the eigenvalues);
5. at the output density of those orbitals: T_s (FP64 stencil apply of the orbitals), E_loc,
   E_nl, E_H (a second Hartree solve), E_xc and their total.  These terms are first order in
   the orbital error (the output density is not self-consistent), so they show the
   eigenvector accuracy of each path rather than a converged-energy difference.

The comparison is non-self-consistent on purpose: the benzene A-grid SCF from atomic
Gaussians does not settle with the linear/Pulay/Anderson/Broyden mixers (charge sloshing
without a Kerker-type preconditioner), so an SCF-level comparison would compare two
unconverged iterates; step 3 is the fixed-potential problem every SCF step solves.

    python -m isogriddft_gb300.precision --shape 192 192 192 --tolerance 1e-4
"""

from __future__ import annotations

import argparse
import json
import time

import numpy as np
import torch

from .config import make_benzene_case
from .grid import build_monitor_grid_for_case, build_two_peak_element_parameters
from .scf import DeviceScfEngine, atomic_gaussian_density_device, resolve_spin_occupations

TERMS = ("kinetic", "local_ionic", "nonlocal_ionic", "hartree", "xc", "ion_ion_repulsion", "total")


def build_study_geometry(case=None, shape=(192, 192, 192), box_half_extents=(9.0, 9.0, 7.0), device=True):
    """The A-grid of the study: refinement peaks at every nucleus (amplitude 4, width 0.5 Bohr)."""

    case = case or make_benzene_case()
    elements = tuple(sorted({a.element for a in case.geometry.atoms}))
    return case, build_monitor_grid_for_case(case, shape=tuple(shape), box_half_extents=tuple(box_half_extents),
                                             element_parameters=build_two_peak_element_parameters(elements, 4.0, 0.5),
                                             device=device)


def solve_one(case, geom, precision: str, *, block: int = 32, eigensolver_tolerance: float = 1.0e-5,
              eigensolver_max_iterations: int = 3000, poisson_tolerance: float = 1.0e-10,
              kinetic_version: str = "trial_fix") -> dict:
    """Steps 1-5 above on one precision path; energies in Ha, wall times in s."""

    occ = resolve_spin_occupations("singlet", case)
    eng = DeviceScfEngine(case, geom, occ, precision=precision, kinetic_version=kinetic_version,
                          include_nonlocal=True, poisson_tolerance=poisson_tolerance, poisson_max_iterations=4000)
    eng.block = block
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    rho = atomic_gaussian_density_device(case, geom, float(occ.total_electrons))
    up = dn = 0.5 * rho
    hart = eng.hartree(rho)
    lx = eng.xc(up, dn)
    v = eng.vloc + hart.potential + lx["v_up"]
    k = len(occ.occupations_up)
    res = eng.eigensolve(v, k, None, tolerance=eigensolver_tolerance, max_iterations=eigensolver_max_iterations,
                         stall_iterations=60)
    eps = np.asarray(res["eigenvalues"], dtype=np.float64)[:k]
    f_up, f_dn = np.asarray(occ.occupations_up, dtype=np.float64), np.asarray(occ.occupations_down, dtype=np.float64)
    band = float(np.dot(f_up, eps) + np.dot(f_dn, eps))
    eh_in = 0.5 * float(eng.wdot(rho, hart.potential).item())
    vxc_rho = float(eng.wdot(up, lx["v_up"]).item() + eng.wdot(dn, lx["v_down"]).item())
    exc_in = float(lx["energy"].item())
    harris = band - eh_in - vxc_rho + exc_in + eng.e_ii
    orb = res["orbitals"]
    up_out = eng.density(orb, occ.occupations_up, occ.n_alpha)
    dn_out = up_out
    energy, hart_out, _ = eng.energy(up_out, dn_out, orb, orb)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    return {
        "precision": precision,
        "energy": {t: float(getattr(energy, t)) for t in TERMS},
        "eigenvalues": [float(x) for x in np.asarray(res["eigenvalues"])[:k]],
        "eigensolver_iterations": int(res["iteration_count"]),
        "eigensolver_converged": bool(res.get("converged", True)),
        "poisson_iterations": [int(x) for x in eng.poisson_history],
        "hartree_input_energy": eh_in,
        "band_energy": band,
        "harris_foulkes_energy": harris,
        "wall_s": wall,
    }


def compare(a: dict, b: dict) -> dict:
    """Per-term |mixed - FP64| energy differences and the largest eigenvalue difference."""

    ea, eb = np.asarray(a["eigenvalues"]), np.asarray(b["eigenvalues"])
    return {
        "energy_abs_diff": {t: abs(a["energy"][t] - b["energy"][t]) for t in TERMS},
        "hartree_input_abs_diff": abs(a["hartree_input_energy"] - b["hartree_input_energy"]),
        "eigenvalue_max_abs_diff": float(np.max(np.abs(ea - eb))),
        "band_energy_abs_diff": abs(a["band_energy"] - b["band_energy"]),
        "harris_foulkes_abs_diff": abs(a["harris_foulkes_energy"] - b["harris_foulkes_energy"]),
    }


def run_study(shape=(192, 192, 192), box_half_extents=(9.0, 9.0, 7.0), block: int = 32,
              eigensolver_tolerance: float = 1.0e-5) -> dict:
    case, geom = build_study_geometry(shape=shape, box_half_extents=box_half_extents)
    out = {"case": "C6H6 (12 atoms, 30 valence electrons, 15 occupied per spin)", "shape": list(shape),
           "box_half_extents": list(box_half_extents), "block": block}
    runs = {p: solve_one(case, geom, p, block=block, eigensolver_tolerance=eigensolver_tolerance)
            for p in ("fp64", "mixed")}
    out["runs"] = runs
    out["mixed_vs_fp64"] = compare(runs["mixed"], runs["fp64"])
    out["speedup_mixed_vs_fp64"] = runs["fp64"]["wall_s"] / runs["mixed"]["wall_s"]
    return out


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--shape", type=int, nargs=3, default=(192, 192, 192))
    ap.add_argument("--box", type=float, nargs=3, default=(9.0, 9.0, 7.0))
    ap.add_argument("--block", type=int, default=32)
    # 1e-4: FP32 orbitals give the mixed eigensolver a residual floor near 1e-5 at 192^3
    ap.add_argument("--tolerance", type=float, default=1.0e-4)
    args = ap.parse_args(argv)
    print(json.dumps(run_study(tuple(args.shape), tuple(args.box), args.block, args.tolerance)), flush=True)


if __name__ == "__main__":
    main()
