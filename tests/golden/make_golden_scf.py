"""Generate SCF golden values by running the reference's own legacy-grid H2 SCF.

Run in a checkout that has the reference sources (read-only):

    PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_golden_scf.py /path/to/reference/src

The reference evaluates LSDA through PySCF/libxc, which is not installed here;
a stand-in ``pyscf.dft.libxc`` module whose ``eval_xc`` returns the oracle's
Slater + VWN5 restatement (pinned against the reference's recorded E_xc) is
placed in ``sys.modules`` first, so the reference's own code runs unmodified.
Writes ``scf_legacy_h2.json`` beside this script: per run the parameters,
converged flag, iteration count, energy components and per-iteration
(residual, total energy).
"""

import json
import os
import sys
import time
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def _install_libxc_shim():
    sys.path.insert(0, ROOT)
    import oracle.xc as OX

    def eval_xc(name, rho, spin=1, deriv=1):
        up, dn = rho
        r = OX.lsda(up, dn, "lda,vwn")
        return r["eps_xc"], (np.stack([r["v_xc_up"], r["v_xc_down"]], axis=1),), None, None

    pyscf, dft, libxc = (types.ModuleType(n) for n in ("pyscf", "pyscf.dft", "pyscf.dft.libxc"))
    libxc.eval_xc = eval_xc
    dft.libxc = libxc
    pyscf.dft = dft
    sys.modules.update({"pyscf": pyscf, "pyscf.dft": dft, "pyscf.dft.libxc": libxc})


RUNS = {
    # the reference defaults (driver.py:2953-2963)
    "singlet_default": ("singlet", {}),
    "triplet_default": ("triplet", {}),
    # tight: the discrete fixed point to ~1e-8 Ha
    "singlet_tight": ("singlet", dict(max_iterations=40, density_tolerance=1e-6, energy_tolerance=1e-10,
                                      eigensolver_tolerance=1e-10)),
    "triplet_tight": ("triplet", dict(max_iterations=40, density_tolerance=1e-6, energy_tolerance=1e-10,
                                      eigensolver_tolerance=1e-10)),
}


def main(src):
    sys.path.insert(0, src)
    _install_libxc_shim()
    from isogrid.scf.driver import run_h2_minimal_scf

    out = {}
    path = os.path.join(HERE, "scf_legacy_h2.json")
    if os.path.exists(path):
        out = json.load(open(path))
    for name, (label, kw) in RUNS.items():
        if name in out:
            continue
        t = time.time()
        r = run_h2_minimal_scf(label, **kw)
        e = r.energy
        out[name] = {
            "spin": label, "params": kw, "converged": bool(r.converged), "iterations": int(r.iteration_count),
            "energy": {k: float(getattr(e, k)) for k in ("kinetic", "local_ionic", "nonlocal_ionic", "hartree", "xc",
                                                          "ion_ion_repulsion", "total")},
            "eigenvalues_up": [float(v) for v in r.eigenvalues_up],
            "eigenvalues_down": [float(v) for v in r.eigenvalues_down],
            "history": [[float(h.density_residual), float(h.energy.total)] for h in r.history],
            "cpu_seconds": time.time() - t,
        }
        print(name, out[name]["iterations"], out[name]["energy"]["total"], out[name]["cpu_seconds"], flush=True)
        json.dump(out, open(path, "w"), indent=1)


if __name__ == "__main__":
    src = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("ISOGRID_REFERENCE_SRC")
    if not src:
        raise SystemExit(f"usage: python {sys.argv[0]} <reference checkout>/src"
                         " (or set ISOGRID_REFERENCE_SRC)")
    main(src)
