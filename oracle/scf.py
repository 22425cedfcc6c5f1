"""Density build, renormalisation, residual and energy-assembly oracle (FP64).

Restates ``src/isogrid/scf/driver.py``: occupations ``:593-627``, expectation
values ``:630-660``, density ``_build_density_from_occupied_orbitals``
``:663-676``, ``_renormalize_density`` ``:679-690``, ``_density_residual``
``:693-702``, H2 trial orbitals ``:705-734``, ion-ion repulsion ``:884-903``;
and the audit trial orbital ``audit/h2_monitor_grid_ts_eloc_audit.py:87-101``.
"""

from __future__ import annotations

import numpy as np

from .kinetic import integrate_field, weighted_l2_norm
from .pseudo import GTH_PADE


def density(orbitals, occupations, geom):
    rho = np.zeros(geom.spec.shape, dtype=np.float64)
    for i, occ in enumerate(occupations):
        rho += occ * np.abs(orbitals[i]) ** 2
    return rho


def renormalize(rho, target, geom):
    if target == 0.0:
        return np.zeros(geom.spec.shape)
    integral = integrate_field(rho, geom)
    if integral <= 0.0:
        raise ValueError("positive density integral required")
    return rho * (target / integral)


def residual(up_in, dn_in, up_out, dn_out, geom):
    a = weighted_l2_norm(up_out - up_in, geom)
    b = weighted_l2_norm(dn_out - dn_in, geom)
    return float(np.sqrt(a * a + b * b))


def bonding_trial_orbital(case, geom, exponent=0.8):
    fields = []
    for atom in case.geometry.atoms:
        dx = geom.x_points - atom.position[0]
        dy = geom.y_points - atom.position[1]
        dz = geom.z_points - atom.position[2]
        fields.append(np.exp(-exponent * (dx * dx + dy * dy + dz * dz)))
    orb = np.asarray(fields[0] + fields[1], dtype=np.float64)
    return orb / np.sqrt(integrate_field(orb * orb, geom))


def ion_ion_repulsion(case):
    atoms = case.geometry.atoms
    e = 0.0
    for i in range(len(atoms)):
        for j in range(i + 1, len(atoms)):
            d = np.linalg.norm(np.subtract(atoms[i].position, atoms[j].position))
            e += GTH_PADE[atoms[i].element][0] * GTH_PADE[atoms[j].element][0] / d
    return float(e)


def single_point_energy(up, dn, orb_up, orb_dn, occ_up, occ_dn, case, geom, closure="production", local_only=False,
                        poisson_solver="direct"):
    """``evaluate_single_point_energy`` (``driver.py:905-1015``) on renormalised densities."""

    from . import kinetic as K
    from . import poisson as P
    from . import pseudo as PS
    from . import xc as X

    na, nb = sum(occ_up), sum(occ_dn)
    up, dn = renormalize(up, na, geom), renormalize(dn, nb, geom)
    rho = up + dn
    kin = 0.0
    for orbs, occ in ((orb_up, occ_up), (orb_dn, occ_dn)):
        for i, o in enumerate(occ):
            kin += o * integrate_field(orbs[i] * K.kinetic(orbs[i], geom, closure), geom)
    eloc = integrate_field(rho * PS.local_potential(case, geom), geom)
    enl = 0.0
    if not local_only:
        for orbs, occ in ((orb_up, occ_up), (orb_dn, occ_dn)):
            for i, o in enumerate(occ):
                enl += o * integrate_field(orbs[i] * PS.nonlocal_action(case, geom, orbs[i]), geom)
    v = P.solve(geom, rho, solver=poisson_solver)["potential"]
    eh = P.hartree_energy(rho, geom, v)
    exc = X.xc_energy(up, dn, geom, case.reference_model.xc)
    eii = ion_ion_repulsion(case)
    return {"kinetic": kin, "local_ionic": eloc, "nonlocal_ionic": enl, "hartree": eh, "xc": exc,
            "ion_ion_repulsion": eii, "total": kin + eloc + enl + eh + exc + eii}


def minimal_scf(case, geom, n_alpha, n_beta, closure="production", max_iterations=40, mixing=0.6,
                density_tolerance=1e-6, energy_tolerance=1e-10, eig_tolerance=1e-9, ncv=20, local_only=False):
    """``run_h2_minimal_scf`` (``driver.py:2953-3159``) with oracle operators: direct
    Poisson, block subspace iteration, linear mixing; returns dict(history, energy, ...)."""

    from . import eigensolver as E
    from . import kinetic as K
    from . import poisson as P
    from . import pseudo as PS
    from . import xc as X

    occ_up, occ_dn = (1.0,) * n_alpha, (1.0,) * n_beta
    # H2 trial pair, W-orthonormalised (``driver.py:705-734``)
    f = []
    for atom in case.geometry.atoms:
        d2 = (geom.x_points - atom.position[0]) ** 2 + (geom.y_points - atom.position[1]) ** 2 + \
            (geom.z_points - atom.position[2]) ** 2
        f.append(np.exp(-0.8 * d2))
    trial = E.weighted_orthonormalize(np.asarray([f[0] + f[1], f[0] - f[1]]), geom.cell_volumes)
    g_up, g_dn = trial[:n_alpha], trial[:n_beta]
    up = renormalize(density(g_up, occ_up, geom), n_alpha, geom)
    dn = renormalize(density(g_dn, occ_dn, geom), n_beta, geom)
    vloc = PS.local_potential(case, geom)
    singlet = n_alpha == n_beta
    hist, prev = [], None
    for it in range(1, max_iterations + 1):
        v = P.solve(geom, up + dn, solver="direct")["potential"]
        xc = X.lsda(up, dn, case.reference_model.xc)

        def solve(vxc, k, guess):
            veff = vloc + v + vxc

            def apply_h(b):
                hb = K.hpsi_block(b, geom, veff, closure)
                if not local_only:
                    hb = hb + np.stack([PS.nonlocal_action(case, geom, x) for x in b])
                return hb
            return E.block_subspace_iteration(apply_h, case, geom, k, max_iterations=3000, tolerance=eig_tolerance,
                                              initial_guess=guess, ncv=ncv)
        ru = solve(xc["v_xc_up"], n_alpha, g_up)
        o_up = ru["orbitals"]
        if singlet:
            o_dn, rd = o_up, ru
        elif n_beta == 0:
            o_dn, rd = np.zeros((0,) + tuple(geom.spec.shape)), {"eigenvalues": np.zeros(0)}
        else:
            rd = solve(xc["v_xc_down"], n_beta, g_dn)
            o_dn = rd["orbitals"]
        up_out = renormalize(density(o_up, occ_up, geom), n_alpha, geom)
        dn_out = renormalize(density(o_dn, occ_dn, geom), n_beta, geom)
        res = residual(up, dn, up_out, dn_out, geom)
        e = single_point_energy(up_out, dn_out, o_up, o_dn, occ_up, occ_dn, case, geom, closure, local_only)
        change = None if prev is None else e["total"] - prev
        hist.append((res, e["total"]))
        if res < density_tolerance and (change is None or abs(change) < energy_tolerance):
            return {"converged": True, "iterations": it, "energy": e, "history": hist,
                    "eigenvalues_up": ru["eigenvalues"], "eigenvalues_down": rd["eigenvalues"]}
        up = renormalize((1 - mixing) * up + mixing * up_out, n_alpha, geom)
        dn = renormalize((1 - mixing) * dn + mixing * dn_out, n_beta, geom)
        g_up, g_dn, prev = o_up, o_dn, e["total"]
    return {"converged": False, "iterations": max_iterations, "energy": e, "history": hist,
            "eigenvalues_up": ru["eigenvalues"], "eigenvalues_down": rd["eigenvalues"]}
