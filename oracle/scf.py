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
