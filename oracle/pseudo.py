"""GTH local and nonlocal pseudopotential oracle (FP64).

Restates ``src/isogrid/pseudo``:
* gth-pade table for H/C/N/O ``gth_data.py:28-120``;
* local term V_loc(r) = -Z erf(r / (sqrt2 rloc)) / r
  + exp(-r^2 / 2 rloc^2) sum_i C_i (r/rloc)^(2i), r = 0 limit
  -Z sqrt(2/pi)/rloc (``local.py:138-205``), summed over atoms (``:303-357``);
* nonlocal separable action sum_lm sum_ij |p_i> h_ij <p_j|psi>_W with radial
  projectors sqrt2 r^(l+2i) exp(-r^2/2r_l^2) / (r_l^(l+(4i+3)/2)
  sqrt(Gamma(l+(4i+3)/2))) and real harmonics l <= 1 (``nonlocal.py:99-283``),
  evaluated on the full grid as the reference does.
"""

from __future__ import annotations

from math import erf, gamma, pi, sqrt

import numpy as np

from .kinetic import integrate_field

# element: (Z_ion, rloc, (C1, C2), [(l, r_l, [[h]])])  -- projector_count 0 channels omitted
GTH_PADE = {
    "H": (1, 0.2, (-4.1802368, 0.72507482), []),
    "C": (4, 0.34883045, (-8.5137711, 1.22843203), [(0, 0.30455321, [[9.52284179]])]),
    "N": (5, 0.28917923, (-12.23481988, 1.76640728), [(0, 0.25660487, [[13.55224272]])]),
    "O": (6, 0.24762086, (-16.58031797, 2.39570092), [(0, 0.22178614, [[18.26691718]])]),
}
_ERF = np.vectorize(erf, otypes=[np.float64])


def _r(geom, pos):
    dx = geom.x_points - pos[0]
    dy = geom.y_points - pos[1]
    dz = geom.z_points - pos[2]
    return dx, dy, dz, np.sqrt(dx * dx + dy * dy + dz * dz, dtype=np.float64)


def atomic_local_potential(r, element):
    z, rloc, coeffs, _ = GTH_PADE[element]
    with np.errstate(divide="ignore", invalid="ignore"):
        coul = -z * _ERF(r / (sqrt(2.0) * rloc)) / r
    coul = np.asarray(coul, dtype=np.float64)
    coul[r == 0.0] = -z * sqrt(2.0 / pi) / rloc
    s = r / rloc
    poly = np.zeros_like(r)
    for i, c in enumerate(coeffs):
        poly += c * s ** (2 * i)
    return coul + np.exp(-0.5 * s**2) * poly


def local_potential(case, geom):
    out = np.zeros(geom.spec.shape, dtype=np.float64)
    for atom in case.geometry.atoms:
        out += atomic_local_potential(_r(geom, atom.position)[3], atom.element)
    return out


def radial_projector(r, l, i, rl):
    g = l + 0.5 * (4 * (i + 1) - 1)
    return sqrt(2.0) / (rl**g * sqrt(gamma(g))) * r ** (l + 2 * i) * np.exp(-0.5 * (r / rl) ** 2)


def real_harmonic(l, m, dx, dy, dz, r):
    if l == 0:
        return np.full(dx.shape, 1.0 / sqrt(4.0 * pi))
    c = sqrt(3.0 / (4.0 * pi))
    with np.errstate(divide="ignore", invalid="ignore"):
        v = c * {-1: dy, 0: dz, 1: dx}[m] / r
    v = np.asarray(v, dtype=np.float64)
    v[r == 0.0] = 0.0
    return v


def projectors(case, geom, extra_channels=None):
    """List of (atom_index, l, m, [projector fields], h matrix)."""

    out = []
    for ia, atom in enumerate(case.geometry.atoms):
        chans = list(GTH_PADE[atom.element][3])
        if extra_channels and atom.element in extra_channels:
            chans += extra_channels[atom.element]
        dx, dy, dz, r = _r(geom, atom.position)
        for l, rl, h in chans:
            h = np.asarray(h, dtype=np.float64)
            for m in ((0,) if l == 0 else (-1, 0, 1)):
                fields = [radial_projector(r, l, i, rl) * real_harmonic(l, m, dx, dy, dz, r) for i in range(h.shape[0])]
                out.append((ia, l, m, fields, h))
    return out


def nonlocal_action(case, geom, psi, extra_channels=None):
    act = np.zeros(geom.spec.shape, dtype=np.float64)
    for _, _, _, fields, h in projectors(case, geom, extra_channels):
        c = np.array([integrate_field(p * psi, geom) for p in fields])
        for p, cr in zip(fields, h @ c):
            act += cr * p
    return act


def local_force(case, geom, rho, h=1.0e-5):
    """-dE_loc/dR_a for E_loc = sum rho W V_loc by central differences of the local
    potential in the atom position (oracle for the Hellmann-Feynman force kernel)."""

    from dataclasses import replace

    atoms = list(case.geometry.atoms)
    out = np.zeros((len(atoms), 3))
    w = geom.cell_volumes
    for a in range(len(atoms)):
        for c in range(3):
            e = []
            for sgn in (1.0, -1.0):
                pos = list(atoms[a].position)
                pos[c] += sgn * h
                moved = atoms[:a] + [replace(atoms[a], position=tuple(pos))] + atoms[a + 1:]
                cs = replace(case, geometry=replace(case.geometry, atoms=tuple(moved)))
                e.append(float(np.sum(rho * local_potential(cs, geom) * w)))
            out[a, c] = -(e[0] - e[1]) / (2.0 * h)
    return out


def nonlocal_energy(case, geom, orbitals, occupations, extra_channels=None):
    """E_nl = sum_o f_o <psi_o | V_nl | psi_o>_W (``pseudo/nonlocal.py:209-337`` applied
    to each occupied orbital)."""

    return float(sum(f * integrate_field(p * nonlocal_action(case, geom, p, extra_channels), geom)
                     for p, f in zip(orbitals, occupations)))


def nonlocal_force(case, geom, orbitals, occupations, h=1.0e-5):
    """-dE_nl/dR_a at fixed orbitals by central differences of the atom positions (the
    oracle for the nonlocal Hellmann-Feynman force; the reference computes no forces)."""

    from dataclasses import replace

    atoms = list(case.geometry.atoms)
    out = np.zeros((len(atoms), 3))
    for a in range(len(atoms)):
        for c in range(3):
            e = []
            for sgn in (1.0, -1.0):
                pos = list(atoms[a].position)
                pos[c] += sgn * h
                moved = atoms[:a] + [replace(atoms[a], position=tuple(pos))] + atoms[a + 1:]
                cs = replace(case, geometry=replace(case.geometry, atoms=tuple(moved)))
                e.append(nonlocal_energy(cs, geom, orbitals, occupations))
            out[a, c] = -(e[0] - e[1]) / (2.0 * h)
    return out
