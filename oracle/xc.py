"""Spin-polarised LSDA oracle: Slater exchange + VWN5 (and PW92) correlation.

The reference evaluates ``lda,vwn`` through PySCF -> libxc
(``src/isogrid/xc/lsda.py:70-121``; PySCF >= 2.3, an optional dependency with
no pinned version, absent here).  libxc's ``LDA_C_VWN`` is the VWN "5" fit
(Vosko, Wilk, Nusair, Can. J. Phys. 58, 1200 (1980)), restated here:

* Slater exchange, e_x = -3/4 (6/pi)^(1/3) (rho_u^(4/3) + rho_d^(4/3)),
  v_x,s = -(6/pi)^(1/3) rho_s^(1/3);
* VWN interpolation form per channel (paramagnetic, ferromagnetic, spin
  stiffness) with x = sqrt(rs), X(x) = x^2 + b x + c, Q = sqrt(4c - b^2);
* spin interpolation eps = eps_P + alpha f(z)(1 - z^4)/f''(0)
  + (eps_F - eps_P) f(z) z^4;
* v_s = eps - rs/3 d eps/d rs +/- (1 -/+ z) d eps/d z.

Points with total density below ``DENSITY_THRESHOLD`` return zeros, as libxc
does.  Input validation (negative-density tolerance 1e-14, clip at zero)
follows ``xc/lsda.py:57-67``.  PW92 (Perdew & Wang, PRB 45, 13244 (1992)) is
offered as an extra functional with no reference counterpart.
"""

from __future__ import annotations

import numpy as np

DENSITY_THRESHOLD = 1.0e-15
NEGATIVE_TOLERANCE = 1.0e-14

_VWN = {  # (A, b, c, x0) in Hartree
    "P": (0.0310907, 3.72744, 12.9352, -0.10498),
    "F": (0.01554535, 7.06042, 18.0578, -0.32500),
    "A": (-1.0 / (6.0 * np.pi**2), 1.13107, 13.0045, -0.0047584),
}
_FPP = 4.0 / (9.0 * (2.0 ** (1.0 / 3.0) - 1.0))
_FDEN = 2.0 ** (4.0 / 3.0) - 2.0


def _vwn_channel(x, A, b, c, x0):
    X = x * x + b * x + c
    X0 = x0 * x0 + b * x0 + c
    Q = np.sqrt(4.0 * c - b * b)
    t = 2.0 * x + b
    at = np.arctan(Q / t)
    k = b * x0 / X0
    g = A * (np.log(x * x / X) + (2.0 * b / Q) * at - k * (np.log((x - x0) ** 2 / X) + (2.0 * (b + 2.0 * x0) / Q) * at))
    den = t * t + Q * Q
    dg = A * (2.0 / x - t / X - 4.0 * b / den - k * (2.0 / (x - x0) - t / X - 4.0 * (b + 2.0 * x0) / den))
    return g, dg  # d/dx


def _fzeta(opz, omz):
    """f(z) and f'(z) from 1 + z and 1 - z (formed from the spin densities, so no cancellation)."""

    a, b = np.cbrt(opz), np.cbrt(omz)
    f = (opz * a + omz * b - 2.0) / _FDEN
    df = (4.0 / 3.0) * (a - b) / _FDEN
    return f, df


def _pw_channel(rs, A, a1, b1, b2, b3, b4):
    s = np.sqrt(rs)
    qd = 2.0 * A * (b1 * s + b2 * rs + b3 * rs * s + b4 * rs * rs)
    dqd = 2.0 * A * (0.5 * b1 / s + b2 + 1.5 * b3 * s + 2.0 * b4 * rs)
    lg = np.log1p(1.0 / qd)
    g = -2.0 * A * (1.0 + a1 * rs) * lg
    dg = -2.0 * A * a1 * lg + 2.0 * A * (1.0 + a1 * rs) * dqd / (qd * qd + qd)
    return g, dg  # d/drs


_PW = {
    "P": (0.031091, 0.21370, 7.5957, 3.5876, 1.6382, 0.49294),
    "F": (0.015545, 0.20548, 14.1189, 6.1977, 3.3662, 0.62517),
    "A": (0.016887, 0.11125, 10.357, 3.6231, 0.88026, 0.49671),
}


def validate_density(rho, name="rho"):
    v = np.asarray(rho, dtype=np.float64)
    if not np.all(np.isfinite(v)):
        raise ValueError(f"{name} must contain only finite values.")
    if np.any(v < -NEGATIVE_TOLERANCE):
        raise ValueError(f"{name} must be non-negative up to roundoff.")
    return np.maximum(v, 0.0)


def lsda(rho_up, rho_down, functional="lda,vwn"):
    """Return dict(eps_xc, v_xc_up, v_xc_down, energy_density, rho_total)."""

    fn = functional.strip().lower()
    if fn not in ("lda,vwn", "lda,pw92", "lda,pw"):
        raise ValueError(f"unsupported functional `{functional}`")
    ru, rd = validate_density(rho_up, "rho_up"), validate_density(rho_down, "rho_down")
    rho = ru + rd
    live = rho >= DENSITY_THRESHOLD
    r = np.where(live, rho, 1.0)
    u = np.where(live, ru, 0.5)
    d = np.where(live, rd, 0.5)
    cx = (6.0 / np.pi) ** (1.0 / 3.0)
    cu, cd = np.cbrt(u), np.cbrt(d)
    ex = -0.75 * cx * (u * cu + d * cd)
    vxu, vxd = -cx * cu, -cx * cd
    z = np.clip((u - d) / r, -1.0, 1.0)
    rs = np.cbrt(3.0 / (4.0 * np.pi * r))
    if fn == "lda,vwn":
        x = np.sqrt(rs)
        (gp, dgp), (gf, dgf), (ga, dga) = (_vwn_channel(x, *_VWN[k]) for k in ("P", "F", "A"))
        to_rs = 1.0 / (2.0 * x)
        dgp, dgf, dga = dgp * to_rs, dgf * to_rs, dga * to_rs
    else:
        (gp, dgp), (gf, dgf), (ga, dga) = (_pw_channel(rs, *_PW[k]) for k in ("P", "F", "A"))
        ga, dga = -ga, -dga
    opz, omz = 2.0 * u / r, 2.0 * d / r
    f, df = _fzeta(opz, omz)
    z3 = z * z * z
    z4 = z3 * z
    ec = gp + ga * f * (1.0 - z4) / _FPP + (gf - gp) * f * z4
    dec_rs = dgp + dga * f * (1.0 - z4) / _FPP + (dgf - dgp) * f * z4
    dec_z = ga * (df * (1.0 - z4) - 4.0 * z3 * f) / _FPP + (gf - gp) * (df * z4 + 4.0 * z3 * f)
    base = ec - rs / 3.0 * dec_rs
    vcu = base + omz * dec_z
    vcd = base - opz * dec_z
    eps = np.where(live, ex / r + ec, 0.0)
    vu = np.where(live, vxu + vcu, 0.0)
    vd = np.where(live, vxd + vcd, 0.0)
    return {"rho_up": ru, "rho_down": rd, "rho_total": rho, "eps_xc": eps, "v_xc_up": vu, "v_xc_down": vd,
            "energy_density": rho * eps}


def xc_energy(rho_up, rho_down, geom, functional="lda,vwn"):
    e = lsda(rho_up, rho_down, functional)
    return float(np.sum(e["energy_density"] * geom.cell_volumes, dtype=np.float64))
