"""Open-boundary Poisson / Hartree oracle (FP64).

Restates ``src/isogrid/poisson/open_boundary.py``:
* multipole moments ``_accumulate_multipole_moments`` :223-264 and the nodal
  moments through ``integrate_field`` :816-851 / :863-891;
* monitor corrected moments: selected cells :182-203 (cell-averaged J at or
  above the 0.9 quantile over interior cells), incident-node fractions
  :206-220 / :267-296, per-cell quadratic least-squares fit over the 4x4x4
  neighbourhood :299-342, 2x2x2 sub-cell trilinear quadrature :370-464;
* ``legacy_split`` boundary correction :559-719;
* boundary potential from moments :467-495; boundary assembly :794-987;
* monitor split ``v = u + b`` with ``-L u = 4 pi rho + L(b)`` :1108-1197 and
  its SciPy BiCGSTAB :1017-1064;
* legacy 7-point operator :122-133 / :990-1014 / :1200-1226 with
  Jacobi-preconditioned BiCGSTAB :1229-1276;
* Hartree energy ``E_H = 1/2 int rho v`` (``poisson/hartree.py:117-129``);
* the JAX route (``poisson/poisson_jax.py``): the CG of ``_run_jax_cg`` :675-750 with its exits,
  and the ``diag`` :248-273, ``separable`` :276-383 and ``line`` :411-579 preconditioners
  (``jax_route_cg``, ``jax_route_preconditioner``).  JAX is absent here, so these are pinned
  through the direct solve of the same system, not through the route's own iterates.

``solve_monitor(..., solver="direct")`` assembles the interior operator by
colour probing and solves it with SuperLU: the converged solution of the
reference's discrete system, which the reference's own ``rtol=1e-8`` BiCGSTAB
only approximates.
"""

from __future__ import annotations

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from .kinetic import integrate_field, monitor_laplacian, step

FOUR_PI = 4.0 * np.pi


def face_mask(shape):
    m = np.ones(shape, dtype=bool)
    m[1:-1, 1:-1, 1:-1] = False
    return m


def _moments_from_weights(w, dx, dy, dz):
    r2 = dx * dx + dy * dy + dz * dz
    q = float(np.sum(w, dtype=np.float64))
    p = np.array([np.sum(w * dx), np.sum(w * dy), np.sum(w * dz)], dtype=np.float64)
    Q = np.array(
        [
            [np.sum(w * (3 * dx * dx - r2)), np.sum(w * (3 * dx * dy)), np.sum(w * (3 * dx * dz))],
            [np.sum(w * (3 * dy * dx)), np.sum(w * (3 * dy * dy - r2)), np.sum(w * (3 * dy * dz))],
            [np.sum(w * (3 * dz * dx)), np.sum(w * (3 * dz * dy)), np.sum(w * (3 * dz * dz - r2))],
        ],
        dtype=np.float64,
    )
    return q, p, Q


def nodal_moments(geom, rho, center):
    dx = geom.x_points - center[0]
    dy = geom.y_points - center[1]
    dz = geom.z_points - center[2]
    r2 = dx * dx + dy * dy + dz * dz
    f = lambda v: integrate_field(v, geom)  # noqa: E731
    q = float(f(rho))
    p = np.array([f(rho * dx), f(rho * dy), f(rho * dz)], dtype=np.float64)
    Q = np.array(
        [
            [f(rho * (3 * dx * dx - r2)), f(rho * (3 * dx * dy)), f(rho * (3 * dx * dz))],
            [f(rho * (3 * dy * dx)), f(rho * (3 * dy * dy - r2)), f(rho * (3 * dy * dz))],
            [f(rho * (3 * dz * dx)), f(rho * (3 * dz * dy)), f(rho * (3 * dz * dz - r2))],
        ],
        dtype=np.float64,
    )
    return q, p, Q


def cell_average(f):
    return (
        f[:-1, :-1, :-1] + f[1:, :-1, :-1] + f[:-1, 1:, :-1] + f[1:, 1:, :-1]
        + f[:-1, :-1, 1:] + f[1:, :-1, 1:] + f[:-1, 1:, 1:] + f[1:, 1:, 1:]
    ) / 8.0


def selected_cells(geom):
    cj = cell_average(np.asarray(geom.jacobian, dtype=np.float64))
    inner = ~face_mask(cj.shape)
    thr = float(np.quantile(cj[inner], 0.9))
    mask = inner & (cj >= thr)
    return mask, np.argwhere(mask)


def _incident_counts(cell_mask):
    c = np.asarray(cell_mask, dtype=np.float64)
    n = np.zeros(tuple(s + 1 for s in c.shape), dtype=np.float64)
    for a in (0, 1):
        for b in (0, 1):
            for d in (0, 1):
                n[a:a + c.shape[0], b:b + c.shape[1], d:d + c.shape[2]] += c
    return n


def _trilinear(c, u, v, w):
    um, vm, wm = 1.0 - u, 1.0 - v, 1.0 - w
    return float(
        um * vm * wm * c[0, 0, 0] + u * vm * wm * c[1, 0, 0] + um * v * wm * c[0, 1, 0] + u * v * wm * c[1, 1, 0]
        + um * vm * w * c[0, 0, 1] + u * vm * w * c[1, 0, 1] + um * v * w * c[0, 1, 1] + u * v * w * c[1, 1, 1]
    )


def _quad_basis(x, y, z):
    return np.column_stack([np.ones_like(x), x, y, z, x * x, y * y, z * z, x * y, x * z, y * z])


def _cell_samples(geom, rho):
    """Yield per selected cell the 8 sub-cell samples (x, y, z, J, rho_quad, rho_tri)."""

    X, Y, Z = (np.asarray(a, dtype=np.float64) for a in (geom.x_points, geom.y_points, geom.z_points))
    J = np.asarray(geom.jacobian, dtype=np.float64)
    R = np.asarray(rho, dtype=np.float64)
    nx, ny, nz = geom.spec.shape
    _, cells = selected_cells(geom)
    subs = [((ix + 0.5) / 2, (iy + 0.5) / 2, (iz + 0.5) / 2) for ix in range(2) for iy in range(2) for iz in range(2)]
    for i, j, k in cells:
        c = (slice(i, i + 2), slice(j, j + 2), slice(k, k + 2))
        s = (slice(max(i - 1, 0), min(i + 3, nx)), slice(max(j - 1, 0), min(j + 3, ny)), slice(max(k - 1, 0), min(k + 3, nz)))
        coef, *_ = np.linalg.lstsq(
            _quad_basis(X[s].reshape(-1), Y[s].reshape(-1), Z[s].reshape(-1)), R[s].reshape(-1), rcond=None
        )
        out = []
        for u, v, w in subs:
            x, y, z = _trilinear(X[c], u, v, w), _trilinear(Y[c], u, v, w), _trilinear(Z[c], u, v, w)
            jv, rt = _trilinear(J[c], u, v, w), _trilinear(R[c], u, v, w)
            rq = float(np.dot(coef, np.array([1.0, x, y, z, x * x, y * y, z * z, x * y, x * z, y * z])))
            out.append((x, y, z, jv, rq, rt))
        yield out


def _subcell_volume(geom):
    return step(geom.logical_x) * step(geom.logical_y) * step(geom.logical_z) / 8.0


def _accumulate(acc_q, acc_p, acc_Q, wgt, dx, dy, dz):
    r2 = dx * dx + dy * dy + dz * dz
    acc_q += wgt
    acc_p += wgt * np.array([dx, dy, dz])
    acc_Q += wgt * np.array(
        [[3 * dx * dx - r2, 3 * dx * dy, 3 * dx * dz], [3 * dy * dx, 3 * dy * dy - r2, 3 * dy * dz], [3 * dz * dx, 3 * dz * dy, 3 * dz * dz - r2]]
    )
    return acc_q


def monitor_moment_correction(geom, rho, center):
    mask, cells = selected_cells(geom)
    if cells.size == 0:
        return 0.0, np.zeros(3), np.zeros((3, 3))
    frac = np.divide(_incident_counts(mask), _incident_counts(np.ones_like(mask)))
    w = np.asarray(rho, dtype=np.float64) * geom.cell_volumes * frac
    nq, npv, nQ = _moments_from_weights(
        w, geom.x_points - center[0], geom.y_points - center[1], geom.z_points - center[2]
    )
    vol = _subcell_volume(geom)
    q, p, Q = 0.0, np.zeros(3), np.zeros((3, 3))
    for samples in _cell_samples(geom, rho):
        for x, y, z, jv, rq, _ in samples:
            q = _accumulate(q, p, Q, rq * jv * vol, x - center[0], y - center[1], z - center[2])
    return q - nq, p - npv, Q - nQ


def boundary_potential(q, p, Q, dx, dy, dz, r, order):
    v = q / r
    if order >= 1:
        v = v + (p[0] * dx + p[1] * dy + p[2] * dz) / r**3
    if order >= 2:
        c = (
            Q[0, 0] * dx * dx + 2 * Q[0, 1] * dx * dy + 2 * Q[0, 2] * dx * dz
            + Q[1, 1] * dy * dy + 2 * Q[1, 2] * dy * dz + Q[2, 2] * dz * dz
        )
        v = v + 0.5 * c / r**5
    return v


def legacy_split_correction(geom, rho, order, bx, by, bz):
    vol = _subcell_volume(geom)
    samples = list(_cell_samples(geom, rho))
    if not samples:
        return np.zeros_like(bx)
    absw, ctr = 0.0, np.zeros(3)
    for cell in samples:
        for x, y, z, jv, rq, rt in cell:
            d = abs((rq - rt) * jv * vol)
            absw += d
            ctr = ctr + d * np.array([x, y, z])
    if absw <= 0.0:
        return np.zeros_like(bx)
    ctr = ctr / absw
    q, p, Q = 0.0, np.zeros(3), np.zeros((3, 3))
    for cell in samples:
        for x, y, z, jv, rq, rt in cell:
            q = _accumulate(q, p, Q, (rq - rt) * jv * vol, x - ctr[0], y - ctr[1], z - ctr[2])
    dx, dy, dz = bx - ctr[0], by - ctr[1], bz - ctr[2]
    return boundary_potential(q, p, Q, dx, dy, dz, np.sqrt(dx * dx + dy * dy + dz * dz), order)


def monitor_center(geom):
    b = geom.spec.box_bounds
    return (0.5 * (b[0][0] + b[0][1]), 0.5 * (b[1][0] + b[1][1]), 0.5 * (b[2][0] + b[2][1]))


def multipole_boundary(geom, rho, order=2, mode="corrected_moments"):
    """Return (boundary_values field, q, p, Q) as in ``open_boundary.py:794-987``."""

    if order not in (0, 1, 2):
        raise ValueError("multipole order must be 0, 1 or 2")
    monitor = hasattr(geom, "inverse_metric_tensor")
    center = monitor_center(geom) if monitor else tuple(geom.spec.reference_center)
    q, p, Q = nodal_moments(geom, rho, center)
    base = (q, p, Q)
    if monitor:
        cq, cp, cQ = monitor_moment_correction(geom, rho, center)
        q, p, Q = q + cq, p + cp, Q + cQ
    fm = face_mask(geom.spec.shape)
    dx = geom.x_points[fm] - center[0]
    dy = geom.y_points[fm] - center[1]
    dz = geom.z_points[fm] - center[2]
    r = np.sqrt(dx * dx + dy * dy + dz * dz)
    if monitor and mode == "legacy_split":
        vb = boundary_potential(*base, dx, dy, dz, r, order) + legacy_split_correction(
            geom, rho, order, geom.x_points[fm], geom.y_points[fm], geom.z_points[fm]
        )
    else:
        vb = boundary_potential(q, p, Q, dx, dy, dz, r, order)
    b = np.zeros(geom.spec.shape, dtype=np.float64)
    b[fm] = vb
    return b, q, p, Q


# ----------------------------------------------------------------- monitor solve
def monitor_interior_matrix(geom, closure="production"):
    """Sparse -L restricted to interior unknowns (colour probing, period 5)."""

    shape = geom.spec.shape
    inner = ~face_mask(shape)
    idx = -np.ones(shape, dtype=np.int64)
    idx[inner] = np.arange(int(inner.sum()))
    I, Jj, K = np.meshgrid(*[np.arange(n) for n in shape], indexing="ij")
    rows, cols, vals = [], [], []
    for a in range(5):
        for b in range(5):
            for c in range(5):
                colour = inner & (I % 5 == a) & (Jj % 5 == b) & (K % 5 == c)
                if not colour.any():
                    continue
                e = colour.astype(np.float64)
                out = -monitor_laplacian(e, geom, closure)
                hit = inner & (out != 0.0)
                # each hit row is reached by exactly one column of this colour:
                # along every axis the unique t in [i-2, i+2] with t = phase mod 5
                ri = np.argwhere(hit)
                src = []
                for ax, ph in enumerate((a, b, c)):
                    t = ri[:, ax]
                    d = (t - ph) % 5
                    src.append(np.where(d <= 2, t - d, t + (5 - d)))
                rows.append(idx[ri[:, 0], ri[:, 1], ri[:, 2]])
                cols.append(idx[src[0], src[1], src[2]])
                vals.append(out[hit])
    n = int(inner.sum())
    rows, cols, vals = np.concatenate(rows), np.concatenate(cols), np.concatenate(vals)
    return sp.csr_matrix((vals, (rows, cols)), shape=(n, n)), inner


def solve_monitor(geom, rho, order=2, tol=1e-8, maxiter=400, solver="direct", mode="corrected_moments"):
    """Monitor-grid open-boundary Poisson; returns dict with potential etc."""

    rho = np.maximum(np.asarray(rho, dtype=np.float64), 0.0)
    b, q, p, Q = multipole_boundary(geom, rho, order, mode)
    fm = face_mask(geom.spec.shape)
    bf = np.array(b, copy=True)
    bf[~fm] = 0.0
    rhs = FOUR_PI * rho + monitor_laplacian(bf, geom, "production")
    inner = ~fm
    iters = -1
    if solver == "direct":
        A, _ = monitor_interior_matrix(geom)
        u = spla.spsolve(A.tocsc(), rhs[inner])
    else:
        shape = geom.spec.shape
        n = int(inner.sum())
        count = [0]

        def mv(x):
            f = np.zeros(shape)
            f[inner] = x
            return -monitor_laplacian(f, geom, "production")[inner]

        def cb(_):
            count[0] += 1

        op = spla.LinearOperator((n, n), matvec=mv, dtype=np.float64)
        u, info = spla.bicgstab(op, rhs[inner], x0=np.zeros(n), rtol=tol, atol=0.0, maxiter=maxiter, callback=cb)
        iters = count[0]
    v = np.array(b, copy=True)
    v[inner] = u
    resid = -monitor_laplacian(v, geom, "production") - FOUR_PI * rho
    return {
        "potential": v, "boundary": b, "q": q, "p": p, "Q": Q, "rhs": rhs,
        "iterations": iters, "residual_max": float(np.max(np.abs(resid[inner]))),
    }


# ------------------------------------------------------------------ legacy solve
def _axis_coeffs(h_pts, logical):
    s = np.asarray(h_pts, dtype=np.float64)
    dl = step(logical)
    inv_face = 1.0 / (0.5 * (s[:-1] + s[1:]))
    c = s[1:-1]
    return inv_face[:-1] / (dl * dl * c), inv_face[1:] / (dl * dl * c)


def legacy_coefficients(geom):
    axm, axp = _axis_coeffs(geom.x_point_jacobian, geom.x_logical)
    aym, ayp = _axis_coeffs(geom.y_point_jacobian, geom.y_logical)
    azm, azp = _axis_coeffs(geom.z_point_jacobian, geom.z_logical)
    diag = axm[:, None, None] + axp[:, None, None] + aym[None, :, None] + ayp[None, :, None] + azm[None, None, :] + azp[None, None, :]
    return axm, axp, aym, ayp, azm, azp, diag


def legacy_apply(u, co):
    axm, axp, aym, ayp, azm, azp, diag = co
    out = diag * u
    out[1:] -= axm[1:, None, None] * u[:-1]
    out[:-1] -= axp[:-1, None, None] * u[1:]
    out[:, 1:] -= aym[None, 1:, None] * u[:, :-1]
    out[:, :-1] -= ayp[None, :-1, None] * u[:, 1:]
    out[:, :, 1:] -= azm[None, None, 1:] * u[:, :, :-1]
    out[:, :, :-1] -= azp[None, None, :-1] * u[:, :, 1:]
    return out


def legacy_rhs(rho, b, co):
    axm, axp, aym, ayp, azm, azp, _ = co
    r = FOUR_PI * np.asarray(rho[1:-1, 1:-1, 1:-1], dtype=np.float64)
    r[0] += axm[0] * b[0, 1:-1, 1:-1]
    r[-1] += axp[-1] * b[-1, 1:-1, 1:-1]
    r[:, 0] += aym[0] * b[1:-1, 0, 1:-1]
    r[:, -1] += ayp[-1] * b[1:-1, -1, 1:-1]
    r[:, :, 0] += azm[0] * b[1:-1, 1:-1, 0]
    r[:, :, -1] += azp[-1] * b[1:-1, 1:-1, -1]
    return r


def solve_legacy(geom, rho, order=2, tol=1e-8, maxiter=400, solver="direct"):
    rho = np.maximum(np.asarray(rho, dtype=np.float64), 0.0)
    b, q, p, Q = multipole_boundary(geom, rho, order)
    co = legacy_coefficients(geom)
    rhs = legacy_rhs(rho, b, co)
    shape = rhs.shape
    n = rhs.size
    iters = -1
    if solver == "direct":
        cols = np.arange(n).reshape(shape)
        rows, cc, vals = [cols.reshape(-1)], [cols.reshape(-1)], [co[-1].reshape(-1)]
        for axis, (cm, cp) in enumerate([(co[0], co[1]), (co[2], co[3]), (co[4], co[5])]):
            shp = [1, 1, 1]
            shp[axis] = -1
            cmf = np.broadcast_to(cm.reshape(shp), shape)
            cpf = np.broadcast_to(cp.reshape(shp), shape)
            lo = [slice(None)] * 3
            hi = [slice(None)] * 3
            lo[axis] = slice(1, None)
            hi[axis] = slice(None, -1)
            rows.append(cols[tuple(lo)].reshape(-1)); cc.append(cols[tuple(hi)].reshape(-1)); vals.append(-cmf[tuple(lo)].reshape(-1))
            rows.append(cols[tuple(hi)].reshape(-1)); cc.append(cols[tuple(lo)].reshape(-1)); vals.append(-cpf[tuple(hi)].reshape(-1))
        A = sp.csc_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cc))), shape=(n, n))
        u = spla.spsolve(A, rhs.reshape(-1)).reshape(shape)
    else:
        count = [0]
        d = co[-1].reshape(-1)
        op = spla.LinearOperator((n, n), matvec=lambda x: legacy_apply(x.reshape(shape), co).reshape(-1), dtype=np.float64)
        M = spla.LinearOperator((n, n), matvec=lambda x: x / d, dtype=np.float64)
        x, info = spla.bicgstab(op, rhs.reshape(-1), x0=np.zeros(n), rtol=tol, atol=0.0, maxiter=maxiter, M=M,
                                callback=lambda _: count.__setitem__(0, count[0] + 1))
        u = x.reshape(shape)
        iters = count[0]
    v = np.array(b, copy=True)
    v[1:-1, 1:-1, 1:-1] = u
    return {"potential": v, "boundary": b, "q": q, "p": p, "Q": Q, "iterations": iters,
            "residual_max": float(np.max(np.abs(legacy_apply(u, co) - rhs)))}


def solve(geom, rho, **kw):
    if hasattr(geom, "inverse_metric_tensor"):
        return solve_monitor(geom, rho, **kw)
    kw.pop("mode", None)
    return solve_legacy(geom, rho, **kw)


def hartree_energy(rho, geom, v):
    return 0.5 * integrate_field(np.maximum(rho, 0.0) * v, geom)


# ------------------------------------------------------- JAX route (CG) oracle
def _logical_step(coords):
    c = np.asarray(coords, dtype=np.float64)
    return float(c[1] - c[0])


def jax_route_preconditioner(geom, kind):
    """The JAX route's preconditioners on interior fields (``poisson/poisson_jax.py``):
    ``diag`` (:248-273, 1 / (2 sum_a g^aa / h_a^2) with a floor), ``separable`` (:276-383,
    axis stiffness from the operator diagonal, Dirichlet sine transform in each axis),
    ``line`` (:411-579, tridiagonal solves along the stiffest axis).  Returns a function of
    the interior field (nx-2, ny-2, nz-2), or None for ``none``."""

    if kind == "none":
        return None
    J = np.asarray(geom.jacobian, dtype=np.float64)
    G = np.asarray(geom.inverse_metric_tensor, dtype=np.float64)
    h = (_logical_step(geom.logical_x), _logical_step(geom.logical_y), _logical_step(geom.logical_z))
    inner = tuple(n - 2 for n in geom.spec.shape)
    if kind == "diag":
        d = 2.0 * (G[..., 0, 0] / h[0] ** 2 + G[..., 1, 1] / h[1] ** 2 + G[..., 2, 2] / h[2] ** 2)
        pos = d[np.isfinite(d) & (d > 0.0)]
        floor = max(1.0e-12, 1.0e-10 * float(np.median(pos)))
        dinv = 1.0 / np.maximum(d, floor)[1:-1, 1:-1, 1:-1]
        return lambda r: dinv * r
    wts = [J * G[..., a, a] for a in range(3)]
    Jc = J[1:-1, 1:-1, 1:-1]
    lows, ups = [], []
    for a in range(3):
        lo, up = [slice(1, -1)] * 3, [slice(1, -1)] * 3
        lo[a], up[a] = slice(0, -2), slice(2, None)
        c = wts[a][1:-1, 1:-1, 1:-1]
        lows.append(0.5 * (c + wts[a][tuple(lo)]) / (Jc * h[a] ** 2))
        ups.append(0.5 * (c + wts[a][tuple(up)]) / (Jc * h[a] ** 2))
    stiff = [0.5 * float(np.mean(lows[a] + ups[a])) * h[a] ** 2 for a in range(3)]
    if kind == "separable":
        S, lam = [], []
        for a in range(3):
            m = inner[a]
            i = np.arange(1, m + 1, dtype=np.float64)
            S.append(np.sqrt(2.0 / (m + 1)) * np.sin(np.pi * np.outer(i, i) / (m + 1)))
            lam.append(4.0 * np.sin(np.pi * i / (2.0 * (m + 1))) ** 2 / h[a] ** 2)
        ev = stiff[0] * lam[0][:, None, None] + stiff[1] * lam[1][None, :, None] + stiff[2] * lam[2][None, None, :]
        inv = 1.0 / np.maximum(ev, max(1.0e-12, 1.0e-12 * float(np.max(ev))))

        def sep(r):
            t = np.einsum("ia,jb,kc,abc->ijk", S[0], S[1], S[2], r)
            return np.einsum("ai,bj,ck,ijk->abc", S[0], S[1], S[2], t * inv)

        return sep
    if kind == "line":
        scores = [2.0 * stiff[a] / h[a] ** 2 for a in range(3)]
        ax = int(np.argmax(scores))
        diag = lows[0] + ups[0] + lows[1] + ups[1] + lows[2] + ups[2]
        lower, upper = np.zeros_like(diag), np.zeros_like(diag)
        sl_lo, sl_up = [slice(None)] * 3, [slice(None)] * 3
        sl_lo[ax], sl_up[ax] = slice(1, None), slice(None, -1)
        lower[tuple(sl_lo)] = -lows[ax][tuple(sl_lo)]
        upper[tuple(sl_up)] = -ups[ax][tuple(sl_up)]
        dl, ll, ul = (np.moveaxis(x, ax, -1) for x in (diag, lower, upper))

        def line(r):
            b = np.moveaxis(r, ax, -1).copy()
            m = b.shape[-1]
            c = np.zeros_like(b)
            d = np.zeros_like(b)
            # Thomas algorithm on every line (lower[..., 0] and upper[..., -1] are zero)
            c[..., 0] = ul[..., 0] / dl[..., 0]
            d[..., 0] = b[..., 0] / dl[..., 0]
            for i in range(1, m):
                den = dl[..., i] - ll[..., i] * c[..., i - 1]
                c[..., i] = ul[..., i] / den
                d[..., i] = (b[..., i] - ll[..., i] * d[..., i - 1]) / den
            x = np.zeros_like(b)
            x[..., -1] = d[..., -1]
            for i in range(m - 2, -1, -1):
                x[..., i] = d[..., i] - c[..., i] * x[..., i + 1]
            return np.moveaxis(x, -1, ax)

        line.axis = ax
        return line
    raise ValueError(f"unknown preconditioner {kind}")


def jax_route_cg(geom, rhs_interior, tolerance=1e-8, max_iterations=400, preconditioner="none"):
    """``_run_jax_cg`` (``poisson/poisson_jax.py:675-750``): CG on the interior -L from x = 0,
    stopping when max |r| < tolerance; returns (x, iterations, residual_max, converged)."""

    shape = geom.spec.shape
    inner_shape = tuple(n - 2 for n in shape)
    M = jax_route_preconditioner(geom, preconditioner)

    def A(x):
        f = np.zeros(shape)
        f[1:-1, 1:-1, 1:-1] = x
        return -monitor_laplacian(f, geom, "production")[1:-1, 1:-1, 1:-1]

    b = np.asarray(rhs_interior, dtype=np.float64).reshape(inner_shape)
    x = np.zeros(inner_shape)
    r = b - A(x)
    z = M(r) if M else r
    p = z.copy()
    rz = float(np.vdot(r, z))
    it, conv, rmax = 0, False, float(np.max(np.abs(r)))
    for k in range(1, max_iterations + 1):
        ap = A(p)
        den = float(np.vdot(p, ap))
        if abs(den) <= 1.0e-20:
            break
        alpha = rz / den
        x = x + alpha * p
        r = r - alpha * ap
        rmax = float(np.max(np.abs(r)))
        it = k
        if rmax < tolerance:
            conv = True
            break
        z = M(r) if M else r
        rz_new = float(np.vdot(r, z))
        if abs(rz) <= 1.0e-30:
            break
        p = z + (rz_new / rz) * p
        rz = rz_new
    return x, it, rmax, conv
