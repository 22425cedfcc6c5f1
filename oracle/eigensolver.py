"""Fixed-potential block eigensolver oracle (FP64).

Restates ``src/isogrid/ks``:
* weighted overlap / SVD orthonormalisation ``eigensolver.py:246-341``;
* default guess block (atomic Gaussians, Cartesian moments, rng 12345 noise)
  ``eigensolver.py:818-913``;
* the A-grid block subspace iteration of ``eigensolver_jax.py:53-524``:
  working block m = max(2k+2, 4, 12k+8, initial_subspace_size, ncv); weighted
  QR start; per iteration Rayleigh-Ritz on B^T W (HB), residuals of the k
  lowest Ritz pairs, projection against B, whitening by the Gram
  eigendecomposition (QR fallback when the smallest eigenvalue <= 1e-10),
  H applied to the residual block only, (m+k)^2 trial Rayleigh-Ritz and
  compression back to m columns followed by whitening;
* the SciPy ``eigsh`` route on W^(1/2) H W^(-1/2) ``eigensolver.py:947-1133``.
"""

from __future__ import annotations

import numpy as np


def _cols(block):
    b = np.asarray(block, dtype=np.float64)
    return b.reshape(b.shape[0], -1).T


def _block(cols, shape):
    return np.asarray(cols.T.reshape((cols.shape[1],) + tuple(shape)))


def weighted_orthonormalize(block, w, require_full_rank=True, rank_tol=1.0e-12):
    X = _cols(block)
    sw = np.sqrt(w.reshape(-1))[:, None]
    _, s, vt = np.linalg.svd(sw * X, full_matrices=False)
    cut = rank_tol * max(X.shape) * s[0]
    rank = int(np.sum(s > cut))
    if require_full_rank and rank < X.shape[1]:
        raise ValueError("rank-deficient block")
    return _block(X @ (vt[:rank].T / s[:rank]), w.shape)


def default_guess(case, geom, count):
    if hasattr(geom, "inverse_metric_tensor"):
        b = geom.spec.box_bounds
        c = np.array([0.5 * (b[0][0] + b[0][1]), 0.5 * (b[1][0] + b[1][1]), 0.5 * (b[2][0] + b[2][1])])
    else:
        c = np.asarray(geom.spec.reference_center, dtype=np.float64)
    xs, ys, zs = geom.x_points - c[0], geom.y_points - c[1], geom.z_points - c[2]
    r2 = xs * xs + ys * ys + zs * zs
    gauss = []
    for atom in case.geometry.atoms:
        dx = geom.x_points - atom.position[0]
        dy = geom.y_points - atom.position[1]
        dz = geom.z_points - atom.position[2]
        gauss.append(np.exp(-0.85 * (dx * dx + dy * dy + dz * dz)))
    g = []
    if gauss:
        g.append(np.sum(gauss, axis=0))
    if len(gauss) >= 2:
        alt = np.zeros_like(gauss[0])
        for i, a in enumerate(gauss):
            alt += a if i % 2 == 0 else -a
        g.append(alt)
    base = np.exp(-0.65 * r2)
    g += [base, zs * np.exp(-0.55 * r2), xs * np.exp(-0.55 * r2), ys * np.exp(-0.55 * r2), np.exp(-1.10 * r2),
          (3.0 * zs * zs - r2) * np.exp(-0.45 * r2)]
    rng = np.random.default_rng(12345)
    n = max(count, 8)
    while len(g) < n:
        g.append(base * rng.normal(size=geom.spec.shape))
    ortho = weighted_orthonormalize(np.asarray(g[:n]), geom.cell_volumes, require_full_rank=False)
    if ortho.shape[0] < count:
        raise ValueError("not enough independent guesses")
    return ortho[:count]


def initial_block(case, geom, k, size, user=None):
    target = max(k, size)
    d = default_guess(case, geom, target)
    if user is None:
        return d[:target]
    u = np.asarray(user, dtype=np.float64)
    if u.ndim == 3:
        u = u[None]
    o = weighted_orthonormalize(np.concatenate([u, d]), geom.cell_volumes, require_full_rank=False)
    if o.shape[0] < k:
        raise ValueError("initial guesses do not span k directions")
    return o[:target]


def block_size(k, initial_subspace_size=None, ncv=None):
    return max(2 * k + 2, 4, 12 * k + 8, int(initial_subspace_size or 0), int(ncv or 0))


def block_subspace_iteration(apply_h, case, geom, k, max_iterations=400, tolerance=1.0e-3,
                             initial_guess=None, initial_subspace_size=None, ncv=None):
    """``apply_h(block (m, nx, ny, nz)) -> block``; returns a result dict."""

    shape = geom.spec.shape
    w = np.asarray(geom.cell_volumes, dtype=np.float64).reshape(-1)
    sw = np.sqrt(w)
    m = block_size(k, initial_subspace_size, ncv)
    guess = initial_block(case, geom, k, m, initial_guess)[:m]

    def gram(a, b):
        return a.T @ (w[:, None] * b)

    def wqr(X):
        q, r = np.linalg.qr(sw[:, None] * X)
        return q / sw[:, None], np.linalg.inv(r)

    def whiten(X):
        G = gram(X, X)
        G = 0.5 * (G + G.T)
        ev, V = np.linalg.eigh(G)
        if np.all(np.isfinite(ev)) and ev.min() > 1.0e-10:
            T = (V * (1.0 / np.sqrt(np.clip(ev, 1e-14, None)))[None, :]) @ V.T
            return X @ T, T
        return wqr(X)

    def H(X):
        return _cols(apply_h(_block(X, shape)))

    B, _ = wqr(_cols(guess))
    HB = H(B)
    res_hist, ritz_hist = [], []
    converged = False
    it = 0
    for it in range(1, max_iterations + 1):
        P = gram(B, HB)
        P = 0.5 * (P + P.T)
        lam, V = np.linalg.eigh(P)
        C = V[:, :k]
        X, HX = B @ C, HB @ C
        R = HX - X * lam[None, :k]
        rn = np.sqrt(np.clip(np.sum(R * R * w[:, None], axis=0), 0.0, None))
        res_hist.append(rn)
        ritz_hist.append(lam[:k].copy())
        eig, orb, ritz = lam[:k].copy(), X, P[:k, :k]
        if rn.max() <= tolerance:
            converged = True
            break
        R = R - B @ gram(B, R)
        R, _ = whiten(R)
        HR = H(R)
        T = np.block([[P, gram(B, HR)], [gram(R, HB), gram(R, HR)]])
        T = 0.5 * (T + T.T)
        _, W = np.linalg.eigh(T)
        Bn = B @ W[:m, :m] + R @ W[m:, :m]
        HBn = HB @ W[:m, :m] + HR @ W[m:, :m]
        B, Tr = whiten(Bn)
        HB = HBn @ Tr
    overlap = gram(orb, orb)
    return {
        "eigenvalues": eig, "orbitals": _block(orb, shape), "converged": converged, "iteration_count": it,
        "residual_norms": rn, "residual_history": np.array(res_hist), "ritz_value_history": np.array(ritz_hist),
        "weighted_overlap": overlap, "max_orthogonality_error": float(np.max(np.abs(overlap - np.eye(k)))),
        "ritz_matrix": ritz, "initial_guess_orbitals": guess, "final_basis_orbitals": _block(B, shape),
    }


def eigsh_route(apply_h, case, geom, k, max_iterations=400, tolerance=1.0e-3, ncv=None, initial_subspace_size=None):
    """SciPy Lanczos on W^(1/2) H W^(-1/2) (``eigensolver.py:993-1133``)."""

    from scipy.sparse.linalg import ArpackNoConvergence, LinearOperator, eigsh

    shape = geom.spec.shape
    w = np.asarray(geom.cell_volumes, dtype=np.float64).reshape(-1)
    sw, isw = np.sqrt(w), 1.0 / np.sqrt(w)
    size = initial_subspace_size or max(2 * k, 4)
    guess = initial_block(case, geom, k, size)
    n = w.size

    def mv(v):
        v = np.asarray(v, dtype=np.float64)
        one = v.ndim == 1
        V = v[:, None] if one else v
        out = sw[:, None] * _cols(apply_h(_block(isw[:, None] * V, shape)))
        return out[:, 0] if one else out

    op = LinearOperator((n, n), matvec=mv, matmat=mv, dtype=np.float64)
    v0 = sw * _cols(guess)[:, 0]
    v0 = v0 / np.linalg.norm(v0)
    nc = int(min(max(ncv or max(20, 2 * k + 1), k + 2), n - 1))
    conv = True
    try:
        vals, vecs = eigsh(op, k=k, which="SA", v0=v0, tol=tolerance, maxiter=max_iterations, ncv=nc)
    except ArpackNoConvergence as exc:
        conv, vals, vecs = False, exc.eigenvalues, exc.eigenvectors
    order = np.argsort(vals)[:k]
    vals, vecs = vals[order], vecs[:, order]
    orbs = _block(isw[:, None] * vecs, shape)
    acts = apply_h(orbs)
    rn = np.array([np.sqrt(np.sum((acts[i] - vals[i] * orbs[i]) ** 2 * geom.cell_volumes)) for i in range(k)])
    return {"eigenvalues": vals, "orbitals": orbs, "residual_norms": rn, "converged": bool(conv and rn.max() <= tolerance)}
