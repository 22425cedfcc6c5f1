"""Kinetic / Laplacian operators and weighted reductions (FP64 oracle).

Restates ``src/isogrid/ops/kinetic.py``:
* ``integrate_field`` :61-66, ``weighted_l2_norm`` :69-74;
* legacy separable flux form ``_apply_axis_laplacian`` :87-114,
  ``apply_legacy_kinetic_operator`` :147-153;
* monitor A-grid: zero-ghost gradient ``_axis_gradient_zero_ghost`` :165-187,
  ``np.gradient(edge_order=2)`` branch :190-209, contravariant fluxes
  :212-252, divergence :255-276, Laplacian / kinetic :279-358;
* the legacy Hamiltonian as a sparse matrix, and the eigenvalues of its right eigenpairs and
  of its cell-volume-symmetric part (the legacy operator is not self-adjoint in that inner
  product, so the definition of "its eigenvalues" matters; the reference's legacy route is
  ARPACK ``eigsh`` on the weighted operator, ``ks/eigensolver.py:993-1133``).
"""

from __future__ import annotations

import numpy as np


def step(coords) -> float:
    d = np.diff(np.asarray(coords, dtype=np.float64))
    return float(d[0])


def integrate_field(field, geom) -> float:
    return float(np.sum(np.asarray(field, dtype=np.float64) * geom.cell_volumes, dtype=np.float64))


def weighted_l2_norm(field, geom) -> float:
    f = np.asarray(field, dtype=np.float64)
    return float(np.sqrt(np.sum(np.abs(f) ** 2 * geom.cell_volumes, dtype=np.float64)))


# ----------------------------------------------------------------- legacy grid
def _legacy_axis(field, scale, h, axis):
    f = np.moveaxis(np.asarray(field, dtype=np.float64), axis, 0)
    s = np.asarray(scale, dtype=np.float64)
    face = 0.5 * (s[:-1] + s[1:])
    bc = (slice(None),) + (None,) * (f.ndim - 1)
    fm = np.empty_like(f)
    fp = np.empty_like(f)
    fm[0] = f[0] / (h * s[0])
    fm[1:] = (f[1:] - f[:-1]) / (h * face[bc])
    fp[:-1] = (f[1:] - f[:-1]) / (h * face[bc])
    fp[-1] = -f[-1] / (h * s[-1])
    return np.moveaxis((fp - fm) / (h * s[bc]), 0, axis)


def legacy_laplacian(psi, geom):
    out = np.zeros(geom.spec.shape, dtype=np.float64)
    out += _legacy_axis(psi, geom.x_point_jacobian, step(geom.x_logical), 0)
    out += _legacy_axis(psi, geom.y_point_jacobian, step(geom.y_logical), 1)
    out += _legacy_axis(psi, geom.z_point_jacobian, step(geom.z_logical), 2)
    return out


def legacy_kinetic(psi, geom):
    return -0.5 * legacy_laplacian(psi, geom)


def legacy_hamiltonian_matrix(geom, veff):
    """Sparse FP64 matrix of -1/2 L + diag(veff) on the legacy grid (``ops/kinetic.py:87-153``).

    The legacy Laplacian is a sum of three one-axis operators, so the matrix is the Kronecker
    sum of the 1-D matrices that ``_legacy_axis`` applies (assembled column by column)."""

    from scipy.sparse import csr_matrix, diags, identity, kron

    def axis_matrix(scale, h):
        n = len(scale)
        m = np.zeros((n, n))
        for j in range(n):
            e = np.zeros(n)
            e[j] = 1.0
            m[:, j] = _legacy_axis(e, scale, h, 0)
        return csr_matrix(m)

    nx, ny, nz = geom.spec.shape
    lx = axis_matrix(geom.x_point_jacobian, step(geom.x_logical))
    ly = axis_matrix(geom.y_point_jacobian, step(geom.y_logical))
    lz = axis_matrix(geom.z_point_jacobian, step(geom.z_logical))
    lap = (kron(kron(lx, identity(ny)), identity(nz)) + kron(kron(identity(nx), ly), identity(nz))
           + kron(kron(identity(nx), identity(ny)), lz))
    return (-0.5 * lap + diags(np.asarray(veff, dtype=np.float64).reshape(-1))).tocsr()


def weighted_symmetric_eigenvalues(h, geom, k):
    """Lowest k eigenvalues of the cell-volume-symmetric part of ``h``:
    S = 1/2 (W^1/2 H W^-1/2 + (W^1/2 H W^-1/2)^T), the limit of a Rayleigh-Ritz iteration
    whose projected matrices are symmetrised (H is not self-adjoint in the W inner product
    on the legacy grid)."""

    from scipy.sparse import diags
    from scipy.sparse.linalg import eigsh

    sw = np.sqrt(np.asarray(geom.cell_volumes, dtype=np.float64).reshape(-1))
    a = diags(sw) @ h @ diags(1.0 / sw)
    return np.sort(eigsh(0.5 * (a + a.T), k=k, which="SA", tol=1e-13)[0])


def nonsymmetric_eigenvalues(h, k):
    """Lowest-real-part k eigenvalues of ``h`` itself (right eigenvalues, Arnoldi)."""

    from scipy.sparse.linalg import eigs

    return np.sort(eigs(h.tocsc(), k=k, which="SR", tol=1e-13)[0].real)


# --------------------------------------------------------------- monitor grid
def _zero_ghost_gradient(f, coords, axis):
    h = step(coords)
    m = np.moveaxis(np.asarray(f, dtype=np.float64), axis, 0)
    g = np.empty_like(m)
    g[1:-1] = (m[2:] - m[:-2]) / (2.0 * h)
    g[0] = (m[1] - 0.0) / (2.0 * h)
    g[-1] = (0.0 - m[-2]) / (2.0 * h)
    return np.moveaxis(g, 0, axis)


def _logical(geom):
    return (
        np.asarray(geom.logical_x, dtype=np.float64),
        np.asarray(geom.logical_y, dtype=np.float64),
        np.asarray(geom.logical_z, dtype=np.float64),
    )


def _gradient(f, geom, closure):
    lx, ly, lz = _logical(geom)
    if closure == "trial_fix":
        return _zero_ghost_gradient(f, lx, 0), _zero_ghost_gradient(f, ly, 1), _zero_ghost_gradient(f, lz, 2)
    gx, gy, gz = np.gradient(np.asarray(f, dtype=np.float64), lx, ly, lz, edge_order=2)
    return gx, gy, gz


def _divergence(fx, fy, fz, geom, closure):
    lx, ly, lz = _logical(geom)
    if closure == "trial_fix":
        return _zero_ghost_gradient(fx, lx, 0) + _zero_ghost_gradient(fy, ly, 1) + _zero_ghost_gradient(fz, lz, 2)
    return (
        np.gradient(fx, lx, axis=0, edge_order=2)
        + np.gradient(fy, ly, axis=1, edge_order=2)
        + np.gradient(fz, lz, axis=2, edge_order=2)
    )


def monitor_laplacian(psi, geom, closure="production"):
    """nabla^2 psi = J^-1 d_a (J g^{ab} d_b psi) on the uniform logical cube."""

    J = np.asarray(geom.jacobian, dtype=np.float64)
    G = np.asarray(geom.inverse_metric_tensor, dtype=np.float64)
    d0, d1, d2 = _gradient(psi, geom, closure)
    fx = J * (G[..., 0, 0] * d0 + G[..., 0, 1] * d1 + G[..., 0, 2] * d2)
    fy = J * (G[..., 1, 0] * d0 + G[..., 1, 1] * d1 + G[..., 1, 2] * d2)
    fz = J * (G[..., 2, 0] * d0 + G[..., 2, 1] * d1 + G[..., 2, 2] * d2)
    return _divergence(fx, fy, fz, geom, closure) / J


def monitor_kinetic(psi, geom, closure="production"):
    return -0.5 * monitor_laplacian(psi, geom, closure)


def kinetic(psi, geom, closure="production"):
    if hasattr(geom, "inverse_metric_tensor"):
        return monitor_kinetic(psi, geom, closure)
    return legacy_kinetic(psi, geom)


def hpsi_block(block, geom, veff, closure="trial_fix"):
    """H psi = T psi + v_eff psi per orbital (``ks/eigensolver.py:729-784``)."""

    b = np.asarray(block, dtype=np.float64)
    if b.ndim == 3:
        b = b[None]
    return np.stack([kinetic(p, geom, closure) + veff * p for p in b])


def weighted_overlap(left, geom, right=None):
    """<a_i|b_j>_W over (k, nx, ny, nz) blocks (``ks/eigensolver.py:246-272``)."""

    L = np.asarray(left, dtype=np.float64).reshape(len(left), -1).T
    R = L if right is None else np.asarray(right, dtype=np.float64).reshape(len(right), -1).T
    w = np.asarray(geom.cell_volumes, dtype=np.float64).reshape(-1)
    return L.T @ (w[:, None] * R)
