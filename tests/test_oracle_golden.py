"""Pin the CPU oracle and the host grid builders against reference outputs.

Fixtures in ``tests/golden`` were produced by running the reference's own
NumPy functions (``tests/golden/make_golden.py``); the recorded numbers come
from the reference's ``src/isogrid/audit/baselines.py``.
"""

import numpy as np
import pytest

from tests.conftest import load_golden

import oracle
from oracle import eigensolver as OE
from oracle import kinetic as K
from oracle import poisson as P
from oracle import pseudo as PS
from oracle import scf as S
from oracle import xc as X


def test_monitor_grid_bit_exact(golden_monitor, monitor_geom):
    g = golden_monitor
    for name, attr in [("x", "x_points"), ("y", "y_points"), ("z", "z_points"), ("jacobian", "jacobian"),
                       ("inverse_metric", "inverse_metric_tensor"), ("cell_volumes", "cell_volumes")]:
        np.testing.assert_array_equal(getattr(monitor_geom, attr), g[name], err_msg=name)


def test_legacy_grid_bit_exact(golden_legacy, legacy_geom):
    np.testing.assert_array_equal(legacy_geom.x_points, golden_legacy["x"])
    np.testing.assert_array_equal(legacy_geom.cell_volumes, golden_legacy["cell_volumes"])
    from isogriddft_gb300.grid import build_default_h2_grid_geometry

    d = build_default_h2_grid_geometry()
    a = load_golden("legacy_default_axes.npz")
    np.testing.assert_array_equal(d.x_coordinates, a["x"])
    np.testing.assert_array_equal(d.z_coordinates, a["z"])
    np.testing.assert_array_equal(d.cell_widths_z, a["wz"])
    np.testing.assert_array_equal(d.z_point_jacobian, a["hz"])


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def test_oracle_monitor_kinetic(golden_monitor, monitor_geom):
    g = golden_monitor
    assert _rel(K.monitor_kinetic(g["psi"], monitor_geom, "production"), g["kin_prod_psi"]) < 1e-13
    assert _rel(K.monitor_kinetic(g["psi"], monitor_geom, "trial_fix"), g["kin_trial_psi"]) < 1e-13
    for i in range(3):
        assert _rel(K.monitor_kinetic(g["rnd"][i], monitor_geom, "production"), g["kin_prod_rnd"][i]) < 1e-13
        assert _rel(K.monitor_kinetic(g["rnd"][i], monitor_geom, "trial_fix"), g["kin_trial_rnd"][i]) < 1e-13
    assert _rel(K.monitor_laplacian(g["rnd"][0], monitor_geom), g["lap_prod_rnd0"]) < 1e-13


def test_oracle_legacy_kinetic(golden_legacy, legacy_geom):
    g = golden_legacy
    assert _rel(K.legacy_kinetic(g["rnd"], legacy_geom), g["kin_rnd"]) < 1e-13
    assert _rel(K.legacy_kinetic(g["psi"], legacy_geom), g["kin_psi"]) < 1e-13


def test_oracle_local_and_nonlocal(golden_monitor, golden_legacy, monitor_geom, legacy_geom):
    from isogriddft_gb300.config import H2_BENCHMARK_CASE, make_molecule_case

    assert _rel(PS.local_potential(H2_BENCHMARK_CASE, monitor_geom), golden_monitor["vloc"]) < 1e-14
    assert _rel(PS.local_potential(H2_BENCHMARK_CASE, legacy_geom), golden_legacy["vloc"]) < 1e-14
    n2 = make_molecule_case("N2", [("N", (0.0, 0.0, -1.037)), ("N", (0.0, 0.0, 1.037))])
    assert _rel(PS.nonlocal_action(n2, monitor_geom, golden_monitor["psi"]), golden_monitor["n2_nonlocal_psi"]) < 1e-13


def test_oracle_multipole_boundary(golden_monitor, golden_legacy, monitor_geom, legacy_geom):
    g = golden_monitor
    b, q, p, Q = P.multipole_boundary(monitor_geom, g["rho"], 2, "corrected_moments")
    assert abs(q - float(g["q"])) < 1e-13
    np.testing.assert_allclose(p, g["p"], atol=1e-13)
    np.testing.assert_allclose(Q, g["Q"], atol=1e-12)
    assert _rel(b, g["boundary_values"]) < 1e-13
    b2, *_ = P.multipole_boundary(monitor_geom, g["rho"], 2, "legacy_split")
    assert _rel(b2, g["legacy_split_boundary"]) < 1e-12
    gl = golden_legacy
    bl, ql, pl, Ql = P.multipole_boundary(legacy_geom, gl["rho"], 2)
    assert abs(ql - float(gl["q"])) < 1e-13 and _rel(bl, gl["boundary_values"]) < 1e-13


def test_oracle_poisson_solutions(golden_monitor, golden_legacy, monitor_geom, legacy_geom):
    g = golden_monitor
    ref = P.solve_monitor(monitor_geom, g["rho"], solver="bicgstab")
    assert ref["iterations"] == int(g["hartree_iterations"])
    assert _rel(ref["potential"], g["hartree_potential"]) < 1e-12
    tight = P.solve_monitor(monitor_geom, g["rho"], solver="direct")
    # the reference BiCGSTAB stops at rtol 1e-8: the converged discrete solution differs by less than that
    assert _rel(tight["potential"], g["hartree_potential"]) < 1e-6
    assert abs(P.hartree_energy(g["rho"], monitor_geom, ref["potential"]) - float(g["hartree_energy"])) < 1e-12
    gl = golden_legacy
    lref = P.solve_legacy(legacy_geom, gl["rho"], solver="bicgstab")
    assert lref["iterations"] == int(gl["hartree_iterations"])
    assert _rel(lref["potential"], gl["hartree_potential"]) < 1e-12
    ltight = P.solve_legacy(legacy_geom, gl["rho"], solver="direct")
    assert _rel(ltight["potential"], gl["hartree_potential"]) < 1e-6


def test_oracle_recorded_legacy_chain():
    """Recorded legacy 51^3 static chain (``audit/baselines.py:819-822``)."""

    from isogriddft_gb300.config import H2_BENCHMARK_CASE
    from isogriddft_gb300.grid import build_default_h2_grid_geometry

    geom = build_default_h2_grid_geometry()
    psi = S.bonding_trial_orbital(H2_BENCHMARK_CASE, geom)
    rho = 2.0 * psi * psi
    assert abs(2.0 * K.integrate_field(psi * K.legacy_kinetic(psi, geom), geom) - 1.995064629672) < 1e-11
    assert abs(K.integrate_field(rho * PS.local_potential(H2_BENCHMARK_CASE, geom), geom) + 4.347356525602) < 1e-11
    assert abs(X.xc_energy(psi * psi, psi * psi, geom) + 0.869107874980) < 1e-11
    v = P.solve_legacy(geom, rho, solver="bicgstab")["potential"]
    assert abs(P.hartree_energy(rho, geom, v) - 1.748670071699) < 5e-9


def test_oracle_xc_properties():
    rng = np.random.default_rng(0)
    ru = rng.uniform(1e-6, 1.0, 200)
    rd = rng.uniform(1e-6, 1.0, 200)
    e = X.lsda(ru, rd)
    # potentials are the functional derivative of the energy density (central differences)
    h = 1e-7
    for key, du, dd in (("v_xc_up", h, 0.0), ("v_xc_down", 0.0, h)):
        fd = (X.lsda(ru + du, rd + dd)["energy_density"] - X.lsda(ru - du, rd - dd)["energy_density"]) / (2 * h)
        np.testing.assert_allclose(e[key], fd, rtol=2e-6, atol=1e-8)
    # spin symmetry and zero density
    sw = X.lsda(rd, ru)
    np.testing.assert_allclose(sw["v_xc_up"], e["v_xc_down"], rtol=1e-14)
    z = X.lsda(np.zeros(3), np.zeros(3))
    assert np.all(z["eps_xc"] == 0) and np.all(z["v_xc_up"] == 0)
    with pytest.raises(ValueError):
        X.lsda(-np.ones(3), np.ones(3))


def test_oracle_eigensolver(golden_monitor, monitor_geom):
    from isogriddft_gb300.config import H2_BENCHMARK_CASE

    g = golden_monitor
    guess = OE.default_guess(H2_BENCHMARK_CASE, monitor_geom, 8)
    assert np.max(np.abs(np.abs(guess) - np.abs(g["guess8"]))) < 1e-10
    veff = g["veff"]
    apply_h = lambda b: K.hpsi_block(b, monitor_geom, veff, "trial_fix")  # noqa: E731
    res = OE.block_subspace_iteration(apply_h, H2_BENCHMARK_CASE, monitor_geom, 2, tolerance=1e-7, max_iterations=3000)
    assert res["converged"]
    np.testing.assert_allclose(res["eigenvalues"], g["eig_values"], atol=1e-8)
    ev = OE.eigsh_route(apply_h, H2_BENCHMARK_CASE, monitor_geom, 2, tolerance=1e-8, max_iterations=4000)
    np.testing.assert_allclose(ev["eigenvalues"], g["eig_values"], atol=1e-8)


def test_oracle_density_helpers(golden_monitor, monitor_geom):
    g = golden_monitor
    d = S.density(g["eig_orbitals"], (1.0, 1.0), monitor_geom)
    np.testing.assert_allclose(d, g["density"], rtol=1e-14, atol=1e-300)
    r = S.renormalize(d, 2.0, monitor_geom)
    np.testing.assert_allclose(r, g["density_renorm"], rtol=1e-13)
    assert abs(S.residual(g["rho"] / 2, g["rho"] / 2, r / 2, r / 2, monitor_geom) - float(g["density_residual"])) < 1e-13


@pytest.mark.parametrize("pre", ["none", "diag", "separable", "line"])
def test_oracle_jax_route_cg_reaches_the_direct_solution(golden_monitor, monitor_geom, pre):
    """The oracle's restatement of the reference's JAX-route CG and its three preconditioners
    (``poisson/poisson_jax.py:248-750``; JAX is absent here, so the route itself cannot be run:
    parity of the iterates is unpinned) converges to the direct solution of the same system.
    Tolerance 1e-8 on max |r|: with the separable preconditioner CG stalls near 6e-10 on this
    operator (the production closure makes -L slightly non-symmetric)."""

    ref = P.solve_monitor(monitor_geom, golden_monitor["rho"], solver="direct")
    x, it, rmax, conv = P.jax_route_cg(monitor_geom, ref["rhs"][1:-1, 1:-1, 1:-1], tolerance=1e-8,
                                       max_iterations=2000, preconditioner=pre)
    assert conv and rmax < 1e-8 and 0 < it < 2000
    want = ref["potential"][1:-1, 1:-1, 1:-1]
    assert np.max(np.abs(x - want)) < 5e-8 * np.max(np.abs(want))
    if pre == "line":
        assert P.jax_route_preconditioner(monitor_geom, "line").axis in (0, 1, 2)


def test_legacy_hamiltonian_matrix_matches_the_stencil(legacy_geom, golden_legacy):
    """The oracle's sparse legacy Hamiltonian equals its stencil apply (the matrix behind the
    eigenvalue-definition check); the operator is W-asymmetric by a few 1e-4 (Frobenius), so
    the true eigenvalues and those of the W-symmetric part differ slightly."""

    rng = np.random.default_rng(4)
    veff = rng.normal(size=legacy_geom.spec.shape)
    h = K.legacy_hamiltonian_matrix(legacy_geom, veff)
    psi = rng.normal(size=legacy_geom.spec.shape)
    want = K.legacy_kinetic(psi, legacy_geom) + veff * psi
    assert np.max(np.abs(h @ psi.reshape(-1) - want.reshape(-1))) <= 1e-13 * np.max(np.abs(want))
    sw = np.sqrt(legacy_geom.cell_volumes.reshape(-1))
    a = (h.multiply(sw[:, None])).multiply(1.0 / sw[None, :])
    asym = np.sqrt((a - a.T).multiply(a - a.T).sum()) / np.sqrt(a.multiply(a).sum())
    assert 1e-6 < asym < 1e-2
    vs = K.weighted_symmetric_eigenvalues(h, legacy_geom, 2)
    vn = K.nonsymmetric_eigenvalues(h, 2)
    assert np.all(np.abs(vs - vn) < 1e-2)


@pytest.mark.parametrize("pre", ["diag", "line", "separable"])
def test_jax_route_preconditioner_host_data_applies_as_the_oracle(monitor_geom, pre):
    """The host-built data of the GPU JAX-route preconditioners (``poisson._pcg_preconditioner``),
    applied in NumPy in the device kernels' order (diagonal scaling; the Thomas forward and
    backward sweeps along the chosen axis; gather, three sine-basis mode products, the
    spectral division, three more, scatter), equals the oracle's preconditioner
    (``poisson/poisson_jax.py:248-579``): FP64 data to 1e-12, the FP32 separable data to 1e-5."""

    from isogriddft_gb300.poisson import _pcg_preconditioner

    geom = monitor_geom
    shape = geom.spec.shape
    inner = tuple(n - 2 for n in shape)
    r = np.random.default_rng(17).normal(size=inner)
    want = P.jax_route_preconditioner(geom, pre)(r)
    d64, d32, axis = _pcg_preconditioner(geom, pre, "cpu")
    full_r = np.zeros(shape)
    full_r[1:-1, 1:-1, 1:-1] = r
    if pre == "diag":
        z = (d64.numpy().reshape(shape) * full_r)[1:-1, 1:-1, 1:-1]
        tol = 1e-12
    elif pre == "line":
        lower, cprime, inv_den = (a.reshape(shape) for a in d64.numpy().reshape(3, -1))
        mv = lambda a: np.moveaxis(a[1:-1, 1:-1, 1:-1], axis, -1)  # noqa: E731
        L, C, D, R = mv(lower), mv(cprime), mv(inv_den), mv(full_r)
        m = R.shape[-1]
        dd = np.zeros_like(R)
        prev = np.zeros(R.shape[:-1])
        for i in range(m):
            prev = (R[..., i] - L[..., i] * prev) * D[..., i]
            dd[..., i] = prev
        zz = dd.copy()
        for i in range(m - 2, -1, -1):
            zz[..., i] = dd[..., i] - C[..., i] * zz[..., i + 1]
        z = np.moveaxis(zz, -1, axis)
        tol = 1e-12
    else:
        data = d32.numpy().astype(np.float64)
        mx, my, mz = inner
        Sx = data[: mx * mx].reshape(mx, mx)
        Sy = data[mx * mx: mx * mx + my * my].reshape(my, my)
        Sz = data[mx * mx + my * my: mx * mx + my * my + mz * mz].reshape(mz, mz)
        inv = data[mx * mx + my * my + mz * mz:].reshape(inner)
        modes = lambda t: np.einsum("ia,jb,kc,abc->ijk", Sx, Sy, Sz, t)  # noqa: E731
        z = modes(modes(r) * inv)
        tol = 1e-5
    assert np.max(np.abs(z - want)) <= tol * np.max(np.abs(want)), np.max(np.abs(z - want)) / np.max(np.abs(want))
