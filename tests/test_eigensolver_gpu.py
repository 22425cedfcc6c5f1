"""GPU parity of the block linear algebra (Gram, rotation), the GTH terms and
the fixed-potential block eigensolver against the oracle and the reference's
golden values (H2 on the 13x13x15 A-grid)."""

import numpy as np
import pytest

from tests.conftest import gpu_available

import oracle.kinetic as OK
import oracle.pseudo as OP

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not gpu_available():
        pytest.skip("needs a CUDA GPU")


def _rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / max(np.max(np.abs(b)), 1e-300))


@pytest.mark.parametrize("n,a,b", [(1, 1, 1), (1000, 3, 5), (70001, 70, 9), (4096, 130, 130), (2000003, 16, 16),
                                   (300001, 13, 12), (100003, 64, 64), (777, 1, 33), (2000000, 16, 16),
                                   (300000, 13, 12), (100004, 64, 64), (4096, 60, 60), (262144, 32, 7), (36, 5, 5)])
@pytest.mark.parametrize("dt", ["fp64", "fp32"])
def test_block_gram_and_rotate_match_numpy(n, a, b, dt):
    import torch

    from isogriddft_gb300 import _lib
    from isogriddft_gb300.device import ptr, stream_ptr

    rng = np.random.default_rng(n + a + b)
    A = rng.normal(size=(a, n))
    B = rng.normal(size=(b, n))
    w = rng.uniform(0.5, 2.0, n)
    tdt = torch.float64 if dt == "fp64" else torch.float32
    igd = _lib.IGD_F64 if dt == "fp64" else _lib.IGD_F32
    Ad, Bd = torch.tensor(A, device="cuda", dtype=tdt), torch.tensor(B, device="cuda", dtype=tdt)
    wd = torch.tensor(w, device="cuda")
    out = torch.full((a, b), 7.0, dtype=torch.float64, device="cuda")
    wsb = int(_lib.call("igd_block_gram_workspace_bytes", n, a, b))
    ws = torch.empty(wsb, dtype=torch.uint8, device="cuda")
    _lib.check(_lib.call("igd_block_gram", igd, n, a, ptr(Ad), n, b, ptr(Bd), n, ptr(wd), ptr(out), 0, ptr(ws), wsb,
                         stream_ptr()))
    Ah, Bh = Ad.double().cpu().numpy(), Bd.double().cpu().numpy()
    ref = Ah @ (w[:, None] * Bh.T)
    tol = 1e-12 if dt == "fp64" else 2e-6
    assert _rel(out.cpu().numpy(), ref) < tol
    # accumulate, unweighted
    _lib.check(_lib.call("igd_block_gram", igd, n, a, ptr(Ad), n, b, ptr(Bd), n, None, ptr(out), 1, ptr(ws), wsb,
                         stream_ptr()))
    assert _rel(out.cpu().numpy(), ref + Ah @ Bh.T) < tol * 4
    # two-part rotation: out = A^T C1 + B^T C2
    c = 37
    C1, C2 = rng.normal(size=(a, c)), rng.normal(size=(b, c))
    o = torch.empty((c, n), dtype=tdt, device="cuda")
    C1d, C2d = torch.tensor(C1, device="cuda"), torch.tensor(C2, device="cuda")
    _lib.check(_lib.call("igd_block_rotate", igd, n, a, ptr(Ad), n, ptr(C1d), b, ptr(Bd), n, ptr(C2d), c, ptr(o), n, 0,
                         stream_ptr()))
    rref = C1.T @ Ah + C2.T @ Bh
    assert _rel(o.double().cpu().numpy(), rref) < (1e-13 if dt == "fp64" else 1e-5)


def test_gth_local_potential_matches_golden(golden_monitor, golden_legacy, monitor_geom, legacy_geom):
    from isogriddft_gb300 import pseudo
    from isogriddft_gb300.config import H2_BENCHMARK_CASE

    v = pseudo.evaluate_local_ionic_potential(H2_BENCHMARK_CASE, monitor_geom).total_local_potential
    assert _rel(v, golden_monitor["vloc"]) < 1e-13
    v = pseudo.evaluate_local_ionic_potential(H2_BENCHMARK_CASE, legacy_geom).total_local_potential
    assert _rel(v, golden_legacy["vloc"]) < 1e-13


def test_gth_nonlocal_matches_golden_and_oracle(golden_monitor, monitor_geom):
    import torch

    from isogriddft_gb300 import pseudo
    from isogriddft_gb300.config import make_molecule_case
    from isogriddft_gb300.device import device_grid

    n2 = make_molecule_case("N2", [("N", (0.0, 0.0, -1.037)), ("N", (0.0, 0.0, 1.037))])
    got = pseudo.evaluate_nonlocal_ionic_action(n2, monitor_geom, golden_monitor["psi"]).total_nonlocal_action
    assert _rel(got, golden_monitor["n2_nonlocal_psi"]) < 1e-12
    # a block of orbitals with an extra p channel on N, in FP64 and FP32
    extra = {"N": ((1, 0.27013369, ((8.0, 1.5), (1.5, -2.0))),)}
    rnd = golden_monitor["rnd"]
    ref = np.stack([OP.nonlocal_action(n2, monitor_geom, r, extra_channels=extra) for r in rnd])
    dg = device_grid(monitor_geom)
    tab = pseudo.projector_table(n2, monitor_geom, extra)
    for tdt, tol in ((torch.float64, 1e-12), (torch.float32, 2e-5)):
        p = torch.tensor(rnd.reshape(3, -1), device="cuda", dtype=tdt)
        out = torch.zeros_like(p)
        tab.apply(dg, p, out)
        assert _rel(out.double().cpu().numpy().reshape(rnd.shape), ref) < tol


def test_default_guess_matches_golden(golden_monitor, monitor_geom):
    from isogriddft_gb300 import ks
    from isogriddft_gb300.config import H2_BENCHMARK_CASE
    from isogriddft_gb300.device import device_grid

    g = ks.default_guess_device(H2_BENCHMARK_CASE, monitor_geom, device_grid(monitor_geom), 8)
    # The x and y moment functions of H2 (atoms on the z axis) have equal
    # weighted norms, so any rotation within that pair is an equally valid SVD
    # basis: compare through the W-overlap with the golden block, which must be
    # orthogonal and couple only neighbours in the singular-value order.
    g = g.cpu().numpy().reshape(8, -1)
    ref = golden_monitor["guess8"].reshape(8, -1)
    M = g @ (monitor_geom.cell_volumes.reshape(-1)[:, None] * ref.T)
    np.testing.assert_allclose(M @ M.T, np.eye(8), atol=1e-10)
    far = np.abs(np.subtract.outer(np.arange(8), np.arange(8))) > 1
    assert np.max(np.abs(M[far])) < 1e-8


def test_weighted_orthonormalize(monitor_geom, golden_monitor):
    from isogriddft_gb300 import ks

    q = ks.weighted_orthonormalize_orbitals(golden_monitor["rnd"], monitor_geom)
    ov = ks.weighted_overlap_matrix(q, monitor_geom)
    np.testing.assert_allclose(ov, np.eye(3), atol=1e-12)
    with pytest.raises(ValueError):
        ks.weighted_orthonormalize_orbitals(np.stack([golden_monitor["psi"]] * 2), monitor_geom)


@pytest.mark.parametrize("fused", [True, False])
@pytest.mark.parametrize("precision,tol,atol", [("fp64", 1e-7, 1e-8), ("fp32", 3e-4, 1e-5)])
def test_eigensolver_matches_golden(golden_monitor, monitor_geom, precision, tol, atol, fused, monkeypatch):
    from isogriddft_gb300 import ks
    from isogriddft_gb300.config import H2_BENCHMARK_CASE

    if not fused:
        orig = ks.block_subspace_iteration_device
        monkeypatch.setattr(ks, "block_subspace_iteration_device", lambda *a, **kw: orig(*a, fused=False, **kw))
    g = golden_monitor
    rho = g["rho"]
    res = ks.solve_fixed_potential_static_local_eigenproblem(
        monitor_geom, rho / 2, rho / 2, "up", 2, case=H2_BENCHMARK_CASE, xc_potential=g["vxc"],
        hartree_potential=g["hartree_potential"], kinetic_version="trial_fix", tolerance=tol, max_iterations=3000,
        precision=precision)
    assert res.converged
    np.testing.assert_allclose(res.operator_context.effective_local_potential, g["veff"], rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(res.eigenvalues, g["eig_values"], atol=atol)
    assert res.max_orthogonality_error < (1e-10 if precision == "fp64" else 1e-5)
    # Ritz vectors satisfy H x = lambda x (oracle operator, FP64)
    for lam, x in zip(res.eigenvalues, res.orbitals):
        hx = OK.hpsi_block(x[None], monitor_geom, g["veff"], "trial_fix")[0]
        r = np.sqrt(np.sum((hx - lam * x) ** 2 * monitor_geom.cell_volumes))
        assert r < (10 * tol if precision == "fp64" else 5e-3)


def test_static_ks_route_with_nonlocal(monitor_geom, golden_monitor):
    """N2 pseudopotential on the H2 grid, nonlocal term included, against the oracle operator.

    With the trial-fix closure H is symmetric and the iteration converges; the
    production closure (one-sided second-order edge derivatives) is not
    self-adjoint, so the residual stalls near 2e-2 while the Ritz values settle:
    that route is compared after a fixed 60 iterations."""

    from isogriddft_gb300 import ks
    from isogriddft_gb300.config import make_molecule_case

    import oracle.eigensolver as OE

    n2 = make_molecule_case("N2", [("N", (0.0, 0.0, -1.037)), ("N", (0.0, 0.0, 1.037))])
    g = golden_monitor
    rho = g["rho"]
    veff = g["veff"]
    zero = np.zeros_like(veff)

    def oracle_h(kin):
        def apply_h(b):
            hb = OK.hpsi_block(b, monitor_geom, veff, kin)
            return hb + np.stack([OP.nonlocal_action(n2, monitor_geom, x) for x in b])
        return apply_h

    ctx = ks.prepare_fixed_potential_static_local_operator(
        monitor_geom, rho / 2, rho / 2, "up", n2, zero, zero, veff, kinetic_version="trial_fix", include_nonlocal=True)
    res = ks.solve_fixed_potential_static_local_eigenproblem(monitor_geom, rho / 2, rho / 2, "up", 2, case=n2,
                                                             operator_context=ctx, tolerance=1e-7,
                                                             max_iterations=3000)
    assert res.converged
    ref = OE.block_subspace_iteration(oracle_h("trial_fix"), n2, monitor_geom, 2, tolerance=1e-7, max_iterations=3000)
    np.testing.assert_allclose(res.eigenvalues, ref["eigenvalues"], atol=1e-8)

    res = ks.solve_fixed_potential_eigenproblem(monitor_geom, rho / 2, rho / 2, "up", 2, case=n2,
                                                local_ionic_potential=zero, hartree_potential=zero, xc_potential=veff,
                                                tolerance=1e-7, max_iterations=60)
    assert not res.converged and res.iteration_count == 60
    ref = OE.block_subspace_iteration(oracle_h("production"), n2, monitor_geom, 2, tolerance=1e-7, max_iterations=60)
    np.testing.assert_allclose(res.eigenvalues, ref["eigenvalues"], atol=1e-8)


def test_preconditioned_iteration_matches_golden(golden_monitor, monitor_geom):
    """Jacobi-preconditioned residual expansion: same Ritz pairs, fewer iterations; probed diag(T)."""

    import torch

    from isogriddft_gb300 import ks
    from isogriddft_gb300.config import H2_BENCHMARK_CASE
    from isogriddft_gb300.device import device_grid

    g = golden_monitor
    rho = g["rho"]
    ctx = ks.prepare_fixed_potential_static_local_operator(
        monitor_geom, rho / 2, rho / 2, "up", H2_BENCHMARK_CASE, hartree_potential=g["hartree_potential"],
        xc_potential=g["vxc"], kinetic_version="trial_fix")
    op = ks.operator_for(ctx, "fp64")
    plain = ks.block_subspace_iteration_device(op, H2_BENCHMARK_CASE, 2, tolerance=1e-7, max_iterations=3000)
    pre = ks.block_subspace_iteration_device(op, H2_BENCHMARK_CASE, 2, tolerance=1e-7, max_iterations=3000,
                                             preconditioner=ks.JacobiPreconditioner(op))
    assert plain["converged"] and pre["converged"]
    np.testing.assert_allclose(pre["eigenvalues"], g["eig_values"], atol=1e-8)
    assert pre["iteration_count"] <= plain["iteration_count"]
    # probed diagonal vs the oracle operator on unit vectors
    d = ks.kinetic_diagonal(device_grid(monitor_geom), "trial_fix", torch.float64).cpu().numpy()
    shape = monitor_geom.spec.shape
    for idx in [(0, 0, 0), (6, 6, 7), (12, 3, 14), (1, 12, 0)]:
        e = np.zeros(shape)
        e[idx] = 1.0
        assert abs(OK.kinetic(e, monitor_geom, "trial_fix")[idx] - d[np.ravel_multi_index(idx, shape)]) < 1e-10
