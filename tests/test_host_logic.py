"""Host-side logic that needs no GPU: occupations, ion-ion energy, scan layout, block rules,
small-matrix whitening, precision names."""

import numpy as np
import pytest

import oracle.scf as OS


def test_occupations_and_ion_repulsion():
    from isogriddft_gb300 import scf
    from isogriddft_gb300.config import H2_BENCHMARK_CASE, make_benzene_case, make_molecule_case

    s = scf.resolve_h2_spin_occupations("singlet")
    t = scf.resolve_h2_spin_occupations("triplet")
    assert (s.n_alpha, s.n_beta, t.n_alpha, t.n_beta) == (1, 1, 2, 0)
    assert scf.evaluate_ion_ion_repulsion(H2_BENCHMARK_CASE) == pytest.approx(1.0 / 1.4, rel=1e-15)
    n2 = make_molecule_case("N2", [("N", (0.0, 0.0, -1.037)), ("N", (0.0, 0.0, 1.037))])
    assert scf.evaluate_ion_ion_repulsion(n2) == pytest.approx(OS.ion_ion_repulsion(n2), rel=1e-14)
    occ = scf.resolve_spin_occupations("singlet", n2)
    assert occ.n_alpha == occ.n_beta == 5
    bz = make_benzene_case()
    assert scf.resolve_spin_occupations("singlet", bz).n_alpha == 15
    with pytest.raises(ValueError):
        scf.resolve_h2_spin_occupations("singlet", n2)
    with pytest.raises(ValueError):
        scf.resolve_h2_spin_occupations("quintet")


def test_scan_points_are_seeded_and_tma_aligned():
    from isogriddft_gb300 import scan

    a, b = scan.scan_points(64), scan.scan_points(64)
    assert a == b and len(a) == 64
    assert a[0].bond_length == 1.0 and a[-1].bond_length == 3.0
    assert [p.spin for p in a[:4]] == ["singlet", "triplet", "singlet", "triplet"]
    assert all(64 <= e <= 128 and e % 4 == 0 for p in a for e in p.shape)


def test_block_rules_and_whitening():
    from isogriddft_gb300 import ks

    assert ks.block_size(1) == 20 and ks.block_size(4) == 56 and ks.block_size(2, ncv=40) == 40
    rng = np.random.default_rng(0)
    A = rng.normal(size=(9, 9))
    G = A @ A.T + 1e-3 * np.eye(9)
    for T in (ks._whitening(G), ks._chol_whitening(G)):
        np.testing.assert_allclose(T.T @ G @ T, np.eye(9), atol=1e-9)
    # rank-deficient projected Gram: the truncated whitening drops the null direction
    B = rng.normal(size=(6, 3))
    M = B @ B.T
    T = ks._whiten_truncated(M, float(np.max(np.diag(M))), 1e-10)
    assert T.shape == (6, 3)
    np.testing.assert_allclose(T.T @ M @ T, np.eye(3), atol=1e-9)


def test_precision_names():
    from isogriddft_gb300.device import normalize_precision

    assert normalize_precision("FP64") == "fp64"
    assert normalize_precision("mixed") == "fp32"
    with pytest.raises(ValueError):
        normalize_precision("bf16")


def test_pulay_mixer_follows_the_reference_diis_rule():
    """``scf.PulayMixer`` on host tensors (a stand-in engine for the weighted sums) against a
    NumPy restatement of the reference's monitor-grid density DIIS (``scf/driver.py:2234-2294``:
    residual Gram with 1e-12 regularisation, coefficients rejected beyond 20, clip at zero,
    renormalise) and its schedule (``:4297-4318``: history of 4, extrapolation from iteration 3)."""

    from types import SimpleNamespace

    import numpy as np
    import torch

    from isogriddft_gb300.scf import PulayMixer

    rng = np.random.default_rng(4)
    n = 50
    w = rng.uniform(0.5, 1.5, n)
    wt = torch.as_tensor(w)

    class Engine:
        dg = SimpleNamespace(cell_volumes=wt, device=torch.device("cpu"))
        occ = SimpleNamespace(n_alpha=2, n_beta=1)

        def wdot(self, a, b=None):
            return torch.sum(a * wt * (1.0 if b is None else b)).reshape(1)

        def renormalized(self, rho, target):
            return torch.zeros_like(rho) if target == 0 else rho * (target / float(torch.sum(rho * wt)))

    def ref_diis(hist, na, nb):
        h = len(hist)
        B = -np.ones((h + 1, h + 1))
        B[-1, -1] = 0.0
        for i in range(h):
            for j in range(h):
                B[i, j] = np.sum(w * (hist[i][2] * hist[j][2] + hist[i][3] * hist[j][3]))
        B[:-1, :-1] += 1e-12 * max(float(np.max(np.abs(B[:-1, :-1]))), 1.0) * np.eye(h)
        rhs = np.zeros(h + 1)
        rhs[-1] = -1.0
        c = np.linalg.solve(B, rhs)[:-1]
        if not np.all(np.isfinite(c)) or np.max(np.abs(c)) > 20.0:
            return None
        up = np.maximum(sum(ci * e[0] for ci, e in zip(c, hist)), 0.0)
        dn = np.maximum(sum(ci * e[1] for ci, e in zip(c, hist)), 0.0)
        return up * na / np.sum(up * w), dn * nb / np.sum(dn * w)

    mixer = PulayMixer(Engine(), depth=4, warmup=3)
    hist = []
    for it in range(1, 8):
        up, dn = rng.uniform(0.1, 1.0, n), rng.uniform(0.1, 1.0, n)
        ru, rd = 0.05 * rng.normal(size=n) / it, 0.05 * rng.normal(size=n) / it
        got = mixer(*(torch.as_tensor(x) for x in (up, dn, ru, rd)))
        hist = (hist + [(up, dn, ru, rd)])[-4:]
        want = ref_diis(hist, 2, 1) if (it >= 3 and len(hist) >= 2) else None
        if want is None:
            want = (up, dn)
        np.testing.assert_allclose(got[0].numpy(), want[0], rtol=1e-12, atol=1e-14)
        np.testing.assert_allclose(got[1].numpy(), want[1], rtol=1e-12, atol=1e-14)


def test_reference_dry_run_fixture_schedule():
    """The reference's own A-grid dry runs (``tests/golden/dryrun_agrid_h2.json``): its Pulay run
    leaves the first three steps to linear mixing (they match the default run to the eigensolver
    tolerance) and converges; the default ten-step run does not."""

    import json
    import os

    from tests.conftest import GOLDEN

    d = json.load(open(os.path.join(GOLDEN, "dryrun_agrid_h2.json")))
    lin, pul = d["triplet_default"], d["triplet_diis_tight"]
    assert not lin["converged"] and lin["iterations"] == 10
    assert pul["converged"] and pul["iterations"] == len(pul["history"])
    for k in range(3):
        assert abs(lin["history"][k][1] - pul["history"][k][1]) < 5e-6
    assert abs(lin["history"][3][1] - pul["history"][3][1]) > 1e-3  # extrapolation from step 3 on
    assert abs(pul["energy"]["total"] - pul["history"][-1][1]) < 1e-12


def _fixture_engine(w, na, nb):
    from types import SimpleNamespace

    import torch

    wt = torch.as_tensor(w)

    class Engine:
        dg = SimpleNamespace(cell_volumes=wt, device=torch.device("cpu"))
        occ = SimpleNamespace(n_alpha=na, n_beta=nb)

        def wdot(self, a, b=None):
            return torch.sum(a * wt * (1.0 if b is None else b)).reshape(1)

        def renormalized(self, rho, target):
            return torch.zeros_like(rho) if target == 0 else rho * (target / float(torch.sum(rho * wt)))

    return Engine()


@pytest.mark.parametrize("name", ["diis", "anderson_default", "anderson_guarded", "anderson_strict", "broyden"])
def test_mixers_match_reference_fixture(name):
    """``mixing.PulayMixer`` / ``AndersonMixer`` / ``BroydenMixer`` on host tensors against the
    reference's own ``_apply_monitor_grid_density_diis`` / ``_anderson`` / ``_broyden_like``
    driven through its dry-run schedule (``tests/golden/mixers_h2.npz``, written by
    ``make_golden_mixers.py``): the densities returned at every iteration (FP64, 1e-10), and
    the used / fallback / rejected / reset iterations, history sizes, filtered sizes,
    effective damping and projected residual ratios."""

    import json
    import os

    import numpy as np
    import torch

    from isogriddft_gb300.mixing import AndersonMixer, BroydenMixer, PulayMixer
    from tests.conftest import GOLDEN

    d = np.load(os.path.join(GOLDEN, "mixers_h2.npz"))
    meta = json.loads(str(d["meta"]))[name]
    na, nb = (int(x) for x in d["occupations"])
    w = d["cell_volumes"].reshape(-1)
    eng = _fixture_engine(w, na, nb)
    p = dict(meta["params"])
    kind = meta["kind"]
    if kind == "diis":
        mixer = PulayMixer(eng, depth=p["history_length"], warmup=p["warmup"])
    elif kind == "anderson":
        mixer = AndersonMixer(eng, **p)
    else:
        mixer = BroydenMixer(eng, **p)
    want = d[f"{name}_out"]
    k = 0
    while f"in_{k}" in d:
        mu, md, ru, rd = (torch.as_tensor(np.ascontiguousarray(x.reshape(-1))) for x in d[f"in_{k}"])
        up, dn = mixer(mu, md, ru, rd)
        scale = np.max(np.abs(want[k]))
        np.testing.assert_allclose(up.numpy(), want[k][0].reshape(-1), rtol=0, atol=1e-10 * scale)
        np.testing.assert_allclose(dn.numpy(), want[k][1].reshape(-1), rtol=0, atol=1e-10 * scale)
        k += 1
    assert mixer.used == meta["used"]
    assert mixer.fallback == meta["fallback"]
    assert mixer.history_sizes == meta["sizes"]
    if kind == "anderson":
        assert mixer.rejected == meta["rejected"]
        assert mixer.resets == meta["resets"]
        assert mixer.filtered_sizes == meta["filtered"]
        np.testing.assert_allclose(mixer.effective_damping, d[f"{name}_damping"], rtol=1e-14)
        ratios = np.asarray([np.nan if r is None else r for r in mixer.projected_ratios])
        np.testing.assert_allclose(ratios, d[f"{name}_ratios"], rtol=1e-10)


def test_dry_run_options_are_validated_as_the_reference():
    """``scf._dry_run_hartree_options`` mirrors ``scf/driver.py:3380-3429``: unknown values and
    JAX-only options with the python backend raise ValueError with the reference's words;
    ``jacobi`` reads as ``diag``."""

    from isogriddft_gb300.scf import _dry_run_hartree_options

    assert _dry_run_hartree_options("python", "baseline", "none", "baseline", False) == \
        ("python", "baseline", "none", "baseline")
    assert _dry_run_hartree_options("JAX", "jax_loop", "Jacobi", "optimized", True) == \
        ("jax", "jax_loop", "diag", "optimized")
    for args, words in [(("cuda", "baseline", "none", "baseline", False), "hartree_backend must be"),
                        (("python", "baseline", "none", "baseline", True), "requires hartree_backend='jax'"),
                        (("jax", "fast", "none", "baseline", False), "jax_hartree_cg_impl must be"),
                        (("python", "jax_loop", "none", "baseline", False), "jax_hartree_cg_impl requires"),
                        (("jax", "jax_loop", "ilu", "baseline", False), "jax_hartree_cg_preconditioner must be"),
                        (("jax", "jax_loop", "none", "fast", False), "jax_hartree_line_preconditioner_impl must"),
                        (("python", "baseline", "line", "baseline", False), "requires hartree_backend='jax'"),
                        (("jax", "baseline", "line", "baseline", False), "currently requires jax_hartree_cg_impl")]:
        with pytest.raises(ValueError, match=words.replace("(", r"\(")):
            _dry_run_hartree_options(*args)


def test_hartree_potential_rejects_unknown_solver_options():
    """``poisson.solve_hartree_potential`` validates ``cg_impl``, ``cg_preconditioner`` and
    ``line_preconditioner_impl`` as ``poisson/poisson_jax.py:204-239`` does before any work."""

    from isogriddft_gb300.poisson import validate_hartree_solver_options

    assert validate_hartree_solver_options(cg_preconditioner="jacobi")[2] == "diag"
    with pytest.raises(ValueError, match="cg_impl must be"):
        validate_hartree_solver_options(cg_impl="scipy")
    with pytest.raises(ValueError, match="cg_preconditioner must be"):
        validate_hartree_solver_options(cg_preconditioner="ilu")
    with pytest.raises(ValueError, match="line_preconditioner_impl must be"):
        validate_hartree_solver_options(line_preconditioner_impl="fast")


def test_dry_run_result_has_the_reference_fields():
    """The reference-shaped dry-run result carries every field name of
    ``H2StaticLocalScfDryRunResult`` (``scf/driver.py:357-548``) that a caller reads, with the
    mixer diagnostics filled from the mixer object."""

    from types import SimpleNamespace

    import numpy as np

    from isogriddft_gb300.dryrun import H2StaticLocalScfDryRunResult, build_dry_run_result
    from isogriddft_gb300.pseudo import DEFAULT_MONITOR_PATCH_PARAMETERS
    from isogriddft_gb300.scf import SpinOccupations

    occ = SpinOccupations("triplet", 2, 2, 2, 0, (1.0, 1.0), ())
    energy = SimpleNamespace(total=-1.0)
    rec = [SimpleNamespace(energy=SimpleNamespace(total=-1.0 - 0.1 * i), density_residual=0.1 / (i + 1),
                           wall_time_seconds=0.01) for i in range(4)]
    res = SimpleNamespace(history=tuple(rec), converged=True, occupations=occ, eigenvalues_up=np.array([-0.7, -0.2]),
                          eigenvalues_down=np.array([]), orbitals_up=np.zeros((2, 3)), orbitals_down=np.zeros((0, 3)),
                          rho_up=np.zeros(3), rho_down=np.zeros(3), energy=energy, solve_up=None, solve_down=None)
    mixer = SimpleNamespace(used=[3, 4], fallback=[], rejected=[2], resets=[], history_sizes=[1, 2, 3, 4],
                            filtered_sizes=[1, 2, 3, 4], effective_damping=[0.5, 0.5, 0.5],
                            projected_ratios=[1.2, 0.8, 0.7])
    opts = dict(diis_warmup_iterations=3, diis_history_length=4, anderson_warmup_iterations=2,
                anderson_history_length=4, anderson_regularization=1e-8, anderson_damping=0.5,
                anderson_step_clip_factor=None, anderson_reset_on_growth=False, anderson_reset_growth_factor=1.1,
                anderson_adaptive_damping_enabled=False, anderson_min_damping=0.35, anderson_max_damping=0.75,
                anderson_acceptance_residual_ratio_threshold=1.02, anderson_collinearity_cosine_threshold=0.995,
                broyden_warmup_iterations=3, broyden_history_length=4, broyden_regularization=1e-8,
                broyden_damping=0.5)
    r = build_dry_run_result(res, kinetic_version="trial_fix", mixer=mixer, mixer_name="anderson", options=opts,
                             hartree_iterations=[40, 20, 10, 8], hartree_options=("python", "baseline", "none",
                                                                                 "baseline"),
                             patch_parameters=DEFAULT_MONITOR_PATCH_PARAMETERS, total_wall=1.0)
    assert isinstance(r, H2StaticLocalScfDryRunResult)
    assert r.path_type == "monitor_a_grid_plus_patch" and r.anderson_enabled and not r.diis_enabled
    assert r.anderson_used_iterations == (3, 4) and r.anderson_rejected_iterations == (2,)
    assert r.diis_history_sizes == (0, 0, 0, 0) and r.diis_used_iterations == ()
    assert r.iteration_count == 4 and r.lowest_eigenvalue == -0.7
    assert r.hartree_cg_iterations_history == (40, 20, 10, 8) and r.first_hartree_cg_iterations == 40
    assert r.parameter_summary.grid_shape == (83, 83, 101) and r.controller_name == "baseline_linear"
    assert r.energy_history == tuple(x.energy.total for x in rec)


def test_right_ritz_host_step():
    """The fused eigensolver's host step with right Ritz pairs: on a symmetric operator it is
    the symmetrised step (same Ritz values, same next rotation up to column signs); on a
    non-symmetric one its Ritz pairs are eigenpairs of the projected matrix it returns
    (P V = V diag(lam)) and its Ritz values move away from the symmetrised step's."""

    from isogriddft_gb300.ks import subspace_host_step_numpy

    rng = np.random.default_rng(21)
    n, m, k = 240, 8, 3
    A = rng.standard_normal((n, n))
    H = A + A.T + np.diag(np.arange(n, dtype=float))
    B, _ = np.linalg.qr(rng.standard_normal((n, m)))
    R = rng.standard_normal((n, m))
    X = np.hstack([B, R])
    for op, symmetric in ((H, True), (H + 2e-3 * rng.standard_normal((n, n)), False)):
        G0, G1 = X.T @ (op @ X), X.T @ X
        c_s, P_s, l_s, V_s = subspace_host_step_numpy(G0, G1, m, k, 1e-10)
        c_r, P_r, l_r, V_r = subspace_host_step_numpy(G0, G1, m, k, 1e-10, right=True)
        assert c_r.shape == c_s.shape and V_r.shape == V_s.shape
        np.testing.assert_allclose(np.linalg.norm(V_r, axis=0), 1.0, rtol=1e-12)
        np.testing.assert_allclose(P_r @ V_r[:, :k], V_r[:, :k] * l_r[None, :k], atol=1e-8 * np.abs(l_r).max())
        if symmetric:
            np.testing.assert_allclose(l_r, l_s, rtol=1e-12, atol=1e-10)
            np.testing.assert_allclose(np.abs(V_r[:, :k]), np.abs(V_s[:, :k]), atol=1e-8)
        else:
            assert np.max(np.abs(l_r[:k] - l_s[:k])) > 1e-9


def test_jax_route_rejects_nonuniform_logical_axes(monitor_geom):
    """The GPU JAX route builds its operator data from the logical spacing and, like the
    reference (``poisson/poisson_jax.py:236-245``), rejects a non-uniform logical axis."""

    from dataclasses import replace

    from isogriddft_gb300.poisson import _pcg_preconditioner

    assert _pcg_preconditioner(monitor_geom, "none", "cpu") == (None, None, 0)
    lx = np.asarray(monitor_geom.logical_x, dtype=np.float64).copy()
    lx[1:-1] += 0.1 * np.diff(lx)[0] * np.sin(np.arange(1, lx.size - 1))
    bad = replace(monitor_geom, logical_x=lx)
    for kind in ("none", "diag", "separable", "line"):
        with pytest.raises(ValueError, match="expect uniform logical axes"):
            _pcg_preconditioner(bad, kind, "cpu")


def test_poisson_rejects_nonuniform_logical_axes(monitor_geom):
    """The Poisson drop-in checks the logical axes before any device work, with the reference's
    message (``poisson/open_boundary.py:112-119``)."""

    from dataclasses import replace

    from isogriddft_gb300 import poisson

    ly = np.asarray(monitor_geom.logical_y, dtype=np.float64).copy()
    ly[1:-1] += 0.1 * np.diff(ly)[0] * np.cos(np.arange(1, ly.size - 1))
    bad = replace(monitor_geom, logical_y=ly)
    with pytest.raises(ValueError, match="expects a uniform logical y-axis"):
        poisson.solve_open_boundary_poisson(bad, np.zeros(monitor_geom.spec.shape))


def test_poisson_axis_check_reads_both_grid_types(legacy_geom):
    """The legacy geometry names its axes ``x_logical``: the same check applies to it."""

    from dataclasses import replace

    from isogriddft_gb300 import poisson

    xl = np.asarray(legacy_geom.x_logical, dtype=np.float64).copy()
    xl[1:-1] += 0.1 * np.diff(xl)[0] * np.sin(np.arange(1, xl.size - 1))
    with pytest.raises(ValueError, match="expects a uniform logical x-axis"):
        poisson.solve_open_boundary_poisson(replace(legacy_geom, x_logical=xl), np.zeros(legacy_geom.spec.shape))


def test_geometry_checks_use_the_reference_messages(monitor_geom, legacy_geom):
    """``device.validate_geometry`` (run before any device copy) raises the reference
    operators' messages (``ops/kinetic.py:76-84, 156-162``)."""

    from dataclasses import replace

    from isogriddft_gb300 import device

    device.validate_geometry(monitor_geom)
    device.validate_geometry(legacy_geom)
    lz = np.asarray(monitor_geom.logical_z, dtype=np.float64).copy()
    lz[1:-1] += 0.1 * np.diff(lz)[0] * np.sin(np.arange(1, lz.size - 1))
    cases = [(replace(monitor_geom, logical_z=lz), "uniform logical z-axis")]
    j = np.array(monitor_geom.jacobian, dtype=np.float64)
    j[3, 4, 5] = np.nan
    cases.append((replace(monitor_geom, jacobian=j), "Jacobian must be finite"))
    j = np.array(monitor_geom.jacobian, dtype=np.float64)
    j[3, 4, 5] = -1.0
    cases.append((replace(monitor_geom, jacobian=j), "Jacobian must stay strictly positive"))
    g = np.array(monitor_geom.inverse_metric_tensor, dtype=np.float64)
    g[1, 1, 1, 0, 2] = np.inf
    cases.append((replace(monitor_geom, inverse_metric_tensor=g), "inverse metric tensor must be finite"))
    yl = np.asarray(legacy_geom.y_logical, dtype=np.float64).copy()
    yl[1:-1] += 0.1 * np.diff(yl)[0] * np.cos(np.arange(1, yl.size - 1))
    cases.append((replace(legacy_geom, y_logical=yl), "uniform logical y-axis"))
    for geom, msg in cases:
        with pytest.raises(ValueError, match=msg):
            device.validate_geometry(geom)
        with pytest.raises(ValueError, match=msg):  # before any device work
            device.DeviceGrid(geom)


def test_eigensolver_options_use_the_reference_messages(monitor_geom, legacy_geom):
    """Option checks of the fixed-potential eigensolver drop-in, with the reference's messages
    (``ks/eigensolver.py``), raised before any device work."""

    from isogriddft_gb300 import ks

    shape = monitor_geom.spec.shape
    rho = np.zeros(shape)
    with pytest.raises(ValueError, match="spin_channel must be `up` or `down`; received `sideways`"):
        ks.prepare_fixed_potential_static_local_operator(monitor_geom, rho, rho, "sideways")
    with pytest.raises(ValueError, match="kinetic_version must be `production` or `trial_fix`"):
        ks.prepare_fixed_potential_static_local_operator(monitor_geom, rho, rho, "up", kinetic_version="exact")
    with pytest.raises(ValueError, match="solver_backend must be `auto`, `jax`, or `scipy_fallback`"):
        ks.solve_fixed_potential_static_local_eigenproblem(monitor_geom, rho, rho, "up", 2, solver_backend="gpu")
    with pytest.raises(ValueError, match="initial_subspace_size must be at least k"):
        ks.solve_fixed_potential_static_local_eigenproblem(monitor_geom, rho, rho, "up", 3, initial_subspace_size=2)
    with pytest.raises(ValueError, match="requires `use_jax_block_kernels=True` and a MonitorGridGeometry"):
        ks.solve_fixed_potential_static_local_eigenproblem(monitor_geom, rho, rho, "up", 2, solver_backend="jax")
    lrho = np.zeros(legacy_geom.spec.shape)
    with pytest.raises(ValueError, match="requires `use_jax_block_kernels=True` and a MonitorGridGeometry"):
        ks.solve_fixed_potential_static_local_eigenproblem(legacy_geom, lrho, lrho, "up", 2, solver_backend="jax",
                                                           use_jax_block_kernels=True)


def test_scf_case_and_dry_run_messages_follow_the_reference():
    """H2 case and spin-state checks (``scf/driver.py:557-590``) and the dry run's argument checks
    in the reference's order (``scf/driver.py:3229-3247``), all raised before any device work."""

    from dataclasses import replace

    from isogriddft_gb300 import scf
    from isogriddft_gb300.config import H2_BENCHMARK_CASE, make_h2_case, make_molecule_case

    with pytest.raises(ValueError, match=r"Spin state `quintet` is not configured for `h2_r1p4_bohr`\. "
                                         r"Available states: singlet, triplet\."):
        scf.resolve_h2_spin_occupations("quintet")
    assert scf.resolve_h2_spin_occupations(" Triplet ").n_alpha == 2
    assert scf.resolve_h2_spin_occupations("singlet", make_h2_case(1.6)).total_electrons == 2
    cation = replace(H2_BENCHMARK_CASE, charge=1)
    with pytest.raises(ValueError, match="supports only neutral H2; received charge=1"):
        scf.resolve_h2_spin_occupations("singlet", cation)
    n2 = make_molecule_case("N2", [("N", (0.0, 0.0, -1.037)), ("N", (0.0, 0.0, 1.037))])
    with pytest.raises(ValueError, match="supports only H2 geometries; received `N2`"):
        scf.resolve_h2_spin_occupations("singlet", n2)
    angstrom = replace(H2_BENCHMARK_CASE, geometry=replace(H2_BENCHMARK_CASE.geometry, unit="Angstrom"))
    with pytest.raises(ValueError, match="expects Bohr geometries; received `Angstrom`"):
        scf.resolve_h2_spin_occupations("singlet", angstrom)

    dry = scf.run_h2_monitor_grid_scf_dry_run
    with pytest.raises(ValueError, match="supports only neutral H2"):
        dry("singlet", cation, enable_cycle_breaker=True, enable_diis=True)
    with pytest.raises(ValueError, match="max_iterations must be positive"):
        dry("singlet", max_iterations=0, mixing=2.0)
    with pytest.raises(ValueError, match="cycle_breaker_weight must satisfy 0 <= cycle_breaker_weight <= 1"):
        dry("singlet", cycle_breaker_weight=1.5, enable_diis=True, enable_anderson=True)
    with pytest.raises(ValueError, match="at most one of cycle-breaker, DIIS, Anderson, or Broyden-like mixing"):
        dry("singlet", enable_cycle_breaker=True, enable_broyden=True)
    with pytest.raises(ValueError, match="diis_history_length must be at least 2"):  # checks before "not built"
        dry("singlet", diis_history_length=1, enable_hartree_tail_guard=True)
    with pytest.raises(NotImplementedError, match="enable_hartree_tail_guard"):
        dry("singlet", enable_cycle_breaker=True, enable_hartree_tail_guard=True)


def test_lsda_input_errors_name_the_field():
    """Once the kernel flags bad input, the error names the field in the reference's order
    (``xc/lsda.py:56-67``): rho_up before rho_down, finite values before the sign."""

    import torch

    from isogriddft_gb300 import xc

    ok = torch.ones(8, dtype=torch.float64)
    bad_sign = ok.clone()
    bad_sign[3] = -1e-10
    bad_nan = ok.clone()
    bad_nan[5] = float("nan")
    with pytest.raises(ValueError, match="^rho_up must contain only finite values"):
        xc._raise_input_error(bad_nan, bad_sign)
    with pytest.raises(ValueError, match="^rho_up must be non-negative up to roundoff"):
        xc._raise_input_error(bad_sign, bad_nan)
    with pytest.raises(ValueError, match="^rho_down must contain only finite values"):
        xc._raise_input_error(ok, bad_nan)
    with pytest.raises(ValueError, match="^rho_down must be non-negative up to roundoff"):
        xc._raise_input_error(ok.float(), bad_sign.float())
    tiny = ok.clone()
    tiny[0] = -1e-15  # within roundoff
    with pytest.raises(ValueError, match="^rho_up / rho_down"):
        xc._raise_input_error(tiny, ok)
    with pytest.raises(ValueError, match="supports only the PySCF-aligned `lda,vwn` functional"):
        xc._functional_id("gga,pbe")
    assert xc._functional_id(" LDA,VWN ")[0] == "lda,vwn"
    with pytest.raises(ValueError, match="rho_up must be a contiguous CUDA field of 8 points"):
        xc.lsda_device(ok, ok)  # host tensors never reach the kernel


def test_hpsi_device_refuses_blocks_the_kernel_would_overrun():
    """``ops.hpsi_device`` hands raw pointers to the stencil kernels, so a block of the wrong
    size, layout or device is refused on the host before any launch."""

    from types import SimpleNamespace

    import torch

    from isogriddft_gb300 import ops

    dg = SimpleNamespace(shape=(3, 4, 5), n=60, monitor=True)
    with pytest.raises(ValueError, match="psi must be a contiguous CUDA block of 2 x 60 points"):
        ops.hpsi_device(dg, torch.zeros((2, 60)))
    with pytest.raises(ValueError, match="psi must be a contiguous CUDA block of 2 x 60 points"):
        ops.hpsi_device(dg, torch.zeros((2, 61)))
    with pytest.raises(ValueError, match="psi must be a contiguous CUDA block of 1 x 60 points"):
        ops.hpsi_device(dg, torch.zeros((4, 5, 3)).transpose(0, 2))


def test_density_drop_ins_check_shapes_as_the_reference(monitor_geom):
    """``scf/driver.py:663-702``: the orbital block and the fields are checked against the grid
    shape with the reference's messages, before anything reaches the device."""

    from isogriddft_gb300 import density

    shape = monitor_geom.spec.shape
    with pytest.raises(ValueError, match=r"orbitals must match the grid shape \(13, 13, 15\); received \(13, 13, 14\)"):
        density.build_density_from_occupied_orbitals(np.zeros((2, 13, 13, 14)), (1.0, 1.0), monitor_geom)
    with pytest.raises(ValueError, match="orbitals must be a 3D orbital or a 4D orbital block"):
        density.build_density_from_occupied_orbitals(np.zeros((2, 13 * 13 * 15)), (1.0, 1.0), monitor_geom)
    with pytest.raises(ValueError, match=r"rho must match the grid shape"):
        density.renormalize_density(np.ones((13, 13, 16)), 2.0, monitor_geom)
    assert np.all(density.renormalize_density(np.ones((1, 2)), 0.0, monitor_geom) == 0.0)  # as the reference
    ok, bad = np.zeros(shape), np.zeros((13, 13, 16))
    with pytest.raises(ValueError, match=r"field must match the grid shape"):
        density.density_residual(bad, bad, bad, bad, monitor_geom)
    assert density.build_density_from_occupied_orbitals(ok, (), monitor_geom).shape == shape


def test_hartree_and_gth_inputs_checked_as_the_reference(monitor_geom):
    """``poisson/hartree.py:32-44, 100-140`` and ``pseudo/nonlocal.py:286-299``: densities,
    potentials and orbitals are checked against the grid (and the units against the case) with
    the reference's messages before any device work."""

    from dataclasses import replace

    from isogriddft_gb300 import poisson, pseudo
    from isogriddft_gb300.config import H2_BENCHMARK_CASE

    shape = monitor_geom.spec.shape
    ok = np.ones(shape)
    with pytest.raises(ValueError, match="rho must be a 3D field; received ndim=1"):
        poisson.validate_density_field(np.ones(10), monitor_geom)
    with pytest.raises(ValueError, match=r"rho must match the grid shape \(13, 13, 15\)"):
        poisson.evaluate_hartree_energy(np.ones((13, 13, 14)), monitor_geom, ok)
    with pytest.raises(ValueError, match="rho must be non-negative up to roundoff"):
        poisson.validate_density_field(-ok, monitor_geom)
    with pytest.raises(ValueError, match=r"hartree_potential must match the grid shape"):
        poisson.evaluate_hartree_energy(ok, monitor_geom, np.ones((13, 13, 14)))
    with pytest.raises(ValueError, match=r"psi must match the grid shape"):
        poisson.build_hartree_action(np.ones((13, 13, 14)), monitor_geom, ok)
    np.testing.assert_array_equal(poisson.build_hartree_action(ok, monitor_geom, 2 * ok), 2 * ok)
    with pytest.raises(ValueError, match=r"rho must match the grid shape"):
        import torch

        poisson.validate_density_field(torch.ones(7), monitor_geom)
    with pytest.raises(ValueError, match=r"psi must match the grid shape"):
        pseudo.evaluate_nonlocal_ionic_action(H2_BENCHMARK_CASE, monitor_geom, np.ones((13, 13, 14)))
    angstrom = replace(H2_BENCHMARK_CASE, geometry=replace(H2_BENCHMARK_CASE.geometry, unit="Angstrom"))
    with pytest.raises(ValueError, match="must use the same unit system; received `Angstrom` and `Bohr`"):
        pseudo.evaluate_nonlocal_ionic_action(angstrom, monitor_geom, ok)
