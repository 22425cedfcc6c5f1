"""The H2 singlet controls of the A-grid dry run against the reference's own functions
(``tests/golden/make_golden_singlet.py`` -> ``singlet_h2.npz``): active-subspace tracking
(``scf/active_subspace.py``), the Hartree-aware singlet mixing weight and baseline update and the
potential-change channel shares (``scf/driver.py:1565-1583``, ``:1825-1937``).  The host algebra
runs on CPU tensors here; on the GPU the same code takes its Grams and sums from the library."""

import json
import os

import numpy as np
import pytest
import torch

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def golden():
    with open(os.path.join(HERE, "singlet_h2.json")) as f:
        meta = json.load(f)
    return np.load(os.path.join(HERE, "singlet_h2.npz")), meta


def test_active_subspace_tracking_matches_the_reference(golden):
    """Occupied orbital (up to sign) to 1e-10, the aligned span, every diagnostic and verdict,
    through the initial step, rotations, sign flips, an order swap, a strong rotation inside the
    span and a step that loses the tracked direction."""

    from isogriddft_gb300.active_subspace import (ActiveSubspaceConfig, initialize_active_subspace,
                                                  update_active_subspace)

    g, meta = golden
    w = torch.as_tensor(g["cell_volumes"].reshape(-1))
    n = w.numel()
    steps = len(meta["verdicts"])
    config = ActiveSubspaceConfig.local_only_h2_singlet_default()
    state = None
    for t in range(steps):
        raw = torch.as_tensor(g[f"raw_{t}"].reshape(2, n))
        sel = (initialize_active_subspace(raw_subspace_orbitals=raw, config=config) if state is None
               else update_active_subspace(raw_subspace_orbitals=raw, state=state, weights=w))
        state = sel.state
        occ, ref_occ = sel.occupied_orbitals.numpy(), g[f"occupied_{t}"].reshape(1, n)
        sign = np.sign(np.sum(occ * ref_occ * w.numpy()))
        np.testing.assert_allclose(sign * occ, ref_occ, rtol=0, atol=1e-10 * np.abs(ref_occ).max(), err_msg=str(t))
        # same span: the aligned bases' cross-overlap is orthogonal
        A, B = sel.aligned_subspace_orbitals.numpy(), g[f"aligned_{t}"].reshape(2, n)
        s = np.linalg.svd((A * w.numpy()) @ B.T, compute_uv=False)
        np.testing.assert_allclose(s, 1.0, atol=1e-10, err_msg=str(t))
        want = g[f"diag_{t}"]
        got = [sel.raw_occupied_overlap_abs, sel.best_in_subspace_occupied_overlap_abs,
               sel.internal_rotation_angle_deg, sel.projector_drift_frobenius_norm,
               sel.subspace_rotation_max_angle_deg, *sel.subspace_overlap_singular_values]
        np.testing.assert_allclose(got[:2], want[:2], atol=1e-10, err_msg=str(t))
        np.testing.assert_allclose([got[2], got[4]], [want[2], want[4]], atol=1e-5, err_msg=str(t))  # degrees
        np.testing.assert_allclose(got[3], want[3], atol=1e-6, err_msg=str(t))
        np.testing.assert_allclose(got[5:], want[5:], atol=1e-10, err_msg=str(t))
        assert sel.verdict == meta["verdicts"][t]
    assert len(set(meta["verdicts"])) == 4  # initial + the three update verdicts


def test_active_subspace_config_checks():
    from isogriddft_gb300.active_subspace import ActiveSubspaceConfig, initialize_active_subspace

    raw = torch.ones((2, 5), dtype=torch.float64)
    for cfg, msg in ((ActiveSubspaceConfig(True, 0, 1), "subspace_size must be positive"),
                     (ActiveSubspaceConfig(True, 2, 0), "target_occupied_count must be positive"),
                     (ActiveSubspaceConfig(True, 2, 3), "target_occupied_count must not exceed subspace_size"),
                     (ActiveSubspaceConfig(True, 3, 1), "At least 3 orbitals are required; received 2")):
        with pytest.raises(ValueError, match=msg):
            initialize_active_subspace(raw_subspace_orbitals=raw, config=cfg)


def test_singlet_mixing_matches_the_reference(golden):
    from isogriddft_gb300 import mixing
    from isogriddft_gb300.scf import resolve_h2_spin_occupations

    g, meta = golden
    for (m, h, r), want in zip(meta["mix_cases"], g["mix_factor"]):
        h = float(h) if isinstance(h, str) else h
        assert mixing.closed_shell_singlet_mixing_factor(m, h, r) == pytest.approx(want, abs=1e-15)
    w = torch.as_tensor(g["cell_volumes"].reshape(-1))

    def renormalized(rho, target):  # driver.py:679-690
        if target == 0.0:
            return torch.zeros_like(rho)
        return rho * (float(target) / float(torch.sum(rho * w)))

    for label in ("singlet", "triplet"):
        occ = resolve_h2_spin_occupations(label)
        up, dn, uo, do, want_up, want_dn = (torch.as_tensor(a.reshape(-1)) for a in g[f"mix_{label}"])
        got_up, got_dn, _ = mixing.closed_shell_singlet_baseline_mix(renormalized, occ, up, dn, uo, do, 0.35, 0.72,
                                                                     0.97)
        np.testing.assert_allclose(got_up.numpy(), want_up.numpy(), rtol=1e-12, atol=1e-14)
        np.testing.assert_allclose(got_dn.numpy(), want_dn.numpy(), rtol=1e-12, atol=1e-14)
    p = [torch.as_tensor(a.reshape(-1)) for a in g["share_in"]]
    shares = mixing.singlet_hartree_tail_channel_shares(p[3] - p[0], p[4] - p[1], p[5] - p[2], w)
    np.testing.assert_allclose(shares, g["shares"], rtol=1e-12)
    assert mixing.weighted_field_norm(p[0], w) == pytest.approx(float(g["field_norm"][0]), rel=1e-13)
    zero = torch.zeros_like(p[0])
    assert mixing.singlet_hartree_tail_channel_shares(zero, zero, zero, w) == (None, None, None)


def test_previous_density_residual_ratio():
    from types import SimpleNamespace

    from isogriddft_gb300.mixing import previous_density_residual_ratio

    assert previous_density_residual_ratio([], 1.0) is None
    assert previous_density_residual_ratio([SimpleNamespace(density_residual=0.0)], 1.0) is None
    assert previous_density_residual_ratio([SimpleNamespace(density_residual=0.5)], 0.25) == 0.5


class _FakeEngine:
    """CPU stand-in for the device SCF engine: a rotating lowest pair of orbitals, a smoothing
    'Hartree' map and a cube-root 'XC' potential.  Only the loop's glue is under test."""

    def __init__(self, n, w, occ):
        from types import SimpleNamespace

        self.dg = SimpleNamespace(cell_volumes=w, n=n, device=torch.device("cpu"))
        self.occ, self.vloc, self.patch, self.prec = occ, -torch.linspace(1.0, 2.0, n, dtype=torch.float64), None, "fp64"
        self.poisson_iterations, self.eigensolver_iterations, self.poisson_history = 0, [], []
        g = torch.Generator().manual_seed(5)
        basis = torch.randn((3, n), generator=g, dtype=torch.float64)
        q, _ = torch.linalg.qr((basis * w.sqrt()).T)
        self.phi = (q.T / w.sqrt()).contiguous()
        self.calls = 0

    def wdot(self, a, b=None):
        return torch.sum(a * (a if b is None else b) * self.dg.cell_volumes).reshape(1)

    def renormalized(self, rho, target):
        return torch.zeros_like(rho) if target == 0.0 else rho * (float(target) / float(self.wdot(rho, torch.ones_like(rho))))

    def density(self, orbitals, occupations, target):
        rho = torch.zeros(self.dg.n, dtype=torch.float64)
        for i, o in enumerate(occupations):
            rho = rho + o * orbitals[i] ** 2
        return self.renormalized(rho, target)

    def hartree(self, rho):
        from types import SimpleNamespace

        self.poisson_iterations += 3
        self.poisson_history.append(3)
        return SimpleNamespace(potential=0.5 * rho + 0.1 * rho.roll(1))

    def xc(self, up, dn):
        return {"v_up": -(up.clamp_min(0) ** (1 / 3)), "v_down": -(dn.clamp_min(0) ** (1 / 3)),
                "energy": torch.zeros(1, dtype=torch.float64)}

    def eigensolve(self, veff, k, guess, **kw):
        self.calls += 1
        th = 0.3 * self.calls
        a = np.cos(th) * self.phi[0] + np.sin(th) * self.phi[1]
        b = -np.sin(th) * self.phi[0] + np.cos(th) * self.phi[1]
        orbs = torch.stack([a, b, self.phi[2]])[:max(k, 2)]
        self.eigensolver_iterations.append(4)
        m = orbs.shape[0]
        return {"orbitals": orbs, "eigenvalues": np.array([-0.6, -0.2, 0.1])[:m], "converged": True,
                "residual_norms": np.zeros(m), "iteration_count": 4, "residual_history": np.zeros((4, m)),
                "ritz_value_history": np.zeros((4, m)), "subspace_dimensions": (m,) * 4, "weighted_overlap": np.eye(m),
                "max_orthogonality_error": 0.0, "ritz_matrix": np.eye(m), "initial_guess": orbs, "final_basis": orbs}

    def energy(self, up, dn, orb_up, orb_dn, *, local_only=False, hartree=None, lsda=None):
        from isogriddft_gb300.scf import SinglePointEnergyComponents

        h, x = self.hartree(up + dn), self.xc(up, dn)
        t = float(self.wdot(up + dn, up + dn))
        return SinglePointEnergyComponents(t, 0.0, 0.0, 0.0, 0.0, 0.0, t), h, x


@pytest.mark.parametrize("spin,cycle_breaker", [("singlet", None), ("triplet", None), ("singlet", 0.5)])
def test_singlet_controls_in_the_scf_loop(monkeypatch, spin, cycle_breaker):
    """The device SCF loop with ``singlet_controls`` on, driven by a CPU stand-in engine: the
    singlet solves two orbitals, tracks one (diagnostics per step, no gap on the first), and its
    mixed spin densities are the even split of the Hartree-aware total mix; the triplet keeps
    the per-spin linear mix."""

    from types import SimpleNamespace

    from isogriddft_gb300 import scf
    from isogriddft_gb300.config import H2_BENCHMARK_CASE

    shape = (4, 5, 6)
    n = int(np.prod(shape))
    w = torch.linspace(0.5, 1.5, n, dtype=torch.float64)
    occ = scf.resolve_h2_spin_occupations(spin)
    fake = _FakeEngine(n, w, occ)
    monkeypatch.setattr(scf, "DeviceScfEngine", lambda *a, **k: fake)
    monkeypatch.setattr(scf, "h2_trial_orbitals_device", lambda case, geom: fake.phi[:2].clone())
    monkeypatch.setattr(scf, "residual_device", lambda dg, a, b, c, d: float(
        torch.sqrt(torch.sum(((c - a) ** 2 + (d - b) ** 2) * dg.cell_volumes))))
    monkeypatch.setattr(torch.cuda, "current_stream", lambda *a, **k: SimpleNamespace(synchronize=lambda: None))
    geom = SimpleNamespace(spec=SimpleNamespace(shape=shape))
    diag: dict = {}
    res = scf._run_scf_device(H2_BENCHMARK_CASE, geom, spin, max_iterations=3, mixing=0.35, density_tolerance=1e-12,
                              energy_tolerance=1e-12, diagnostics=diag, singlet_controls=True, include_nonlocal=False,
                              cycle_breaker_weight=cycle_breaker)
    assert isinstance(diag["cycle_breaker_triggered"], list)
    if cycle_breaker is not None:
        assert all(it >= 3 for it in diag["cycle_breaker_triggered"])  # needs two earlier steps
        return
    assert res.iteration_count == 3 or spin == "triplet"  # the triplet's density is span-invariant: one step
    # the last step's eigensolver results, the singlet's down channel being its up solve
    assert res.solve_up.orbitals.shape == (2,) + shape and res.solve_up.eigenvalues[0] == -0.6
    assert (res.solve_down is res.solve_up) == (spin == "singlet")
    for rec in res.history:
        lin = [fake.renormalized((1 - 0.35) * torch.as_tensor(a).reshape(-1) + 0.35 * torch.as_tensor(b).reshape(-1), t)
               for a, b, t in ((rec.input_rho_up, rec.output_rho_up, occ.n_alpha),
                               (rec.input_rho_down, rec.output_rho_down, occ.n_beta))]
        if spin == "singlet":
            np.testing.assert_array_equal(rec.mixed_rho_up, rec.mixed_rho_down)
            assert not np.allclose(rec.mixed_rho_up.reshape(-1), lin[0].numpy())
        else:
            np.testing.assert_allclose(rec.mixed_rho_up.reshape(-1), lin[0].numpy(), rtol=1e-14)
    if spin == "singlet":
        cfg, steps = diag["active_subspace"]
        assert cfg.subspace_size == 2 and [s.iteration for s in steps] == [1, 2, 3]
        assert steps[0].lowest_gap_ha is None and steps[1].lowest_gap_ha == pytest.approx(0.4)
        assert res.orbitals_up.shape == (1,) + shape and np.array_equal(res.orbitals_up, res.orbitals_down)
        # the tracked orbital stays on the first step's lowest orbital while the raw pair rotates
        tracked = torch.as_tensor(res.orbitals_up.reshape(1, -1))
        first = np.cos(0.3) * fake.phi[0] + np.sin(0.3) * fake.phi[1]
        assert abs(float(torch.sum(tracked[0] * first * w))) == pytest.approx(1.0, abs=1e-12)
    else:
        assert "active_subspace" not in diag


def test_cycle_breaker_alternation_test_matches_the_reference(golden):
    """``driver.py:1177-1206`` on seeded outputs: a sign flip of the energy change with the new
    output closer to the one two steps back triggers; same-sign changes, a short history, a
    missing change or an output that does not return do not."""

    from isogriddft_gb300.mixing import cycle_breaker_mix, detect_singlet_alternation
    from isogriddft_gb300.scf import resolve_h2_spin_occupations

    g, meta = golden
    w = torch.as_tensor(g["cell_volumes"].reshape(-1))
    outs = [[torch.as_tensor(s.reshape(-1)) for s in o] for o in g["cb_outputs"]]

    def dist(a, b, c, d):
        return float(torch.sqrt(torch.sum(((c - a) ** 2 + (d - b) ** 2) * w)))

    got = [detect_singlet_alternation([(outs[i][0], outs[i][1], c) for i, c in hist], outs[k][0], outs[k][1], c, dist)
           for hist, k, c in meta["cb_cases"]]
    assert got == meta["cb_detect"] and any(got) and not all(got)
    occ = resolve_h2_spin_occupations("singlet")

    def renormalized(rho, target):
        return rho * (float(target) / float(torch.sum(rho * w)))

    up, dn = cycle_breaker_mix(renormalized, occ, outs[0][0], outs[0][1], outs[1][0], outs[1][1], 0.5)
    want = renormalized(0.5 * outs[0][0] + 0.5 * outs[1][0], 1)
    np.testing.assert_allclose(up.numpy(), want.numpy(), rtol=1e-14)
    assert float(torch.sum(dn * w)) == pytest.approx(1.0, rel=1e-14)
