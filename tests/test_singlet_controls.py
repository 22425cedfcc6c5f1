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
