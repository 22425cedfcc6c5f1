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
