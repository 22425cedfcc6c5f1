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
