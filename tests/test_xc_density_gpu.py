"""GPU parity of LSDA (Slater + VWN5 / PW92) and the density helpers."""

import numpy as np
import pytest

from tests.conftest import gpu_available

import oracle.scf as OS
import oracle.xc as OX

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not gpu_available():
        pytest.skip("needs a CUDA GPU")


@pytest.mark.parametrize("functional", ["lda,vwn", "lda,pw92"])
def test_lsda_fp64_matches_oracle(functional):
    from isogriddft_gb300 import xc

    rng = np.random.default_rng(3)
    shape = (9, 10, 11)
    up = rng.uniform(0.0, 2.0, shape) ** 3
    dn = rng.uniform(0.0, 2.0, shape) ** 3
    up[0, 0, :4] = 0.0  # fully polarised and empty points
    dn[0, 1, :4] = 0.0
    up[0, 2, :2] = dn[0, 2, :2] = 0.0
    up[1, 0, 0] = -5e-15  # roundoff negatives are clipped
    got = xc.evaluate_lsda_terms(up, dn, functional)
    ref = OX.lsda(up, dn, functional)
    for key in ("eps_xc", "v_xc_up", "v_xc_down", "energy_density"):
        np.testing.assert_allclose(getattr(got, key), ref[key], rtol=1e-12, atol=1e-13, err_msg=key)
    f32 = xc.evaluate_lsda_terms(up, dn, functional, precision="fp32")
    np.testing.assert_allclose(f32.v_xc_up, ref["v_xc_up"], rtol=3e-5, atol=1e-6)


def test_lsda_energy_recorded_legacy_value():
    """Recorded legacy 51^3 E_xc (audit/baselines.py:822) through the GPU kernel."""

    from isogriddft_gb300 import xc
    from isogriddft_gb300.config import H2_BENCHMARK_CASE
    from isogriddft_gb300.grid import build_default_h2_grid_geometry

    geom = build_default_h2_grid_geometry()
    psi = OS.bonding_trial_orbital(H2_BENCHMARK_CASE, geom)
    e = xc.evaluate_lsda_energy(psi * psi, psi * psi, geom)
    assert abs(e + 0.869107874980) < 1e-11
    e32 = xc.evaluate_lsda_energy(psi * psi, psi * psi, geom, precision="fp32")
    assert abs(e32 + 0.869107874980) < 1e-6


def test_lsda_rejects_bad_density():
    from isogriddft_gb300 import xc

    a = np.ones((4, 4, 4))
    b = a.copy()
    b[1, 1, 1] = -1.0
    with pytest.raises(ValueError):
        xc.evaluate_lsda_terms(a, b)
    b[1, 1, 1] = np.inf
    with pytest.raises(ValueError):
        xc.evaluate_lsda_terms(a, b)
    with pytest.raises(ValueError):
        xc.evaluate_lsda_terms(a, a, "gga,pbe")


def test_density_helpers_match_reference(golden_monitor, monitor_geom):
    from isogriddft_gb300 import density

    g = golden_monitor
    d = density.build_density_from_occupied_orbitals(g["eig_orbitals"], (1.0, 1.0), monitor_geom)
    np.testing.assert_allclose(d, g["density"], rtol=1e-13, atol=1e-300)
    r = density.renormalize_density(d, 2.0, monitor_geom)
    np.testing.assert_allclose(r, g["density_renorm"], rtol=1e-12)
    res = density.density_residual(g["rho"] / 2, g["rho"] / 2, r / 2, r / 2, monitor_geom)
    assert abs(res - float(g["density_residual"])) < 1e-12
    with pytest.raises(ValueError):
        density.renormalize_density(np.zeros(monitor_geom.spec.shape), 2.0, monitor_geom)


@pytest.mark.parametrize("n,nb,stride_pad", [(4096, 1, 0), (2_097_152, 16, 0), (10_000, 5, 4), (8192, 64, 0),
                                             (8192, 65, 0), (10_001, 3, 0)])
def test_fp32_density_matches_fp64(n, nb, stride_pad):
    """``igd_density`` on FP32 orbitals (the 16-byte kernel when n, the orbital stride and the
    pointers allow and nb <= 64, the scalar kernel otherwise): rho = sum occ psi^2 in FP32
    sums, stored in FP64, accumulated on request, and its weighted integral, against FP64
    NumPy to FP32 rounding (4e-6 relative: up to 65 positive FP32 terms per point)."""

    import torch

    from isogriddft_gb300 import _lib
    from isogriddft_gb300.device import ptr, stream_ptr

    g = torch.Generator(device="cuda").manual_seed(n + nb)
    stride = n + stride_pad
    psi = torch.randn((nb, stride), device="cuda", generator=g)
    occ = torch.rand(nb, device="cuda", dtype=torch.float64, generator=g) + 0.5
    w = torch.rand(n, device="cuda", dtype=torch.float64, generator=g) + 0.5
    rho0 = torch.rand(n, device="cuda", dtype=torch.float64, generator=g)
    P = psi[:, :n].double().cpu().numpy()
    ref = (occ.cpu().numpy()[:, None] * P * P).sum(axis=0)
    for acc in (0, 1):
        rho = rho0.clone()
        integral = torch.empty(1, dtype=torch.float64, device="cuda")
        _lib.check(_lib.call("igd_density", _lib.IGD_F32, n, nb, stride, ptr(psi), ptr(occ), ptr(w), ptr(rho),
                             ptr(integral), acc, stream_ptr()), "igd_density")
        want = ref + (rho0.cpu().numpy() if acc else 0.0)
        got = rho.cpu().numpy()
        assert np.max(np.abs(got - want)) <= 4e-6 * np.max(np.abs(want))
        wi = float(np.sum(want * w.cpu().numpy()))
        assert abs(float(integral.item()) - wi) <= 4e-6 * abs(wi)
