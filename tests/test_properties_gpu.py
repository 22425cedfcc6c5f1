"""Property tests in the style of the reference's own suite, run on the GPU path:
a constant field has zero interior kinetic action and the operators keep the mirror symmetry
of a symmetric molecule (tests/test_local_hamiltonian.py:59-77), the Hartree energy of a positive
density is positive and its multipole charge is the electron count (tests/test_hartree_poisson.py:
172-306), and device-built monitor grids for N2, CO and H2O have a positive Jacobian with finer
spacing near the nuclei (tests/test_monitor_grid.py)."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _h2_agrid(shape=(19, 19, 23), device=False):
    from isogriddft_gb300.config import H2_BENCHMARK_CASE
    from isogriddft_gb300.grid import build_monitor_grid_for_case, build_two_peak_element_parameters

    return build_monitor_grid_for_case(H2_BENCHMARK_CASE, shape=shape, box_half_extents=(6.0, 6.0, 8.0),
                                       element_parameters=build_two_peak_element_parameters(("H",), 4.0, 0.5),
                                       device=device)


@pytest.mark.parametrize("dtype", ["float64", "float32"])
@pytest.mark.parametrize("closure", ["trial_fix", "production"])
def test_constant_field_has_zero_interior_kinetic_action(closure, dtype):
    """Every difference of a constant field is exactly zero, so the action is exactly zero two
    points in from the faces (the trial fix's zero ghost acts at the faces) and everywhere for the
    production closure (its one-sided ghost 3 f0 - 3 f1 + f2 reproduces the constant)."""

    import torch

    from isogriddft_gb300 import device, ops

    geom = _h2_agrid()
    shape = geom.spec.shape
    dg = device.device_grid(geom)
    one = torch.ones((2, dg.n), dtype=getattr(torch, dtype), device="cuda")
    t = ops.hpsi_device(dg, one, closure=closure, kscale=-0.5).double().cpu().numpy().reshape((2,) + shape)
    assert np.all(t[:, 2:-2, 2:-2, 2:-2] == 0.0)
    if closure == "production":
        assert np.all(t == 0.0)
    else:
        assert np.any(t != 0.0)  # the zero ghost does act at the faces


def test_constant_field_legacy_kinetic():
    """Legacy separable operator: zero action at every point not next to a face."""

    import torch

    from isogriddft_gb300 import device, ops
    from isogriddft_gb300.config import H2_BENCHMARK_CASE
    from isogriddft_gb300.grid import build_default_h2_grid_spec, build_grid_geometry
    from dataclasses import replace

    geom = build_grid_geometry(replace(build_default_h2_grid_spec(H2_BENCHMARK_CASE), nx=15, ny=17, nz=19))
    dg = device.device_grid(geom)
    one = torch.ones((1, dg.n), dtype=torch.float64, device="cuda")
    t = ops.hpsi_device(dg, one, kscale=-0.5).cpu().numpy().reshape(geom.spec.shape)
    assert np.all(t[1:-1, 1:-1, 1:-1] == 0.0)


@pytest.mark.parametrize("closure", ["trial_fix", "production"])
def test_mirror_symmetry_of_the_kinetic_action(closure):
    """H2 lies on the z axis in a box symmetric about the origin, so its A-grid is mirror
    symmetric in x, y and z: mirroring psi mirrors T psi (to the rounding of the grid
    construction)."""

    import torch

    from isogriddft_gb300 import device, ops

    geom = _h2_agrid()
    shape = geom.spec.shape
    dg = device.device_grid(geom)
    psi = np.random.default_rng(3).normal(size=shape)
    t = lambda f: ops.hpsi_device(dg, torch.as_tensor(f.reshape(1, -1).copy(), device="cuda"),  # noqa: E731
                                  closure=closure, kscale=-0.5).cpu().numpy().reshape(shape)
    base = t(psi)
    scale = np.max(np.abs(base))
    for axis in range(3):
        mirrored = t(np.flip(psi, axis=axis))
        assert np.max(np.abs(mirrored - np.flip(base, axis=axis))) < 1e-10 * scale, axis


def test_hartree_energy_positive_and_charge_recovered():
    """A positive density gives E_H > 0 (the device reduction equal to the plain sum), a positive
    potential at its centre, and a multipole boundary whose charge is the electron count (within
    5e-2, as the reference's check)."""

    from isogriddft_gb300 import poisson

    geom = _h2_agrid(device=True)
    r2 = geom.x_points**2 + geom.y_points**2 + (geom.z_points - 0.2) ** 2
    rho = np.exp(-r2 / (2 * 0.9**2))
    rho *= 2.0 / np.sum(rho * geom.cell_volumes)
    res = poisson.solve_hartree_potential(geom, rho)
    eh = poisson.evaluate_hartree_energy(rho, geom, res)
    assert eh > 0.0 and eh == pytest.approx(0.5 * float(np.sum(rho * res.potential * geom.cell_volumes)), rel=1e-12)
    centre = tuple(n // 2 for n in geom.spec.shape)
    assert res.potential[centre] > 0.0
    assert abs(res.boundary_condition.total_charge - 2.0) < 5e-2


@pytest.mark.parametrize("name", ["N2", "CO", "H2O"])
def test_device_monitor_grids_refine_near_nuclei(name):
    """Device-built 21^3 monitor grids: positive Jacobian everywhere, mean spacing within 1 Bohr
    of a nucleus finer than beyond 3 Bohr, and the host builder's grid to 1e-10."""

    from isogriddft_gb300.config import make_molecule_case
    from isogriddft_gb300.grid import build_monitor_grid_for_case, build_two_peak_element_parameters

    atoms = {"N2": [("N", (0.0, 0.0, -1.037)), ("N", (0.0, 0.0, 1.037))],
             "CO": [("C", (0.0, 0.0, -1.066)), ("O", (0.0, 0.0, 1.066))],
             "H2O": [("O", (0.0, 0.0, 0.0)), ("H", (0.0, 1.43, 1.11)), ("H", (0.0, -1.43, 1.11))]}[name]
    case = make_molecule_case(name, atoms)
    params = build_two_peak_element_parameters(tuple(sorted({a for a, _ in atoms})), 4.0, 0.5)
    kw = dict(shape=(21, 21, 21), box_half_extents=(6.0, 6.0, 6.0), element_parameters=params)
    g = build_monitor_grid_for_case(case, device=True, **kw)
    h = build_monitor_grid_for_case(case, device=False, **kw)
    assert np.all(g.jacobian > 0.0)
    sp = np.asarray(g.spacing_measure)
    X = np.stack([g.x_points, g.y_points, g.z_points], -1)
    pos = np.array([p for _, p in atoms])
    d = np.min(np.linalg.norm(X[..., None, :] - pos[None, None, None], axis=-1), axis=-1)
    assert sp[d < 1.0].mean() < sp[d > 3.0].mean()
    np.testing.assert_allclose(X, np.stack([h.x_points, h.y_points, h.z_points], -1), rtol=0, atol=1e-10 * 6.0)
