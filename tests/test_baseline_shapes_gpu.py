"""Parity at the benchmark shapes.

* The bench's own workload: the 128^3 two-peak A-grid H.Psi (trial-fix closure,
  v_eff present) on the whole-row kernel, FP32 and FP64, against the FP64 oracle
  on a few of the bench's orbitals.
* Rows longer than 128 points (nz = 160 and 192, the shapes of the C6H6 and
  H2O/CH4 configurations), which the whole-row kernel does not take: the tiled
  and cp.async kernels on small nx x ny, both closures.
* The 128^3 mixed-precision Poisson solve of the sigma = 0.8 Bohr Gaussian
  against the FP64 solve of the same discrete problem (potential, E_H, the
  far-field boundary values) and against the analytic free-space E_H.
"""

import numpy as np
import pytest

from tests.conftest import gpu_available

import oracle.kinetic as OK

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not gpu_available():
        pytest.skip("needs a CUDA GPU")


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.fixture(scope="module")
def bench_geom():
    from isogriddft_gb300.config import H2_BENCHMARK_CASE
    from isogriddft_gb300.grid import build_monitor_grid_for_case, build_two_peak_element_parameters

    return build_monitor_grid_for_case(H2_BENCHMARK_CASE, shape=(128, 128, 128), box_half_extents=(8.0, 8.0, 10.0),
                                       element_parameters=build_two_peak_element_parameters(("H",), 4.0, 0.5),
                                       device=True)


def test_bench_workload_hpsi_matches_oracle(bench_geom):
    """Two orbitals of the bench's 16 (its own seeded inputs) through the FP32 and FP64
    kernels the bench times, against the FP64 oracle: FP32 2e-5, FP64 1e-12."""

    import torch

    from isogriddft_gb300 import _lib, device, ops
    from isogriddft_gb300.config import H2_BENCHMARK_CASE

    geom = bench_geom
    shape = geom.spec.shape
    rng = np.random.default_rng(0)
    psi = rng.standard_normal((16,) + shape).astype(np.float32)[[0, 9]]
    veff = np.zeros(shape)
    for atom in H2_BENCHMARK_CASE.geometry.atoms:
        d2 = ((geom.x_points - atom.position[0]) ** 2 + (geom.y_points - atom.position[1]) ** 2
              + (geom.z_points - atom.position[2]) ** 2)
        veff += -2.0 / np.sqrt(d2 + 0.1)
    ref = OK.hpsi_block(psi.astype(np.float64), geom, veff, "trial_fix")
    dg = device.device_grid(geom)
    for dtype, tol in ((torch.float32, 2e-5), (torch.float64, 1e-12)):
        t = torch.as_tensor(psi, device="cuda").to(dtype)
        v = torch.as_tensor(veff, device="cuda", dtype=dtype)
        got = ops.hpsi_device(dg, t, closure="trial_fix", kscale=-0.5, veff=v).double().cpu().numpy()
        assert _rel(got, ref) < tol, (dtype, _rel(got, ref))
    assert _lib.error_flags(clear=True, stream=device.stream_ptr()) == 0


@pytest.mark.parametrize("shape", [(12, 14, 160), (10, 23, 192), (7, 9, 188)])
@pytest.mark.parametrize("closure", ["trial_fix", "production"])
def test_long_rows_match_oracle(shape, closure):
    """Rows of 160 and 192 points (and a ragged 188) on every FP32 kernel that takes them
    (the whole-row kernel's two-chunk form for one orbital, the tiled kernel, the cp.async
    kernel), and FP64, against the oracle (FP32 2e-5, FP64 1e-12); four orbitals, a partial
    group of three and one."""

    import torch

    from isogriddft_gb300 import _lib, device, ops
    from isogriddft_gb300.config import H2_BENCHMARK_CASE
    from isogriddft_gb300.grid import assemble_monitor_geometry, build_monitor_grid_spec_for_case, monitor_box_axes

    spec = build_monitor_grid_spec_for_case(H2_BENCHMARK_CASE, shape=shape, box_half_extents=(5.0, 6.0, 9.0))
    lx, ly, lz, box = monitor_box_axes(spec)
    X = box.copy()
    X[..., 0] += 0.25 * np.sin(box[..., 2] * 0.45) * np.exp(-np.sum(box**2, axis=-1) / 25)
    X[..., 2] += 0.3 * np.sin(box[..., 1] * 0.4) * np.exp(-np.sum(box**2, axis=-1) / 30)
    geom = assemble_monitor_geometry(H2_BENCHMARK_CASE, spec, lx, ly, lz, X)
    rng = np.random.default_rng(sum(shape))
    psi = rng.normal(size=(4,) + shape)
    veff = rng.normal(size=shape)
    ref = OK.hpsi_block(psi, geom, veff, closure)
    dg = device.device_grid(geom)
    try:
        for path in (0, 1, 2):
            _lib.check(_lib.call("igd_hpsi_select", path), "igd_hpsi_select")
            for nb in (4, 3, 1):
                for dtype, tol in ((torch.float32, 2e-5), (torch.float64, 1e-12)):
                    got = ops.hpsi_device(dg, torch.as_tensor(psi[:nb], device="cuda", dtype=dtype),
                                          closure=closure, kscale=-0.5,
                                          veff=torch.as_tensor(veff, device="cuda", dtype=dtype))
                    err = _rel(got.double().cpu().numpy(), ref[:nb])
                    assert err < tol, (path, nb, dtype, err)
    finally:
        _lib.call("igd_hpsi_select", 0)
    assert _lib.error_flags(clear=True, stream=device.stream_ptr()) == 0


def test_bench_poisson_mixed_matches_fp64(bench_geom):
    """The bench's Poisson problem (sigma = 0.8 Bohr Gaussian of 2 electrons on the 128^3
    two-peak grid): the mixed solve (FP32 inside FP64 refinement) against the FP64 solve of
    the same discrete problem to 5e-9 (both stop at 1e-10 relative residual, each with its
    own Krylov path; measured 1.0e-9 of max |v_H|, E_H to 1e-10), identical
    multipole boundary values, and E_H = 1/2 <rho, v_H> within 5e-3 of the analytic
    free-space value Q^2 / (2 sigma sqrt(pi)): the discretisation error of this grid and
    its l <= 2 multipole boundary, measured 2.4e-3 (1.41380 against 1.41047 Ha)."""

    import torch

    from isogriddft_gb300.device import device_grid
    from isogriddft_gb300.poisson import solve_poisson_device

    dg = device_grid(bench_geom)
    sigma, q = 0.8, 2.0
    r2 = dg.x * dg.x + dg.y * dg.y + dg.z * dg.z
    rho = torch.exp(-0.5 * r2 / sigma**2)
    rho *= q / float(torch.sum(rho * dg.cell_volumes))
    sols = {p: solve_poisson_device(dg, bench_geom, rho, tolerance=1e-10, max_iterations=4000, precision=p)
            for p in ("fp64", "mixed")}
    for s in sols.values():
        assert s.relative_residual <= 1e-10
    v64, vmx = (sols[p].potential.double().cpu().numpy() for p in ("fp64", "mixed"))
    assert _rel(vmx, v64) < 5e-9
    w = dg.cell_volumes.cpu().numpy()
    rh = rho.cpu().numpy()
    e64, emx = (0.5 * float(np.sum(rh * v * w)) for v in (v64, vmx))
    assert abs(emx - e64) < 5e-9 * abs(e64)
    exact = q * q / (2.0 * sigma * np.sqrt(np.pi))
    assert abs(e64 - exact) < 5e-3 * exact, (e64, exact)
    # far field: the boundary values are the multipole expansion, the same for both solves
    nx, ny, nz = dg.shape
    face = np.zeros((nx, ny, nz), dtype=bool)
    face[[0, -1], :, :] = face[:, [0, -1], :] = face[:, :, [0, -1]] = True
    fv64, fvmx = v64.reshape(nx, ny, nz)[face], vmx.reshape(nx, ny, nz)[face]
    assert _rel(fvmx, fv64) < 1e-12
