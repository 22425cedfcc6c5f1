"""GPU parity of the fused H.Psi stencils against the oracle and reference fixtures."""

import numpy as np
import pytest

from tests.conftest import gpu_available

import oracle.kinetic as OK

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not gpu_available():
        pytest.skip("needs a CUDA GPU")


def test_monitor_kinetic_matches_reference_fixture(golden_monitor, monitor_geom):
    from isogriddft_gb300 import ops

    g = golden_monitor
    assert _rel(ops.apply_monitor_grid_kinetic_operator(g["psi"], monitor_geom), g["kin_prod_psi"]) < 1e-12
    assert _rel(ops.apply_monitor_grid_kinetic_operator_trial_boundary_fix(g["psi"], monitor_geom), g["kin_trial_psi"]) < 1e-12
    for i in range(3):
        assert _rel(ops.apply_monitor_grid_kinetic_operator(g["rnd"][i], monitor_geom), g["kin_prod_rnd"][i]) < 1e-12
        assert _rel(ops.apply_monitor_grid_kinetic_operator_trial_boundary_fix(g["rnd"][i], monitor_geom),
                    g["kin_trial_rnd"][i]) < 1e-12
    assert _rel(ops.apply_monitor_grid_laplacian_operator(g["rnd"][0], monitor_geom), g["lap_prod_rnd0"]) < 1e-12


def test_legacy_kinetic_matches_reference_fixture(golden_legacy, legacy_geom):
    from isogriddft_gb300 import ops

    g = golden_legacy
    assert _rel(ops.apply_legacy_kinetic_operator(g["rnd"], legacy_geom), g["kin_rnd"]) < 1e-12
    assert _rel(ops.apply_kinetic_operator(g["psi"], legacy_geom), g["kin_psi"]) < 1e-12


@pytest.mark.parametrize("shape", [(9, 10, 11), (21, 19, 40), (33, 17, 67), (40, 9, 33), (12, 35, 97),
                                   (15, 31, 32), (37, 14, 96), (9, 40, 8), (6, 16, 36)])
@pytest.mark.parametrize("closure", ["trial_fix", "production"])
def test_monitor_block_shapes_fp64_fp32(shape, closure):
    """Ragged tiles, tiles larger than the grid, chunked marches, several orbitals."""

    import torch

    from isogriddft_gb300 import device, ops
    from isogriddft_gb300.config import H2_BENCHMARK_CASE
    from isogriddft_gb300.grid import build_monitor_grid_spec_for_case, monitor_box_axes, assemble_monitor_geometry

    spec = build_monitor_grid_spec_for_case(H2_BENCHMARK_CASE, shape=shape, box_half_extents=(6.0, 7.0, 8.0))
    lx, ly, lz, box = monitor_box_axes(spec)
    # smooth non-trivial mapping: box coordinates plus a bump (no harmonic solve, fast)
    X = box.copy()
    r2 = np.sum(box**2, axis=-1)
    X[..., 0] += 0.3 * np.sin(box[..., 1] * 0.4) * np.exp(-r2 / 30)
    X[..., 2] += 0.4 * np.sin(box[..., 0] * 0.3) * np.exp(-r2 / 40)
    geom = assemble_monitor_geometry(H2_BENCHMARK_CASE, spec, lx, ly, lz, X)
    rng = np.random.default_rng(1)
    nb = 5
    psi = rng.normal(size=(nb,) + shape)
    veff = rng.normal(size=shape)
    ref = OK.hpsi_block(psi, geom, veff, closure)
    dg = device.device_grid(geom)
    for dtype, tol in ((torch.float64, 1e-12), (torch.float32, 2e-5)):
        t = torch.as_tensor(psi, device="cuda", dtype=dtype)
        v = torch.as_tensor(veff, device="cuda", dtype=dtype)
        got = ops.hpsi_device(dg, t, closure=closure, kscale=-0.5, veff=v).double().cpu().numpy()
        assert _rel(got, ref) < tol, (dtype, closure, shape, _rel(got, ref))
    from isogriddft_gb300 import _lib

    assert _lib.error_flags(clear=True, stream=device.stream_ptr()) == 0


@pytest.mark.parametrize("nb", [1, 2, 3, 8, 12, 16])
@pytest.mark.parametrize("shape", [(15, 31, 32), (21, 19, 40), (5, 7, 12), (64, 20, 64), (3, 9, 8)])
@pytest.mark.parametrize("closure", ["trial_fix", "production"])
def test_monitor_small_blocks(shape, nb, closure):
    """Orbital counts that select every kernel variant (1, 2, 4, 8 orbitals per CTA, full and
    partial last group), x-chunked marches (64 planes) and the shortest march (3 planes)."""

    import torch

    from isogriddft_gb300 import _lib, device, ops
    from isogriddft_gb300.config import H2_BENCHMARK_CASE
    from isogriddft_gb300.grid import build_monitor_grid_spec_for_case, monitor_box_axes, assemble_monitor_geometry

    spec = build_monitor_grid_spec_for_case(H2_BENCHMARK_CASE, shape=shape, box_half_extents=(5.0, 6.0, 7.0))
    lx, ly, lz, box = monitor_box_axes(spec)
    X = box.copy()
    X[..., 1] += 0.2 * np.sin(box[..., 2] * 0.5) * np.exp(-np.sum(box**2, axis=-1) / 20)
    geom = assemble_monitor_geometry(H2_BENCHMARK_CASE, spec, lx, ly, lz, X)
    rng = np.random.default_rng(nb)
    psi = rng.normal(size=(nb,) + shape)
    veff = rng.normal(size=shape)
    ref = OK.hpsi_block(psi, geom, veff, closure)
    dg = device.device_grid(geom)
    for dtype, tol in ((torch.float64, 1e-12), (torch.float32, 2e-5)):
        got = ops.hpsi_device(dg, torch.as_tensor(psi, device="cuda", dtype=dtype), closure=closure, kscale=-0.5,
                              veff=torch.as_tensor(veff, device="cuda", dtype=dtype)).double().cpu().numpy()
        assert _rel(got, ref) < tol, (dtype, _rel(got, ref))
    assert _lib.error_flags(clear=True, stream=device.stream_ptr()) == 0


@pytest.mark.parametrize("shape", [(7, 29, 128), (6, 45, 64), (5, 43, 8), (9, 31, 4), (4, 16, 124), (33, 30, 40),
                                   (6, 29, 200), (5, 13, 136), (4, 11, 256)])
@pytest.mark.parametrize("closure", ["trial_fix", "production"])
def test_monitor_kernel_paths(shape, closure):
    """Every FP32 kernel (whole-row z-vectorised, tiled TMA, cp.async) against the oracle:
    full 128-point rows, one-lane rows, ragged last y tiles whose halo row touches the
    upper face (ny = 29, 43 for 14-row tiles; ny = 45 for 22-row tiles), partial orbital
    groups; with one orbital, rows of 136, 200 and 256 points take the whole-row kernel's
    two-chunk form (17, 25 and 32 lanes of eight points).  The whole-row kernel runs tuned and
    with its fixed rule (four orbitals per CTA for both closures; the production closure keeps
    its x-face values in shared slots, and nx = 4 and 5 reuse those slots early)."""

    import torch

    from isogriddft_gb300 import _lib, device, ops
    from isogriddft_gb300.config import H2_BENCHMARK_CASE
    from isogriddft_gb300.grid import build_monitor_grid_spec_for_case, monitor_box_axes, assemble_monitor_geometry

    spec = build_monitor_grid_spec_for_case(H2_BENCHMARK_CASE, shape=shape, box_half_extents=(5.0, 6.0, 7.0))
    lx, ly, lz, box = monitor_box_axes(spec)
    X = box.copy()
    X[..., 0] += 0.25 * np.sin(box[..., 2] * 0.45) * np.exp(-np.sum(box**2, axis=-1) / 25)
    X[..., 1] += 0.2 * np.sin(box[..., 0] * 0.5) * np.exp(-np.sum(box**2, axis=-1) / 20)
    geom = assemble_monitor_geometry(H2_BENCHMARK_CASE, spec, lx, ly, lz, X)
    rng = np.random.default_rng(7)
    dg = device.device_grid(geom)
    try:
        for nb in (1, 6):
            psi = rng.normal(size=(nb,) + shape)
            veff = rng.normal(size=shape)
            ref = OK.hpsi_block(psi, geom, veff, closure)
            t = torch.as_tensor(psi, device="cuda", dtype=torch.float32)
            v = torch.as_tensor(veff, device="cuda", dtype=torch.float32)
            for path in (0, 1, 2):
                _lib.check(_lib.call("igd_hpsi_select", path), "igd_hpsi_select")
                # the whole-row kernel tuned, and with the fixed rule (4 orbitals per CTA)
                for tune in ((1, 0) if path == 0 else (1,)):
                    _lib.check(_lib.call("igd_hpsi_autotune", tune), "igd_hpsi_autotune")
                    got = ops.hpsi_device(dg, t, closure=closure, kscale=-0.5, veff=v).double().cpu().numpy()
                    assert _rel(got, ref) < 2e-5, (path, tune, nb, _rel(got, ref))
    finally:
        _lib.call("igd_hpsi_select", 0)
        _lib.call("igd_hpsi_autotune", 1)
    assert _lib.error_flags(clear=True, stream=device.stream_ptr()) == 0


def test_host_block_apply_pipelined_matches_device():
    """Pinned host buffers stream through in orbital chunks (copies overlapped with the stencil,
    one native call: igd_hpsi_agrid_host); the result equals the device apply bit for bit, for
    every chunk size, FP32 and FP64, and also for the unpinned and 3-D forms."""

    import torch

    from isogriddft_gb300 import device, ops
    from isogriddft_gb300.config import H2_BENCHMARK_CASE
    from isogriddft_gb300.grid import build_monitor_grid_spec_for_case, monitor_box_axes, assemble_monitor_geometry

    shape = (20, 24, 32)
    spec = build_monitor_grid_spec_for_case(H2_BENCHMARK_CASE, shape=shape, box_half_extents=(5.0, 6.0, 7.0))
    lx, ly, lz, box = monitor_box_axes(spec)
    geom = assemble_monitor_geometry(H2_BENCHMARK_CASE, spec, lx, ly, lz, box.copy())
    rng = np.random.default_rng(5)
    psi = rng.normal(size=(13,) + shape).astype(np.float32)
    veff = rng.normal(size=shape)
    dg = device.device_grid(geom)
    want = ops.hpsi_device(dg, torch.as_tensor(psi, device="cuda").reshape(13, -1), closure="trial_fix",
                           veff=dg.potential(veff, torch.float32)).reshape(psi.shape).cpu().numpy()
    host_in = torch.from_numpy(psi).pin_memory()
    host_out = torch.empty_like(host_in).pin_memory()
    got = ops.apply_hamiltonian_block(host_in, geom, veff, out=host_out)
    assert got is host_out
    np.testing.assert_array_equal(host_out.numpy(), want)
    np.testing.assert_array_equal(ops.apply_hamiltonian_block(psi, geom, veff).numpy(), want)
    one = ops.apply_hamiltonian_block(torch.from_numpy(psi[3]).pin_memory(), geom, veff)
    np.testing.assert_array_equal(one.numpy(), want[3])
    # the native pipeline (igd_hpsi_agrid_host) in chunks of 1, 3 and 5 orbitals (ragged last chunk)
    v32 = dg.potential(veff, torch.float32)
    for ch in (1, 3, 5):
        out2 = torch.zeros_like(host_in).pin_memory()
        ops._pipelined_host_apply(dg, host_in, out2, "trial_fix", v32, chunk=ch)
        np.testing.assert_array_equal(out2.numpy(), want)
    # FP64 host block
    psi64 = psi.astype(np.float64)
    want64 = ops.hpsi_device(dg, torch.as_tensor(psi64, device="cuda").reshape(13, -1), closure="trial_fix",
                             veff=dg.potential(veff, torch.float64)).reshape(psi.shape).cpu().numpy()
    got64 = ops.apply_hamiltonian_block(torch.from_numpy(psi64).pin_memory(), geom, veff, precision="fp64")
    np.testing.assert_array_equal(got64.numpy(), want64)
    assert _lib_flags_clear()


def _lib_flags_clear():
    from isogriddft_gb300 import _lib, device

    return _lib.error_flags(clear=True, stream=device.stream_ptr()) == 0


def test_autotuner_picks_are_recorded_and_change_no_value():
    """The whole-row kernel's autotuner times 4, 2 and 1 orbitals per CTA on the first call
    of a shape and keeps the fastest; every candidate computes the same values, so the
    tuned apply equals the fixed-rule apply bit for bit, and the pick is reported."""

    import torch

    from isogriddft_gb300 import _lib, device, ops
    from isogriddft_gb300.config import H2_BENCHMARK_CASE
    from isogriddft_gb300.grid import assemble_monitor_geometry, build_monitor_grid_spec_for_case, monitor_box_axes

    shape = (23, 37, 64)
    spec = build_monitor_grid_spec_for_case(H2_BENCHMARK_CASE, shape=shape, box_half_extents=(5.0, 6.0, 7.0))
    lx, ly, lz, box = monitor_box_axes(spec)
    X = box.copy()
    X[..., 1] += 0.2 * np.sin(box[..., 2] * 0.5) * np.exp(-np.sum(box**2, axis=-1) / 20)
    geom = assemble_monitor_geometry(H2_BENCHMARK_CASE, spec, lx, ly, lz, X)
    dg = device.device_grid(geom)
    rng = np.random.default_rng(5)
    psi = torch.as_tensor(rng.normal(size=(6,) + shape), device="cuda", dtype=torch.float32)
    v = torch.as_tensor(rng.normal(size=shape), device="cuda", dtype=torch.float32)
    try:
        _lib.check(_lib.call("igd_hpsi_autotune", 0), "igd_hpsi_autotune")
        fixed = ops.hpsi_device(dg, psi, closure="trial_fix", kscale=-0.5, veff=v).cpu()
        _lib.check(_lib.call("igd_hpsi_autotune", 1), "igd_hpsi_autotune")
        tuned = ops.hpsi_device(dg, psi, closure="trial_fix", kscale=-0.5, veff=v).cpu()
        again = ops.hpsi_device(dg, psi, closure="trial_fix", kscale=-0.5, veff=v).cpu()
    finally:
        _lib.call("igd_hpsi_autotune", 1)
    assert torch.equal(fixed, tuned) and torch.equal(tuned, again)
    picks = [line for line in ops.autotune_report() if line.startswith("trial_fix 23 37 64 6 1 ->")]
    assert len(picks) == 1 and picks[0].split("->")[1].split()[0] in ("1", "2", "4"), ops.autotune_report()
    assert _lib.call("igd_hpsi_autotune", 2) == _lib.IGD_ERR_ARG


def test_bounded_wait_timeout_is_reported_and_the_context_survives():
    """Failure path of every bounded in-kernel wait: a wait that nothing satisfies gives up after
    its poll limit and sets bit 0 of the calling thread's error word (no fault, no hang); the
    next H.Psi apply on the same context is exact again and leaves the word clear."""

    import torch

    from isogriddft_gb300 import _lib, device, ops
    from isogriddft_gb300.config import H2_BENCHMARK_CASE
    from isogriddft_gb300.grid import assemble_monitor_geometry, build_monitor_grid_spec_for_case, monitor_box_axes

    st = device.stream_ptr()
    _lib.error_flags(clear=True, stream=st)
    _lib.check(_lib.call("igd_selftest_wait_timeout", 1000, st), "igd_selftest_wait_timeout")
    assert _lib.error_flags(clear=True, stream=st) & 1
    assert _lib.call("igd_selftest_wait_timeout", 0, st) == _lib.IGD_ERR_ARG
    shape = (12, 14, 16)
    spec = build_monitor_grid_spec_for_case(H2_BENCHMARK_CASE, shape=shape, box_half_extents=(5.0, 6.0, 7.0))
    lx, ly, lz, box = monitor_box_axes(spec)
    geom = assemble_monitor_geometry(H2_BENCHMARK_CASE, spec, lx, ly, lz, box.copy())
    psi = np.random.default_rng(2).normal(size=(2,) + shape)
    got = ops.hpsi_device(device.device_grid(geom), torch.as_tensor(psi, device="cuda"), closure="trial_fix",
                          kscale=-0.5).cpu().numpy()
    assert _rel(got, OK.hpsi_block(psi, geom, np.zeros(shape), "trial_fix")) < 1e-12
    assert _lib.error_flags(clear=True, stream=st) == 0
