"""Differentiable H.Psi: gradcheck of the hand-written backward (adjoint stencil)."""

import numpy as np
import pytest

from tests.conftest import gpu_available

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not gpu_available():
        pytest.skip("needs a CUDA GPU")


def _geom(shape):
    from isogriddft_gb300.config import H2_BENCHMARK_CASE
    from isogriddft_gb300.grid import assemble_monitor_geometry, build_monitor_grid_spec_for_case, monitor_box_axes

    spec = build_monitor_grid_spec_for_case(H2_BENCHMARK_CASE, shape=shape, box_half_extents=(5.0, 6.0, 7.0))
    lx, ly, lz, box = monitor_box_axes(spec)
    X = box.copy()
    X[..., 0] += 0.3 * np.sin(box[..., 1] * 0.4) * np.exp(-np.sum(box**2, axis=-1) / 30)
    return assemble_monitor_geometry(H2_BENCHMARK_CASE, spec, lx, ly, lz, X)


@pytest.mark.parametrize("shape,fast", [((6, 7, 8), False), ((32, 32, 32), True)])
def test_hpsi_gradcheck(shape, fast):
    import torch

    from isogriddft_gb300.autograd import hpsi

    geom = _geom(shape)
    n = int(np.prod(shape))
    g = torch.Generator(device="cuda").manual_seed(0)
    psi = torch.randn((2, n), device="cuda", dtype=torch.float64, generator=g, requires_grad=True)
    veff = torch.randn(n, device="cuda", dtype=torch.float64, generator=g, requires_grad=True)
    assert torch.autograd.gradcheck(lambda p, v: hpsi(p, v, geom), (psi, veff), eps=1e-6, atol=1e-7, rtol=1e-6,
                                    fast_mode=fast)
