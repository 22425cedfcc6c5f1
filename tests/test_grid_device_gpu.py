"""Device monitor-grid generator vs the bit-exact host builder and the reference fixture."""

import numpy as np
import pytest

from tests.conftest import gpu_available

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not gpu_available():
        pytest.skip("needs a CUDA GPU")


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def test_device_generator_matches_reference_fixture(golden_monitor):
    from isogriddft_gb300.config import H2_BENCHMARK_CASE
    from isogriddft_gb300.grid import build_h2_local_patch_development_element_parameters, build_monitor_grid_for_case

    g = build_monitor_grid_for_case(H2_BENCHMARK_CASE, shape=(13, 13, 15), box_half_extents=(8.0, 8.0, 10.0),
                                    element_parameters=build_h2_local_patch_development_element_parameters(),
                                    device=True)
    gm = golden_monitor
    assert _rel(g.x_points, gm["x"]) < 1e-11
    assert _rel(g.z_points, gm["z"]) < 1e-11
    assert _rel(g.jacobian, gm["jacobian"]) < 1e-10
    assert _rel(g.inverse_metric_tensor, gm["inverse_metric"]) < 1e-10
    assert _rel(g.cell_volumes, gm["cell_volumes"]) < 1e-10


@pytest.mark.parametrize("shape", [(17, 19, 23), (24, 20, 28)])
def test_device_generator_matches_host(shape):
    from isogriddft_gb300.config import H2_BENCHMARK_CASE, make_h2o_case
    from isogriddft_gb300.grid import build_monitor_grid_for_case, build_two_peak_element_parameters

    for case, params in ((H2_BENCHMARK_CASE, build_two_peak_element_parameters(("H",))), (make_h2o_case(), None)):
        kw = dict(shape=shape, element_parameters=params)
        h = build_monitor_grid_for_case(case, **kw)
        d = build_monitor_grid_for_case(case, device=True, **kw)
        for attr in ("x_points", "y_points", "z_points", "jacobian", "inverse_metric_tensor", "metric_tensor",
                     "covariant_basis", "cell_volumes", "spacing_measure"):
            assert _rel(getattr(d, attr), getattr(h, attr)) < 1e-10, attr
        assert abs(d.quality_report.min_jacobian - h.quality_report.min_jacobian) < 1e-10 * h.quality_report.max_jacobian
        assert np.allclose(d.monitor_field.values, h.monitor_field.values, rtol=1e-12)
