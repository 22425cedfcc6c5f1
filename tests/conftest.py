import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built extension")


def load_golden(name):
    return dict(np.load(os.path.join(GOLDEN, name)))


@pytest.fixture(scope="session")
def golden_monitor():
    return load_golden("monitor_h2_13x13x15.npz")


@pytest.fixture(scope="session")
def golden_legacy():
    return load_golden("legacy_h2_17x17x19.npz")


@pytest.fixture(scope="session")
def monitor_geom():
    from isogriddft_gb300.config import H2_BENCHMARK_CASE
    from isogriddft_gb300.grid import build_h2_local_patch_development_element_parameters, build_monitor_grid_for_case

    return build_monitor_grid_for_case(
        H2_BENCHMARK_CASE, shape=(13, 13, 15), box_half_extents=(8.0, 8.0, 10.0),
        element_parameters=build_h2_local_patch_development_element_parameters(),
    )


@pytest.fixture(scope="session")
def legacy_geom():
    from dataclasses import replace

    from isogriddft_gb300.config import H2_BENCHMARK_CASE
    from isogriddft_gb300.grid import build_default_h2_grid_spec, build_grid_geometry

    return build_grid_geometry(replace(build_default_h2_grid_spec(H2_BENCHMARK_CASE), nx=17, ny=17, nz=19))


def gpu_available():
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False
