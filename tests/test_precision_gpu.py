"""Mixed-precision vs FP64 study on a benzene-sized molecule, reduced grid (no reference
counterpart): the FP32 stencil / mixed Poisson / 3xTF32 Gram path against the all-FP64
GPU path on the same A-grid and input density (``isogriddft_gb300/precision.py``)."""

import pytest

from tests.conftest import gpu_available

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not gpu_available():
        pytest.skip("needs a CUDA GPU")


def test_benzene_mixed_vs_fp64_small_grid():
    """C6H6 (30 electrons, C s projectors) on a 64 x 64 x 48 A-grid, 15 states per spin with a
    32-column block: both eigensolves converge to 1e-5; the Hartree energy of the input
    density (mixed Poisson vs FP64) agrees to 1e-6 Ha, the eigenvalues to 1e-5 Ha and the
    stationary Harris-Foulkes energy to 1e-4 Ha (30 electrons, FP32 orbitals)."""

    from isogriddft_gb300 import precision

    case, geom = precision.build_study_geometry(shape=(64, 64, 48))
    runs = {p: precision.solve_one(case, geom, p, block=32) for p in ("fp64", "mixed")}
    for r in runs.values():
        assert r["eigensolver_converged"], r
    d = precision.compare(runs["mixed"], runs["fp64"])
    print(d)
    assert d["hartree_input_abs_diff"] < 1e-6
    assert d["eigenvalue_max_abs_diff"] < 1e-5
    assert d["harris_foulkes_abs_diff"] < 1e-4
    assert d["energy_abs_diff"]["ion_ion_repulsion"] == 0.0
