"""Bond-length scan: geometries solved concurrently (host threads, one stream each) give the
same SCF results as one at a time."""

import pytest

from tests.conftest import gpu_available

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not gpu_available():
        pytest.skip("needs a CUDA GPU")


def test_concurrent_scan_matches_serial():
    from isogriddft_gb300 import scan

    pts = [scan.ScanPoint(1.2, "triplet", (64, 64, 72)), scan.ScanPoint(1.5, "singlet", (68, 64, 64)),
           scan.ScanPoint(1.8, "triplet", (64, 68, 64)), scan.ScanPoint(2.1, "singlet", (64, 64, 68))]
    kw = dict(precision="mixed", bands=2, max_iterations=25)
    serial = scan.run_scan(pts, **kw)
    concurrent = scan.run_scan(pts, workers=3, **kw)
    # the FP64 atomic reductions make every run differ in the last bits; through the SCF
    # (stop at |dE| < 1e-6 Ha, density residual < 1e-4) that reaches 3e-8 Ha (measured)
    # A-grid singlets do not converge (a two-cycle, as in the reference): their iterates
    # are chaotic, so only the converged triplets are compared by value
    for a, b in zip(serial, concurrent):
        assert a.point == b.point
        assert a.converged == b.converged
        if not a.converged:
            continue
        assert abs(a.scf_iterations - b.scf_iterations) <= 2
        assert abs(a.energy - b.energy) < 1e-6, (a.point, a.energy, b.energy)
        # eigenvalues to the eigensolver's residual tolerance (1e-4): the two up-spin states
        # of the triplet are near-degenerate
        assert max(abs(x - y) for x, y in zip(a.eigenvalues_up, b.eigenvalues_up)) < 1e-4
    assert sum(a.converged for a in serial) >= 1
