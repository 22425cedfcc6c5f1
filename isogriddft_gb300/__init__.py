"""GB300-native (sm_103a) Kohn-Sham hot path for IsoGridDFT.

Drop-in replacements for the reference's operator API (kinetic / Hamiltonian
apply, open-boundary Hartree solve, block eigensolver, LSDA XC, density
build) backed by hand-written CUDA kernels in ``libisogrid_gb300.so``.
"""

from . import config, grid  # noqa: F401
from .config import H2_BENCHMARK_CASE, BenchmarkCase  # noqa: F401

__version__ = "0.1.0"


def build(force: bool = False) -> str:
    """Compile the in-tree CUDA library for sm_103a and return its path."""

    from ._build import build as _b

    return _b(force=force)
