"""CPU oracle for the IsoGridDFT Kohn-Sham hot path -- TEST INFRASTRUCTURE ONLY.

This package restates, in FP64 NumPy/SciPy, the reference algorithms that the
GB300 kernels replace.  Every function cites the reference file:line it
follows (paths relative to the reference project root).  It exists to check
the CUDA path and to time the CPU baseline; nothing in the product package
imports it.  Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU legs of
``bench.py`` may import it.

Pinning: ``tests/golden/make_golden.py`` runs the reference's own NumPy
functions on small grids and stores inputs and outputs under ``tests/golden``;
``tests/test_oracle_golden.py`` checks every oracle function against those
fixtures and against the numbers recorded in the reference's
``src/isogrid/audit/baselines.py``.  The reference's LSDA delegates to
PySCF/libxc (absent); ``oracle.xc`` restates Slater exchange + VWN5
correlation from the published forms and is pinned at zeta = 0 by the recorded
legacy E_xc (``audit/baselines.py:822``); spin-polarised XC is pinned only
through the recorded triplet energies.
"""

from . import kinetic, poisson, xc, pseudo, eigensolver, scf  # noqa: F401
