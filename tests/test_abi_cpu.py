"""The C-ABI library loads on a host without a GPU and exports every function the header declares."""

import os
import re

from tests.conftest import ROOT


def _declared():
    src = open(os.path.join(ROOT, "include", "isogrid_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:int|long long|const char\s*\*)\s+(igd_\w+)\s*\(", src, flags=re.M)))


def test_header_functions_are_exported_and_bound():
    import ctypes

    from isogriddft_gb300 import _build, _lib

    if not os.path.exists(_lib.LIB_PATH):
        _build.build()
    lib = ctypes.CDLL(_lib.LIB_PATH)
    names = _declared()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    unbound = [n for n in names if n not in _lib.SIGNATURES]
    assert not unbound, unbound
    assert _lib.load() is not None


def test_status_codes_map_to_exceptions():
    import pytest

    from isogriddft_gb300 import _lib

    _lib.check(_lib.IGD_OK, "ok")
    for code, exc in ((_lib.IGD_ERR_ARG, ValueError), (_lib.IGD_ERR_DTYPE, ValueError),
                      (_lib.IGD_ERR_TOO_LARGE, ValueError), (_lib.IGD_ERR_NONFINITE, ValueError),
                      (_lib.IGD_ERR_BREAKDOWN, _lib.KrylovBreakdown), (_lib.IGD_ERR_CUDA, RuntimeError)):
        with pytest.raises(exc):
            _lib.check(code, "x")
