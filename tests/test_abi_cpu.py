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


def _synthetic_grams(m, k, n=240, seed=0, deficient=False):
    import numpy as np

    rng = np.random.default_rng(seed)
    H = rng.normal(size=(n, n))
    H = 0.5 * (H + H.T) + np.diag(np.linspace(-3.0, 3.0, n))
    w = rng.uniform(0.5, 1.5, size=n)
    Q, _ = np.linalg.qr(rng.normal(size=(n, m)) * np.sqrt(w)[:, None] ** -1)
    B = Q.T / np.sqrt(w)[None, :]                       # W-orthonormal rows
    R = rng.normal(size=(k, n)) * 0.1
    if deficient and k > 1:
        R[-1] = R[0] + 1e-9 * rng.normal(size=n)        # a direction lost in the projection
    X = np.vstack([B, R])
    HX = X @ H                                          # rows: H applied to each vector (H symmetric)
    G0 = (X * w[None, :]) @ HX.T
    G1 = (X * w[None, :]) @ X.T
    return X, w, G0, G1


def test_native_subspace_step_matches_numpy():
    """``igd_subspace_step_host`` (plain C++, runs on the host) against the NumPy algebra of the
    fused eigensolver: same Ritz values, same Ritz vectors up to sign, same next subspace."""

    import numpy as np

    from isogriddft_gb300 import _build, _lib, ks

    if not os.path.exists(_lib.LIB_PATH):
        _build.build()
    for m, k, deficient, cut in ((12, 1, False, 1e-10), (12, 2, False, 1e-5), (8, 4, False, 1e-10),
                                 (8, 4, True, 1e-5), (10, 6, False, 1e-10)):
        X, w, G0, G1 = _synthetic_grams(m, k, seed=m + k, deficient=deficient)
        c_num, P_num, lam_num, V_num = ks.subspace_host_step_numpy(G0, G1, m, k, cut)
        c_nat, P_nat, lam_nat, V_nat = ks.subspace_host_step(G0, G1, m, k, cut)
        assert c_nat is not c_num
        np.testing.assert_allclose(lam_nat, lam_num, rtol=1e-10, atol=1e-11)
        mk = m + k

        def ritz(c, V):
            Q = c[: mk * m].reshape(mk, m)                # [CB; CR]
            return (Q @ V).T @ X                          # Ritz vectors as rows

        a, b = ritz(c_num, V_num), ritz(c_nat, V_nat)
        for i in range(m):
            s = np.sign(np.dot(a[i] * w, b[i]))
            np.testing.assert_allclose(s * b[i], a[i], atol=1e-8 * np.max(np.abs(a[i])))
        # the next residual coefficients are V_k and -V_k diag(lam_k)
        Vk = c_nat[mk * m: mk * m + m * k].reshape(m, k)
        np.testing.assert_allclose(c_nat[mk * m + m * k:].reshape(m, k), -Vk * lam_nat[None, :k], rtol=1e-14)


def test_header_is_plain_c_and_links(tmp_path):
    """include/isogrid_gb300.h compiles as C (what a cgo / JNI / N-API binding includes) and a C
    caller of the host-buffer entry point links against the in-tree library."""

    import shutil
    import subprocess

    import pytest

    from isogriddft_gb300 import _lib

    cc = shutil.which("gcc") or shutil.which("cc")
    cuda_inc = "/usr/local/cuda/include"
    if cc is None or not os.path.isdir(cuda_inc):
        pytest.skip("no C compiler or CUDA headers")
    src = tmp_path / "caller.c"
    src.write_text(
        '#include <cuda_runtime.h>\n#include "isogrid_gb300.h"\n'
        "int main(void) {\n"
        "  float h[8] = {0};\n"
        "  return igd_hpsi_agrid_host(IGD_F32, IGD_CLOSURE_TRIAL_FIX, 2, 2, 2, 0, 0, h, h, 1, -0.5, 1.0, 0, 0, 0, 0)"
        " == IGD_ERR_ARG ? 0 : 1;\n}\n")
    libdir = os.path.dirname(_lib.LIB_PATH)
    r = subprocess.run([cc, "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), "-I", cuda_inc,
                        str(src), "-o", str(tmp_path / "caller"), "-L", libdir, "-lisogrid_gb300",
                        f"-Wl,-rpath,{libdir}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    # the argument checks run before any CUDA call: nx < 3 is rejected on a host without a GPU
    run = subprocess.run([str(tmp_path / "caller")], capture_output=True, text=True)
    assert run.returncode == 0, (run.stdout, run.stderr)
