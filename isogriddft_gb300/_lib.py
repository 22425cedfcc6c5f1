"""ctypes binding to the in-tree C ABI library ``libisogrid_gb300.so``.

The product path has no CPU fallback: if the library is missing or no CUDA
device is visible, every operator raises ``RuntimeError``.
"""

from __future__ import annotations

import ctypes
import os

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "libisogrid_gb300.so")

IGD_OK, IGD_ERR_ARG, IGD_ERR_DTYPE, IGD_ERR_CUDA, IGD_ERR_BREAKDOWN, IGD_ERR_NOT_CONVERGED, IGD_ERR_NONFINITE, IGD_ERR_TOO_LARGE = range(8)
IGD_F32, IGD_F64 = 0, 1
IGD_CLOSURE_TRIAL_FIX, IGD_CLOSURE_PRODUCTION = 0, 1
IGD_GRID_MONITOR, IGD_GRID_LEGACY = 0, 1
IGD_PREC_FP64, IGD_PREC_MIXED = 0, 1

_c_int, _c_ll, _c_dbl, _vp = ctypes.c_int, ctypes.c_longlong, ctypes.c_double, ctypes.c_void_p

# name -> argtypes (all return int status)
SIGNATURES: dict[str, list] = {
    "igd_version": [],
    "igd_error_flags": [_vp, _c_int, _vp],
    "igd_selftest_wait_timeout": [_c_int, _vp],
    "igd_agrid_prepare_geometry": [_c_int, _c_int, _c_int, _c_int, _c_dbl, _c_dbl, _c_dbl, _vp, _vp, _vp, _vp],
    "igd_hpsi_select": [_c_int],
    "igd_hpsi_agrid": [_c_int, _c_int, _c_int, _c_int, _c_int, _vp, _vp, _vp, _vp, _c_int, _c_ll, _c_dbl, _c_dbl, _vp],
    "igd_hpsi_agrid_host": [_c_int, _c_int, _c_int, _c_int, _c_int, _vp, _vp, _vp, _vp, _c_int, _c_dbl, _c_dbl, _vp, _vp,
                            _c_int, _vp],
    "igd_hpsi_legacy": [_c_int, _c_int, _c_int, _c_int, _vp, _vp, _vp, _vp, _c_int, _c_ll, _c_dbl, _c_dbl, _vp],
    "igd_poisson_workspace_bytes": [_c_int, _c_ll],
    "igd_poisson_solve": [_c_int, _c_int, _c_int, _c_int, _c_int, _vp, _vp, _vp, _vp, _c_dbl, _c_int, _vp, _c_ll, _vp,
                          _vp],
    "igd_poisson_solve_from": [_c_int, _c_int, _c_int, _c_int, _c_int, _vp, _vp, _vp, _vp, _c_dbl, _c_int, _vp, _c_ll,
                               _vp, _vp],
    "igd_multipole_nodal_moments": [_c_ll, _vp, _vp, _vp, _vp, _vp, _vp, _c_dbl, _c_dbl, _c_dbl, _vp, _vp],
    "igd_multipole_cell_quadrature": [_c_int, _c_int, _c_int, _vp, _vp, _vp, _vp, _vp, _vp, _c_int, _c_dbl, _c_int,
                                      _c_dbl, _c_dbl, _c_dbl, _vp, _vp, _vp],
    "igd_multipole_boundary": [_c_int, _c_int, _c_int, _vp, _vp, _vp, _vp, _c_int, _c_dbl, _c_dbl, _c_dbl, _vp,
                               _c_int, _vp],
    "igd_poisson_rhs": [_c_int, _c_int, _c_int, _vp, _vp, _vp, _vp],
    "igd_poisson_compose": [_c_int, _c_int, _c_int, _vp, _vp, _vp, _vp],
    "igd_weighted_sum": [_c_int, _c_ll, _vp, _vp, _vp, _vp, _vp],
    "igd_lsda": [_c_int, _c_int, _c_int, _c_ll, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp],
    "igd_density": [_c_int, _c_ll, _c_int, _c_ll, _vp, _vp, _vp, _vp, _vp, _c_int, _vp],
    "igd_density_renormalize": [_c_ll, _vp, _vp, _c_dbl, _vp, _vp],
    "igd_density_residual2": [_c_ll, _vp, _vp, _vp, _vp, _vp, _vp, _vp],
    "igd_gram_select": [_c_int],
    "igd_hpsi_autotune": [_c_int],
    "igd_hpsi_autotune_report": [_vp, _c_int],
    "igd_poisson_select": [_c_int],
    "igd_poisson_pcg_workspace_bytes": [_c_int, _c_int, _c_int, _c_int],
    "igd_poisson_pcg": [_c_int, _c_int, _c_int, _vp, _vp, _vp, _c_dbl, _c_int, _c_int, _vp, _vp, _c_int, _vp, _c_ll,
                        _vp, _vp],
    "igd_gram_last_path": [],
    "igd_block_gram_workspace_bytes": [_c_ll, _c_int, _c_int],
    "igd_block_gram": [_c_int, _c_ll, _c_int, _vp, _c_ll, _c_int, _vp, _c_ll, _vp, _vp, _c_int, _vp, _c_ll, _vp],
    "igd_block_rotate": [_c_int, _c_ll, _c_int, _vp, _c_ll, _vp, _c_int, _vp, _c_ll, _vp, _c_int, _vp, _c_ll, _c_int,
                         _vp],
    "igd_copy_h2d": [_vp, _vp, _c_ll, _vp],
    "igd_subspace_step_host": [_c_int, _c_int, _vp, _vp, _c_dbl, _vp, _vp, _vp, _vp, _vp],
    "igd_precond_jacobi": [_c_int, _c_ll, _c_int, _vp, _c_ll, _vp, _c_ll, _vp, _c_ll, _vp, _c_dbl, _c_dbl, _c_int,
                           _vp],
    "igd_gth_local_potential": [_c_ll, _vp, _vp, _vp, _c_int, _vp, _vp, _vp],
    "igd_gth_local_force": [_c_ll, _vp, _vp, _vp, _vp, _vp, _c_int, _vp, _vp, _vp],
    "igd_patch_knn": [_c_int, _vp, _vp, _vp, _c_ll, _vp, _vp, _vp, _c_int, _vp, _vp, _vp],
    "igd_patch_gather": [_c_int, _c_int, _vp, _vp, _vp, _vp, _vp],
    "igd_gth_projections": [_c_int, _c_int, _vp, _vp, _vp, _vp, _vp, _c_int, _c_ll, _vp, _vp],
    "igd_gth_nonlocal_apply": [_c_int, _c_int, _vp, _vp, _vp, _c_int, _vp, _vp, _vp, _vp, _vp, _vp, _c_int, _c_ll,
                               _c_dbl, _vp, _vp],
    "igd_grid_monitor_field": [_c_ll, _vp, _vp, _vp, _c_int, _vp, _vp, _vp, _vp],
    "igd_grid_smooth": [_c_int, _c_int, _c_int, _vp, _vp, _c_dbl, _vp],
    "igd_grid_harmonic_sweeps": [_c_int, _c_int, _c_int, _vp, _vp, _vp, _c_dbl, _c_dbl, _c_dbl, _c_dbl, _c_dbl,
                                 _c_int, _vp, _vp],
    "igd_grid_harmonic_sweeps_noalloc": [_c_int, _c_int, _c_int, _vp, _vp, _c_dbl, _c_dbl, _c_dbl, _c_dbl, _c_dbl,
                                         _c_int, _vp, _vp],
    "igd_grid_min_jacobian": [_c_int, _c_int, _c_int, _vp, _vp, _c_dbl, _c_dbl, _c_dbl, _c_dbl, _vp, _vp, _vp],
    "igd_grid_relax_update": [_c_ll, _vp, _vp, _c_dbl, _vp, _vp, _vp],
    "igd_grid_geometry": [_c_int, _c_int, _c_int, _vp, _c_dbl, _c_dbl, _c_dbl, _vp, _vp, _vp, _vp, _vp, _vp, _vp],
}

_LIB = None


def load(path: str = LIB_PATH):
    """Load the shared library and declare every exported signature."""

    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(path):
        raise RuntimeError(
            f"{path} is not built: run `python -c 'import __graft_entry__ as g; g.build()'` "
            "(the GB300 operators have no CPU fallback)"
        )
    lib = ctypes.CDLL(path)
    for name, argtypes in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = argtypes
        fn.restype = ctypes.c_longlong if name.endswith("_bytes") else ctypes.c_int
    _LIB = lib
    return lib


class KrylovBreakdown(RuntimeError):
    pass


def check(status: int, what: str = "isogrid_gb300 call") -> None:
    if status == IGD_OK:
        return
    msg = {
        IGD_ERR_ARG: "invalid argument",
        IGD_ERR_DTYPE: "unsupported dtype",
        IGD_ERR_CUDA: "CUDA launch/runtime error",
        IGD_ERR_BREAKDOWN: "Krylov breakdown",
        IGD_ERR_NOT_CONVERGED: "not converged",
        IGD_ERR_NONFINITE: "non-finite values",
        IGD_ERR_TOO_LARGE: "size above the fixed maximum",
    }.get(status, f"status {status}")
    if status in (IGD_ERR_ARG, IGD_ERR_DTYPE, IGD_ERR_NONFINITE, IGD_ERR_TOO_LARGE):
        raise ValueError(f"{what}: {msg}")
    if status == IGD_ERR_BREAKDOWN:
        raise KrylovBreakdown(f"{what}: {msg}")
    raise RuntimeError(f"{what}: {msg}")


def error_flags(clear: bool = True, stream: int | None = None) -> int:
    """Device error word (bit 0 = a bounded in-kernel wait timed out)."""

    out = ctypes.c_uint(0)
    check(call("igd_error_flags", ctypes.byref(out), int(clear), stream), "igd_error_flags")
    return int(out.value)


def call(name: str, *args) -> int:
    return getattr(load(), name)(*args)
