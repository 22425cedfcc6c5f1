"""Fixed-potential Kohn-Sham operator and block eigensolver on the GPU.

Drop-in for ``src/isogrid/ks/eigensolver.py``:
* operator contexts ``prepare_fixed_potential_static_local_operator[_profiled]``
  (:571-727) freezing v_eff = V_loc + V_H + V_xc,sigma (all three evaluated on
  the device), ``apply_fixed_potential_static_local_operator`` / ``_block``
  (:729-784) -> one fused H.Psi launch (plus the GTH nonlocal term when the
  case has projectors, ``ks/static_hamiltonian.py:238-313``);
* ``weighted_overlap_matrix`` (:246), ``weighted_orthonormalize_orbitals``
  (:292, by the Gram eigendecomposition, which spans the same directions as the
  reference's SVD of sqrt(W) Psi), default guesses (:818-913);
* ``solve_fixed_potential_static_local_eigenproblem`` (:1183) and
  ``solve_fixed_potential_eigenproblem`` (:1136): the block subspace iteration
  of ``ks/eigensolver_jax.py:53-524`` (working block m = max(2k+2, 4, 12k+8,
  initial_subspace_size, ncv), residual expansion, whitening with QR-like
  fallback, (m+k)^2 Rayleigh-Ritz restart) with H.Psi, Gram and rotation
  kernels on the device and the small FP64 symmetric eigenproblems on the
  host.  All solver backends ("auto", "jax", "scipy_fallback") run it; parity
  with the reference is on converged eigenvalues and orbitals.

``precision="fp32"`` keeps orbitals, the stencil and rotations in FP32 with
FP64 Gram accumulation and FP64 Rayleigh-Ritz; the default is FP64.
"""

from __future__ import annotations

import ctypes
import threading
import time
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _lib
from .config import H2_BENCHMARK_CASE
from .device import device_grid, normalize_precision, ptr, stream_ptr, torch_dtype
from .grid import is_monitor_geometry
from .ops import hpsi_device

_VALID_SPIN = {"up", "down"}
_VALID_KINETIC = {"production", "trial_fix"}
_VALID_BACKENDS = {"auto", "jax", "scipy_fallback", "gb300"}


@dataclass(frozen=True)
class FixedPotentialStaticLocalPreparationProfile:
    density_build_wall_time_seconds: float
    local_ionic_resolve_wall_time_seconds: float
    hartree_resolve_wall_time_seconds: float
    xc_resolve_wall_time_seconds: float
    total_wall_time_seconds: float


@dataclass(frozen=True)
class FixedPotentialStaticLocalOperatorContext:
    grid_geometry: object
    case: object
    spin_channel: str
    rho_up: np.ndarray
    rho_down: np.ndarray
    rho_total: np.ndarray
    local_ionic_potential: np.ndarray
    hartree_potential: np.ndarray
    xc_potential: np.ndarray
    effective_local_potential: np.ndarray
    local_ionic_evaluation: object | None
    frozen_patch_local_embedding: object | None
    hartree_poisson_result: object | None
    lsda_evaluation: object | None
    kinetic_version: str = "production"
    include_nonlocal: bool = False
    device_cache: dict = field(default_factory=dict, repr=False, compare=False)


FixedPotentialOperatorContext = FixedPotentialStaticLocalOperatorContext


@dataclass(frozen=True)
class FixedPotentialEigensolverResult:
    target_orbitals: int
    solver_backend: str
    use_scipy_fallback: bool
    solver_method: str
    solver_note: str
    converged: bool
    iteration_count: int
    tolerance: float
    eigenvalues: np.ndarray
    orbitals: np.ndarray
    weighted_overlap: np.ndarray
    max_orthogonality_error: float
    residual_norms: np.ndarray
    residual_history: np.ndarray
    ritz_value_history: np.ndarray
    subspace_dimensions: tuple
    ritz_matrix: np.ndarray
    initial_guess_orbitals: np.ndarray
    final_basis_orbitals: np.ndarray
    operator_context: object
    static_local_preparation_profile: object | None = None
    use_jax_block_kernels: bool = False
    use_jax_cached_kernels: bool = False
    wall_time_seconds: float | None = None
    jax_internal_profile: object | None = None

    @property
    def internal_profile(self):
        return self.jax_internal_profile


# the reference's messages for its enumerated options (ks/eigensolver.py)
_CHOICE_MESSAGES = {
    "spin_channel": "spin_channel must be `up` or `down`; received `{}`.",
    "kinetic_version": "kinetic_version must be `production` or `trial_fix`; received `{}`.",
    "solver_backend": "solver_backend must be `auto`, `jax`, or `scipy_fallback`; received `{}`.",
}


def _norm_choice(value: str, valid, name):
    v = value.strip().lower()
    if v not in valid:
        msg = _CHOICE_MESSAGES.get(name)
        raise ValueError(msg.format(value) if msg else f"{name} must be one of {sorted(valid)}; received `{value}`.")
    return v


def _check_solver_request(k, initial_subspace_size, backend, use_jax_block_kernels, geom):
    """The reference's request checks (``ks/eigensolver.py:1011-1014``, ``:1248-1263``): its SciPy
    route (the default unless JAX block kernels are asked for on a monitor grid) rejects an
    initial subspace smaller than k; ``solver_backend="jax"`` needs the JAX block kernels and a
    monitor grid."""

    jax_route = backend == "jax" or (backend == "auto" and use_jax_block_kernels and is_monitor_geometry(geom))
    if not jax_route and initial_subspace_size is not None and initial_subspace_size < k:
        raise ValueError("initial_subspace_size must be at least k.")
    if backend == "jax" and not (use_jax_block_kernels and is_monitor_geometry(geom)):
        raise ValueError("solver_backend='jax' currently requires `use_jax_block_kernels=True` and a "
                         "MonitorGridGeometry static-local operator context.")


def _field(a, geom, name):
    arr = np.asarray(a, dtype=np.float64)
    if arr.shape != tuple(geom.spec.shape):
        raise ValueError(f"{name} must match the grid shape {geom.spec.shape}; received {arr.shape}.")
    return arr


def prepare_fixed_potential_static_local_operator_profiled(
    grid_geometry, rho_up, rho_down, spin_channel, case=H2_BENCHMARK_CASE, local_ionic_potential=None,
    hartree_potential=None, xc_potential=None, xc_functional=None, *, use_monitor_patch: bool = False,
    patch_parameters=None, kinetic_version: str = "production", base_local_ionic_evaluation=None,
    hartree_backend: str = "python", use_jax_hartree_cached_operator: bool = False,
    jax_hartree_cg_impl: str = "baseline", jax_hartree_cg_preconditioner: str = "none",
    jax_hartree_line_preconditioner_impl: str = "baseline",
    monitor_boundary_construction_mode: str = "corrected_moments", include_nonlocal: bool = False,
    hartree_precision: str = "fp64",
):
    """Freeze T + V_loc + V_H + V_xc (+ V_nl with include_nonlocal) on one grid."""

    from . import pseudo, poisson, xc

    t0 = time.perf_counter()
    spin = _norm_choice(spin_channel, _VALID_SPIN, "spin_channel")
    kin = _norm_choice(kinetic_version, _VALID_KINETIC, "kinetic_version")
    up = _field(rho_up, grid_geometry, "rho_up")
    dn = _field(rho_down, grid_geometry, "rho_down")
    t1 = time.perf_counter()
    rho = up + dn
    t2 = time.perf_counter()
    local_eval = None
    embedding = None
    if local_ionic_potential is None and use_monitor_patch and is_monitor_geometry(grid_geometry):
        # frozen near-core patch embedding of rho_total (``eigensolver.py:430-468``)
        embedding = pseudo.evaluate_monitor_grid_local_ionic_potential_with_frozen_patch_field(
            case, grid_geometry, rho, patch_parameters=patch_parameters, base_evaluation=base_local_ionic_evaluation)
        local_eval = embedding.base_evaluation
        vloc = embedding.corrected_total_local_potential
    elif local_ionic_potential is None:
        local_eval = pseudo.evaluate_local_ionic_potential(case, grid_geometry)
        vloc = local_eval.total_local_potential
    elif hasattr(local_ionic_potential, "total_local_potential"):
        local_eval = local_ionic_potential
        vloc = _field(local_ionic_potential.total_local_potential, grid_geometry, "local_ionic_potential")
    else:
        vloc = _field(local_ionic_potential, grid_geometry, "local_ionic_potential")
    t3 = time.perf_counter()
    hres = None
    if hartree_potential is None:
        hres = poisson.solve_hartree_potential(grid_geometry, rho, backend="python",
                                               monitor_boundary_construction_mode=monitor_boundary_construction_mode,
                                               precision=hartree_precision)
        vh = hres.potential
    elif hasattr(hartree_potential, "potential"):
        hres = hartree_potential
        vh = _field(hartree_potential.potential, grid_geometry, "hartree_potential")
    else:
        vh = _field(hartree_potential, grid_geometry, "hartree_potential")
    t4 = time.perf_counter()
    lsda = None
    if xc_potential is None:
        lsda = xc.evaluate_lsda_terms(up, dn, case.reference_model.xc if xc_functional is None else xc_functional)
        vxc = lsda.v_xc_up if spin == "up" else lsda.v_xc_down
    else:
        vxc = _field(xc_potential, grid_geometry, "xc_potential")
    t5 = time.perf_counter()
    ctx = FixedPotentialStaticLocalOperatorContext(
        grid_geometry=grid_geometry, case=case, spin_channel=spin, rho_up=up, rho_down=dn, rho_total=rho,
        local_ionic_potential=vloc, hartree_potential=vh, xc_potential=vxc,
        effective_local_potential=np.asarray(vloc + vh + vxc, dtype=np.float64), local_ionic_evaluation=local_eval,
        frozen_patch_local_embedding=embedding, hartree_poisson_result=hres, lsda_evaluation=lsda, kinetic_version=kin,
        include_nonlocal=bool(include_nonlocal),
    )
    prof = FixedPotentialStaticLocalPreparationProfile(t2 - t1, t3 - t2, t4 - t3, t5 - t4, time.perf_counter() - t0)
    return ctx, prof


def prepare_fixed_potential_static_local_operator(*args, **kwargs):
    return prepare_fixed_potential_static_local_operator_profiled(*args, **kwargs)[0]


def prepare_fixed_potential_static_ks_operator(grid_geometry, rho_up, rho_down, spin_channel, case=H2_BENCHMARK_CASE,
                                               local_ionic_potential=None, hartree_potential=None, xc_potential=None,
                                               xc_functional=None):
    """Static KS operator context (nonlocal term included; ``eigensolver.py:477-531``)."""

    return prepare_fixed_potential_static_local_operator(
        grid_geometry, rho_up, rho_down, spin_channel, case, local_ionic_potential, hartree_potential, xc_potential,
        xc_functional, kinetic_version="production", include_nonlocal=True)


class DeviceOperator:
    """H = T + v_eff (+ V_nl) on device blocks of a given dtype."""

    def __init__(self, ctx, dtype: torch.dtype):
        self.ctx = ctx
        self.geom = ctx.grid_geometry
        self.dg = device_grid(self.geom)
        self.dtype = dtype
        self.closure = ctx.kinetic_version if is_monitor_geometry(self.geom) else "legacy"
        key = ("veff", dtype)
        v = ctx.device_cache.get(key)
        if v is None:
            v = torch.as_tensor(np.ascontiguousarray(ctx.effective_local_potential), device=self.dg.device)
            v = v.reshape(-1).to(dtype).contiguous()
            ctx.device_cache[key] = v
        self.veff = v
        self.nonlocal_table = None
        if ctx.include_nonlocal:
            from .pseudo import projector_table

            t = projector_table(ctx.case, self.geom)
            self.nonlocal_table = t if t.nproj else None
        self.applies = 0

    @classmethod
    def from_potential(cls, geom, case, veff: torch.Tensor, *, closure: str, dtype: torch.dtype,
                       include_nonlocal: bool = False) -> "DeviceOperator":
        """Operator over a device-resident v_eff (n,) of the operator dtype (SCF steps)."""

        self = cls.__new__(cls)
        self.ctx, self.geom, self.dg, self.dtype = None, geom, device_grid(geom), dtype
        self.closure = closure if is_monitor_geometry(geom) else "legacy"
        self.veff = veff.reshape(-1).to(dtype).contiguous()
        self.nonlocal_table = None
        if include_nonlocal:
            from .pseudo import projector_table

            t = projector_table(case, geom)
            self.nonlocal_table = t if t.nproj else None
        self.applies = 0
        return self

    def __call__(self, block: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
        out = hpsi_device(self.dg, block, closure=self.closure, kscale=-0.5, veff=self.veff, out=out)
        if self.nonlocal_table is not None:
            self.nonlocal_table.apply(self.dg, block, out)
        self.applies += block.shape[0]
        return out


def operator_for(ctx, precision: str = "fp64") -> DeviceOperator:
    dt = torch_dtype(normalize_precision(precision))
    key = ("op", dt)
    op = ctx.device_cache.get(key)
    if op is None:
        op = DeviceOperator(ctx, dt)
        ctx.device_cache[key] = op
    return op


def validate_orbital_block(orbitals, grid_geometry, name: str = "orbitals"):
    block = np.asarray(orbitals)
    if block.ndim == 3:
        block = block[np.newaxis, ...]
    if block.ndim != 4:
        raise ValueError(f"{name} must be a 3D orbital or a 4D orbital block.")
    if block.shape[1:] != tuple(grid_geometry.spec.shape):
        raise ValueError(f"{name} must match the grid shape {grid_geometry.spec.shape}; received {block.shape[1:]}.")
    if not np.issubdtype(block.dtype, np.inexact):
        block = block.astype(np.float64)
    return block


def apply_fixed_potential_static_local_block(orbitals, operator_context, *, precision: str = "fp64"):
    block = validate_orbital_block(orbitals, operator_context.grid_geometry)
    op = operator_for(operator_context, precision)
    t = torch.as_tensor(np.ascontiguousarray(block), device=op.dg.device).to(op.dtype).reshape(block.shape[0], -1)
    return op(t).to(torch.float64).cpu().numpy().reshape(block.shape)


def apply_fixed_potential_static_local_operator(psi, operator_context, *, precision: str = "fp64"):
    return apply_fixed_potential_static_local_block(psi, operator_context, precision=precision)[0]


apply_fixed_potential_static_ks_block = apply_fixed_potential_static_local_block
apply_fixed_potential_static_ks_operator = apply_fixed_potential_static_local_operator


# ----------------------------------------------------------------- block algebra
class BlockLA:
    """Gram / rotation on row-major (k, n) device blocks."""

    def __init__(self, dg, stream: int | None = None, workspace: torch.Tensor | None = None):
        self.dg = dg
        self.w = dg.cell_volumes
        self.st = stream_ptr() if stream is None else stream
        self._wsb: dict = {}
        self._ws = workspace  # a private Gram workspace (graph capture needs a fixed one)

    def gram(self, A: torch.Tensor, B: torch.Tensor, weighted: bool = True, out=None) -> torch.Tensor:
        a, b = A.shape[0], B.shape[0]
        if out is None:
            out = torch.empty((a, b), dtype=torch.float64, device=self.dg.device)
        wsb = self._wsb.get((a, b))
        if wsb is None:
            wsb = self._wsb[(a, b)] = int(_lib.call("igd_block_gram_workspace_bytes", self.dg.n, a, b))
        if self._ws is not None and self._ws.numel() >= wsb:
            ws = self._ws
        else:
            ws = self.dg.workspace("gram", wsb)
        dt = _lib.IGD_F32 if A.dtype == torch.float32 else _lib.IGD_F64
        _lib.check(_lib.call("igd_block_gram", dt, self.dg.n, a, ptr(A), A.stride(0), b, ptr(B), B.stride(0),
                             ptr(self.w) if weighted else None, ptr(out), 0, ptr(ws), wsb, self.st),
                   "igd_block_gram")
        return out

    def rotate(self, A, C1, B=None, C2=None, out=None, accumulate=False) -> torch.Tensor:
        """out = A^T C1 (+ B^T C2) (+ out); C are FP64 device (a, c) matrices."""

        c = C1.shape[1]
        if out is None:
            out = torch.empty((c, self.dg.n), dtype=A.dtype, device=self.dg.device)
        C1 = C1.contiguous()
        b = 0 if B is None else B.shape[0]
        if B is not None:
            C2 = C2.contiguous()
        dt = _lib.IGD_F32 if A.dtype == torch.float32 else _lib.IGD_F64
        _lib.check(_lib.call("igd_block_rotate", dt, self.dg.n, A.shape[0], ptr(A), A.stride(0), ptr(C1), b,
                             ptr(B) if b else None, B.stride(0) if b else 0, ptr(C2) if b else None, c, ptr(out),
                             out.stride(0), int(accumulate), self.st), "igd_block_rotate")
        return out


def _dev64(m, dev):
    return torch.as_tensor(np.ascontiguousarray(m, dtype=np.float64), device=dev)


class _Uploader:
    """Small FP64 host matrices to the device through pinned staging slots.

    A plain copy from pageable memory waits for all queued work on the stream;
    the staged copy does not.  A slot is reused only after ``slots`` later
    uploads; callers synchronise with the device at least once every
    ``slots / 2`` uploads (the fused eigensolver: one upload and one host read
    per iteration).  The copy is one ``igd_copy_h2d`` call on the held stream."""

    _local = threading.local()  # staging slots are per thread (released with the thread)

    def __init__(self, dev, max_elems: int, slots: int = 4):
        pool = getattr(_Uploader._local, "pool", None)
        if pool is None:
            pool = _Uploader._local.pool = {}
        key = (str(dev), int(max_elems), slots)
        bufs = pool.get(key)
        if bufs is None:
            host = [torch.empty(max_elems, dtype=torch.float64, pin_memory=True) for _ in range(slots)]
            bufs = (host, [torch.empty(max_elems, dtype=torch.float64, device=dev) for _ in range(slots)],
                    [h.numpy() for h in host])
            pool[key] = bufs
        self.host, self.dev, self.hnp = bufs
        self.host_ptrs = [h.data_ptr() for h in self.host]
        self.i = 0

    def __call__(self, a, dst: torch.Tensor | None = None) -> torch.Tensor:
        """Device copy of ``a`` (an array, or a sequence of arrays laid end to end) into a
        ring slot, or into ``dst`` when given; returns the flat device view for a sequence."""

        parts = a if isinstance(a, (list, tuple)) else (a,)
        k = self.i
        self.i = (self.i + 1) % len(self.host)
        hv, size = self.hnp[k], 0
        for part in parts:
            part = np.asarray(part, dtype=np.float64)
            hv[size: size + part.size] = part.reshape(-1)
            size += part.size
        d = self.dev[k][:size] if dst is None else dst.view(-1)[:size]
        _lib.check(_lib.call("igd_copy_h2d", d.data_ptr(), self.host[k].data_ptr(), size * 8, stream_ptr()),
                   "igd_copy_h2d")
        return d if isinstance(a, (list, tuple)) else d.view(np.shape(a))

    def flat(self, a: np.ndarray, dst_ptr: int, stream: int) -> None:
        """The per-iteration form: a flat FP64 array to a fixed device address on a known
        stream (no tensor views or stream lookups per call)."""

        k = self.i
        self.i = (self.i + 1) % len(self.host)
        self.hnp[k][: a.size] = a
        _lib.check(_lib.call("igd_copy_h2d", dst_ptr, self.host_ptrs[k], a.size * 8, stream), "igd_copy_h2d")


def _chol_whitening(G: np.ndarray) -> np.ndarray:
    """L^-T of the Cholesky factor (same span as the symmetric whitening, cheaper)."""

    try:
        return np.linalg.inv(np.linalg.cholesky(_sym(G))).T
    except np.linalg.LinAlgError:
        return _whitening(G)


def _whitening(G: np.ndarray):
    """Inverse square root of a Gram matrix, or a Cholesky-based fallback (QR-equivalent)
    when its smallest eigenvalue is <= 1e-10 (``eigensolver_jax.py:119-146``)."""

    G = 0.5 * (G + G.T)
    ev, V = np.linalg.eigh(G)
    if np.all(np.isfinite(ev)) and ev.min() > 1.0e-10:
        return (V * (1.0 / np.sqrt(np.clip(ev, 1e-14, None)))[None, :]) @ V.T
    # R^-1 of a QR of sqrt(W) X equals the inverse Cholesky factor of G (rank-deficient: jittered)
    jitter = 0.0
    for _ in range(8):
        try:
            L = np.linalg.cholesky(G + jitter * np.eye(len(G)))
            return np.linalg.inv(L).T
        except np.linalg.LinAlgError:
            jitter = max(1e-14, 10 * jitter) * max(1.0, float(np.max(np.abs(np.diag(G)))))
    return (V * (1.0 / np.sqrt(np.clip(ev, 1e-14, None)))[None, :]) @ V.T


def weighted_overlap_matrix(orbitals, grid_geometry, other=None, *, use_jax_block_kernels: bool = False):
    dg = device_grid(grid_geometry)
    la = BlockLA(dg)
    A = torch.as_tensor(np.ascontiguousarray(validate_orbital_block(orbitals, grid_geometry), dtype=np.float64),
                        device=dg.device)
    A = A.reshape(A.shape[0], -1)
    B = A if other is None else torch.as_tensor(
        np.ascontiguousarray(validate_orbital_block(other, grid_geometry), dtype=np.float64), device=dg.device
    ).reshape(-1, dg.n)
    return la.gram(A, B).cpu().numpy()


def weighted_orbital_norms(orbitals, grid_geometry, *, use_jax_block_kernels: bool = False):
    return np.sqrt(np.clip(np.diag(weighted_overlap_matrix(orbitals, grid_geometry)), 0.0, None))


def orthonormalize_device(la: BlockLA, X: torch.Tensor, require_full_rank=True, rank_tolerance=1.0e-12):
    """W-orthonormal basis of span(X) ordered by decreasing singular value (SVD of sqrt(W) X)."""

    G = la.gram(X, X).cpu().numpy()
    G = 0.5 * (G + G.T)
    ev, V = np.linalg.eigh(G)
    ev, V = ev[::-1], V[:, ::-1]
    s = np.sqrt(np.clip(ev, 0.0, None))
    if s.size == 0 or s[0] == 0.0:
        if require_full_rank:
            raise ValueError("The orbital block is numerically rank-deficient in the weighted metric.")
        return X[:0]
    cut = rank_tolerance * max(la.dg.n, X.shape[0]) * s[0]
    rank = int(np.sum(s > cut))
    if require_full_rank and rank < X.shape[0]:
        raise ValueError(f"The orbital block is rank-deficient under weighted orthonormalization: rank={rank}, "
                         f"requested={X.shape[0]}.")
    T = V[:, :rank] / s[:rank]
    return la.rotate(X, _dev64(T, la.dg.device))


def weighted_orthonormalize_orbitals(orbitals, grid_geometry, *, require_full_rank: bool = True,
                                     rank_tolerance: float = 1.0e-12, use_jax_block_kernels: bool = False):
    block = validate_orbital_block(orbitals, grid_geometry)
    if block.shape[0] == 0:
        return block.copy()
    dg = device_grid(grid_geometry)
    X = torch.as_tensor(np.ascontiguousarray(block, dtype=np.float64), device=dg.device).reshape(block.shape[0], -1)
    Q = orthonormalize_device(BlockLA(dg), X, require_full_rank, rank_tolerance)
    return Q.cpu().numpy().reshape((Q.shape[0],) + tuple(grid_geometry.spec.shape))


def default_guess_device(case, geom, dg, count: int) -> torch.Tensor:
    """``_build_default_guess_orbitals`` (eigensolver.py:818-879) on the device grid."""

    dev = dg.device
    x, y, z = dg.x, dg.y, dg.z
    if is_monitor_geometry(geom):
        b = geom.spec.box_bounds
        c = (0.5 * (b[0][0] + b[0][1]), 0.5 * (b[1][0] + b[1][1]), 0.5 * (b[2][0] + b[2][1]))
    else:
        c = tuple(geom.spec.reference_center)
    xs, ys, zs = x - c[0], y - c[1], z - c[2]
    r2 = xs * xs + ys * ys + zs * zs
    gauss = [torch.exp(-0.85 * ((x - a.position[0]) ** 2 + (y - a.position[1]) ** 2 + (z - a.position[2]) ** 2))
             for a in case.geometry.atoms]
    g = []
    if gauss:
        g.append(torch.stack(gauss).sum(0))
    if len(gauss) >= 2:
        alt = torch.zeros_like(gauss[0])
        for i, a in enumerate(gauss):
            alt = alt + a if i % 2 == 0 else alt - a
        g.append(alt)
    base = torch.exp(-0.65 * r2)
    g += [base, zs * torch.exp(-0.55 * r2), xs * torch.exp(-0.55 * r2), ys * torch.exp(-0.55 * r2),
          torch.exp(-1.10 * r2), (3.0 * zs * zs - r2) * torch.exp(-0.45 * r2)]
    need = max(count, 8)
    if len(g) < need:
        rng = np.random.default_rng(12345)
        shape = tuple(geom.spec.shape)
        while len(g) < need:
            g.append(base * torch.as_tensor(rng.normal(size=shape).reshape(-1), device=dev))
    X = torch.stack(g[:need]).contiguous()
    Q = orthonormalize_device(BlockLA(dg), X, require_full_rank=False)
    if Q.shape[0] < count:
        raise ValueError("Unable to build enough independent default guess orbitals for the fixed-potential solve.")
    return Q[:count].contiguous()


def block_size(k, initial_subspace_size=None, ncv=None):
    return max(2 * k + 2, 4, 12 * k + 8, int(initial_subspace_size or 0), int(ncv or 0))


def block_subspace_iteration_device(op: DeviceOperator, case, k: int, *, max_iterations: int = 400,
                                    tolerance: float = 1.0e-3, initial_guess=None, initial_subspace_size=None,
                                    ncv=None, check_every: int = 1, default_guess: torch.Tensor | None = None,
                                    stall_iterations: int | None = None, fused: bool = True,
                                    preconditioner=None, block: int | None = None, graphs: bool = True,
                                    ritz: str = "symmetric"):
    """GPU twin of the JAX block iteration (``eigensolver_jax.py:417-524``); returns a dict.

    ``fused`` (default) runs :func:`block_subspace_iteration_fused` (one host
    round trip per iteration); ``fused=False`` runs the step-by-step form with
    a device Gram product for every small matrix the reference forms.

    ``ritz``: ``"symmetric"`` (the reference's Rayleigh-Ritz, on the symmetrised
    projected matrices) or ``"right"`` (the fused iteration only): eigenpairs of the
    projected matrices themselves, so the Ritz pairs converge to right eigenpairs
    H x = lambda x with a vanishing residual also where H is not self-adjoint in
    the cell-volume inner product (the legacy grid, the production closure)."""

    if ritz not in ("symmetric", "right"):
        raise ValueError(f"ritz must be 'symmetric' or 'right'; received {ritz!r}.")
    if fused:
        return block_subspace_iteration_fused(op, case, k, max_iterations=max_iterations, tolerance=tolerance,
                                              initial_guess=initial_guess, initial_subspace_size=initial_subspace_size,
                                              ncv=ncv, default_guess=default_guess, stall_iterations=stall_iterations,
                                              preconditioner=preconditioner, block=block, graphs=graphs, ritz=ritz)
    if preconditioner is not None:
        raise ValueError("a residual preconditioner needs the fused iteration")
    if ritz != "symmetric":
        raise ValueError("ritz='right' needs the fused iteration")

    if k <= 0:
        raise ValueError(f"k must be positive; received {k}.")
    if max_iterations <= 0:
        raise ValueError(f"max_iterations must be positive; received {max_iterations}.")
    if tolerance <= 0.0:
        raise ValueError(f"tolerance must be positive; received {tolerance}.")
    dg, geom, dt = op.dg, op.geom, op.dtype
    dev = dg.device
    la = BlockLA(dg)
    m = block_size(k, initial_subspace_size, ncv)
    target = max(k, m)
    guess = default_guess[:target] if default_guess is not None and default_guess.shape[0] >= target else \
        default_guess_device(case, geom, dg, target)
    if initial_guess is not None:
        if isinstance(initial_guess, torch.Tensor):
            user = initial_guess.to(device=dev, dtype=torch.float64).reshape(-1, dg.n)
        else:
            user = torch.as_tensor(np.ascontiguousarray(validate_orbital_block(initial_guess, geom), dtype=np.float64),
                                   device=dev).reshape(-1, dg.n)
        comb = orthonormalize_device(la, torch.cat([user, guess]), require_full_rank=False)
        if comb.shape[0] < k:
            raise ValueError("The provided initial guesses do not span enough weighted-independent directions.")
        guess = comb[:target]
    guess = guess[:m].contiguous()
    X0 = guess.to(dt)
    # weighted QR of the start block (R^-1 from the Cholesky factor of its Gram matrix)
    B = la.rotate(X0, _dev64(np.linalg.inv(np.linalg.cholesky(_sym(la.gram(X0, X0).cpu().numpy()))).T, dev))
    HB = op(B)
    res_hist, ritz_hist, dims = [], [], []
    converged = False
    it = 0
    eig = np.zeros(k)
    rn = np.full(k, np.inf)
    ritz_mat = np.zeros((k, k))
    X = B[:k]
    best_rn, best_it, stalled = np.inf, 0, False
    for it in range(1, max_iterations + 1):
        P = _sym(la.gram(B, HB).cpu().numpy())
        lam, V = np.linalg.eigh(P)
        Vk = V[:, :k]
        X = la.rotate(B, _dev64(Vk, dev))
        R = la.rotate(HB, _dev64(Vk, dev), B, _dev64(-Vk * lam[None, :k], dev))
        rn = np.sqrt(np.clip(np.diag(la.gram(R, R).cpu().numpy()), 0.0, None))
        eig, ritz_mat = lam[:k].copy(), P[:k, :k].copy()
        res_hist.append(rn)
        ritz_hist.append(eig)
        dims.append(m)
        if float(rn.max()) <= tolerance:
            converged = True
            break
        # optional stop once the residual has stopped falling and the Ritz values
        # have settled (a non-self-adjoint operator leaves a residual floor above
        # the tolerance while its Ritz values converge)
        if stall_iterations:
            cur = float(rn.max())
            if cur < best_rn * (1.0 - 1.0e-2):
                best_rn, best_it = cur, it
            elif it - best_it >= stall_iterations and len(ritz_hist) > stall_iterations:
                drift = float(np.max(np.abs(ritz_hist[-1] - ritz_hist[-1 - stall_iterations])))
                if drift <= 1.0e-12 * max(1.0, float(np.max(np.abs(ritz_hist[-1])))):
                    stalled = True
                    break
        G1 = la.gram(B, R)  # (m, k) device
        la.rotate(B, -G1, out=R, accumulate=True)
        R = la.rotate(R, _dev64(_whitening(la.gram(R, R).cpu().numpy()), dev))
        HR = op(R)
        BHR = la.gram(B, HR).cpu().numpy()
        RHB = la.gram(R, HB).cpu().numpy()
        RHR = la.gram(R, HR).cpu().numpy()
        T = _sym(np.block([[P, BHR], [RHB, RHR]]))
        _, Wt = np.linalg.eigh(T)
        W11, W21 = _dev64(Wt[:m, :m], dev), _dev64(Wt[m:, :m], dev)
        Bn = la.rotate(B, W11, R, W21)
        HBn = la.rotate(HB, W11, HR, W21)
        Tw = _dev64(_whitening(la.gram(Bn, Bn).cpu().numpy()), dev)
        B = la.rotate(Bn, Tw)
        HB = la.rotate(HBn, Tw)
        del Bn, HBn, HR
    overlap = la.gram(X, X).cpu().numpy()
    return {
        "eigenvalues": eig, "orbitals": X, "converged": converged, "iteration_count": it, "residual_norms": rn,
        "residual_history": np.asarray(res_hist), "ritz_value_history": np.asarray(ritz_hist),
        "subspace_dimensions": tuple(dims), "weighted_overlap": overlap,
        "max_orthogonality_error": float(np.max(np.abs(overlap - np.eye(k)))), "ritz_matrix": ritz_mat,
        "initial_guess": guess, "final_basis": B, "stalled": stalled,
    }


def _sym(M):
    return 0.5 * (M + M.T)


def _result(res, ctx, k, tolerance, backend, profile, wall, geom, precision):
    shape = tuple(geom.spec.shape)
    host = lambda t: t.to(torch.float64).cpu().numpy().reshape((t.shape[0],) + shape)  # noqa: E731
    return FixedPotentialEigensolverResult(
        target_orbitals=k, solver_backend=backend, use_scipy_fallback=(backend == "scipy_fallback"),
        solver_method="gb300_block_subspace_iteration",
        solver_note=("Block subspace iteration with residual expansion and Rayleigh-Ritz restart on the GB300: "
                     f"fused H.Psi, Gram and rotation kernels in {precision}, FP64 Rayleigh-Ritz on the host."),
        converged=bool(res["converged"]), iteration_count=int(res["iteration_count"]), tolerance=float(tolerance),
        eigenvalues=np.asarray(res["eigenvalues"], dtype=np.float64), orbitals=host(res["orbitals"]),
        weighted_overlap=res["weighted_overlap"], max_orthogonality_error=res["max_orthogonality_error"],
        residual_norms=np.asarray(res["residual_norms"]), residual_history=res["residual_history"],
        ritz_value_history=res["ritz_value_history"], subspace_dimensions=res["subspace_dimensions"],
        ritz_matrix=res["ritz_matrix"], initial_guess_orbitals=host(res["initial_guess"]),
        final_basis_orbitals=host(res["final_basis"]), operator_context=ctx, static_local_preparation_profile=profile,
        use_jax_block_kernels=False, use_jax_cached_kernels=False, wall_time_seconds=wall,
    )


def solve_fixed_potential_static_local_eigenproblem(
    grid_geometry, rho_up, rho_down, spin_channel, k, case=H2_BENCHMARK_CASE, initial_guess_orbitals=None,
    local_ionic_potential=None, hartree_potential=None, xc_potential=None, xc_functional=None, operator_context=None,
    max_iterations: int = 400, tolerance: float = 1.0e-3, initial_subspace_size=None, ncv=None, *,
    use_monitor_patch: bool = False, patch_parameters=None, kinetic_version: str = "production",
    use_jax_block_kernels: bool = False, operator_preparation_profile=None, base_local_ionic_evaluation=None,
    hartree_backend: str = "python", use_jax_hartree_cached_operator: bool = False,
    jax_hartree_cg_impl: str = "baseline", jax_hartree_cg_preconditioner: str = "none",
    jax_hartree_line_preconditioner_impl: str = "baseline",
    monitor_boundary_construction_mode: str = "corrected_moments", solver_backend: str = "auto",
    profile_jax_internals: bool = False, precision: str = "fp64", ritz: str = "symmetric",
) -> FixedPotentialEigensolverResult:
    """GPU twin of ``ks/eigensolver.py:1183-1320``.  ``ritz="right"`` (no reference
    counterpart) converges to right eigenpairs where the operator is not self-adjoint in the
    cell-volume inner product (see :func:`block_subspace_iteration_device`)."""

    backend = _norm_choice(solver_backend, _VALID_BACKENDS, "solver_backend")
    _check_solver_request(k, initial_subspace_size, backend, use_jax_block_kernels,
                          operator_context.grid_geometry if operator_context is not None else grid_geometry)
    if operator_context is None:
        operator_context, operator_preparation_profile = prepare_fixed_potential_static_local_operator_profiled(
            grid_geometry, rho_up, rho_down, spin_channel, case, local_ionic_potential, hartree_potential,
            xc_potential, xc_functional, use_monitor_patch=use_monitor_patch, patch_parameters=patch_parameters,
            kinetic_version=kinetic_version, monitor_boundary_construction_mode=monitor_boundary_construction_mode)
    if backend == "auto":
        backend = "jax" if use_jax_block_kernels and is_monitor_geometry(operator_context.grid_geometry) \
            else "scipy_fallback"
    prec = normalize_precision(precision)
    op = operator_for(operator_context, prec)
    t0 = time.perf_counter()
    res = block_subspace_iteration_device(op, operator_context.case, k, max_iterations=max_iterations,
                                          tolerance=tolerance, initial_guess=initial_guess_orbitals,
                                          initial_subspace_size=initial_subspace_size, ncv=ncv, ritz=ritz)
    torch.cuda.current_stream().synchronize()
    return _result(res, operator_context, k, tolerance, backend, operator_preparation_profile,
                   time.perf_counter() - t0, operator_context.grid_geometry, prec)


def solve_fixed_potential_eigenproblem(grid_geometry, rho_up, rho_down, spin_channel, k, case=H2_BENCHMARK_CASE,
                                       initial_guess_orbitals=None, local_ionic_potential=None, hartree_potential=None,
                                       xc_potential=None, xc_functional=None, max_iterations: int = 400,
                                       tolerance: float = 1.0e-3, initial_subspace_size=None, ncv=None, *,
                                       precision: str = "fp64") -> FixedPotentialEigensolverResult:
    """Static KS route (``eigensolver.py:1136-1180``): production kinetic, nonlocal term included."""

    ctx = prepare_fixed_potential_static_ks_operator(grid_geometry, rho_up, rho_down, spin_channel, case,
                                                     local_ionic_potential, hartree_potential, xc_potential,
                                                     xc_functional)
    prec = normalize_precision(precision)
    op = operator_for(ctx, prec)
    t0 = time.perf_counter()
    res = block_subspace_iteration_device(op, case, k, max_iterations=max_iterations, tolerance=tolerance,
                                          initial_guess=initial_guess_orbitals,
                                          initial_subspace_size=initial_subspace_size, ncv=ncv)
    torch.cuda.current_stream().synchronize()
    return _result(res, ctx, k, tolerance, "scipy_fallback", None, time.perf_counter() - t0, grid_geometry, prec)


def kinetic_diagonal(dg, closure: str, dtype: torch.dtype) -> torch.Tensor:
    """diag(T) of the stencil operator, probed with 5^3 interleaved unit combs (the
    stencil reaches two points along each axis, so combs with period 5 never
    overlap).  Cached per grid, closure and dtype."""

    cache = getattr(dg, "_kdiag", None)
    if cache is None:
        cache = dg._kdiag = {}
    key = (closure, dtype)
    d = cache.get(key)
    if d is not None:
        return d
    nx, ny, nz = dg.shape
    d = torch.zeros(dg.n, dtype=dtype, device=dg.device)
    E = torch.empty((25, nx, ny, nz), dtype=dtype, device=dg.device)
    for a in range(5):  # 25 combs per stencil launch
        E.zero_()
        for b in range(5):
            for c in range(5):
                E[5 * b + c, a::5, b::5, c::5] = 1.0
        Ef = E.reshape(25, -1)
        d += (hpsi_device(dg, Ef, closure=closure, kscale=-0.5) * Ef).sum(0)
    cache[key] = d
    return d


class JacobiPreconditioner:
    """t ~ (T + sigma)^-1 r by damped Jacobi sweeps (``igd_precond_jacobi`` + stencil applies).

    Four sweeps by default.  On H2 A-grid scan points (0.5-0.6M points, 4 bands) the mixed
    SCF took 0.77 / 0.72 / 0.67 s per geometry with 4 / 8 / 12 sweeps, and the legacy 51^3
    singlet 0.45 / 0.37 / 0.34 s (FP64).  The different Ritz vectors also move SCF
    trajectories: with 8 sweeps the Anderson-mixed A-grid dry run no longer converges within
    the reference run's step budget, so the default stays at 4.  Two sweeps stall the
    eigensolver, and omega = 0.9 diverges."""

    def __init__(self, op: "DeviceOperator", sigma: float = 1.0, omega: float = 0.7, sweeps: int = 4):
        self.op, self.sigma, self.omega, self.sweeps = op, float(sigma), float(omega), int(sweeps)
        d = kinetic_diagonal(op.dg, op.closure, op.dtype)
        self.dinv = (1.0 / torch.clamp(d + self.sigma, min=1.0e-3 * self.sigma)).contiguous()

    def __call__(self, r: torch.Tensor, out: torch.Tensor, work: torch.Tensor) -> torch.Tensor:
        k, n = r.shape
        dt = _lib.IGD_F32 if r.dtype == torch.float32 else _lib.IGD_F64
        st = stream_ptr()
        _lib.check(_lib.call("igd_precond_jacobi", dt, n, k, ptr(r), r.stride(0), ptr(out), out.stride(0), None, 0,
                             ptr(self.dinv), self.sigma, self.omega, 1, st), "igd_precond_jacobi")
        for _ in range(self.sweeps - 1):
            hpsi_device(self.op.dg, out, closure=self.op.closure, kscale=-0.5, out=work)
            _lib.check(_lib.call("igd_precond_jacobi", dt, n, k, ptr(r), r.stride(0), ptr(out), out.stride(0),
                                 ptr(work), work.stride(0), ptr(self.dinv), self.sigma, self.omega, 0, st),
                       "igd_precond_jacobi")
        return out


def _whiten_truncated(M: np.ndarray, scale: float, rel: float) -> np.ndarray:
    """Columns V_r / sqrt(e_r) over the eigenpairs of M with e_r > rel * scale.

    M is the Gram matrix of the W-projected residual block, formed on the host as
    R^T W R - (B^T W R)^T G1; directions whose projected norm is lost in that
    subtraction are dropped instead of amplified (the reference falls back to a
    QR of the projected block, ``eigensolver_jax.py:119-146``)."""

    ev, V = np.linalg.eigh(_sym(M))
    keep = ev > rel * max(scale, 1e-300)
    return V[:, keep] / np.sqrt(ev[keep])[None, :]


def _right_eig(M: np.ndarray):
    """Eigenpairs of a real non-symmetric matrix by ascending real part (real parts kept; the
    wanted low states of these near-symmetric projections are real)."""

    ev, Vc = np.linalg.eig(M)
    order = np.argsort(ev.real, kind="stable")
    return ev.real[order], Vc[:, order]


def _unit_columns(V: np.ndarray) -> np.ndarray:
    """Columns scaled to unit length (a column that is numerically zero, the real part of a
    purely imaginary eigenvector, is left as it is)."""

    return V / np.maximum(np.linalg.norm(V, axis=0), 1e-300)[None, :]


def _right_span(M: np.ndarray, m: int) -> np.ndarray:
    """Orthonormal basis of the invariant subspace of the m eigenvalues of M with the lowest
    real parts (real and imaginary parts of complex eigenvectors both kept)."""

    _, Vc = _right_eig(M)
    sel = Vc[:, :m]
    cols = [sel.real] + ([sel.imag[:, np.any(np.abs(sel.imag) > 0.0, axis=0)]] if np.iscomplexobj(sel) else [])
    Q, _ = np.linalg.qr(np.concatenate(cols, axis=1))
    return Q[:, :m]


def subspace_host_step_numpy(G0: np.ndarray, G1: np.ndarray, m: int, k: int, cut: float, right: bool = False):
    """Host algebra of one fused iteration from the Gram matrices G0 = [B;R]^T W [HB;HR] and
    G1 = [B;R]^T W [B;R]: returns (coeff, P, lam, V) with coeff = [CB; CR; V_k; -V_k diag(lam_k)]
    flattened (this iteration's two-part rotation, the next iteration's residual coefficients).
    ``right``: Rayleigh-Ritz on the projected matrices as they are (right eigenpairs)
    instead of their symmetric parts."""

    BHB, BHR, RHB, RHR = G0[:m, :m], G0[:m, m:], G0[m:, :m], G0[m:, m:]
    GB, BR, RR = G1[:m, :m], G1[:m, m:], G1[m:, m:]
    # W-projection of R against B and whitening: R' = (R - B G1m) T
    G1m = np.linalg.solve(_sym(GB), BR)
    T = _whiten_truncated(RR - BR.T @ G1m, float(np.max(np.diag(RR))), cut)
    r = T.shape[1]
    # trial Rayleigh-Ritz on [B R'] with H[B R'] = [HB (HR - HB G1m) T]
    BHRp = (BHR - BHB @ G1m) @ T
    RpHB = T.T @ (RHB - G1m.T @ BHB)
    RpHRp = T.T @ (RHR - RHB @ G1m - G1m.T @ BHR + G1m.T @ BHB @ G1m) @ T
    Tns = np.block([[BHB, BHRp], [RpHB, RpHRp]])
    if right:
        W1 = _right_span(Tns, m)
    else:
        _, Wt = np.linalg.eigh(_sym(Tns))
        W1 = Wt[:, :m]
    # re-whitening of the compressed basis (its Gram from the fresh B^T W B)
    S = np.zeros((m + r, m + r))
    S[:m, :m] = _sym(GB)
    S[m:, m:] = np.eye(r)
    Tb = _chol_whitening(W1.T @ S @ W1)
    CB = (W1[:m] - G1m @ T @ W1[m:]) @ Tb
    CR = (T @ W1[m:]) @ Tb
    P = Tb.T @ (W1.T @ Tns @ W1) @ Tb
    if right:
        lam, Vc = _right_eig(P)
        V = _unit_columns(Vc.real)
    else:
        P = _sym(P)
        lam, V = np.linalg.eigh(P)
    coeff = np.concatenate([CB.ravel(), CR.ravel(), V[:, :k].ravel(), (-V[:, :k] * lam[None, :k]).ravel()])
    return coeff, P, lam, V


class _HostStepBuffers:
    """Output arrays of the native host step, reused across the iterations of one solve
    (their addresses are fixed once; each iteration's results are consumed before the next
    call overwrites them)."""

    def __init__(self, m: int, k: int):
        self.coeff = np.empty((m + k) * m + 2 * m * k)
        self.P, self.V, self.lam, self.rank = np.empty((m, m)), np.empty((m, m)), np.empty(m), ctypes.c_int(0)
        self.ptrs = (self.coeff.ctypes.data, self.P.ctypes.data, self.lam.ctypes.data, self.V.ctypes.data,
                     ctypes.byref(self.rank))


def subspace_host_step(G0: np.ndarray, G1: np.ndarray, m: int, k: int, cut: float, right: bool = False,
                       bufs: _HostStepBuffers | None = None):
    """:func:`subspace_host_step_numpy` in one native call (``igd_subspace_step_host``) for
    blocks of up to 16 columns (its Jacobi eigensolver is slower than LAPACK beyond that);
    the NumPy form for larger blocks, for right Ritz pairs, or if the native step reports a
    numerical failure.  ``bufs``: reused output arrays (the returned arrays are then those
    buffers, valid until the next call with them)."""

    if right:
        return subspace_host_step_numpy(G0, G1, m, k, cut, right=True)
    if m + k <= 16:
        G0 = np.ascontiguousarray(G0, dtype=np.float64)
        G1 = np.ascontiguousarray(G1, dtype=np.float64)
        b = bufs if bufs is not None else _HostStepBuffers(m, k)
        st = _lib.call("igd_subspace_step_host", m, k, G0.ctypes.data, G1.ctypes.data, float(cut), *b.ptrs)
        if st == _lib.IGD_OK:
            return b.coeff, b.P, b.lam, b.V
    return subspace_host_step_numpy(G0, G1, m, k, cut)


def block_subspace_iteration_fused(op: DeviceOperator, case, k: int, **kw):
    """See :func:`_block_subspace_iteration_fused` (runs with the stream resolved once)."""

    from .device import held_stream

    with held_stream():
        return _block_subspace_iteration_fused(op, case, k, **kw)


def _block_subspace_iteration_fused(op: DeviceOperator, case, k: int, *, max_iterations: int = 400,
                                   tolerance: float = 1.0e-3, initial_guess=None, initial_subspace_size=None,
                                   ncv=None, default_guess: torch.Tensor | None = None,
                                   stall_iterations: int | None = None, preconditioner=None,
                                   block: int | None = None, graphs: bool = True, ritz: str = "symmetric"):
    """The block iteration of ``eigensolver_jax.py:417-524`` with one host round trip per iteration.

    ``preconditioner`` (e.g. :class:`JacobiPreconditioner`) maps the residual
    block before it expands the subspace (a Davidson-type expansion; the
    converged Ritz pairs are the same, the iteration count drops); residual
    norms are always those of the raw residual.

    Each iteration forms R = HB V_k - B V_k diag(lambda_k) and HR = H R on the
    device, then two fused Gram products [B; R]^T W [HB; HR] and
    [B; R]^T W [B; R] (one copy to the host).  The residual norms, the W-projection
    of R against B, its whitening, the (m+k)^2 trial Rayleigh-Ritz matrix, the
    compression to m columns and the re-whitening are then small host matrix
    products; B and H B advance by one two-part rotation each (projection and
    whitening are linear maps, so H of the processed residual block is the same
    map applied to H R).  The subspace sequence is the reference's; only the
    order of the linear algebra differs."""

    if k <= 0:
        raise ValueError(f"k must be positive; received {k}.")
    if max_iterations <= 0:
        raise ValueError(f"max_iterations must be positive; received {max_iterations}.")
    if tolerance <= 0.0:
        raise ValueError(f"tolerance must be positive; received {tolerance}.")
    dg, geom, dt = op.dg, op.geom, op.dtype
    dev, n = dg.device, dg.n
    la = BlockLA(dg)
    # ``block`` overrides the reference's working-block rule (used with a
    # preconditioned expansion, which needs far fewer than 12k + 8 columns)
    m = max(int(block), k + 1) if block else block_size(k, initial_subspace_size, ncv)
    target = max(k, m)
    guess = default_guess[:target] if default_guess is not None and default_guess.shape[0] >= target else \
        default_guess_device(case, geom, dg, target)
    if initial_guess is not None:
        if isinstance(initial_guess, torch.Tensor):
            user = initial_guess.to(device=dev, dtype=torch.float64).reshape(-1, n)
        else:
            user = torch.as_tensor(np.ascontiguousarray(validate_orbital_block(initial_guess, geom), dtype=np.float64),
                                   device=dev).reshape(-1, n)
        comb = orthonormalize_device(la, torch.cat([user, guess]), require_full_rank=False)
        if comb.shape[0] < k:
            raise ValueError("The provided initial guesses do not span enough weighted-independent directions.")
        guess = comb[:target]
    guess = guess[:m].contiguous()
    mk = m + k
    la = BlockLA(dg)
    up = _Uploader(dev, 2 * mk * mk)
    # ping-pong buffers: X = [B; R], Y = [H B; H R]
    X = [torch.empty((mk, n), dtype=dt, device=dev) for _ in range(2)]
    Y = [torch.empty((mk, n), dtype=dt, device=dev) for _ in range(2)]
    X0 = guess.to(dt)
    la.rotate(X0, _dev64(np.linalg.inv(np.linalg.cholesky(_sym(la.gram(X0, X0).cpu().numpy()))).T, dev),
              out=X[0][:m])
    op(X[0][:m], out=Y[0][:m])
    right = ritz == "right"
    P = la.gram(X[0][:m], Y[0][:m]).cpu().numpy()
    P = P if right else _sym(P)
    G = torch.empty((3, mk, mk), dtype=torch.float64, device=dev)
    Rraw = torch.empty((k, n), dtype=dt, device=dev) if preconditioner is not None else None
    Rwork = torch.empty((k, n), dtype=dt, device=dev) if preconditioner is not None else None
    # fixed coefficient buffers and Gram workspace: the graph-replayed stages read them
    dco = torch.empty(mk * m + 2 * m * k, dtype=torch.float64, device=dev)
    dcc, dcR = dco[: mk * m].view(mk, m), dco[mk * m:].view(2 * m, k)  # one upload fills both
    gws = torch.empty(int(_lib.call("igd_block_gram_workspace_bytes", n, mk, mk)) + 256, dtype=torch.uint8,
                      device=dev)
    # per-iteration host traffic without allocations: the Gram matrices come back into a
    # pinned buffer, the coefficients go up to a fixed address on the held stream
    Gpin = torch.empty((3, mk, mk), dtype=torch.float64, pin_memory=True)
    Gnp = Gpin.numpy()
    hbufs = _HostStepBuffers(m, k)
    held = torch.cuda.current_stream(dev)
    held_ptr, dco_ptr = stream_ptr(), dco.data_ptr()

    def stage_a(c, lin):
        """R = HB V_k - B V_k Lambda (preconditioned), H R, and the fused Gram products."""

        Xc, Yc = X[c], Y[c]
        B_, HB_, R_, HR_ = Xc[:m], Yc[:m], Xc[m:], Yc[m:]
        if preconditioner is None:
            lin.rotate(HB_, dcR[:m], B_, dcR[m:], out=R_)
        else:
            lin.rotate(HB_, dcR[:m], B_, dcR[m:], out=Rraw)
            lin.gram(Rraw, Rraw, out=G[2].view(-1)[: k * k].view(k, k))
            preconditioner(Rraw, out=R_, work=Rwork)
        op(R_, out=HR_)
        lin.gram(Xc, Yc, out=G[0])   # [B;R]^T W [HB;HR]
        lin.gram(Xc, Xc, out=G[1])   # [B;R]^T W [B;R]

    def stage_b(c, lin):
        """B, HB of the next iteration by one two-part rotation each."""

        Xc, Yc, nx_ = X[c], Y[c], 1 - c
        lin.rotate(Xc[:m], dcc[:m], Xc[m:], dcc[m:], out=X[nx_][:m])
        lin.rotate(Yc[:m], dcc[:m], Yc[m:], dcc[m:], out=Y[nx_][:m])

    graphs_ok = bool(graphs) and dev.type == "cuda"
    gA, gB = {}, {}

    def capture():
        """CUDA graphs of both stages for both ping-pong phases (after one eager iteration
        has initialised every kernel); any failure falls back to direct launches."""

        from .device import held_stream

        try:
            for c in (0, 1):
                for store, fn in ((gA, stage_a), (gB, stage_b)):
                    g_ = torch.cuda.CUDAGraph()
                    with torch.cuda.graph(g_, capture_error_mode="thread_local"):
                        with held_stream():
                            fn(c, BlockLA(dg, workspace=gws))
                    store[c] = g_
            return True
        except Exception:
            gA.clear()
            gB.clear()
            return False

    lin0 = BlockLA(dg, workspace=gws)
    cur = 0
    res_hist, ritz_hist, dims = [], [], []
    converged, stalled = False, False
    best_rn, best_it = np.inf, 0
    it = 0
    eig, rn, ritz_mat = np.zeros(k), np.full(k, np.inf), np.zeros((k, k))
    if right:
        lam, Vc = _right_eig(P)
        V = _unit_columns(Vc.real)
    else:
        lam, V = np.linalg.eigh(P)
    cut = 1.0e-10 if dt == torch.float64 else 1.0e-5
    up([V[:, :k], -V[:, :k] * lam[None, :k]], dst=dcR)
    for it in range(1, max_iterations + 1):
        eig, ritz_mat = lam[:k].copy(), P[:k, :k].copy()
        if cur in gA:
            gA[cur].replay()
            op.applies += k
        else:
            stage_a(cur, lin0)
        Gpin.copy_(G, non_blocking=True)
        held.synchronize()
        Gh = Gnp
        BHB, BHR, RHB, RHR = Gh[0][:m, :m], Gh[0][:m, m:], Gh[0][m:, :m], Gh[0][m:, m:]
        GB, BR, RR = Gh[1][:m, :m], Gh[1][:m, m:], Gh[1][m:, m:]
        RRraw = RR if preconditioner is None else Gh[2].reshape(-1)[: k * k].reshape(k, k)
        rn = np.sqrt(np.clip(np.diag(RRraw), 0.0, None))
        res_hist.append(rn)
        ritz_hist.append(eig)
        dims.append(m)
        if float(rn.max()) <= tolerance:
            converged = True
            break
        if stall_iterations:
            cr = float(rn.max())
            if cr < best_rn * (1.0 - 1.0e-2):
                best_rn, best_it = cr, it
            elif it - best_it >= stall_iterations and len(ritz_hist) > stall_iterations:
                drift = float(np.max(np.abs(ritz_hist[-1] - ritz_hist[-1 - stall_iterations])))
                if drift <= 1.0e-12 * max(1.0, float(np.max(np.abs(ritz_hist[-1])))):
                    stalled = True
                    break
        coeff, P, lam, V = subspace_host_step(Gh[0], Gh[1], m, k, cut, right=right, bufs=hbufs)
        up.flat(coeff, dco_ptr, held_ptr)
        if cur in gB:
            gB[cur].replay()
        else:
            stage_b(cur, lin0)
        cur = 1 - cur
        if it == 1 and graphs_ok:
            graphs_ok = capture()
    B = X[cur][:m]
    Xk = la.rotate(B, _dev64(V[:, :k], dev))
    overlap = la.gram(Xk, Xk).cpu().numpy()
    return {
        "eigenvalues": eig, "orbitals": Xk, "converged": converged, "iteration_count": it, "residual_norms": rn,
        "residual_history": np.asarray(res_hist), "ritz_value_history": np.asarray(ritz_hist),
        "subspace_dimensions": tuple(dims), "weighted_overlap": overlap,
        "max_orthogonality_error": float(np.max(np.abs(overlap - np.eye(k)))), "ritz_matrix": ritz_mat,
        "initial_guess": guess, "final_basis": B.clone(), "stalled": stalled,
    }
