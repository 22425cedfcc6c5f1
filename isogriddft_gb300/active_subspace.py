"""Active-subspace tracking of the closed-shell H2 singlet's occupied orbital.

Device counterpart of ``scf/active_subspace.py`` (same dataclasses, field names, rules and
verdict texts).  The monitor-grid dry run of the reference turns it on by default for the H2
singlet (``scf/driver.py:3437-3447``, ``:3823-3867``): each SCF step solves the lowest two
orbitals, and the occupied orbital is the previous one carried into their span rather than
the lowest eigenvector, so the occupied direction stays continuous when the two lowest
states rotate into each other.

One step (``update_active_subspace``, ``active_subspace.py:225-301``):

* the stored reference subspace is projected onto the span of the new raw block and
  weighted-orthonormalised (the aligned subspace; the raw block where it loses rank);
* the stored occupied orbital is projected onto the aligned subspace and normalised (the
  first aligned orbital where that projection vanishes);
* diagnostics: singular values of the raw/reference overlap, the largest principal angle, the
  projector drift, the occupied overlaps before and after alignment and the internal rotation.

Orbitals are (k, n) device tensors; every weighted inner product is one FP64 Gram of the
library (``igd_block_gram``) read back as a k x k matrix, and projections are elementwise
combinations of the rows.  Weighted orthonormalisation follows the reference's SVD of
sqrt(W) X (``ks/eigensolver.py:292-341``) through the eigendecomposition of the k x k Gram:
the same singular values, rank cut and span; singular vectors are fixed only up to sign,
so orbitals may differ from the reference's in sign (densities and diagnostics do not).
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np
import torch


@dataclass(frozen=True)
class ActiveSubspaceConfig:
    """``active_subspace.py:19-37``."""

    enabled: bool
    subspace_size: int
    target_occupied_count: int
    only_closed_shell_singlet: bool = True

    @classmethod
    def local_only_h2_singlet_default(cls) -> "ActiveSubspaceConfig":
        return cls(enabled=True, subspace_size=2, target_occupied_count=1, only_closed_shell_singlet=True)


@dataclass(frozen=True)
class ActiveSubspaceState:
    """``active_subspace.py:40-46``; orbitals are (k, n) tensors."""

    config: ActiveSubspaceConfig
    reference_subspace_orbitals: torch.Tensor
    reference_occupied_orbitals: torch.Tensor


@dataclass(frozen=True)
class ActiveSubspaceSelectionResult:
    """``active_subspace.py:49-62``."""

    state: ActiveSubspaceState
    raw_subspace_orbitals: torch.Tensor
    aligned_subspace_orbitals: torch.Tensor
    occupied_orbitals: torch.Tensor
    raw_occupied_overlap_abs: float | None
    best_in_subspace_occupied_overlap_abs: float | None
    internal_rotation_angle_deg: float | None
    projector_drift_frobenius_norm: float | None
    subspace_overlap_singular_values: tuple[float, ...]
    subspace_rotation_max_angle_deg: float | None
    verdict: str


@dataclass(frozen=True)
class MonitorGridActiveSubspaceIterationDiagnostics:
    """One SCF step's tracking snapshot in the dry-run result (``scf/driver.py:322-335``)."""

    iteration: int
    subspace_size: int
    target_occupied_count: int
    raw_occupied_overlap_abs: float | None
    best_in_subspace_occupied_overlap_abs: float | None
    internal_rotation_angle_deg: float | None
    projector_drift_frobenius_norm: float | None
    subspace_rotation_max_angle_deg: float | None
    lowest_gap_ha: float | None
    verdict: str


def _validate_config(config: ActiveSubspaceConfig) -> None:
    """``active_subspace.py:65-71`` (same messages)."""

    if config.subspace_size <= 0:
        raise ValueError("subspace_size must be positive.")
    if config.target_occupied_count <= 0:
        raise ValueError("target_occupied_count must be positive.")
    if config.target_occupied_count > config.subspace_size:
        raise ValueError("target_occupied_count must not exceed subspace_size.")


def _prefix(orbitals: torch.Tensor, count: int) -> torch.Tensor:
    if orbitals.shape[0] < count:
        raise ValueError(f"At least {count} orbitals are required; received {orbitals.shape[0]}.")
    return orbitals[:count].contiguous()


def weighted_gram(A: torch.Tensor, B: torch.Tensor, w: torch.Tensor) -> np.ndarray:
    """<A_i|B_j> = sum_p A_i B_j W_p in FP64 as a host (a, b) matrix: one ``igd_block_gram`` on
    the device; host tensors (tests) take the same product on the CPU."""

    if not A.is_cuda:
        return ((A.double() * w) @ B.double().T).numpy()
    from . import _lib
    from .device import ptr, stream_ptr

    A, B = A.contiguous(), B.contiguous()
    if B.dtype != A.dtype:
        B = B.to(A.dtype)
    n, a, b = int(w.numel()), A.shape[0], B.shape[0]
    dt = _lib.IGD_F32 if A.dtype == torch.float32 else _lib.IGD_F64
    out = torch.empty((a, b), dtype=torch.float64, device=A.device)
    wsb = int(_lib.call("igd_block_gram_workspace_bytes", n, a, b))
    ws = torch.empty(max(wsb, 1), dtype=torch.uint8, device=A.device)
    _lib.check(_lib.call("igd_block_gram", dt, n, a, ptr(A), n, b, ptr(B), n, ptr(w), ptr(out), 0, ptr(ws), wsb,
                         stream_ptr()), "igd_block_gram")
    return out.cpu().numpy()


def _combine(C: np.ndarray, X: torch.Tensor) -> torch.Tensor:
    """Rows out_j = sum_i C[j, i] X_i (elementwise updates; no small-dimension GEMM)."""

    rows = []
    for j in range(C.shape[0]):
        acc = float(C[j, 0]) * X[0]
        for i in range(1, X.shape[0]):
            acc = acc.add(X[i], alpha=float(C[j, i]))
        rows.append(acc)
    if not rows:
        return X[:0].clone()
    return torch.stack(rows).contiguous()


def weighted_orthonormalize(X: torch.Tensor, w: torch.Tensor, rank_tolerance: float = 1.0e-12) -> torch.Tensor:
    """Orthonormal basis of span(X) in the W metric, ordered by decreasing singular value of
    sqrt(W) X, rank cut at ``rank_tolerance * max(n, k) * s_0`` (``ks/eigensolver.py:292-341``
    with ``require_full_rank=False``); zero rows when nothing is left."""

    if X.shape[0] == 0:
        return X.clone()
    G = weighted_gram(X, X, w)
    ev, V = np.linalg.eigh(0.5 * (G + G.T))
    ev, V = ev[::-1], V[:, ::-1]
    s = np.sqrt(np.clip(ev, 0.0, None))
    if s[0] == 0.0:
        return X[:0].clone()
    rank = int(np.sum(s > rank_tolerance * max(int(w.numel()), X.shape[0]) * s[0]))
    if rank == 0:
        return X[:0].clone()
    return _combine((V[:, :rank] / s[:rank]).T, X)


def _project(reference: torch.Tensor, current: torch.Tensor, w: torch.Tensor) -> torch.Tensor:
    """``active_subspace.py:84-104``: each reference orbital's expansion on ``current``,
    weighted-orthonormalised without requiring full rank."""

    overlaps = weighted_gram(current, reference, w)          # (k_current, k_reference)
    return weighted_orthonormalize(_combine(overlaps.T, current), w)


def _min_singular(M: np.ndarray) -> float:
    return float(np.min(np.clip(np.linalg.svd(np.asarray(M, dtype=np.float64), compute_uv=False), 0.0, 1.0)))


def initialize_active_subspace(*, raw_subspace_orbitals: torch.Tensor, config: ActiveSubspaceConfig,
                               weights: torch.Tensor | None = None) -> ActiveSubspaceSelectionResult:
    """``active_subspace.py:179-222``: the raw lowest block becomes the reference."""

    _validate_config(config)
    raw = _prefix(raw_subspace_orbitals, config.subspace_size)
    occupied = raw[: config.target_occupied_count].clone()
    return ActiveSubspaceSelectionResult(
        state=ActiveSubspaceState(config, raw.clone(), occupied),
        raw_subspace_orbitals=raw, aligned_subspace_orbitals=raw, occupied_orbitals=occupied,
        raw_occupied_overlap_abs=1.0, best_in_subspace_occupied_overlap_abs=1.0, internal_rotation_angle_deg=0.0,
        projector_drift_frobenius_norm=0.0, subspace_overlap_singular_values=(1.0,) * config.subspace_size,
        subspace_rotation_max_angle_deg=0.0,
        verdict="Initialized active-subspace tracking from the current raw subspace.")


def update_active_subspace(*, raw_subspace_orbitals: torch.Tensor, state: ActiveSubspaceState,
                           weights: torch.Tensor) -> ActiveSubspaceSelectionResult:
    """``active_subspace.py:225-301``: align the stored reference to the new raw block."""

    config = state.config
    _validate_config(config)
    w = weights
    raw = _prefix(raw_subspace_orbitals, config.subspace_size)
    ref_sub, ref_occ = state.reference_subspace_orbitals, state.reference_occupied_orbitals
    # principal angles between the raw block and the reference subspace (:107-127)
    sv = np.clip(np.linalg.svd(weighted_gram(raw, ref_sub, w), compute_uv=False), 0.0, 1.0)
    max_angle = float(np.degrees(np.arccos(float(np.min(sv)))))
    drift = float(np.sqrt(max(0.0, 2.0 * float(np.sum(1.0 - sv * sv)))))
    aligned = _project(ref_sub, raw, w)
    aligned = raw if aligned.shape[0] < config.subspace_size else aligned[: config.subspace_size].contiguous()
    projected = _project(ref_occ, aligned, w)
    t = config.target_occupied_count
    occupied = (aligned[:t] if projected.shape[0] < t else projected[:t]).contiguous()
    # occupied overlaps before and after alignment, and the rotation inside the subspace (:130-176)
    c = ref_occ.shape[0]
    raw_abs = _min_singular(weighted_gram(raw[:c], ref_occ, w))
    best_abs = _min_singular(weighted_gram(occupied, ref_occ, w))
    internal = float(np.degrees(np.arccos(_min_singular(weighted_gram(occupied, raw[:c], w)))))
    if best_abs >= 0.95 and raw_abs <= 0.2 and internal >= 45.0:
        verdict = ("The reference occupied direction stays inside the current active subspace, "
                   "but the raw basis rotates strongly inside that subspace.")
    elif best_abs <= 0.2:
        verdict = ("The reference occupied direction is no longer well represented by the current "
                   "active subspace; the subspace size may be too small.")
    else:
        verdict = "The active subspace remains locally continuous under this update."
    return ActiveSubspaceSelectionResult(
        state=ActiveSubspaceState(config, aligned, occupied), raw_subspace_orbitals=raw,
        aligned_subspace_orbitals=aligned, occupied_orbitals=occupied, raw_occupied_overlap_abs=raw_abs,
        best_in_subspace_occupied_overlap_abs=best_abs, internal_rotation_angle_deg=internal,
        projector_drift_frobenius_norm=drift, subspace_overlap_singular_values=tuple(float(v) for v in sv),
        subspace_rotation_max_angle_deg=max_angle, verdict=verdict)
