"""H2 bond-length scan: many independent single-point SCFs on the GPU.

Each geometry gets its own A-grid (monitor generator on the device), its own
device-resident SCF (``scf.run_scf_device``) and its own timing; geometries are
independent, so a multi-GPU run would hand whole geometries to each GPU
(replicas).  The scan definition follows the bond-length study the reference
runs one geometry at a time: R evenly spaced, singlets and triplets
alternating, grid edges drawn from a seeded generator.

    python -m isogriddft_gb300.scan --count 64 --precision mixed [--workers 4]
"""

from __future__ import annotations

import argparse
import json
import threading
import time
from dataclasses import dataclass

import numpy as np
import torch

from .config import make_h2_case
from .grid import build_h2_local_patch_development_element_parameters, build_monitor_grid_for_case
from .scf import run_scf_device


@dataclass(frozen=True)
class ScanPoint:
    bond_length: float
    spin: str
    shape: tuple


@dataclass(frozen=True)
class ScanResult:
    point: ScanPoint
    precision: str
    converged: bool
    scf_iterations: int
    energy: float
    eigenvalues_up: tuple
    grid_seconds: float
    scf_seconds: float


def scan_points(count: int = 64, r_min: float = 1.0, r_max: float = 3.0, edge_min: int = 64, edge_max: int = 128,
                seed: int = 3, edge_multiple: int = 4) -> list:
    """Even-spaced bond lengths, singlet at even and triplet at odd index, seeded grid edges.

    Edges are rounded to ``edge_multiple`` so rows stay 16-byte aligned for the
    TMA stencil."""

    rng = np.random.default_rng(seed)
    pts = []
    for i, r in enumerate(np.linspace(r_min, r_max, count)):
        e = rng.integers(edge_min, edge_max + 1, size=3)
        e = tuple(int(max(edge_min, (x // edge_multiple) * edge_multiple)) for x in e)
        pts.append(ScanPoint(float(r), "singlet" if i % 2 == 0 else "triplet", e))
    return pts


def run_point(p: ScanPoint, *, precision: str = "mixed", bands: int = 4, energy_tolerance: float = 1.0e-6,
              density_tolerance: float = 1.0e-4, eigensolver_tolerance: float = 1.0e-4, max_iterations: int = 60,
              box_half_extents=(8.0, 8.0, 10.0), eigensolver_graphs: bool = True) -> ScanResult:
    """One geometry on the calling thread's current stream (timed with that stream's syncs)."""

    case = make_h2_case(p.bond_length)
    st = torch.cuda.current_stream()
    st.synchronize()
    t0 = time.perf_counter()
    geom = build_monitor_grid_for_case(case, shape=p.shape, box_half_extents=box_half_extents,
                                       element_parameters=build_h2_local_patch_development_element_parameters(),
                                       device=True)
    st.synchronize()
    t1 = time.perf_counter()
    r = run_scf_device(case, geom, p.spin, precision=precision, max_iterations=max_iterations, mixing=0.35,
                       density_tolerance=density_tolerance, energy_tolerance=energy_tolerance,
                       eigensolver_tolerance=eigensolver_tolerance, mixer="diis", kinetic_version="trial_fix",
                       local_only_energy=True, poisson_tolerance=1e-10, poisson_max_iterations=2000,
                       record_fields=False, bands=bands, adaptive_eigensolver_tolerance=0.1,
                       poisson_warm_start=True, eigensolver_graphs=eigensolver_graphs)
    st.synchronize()
    t2 = time.perf_counter()
    return ScanResult(p, precision, bool(r.converged), r.iteration_count, float(r.energy.total),
                      tuple(float(v) for v in r.eigenvalues_up), t1 - t0, t2 - t1)


def run_scan(points, *, workers: int = 1, **kw) -> list:
    """All geometries, one at a time (``workers`` = 1) or ``workers`` at a time.

    Concurrent geometries run on host threads, each with its own CUDA stream:
    one SCF leaves the GPU idle while its host does the small Rayleigh-Ritz
    algebra and reads results back, and the other geometries' kernels fill those
    gaps.  Every device buffer, staging slot and held stream is per geometry or
    per thread; the eigensolver's CUDA-graph replay is off in this mode (a graph
    capture must not overlap other threads' allocations)."""

    points = list(points)
    if workers <= 1:
        return [run_point(p, **kw) for p in points]
    from concurrent.futures import ThreadPoolExecutor

    dev = torch.cuda.current_device()
    local = threading.local()

    def one(p):
        if not hasattr(local, "stream"):
            torch.cuda.set_device(dev)
            local.stream = torch.cuda.Stream(device=dev)
        with torch.cuda.stream(local.stream):
            return run_point(p, eigensolver_graphs=False, **kw)

    with ThreadPoolExecutor(max_workers=workers) as ex:
        return list(ex.map(one, points))


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--count", type=int, default=64)
    ap.add_argument("--precision", default="mixed")
    ap.add_argument("--bands", type=int, default=4)
    ap.add_argument("--workers", type=int, default=1, help="geometries solved concurrently (host threads)")
    args = ap.parse_args(argv)
    pts = scan_points(args.count)
    t0 = time.perf_counter()
    for res in run_scan(pts, precision=args.precision, bands=args.bands, workers=args.workers):
        print(json.dumps({"R": res.point.bond_length, "spin": res.point.spin, "shape": res.point.shape,
                          "converged": res.converged, "iterations": res.scf_iterations, "energy": res.energy,
                          "grid_s": round(res.grid_seconds, 3), "scf_s": round(res.scf_seconds, 3)}), flush=True)
    from .ops import autotune_report

    print(json.dumps({"geometries": len(pts), "workers": args.workers, "wall_s": round(time.perf_counter() - t0, 3),
                      "autotune": autotune_report()}), flush=True)


if __name__ == "__main__":
    main()
