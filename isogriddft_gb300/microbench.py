"""Per-kernel timings on the 128^3 A-grid workload (CUDA events, inputs larger than L2).

    python -m isogriddft_gb300.microbench [--reps N] [--only SECTIONS] [--shape NX NY NZ]

Prints one JSON line per kernel: milliseconds per launch, algorithmic bytes per
launch (each array counted once per pass) and the achieved GB/s.  Workloads:
LSDA on a two-spin density (FP64 data), the density build of 16 FP32 orbitals,
the weighted Gram matrix and the two-part rotation of the eigensolver (FP32
blocks of 16 and 32 columns), one BiCGSTAB solve (mixed precision) split into
its stencil and vector kernels by the solver's own iteration count, and the
H.Psi apply itself (the Poisson operator on one orbital and 16 orbitals with
v_eff, trial fix and production closure; ``hpsipaths`` times the one-orbital
Poisson operator and the 16-orbital trial-fix apply on each kernel: whole-row,
tiled TMA, cp.async; ``bicgstabpaths`` the fused and the unfused mixed
BiCGSTAB iteration).  ``--shape``
runs the same workloads on another grid (192^3 and 160^3 are the C6H6 and
force-check grids, whose rows the whole-row kernel covers with two chunks per
lane).
"""

from __future__ import annotations

import argparse
import json

import torch

from . import _lib
from .config import H2_BENCHMARK_CASE
from .device import device_grid, ptr, stream_ptr
from .grid import build_monitor_grid_for_case, build_two_peak_element_parameters

SHAPE = (128, 128, 128)


def _timed(fn, reps: int) -> float:
    for _ in range(3):
        fn()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(reps):
        fn()
    b.record()
    torch.cuda.synchronize()
    return a.elapsed_time(b) / reps


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--reps", type=int, default=20)
    ap.add_argument("--only", default="", help="comma-separated subset of " + ",".join(SECTIONS)
                    + " (for profiling one kernel)")
    ap.add_argument("--shape", type=int, nargs=3, default=SHAPE)
    args = ap.parse_args(argv)
    for rec in run(args.reps, only=[x for x in args.only.split(",") if x] or None, shape=tuple(args.shape)):
        print(json.dumps(rec), flush=True)
    print(json.dumps({"note": "FP32 data unless noted; bytes count each array once per pass"}), flush=True)


SECTIONS = ("lsda", "density", "gram16", "rotate16", "gram32", "rotate32", "bicgstab", "bicgstabpaths", "hpsi1",
            "hpsi16", "hpsi16prod", "hpsi16fp64", "hpsipaths")


def run(reps: int = 20, only=None, shape=SHAPE) -> list:
    """One record per kernel: milliseconds per launch, algorithmic bytes, GB/s (and TFLOP/s).
    ``only``: a subset of ``SECTIONS`` to run."""

    bad = set(only or ()) - set(SECTIONS)
    if bad:
        raise ValueError(f"unknown sections {sorted(bad)}; choose from {SECTIONS}")

    def want(name):
        return only is None or name in only

    records = []
    geom = build_monitor_grid_for_case(H2_BENCHMARK_CASE, shape=tuple(shape), box_half_extents=(8.0, 8.0, 10.0),
                                       element_parameters=build_two_peak_element_parameters(("H",), 4.0, 0.5),
                                       device=True)
    dg = device_grid(geom)
    st = stream_ptr()
    g = torch.Generator(device=dg.device).manual_seed(0)

    def line(name, ms, nbytes, **extra):
        records.append({"kernel": name, "ms": round(ms, 5), "alg_bytes": int(nbytes),
                        "gbs": round(nbytes / (ms * 1e-3) / 1e9, 1), **extra})

    if want("lsda"):
        _lsda(dg, g, st, reps, line)
    if want("density"):
        _density(dg, g, st, reps, line)
    for a in (16, 32):
        if want(f"gram{a}") or want(f"rotate{a}"):
            _gram_rotate(dg, g, st, reps, line, a, want(f"gram{a}"), want(f"rotate{a}"))
    if want("bicgstab"):
        _bicgstab(dg, geom, reps, line)
    if want("bicgstabpaths"):
        try:
            for path, name in ((0, "fused"), (1, "unfused")):
                _lib.check(_lib.call("igd_poisson_select", path), "igd_poisson_select")
                _bicgstab(dg, geom, reps, line, name)
        finally:
            _lib.call("igd_poisson_select", 0)
    if any(want(x) for x in ("hpsi1", "hpsi16", "hpsi16prod", "hpsipaths")):
        _hpsi(dg, g, reps, line, want("hpsi1"), want("hpsi16"), want("hpsi16prod"), want("hpsipaths"))
    if want("hpsi16fp64"):
        _hpsi_fp64(dg, g, reps, line)
    return records


def _lsda(dg, g, st, reps, line):
    # LSDA: rho_up, rho_down in; eps, v_up, v_down, energy density out; FP64 energy sum
    n, dev = dg.n, dg.device
    up = torch.rand(n, device=dev, dtype=torch.float64, generator=g) ** 3
    dn = torch.rand(n, device=dev, dtype=torch.float64, generator=g) ** 3
    outs = [torch.empty_like(up) for _ in range(4)]
    en = torch.zeros(1, dtype=torch.float64, device=dev)
    fl = torch.zeros(1, dtype=torch.int32, device=dev)
    ms = _timed(lambda: _lib.call("igd_lsda", _lib.IGD_F64, _lib.IGD_F64, 0, n, ptr(up), ptr(dn), ptr(outs[0]),
                                  ptr(outs[1]), ptr(outs[2]), ptr(outs[3]), ptr(dg.cell_volumes), ptr(en), ptr(fl),
                                  st), reps)
    line("lsda_kernel<f64> (Slater+VWN5)", ms, n * 8 * (2 + 4 + 1))


def _density(dg, g, st, reps, line):
    # density of 16 FP32 orbitals, FP64 density and integral
    n, dev = dg.n, dg.device
    psi = torch.randn((16, n), device=dev, dtype=torch.float32, generator=g)
    occ = torch.ones(16, dtype=torch.float64, device=dev)
    rho = torch.empty(n, dtype=torch.float64, device=dev)
    integ = torch.zeros(1, dtype=torch.float64, device=dev)
    ms = _timed(lambda: _lib.call("igd_density", _lib.IGD_F32, n, 16, n, ptr(psi), ptr(occ), ptr(dg.cell_volumes),
                                  ptr(rho), ptr(integ), 0, st), reps)
    line("density_kernel<f32> (16 orbitals)", ms, n * (16 * 4 + 8 + 8))


def _gram_rotate(dg, g, st, reps, line, a, gram, rotate):
    # Gram A W B^T and rotation of FP32 blocks
    n, dev = dg.n, dg.device
    A = torch.randn((a, n), device=dev, dtype=torch.float32, generator=g)
    B = torch.randn((a, n), device=dev, dtype=torch.float32, generator=g)
    if gram:
        out = torch.empty((a, a), dtype=torch.float64, device=dev)
        wsb = int(_lib.call("igd_block_gram_workspace_bytes", n, a, a))
        ws = torch.empty(wsb, dtype=torch.uint8, device=dev)
        ms = _timed(lambda: _lib.call("igd_block_gram", _lib.IGD_F32, n, a, ptr(A), n, a, ptr(B), n,
                                      ptr(dg.cell_volumes), ptr(out), 0, ptr(ws), wsb, st), reps)
        line(f"igd_block_gram<f32> ({a}x{a})", ms, n * (2 * a * 4 + 8), tflops=round(2 * n * a * a / ms / 1e9, 2))
    if rotate:
        C = torch.randn((a, a), device=dev, dtype=torch.float64, generator=g)
        O = torch.empty((a, n), device=dev, dtype=torch.float32)
        ms = _timed(lambda: _lib.call("igd_block_rotate", _lib.IGD_F32, n, a, ptr(A), n, ptr(C), a, ptr(B), n, ptr(C),
                                      a, ptr(O), n, 0, st), reps)
        line(f"rotate_kernel<f32> ({2 * a}->{a})", ms, n * 3 * a * 4, tflops=round(2 * n * 2 * a * a / ms / 1e9, 2))


def _bicgstab(dg, geom, reps, line, variant=""):
    # BiCGSTAB (mixed) on the Gaussian charge: per-iteration time
    from .poisson import solve_poisson_device

    n = dg.n

    r2 = dg.x * dg.x + dg.y * dg.y + dg.z * dg.z
    q = torch.exp(-0.5 * r2 / 0.64)
    q *= 2.0 / float(torch.sum(q * dg.cell_volumes))
    solve_poisson_device(dg, geom, q, tolerance=1e-10, max_iterations=4000, precision="mixed")
    torch.cuda.synchronize()
    a_, b_ = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a_.record()
    sol = solve_poisson_device(dg, geom, q, tolerance=1e-10, max_iterations=4000, precision="mixed")
    b_.record()
    torch.cuda.synchronize()
    ms = a_.elapsed_time(b_)
    per_it = ms / max(sol.iterations, 1)
    # per iteration: 2 stencil applies (psi 4 B in/out, 7 FP32 geometry values) + 9 FP32 vector passes
    shape = "x".join(str(v) for v in dg.shape)
    line(f"bicgstab iteration (mixed, {shape}{', ' + variant if variant else ''})", per_it, n * (2 * (8 + 28) + 9 * 4), iterations=sol.iterations,
         solve_ms=round(ms, 3))


def _hpsi(dg, g, reps, line, one, sixteen, sixteen_prod=False, paths=False):
    from .ops import hpsi_device

    n, dev = dg.n, dg.device
    if one:
        x = torch.randn((1, n), device=dev, dtype=torch.float32, generator=g)
        y = torch.empty_like(x)
        ms = _timed(lambda: hpsi_device(dg, x, closure="production", kscale=-1.0, out=y), reps)
        line("hpsi_agrid, production, 1 orbital (Poisson operator)", ms, n * (8 + 28))
    if not (sixteen or sixteen_prod or paths):
        return
    # the H.Psi bench workload: 16 FP32 orbitals, v_eff (no L2 flush: per-launch inputs
    # of 134 MB + geometry already exceed the 129 MB L2 when alternated)
    xs = [torch.randn((16, n), device=dev, dtype=torch.float32, generator=g) for _ in range(2)]
    ys = [torch.empty_like(t) for t in xs]
    v32 = torch.randn(n, device=dev, dtype=torch.float32, generator=g)
    it = [0]

    def apply16(closure):
        i = it[0] = it[0] + 1
        hpsi_device(dg, xs[i % 2], closure=closure, kscale=-0.5, veff=v32, out=ys[i % 2])

    nbytes = n * (16 * 8 + 28 + 4)
    if sixteen:
        line("hpsi_agrid, trial fix, 16 orbitals", _timed(lambda: apply16("trial_fix"), reps), nbytes)
    if sixteen_prod:
        line("hpsi_agrid, production, 16 orbitals", _timed(lambda: apply16("production"), reps), nbytes)
    if paths:
        names = ("whole-row", "tiled TMA", "cp.async")
        x1 = xs[0][:1].contiguous()
        y1 = torch.empty_like(x1)
        try:
            for path in (0, 1, 2):
                _lib.check(_lib.call("igd_hpsi_select", path), "igd_hpsi_select")
                tag = f"{names[path]} kernel" + (" (first applicable)" if path == 0 else "")
                line(f"hpsi_agrid, production, 1 orbital, {tag}",
                     _timed(lambda: hpsi_device(dg, x1, closure="production", kscale=-1.0, out=y1), reps),
                     n * (8 + 28))
                line(f"hpsi_agrid, trial fix, 16 orbitals, {tag}", _timed(lambda: apply16("trial_fix"), reps), nbytes)
        finally:
            _lib.call("igd_hpsi_select", 0)


def _hpsi_fp64(dg, g, reps, line):
    """The FP64 trial-fix apply of 16 orbitals (the reference-precision path; FP64 pipe): about
    26 FP64 flops per orbital and point (gradients 3, fluxes 3 x 5, divergence 5, scale 1,
    v psi 2; an FMA counts 2)."""

    from .ops import hpsi_device

    n, dev = dg.n, dg.device
    xs = [torch.randn((16, n), device=dev, dtype=torch.float64, generator=g) for _ in range(2)]
    ys = [torch.empty_like(t) for t in xs]
    v = torch.randn(n, device=dev, dtype=torch.float64, generator=g)
    it = [0]

    def apply16():
        i = it[0] = it[0] + 1
        hpsi_device(dg, xs[i % 2], closure="trial_fix", kscale=-0.5, veff=v, out=ys[i % 2])

    ms = _timed(apply16, reps)
    line("hpsi_agrid FP64, trial fix, 16 orbitals", ms, n * (16 * 16 + 56 + 8),
         fp64_tflops=round(16 * n * 26 / (ms * 1e-3) / 1e12, 3))


if __name__ == "__main__":
    main()
