"""Density mixers of the SCF loop on device densities (FP64).

Each mixer follows the reference's monitor-grid dry-run mixer step by step
(``scf/driver.py``), with the weighted spin-density inner product
<a|b> = sum_p (a_up b_up + a_down b_down) W_p, taken for all pairs of a
history at once as one FP64 Gram of the library (``igd_block_gram``):

* :class:`PulayMixer` - DIIS on the linearly mixed densities
  (``_apply_monitor_grid_density_diis``, ``driver.py:2234-2294``; schedule
  ``:4297-4318``);
* :class:`AndersonMixer` - Anderson on secant differences with collinearity
  filtering, adaptive damping, residual-ratio acceptance, step clipping and an
  optional reset on residual growth (``driver.py:2125-2231``, ``:2297-2545``;
  schedule ``:4319-4400``);
* :class:`BroydenMixer` - the Broyden-like inverse-Jacobian update
  (``driver.py:2548-2651``; schedule ``:4401-4430``).

A mixer is called once per SCF iteration with the linearly mixed densities and
the residuals rho_out - rho_in, and returns the next input densities.  It keeps
the per-iteration diagnostics the reference reports (iterations where the
extrapolation was used, fell back or was rejected, history sizes, damping).

A library FP64 GEMM with two tiny dimensions and a contraction over the grid
(what ``(R * w) @ R.T`` becomes) runs on a handful of thread blocks and can
take hundreds of milliseconds on this part; the library Gram splits the grid
over every SM.
"""

from __future__ import annotations

import numpy as np
import torch


class _Mixer:
    def __init__(self, engine):
        self.e = engine
        self.iteration = 0
        self.used: list[int] = []
        self.fallback: list[int] = []
        self.history_sizes: list[int] = []

    # -- FP64 algebra on (up, down) pairs
    def gram(self, left: list, right: list) -> np.ndarray:
        """<left_i | right_j> for lists of (up, down) pairs, one host read."""

        L = torch.stack([torch.cat([a, b]) for a, b in left]).contiguous()
        R = torch.stack([torch.cat([a, b]) for a, b in right]).contiguous()
        w = self.e.dg.cell_volumes
        w2 = torch.cat([w, w])
        if not L.is_cuda:  # host tensors (tests): the same product on the CPU
            return ((L * w2) @ R.T).numpy()
        from . import _lib
        from .device import ptr, stream_ptr

        n, a, b = int(w2.numel()), L.shape[0], R.shape[0]
        out = torch.empty((a, b), dtype=torch.float64, device=L.device)
        wsb = int(_lib.call("igd_block_gram_workspace_bytes", n, a, b))
        ws = torch.empty(wsb, dtype=torch.uint8, device=L.device)
        _lib.check(_lib.call("igd_block_gram", _lib.IGD_F64, n, a, ptr(L), n, b, ptr(R), n, ptr(w2), ptr(out), 0,
                             ptr(ws), wsb, stream_ptr()), "igd_block_gram")
        return out.cpu().numpy()

    def norm(self, v) -> float:
        return float(np.sqrt(max(float(self.gram([v], [v])[0, 0]), 0.0)))

    @staticmethod
    def combine(coeffs, vectors):
        """sum_i c_i v_i by elementwise updates (no small-dimension GEMM)."""

        out = float(coeffs[0]) * vectors[0]
        for c, v in zip(coeffs[1:], vectors[1:]):
            out = out.add(v, alpha=float(c))
        return out

    def finish(self, up, dn):
        """Clip at zero, reject a non-positive integral, renormalise
        (``driver.py:2277-2294``); None when rejected."""

        occ = self.e.occ
        outs = []
        for rho, target in ((up, occ.n_alpha), (dn, occ.n_beta)):
            if target > 0:
                rho = torch.clamp(rho, min=0.0)
                if float(self.e.wdot(rho).reshape(-1)[0]) <= 0.0:
                    return None
                outs.append(self.e.renormalized(rho, target))
            else:
                outs.append(torch.zeros_like(rho))
        return outs[0], outs[1]


class PulayMixer(_Mixer):
    """DIIS on the linearly mixed spin densities (``driver.py:2234-2294``).

    History entries hold the mixed densities and the residuals rho_out - rho_in;
    the next density is the residual-minimising combination of the mixed ones,
    clipped at zero and renormalised.  Falls back to the plain linear mix when
    the DIIS system is singular or its coefficients exceed 20 in magnitude.  The
    extrapolation starts at iteration ``warmup`` (1-based, ``driver.py:4307``)."""

    def __init__(self, engine, depth: int = 6, warmup: int = 3):
        super().__init__(engine)
        self.depth, self.warmup = depth, warmup
        self.hist: list = []

    def __call__(self, mixed_up, mixed_dn, res_up, res_dn):
        self.iteration += 1
        it = self.iteration
        self.hist.append((mixed_up, mixed_dn, res_up, res_dn))
        if len(self.hist) > self.depth:
            self.hist.pop(0)
        h = len(self.hist)
        self.history_sizes.append(h)
        if h < 2 or it < self.warmup:
            return mixed_up, mixed_dn
        res = [(r[2], r[3]) for r in self.hist]
        B = self.gram(res, res)
        M = -np.ones((h + 1, h + 1))
        M[-1, -1] = 0.0
        M[:-1, :-1] = B + 1.0e-12 * max(float(np.abs(B).max()), 1.0) * np.eye(h)
        rhs = np.zeros(h + 1)
        rhs[-1] = -1.0
        try:
            c = np.linalg.solve(M, rhs)[:-1]
        except np.linalg.LinAlgError:
            c = None
        out = None
        if c is not None and np.all(np.isfinite(c)) and float(np.max(np.abs(c))) <= 20.0:
            out = self.finish(self.combine(c, [r[0] for r in self.hist]), self.combine(c, [r[1] for r in self.hist]))
        if out is None:
            self.fallback.append(it)
            return mixed_up, mixed_dn
        self.used.append(it)
        return out


class AndersonMixer(_Mixer):
    """Anderson mixing on secant differences (``driver.py:2297-2545``).

    From the history of (mixed density, residual) pairs: the secants of
    consecutive entries whose residual differences are neither tiny nor within
    ``collinearity`` (|cosine|) of a kept one (``:2125-2190``) enter a
    regularised least-squares fit of the current residual; the candidate is the
    damped extrapolation (damping adapted to the residual ratio when
    ``adaptive_damping``, ``:2193-2231``), rejected when its projected residual
    ratio exceeds ``acceptance_ratio`` or its coefficients exceed 50, its step
    clipped to ``step_clip_factor`` x ||residual||, then clipped at zero and
    renormalised.  ``reset_on_growth`` keeps only the newest entry when the
    residual norm grew by more than ``reset_growth_factor`` (``:4330-4360``)."""

    def __init__(self, engine, history_length: int = 4, warmup: int = 3, regularization: float = 1.0e-8,
                 damping: float = 0.5, step_clip_factor: float | None = None, reset_on_growth: bool = False,
                 reset_growth_factor: float = 1.10, adaptive_damping: bool = False, min_damping: float = 0.35,
                 max_damping: float = 0.75, acceptance_ratio: float = 1.02, collinearity: float = 0.995):
        super().__init__(engine)
        self.depth, self.warmup = history_length, warmup
        self.regularization, self.damping, self.step_clip = regularization, damping, step_clip_factor
        self.reset_on_growth, self.growth = reset_on_growth, reset_growth_factor
        self.adaptive, self.min_damping, self.max_damping = adaptive_damping, min_damping, max_damping
        self.acceptance, self.collinearity = acceptance_ratio, collinearity
        self.hist: list = []
        self.rejected: list[int] = []
        self.resets: list[int] = []
        self.filtered_sizes: list[int] = []
        self.effective_damping: list[float] = []
        self.projected_ratios: list = []

    def _damping(self, rn: np.ndarray) -> float:
        """``_select_monitor_grid_anderson_damping`` from the residual norms of the history."""

        base = float(np.clip(self.damping, self.min_damping, self.max_damping))
        if not self.adaptive or len(rn) < 2:
            return base
        cur, prev = rn[-1], rn[-2]
        if not np.isfinite(cur) or not np.isfinite(prev) or prev <= 1.0e-16:
            return base
        ratio = cur / prev
        if ratio > 1.05:
            return float(self.min_damping)
        if ratio > 0.99:
            return float(np.clip(0.5 * (base + self.min_damping), self.min_damping, self.max_damping))
        if ratio < 0.90:
            return float(self.max_damping)
        return base

    def _apply(self):
        """One Anderson candidate: (densities or None, filtered length, damping, projected ratio)."""

        hist, h = self.hist, len(self.hist)
        cur = hist[-1]
        # residual differences of consecutive entries and the residuals, one Gram
        dres = [(b[2] - a[2], b[3] - a[3]) for a, b in zip(hist[:-1], hist[1:])]
        res = [(x[2], x[3]) for x in hist]
        G = self.gram(dres + res, dres + res)
        m = len(dres)
        Gdd, Gdr = G[:m, :m], G[:m, m:]
        rn = np.sqrt(np.maximum(np.diag(G)[m:], 0.0))
        # secant filter (driver.py:2125-2190)
        kept = []
        for i in range(m):
            ni = np.sqrt(max(Gdd[i, i], 0.0))
            if not np.isfinite(ni) or ni <= 1.0e-14:
                continue
            collinear = False
            for k in kept:
                nk = np.sqrt(max(Gdd[k, k], 0.0))
                if not np.isfinite(nk) or nk <= 1.0e-14:
                    continue
                if abs(float(Gdd[i, k] / (ni * nk))) >= self.collinearity:
                    collinear = True
                    break
            if not collinear:
                kept.append(i)
        flen = len(kept) + 1
        damping = self._damping(rn)
        if not kept:
            return None, flen, damping, None
        A = Gdd[np.ix_(kept, kept)].copy()
        rhs = Gdr[kept, h - 1].copy()
        A += max(float(self.regularization), 0.0) * max(float(np.max(np.abs(A))), 1.0) * np.eye(len(kept))
        try:
            c = np.linalg.solve(A, rhs)
        except np.linalg.LinAlgError:
            return None, flen, damping, None
        if not np.all(np.isfinite(c)) or float(np.max(np.abs(c))) > 50.0:
            return None, flen, damping, None
        dmix = [(hist[i + 1][0] - hist[i][0], hist[i + 1][1] - hist[i][1]) for i in kept]
        # candidate = cur - d sum c_k dmix_k; projected residual = r - d sum c_k dres_k
        neg = [-damping * float(x) for x in c]
        cand_up = self.combine([1.0] + neg, [cur[0]] + [d[0] for d in dmix])
        cand_dn = self.combine([1.0] + neg, [cur[1]] + [d[1] for d in dmix])
        proj_up = self.combine([1.0] + neg, [cur[2]] + [dres[i][0] for i in kept])
        proj_dn = self.combine([1.0] + neg, [cur[3]] + [dres[i][1] for i in kept])
        cur_norm = rn[-1]
        proj_norm = self.norm((proj_up, proj_dn))
        ratio = 0.0 if cur_norm <= 1.0e-16 else float(proj_norm / cur_norm)
        if not np.isfinite(ratio) or ratio > self.acceptance:
            return None, flen, damping, ratio
        if self.step_clip is not None:
            clip = float(self.step_clip)
            if not np.isfinite(clip) or clip <= 0.0:
                return None, flen, damping, ratio
            step = (cand_up - cur[0], cand_dn - cur[1])
            snorm = self.norm(step)
            cap = clip * max(float(cur_norm), 1.0e-16)
            if snorm > cap:
                scale = cap / max(float(snorm), 1.0e-16)
                cand_up, cand_dn = cur[0] + scale * step[0], cur[1] + scale * step[1]
        return self.finish(cand_up, cand_dn), flen, damping, ratio

    def __call__(self, mixed_up, mixed_dn, res_up, res_dn):
        self.iteration += 1
        it = self.iteration
        self.hist.append((mixed_up, mixed_dn, res_up, res_dn))
        if len(self.hist) > self.depth:
            self.hist = self.hist[-self.depth:]
        if self.reset_on_growth and len(self.hist) >= 2:
            prev, cur = self.norm((self.hist[-2][2], self.hist[-2][3])), self.norm((res_up, res_dn))
            if not np.isfinite(cur) or (prev > 0.0 and cur > float(self.growth) * prev):
                self.hist = self.hist[-1:]
                self.resets.append(it)
        out = (mixed_up, mixed_dn)
        if it >= self.warmup and len(self.hist) >= 2:
            cand, flen, damping, ratio = self._apply()
            self.filtered_sizes.append(flen)
            self.effective_damping.append(damping)
            self.projected_ratios.append(ratio)
            if cand is not None:
                out = cand
                self.used.append(it)
            elif ratio is None:
                self.fallback.append(it)
            else:
                self.rejected.append(it)
        else:
            self.filtered_sizes.append(len(self.hist))
        self.history_sizes.append(len(self.hist))
        return out


class BroydenMixer(_Mixer):
    """Broyden-like mixing (``driver.py:2548-2651``): an inverse-Jacobian model
    G0 = ``mixing`` x identity updated by the secants of consecutive history
    entries (those with |dres|^2 above ``regularization``); the next density is
    rho + ``damping`` x G r, clipped at zero and renormalised."""

    def __init__(self, engine, mixing: float = 0.35, history_length: int = 4, warmup: int = 3,
                 regularization: float = 1.0e-8, damping: float = 0.5):
        super().__init__(engine)
        self.mixing, self.depth, self.warmup = mixing, history_length, warmup
        self.regularization, self.damping = regularization, damping
        self.hist: list = []

    def _apply(self):
        if not (0.0 < self.mixing <= 1.0) or not (0.0 < self.damping <= 1.0):
            return None
        hist = self.hist
        cur = hist[-1]
        ups: list = []   # update vectors u_k
        secs: list = []  # secant residuals y_k
        dens: list = []  # |y_k|^2

        def inverse_map(v):
            # G v = mixing v + sum_k (<y_k|v> / |y_k|^2) u_k (one Gram for all <y_k|v>)
            coef = [self.mixing]
            vecs_up, vecs_dn = [v[0]], [v[1]]
            if secs:
                g = self.gram(secs, [v])[:, 0]
                for k, uk in enumerate(ups):
                    coef.append(float(g[k] / dens[k]))
                    vecs_up.append(uk[0])
                    vecs_dn.append(uk[1])
            return self.combine(coef, vecs_up), self.combine(coef, vecs_dn)

        for a, b in zip(hist[:-1], hist[1:]):
            s = (b[0] - a[0], b[1] - a[1])
            y = (b[2] - a[2], b[3] - a[3])
            d = float(self.gram([y], [y])[0, 0])
            if d <= max(float(self.regularization), 1.0e-16):
                continue
            gy = inverse_map(y)
            ups.append((s[0] - gy[0], s[1] - gy[1]))
            secs.append(y)
            dens.append(d)
        if not dens:
            return None
        cu, cd = inverse_map((cur[2], cur[3]))
        return self.finish(cur[0] + self.damping * cu, cur[1] + self.damping * cd)

    def __call__(self, mixed_up, mixed_dn, res_up, res_dn):
        self.iteration += 1
        it = self.iteration
        self.hist.append((mixed_up, mixed_dn, res_up, res_dn))
        if len(self.hist) > self.depth:
            self.hist = self.hist[-self.depth:]
        out = (mixed_up, mixed_dn)
        if it >= self.warmup and len(self.hist) >= 2:
            cand = self._apply()
            if cand is not None:
                out = cand
                self.used.append(it)
            else:
                self.fallback.append(it)
        self.history_sizes.append(len(self.hist))
        return out


# ------------------------------------------------------------ closed-shell H2 singlet baseline
def closed_shell_singlet_mixing_factor(baseline_mixing: float, hartree_share: float | None,
                                       previous_residual_ratio: float | None) -> float:
    """Hartree-aware linear-mixing weight of the H2 singlet (``driver.py:1871-1886``): 0.6 x
    the baseline, cut by up to 45 % as the Hartree share of the potential change rises from
    0.55 to 0.85, and by up to 65 % as the residual ratio rises from 0.90 to 1.05, clipped to
    [min(0.08, baseline), baseline]."""

    eff = 0.60 * float(baseline_mixing)
    if hartree_share is not None and np.isfinite(hartree_share):
        eff *= 1.0 - 0.45 * float(np.clip((hartree_share - 0.55) / 0.30, 0.0, 1.0))
    if previous_residual_ratio is not None and np.isfinite(previous_residual_ratio):
        eff *= 1.0 - 0.65 * float(np.clip((previous_residual_ratio - 0.90) / 0.15, 0.0, 1.0))
    return float(np.clip(eff, min(0.08, baseline_mixing), baseline_mixing))


def weighted_field_norm(field: torch.Tensor, w: torch.Tensor) -> float:
    """sqrt(max(sum f^2 W, 0)) (``driver.py:1565-1571``): one FP64 device reduction
    (``igd_weighted_sum``); host tensors (tests) take the same sum on the CPU."""

    if not field.is_cuda:
        return float(np.sqrt(max(float(torch.sum(field.double() ** 2 * w)), 0.0)))
    from . import _lib
    from .device import ptr, stream_ptr

    f = field.contiguous()
    out = torch.empty(1, dtype=torch.float64, device=f.device)
    dt = _lib.IGD_F32 if f.dtype == torch.float32 else _lib.IGD_F64
    _lib.check(_lib.call("igd_weighted_sum", dt, f.numel(), ptr(f), ptr(f), ptr(w), ptr(out), stream_ptr()),
               "igd_weighted_sum")
    return float(np.sqrt(max(float(out.item()), 0.0)))


def singlet_hartree_tail_channel_shares(delta_hartree: torch.Tensor, delta_xc: torch.Tensor,
                                        delta_total: torch.Tensor, w: torch.Tensor):
    """Shares of the Hartree, XC and remaining local (ionic + frozen patch) channels in the
    change of the effective potential between the input and output densities
    (``driver.py:1825-1868``); (None, None, None) when the change vanishes."""

    h = weighted_field_norm(delta_hartree, w)
    x = weighted_field_norm(delta_xc, w)
    o = weighted_field_norm(delta_total - delta_hartree - delta_xc, w)
    total = h + x + o
    if total <= 1.0e-16:
        return None, None, None
    return h / total, x / total, o / total


def previous_density_residual_ratio(history, current_density_residual: float) -> float | None:
    """Residual over the previous step's (``driver.py:1574-1583``); None on the first step."""

    if not history:
        return None
    prev = float(history[-1].density_residual)
    if prev <= 1.0e-16:
        return None
    return float(current_density_residual / prev)


def closed_shell_singlet_baseline_mix(renormalized, occupations, up, dn, up_out, dn_out, baseline_mixing: float,
                                      hartree_share: float | None, previous_residual_ratio: float | None):
    """Baseline density update of the dry run (``driver.py:1889-1937``).  For the H2 closed-shell
    singlet the total density is mixed with the Hartree-aware weight, renormalised to the
    electron count, and split evenly between the spins; otherwise each spin is mixed linearly.
    ``renormalized(rho, target)`` rescales a density to ``target`` electrons.  Returns the two
    mixed densities and the weight used."""

    occ = occupations
    if not (occ.spin == 0 and occ.n_alpha == 1 and occ.n_beta == 1):
        m = float(baseline_mixing)
        return (renormalized((1.0 - m) * up + m * up_out, occ.n_alpha),
                renormalized((1.0 - m) * dn + m * dn_out, occ.n_beta), m)
    m = closed_shell_singlet_mixing_factor(baseline_mixing, hartree_share, previous_residual_ratio)
    total = renormalized((1.0 - m) * (up + dn) + m * (up_out + dn_out), occ.total_electrons)
    half = 0.5 * total
    return renormalized(half, occ.n_alpha), renormalized(half, occ.n_beta), m


def detect_singlet_alternation(previous, up_out, dn_out, energy_change, residual) -> bool:
    """Even/odd alternation test of the singlet cycle breaker (``driver.py:1177-1206``).
    ``previous`` holds the last two steps' (output up, output down, energy change), oldest first;
    ``residual(a_up, a_dn, b_up, b_dn)`` is the weighted spin-density distance.  True when the
    energy change flips sign and the new output is closer to the output two steps back than to
    the last one (by 5 %)."""

    if len(previous) < 2 or energy_change is None:
        return False
    last_change = previous[-1][2]
    if last_change is None or energy_change * last_change >= 0.0:
        return False
    to_last = residual(previous[-1][0], previous[-1][1], up_out, dn_out)
    to_two_back = residual(previous[-2][0], previous[-2][1], up_out, dn_out)
    return bool(to_two_back < 0.95 * to_last)


def cycle_breaker_mix(renormalized, occupations, mixed_up, mixed_dn, last_mixed_up, last_mixed_dn,
                      weight: float):
    """Blend the new mixed densities with the previous step's by ``weight`` and renormalise
    each spin (``driver.py:4272-4295``)."""

    return (renormalized((1.0 - weight) * mixed_up + weight * last_mixed_up, occupations.n_alpha),
            renormalized((1.0 - weight) * mixed_dn + weight * last_mixed_dn, occupations.n_beta))
