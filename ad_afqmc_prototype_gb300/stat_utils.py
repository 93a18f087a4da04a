"""Statistics of block energies (stat_utils.py of the reference: the same
estimators, names, arguments and outputs; host NumPy, as the block energies
are a few thousand scalars).

* ``blocking_analysis_ratio`` (stat_utils.py:26-166): the weighted mean
  mu = sum(w e) / sum(w) and its standard error by blocking: for each block
  size B of a grid, the n samples are summed in G = n // B consecutive groups,
  the leave-one-group-out ratios mu_(g) give the jackknife error
  sqrt((G - 1)/G sum (mu_(g) - mean)^2), and B* is picked on the plateau of
  the error curve (first B whose error has risen 20 % above B = 1 and stays
  within 3 % over the next k sizes; else the first B reaching 95 % of the
  largest error).
* ``reject_outliers`` (stat_utils.py:169-181): robust z-score against the
  median with the larger of the median absolute deviation and IQR / 1.349.
* ``jackknife_ratios`` (stat_utils.py:184-213): jackknife mean and error of
  a ratio of means.
"""
from __future__ import annotations

from typing import Any, Dict, Iterable, Tuple

import numpy as np


def _default_grid(n: int, min_blocks: int) -> list[int]:
    top = max(2, n // min_blocks)
    cand = np.unique(np.rint(np.geomspace(1, top, 18)).astype(int))
    grid = [int(b) for b in cand if b >= 1 and n // b >= min_blocks]
    if n // int(cand[-1]) >= 5 and int(cand[-1]) not in grid:
        grid.append(int(cand[-1]))
    return grid


def _plateau(sizes, errs, groups, min_blocks, min_rise, flat_tol, k) -> Tuple[int, float, int]:
    sizes, errs, groups = np.asarray(sizes), np.asarray(errs), np.asarray(groups)
    keep = groups >= min_blocks
    if not keep.any():
        return int(sizes[0]), float(errs[0]), int(groups[0])
    b, e, g = sizes[keep], errs[keep], groups[keep]
    risen = e >= (1.0 + min_rise) * e[0]
    for i in range(e.size - k):
        if risen[i]:
            win = e[i:i + k + 1]
            if np.all(np.abs(win[1:] - win[:-1]) <= flat_tol * win[:-1]):
                return int(b[i]), float(e[i]), int(g[i])
    first = int(np.flatnonzero(e >= 0.95 * e.max())[0])
    return int(b[first]), float(e[first]), int(g[first])


def _loo(num: np.ndarray, den: np.ndarray, B: int):
    G = num.size // B
    ng = num[:G * B].reshape(G, B).sum(1)
    dg = den[:G * B].reshape(G, B).sum(1)
    nt, dt = ng.sum(), dg.sum()
    rest = dt - dg
    ok = np.abs(rest) > 1e-18
    loo = np.where(ok, (nt - ng) / np.where(ok, rest, 1.0), nt / dt)
    mean = loo.mean()
    se = float(np.sqrt(max((G - 1) / G * np.sum((loo - mean) ** 2), 0.0)))
    return loo, mean, G, se


def blocking_analysis_ratio(ene, wt, block_grid: Iterable[int] | None = None, *, min_blocks: int = 20,
                            min_rise: float = 0.20, flat_tol: float = 0.03, k: int = 3, bins: int | str = "fd",
                            figsize: Tuple[float, float] = (12, 4.2), title: str | None = None,
                            print_q: bool = True, plot_q: bool = False, exact: float | None = None) -> Dict[str, Any]:
    """Blocking analysis for mu = sum(wt*ene)/sum(wt)"""
    e = np.asarray(ene, float).ravel()
    w = np.asarray(wt, float).ravel()
    n = e.size
    assert w.size == n
    num, den = w * e, w
    mu = num.sum() / den.sum()
    grid = list(block_grid) if block_grid is not None else _default_grid(n, min_blocks)
    sizes, errs, groups, cache = [], [], [], {}
    for B in grid:
        if n // B < 5:
            continue
        loo, mean, G, se = _loo(num, den, int(B))
        sizes.append(int(B))
        errs.append(se)
        groups.append(G)
        cache[int(B)] = (loo, mean, G)
    sizes = np.array(sizes, int)
    errs = np.array(errs, float)
    groups = np.array(groups, int)
    B_star, se_star, _ = _plateau(sizes, errs, groups, min_blocks, min_rise, flat_tol, k)
    loo, mean, G = cache[B_star]
    out = {
        "mu": float(mu),
        "block_sizes": sizes,
        "se_curve": errs,
        "n_blocks": groups,
        "B_star": int(B_star),
        "se_star": float(se_star),
        "ci95_star": (float(mu - 1.96 * se_star), float(mu + 1.96 * se_star)),
        "estimator_scale_samples": mu + (G - 1) / np.sqrt(G) * (loo - mean),
        "bias": None,
        "z_score": None,
    }
    if exact is not None and np.isfinite(se_star) and se_star > 0:
        out["bias"] = float(mu - exact)
        out["z_score"] = float((mu - exact) / se_star)
    if print_q:
        print(f"mu: {out['mu']:.16g}  SE*: {out['se_star']:.16g}  95% CI: {out['ci95_star']}")
        if out["z_score"] is not None:
            print(f"bias: {out['bias']:.16g}  z: {out['z_score']:.6g}")
        se0 = float(errs[0]) if errs.size else float("nan")
        print("\nBlocking SE curve (ratio LOO):")
        print(f"{'':1s}{'B':>6s} {'G':>6s} {'SE':>14s} {'SE/SE(B=1)':>12s}")
        for B, Gb, se in zip(sizes, groups, errs):
            rel = float(se) / se0 if se0 > 0 and np.isfinite(se0) else float("nan")
            print(f"{'*' if int(B) == B_star else ' '}{int(B):6d} {int(Gb):6d} {float(se):14.6e} {rel:12.3f}")
        print("")
    if plot_q:
        raise ImportError("plotting needs matplotlib, which this package does not depend on")
    return out


def reject_outliers(data, obs, m: float = 10.0, min_threshold: float = 1e-5):
    """Rows of `data` whose column `obs` lies within m robust deviations of
    the median; returns (kept rows, mask)."""
    x = np.asarray(data)[:, obs]
    med = np.median(x)
    dev = np.abs(x - med)
    q1, q3 = np.percentile(x, [25, 75])
    spread = max(np.median(dev), (q3 - q1) / 1.349, min_threshold)
    mask = dev / spread < m
    return np.asarray(data)[mask], mask


def jackknife_ratios(num: np.ndarray, denom: np.ndarray):
    """Jackknife mean and standard deviation of mean(num) / mean(denom)."""
    num = np.asarray(num)
    denom = np.asarray(denom)
    n = num.size
    a, b = num.mean(), denom.mean()
    loo = ((a * n - num) / (n - 1)) / ((b * n - denom) / (n - 1))
    loo = loo.real
    return np.mean(loo), np.sqrt((n - 1) * np.var(loo))
