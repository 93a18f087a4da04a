"""Golden vectors for stat_utils: runs the reference's own stat_utils.py (it
imports only NumPy, so it loads here by file path, without the package's
JAX imports) on seeded synthetic block energies and weights, and stores
inputs and outputs in stat_utils.npz.  Run from the repository root with the
reference checked out at REF (default /root/reference)."""
import importlib.util
import os
import sys

import numpy as np

REF = os.environ.get("REF", "/root/reference")
spec = importlib.util.spec_from_file_location("ref_stat_utils", os.path.join(REF, "ad_afqmc_prototype", "stat_utils.py"))
S = importlib.util.module_from_spec(spec)
spec.loader.exec_module(S)

out = {}
rng = np.random.default_rng(2024)
for case, (n, phi) in enumerate([(400, 0.0), (1000, 0.6), (3000, 0.9), (137, 0.3)]):
    x = np.empty(n)
    x[0] = rng.normal()
    for i in range(1, n):  # AR(1) correlated block energies
        x[i] = phi * x[i - 1] + np.sqrt(1 - phi * phi) * rng.normal()
    e = -10.0 + 0.01 * x
    w = rng.uniform(0.5, 1.5, n) * 4096
    r = S.blocking_analysis_ratio(e, w, print_q=False)
    out[f"e{case}"], out[f"w{case}"] = e, w
    out[f"mu{case}"] = r["mu"]
    out[f"se{case}"] = r["se_star"]
    out[f"B{case}"] = r["B_star"]
    out[f"curve{case}"] = r["se_curve"]
    out[f"sizes{case}"] = r["block_sizes"]
    out[f"est{case}"] = r["estimator_scale_samples"]
    data = np.column_stack((e, w))
    data[::97, 0] += 5.0  # planted outliers
    kept, mask = S.reject_outliers(data, obs=0)
    out[f"data{case}"], out[f"mask{case}"] = data, mask
    m, s = S.jackknife_ratios(e * w, w)
    out[f"jk{case}"] = np.array([m, s])
np.savez(os.path.join(os.path.dirname(os.path.abspath(__file__)), "stat_utils.npz"), **out)
print("wrote", len(out), "arrays")
