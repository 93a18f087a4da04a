"""Golden vectors for the modified Cholesky decomposition: the reference's
own integrals.modified_cholesky (NumPy only) on seeded packed ERI matrices.

Run from the repository root with the reference checked out; writes
tests/golden/cholesky.npz.  The reference module is loaded by file path
(its package __init__ imports JAX, which is not installed here)."""
import importlib.util
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle.cholesky_oracle import packed_eri  # noqa: E402

REF = os.environ.get("AFQ_REFERENCE", "/root/reference")


def main():
    spec = importlib.util.spec_from_file_location("ref_integrals",
                                                  os.path.join(REF, "ad_afqmc_prototype", "integrals.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    out = {}
    for case, (n, g, seed, err) in enumerate([(4, 6, 0, 1e-6), (6, 12, 1, 1e-6), (8, 30, 2, 1e-8),
                                             (10, 20, 3, 1e-4)]):
        rng = np.random.default_rng(seed)
        b = rng.normal(size=(g, n, n))
        L = 0.5 * (b + np.swapaxes(b, 1, 2)) * np.exp(-np.arange(g) / 4.0)[:, None, None]
        M = packed_eri(L)
        ref = mod.modified_cholesky(M, max_error=err)
        out[f"mat{case}"] = M
        out[f"err{case}"] = np.array(err)
        out[f"chol{case}"] = ref
    np.savez_compressed(os.path.join(ROOT, "tests", "golden", "cholesky.npz"), **out)
    print({k: v.shape for k, v in out.items()})


if __name__ == "__main__":
    main()
