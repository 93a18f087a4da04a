"""stat_utils against golden vectors produced by the reference's own
stat_utils.py (tests/golden/make_stat_golden.py): identical estimators, so
the results agree to rounding."""
import os

import numpy as np
import pytest

from ad_afqmc_prototype_gb300 import stat_utils as S

G = np.load(os.path.join(os.path.dirname(__file__), "golden", "stat_utils.npz"))


@pytest.mark.parametrize("case", range(4))
def test_blocking_analysis_matches_reference(case):
    r = S.blocking_analysis_ratio(G[f"e{case}"], G[f"w{case}"], print_q=False)
    assert r["mu"] == pytest.approx(float(G[f"mu{case}"]), rel=1e-14)
    assert r["B_star"] == int(G[f"B{case}"])
    np.testing.assert_array_equal(r["block_sizes"], G[f"sizes{case}"])
    np.testing.assert_allclose(r["se_curve"], G[f"curve{case}"], rtol=1e-10)
    assert r["se_star"] == pytest.approx(float(G[f"se{case}"]), rel=1e-10)
    np.testing.assert_allclose(r["estimator_scale_samples"], G[f"est{case}"], rtol=1e-12)


@pytest.mark.parametrize("case", range(4))
def test_reject_outliers_and_jackknife_match_reference(case):
    kept, mask = S.reject_outliers(G[f"data{case}"], obs=0)
    np.testing.assert_array_equal(mask, G[f"mask{case}"])
    m, s = S.jackknife_ratios(G[f"e{case}"] * G[f"w{case}"], G[f"w{case}"])
    np.testing.assert_allclose([m, s], G[f"jk{case}"], rtol=1e-10)


def test_blocking_prints_and_exact():
    r = S.blocking_analysis_ratio(G["e1"], G["w1"], print_q=True, exact=-10.0)
    assert r["bias"] == pytest.approx(r["mu"] + 10.0)
    assert r["z_score"] == pytest.approx(r["bias"] / r["se_star"])
