"""Failure detection without a GPU fault.

* The bounded device-side wait (the one the tensor-core pipelines use) runs
  out on an mbarrier that nothing arrives at, reports AFQ_STATUS_WAIT_EXPIRED
  to the host, and the context stays usable.
* Faults injected on the host: a NaN walker, a walker with a singular overlap
  matrix (a zero orbital), all-zero weights.  The engine gives the
  reference's results (prop/afqmc.py:116-138 lets a NaN weight through;
  prop/blocks.py:70-73 falls back to e_estimate when the weights sum to 0)
  and counts the non-finite walkers into the workspace status.
"""
import numpy as np
import pytest
import torch

from oracle import afqmc_oracle as O
from tests.test_gpu_step import _setup, api, cpu  # noqa: F401  (fixture)

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def E(cuda):
    from ad_afqmc_prototype_gb300 import engine
    return engine


def test_bounded_wait_expires_and_context_survives(E):
    from ad_afqmc_prototype_gb300 import _lib
    assert E.selftest_wait(2_000, arrive=False) == _lib.AFQ_STATUS_WAIT_EXPIRED
    assert E.selftest_wait(1_000_000_000, arrive=True) == 0
    assert E.selftest_wait(50_000, arrive=False) == _lib.AFQ_STATUS_WAIT_EXPIRED
    with pytest.raises(ValueError):
        E.selftest_wait(0, arrive=True)
    # the context is still usable: a kernel call gives the oracle's numbers
    rng = np.random.default_rng(0)
    n, o, W = 10, 4, 5
    c = np.linalg.qr(rng.normal(size=(n, o)))[0]
    w = rng.normal(size=(W, n, o)) + 1j * rng.normal(size=(W, n, o))
    ov = E.overlap(E.as_device(w, E.C128), E.as_device(c, E.C128), True)
    np.testing.assert_allclose(cpu(ov), O.overlap_r(w, c), rtol=1e-11)


def _c1(api, W):
    H = api["synth"].make_workload(api["synth"].WORKLOADS["c1_n12_o6_g48_w256"])
    return H, O.make_problem(H["h0"], H["h1"], H["chol"], H["mo_coeff"], 0.005)


def _state_with(api, H, W, walkers, weights=None, **pkw):
    """The API state with the given walkers (overlaps recomputed as the
    reference's init does) and weights."""
    sys_, state, kw = _setup(api, H, W, dt=0.005, **pkw)
    wt = torch.as_tensor(walkers, dtype=torch.complex128, device="cuda")
    ov = api["engine"].overlap(wt, kw["trial_data"].mo_coeff, True)
    wts = state.weights if weights is None else torch.as_tensor(weights, dtype=torch.float64, device="cuda")
    return sys_, state._replace(walkers=wt, overlaps=ov, weights=wts), kw


@pytest.mark.parametrize("precision", ["fp64", "mixed_fast"])
def test_nan_walker_counted_and_propagated(api, E, precision):
    from ad_afqmc_prototype_gb300 import _lib
    W, bad = 16, 3
    H, prob = _c1(api, W)
    w = api["synth"].trial_walkers(H["mo_coeff"], W).copy()
    rng = np.random.default_rng(1)
    w = w + 0.05 * (rng.normal(size=w.shape) + 1j * rng.normal(size=w.shape))
    w[bad, 2, 1] = np.nan
    sys_, state, kw = _state_with(api, H, W, w, precision=precision)
    E.workspace_counters()  # clear
    f = rng.standard_normal((W, H["chol"].shape[0]))
    out = api["afqmc_step"](state, fields=f, **kw)
    status, nonfinite = E.workspace_counters()
    assert status == _lib.AFQ_STATUS_NONFINITE
    assert nonfinite >= 1
    wts = cpu(out.weights)
    assert np.isnan(wts[bad])
    assert np.isnan(float(out.pop_control_ene_shift))  # the mean weight is NaN, as in the reference
    good = np.arange(W) != bad
    assert np.all(np.isfinite(wts[good]))
    if precision == "fp64":
        ost = O.State(walkers=w, weights=np.ones(W), overlaps=cpu(state.overlaps),
                      pop_control_ene_shift=float(state.pop_control_ene_shift), e_estimate=float(state.e_estimate))
        ref = O.afqmc_step(prob, O.Params(dt=0.005), ost, f)
        np.testing.assert_allclose(wts[good], ref.weights[good], rtol=1e-10)
        np.testing.assert_allclose(cpu(out.walkers)[good], ref.walkers[good], atol=1e-10)
        assert np.isnan(ref.weights[bad]) and np.isnan(ref.pop_control_ene_shift)
    assert E.workspace_counters() == (0, 0)  # the read cleared both words


@pytest.mark.parametrize("precision", ["fp64", "mixed_fast"])
def test_singular_overlap_walker(api, E, precision):
    """A walker whose overlap matrix C^H W is singular (one of its orbitals is
    zero, so det = 0 exactly): its force bias and weight are not finite and
    are counted; the other walkers' new walkers and weights are the oracle's."""
    from ad_afqmc_prototype_gb300 import _lib
    W, bad = 12, 5
    H, prob = _c1(api, W)
    rng = np.random.default_rng(2)
    w = api["synth"].trial_walkers(H["mo_coeff"], W).copy()
    w = w + 0.05 * (rng.normal(size=w.shape) + 1j * rng.normal(size=w.shape))
    w[bad, :, 2] = 0.0
    sys_, state, kw = _state_with(api, H, W, w, precision=precision)
    assert complex(cpu(state.overlaps)[bad]) == 0.0
    E.workspace_counters()
    f = rng.standard_normal((W, H["chol"].shape[0]))
    out = api["afqmc_step"](state, fields=f, **kw)
    status, nonfinite = E.workspace_counters()
    assert status == _lib.AFQ_STATUS_NONFINITE and nonfinite >= 1
    good = np.arange(W) != bad
    wts = cpu(out.weights)
    assert not np.isfinite(wts[bad])
    if precision == "fp64":
        keep = np.flatnonzero(good)
        ost = O.State(walkers=w[keep], weights=np.ones(W - 1), overlaps=cpu(state.overlaps)[keep],
                      pop_control_ene_shift=float(state.pop_control_ene_shift), e_estimate=float(state.e_estimate))
        ref = O.afqmc_step(prob, O.Params(dt=0.005), ost, f[keep])
        np.testing.assert_allclose(wts[keep], ref.weights, rtol=1e-10)
        np.testing.assert_allclose(cpu(out.walkers)[keep], ref.walkers, atol=1e-10)
    else:
        assert np.all(np.isfinite(wts[good]))


@pytest.mark.parametrize("precision", ["fp64", "mixed_fast"])
def test_all_zero_weights_block(api, E, precision):
    """prop/blocks.py:70-73: a zero weight sum gives the block energy
    e_estimate; the comb then picks walker 0 everywhere and weights stay 0."""
    W = 16
    H, prob = _c1(api, W)
    w = api["synth"].trial_walkers(H["mo_coeff"], W)
    sys_, state, kw = _state_with(api, H, W, w, weights=np.zeros(W), n_prop_steps=10, qr_every=5,
                                  precision=precision)
    E.workspace_counters()
    rng = np.random.default_rng(3)
    fields = rng.standard_normal((10, W, H["chol"].shape[0]))
    out, obs = api["afqmc_block"](state, sys=sys_, fields=fields, zeta=0.5, **kw)
    assert float(obs.scalars["weight"]) == 0.0
    assert float(obs.scalars["energy"]) == float(state.e_estimate)
    assert np.all(cpu(out.weights) == 0.0)
    assert E.workspace_counters() == (0, 0)
    ost = O.State(walkers=w, weights=np.zeros(W), overlaps=cpu(state.overlaps),
                  pop_control_ene_shift=float(state.pop_control_ene_shift), e_estimate=float(state.e_estimate))
    ost, oobs, idx = O.afqmc_block(prob, O.Params(dt=0.005, n_prop_steps=10, qr_every=5), ost, fields, 0.5)
    assert oobs["energy"] == float(state.e_estimate) and oobs["weight"] == 0.0
    np.testing.assert_array_equal(idx, np.zeros(W, dtype=idx.dtype))
    tol = 1e-10 if precision == "fp64" else 1e-4
    assert abs(float(out.pop_control_ene_shift) - ost.pop_control_ene_shift) < tol
