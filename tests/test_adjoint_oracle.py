"""CPU checks of the differentiated-energy oracle (oracle/adjoint_oracle.py):
each adjoint piece against central finite differences of its forward
function, and dL/dlam of a run of blocks against common-random-number
central differences with the comb held at the unperturbed run's indices
(the function the adjoint differentiates)."""
import numpy as np
import pytest

from oracle import adjoint_oracle as A
from oracle import afqmc_oracle as O
from ad_afqmc_prototype_gb300 import synth


def _crand(rng, *shape):
    return rng.normal(size=shape) + 1j * rng.normal(size=shape)


def _dirderiv(f, x, dx, eps=1e-6):
    return (f(x + eps * dx) - f(x - eps * dx)) / (2 * eps)


def test_green_adjoint_matches_fd():
    rng = np.random.default_rng(0)
    nw, n, o = 3, 7, 3
    mo = np.linalg.qr(_crand(rng, n, o))[0]
    W = mo[None] + 0.3 * _crand(rng, nw, n, o)
    gb = _crand(rng, nw, o, n)
    ob = _crand(rng, nw)

    def loss(w):
        g = O.half_green(w, mo)
        ov = O.overlap_r(w, mo)
        return float(np.sum(np.real(np.conj(gb) * g)) + np.sum(np.real(np.conj(ob) * ov)))

    ov = O.overlap_r(W, mo)
    wb = A.green_adjoint(W, mo, gbar=gb, kappa=2.0 * np.conj(ov) * ob)
    dW = _crand(rng, nw, n, o)
    fd = _dirderiv(loss, W, dW)
    assert abs(fd - np.sum(np.real(np.conj(wb) * dW))) < 1e-7 * max(1.0, abs(fd))


def test_qr_adjoint_matches_fd():
    rng = np.random.default_rng(1)
    nw, n, o = 2, 8, 4
    Wm = _crand(rng, nw, n, o)
    qb = _crand(rng, nw, n, o)

    def loss(w):
        return float(np.sum(np.real(np.conj(qb) * O.orthonormalize(w))))

    ab = A.qr_adjoint(Wm, qb)
    dW = _crand(rng, nw, n, o)
    fd = _dirderiv(loss, Wm, dW)
    assert abs(fd - np.sum(np.real(np.conj(ab) * dW))) < 1e-7 * max(1.0, abs(fd))


def test_energy_gbar_matches_fd():
    rng = np.random.default_rng(2)
    ham = synth.make_hamiltonian(6, 2, 9, seed=3)
    prob = O.make_problem(0.0, ham["h1"], ham["chol"], ham["mo_coeff"], 0.01)
    W = ham["mo_coeff"][None] + 0.2 * _crand(rng, 3, 6, 2)
    eb = rng.normal(size=3)

    def loss(w):
        return float(np.sum(eb * np.real(O.energy_r(w, 0.0, prob.meas_ctx, prob.mo_coeff))))

    gb, _ = A.energy_gbar(prob, W, eb)
    wb = A.green_adjoint(W, prob.mo_coeff, gbar=gb)
    dW = _crand(rng, 3, 6, 2)
    fd = _dirderiv(loss, W, dW)
    assert abs(fd - np.sum(np.real(np.conj(wb) * dW))) < 1e-7 * max(1.0, abs(fd))


def _run(lam, ham, params, st0, fields, zetas, sr_fixed=None):
    prob = O.make_problem(0.0, ham["h1"] + lam * ham["D"], ham["chol"], ham["mo_coeff"], params.dt)
    es, ws, tapes = A.run_forward(prob, params, st0, fields, zetas, sr_fixed)
    return prob, es, ws, tapes


def _setup(n=8, o=3, G=12, nw=16, steps=4, qr_every=2, blocks=3, seed=5):
    ham = synth.make_hamiltonian(n, o, G, seed=seed)
    params = O.Params(dt=0.01, n_prop_steps=steps, qr_every=qr_every, n_exp_terms=6)
    prob0 = O.make_problem(0.0, ham["h1"], ham["chol"], ham["mo_coeff"], params.dt)
    st0 = O.init_prop_state(prob0, nw, initial_walkers=synth.trial_walkers(ham["mo_coeff"], nw))
    rng = np.random.default_rng(seed + 100)
    fields = [rng.normal(size=(steps, nw, G)) for _ in range(blocks)]
    zetas = rng.uniform(size=blocks)
    return ham, params, st0, fields, zetas


@pytest.mark.parametrize("loss", ["mixed", "last_block", "weights"])
def test_run_gradient_matches_fixed_comb_fd(loss):
    ham, params, st0, fields, zetas = _setup()
    prob, es, ws, tapes = _run(0.0, ham, params, st0, fields, zetas)
    idx = [t.idx for t in tapes]

    def L(es, ws):
        if loss == "mixed":
            return A.mixed_energy(es, ws)
        if loss == "last_block":
            return float(es[-1])
        return float(np.sum(np.log(ws)))

    if loss == "mixed":
        eb, wb = A.mixed_energy_bar(es, ws)
    elif loss == "last_block":
        eb, wb = np.zeros_like(es), np.zeros_like(ws)
        eb[-1] = 1.0
    else:
        eb, wb = np.zeros_like(es), 1.0 / ws
    h1bar, _ = A.run_backward(prob, params, tapes, eb, wb, st0.walkers.shape[0])
    grad = float(np.sum(h1bar * ham["D"]))
    eps = 1e-5
    _, ep, wp, tp = _run(eps, ham, params, st0, fields, zetas, idx)
    _, em, wm, tm = _run(-eps, ham, params, st0, fields, zetas, idx)
    fd = (L(ep, wp) - L(em, wm)) / (2 * eps)
    assert abs(grad - fd) <= 1e-6 * abs(fd) + 1e-9, (grad, fd)
    # with the comb left free the indices did not move at this step size
    _, ef, wf, tf = _run(eps, ham, params, st0, fields, zetas)
    assert all(np.array_equal(a.idx, b.idx) for a, b in zip(tf, tapes))


def test_forward_matches_block_oracle():
    """The taped forward is afqmc_oracle.afqmc_block."""
    ham, params, st0, fields, zetas = _setup()
    prob, es, ws, tapes = _run(0.0, ham, params, st0, fields, zetas)
    st = st0
    for b in range(len(fields)):
        st, obs, idx = O.afqmc_block(prob, params, st, fields[b], zetas[b])
        assert obs["energy"] == es[b] and obs["weight"] == ws[b]
        assert np.array_equal(idx, tapes[b].idx)
