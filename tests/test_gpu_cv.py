"""The learned exchange control variate: the network's forward, gradient and
Adam kernels against the host restatement (oracle/mlp_oracle.py), and the
control-variate block measurement against the exact one.

Tolerances: forward 1e-4 relative (tensor-core sums of bf16 weights times
two-piece bf16 activations, against float64 sums of the same weights);
gradients 2e-3 relative in norm; Adam to fp32 rounding of the weights; the control-variate energy is
unbiased, so with every walker sampled it equals the exact energy up to the
Coulomb term's source (force-bias GEMM instead of energy GEMM, 1e-5 Ha), and
over random samples its mean is within 4 standard errors of the exact one."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

F, H = 64, 256


def _params(seed=0):
    from ad_afqmc_prototype_gb300.prop.cv import ExchangeControlVariate
    return ExchangeControlVariate(hidden=H, seed=seed)


def _bf16_host(t):
    return t.to(torch.bfloat16).double().cpu().numpy()


def test_mlp_forward_matches_oracle(cuda):
    import oracle.mlp_oracle as O
    from ad_afqmc_prototype_gb300 import engine
    cv = _params(1)
    rng = np.random.default_rng(0)
    x = rng.normal(size=(77, F))
    y = engine.mlp_forward(cv.params, torch.tensor(x, dtype=torch.float32, device="cuda"), H).double().cpu().numpy()
    xf = x.astype(np.float32).astype(np.float64)
    ref, _ = O.forward(_bf16_host(cv.master), xf, H)
    np.testing.assert_allclose(y, ref, rtol=1e-4, atol=1e-4 * np.abs(ref).max())


def test_mlp_gradient_and_adam_match_oracle(cuda):
    import oracle.mlp_oracle as O
    from ad_afqmc_prototype_gb300 import engine
    cv = _params(2)
    rng = np.random.default_rng(1)
    B = 96  # three CTA tiles of 32 rows
    x = rng.normal(size=(B, F)).astype(np.float32)
    t = rng.normal(size=B).astype(np.float32)
    p0 = cv.master.double().cpu().numpy()
    pb = _bf16_host(cv.master)
    xd, td = torch.tensor(x, device="cuda"), torch.tensor(t, device="cuda")
    g, gloss, _ = engine.mlp_gradient(cv.params, xd, td, H)
    g2, _, _ = engine.mlp_gradient(cv.params, xd, td, H)
    assert torch.equal(g, g2)  # the tiles' partial gradients are added in a fixed order
    g_gpu = g.double().cpu().numpy()
    ref_loss, g_ref = O.loss_and_grad(pb, x.astype(np.float64), t.astype(np.float64), H)
    assert abs(float(gloss.item()) - ref_loss) <= 1e-4 * abs(ref_loss)
    rel = np.linalg.norm(g_gpu - g_ref) / np.linalg.norm(g_ref)
    assert rel < 2e-3, rel
    loss, ws = engine.mlp_train_step(cv.master, cv.params, cv.adam_m, cv.adam_v, xd, td, 1e-3, 1, H)
    torch.cuda.synchronize()
    assert float(loss.item()) == float(gloss.item())
    # the Adam step applied to the GPU's own gradient
    P = p0.size
    p1, _, _ = O.adam(p0, g_gpu, np.zeros(P), np.zeros(P), 1e-3, 1)
    got = cv.master.double().cpu().numpy()
    # fp32 master weights: a few ulp of the weight, plus fp32 error in the step of size lr
    np.testing.assert_allclose(got, p1, rtol=4 * 2.0 ** -24, atol=1e-6 * 1e-3)
    # and the bf16 copy follows the master
    assert torch.equal(cv.params, cv.master.to(torch.bfloat16))


def test_mlp_training_reduces_loss(cuda):
    """A smooth target of the features is learnt by the engine's own kernels."""
    from ad_afqmc_prototype_gb300.prop.cv import ExchangeControlVariate
    cv = ExchangeControlVariate(hidden=H, seed=3)
    g = torch.Generator(device="cuda").manual_seed(0)
    X = torch.randn((4096, F), generator=g, device="cuda")
    Y = (X[:, :8] ** 2).sum(1).double() + 0.5 * X[:, 60].double()
    cv.data_x, cv.data_y = [X], [Y]
    losses = cv.fit(epochs=30, batch=512, lr=2e-3)
    assert losses[-1] < 0.05 * losses[0], losses
    pred = cv.predict(X)
    r2 = 1.0 - float(((pred - Y) ** 2).mean() / Y.var())
    assert r2 > 0.95, r2


def _setup_c4(W, prec="mixed_fast", **kw):
    import sys, os
    sys.path.insert(0, os.path.dirname(__file__))
    from test_gpu_mixed import _setup, _dstate
    pb, prb, st = _setup("c4_n200_o30_g1000_w4096", W, prec, **kw)
    return pb, prb, _dstate(st)


def _clone(s):
    from ad_afqmc_prototype_gb300 import engine
    return engine.DeviceState(*[t.clone() for t in (s.walkers, s.weights, s.overlaps, s.pop_shift, s.e_estimate)])


def test_cv_record_is_exact_and_full_sample_equals_exact(cuda):
    from ad_afqmc_prototype_gb300 import engine
    from ad_afqmc_prototype_gb300.prop.cv import ExchangeControlVariate
    W = 128
    pb, prb, s0 = _setup_c4(W, n_prop_steps=3, qr_every=0)
    engine.block(pb, prb, s0, 7, 0)  # walkers off the trial
    z = prb.__class__(**{**prb.__dict__, "n_prop_steps": 0})
    e_exact, _ = engine.block(pb, z, _clone(s0), 7, 50, zeta=0.5)
    cv = ExchangeControlVariate(hidden=H, sample_fraction=1.0, seed=4)
    cv.mode = "record"
    e_rec, _ = engine.block(pb, z, _clone(s0), 7, 50, zeta=0.5, cv=cv.block_args(W))
    cv.after_block()
    assert float(e_rec) == float(e_exact)
    assert cv.data_x[0].shape == (W, 64) and torch.isfinite(cv.data_x[0]).all()
    assert torch.isfinite(cv.data_y[0]).all()
    cv.fit(epochs=2, batch=64)
    cv.mode = "estimate"
    e_cv, _ = engine.block(pb, z, _clone(s0), 7, 50, zeta=0.5, cv=cv.block_args(W))
    cv.after_block()
    st = cv.last_stats.cpu().numpy()
    assert st[3] == W  # every walker sampled
    assert abs(float(e_cv) - float(e_exact)) < 1e-5, (float(e_cv), float(e_exact))
    assert engine.workspace_status() == 0


def test_cv_unbiased_and_network_reduces_variance(cuda):
    """Train on five recorded blocks, then estimate one block-end state's
    energy with 1/8 of the walkers exact, over many random samples: the mean
    matches the exact energy, and the trained network's estimator has a much
    smaller variance than the sample alone (the same estimator with a zero
    prediction)."""
    from ad_afqmc_prototype_gb300 import engine
    from ad_afqmc_prototype_gb300.prop.cv import ExchangeControlVariate
    W = 512
    pb, prb, s = _setup_c4(W, n_prop_steps=10, qr_every=5)
    cv = ExchangeControlVariate(hidden=H, sample_fraction=1 / 8, seed=5)
    cv.mode = "record"
    for b in range(5):
        engine.block(pb, prb, s, 11, 100 * b, cv=cv.block_args(W))
        cv.after_block()
    cv.fit(epochs=40, batch=512, lr=1e-3)
    z = prb.__class__(**{**prb.__dict__, "n_prop_steps": 0})
    e_exact = float(engine.block(pb, z, _clone(s), 13, 0, zeta=0.5)[0])

    def estimates(shift, scale, n=48):
        cv.mode = "estimate"
        out = []
        for k in range(n):
            args = cv.block_args(W)
            args.y_shift, args.y_scale = shift, scale
            out.append(float(engine.block(pb, z, _clone(s), 1000 + k, 0, zeta=0.5, cv=args)[0]))
            cv.after_block()
        return np.array(out)

    with_net = estimates(cv.y_shift, cv.y_scale)
    without = estimates(0.0, 0.0)
    se = with_net.std(ddof=1) / np.sqrt(len(with_net))
    assert abs(with_net.mean() - e_exact) < 4 * se + 1e-6, (with_net.mean(), e_exact, se)
    se0 = without.std(ddof=1) / np.sqrt(len(without))
    assert abs(without.mean() - e_exact) < 4 * se0 + 1e-6, (without.mean(), e_exact, se0)
    print("variance with network %.3e, sample alone %.3e" % (with_net.var(ddof=1), without.var(ddof=1)))
    assert with_net.var(ddof=1) < 0.25 * without.var(ddof=1)
    assert engine.workspace_status() == 0


def test_cv_full_sample_equals_exact_at_nocc_50(cuda):
    """400 orbitals, nocc 50 (the unfused exchange path): with every walker
    sampled the control-variate energy equals the exact measurement."""
    from ad_afqmc_prototype_gb300 import engine
    from ad_afqmc_prototype_gb300.prop.cv import ExchangeControlVariate
    import sys, os
    sys.path.insert(0, os.path.dirname(__file__))
    from test_gpu_mixed import _setup, _dstate
    W = 64
    pb, prb, st = _setup("c5_n400_o50_g2000_w1024", W, "mixed_fast", n_prop_steps=2, qr_every=0)
    s0 = _dstate(st)
    engine.block(pb, prb, s0, 7, 0)
    z = prb.__class__(**{**prb.__dict__, "n_prop_steps": 0})
    e_exact, _ = engine.block(pb, z, _clone(s0), 7, 50, zeta=0.5)
    cv = ExchangeControlVariate(hidden=H, sample_fraction=1.0, seed=4)
    cv.mode = "record"
    engine.block(pb, z, _clone(s0), 7, 50, zeta=0.5, cv=cv.block_args(W))
    cv.after_block()
    cv.fit(epochs=2, batch=32)
    cv.mode = "estimate"
    e_cv, _ = engine.block(pb, z, _clone(s0), 7, 50, zeta=0.5, cv=cv.block_args(W))
    cv.after_block()
    assert abs(float(e_cv) - float(e_exact)) < 1e-5, (float(e_cv), float(e_exact))
    assert engine.workspace_status() == 0
