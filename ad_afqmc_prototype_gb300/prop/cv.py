"""Learned control variate for the exchange energy of the block measurement.

An engine form beside the reference's exact measurement (prop/blocks.py:59-79,
meas/rhf.py:36-50); it has no counterpart in the reference.  A small network
(64 -> H -> H -> 1, GELU, bf16 weights; the engine's own tensor-core
forward, gradient and Adam kernels) predicts each walker's exchange energy
X_w = sum_g tr(f_g f_g) from cheap per-walker features (Coulomb-vector block
norms, the Coulomb and one-body terms, log|overlap|; `afq_cv` in the C
header lists them).  It is trained on exact exchange values the engine
produces (`record` blocks) and then used only as a control variate: exact
exchange runs on a systematic random sample of the walkers each measurement
and corrects the network's sum, so the block energy stays unbiased whatever
the network predicts; the exact measurement remains available (cv=None) and
is the reference the tests compare against.

Usage (with the arguments of ``prop.blocks.afqmc_block``)::

    cv = ExchangeControlVariate(hidden=256, sample_fraction=1 / 8)
    cv.mode = "record"
    for _ in range(5):                      # the first 50 steps
        state, obs = afqmc_block(state, cv=cv, **kw)
    cv.fit()
    cv.mode = "estimate"                    # from now on
    state, obs = afqmc_block(state, cv=cv, **kw)
"""
from __future__ import annotations

import math
from typing import Optional

import torch

from .. import _lib, engine

N_FEATURES = _lib.AFQ_CV_FEATURES


class ExchangeControlVariate:
    """Network parameters, training data and the measurement mode.

    mode: "record" (exact measurement, features and exact exchange of every
    walker kept as training data), "estimate" (network plus sampled exact
    correction) or "off" (the plain exact measurement)."""

    def __init__(self, hidden: int = 256, sample_fraction: float = 0.125, seed: int = 0, device=None):
        if hidden % 32 or not 32 <= hidden <= 256:
            raise ValueError("hidden must be a multiple of 32 in [32, 256]")
        if not 0.0 < sample_fraction <= 1.0:
            raise ValueError("sample_fraction must be in (0, 1]")
        self.hidden = int(hidden)
        self.sample_fraction = float(sample_fraction)
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.mode = "record"
        n = engine.mlp_param_count(N_FEATURES, self.hidden)
        self.master = self._init_params(seed).to(self.device)
        assert self.master.numel() == n
        self.params = torch.empty((n,), dtype=torch.bfloat16, device=self.device)
        engine.mlp_sync(self.master, self.params, N_FEATURES, self.hidden)
        self.adam_m = torch.zeros_like(self.master)
        self.adam_v = torch.zeros_like(self.master)
        self.adam_step = 0
        self.feat_shift = torch.zeros((N_FEATURES,), dtype=torch.float32, device=self.device)
        self.feat_scale = torch.ones((N_FEATURES,), dtype=torch.float32, device=self.device)
        self.y_shift, self.y_scale = 0.0, 1.0
        self.data_x: list[torch.Tensor] = []
        self.data_y: list[torch.Tensor] = []
        self.last_stats: Optional[torch.Tensor] = None
        self.loss_history: list[float] = []
        self._keep = None

    # parameter layout: W1 (H x F), b1 (H), W2 (H x H), b2 (H), w3 (H), b3 (1)
    def _init_params(self, seed: int) -> torch.Tensor:
        F, H = N_FEATURES, self.hidden
        g = torch.Generator().manual_seed(int(seed))
        w1 = torch.randn((H, F), generator=g) * math.sqrt(2.0 / F)
        w2 = torch.randn((H, H), generator=g) * math.sqrt(2.0 / H)
        w3 = torch.randn((H,), generator=g) * math.sqrt(1.0 / H)
        z = torch.zeros
        return torch.cat([w1.flatten(), z(H), w2.flatten(), z(H), w3, z(1)]).to(torch.float32)

    def predict(self, features: torch.Tensor) -> torch.Tensor:
        """Exchange energies predicted from raw features (B, 64)."""
        x = (features.to(self.device, torch.float32) - self.feat_shift) * self.feat_scale
        y = engine.mlp_forward(self.params, x, self.hidden)
        return self.y_shift + self.y_scale * y.double()

    # ------------------------------------------------------------------ blocks
    def block_args(self, n_walkers: int) -> Optional[_lib.afq_cv]:
        """The afq_cv structure of the next block (device buffers kept alive on self)."""
        if self.mode == "off":
            return None
        c = _lib.afq_cv()
        c.hidden = self.hidden
        if self.mode == "record":
            feats = torch.empty((n_walkers, N_FEATURES), dtype=torch.float32, device=self.device)
            exch = torch.empty((n_walkers,), dtype=torch.float64, device=self.device)
            c.mode = _lib.AFQ_CV_RECORD
            c.rec_features = engine.ptr(feats).value
            c.rec_exchange = engine.ptr(exch).value
            self._keep = (feats, exch)
        elif self.mode == "estimate":
            stats = torch.zeros((4,), dtype=torch.float64, device=self.device)
            c.mode = _lib.AFQ_CV_ESTIMATE
            c.n_sample = max(1, int(round(self.sample_fraction * n_walkers)))
            c.net = engine.ptr(self.params).value
            c.feat_shift = engine.ptr(self.feat_shift).value
            c.feat_scale = engine.ptr(self.feat_scale).value
            c.y_shift, c.y_scale = float(self.y_shift), float(self.y_scale)
            c.stats = engine.ptr(stats).value
            self._keep = (stats,)
        else:
            raise ValueError(f"unknown control-variate mode {self.mode!r}")
        return c

    def after_block(self):
        """Files a record block's data, or keeps an estimate block's statistics."""
        if self._keep is None:
            return
        if self.mode == "record":
            self.data_x.append(self._keep[0])
            self.data_y.append(self._keep[1])
        elif self.mode == "estimate":
            self.last_stats = self._keep[0]
        self._keep = None

    # ---------------------------------------------------------------- training
    def fit(self, epochs: int = 20, batch: int = 1024, lr: float = 1e-3, seed: int = 0) -> list[float]:
        """Trains on the recorded blocks with the engine's kernels; sets the
        feature and target standardisation from the data."""
        if not self.data_x:
            raise ValueError("no recorded training data (run blocks with mode='record' first)")
        X = torch.cat(self.data_x).to(torch.float32)
        Y = torch.cat(self.data_y)
        mu = X.mean(0)
        sd = X.std(0)
        sd = torch.where(sd > 1e-6 * mu.abs() + 1e-20, sd, torch.ones_like(sd))
        self.feat_shift = mu.contiguous()
        self.feat_scale = (1.0 / sd).contiguous()
        self.y_shift = float(Y.mean())
        self.y_scale = float(Y.std()) if float(Y.std()) > 0 else 1.0
        Xs = ((X - self.feat_shift) * self.feat_scale).contiguous()
        Ys = ((Y - self.y_shift) / self.y_scale).to(torch.float32).contiguous()
        n = Xs.shape[0]
        g = torch.Generator(device=self.device).manual_seed(int(seed))
        ws = None
        nb = max(1, n // batch) if n >= batch else 1
        bsz = batch if n >= batch else n
        # one device slot per step for the batch losses: the loop issues kernels only
        lbuf = torch.zeros((int(epochs), nb), dtype=torch.float32, device=self.device)
        for ep in range(int(epochs)):
            perm = torch.randperm(n, generator=g, device=self.device)
            Xp, Yp = Xs[perm].contiguous(), Ys[perm].contiguous()  # one gather an epoch; batches are slices
            for k in range(nb):
                self.adam_step += 1
                _, ws = engine.mlp_train_step(self.master, self.params, self.adam_m, self.adam_v,
                                              Xp[k * bsz:(k + 1) * bsz], Yp[k * bsz:(k + 1) * bsz], lr,
                                              self.adam_step, self.hidden, ws, loss_out=lbuf[ep, k:k + 1])
        losses = lbuf.double().mean(1).tolist()
        self.loss_history.extend(losses)
        return losses

    def state_dict(self) -> dict:
        return {"hidden": self.hidden, "master": self.master.cpu().numpy(), "feat_shift": self.feat_shift.cpu().numpy(),
                "feat_scale": self.feat_scale.cpu().numpy(), "y_shift": self.y_shift, "y_scale": self.y_scale}

