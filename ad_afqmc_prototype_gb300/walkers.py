"""Walker batches and population operations (walkers.py:1-265 of the
reference), restricted, unrestricted and generalized walkers on the CUDA
engine.

Unrestricted walkers are the reference's pair (w_up, w_dn); this package
returns the pair as the two halves of one (2, W, n, o) device tensor
(engine.as_pair / engine.pair_views), which the engine reads without a
copy."""
from __future__ import annotations

from typing import Any, Callable

import torch

from . import engine
from .core.system import system


def _natorbs(dm: torch.Tensor, n_occ: int) -> torch.Tensor:
    """walkers.py:13-16."""
    dm = 0.5 * (dm + dm.conj().T)
    vecs = torch.linalg.eigh(dm)[1].flip(-1)
    return vecs[:, :n_occ]


def init_walkers(sys: system, rdm1, n_walkers: int):
    """Walkers from natural orbitals of the total rdm1 (walkers.py:19-77)."""
    wk = sys.walker_kind.lower()
    rdm1 = torch.as_tensor(rdm1)
    if wk == "restricted":
        if rdm1.dim() == 2:
            raise ValueError(
                "For walker_kind in {'restricted','unrestricted'}, rdm1 must be spin-block (2, norb, norb).")
        if rdm1.dim() != 3 or rdm1.shape[0] != 2:
            raise ValueError("Expected rdm1 with shape (2, norb, norb).")
        dm_tot = engine.as_device(rdm1[0] + rdm1[1], engine.C128)
        w0 = _natorbs(dm_tot, sys.nup).to(engine.C128)
        return w0.unsqueeze(0).expand(n_walkers, *w0.shape).contiguous()
    if wk == "unrestricted":
        if rdm1.dim() != 3 or rdm1.shape[0] != 2:
            raise ValueError("For walker_kind in {'restricted','unrestricted'}, rdm1 must be spin-block "
                             "(2, norb, norb).")
        if sys.nup != sys.ndn:
            raise ValueError("unrestricted walkers with the RHF trial need nelec[0] == nelec[1]")
        dev_dm = engine.as_device(rdm1, engine.C128)
        wu = _natorbs(dev_dm[0], sys.nup).to(engine.C128)
        wd = _natorbs(dev_dm[1], sys.ndn).to(engine.C128)
        pair = torch.stack([wu.unsqueeze(0).expand(n_walkers, *wu.shape),
                            wd.unsqueeze(0).expand(n_walkers, *wd.shape)]).contiguous()
        return engine.pair_views(pair)
    if wk == "generalized":
        ne = sys.nup + sys.ndn
        n = sys.norb
        if rdm1.dim() == 2:
            if rdm1.shape[0] != 2 * n or rdm1.shape[1] != 2 * n:
                raise ValueError("For generalized walkers, a 2D rdm1 must have shape (2*norb, 2*norb).")
            w0 = _natorbs(engine.as_device(rdm1, engine.C128), ne).to(engine.C128)
        else:
            if rdm1.dim() != 3 or rdm1.shape[0] != 2:
                raise ValueError("Expected rdm1 with shape (2, norb, norb) for generalized init from spin blocks.")
            dm = engine.as_device(rdm1, engine.C128)
            up = _natorbs(dm[0], sys.nup).to(engine.C128)
            dn = _natorbs(dm[1], sys.ndn).to(engine.C128)
            w0 = torch.zeros((2 * n, ne), dtype=engine.C128, device=up.device)
            w0[:n, :sys.nup] = up
            w0[n:, sys.nup:] = dn
        return w0.unsqueeze(0).expand(n_walkers, *w0.shape).contiguous()
    raise ValueError(f"unknown walker_kind: {wk}")


def is_unrestricted(w) -> bool:
    return isinstance(w, tuple) and len(w) == 2


def n_walkers(w) -> int:
    return w[0].shape[0] if is_unrestricted(w) else w.shape[0]


def _chunk_size(nw: int, n_chunks: int) -> int:
    if nw % n_chunks != 0:
        raise ValueError(f"n_walkers={nw} is not divisible into n_chunks={n_chunks}")
    return nw // n_chunks


def _run(fn: Callable, chunk_args, extra_args, kwargs):
    batched = getattr(fn, "batched", None)
    if batched is not None:
        return batched(*chunk_args, *extra_args, **kwargs)
    return torch.func.vmap(lambda *xs: fn(*xs, *extra_args, **kwargs))(*chunk_args)


def _take(w, a: int, b: int):
    if is_unrestricted(w):
        return (w[0][a:b], w[1][a:b])
    return w[a:b]


def apply_chunked(w, apply_fn: Callable, n_chunks: int, *args, **kwargs):
    """apply_fn(walker_i, *args) over all walkers, in n_chunks sequential
    chunks (walkers.py:94-127).  Engine kernels run a chunk per launch."""
    nw = n_walkers(w)
    if n_chunks == 1:
        return _run(apply_fn, (w,), args, kwargs)
    cs = _chunk_size(nw, n_chunks)
    outs = [_run(apply_fn, (_take(w, i * cs, (i + 1) * cs),), args, kwargs) for i in range(n_chunks)]
    return torch.cat(outs, dim=0)


def apply_chunked_prop(w, fields, prop_fn: Callable, n_chunks: int, *args, **kwargs):
    """prop_fn(walker_i, fields_i, *args) in chunks (walkers.py:130-166)."""
    nw = n_walkers(w)
    if n_chunks == 1:
        return _run(prop_fn, (w, fields), args, kwargs)
    cs = _chunk_size(nw, n_chunks)
    outs = [_run(prop_fn, (_take(w, i * cs, (i + 1) * cs), fields[i * cs:(i + 1) * cs]), args, kwargs)
            for i in range(n_chunks)]
    if is_unrestricted(w):
        pair = torch.cat([engine.as_pair(o) for o in outs], dim=1).contiguous()
        return engine.pair_views(pair)
    return torch.cat(outs, dim=0)


def orthogonalize(w, walker_kind: str):
    """QR with diag(R) >= 0 (walkers.py:183-203); returns (Q, det(R)^2) for
    restricted walkers, ((Q_up, Q_dn), det(R_up) det(R_dn)) for
    unrestricted ones, (Q, det(R)) for generalized ones."""
    wk = walker_kind.lower()
    if wk == "restricted":
        q, det_r = engine.orthogonalize(w)
        return q, det_r * det_r
    if wk == "unrestricted":
        p = engine.as_pair(w)
        W = p.shape[1]
        q, det_r = engine.orthogonalize(p.reshape(2 * W, *p.shape[2:]))
        return engine.pair_views(q.reshape(p.shape)), det_r[:W] * det_r[W:]
    if wk == "generalized":
        return engine.orthogonalize(w)
    raise ValueError(f"unknown walker_kind: {walker_kind}")


def orthonormalize(w, walker_kind: str):
    """walkers.py:206-211."""
    return orthogonalize(w, walker_kind)[0]


def multiply_constants(w, constants: Any):
    """walkers.py:214-230."""
    if is_unrestricted(w):
        wu, wd = w
        if isinstance(constants, (tuple, list)) and len(constants) == 2:
            cu, cd = constants
            return (wu * torch.as_tensor(cu).reshape(-1, 1, 1), wd * torch.as_tensor(cd).reshape(-1, 1, 1))
        c = torch.as_tensor(constants).reshape(-1, 1, 1)
        return (wu * c, wd * c)
    return w * torch.as_tensor(constants).to(w.device).reshape(-1, 1, 1)


def _sr_indices(weights, zeta: float, n_walkers: int):
    """Comb indices (walkers.py:233-240)."""
    idx, _ = engine.sr_indices(weights, float(zeta))
    if idx.shape[0] != n_walkers:
        raise ValueError("n_walkers must equal len(weights)")
    return idx


def stochastic_reconfiguration(w, weights, zeta: float, walker_kind: str):
    """walkers.py:243-265: returns (walkers, weights)."""
    wk = walker_kind.lower()
    if wk == "unrestricted":
        p, weights_new, _ = engine.stochastic_reconfiguration_u(w, weights, float(zeta))
        return engine.pair_views(p), weights_new
    if wk not in ("restricted", "generalized"):
        raise ValueError(f"unknown walker_kind: {walker_kind}")
    w_new, weights_new, _ = engine.stochastic_reconfiguration(w, weights, float(zeta))
    return w_new, weights_new
