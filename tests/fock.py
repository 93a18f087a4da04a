"""Brute-force second quantisation for tiny systems (test helper).

Builds the spin-orbital Fock space (2^(2n) states, Jordan-Wigner signs) and
the Cholesky Hamiltonian
    H = h0 + sum_ij h1_ij E_ij + 1/2 sum_g V_g^2 - 1/2 sum_g sum_il (L_g L_g)_il E_il,
    V_g = sum_ij L_g[i, j] E_ij,   E_ij = sum_sigma a+_{i sigma} a_{j sigma},
which is the Hamiltonian whose mixed estimator the RHF energy kernel
evaluates.  Used to pin the oracle's overlap, force bias and local energy
against first principles instead of against its own formulas.
"""
import numpy as np


def creation_ops(nso):
    dim = 1 << nso
    ops = []
    for p in range(nso):
        a = np.zeros((dim, dim))
        for s in range(dim):
            if not (s >> p) & 1:
                sign = (-1) ** bin(s & ((1 << p) - 1)).count("1")
                a[s | (1 << p), s] = sign
        ops.append(a)
    return ops


def excitation_ops(n):
    cr = creation_ops(2 * n)
    E = np.zeros((n, n, 1 << (2 * n), 1 << (2 * n)))
    for i in range(n):
        for j in range(n):
            for s in (0, n):
                E[i, j] += cr[i + s] @ cr[j + s].T
    return cr, E


def hamiltonian(h0, h1, chol, E):
    n = h1.shape[0]
    dim = E.shape[-1]
    H = h0 * np.eye(dim) + np.einsum("ij,ijab->ab", h1, E)
    for L in chol:
        V = np.einsum("ij,ijab->ab", L, E)
        H = H + 0.5 * V @ V - 0.5 * np.einsum("il,ilab->ab", L @ L, E)
    return H


def determinant(orbs, cr, n):
    """Closed-shell determinant: columns of orbs (n, o) filled for both spins."""
    dim = cr[0].shape[0]
    psi = np.zeros(dim, dtype=complex)
    psi[0] = 1.0
    for s in (0, n):
        for a in range(orbs.shape[1]):
            op = sum(orbs[i, a] * cr[i + s] for i in range(n))
            psi = op @ psi
    return psi
