"""Exact Galerkin matrix elements of the H.psi operator in harmonic-oscillator bases, from
ladder operators: an answer for parity tests that depends neither on the oracle nor on the
library.

In a mode scaled by s (x = s Q, basis chi_n(Q) = s^(1/2) phi_n(s Q) with phi_n the
orthonormal Hermite functions) the matrices of Q and d/dQ are
    Q    = (a + a^+) / (s sqrt 2),     d/dQ = s (a - a^+) / sqrt 2,
both exact on a truncated basis as long as the truncation lies beyond every index the
product reaches.  The operator is that of the workloads:
    H = -1/2 sum_ij d_i G_ij(Q) d_j + V(Q),   G_ij(Q) = G0_ij + sum_k g_ijk Q_k   (type 10)
    H = -1/2 sum_i G0_ii d_i^2 - sum_{i<j} G0_ij d_i d_j + V(Q)               (type 1)
with V a sum of monomials (coef, up to four mode indices, electronic pair).  Integration
by parts is not used: the matrices are products of the mode matrices, so <m|H|n> is the
exact matrix element of the differential operator for every m, n below the truncation.

Where the library's grid algebra is exact (nq > nb, a function whose derivatives stay inside
the basis of its mode, Gauss-Hermite quadrature of enough points), its H.psi columns equal
these matrix elements; on a Smolyak basis the column of a function n is
    H_SG[m, n] = c(m, n) <m|H|n>,   c(m, n) = sum of the weights of the terms holding m and n.
"""
from __future__ import annotations

from itertools import product
from math import comb

import numpy as np


def ladder(nmax: int):
    """X = (a + a^+)/sqrt 2 and P = (a - a^+)/sqrt 2 (the matrix of d/dx) on nmax functions."""
    a = np.diag(np.sqrt(np.arange(1, nmax)), 1)  # a[n-1, n] = sqrt(n)
    ad = a.T
    return (a + ad) / np.sqrt(2.0), (a - ad) / np.sqrt(2.0)


class Galerkin:
    """Applies the exact operator of a spec to vectors given as dense tensors over nmax
    functions per mode (first mode first), for one electronic state (nb0 = 1)."""

    def __init__(self, spec, nmax: int):
        if spec.nb0 != 1:
            raise ValueError("one electronic state")
        self.spec, self.D, self.nmax = spec, spec.D, nmax
        X, P = ladder(nmax)
        s = np.asarray(spec.scaleQ, dtype=np.float64)
        q0 = np.asarray(spec.Q0, dtype=np.float64)
        self.Q = [X / s[i] + q0[i] * np.eye(nmax) for i in range(self.D)]
        self.d1 = [s[i] * P for i in range(self.D)]
        # d^2/dQ^2 as the product of two derivative matrices on a wider truncation, cut back
        X2, P2 = ladder(nmax + 2)
        self.d2 = [(s[i] ** 2 * (P2 @ P2))[:nmax, :nmax] for i in range(self.D)]

    def _mode(self, M, T, i):
        return np.moveaxis(np.tensordot(M, T, axes=([1], [i])), 0, i)

    def apply(self, T):
        """H T for a tensor T of shape (nmax,)*D + (ncols,)."""
        sp, D = self.spec, self.D
        out = np.zeros_like(T)
        for c, idx in zip(sp.mono_coef, sp.mono_idx):
            U = T * c
            for k in idx:
                if k >= 0:
                    U = self._mode(self.Q[k], U, k)
            out += U
        G0 = np.asarray(sp.G0, dtype=np.float64)
        g = np.asarray(sp.g, dtype=np.float64)
        if sp.keo_type == 10:
            for j in range(D):
                dj = self._mode(self.d1[j], T, j)
                for i in range(D):
                    Z = G0[i, j] * dj
                    for k in range(D):
                        if g[i, j, k] != 0.0:
                            Z = Z + g[i, j, k] * self._mode(self.Q[k], dj, k)
                    out -= 0.5 * self._mode(self.d1[i], Z, i)
        else:
            for i in range(D):
                out -= 0.5 * G0[i, i] * self._mode(self.d2[i], T, i)
                for j in range(i + 1, D):
                    out -= G0[i, j] * self._mode(self.d1[i], self._mode(self.d1[j], T, j), i)
        return out

    def columns(self, tuples):
        """<m|H|n> for every m below the truncation and each n of `tuples` (0-based HO
        quantum numbers): array (nmax,)*D + (len(tuples),)."""
        T = np.zeros((self.nmax,) * self.D + (len(tuples),))
        for c, n in enumerate(tuples):
            T[tuple(n) + (c,)] = 1.0
        return self.apply(T)


def level_of(n, Ab, Bb):
    """Smallest Smolyak level l with nb(l) = Ab + Bb l > n (n 0-based)."""
    n = np.asarray(n)
    return np.maximum(0, -((Ab - 1 - n) // Bb))


def smolyak_terms(D: int, L: int):
    """Terms l (|l| between max(0, L-D+1) and L) with their combination weights
    (-1)^(L-|l|) C(D-1, L-|l|)."""
    lmin = max(0, L - D + 1)
    out = []
    for l in product(range(L + 1), repeat=D):
        s = sum(l)
        if lmin <= s <= L:
            out.append((np.array(l), (-1) ** (L - s) * comb(D - 1, L - s)))
    return out


def pair_weights(spec, m_tuples, n_tuple):
    """c(m, n) = sum of the weights of the Smolyak terms whose bases hold both m and n."""
    D, L = spec.D, spec.LG
    Ab, Bb = np.asarray(spec.Ab), np.asarray(spec.Bb)
    lm = level_of(np.asarray(m_tuples), Ab, Bb)           # (M, D)
    ln = level_of(np.asarray(n_tuple), Ab, Bb)            # (D,)
    need = np.maximum(lm, ln[None, :])
    c = np.zeros(len(m_tuples))
    for l, w in smolyak_terms(D, L):
        c += w * np.all(l[None, :] >= need, axis=1)
    return c
