"""Primitive bases handed over as tables (evr_problem_desc.bases): the host's x, w, d0b, d1b,
d2b per (mode, level) replace the library's harmonic-oscillator tables.

* the library's own tables, read back and handed over, give the same derived matrices
  (CPU) and the same H.psi (GPU, 1e-12);
* the oracle's tables (its own Gauss-Hermite and Hermite-function algorithm) handed over
  give the oracle's H.psi (GPU, 1e-12);
* a basis that is not harmonic-oscillator -- Legendre functions on a Gauss-Legendre grid
  of a box -- gives the exact Galerkin matrix of -1/2 d2/dx2 + V on that basis (GPU);
* sizes that contradict the level rules, and non-positive weights, are rejected (CPU).
"""
import dataclasses

import numpy as np
import pytest

from evrgpu import spec as S
from evrgpu import lib as E
from oracle import oracle as O


def tables_of(src, spec):
    """(mode, level) tables of a context or oracle problem, in the descriptor's order."""
    out = []
    levels = spec.LG + 1 if spec.kind == "sg4" else 1
    for i in range(spec.D):
        for L in range(levels):
            b = src.basis(i, L)
            out.append({k: b[k] for k in ("x", "w", "d0b", "d1b", "d2b")})
    return out


CASES = {
    "sg4_d4_l5_type10": lambda: S.config_sg4(4, 5, seed=5),
    "hh6d_l3_type1": lambda: S.henon_heiles(6, 3),
    "dp3_nb8_nq10": lambda: S.config_dp3(nb=8, nq=10),
}


@pytest.mark.parametrize("name", list(CASES))
def test_own_tables_reproduce_the_derived_matrices(name):
    spec = CASES[name]()
    pa = E.Problem(spec, device=-1)
    pb = E.Problem(dataclasses.replace(spec, bases=tables_of(pa, spec)), device=-1)
    levels = spec.LG + 1 if spec.kind == "sg4" else 1
    for i in range(spec.D):
        for L in range(levels):
            a, b = pa.basis(i, L), pb.basis(i, L)
            for k in ("x", "w", "d0b", "bgw", "d1gg", "d2gg"):
                assert np.abs(a[k] - b[k]).max() <= 1e-15 * max(1.0, np.abs(a[k]).max()), (i, L, k)


def test_bad_tables_are_rejected():
    spec = S.config_sg4(3, 2, seed=1)
    pa = E.Problem(spec, device=-1)
    t = tables_of(pa, spec)
    wrong = list(t)
    wrong[1] = dict(t[2])  # level 2's tables in level 1's place: sizes contradict the rules
    with pytest.raises(E.EvrError) as ei:
        E.Problem(dataclasses.replace(spec, bases=wrong), device=-1)
    assert ei.value.code == E.EVR_EINVAL and "level 1" in str(ei.value)
    bad = list(t)
    bad[0] = dict(t[0], w=-np.asarray(t[0]["w"]))
    with pytest.raises(E.EvrError) as ei:
        E.Problem(dataclasses.replace(spec, bases=bad), device=-1)
    assert ei.value.code == E.EVR_EINVAL


def rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(CASES))
def test_host_tables_give_the_same_hpsi(name):
    spec = CASES[name]()
    pa = E.Problem(spec, device=0)
    pb = E.Problem(dataclasses.replace(spec, bases=tables_of(pa, spec)), device=0)
    po = O.OracleProblem(spec)
    pc = E.Problem(dataclasses.replace(spec, bases=tables_of(po, spec)), device=0)
    psi = np.random.default_rng(2).standard_normal((pa.N, 6))
    ref = pa.hpsi(psi)
    assert rel(pb.hpsi(psi), ref) <= 1e-12
    assert rel(pc.hpsi(psi), po.hpsi(psi)) <= 1e-12


def legendre_box(nb, nq, a):
    """Normalised Legendre functions on [-a, a] with their derivatives on the nq-point
    Gauss-Legendre grid (weights of the box): a primitive basis that is not harmonic."""
    t, wt = np.polynomial.legendre.leggauss(nq)
    x, w = a * t, a * wt
    d0 = np.zeros((nq, nb)); d1 = np.zeros((nq, nb)); d2 = np.zeros((nq, nb))
    for n in range(nb):
        c = np.zeros(n + 1); c[n] = np.sqrt((2 * n + 1) / (2 * a))
        d0[:, n] = np.polynomial.legendre.legval(t, c)
        d1[:, n] = np.polynomial.legendre.legval(t, np.polynomial.legendre.legder(c)) / a
        d2[:, n] = np.polynomial.legendre.legval(t, np.polynomial.legendre.legder(c, 2)) / a ** 2
    return dict(x=x, w=w, d0b=d0, d1b=d1, d2b=d2)


@pytest.mark.gpu
def test_legendre_box_basis_gives_the_exact_galerkin_matrix():
    # D=2 direct product of Legendre bases (nb=8, nq=11) on [-3, 3], type 1 with G = 1 and
    # V = 0.3 q0^2 + 0.1 q0 q1: for polynomial bases the grid algebra is exact, so
    # H = -1/2 (D2 x I + I x D2) + V with D2 and Q the exact Legendre matrices
    a, nb, nq = 3.0, 8, 11
    t = legendre_box(nb, nq, a)
    p = S.Poly()
    p.add(0.3, [0, 0])
    p.add(0.1, [0, 1])
    c, idx, el = p.arrays()
    spec = S.ProblemSpec(kind="dp", D=2, nq_dp=[nq, nq], nb_dp=[nb, nb], mono_coef=c, mono_idx=idx,
                         mono_elec=el, keo_type=1, bases=[t, t])
    pg = E.Problem(spec, device=0)
    W = np.diag(t["w"])
    D2 = t["d0b"].T @ W @ t["d2b"]             # exact for polynomials of degree < 2 nq
    Q = t["d0b"].T @ W @ (t["x"][:, None] * t["d0b"])
    Q2 = t["d0b"].T @ W @ ((t["x"] ** 2)[:, None] * t["d0b"])
    I = np.eye(nb)
    # direct-product order: mode 0 fastest
    H = -0.5 * (np.kron(I, D2) + np.kron(D2, I)) + 0.3 * np.kron(I, Q2) + 0.1 * np.kron(Q, Q)
    psi = np.random.default_rng(4).standard_normal((pg.N, 5))
    assert rel(pg.hpsi(psi), H @ psi) <= 1e-12
