"""Restarted Lanczos (evr_lanczos), the library's form of the reference's ARPACK path
(sub_propagation_Arpack_Sym, Source_ElVibRot/sub_propagation/sub_module_Arpack.f90:680).

ARPACK itself is a third-party library that the reference's tree does not hold, so the
parity is anchored on exact answers: the lowest levels of the oracle's dense operator
(numpy eigh) to 1e-10 au, the reference's own 6-D Henon-Heiles benchmark levels (at or
below each, as the Davidson test), the relative residuals |H x - E x|/|E| the call reports
recomputed on the host, and orthonormal Ritz vectors."""
import numpy as np
import pytest

from evrgpu import spec as S
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def dense_levels(spec, sym=False):
    H = O.OracleProblem(spec).dense()
    return H, np.linalg.eigvalsh(0.5 * (H + H.T) if sym else H)


def test_lanczos_small_operator_matches_dense():
    from evrgpu import lib as E

    spec = S.config_sg4(3, 4, seed=7, nq_A=1)  # symmetric operator (nq = nb)
    H, w = dense_levels(spec)
    p = E.Problem(spec, device=0)
    eig, vec, rres, st = p.lanczos(6, want_vectors=True)
    assert st["converged"] == 6 and st["ncv"] == 22
    assert np.abs(eig - w[:6]).max() <= 1e-10
    assert np.abs(vec.T @ vec - np.eye(6)).max() <= 1e-10
    r = np.linalg.norm(H @ vec - vec * eig, axis=0) / np.abs(eig)
    assert np.allclose(r, rres, rtol=1e-3, atol=1e-13)
    assert rres.max() <= 1e-8
    # a restart happens with a small basis, and the levels stay the same
    eig2, _, _, st2 = p.lanczos(6, ncv=9, max_restarts=500)
    assert st2["restarts"] > 1 and st2["converged"] == 6
    assert np.abs(eig2 - w[:6]).max() <= 1e-10


def test_lanczos_full_basis_is_exact():
    """ncv = min(N, 2 nev + 10) reaches N on a small problem (N = 13 here): one sweep spans
    the space and every level comes out exact, without a restart."""
    from evrgpu import lib as E

    spec = S.config_sg4(2, 2, seed=7, nq_A=1)
    H, w = dense_levels(spec)
    p = E.Problem(spec, device=0)
    assert p.N == 13
    eig, vec, rres, st = p.lanczos(3, want_vectors=True)
    assert st["ncv"] == 13 and st["restarts"] == 1 and st["converged"] == 3
    assert np.abs(eig - w[:3]).max() <= 1e-11
    assert np.abs(vec.T @ vec - np.eye(3)).max() <= 1e-11
    assert rres.max() <= 1e-11


def test_lanczos_hh6d_matches_dense_and_benchmark(golden):
    from evrgpu import lib as E

    spec = S.henon_heiles(6, 3)
    H, w = dense_levels(spec)
    p = E.Problem(spec, device=0)
    eig, _, rres, st = p.lanczos(10)
    assert st["converged"] == 10
    assert np.abs(eig - w[:10]).max() <= 1e-9
    bench = np.array(golden["hh6d_levels"])[:10]
    assert np.all(eig <= bench + 1e-9) and np.abs(eig - bench).max() <= 2e-7


def test_lanczos_nonsymmetric_type10_uses_symmetrised_operator():
    from evrgpu import lib as E

    spec = S.config_sg4(4, 3, seed=2)  # nq > nb: H is not symmetric
    H, w = dense_levels(spec, sym=True)
    p = E.Problem(spec, device=0)
    eig, _, _, st = p.lanczos(5, sym=-1)
    assert st["converged"] == 5
    assert np.abs(eig - w[:5]).max() <= 1e-10


def test_lanczos_rejects_bad_options():
    from evrgpu import lib as E

    p = E.Problem(S.config_sg4(3, 4, seed=7, nq_A=1), device=0)
    for kw in (dict(nev=0), dict(nev=5, ncv=5), dict(nev=5, max_restarts=0)):
        with pytest.raises(E.EvrError) as ei:
            p.lanczos(**kw)
        assert ei.value.code == E.EVR_EINVAL
