"""Gaussian filter diagonalisation (evr_filter_diag, sub_GaussianFilterDiagonalization).

CPU: the oracle's restatement (oracle/filter.py) on a small operator resolves levels of the
dense spectrum inside the window: every Ritz pair with a residual below 1e-6 au lies within
residual^2/gap + 1e-10 au of a dense eigenvalue, 16 filters converge at least three of
the window's levels, and more filters never converge fewer; the coefficients have the
properties the reference relies on (a bump at the filter's scaled energy, decaying tail).
GPU: the library against the oracle on the same start vectors: the same series length and
kept count, eigenvalues within 1e-9 au and residual norms within 1e-9 au + 1e-6 relative
on a small operator (the two orthonormalise by different but equivalent steps, so the
spanned subspace and its Ritz pairs agree to rounding); on the 6-D Henon-Heiles operator,
whose filtered basis keeps nearly dependent directions, within 1e-9 au + 1e-5 of each
pair's residual norm."""
import numpy as np
import pytest

from evrgpu import spec as S
from oracle import filter as OF
from oracle import oracle as O


def small_problem():
    return S.config_sg4(3, 4, seed=7, nq_A=1)  # symmetric operator (nq = nb), N = 165


def window_setup(H):
    w = np.linalg.eigvalsh(0.5 * (H + H.T))
    hmin, hmax = w[0], w[-1]
    e0, width = w[3], 6.0 * (w[6] - w[0]) / 6.0  # a window over the lowest levels
    return w, hmin, hmax, e0, width


def test_oracle_filter_finds_the_window_levels():
    op = O.OracleProblem(small_problem())
    H = op.dense()
    w, hmin, hmax, e0, width = window_setup(H)
    rng = np.random.default_rng(5)
    q = rng.standard_normal(op.N)
    r = OF.filter_diag(lambda x: H @ x, q / np.linalg.norm(q), hmin, hmax, e0, width, 16, 4000, conv_resi=1e-6)
    assert 4 <= r["nb"] <= 4001 and r["in_window"] <= r["keep"] <= 16
    assert r["conv_in_window"] >= 3
    good = r["resid"] < 1e-6
    for e, res in zip(r["eig"][good], r["resid"][good]):
        k = np.argmin(np.abs(w - e))
        gap = np.min(np.abs(np.delete(w, k) - w[k]))
        assert abs(e - w[k]) <= res ** 2 / gap + 1e-10
    # Ritz values never fall below the spectrum, and more filters resolve more levels
    assert r["eig"][0] >= w[0] - 1e-12
    r8 = OF.filter_diag(lambda x: H @ x, q / np.linalg.norm(q), hmin, hmax, e0, width, 8, 4000, conv_resi=1e-6)
    assert r8["conv_in_window"] <= r["conv_in_window"]


def test_oracle_filter_coefficients_represent_gaussians():
    # the series sum_n f(n, l) T_n(x) is a smooth bump centred at the filter's energy, and
    # the coefficients decay (the tail that ends the series-length loop)
    st = OF.setup(0.0, 1.0, 0.3, 0.1, 6, 4000)
    f, nb = st["f"], st["nb"]
    x = np.linspace(-0.999, 0.999, 4001)
    T = np.polynomial.chebyshev.chebvander(x, nb - 1)
    for l in range(6):
        g = T @ f[:, l]
        cl = ((st["lmin"] + l * 0.1 / 5) - st["E0"]) / st["Esc"]
        assert abs(x[np.argmax(g)] - cl) < 0.02
        assert np.abs(f[nb - 4:, l]).sum() / 3.0 < 1e-6
    assert np.abs(f[nb - 4:nb, 2]).sum() / 3.0 < 1e-8 or nb > 4000


@pytest.mark.gpu
@pytest.mark.parametrize("nstart", [1, 2])
def test_gpu_filter_matches_oracle(nstart):
    from evrgpu import lib as E

    spec = small_problem()
    op = O.OracleProblem(spec)
    H = op.dense()
    w, hmin, hmax, e0, width = window_setup(H)
    rng = np.random.default_rng(11)
    q = rng.standard_normal((op.N, nstart))
    q /= np.linalg.norm(q, axis=0)
    ref = OF.filter_diag(lambda x: H @ x, q, hmin, hmax, e0, width, 10, 4000, conv_resi=1e-6)
    p = E.Problem(spec, device=0)
    out = p.filter_diag(hmin, hmax, e0, width, 10, max_order=4000, q0=q, conv_resi=1e-6, want_vectors=True)
    assert out["order"] == ref["nb"] and out["kept"] == ref["keep"]
    assert out["hpsi"] == nstart * (ref["nb"] - 1) + ref["keep"]
    assert abs(out["lambda_min"] - ref["lmin"]) < 1e-15 and abs(out["lambda_max"] - ref["lmax"]) < 1e-15
    assert np.abs(out["eig"] - ref["eig"]).max() <= 1e-9
    assert np.all(np.abs(out["resid"] - ref["resid"]) <= 1e-9 + 1e-6 * ref["resid"])
    assert out["in_window"] == ref["in_window"] and out["converged_in_window"] == ref["conv_in_window"]
    # the Ritz vectors: orthonormal, and H v - E v has the reported norms
    V = out["vec"]
    assert np.abs(V.T @ V - np.eye(V.shape[1])).max() <= 1e-10
    R = H @ V - V * out["eig"]
    assert np.allclose(np.linalg.norm(R, axis=0), out["resid"], rtol=1e-6, atol=1e-10)


@pytest.mark.gpu
def test_gpu_filter_hh6d_matches_oracle():
    # the 6-D Henon-Heiles benchmark operator (SG4 L=3), two start vectors and 16 filters
    # over a window of its dense low spectrum: same Ritz pairs as the oracle
    from evrgpu import lib as E

    spec = S.henon_heiles(6, 3)
    op = O.OracleProblem(spec)
    H = op.dense()
    w = np.linalg.eigvalsh(0.5 * (H + H.T))
    rng = np.random.default_rng(3)
    q = rng.standard_normal((op.N, 2))
    q /= np.linalg.norm(q, axis=0)
    e0, width = 4.4, 1.2
    ref = OF.filter_diag(lambda x: H @ x, q, w[0], w[-1], e0, width, 16, 20000)
    p = E.Problem(spec, device=0)
    out = p.filter_diag(w[0], w[-1], e0, width, 16, max_order=20000, q0=q)
    assert out["order"] == ref["nb"] and out["kept"] == ref["keep"]
    # the filtered basis keeps directions down to an overlap eigenvalue of 1e-9, which
    # rounding perturbs: Ritz values of unconverged pairs (residuals ~1e-2 here) move with
    # them, converged ones do not
    assert np.all(np.abs(out["eig"] - ref["eig"]) <= 1e-9 + 1e-5 * ref["resid"])
    assert np.all(np.abs(out["resid"] - ref["resid"]) <= 1e-9 + 1e-5 * ref["resid"])


@pytest.mark.gpu
def test_gpu_filter_rejects_bad_options():
    from evrgpu import lib as E

    p = E.Problem(small_problem(), device=0)
    for kw in (dict(n_filters=1), dict(width=-1.0), dict(max_order=2)):
        args = dict(hmin=0.0, hmax=1.0, e0=0.1, width=0.05, n_filters=4, max_order=100)
        args.update(kw)
        with pytest.raises(E.EvrError) as ei:
            p.filter_diag(**args)
        assert ei.value.code == E.EVR_EINVAL
