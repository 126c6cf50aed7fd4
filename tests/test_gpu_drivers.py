"""Davidson and Chebyshev drivers on the GPU against the oracle and the reference's golden
vectors (through the C ABI)."""
import numpy as np
import pytest

from evrgpu import spec as S
from evrgpu import lib as E
from evrgpu.spec import FS_TO_AU
from oracle import oracle as O

pytestmark = pytest.mark.gpu

EIG_TOL = 1e-9  # au: FP64 Davidson against the oracle's dense spectrum


def dense_levels(spec, n, sym):
    H = O.OracleProblem(spec).dense()
    if sym:
        H = 0.5 * (H + H.T)
    return np.linalg.eigvalsh(0.5 * (H + H.T))[:n], H


def test_davidson_hh6d_matches_dense_oracle_and_benchmark(golden):
    spec = S.henon_heiles(6, 3)
    p = E.Problem(spec, device=0)
    ref, _ = dense_levels(spec, 28, sym=False)
    eig, vec, st = p.davidson(28, block=16, conv_resi=1e-7, conv_ene=1e-11, want_vectors=True)
    assert st["converged"]
    assert np.abs(eig - ref).max() <= EIG_TOL
    # 6D_Davidson_S0/benchmark: Davidson upper bounds of the same levels
    bench = np.array(golden["hh6d_levels"])
    assert (eig - bench).max() <= 1e-9 and np.abs(eig - bench).max() <= 2e-7
    # eigenvectors: orthonormal and H v = E v
    assert np.abs(vec.T @ vec - np.eye(28)).max() <= 1e-10
    hv = p.hpsi(vec)
    assert np.abs(hv - vec * eig).max() <= 1e-6


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_davidson_nonsymmetric_type10_uses_symmetrised_operator(prec):
    spec = S.config_sg4(4, 5, seed=5)
    p = E.Problem(spec, device=0)
    ref, _ = dense_levels(spec, 12, sym=True)
    eig, _, st = p.davidson(12, block=8, conv_resi=1e-8, conv_ene=1e-12, prec=prec)
    assert st["converged"], st
    assert np.abs(eig - ref).max() <= EIG_TOL
    if prec == "fp32":
        assert st["hpsi_fp32"] > 0 and st["hpsi_fp64"] > 0


def test_davidson_direct_product_fp32_refined_to_fp64():
    spec = S.config_dp3(nb=10, nq=12)
    p = E.Problem(spec, device=0)
    ref, _ = dense_levels(spec, 20, sym=True)
    eig, _, st = p.davidson(20, block=16, conv_resi=1e-8, conv_ene=1e-12, prec="fp32")
    assert st["converged"], st
    assert np.abs(eig - ref).max() <= EIG_TOL


def test_operator_forms_transpose_and_symmetrised():
    spec = S.config_sg4(4, 4, seed=9)
    p = E.Problem(spec, device=0)
    H = O.OracleProblem(spec).dense()
    rng = np.random.default_rng(5)
    x = rng.standard_normal((p.N, 6))
    for form, M in (("HT", H.T), ("HSYM", 0.5 * (H + H.T)), ("H", H)):
        p.set_operator(form)
        y = p.hpsi(x)
        ref = M @ x
        assert np.abs(y - ref).max() <= 1e-12 * np.abs(ref).max(), form


def _pyrazine_bounds(H):
    w = np.linalg.eigvals(H).real
    span = w.max() - w.min()
    return w.min() - 0.02 * span, w.max() + 0.02 * span


@pytest.mark.parametrize("steps_per_micro", [1, 4])
def test_chebyshev_pyrazine12d_matches_benchmark(golden, steps_per_micro):
    # 12D_propagation_S0/benchmark: autocorrelation every 0.1 fs up to 6 fs, checked at 1e-8
    spec = S.pyrazine_12d(1)
    p = E.Problem(spec, device=0)
    H = O.OracleProblem(spec).dense()
    emin, emax = _pyrazine_bounds(H)
    psi0 = np.zeros(p.N, dtype=np.complex128)
    psi0[p.Np] = 1.0  # |1,...,1> on electronic state 2
    ref = np.array(golden["pyr12d_autocorr"])
    dt = 0.1 * FS_TO_AU / steps_per_micro
    nsteps = (len(ref) - 1) * steps_per_micro
    ac, _, st = p.chebyshev(psi0, dt, nsteps, emin, emax, poly_tol=1e-13)
    ac = ac[::steps_per_micro, 0]
    assert st["status"] == -1
    assert np.abs(ac - (ref[:, 1] + 1j * ref[:, 2])).max() <= 1e-8


def test_chebyshev_batched_packets_match_exact_propagation():
    spec = S.config_sg4(3, 4, seed=7, nq_A=1)  # symmetric operator (nq = nb)
    p = E.Problem(spec, device=0)
    H = O.OracleProblem(spec).dense()
    Hs = 0.5 * (H + H.T)
    w, V = np.linalg.eigh(Hs)
    assert np.abs(H - Hs).max() < 1e-13
    rng = np.random.default_rng(3)
    psi0 = rng.standard_normal((p.N, 3)) + 1j * rng.standard_normal((p.N, 3))
    psi0 /= np.linalg.norm(psi0, axis=0)
    span = w[-1] - w[0]
    dt, nsteps = 40.0, 12
    ac, psi, st = p.chebyshev(psi0, dt, nsteps, w[0] - 0.05 * span, w[-1] + 0.05 * span, poly_tol=1e-14,
                              want_psi=True)
    assert st["status"] == -1
    c0 = V.T @ psi0
    exact_psi = V @ (np.exp(-1j * w * dt * nsteps)[:, None] * c0)
    assert np.abs(psi - exact_psi).max() <= 1e-10
    for n in range(nsteps + 1):
        ex = np.einsum("ij,ij->j", psi0.conj(), V @ (np.exp(-1j * w * dt * n)[:, None] * c0))
        assert np.abs(ac[n] - ex).max() <= 1e-10


def test_chebyshev_reports_spectrum_outside_bounds():
    spec = S.config_sg4(3, 3, seed=7, nq_A=1)
    p = E.Problem(spec, device=0)
    psi0 = np.zeros(p.N, dtype=np.complex128)
    psi0[0] = 1.0
    with pytest.raises(E.EvrError) as ei:
        # bounds far inside the spectrum: the expansion diverges, the call reports it
        p.chebyshev(psi0, 200.0, 3, 0.0, 1e-3, poly_tol=1e-12)
    assert ei.value.code == E.EVR_ENOCONV
    out = p.hpsi(np.ones((p.N, 1)))  # the context stays usable
    assert np.isfinite(out).all()


def test_davidson_hh21d_matches_dense_oracle_and_benchmark(golden):
    # 21-D Henon-Heiles on SG4 L=2 (21D_Davidson_S0/benchmark, 22 levels) through the
    # library: the GPU Davidson against the oracle's dense spectrum (1e-9 au) and the
    # benchmark's Davidson upper bounds (at or below each, within 2e-7 au)
    spec = S.henon_heiles(21, 2)
    p = E.Problem(spec, device=0)
    assert (p.Np, p.nterm, p.sum_nb) == (925, 253, 2059)
    ref, _ = dense_levels(spec, 22, sym=False)
    eig, _, st = p.davidson(22, block=16, conv_resi=1e-7, conv_ene=1e-11)
    assert st["converged"], st
    assert np.abs(eig - ref).max() <= EIG_TOL
    bench = np.array(golden["hh21d_levels"])
    assert (eig - bench).max() <= 1e-9 and np.abs(eig - bench).max() <= 2e-7


def test_chebyshev_pyrazine24d_matches_benchmark(golden):
    # 24-D two-state pyrazine on SG4 L=2 (24D_propagation_S0/benchmark, checked at 1e-8)
    m = golden["pyr24d_model"]
    spec = S.pyrazine_vibronic(m["w"], m["k1"], m["k2"], m["delta"], m["lam"], m["B"], m["L"])
    p = E.Problem(spec, device=0)
    assert (p.Np, p.nterm) == (1502, 325)
    H = O.OracleProblem(spec).dense()
    emin, emax = _pyrazine_bounds(H)
    psi0 = np.zeros(p.N, dtype=np.complex128)
    psi0[p.Np] = 1.0  # |1,...,1> on electronic state 2
    ref = np.array(golden["pyr24d_autocorr"])
    dt = ref[1, 0] - ref[0, 0]
    ac, _, st = p.chebyshev(psi0, dt, len(ref) - 1, emin, emax, poly_tol=1e-13)
    assert st["status"] == -1
    assert np.abs(ac[:, 0] - (ref[:, 1] + 1j * ref[:, 2])).max() <= 1e-8
