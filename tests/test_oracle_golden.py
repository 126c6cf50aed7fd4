"""Pins the CPU oracle to the reference's own golden vectors (no GPU needed)."""
import numpy as np
import pytest

from evrgpu import spec as S
from oracle import oracle as O


@pytest.mark.parametrize("n", list(range(1, 41)))
def test_gauss_hermite_matches_reference_tables(golden, n):
    # Internal_data/HermQuadra/herm<n>.txt, read by sub_quadra_herm.f90:322-343
    ref = np.array(golden["herm"][str(n)])
    x, w = O.gauss_hermite(n)
    assert np.max(np.abs(x - ref[:, 0])) <= 4e-15 * max(1.0, np.abs(ref[:, 0]).max())
    assert np.max(np.abs(w - ref[:, 1]) / ref[:, 1]) <= 1e-13


def test_hh6d_spectrum_matches_davidson_benchmark(golden):
    # Working_tests/MPI_tests/6D_Davidson_S0/benchmark: Davidson levels from a run
    # with conv_resi = 5e-4 au, i.e. variational upper bounds of the exact levels to
    # ~(5e-4)^2.  The oracle's dense spectrum of the same SG4 operator must lie at or
    # below each level, within 2e-7 au.
    ref = np.array(golden["hh6d_levels"])
    op = O.OracleProblem(S.henon_heiles(6, 3))
    assert (op.Np, op.nterm, op.sum_nb) == (377, 84, 1216)
    H = op.dense()
    assert np.abs(H - H.T).max() < 1e-12
    ev = np.linalg.eigvalsh(0.5 * (H + H.T))[: len(ref)]
    d = ev - ref
    assert d.max() <= 1e-9
    assert np.abs(d).max() <= 2e-7


def test_hh21d_spectrum_matches_davidson_benchmark(golden):
    # Working_tests/MPI_tests/21D_Davidson_S0/benchmark: 22 levels of the 21-D Henon-Heiles
    # model on SG4 L=2 (same potential file as the 6-D case), from a Davidson run with
    # conv_resi = 5e-4 au.  The oracle's dense spectrum lies at or below each level, within
    # 2e-7 au.  (The GPU library runs the same case in tests/test_gpu_drivers.py.)
    ref = np.array(golden["hh21d_levels"])
    op = O.OracleProblem(S.henon_heiles(21, 2))
    assert (op.Np, op.nterm, op.sum_nb) == (925, 253, 2059)
    H = op.dense()
    assert np.abs(H - H.T).max() < 1e-12
    ev = np.linalg.eigvalsh(0.5 * (H + H.T))[: len(ref)]
    d = ev - ref
    assert d.max() <= 1e-9
    assert np.abs(d).max() <= 2e-7


def test_pyrazine12d_autocorrelation_matches_benchmark(golden):
    # Working_tests/MPI_tests/12D_propagation_S0/benchmark (checked at 1e-8 by MPI_test.sh):
    # exact propagation of psi0 = |1..1> on electronic state 2 with the oracle's operator.
    ref = np.array(golden["pyr12d_autocorr"])
    op = O.OracleProblem(S.pyrazine_12d(1))
    assert (op.Np, op.nterm) == (27, 13)
    H = op.dense()
    psi0 = np.zeros(op.N)
    psi0[op.Np] = 1.0
    w, V = np.linalg.eig(H)
    c0 = np.linalg.solve(V, psi0)
    for t, re, im, _ in ref:
        C = np.vdot(psi0, V @ (np.exp(-1j * w * t) * c0))
        assert abs(C - (re + 1j * im)) < 1e-8


def test_term_and_packed_tables_sg4_6d_l8():
    # Sizes of the D=6, L=8 Smolyak workload (nb=2l+1, nq=2l+3)
    op = O.OracleProblem(S.config_sg4_6d_l8())
    assert (op.nterm, op.Np, op.sum_nb, op.sum_nq) == (2975, 40081, 860455, 37769167)
    t = op.tables()
    assert set(np.unique(t["weight"])) <= {-10.0, -5.0, -1.0, 1.0, 5.0, 10.0}
    assert t["map"].min() == 0 and t["map"].max() == op.Np - 1


def test_pyrazine24d_autocorrelation_matches_benchmark(golden):
    # Working_tests/MPI_tests/24D_propagation_S0/benchmark (checked at 1e-8 by MPI_test.sh):
    # the 24-D two-state pyrazine model of that run (parameters read from its potential file
    # into the fixture), SG4 L=2, exact propagation of |1..1> on electronic state 2.
    m = golden["pyr24d_model"]
    ref = np.array(golden["pyr24d_autocorr"])
    sp = S.pyrazine_vibronic(m["w"], m["k1"], m["k2"], m["delta"], m["lam"], m["B"], m["L"])
    op = O.OracleProblem(sp)
    assert (op.Np, op.nterm) == (1502, 325)
    H = op.dense()
    assert np.abs(H - H.T).max() < 1e-12
    w, V = np.linalg.eigh(0.5 * (H + H.T))
    psi0 = np.zeros(op.N)
    psi0[op.Np] = 1.0
    c0 = V.T @ psi0
    for t, re, im, _ in ref:
        a = psi0 @ (V @ (np.exp(-1j * w * t) * c0))
        assert abs(a - (re + 1j * im)) <= 1e-8
