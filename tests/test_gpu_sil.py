"""Short-iterative-Lanczos propagation (evr_sil_propagate, march_SIL) on the GPU against
exact propagation (eigen-decomposition of the oracle's dense H, 1e-10) and against the
reference's own 12-D pyrazine autocorrelation benchmark (its script's 1e-8)."""
import numpy as np
import pytest

from evrgpu import spec as S
from evrgpu import lib as E
from evrgpu.spec import FS_TO_AU
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def test_sil_packets_match_exact_propagation():
    spec = S.config_sg4(3, 4, seed=7, nq_A=1)  # symmetric operator (nq = nb)
    p = E.Problem(spec, device=0)
    H = O.OracleProblem(spec).dense()
    w, V = np.linalg.eigh(0.5 * (H + H.T))
    rng = np.random.default_rng(3)
    psi0 = rng.standard_normal((p.N, 3)) + 1j * rng.standard_normal((p.N, 3))
    psi0 /= np.linalg.norm(psi0, axis=0)
    psi0[:, 2] *= 0.5  # packets need not be normalised
    dt, nsteps = 40.0, 12
    ac, psi, st = p.sil(psi0, dt, nsteps, npoly=64, poly_tol=1e-13, want_psi=True)
    assert st["status"] == -1 and 1 <= st["krylov_dim"] < 64
    c0 = V.T @ psi0
    exact_psi = V @ (np.exp(-1j * w * dt * nsteps)[:, None] * c0)
    assert np.abs(psi - exact_psi).max() <= 1e-10
    for n in range(nsteps + 1):
        ex = np.einsum("ij,ij->j", psi0.conj(), V @ (np.exp(-1j * w * dt * n)[:, None] * c0))
        assert np.abs(ac[n] - ex).max() <= 1e-10


def test_sil_pyrazine12d_matches_benchmark(golden):
    spec = S.pyrazine_12d(1)
    p = E.Problem(spec, device=0)
    psi0 = np.zeros(p.N, dtype=np.complex128)
    psi0[p.Np] = 1.0  # |1,...,1> on electronic state 2
    ref = np.array(golden["pyr12d_autocorr"])
    ac, _, st = p.sil(psi0, 0.1 * FS_TO_AU, len(ref) - 1, npoly=100, poly_tol=1e-13)
    assert st["status"] == -1
    assert np.abs(ac[:, 0] - (ref[:, 1] + 1j * ref[:, 2])).max() <= 1e-8
