"""Algebra of the type-10 operator on CPU, from the oracle's 1-D tables.

For one direct-product term (sub_OpPsi_WITH_MemGrid_BGG_Hamil10,
Source_ElVibRot/sub_Operator/sub_OpPsi.f90:1528-1794) the operator is
    H = B^T W (V - 1/2 sum_ij D_i G_ij D_j) B,
B the basis->grid product of the d0b, W the product grid weights, D_i the grid derivative
d1gg of mode i, G_ij(Q) the metric per grid point.  The first test rebuilds H with dense
Kronecker products and compares it with the oracle's H.psi (nq > nb, a host G(Q) grid).
The second checks the fused form of the symmetrised operator that one basis->grid and one
grid->basis chain serve:
    (H + H^T)/2 psi = B^T [W V u - 1/4 W sum_i D_i sum_j G_ij D_j u
                           - 1/4 sum_j D_j^T sum_i G_ij D_i^T (W u)],  u = B psi,
on the same operator, which is not symmetric (nq > nb), so the identity is not trivial.
"""
import numpy as np
import pytest

from evrgpu import spec as S
from oracle import oracle as O


@pytest.fixture(scope="module")
def dp2():
    omega = np.array([0.010, 0.006])
    rng = np.random.default_rng(3)
    c, idx, el, g = S.anharmonic_poly(2, omega, rng, 1e-5, 1e-6, 0.01)
    spec = S.ProblemSpec(kind="dp", D=2, nq_dp=[9, 8], nb_dp=[6, 5], scaleQ=np.sqrt(omega), mono_coef=c,
                         mono_idx=idx, mono_elec=el, keo_type=10, g=g, name="DP2_type10")
    po = O.OracleProblem(spec)
    b0, b1 = po.basis(0, 0), po.basis(1, 0)
    nq = b0["nq"] * b1["nq"]
    rg = np.random.default_rng(5)
    Gq = np.empty((nq, 2, 2))
    for q in range(nq):
        a = 0.05 * rg.standard_normal((2, 2))
        Gq[q] = np.eye(2) + 0.5 * (a + a.T)
    po.set_metric(G=Gq)
    # grid and basis order: mode 0 fastest
    B = np.kron(b1["d0b"], b0["d0b"])
    W = np.kron(b1["w"], b0["w"])
    Dm = [np.kron(np.eye(b1["nq"]), b0["d1gg"]), np.kron(b1["d1gg"], np.eye(b0["nq"]))]
    return dict(H=po.dense(), B=B, W=W, V=po.vgrid(), D=Dm, G=Gq, N=po.N)


def test_type10_operator_is_the_grid_sandwich(dp2):
    B, W, V, Dm, G = dp2["B"], dp2["W"], dp2["V"], dp2["D"], dp2["G"]
    K = sum(Dm[i] @ np.diag(G[:, i, j]) @ Dm[j] for i in range(2) for j in range(2))
    H = B.T @ np.diag(W) @ (np.diag(V) - 0.5 * K) @ B
    ref = dp2["H"]
    assert np.abs(H - ref).max() <= 1e-13 * np.abs(ref).max()


def test_fused_symmetrised_operator(dp2):
    B, W, V, Dm, G, H = dp2["B"], dp2["W"], dp2["V"], dp2["D"], dp2["G"], dp2["H"]
    scale = np.abs(H).max()
    assert np.abs(H - H.T).max() > 1e-3 * scale  # nq > nb: H is not symmetric
    u = B @ np.eye(dp2["N"])
    a = (W * V)[:, None] * u
    a -= 0.25 * W[:, None] * sum(Dm[i] @ (G[:, i, j][:, None] * (Dm[j] @ u)) for i in range(2) for j in range(2))
    Wu = W[:, None] * u
    a -= 0.25 * sum(Dm[j].T @ (G[:, i, j][:, None] * (Dm[i].T @ Wu)) for i in range(2) for j in range(2))
    assert np.abs(B.T @ a - 0.5 * (H + H.T)).max() <= 1e-13 * scale
