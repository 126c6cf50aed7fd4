"""A general Tnum metric on the type-10 operator: G(Q), the Jacobian and rho as grid values
(evr_set_ggrid, evr_set_jacobian), against the oracle's restatement of
sub_TabOpPsi_OF_ONEDP_FOR_SGtype4 with Jac and sqRhoOVERJac
(Source_ElVibRot/sub_Operator/sub_OpPsi_SG4.f90:1579-1620).

Tolerances: FP64 1e-12 relative (max norm), FP32 2e-5.
"""
import numpy as np
import pytest

from evrgpu import spec as S
from evrgpu import lib as E
from oracle import oracle as O
from test_host_tables import grid_points

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


def metric(spec, Q):
    """A non-linear metric of the points Q (npoints x D): G = G0 + g.Q + 0.01 diag(Q^2 s^2),
    Jac = 1 + 0.2 tanh(sum_k a_k q_k), rho = Jac (1 + 0.1 q_0^2 / (1 + q_0^2)), with q = s Q
    the dimensionless coordinates (s = scaleQ)."""
    s = np.asarray(spec.scaleQ)
    q = Q * s[None, :]
    D = spec.D
    G = np.asarray(spec.G0)[None] + np.einsum("ijk,pk->pij", np.asarray(spec.g), Q)
    G = G + 0.01 * np.einsum("pi,ij->pij", q ** 2, np.eye(D))
    a = np.linspace(0.3, -0.2, D)
    jac = 1.0 + 0.2 * np.tanh(q @ a)
    rho = jac * (1.0 + 0.1 * q[:, 0] ** 2 / (1.0 + q[:, 0] ** 2))
    return G, jac, rho


CASES = {
    "sg4_d4_l5": lambda: S.config_sg4(4, 5, seed=5),
    "sg4_d6_l4": lambda: S.config_sg4(6, 4, seed=6),
    "dp3_nb6_nq8": lambda: S.config_dp3(nb=6, nq=8),
}


@pytest.mark.parametrize("name", list(CASES))
def test_jacobian_and_metric_grid_match_oracle(name):
    spec = CASES[name]()
    pg = E.Problem(spec, device=0)
    po = O.OracleProblem(spec)
    G, jac, rho = metric(spec, grid_points(pg, spec))
    pg.set_ggrid(G)
    pg.set_jacobian(jac, rho)
    po.set_metric(jac=jac, rho=rho, G=G)
    psi = np.random.default_rng(3).standard_normal((pg.N, 7))
    ref = po.hpsi(psi)
    assert rel(pg.hpsi(psi), ref) <= 1e-12
    assert rel(pg.hpsi(psi, prec="fp32"), ref) <= 2e-5
    # without the Jacobian the same context is back to the G-grid operator
    pg.set_jacobian(None, None)
    po.set_metric(jac=None, rho=None, G=G)
    assert rel(pg.hpsi(psi), po.hpsi(psi)) <= 1e-12


def test_jacobian_operator_forms_direct_product():
    # H^T and (H + H^T)/2 of the operator with a Jacobian (the transposed pipeline takes
    # the point factors in the reverse order)
    spec = S.config_dp3(nb=5, nq=7)
    pg = E.Problem(spec, device=0)
    po = O.OracleProblem(spec)
    G, jac, rho = metric(spec, grid_points(pg, spec))
    pg.set_ggrid(G)
    pg.set_jacobian(jac, rho)
    po.set_metric(jac=jac, rho=rho, G=G)
    H = po.dense()
    psi = np.random.default_rng(5).standard_normal((pg.N, 4))
    try:
        for form, ref in (("HT", H.T @ psi), ("HSYM", 0.5 * (H + H.T) @ psi), ("H", H @ psi)):
            pg.set_operator(form)
            assert rel(pg.hpsi(psi), ref) <= 1e-12, form
    finally:
        pg.set_operator("H")


def test_constant_jacobian_and_rho_leave_the_operator_unchanged():
    spec = S.config_sg4(4, 4, seed=9)
    pg = E.Problem(spec, device=0)
    psi = np.random.default_rng(6).standard_normal((pg.N, 3))
    ref = pg.hpsi(psi)
    pg.set_jacobian(np.full(pg.sum_nq, 2.5), np.full(pg.sum_nq, 0.7))
    assert rel(pg.hpsi(psi), ref) <= 1e-12
