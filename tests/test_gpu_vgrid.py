"""evr_set_vgrid: a potential handed over as grid values (as a Fortran host's calcN_op grid
cache holds it) replaces the one the context evaluated from its monomials.

Parity: after set_vgrid(values), H.psi equals H.psi of the problem whose potential gave
those values (FP64 1e-12 relative, FP32 2e-5), in both layouts, on the Smolyak term kernels
(two states, dropped 1-point modes) and the direct-product stage kernels.
"""
import dataclasses

import numpy as np
import pytest

from evrgpu import spec as S
from evrgpu import lib as E
from oracle import oracle as O

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
FP32_TOL = 2e-5


def rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


def with_v_scaled(spec, s):
    return dataclasses.replace(spec, mono_coef=np.asarray(spec.mono_coef) * s)


def terms_to_ref(v, pg, spec):
    """Terms layout (evr_get_vgrid) -> the reference's OpGrid%Grid(sum_nq, nb0, nb0)."""
    nb2 = spec.nb0 ** 2
    term_l = pg.tables()["term_l"]
    nq = [[pg.basis(d, l)["nq"] for l in range(spec.LG + 1)] for d in range(spec.D)]
    out = np.zeros(pg.sum_nq * nb2)
    off = 0
    for t in range(pg.nterm):
        NQ = int(np.prod([nq[d][term_l[t, d]] for d in range(spec.D)]))
        blk = v[off * nb2:(off + NQ) * nb2].reshape(nb2, NQ)
        for ab in range(nb2):
            out[ab * pg.sum_nq + off: ab * pg.sum_nq + off + NQ] = blk[ab]
        off += NQ
    assert off == pg.sum_nq
    return out


def test_set_vgrid_sg4_two_states_both_layouts():
    spec = S.pyrazine_12d(1)
    pa = E.Problem(spec)
    pb = E.Problem(with_v_scaled(spec, 0.0))
    v = pa.vgrid()
    psi = np.random.default_rng(4).standard_normal((pa.N, 5))
    ref64, ref32 = pa.hpsi(psi), pa.hpsi(psi, prec="fp32")
    assert rel(pb.hpsi(psi), ref64) > 1e-3  # the zero-potential problem differs before the update
    pb.set_vgrid(v)
    assert np.abs(pb.vgrid() - v).max() <= 1e-15 * np.abs(v).max()
    assert rel(pb.hpsi(psi), ref64) <= FP64_TOL
    assert rel(pb.hpsi(psi, prec="fp32"), ref32) <= FP32_TOL
    pc = E.Problem(with_v_scaled(spec, 0.0))
    pc.set_vgrid(terms_to_ref(v, pc, spec), layout="ref")
    assert rel(pc.hpsi(psi), ref64) <= FP64_TOL


def test_set_vgrid_direct_product_stage_kernels():
    spec = S.config_dp3(nb=8, nq=10)
    pg = E.Problem(spec)
    pg.set_vgrid(2.0 * pg.vgrid())
    po = O.OracleProblem(with_v_scaled(spec, 2.0))
    psi = np.random.default_rng(5).standard_normal((pg.N, 4))
    assert rel(pg.hpsi(psi), po.hpsi(psi)) <= FP64_TOL


def test_set_dipole_grid_matches_monomial_dipole():
    """evr_set_dipole_grid against evr_set_dipole on the same mu: the field operators
    H0 - E mu and mu alone, and the control propagation (whose spectral range the dipole
    bound widens)."""
    from oracle import control as OC
    sp = S.config_oc(seed=1, nb=6, nq=8, D=3)
    pa = E.Problem(sp)  # dipole from its monomials
    no_dip = dict(dip_coef=None, dip_idx=None, dip_elec=None)
    mu = E.Problem(dataclasses.replace(sp, mono_coef=sp.dip_coef, mono_idx=sp.dip_idx, mono_elec=sp.dip_elec,
                                       **no_dip)).vgrid()  # mu on the grid, as a potential
    pb = E.Problem(dataclasses.replace(sp, **no_dip))
    pb.set_dipole_grid(mu)
    psi = np.random.default_rng(6).standard_normal((pa.N, 3))
    for vw, mw, keo in ((1.0, -0.02, True), (0.0, 1.0, False)):
        pa.set_field(vw, mw, keo)
        pb.set_field(vw, mw, keo)
        assert rel(pb.hpsi(psi), pa.hpsi(psi)) <= FP64_TOL
    pa.set_field(1.0, 0.0, True)
    pb.set_field(1.0, 0.0, True)
    H0, _ = OC.operators(O.OracleProblem(sp))
    w = np.sort(np.linalg.eigvals(H0).real)
    psi0 = np.zeros(pa.N, dtype=complex)
    psi0[0] = 1.0
    target = np.zeros(pa.N, dtype=complex)
    target[3] = 1.0
    field = S.oc_field(20, 10.0, seed=3, amp=0.01)
    Ja = pa.oc_forward(field, psi0, target, 10.0, w[0] - 1e-3, w[-1] + 1e-3)[0]
    Jb = pb.oc_forward(field, psi0, target, 10.0, w[0] - 1e-3, w[-1] + 1e-3)[0]
    assert abs(Ja - Jb) <= 1e-12


def _g_linear(spec, Q):
    """G(Q) = G0 + sum_k g[:, :, k] Q_k at the points Q (npoints x D)."""
    return np.asarray(spec.G0)[None] + np.einsum("ijk,qk->qij", np.asarray(spec.g), Q)


@pytest.mark.parametrize("mk", [lambda: S.config_sg4(4, 5, seed=5), lambda: S.config_dp3(nb=6, nq=8)],
                         ids=["sg4_term_kernels", "dp_stage_kernels"])
def test_set_ggrid_matches_the_linear_model(mk):
    """evr_set_ggrid: a context made with constant G, given G(Q) = G0 + g.Q as grid values,
    applies the same H as the context that evaluated that model itself."""
    from test_host_tables import grid_points
    spec = mk()
    pa = E.Problem(spec)
    pb = E.Problem(dataclasses.replace(spec, g=np.zeros_like(np.asarray(spec.g))))  # no G table yet
    G = _g_linear(spec, grid_points(pb, spec))
    psi = np.random.default_rng(8).standard_normal((pa.N, 5))
    ref64, ref32 = pa.hpsi(psi), pa.hpsi(psi, prec="fp32")
    assert rel(pb.hpsi(psi), ref64) > 1e-6  # constant G differs before the update
    pb.set_ggrid(G)
    assert rel(pb.hpsi(psi), ref64) <= FP64_TOL
    assert rel(pb.hpsi(psi, prec="fp32"), ref32) <= FP32_TOL
