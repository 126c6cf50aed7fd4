"""Field coupling and the optimal-control gradient on the GPU against the oracle.

* H0 - E mu, mu alone and H0 through evr_set_field on every kernel path: 1e-12 relative
  to the oracle (fcn_field's (H - E Dip), sub_module_propa_march.f90:1494-1503).
* evr_oc_forward: J = |<target|psi(T)>|^2 against exact matrix-exponential propagation,
  1e-10 absolute.
* evr_oc_backward: the adjoint gradient against the exact gradient of the discrete problem
  (Frechet derivative of expm), 1e-8 relative to max |dJ/dE|; against central finite
  differences of the GPU forward pass (h = 1e-7), 1e-6 relative; the same for every
  checkpoint interval; the continuous-time build_field gradient (sub_control.f90:955-975)
  against the oracle's, 1e-9 relative.
"""
import numpy as np
import pytest

from evrgpu import spec as S
from evrgpu import lib as E
from oracle import control as OC
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def sg4_with_dipole(D=4, L=4, seed=2):
    sp = S.config_sg4(D, L, seed=seed)
    rng = np.random.default_rng(seed + 100)
    sp.dip_coef, sp.dip_idx, sp.dip_elec = S.dipole_poly(D, sp.extra["omega"], rng)
    return sp


FIELD_CASES = {
    "dp3_nb6_nq8": lambda: S.config_oc(seed=1, nb=6, nq=8, D=3),
    "sg4_d4_l4": sg4_with_dipole,
}


@pytest.mark.parametrize("path", [1, 2, 0], ids=["auto", "slab", "general"])
@pytest.mark.parametrize("name", list(FIELD_CASES))
def test_field_operator_matches_oracle(name, path):
    sp = FIELD_CASES[name]()
    pg = E.Problem(sp, device=0)
    po = O.OracleProblem(sp)
    pg.set_kernel_path(path)
    rng = np.random.default_rng(9)
    psi = rng.standard_normal((pg.N, 5))
    for vw, mw, keo in ((1.0, -0.02, True), (0.0, 1.0, False), (1.0, 0.0, True), (0.5, 0.3, False)):
        pg.set_field(vw, mw, keo)
        po.set_field(vw, mw, keo)
        ref = po.hpsi(psi)
        assert rel(pg.hpsi(psi), ref) <= 1e-12
        assert rel(pg.hpsi(psi, prec="fp32"), ref) <= 2e-5


def test_field_without_dipole_is_rejected():
    pg = E.Problem(S.config_dp3(nb=4, nq=5), device=0)
    with pytest.raises(E.EvrError) as ei:
        pg.set_field(1.0, -0.01, True)
    assert ei.value.code == E.EVR_EINVAL


class Case:
    def __init__(self, nb=6, nq=8, D=3, nst=30, dt=10.0, seed=4, amp=0.01):
        self.sp = S.config_oc(seed=seed, nb=nb, nq=nq, D=D)
        self.pg = E.Problem(self.sp, device=0)
        op = O.OracleProblem(self.sp)
        self.H0, self.M = OC.operators(op)
        w, v = np.linalg.eig(self.H0)
        order = np.argsort(w.real)
        w, v = w.real[order], v[:, order].real
        self.psi0 = v[:, 0] / np.linalg.norm(v[:, 0]) + 0j
        self.target = v[:, 3] / np.linalg.norm(v[:, 3]) + 0j
        self.field = S.oc_field(nst, dt, seed=seed + 1, amp=amp)
        self.dt = dt
        self.emin, self.emax = w[0] - 1e-3, w[-1] + 1e-3

    def forward(self, field=None, checkpoint=0):
        f = self.field if field is None else field
        return self.pg.oc_forward(f, self.psi0, self.target, self.dt, self.emin, self.emax, checkpoint=checkpoint)


_cases = {}


def case(key):
    if key not in _cases:
        _cases[key] = Case() if key == "nonsym" else Case(nb=6, nq=6, seed=7)
    return _cases[key]


@pytest.mark.parametrize("key", ["nonsym", "sym"])
def test_oc_forward_matches_exact_propagation(key):
    c = case(key)
    J, ovl, _, info = c.forward()
    Jx, ovlx = OC.objective(c.H0, c.M, c.field, c.dt, c.psi0, c.target)
    assert abs(J - Jx) <= 1e-10
    assert abs(ovl - ovlx) <= 1e-10
    assert info["order"] >= 2


@pytest.mark.parametrize("key", ["nonsym", "sym"])
def test_oc_gradient_matches_exact_gradient(key):
    c = case(key)
    c.forward()
    g, ref, info = c.pg.oc_backward(len(c.field))
    gx = OC.gradient_exact(c.H0, c.M, c.field, c.dt, c.psi0, c.target)
    assert rel(g, gx) <= 1e-8
    rx = OC.gradient_continuous(c.H0, c.M, c.field, c.dt, c.psi0, c.target)
    assert rel(ref, rx) <= 1e-9


def test_oc_gradient_matches_finite_differences():
    c = case("nonsym")
    c.forward()
    g, _, _ = c.pg.oc_backward(len(c.field))
    h = 1e-7
    for n in (0, len(c.field) // 2, len(c.field) - 1):
        fp, fm = c.field.copy(), c.field.copy()
        fp[n] += h
        fm[n] -= h
        Jp = c.forward(fp)[0]
        Jm = c.forward(fm)[0]
        assert abs((Jp - Jm) / (2 * h) - g[n]) <= 1e-6 * np.abs(g).max()


def test_oc_gradient_independent_of_checkpoint_interval():
    c = case("sym")
    grads = []
    for cp in (1, 0, 7, len(c.field)):
        c.forward(checkpoint=cp)
        grads.append(c.pg.oc_backward(len(c.field))[0])
    for g in grads[1:]:
        assert np.array_equal(g, grads[0])


def test_oc_backward_needs_forward_and_dipole():
    pg = E.Problem(S.config_oc(seed=3, nb=4, nq=5, D=2), device=0)
    with pytest.raises(E.EvrError) as ei:
        pg.oc_backward(10)
    assert ei.value.code == E.EVR_EINVAL
    p2 = E.Problem(S.config_dp3(nb=4, nq=5), device=0)
    psi = np.zeros(p2.N, dtype=complex)
    psi[0] = 1.0
    with pytest.raises(E.EvrError) as ei:
        p2.oc_forward(np.zeros(5), psi, psi, 5.0, 0.0, 0.1)
    assert ei.value.code == E.EVR_EINVAL


def test_oc_gradient_finite_differences_at_workload_size():
    # the optimal-control workload itself: D=3, nb=20, nq=24, 4000 steps of dt = 5 au, field
    # of 8 sinusoids of amplitude 0.005, ground state -> level 5; the adjoint gradient against
    # central differences (h = 1e-7) of the GPU forward pass at three steps, 1e-6 relative
    sp = S.config_oc(seed=0)
    pg = E.Problem(sp, device=0)
    e, vec, _ = pg.davidson(8, block=16, conv_resi=1e-9, conv_ene=1e-12, want_vectors=True, sym=0)
    rng = np.random.default_rng(0)
    v = rng.standard_normal((pg.N, 1))
    for _ in range(200):  # spectral radius by power iterations
        hv = pg.hpsi(v)
        lam = float(np.linalg.norm(hv))
        v = hv / lam
    psi0 = vec[:, 0] / np.linalg.norm(vec[:, 0]) + 0j
    tgt = vec[:, 5] / np.linalg.norm(vec[:, 5]) + 0j
    field = S.oc_field(4000, 5.0, seed=0)
    emin, emax = e[0] - 0.01, 1.05 * lam

    def J(f):
        return pg.oc_forward(f, psi0, tgt, 5.0, emin, emax)[0]

    J(field)
    g, _, _ = pg.oc_backward(len(field))
    h = 1e-7
    for n in (7, 2000, 3998):
        fp, fm = field.copy(), field.copy()
        fp[n] += h
        fm[n] -= h
        assert abs((J(fp) - J(fm)) / (2 * h) - g[n]) <= 1e-6 * np.abs(g).max()


def test_operator_update_discards_the_forward_state():
    # a gradient must not mix two operators: evr_set_ggrid after evr_oc_forward drops the
    # forward state, and evr_oc_backward asks for a new forward pass
    c = Case(nb=5, nq=7, nst=10, seed=11)
    c.forward()
    G = np.tile(np.eye(c.sp.D), (c.pg.sum_nq, 1, 1))
    c.pg.set_ggrid(G)
    with pytest.raises(E.EvrError) as ei:
        c.pg.oc_backward(len(c.field))
    assert ei.value.code == E.EVR_EINVAL
    c.forward()
    g, _, _ = c.pg.oc_backward(len(c.field))
    assert np.isfinite(g).all()
