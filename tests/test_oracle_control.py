"""CPU checks of the optimal-control oracle (oracle/control.py) on small systems: the
exact discrete gradient against central finite differences, and the continuous-time
build_field gradient (sub_control.f90:955-975) against it."""
import numpy as np
import pytest

from evrgpu import spec as S
from oracle import control as OC
from oracle import oracle as O


def small_system(nb=4, nq=5, D=2, seed=3):
    sp = S.config_oc(seed=seed, nb=nb, nq=nq, D=D)
    op = O.OracleProblem(sp)
    H0, M = OC.operators(op)
    w, v = np.linalg.eig(H0)
    order = np.argsort(w.real)
    return sp, H0, M, w.real[order], v[:, order].real


def test_dipole_operator_is_symmetric_and_field_is_linear():
    sp, H0, M, _, _ = small_system()
    assert np.abs(M - M.T).max() < 1e-14 * np.abs(M).max()
    op = O.OracleProblem(sp)
    op.set_field(1.0, -0.03, True)
    HE = op.dense()
    assert np.abs(HE - (H0 - 0.03 * M)).max() < 1e-13 * np.abs(H0).max()


def test_exact_gradient_matches_finite_differences():
    sp, H0, M, w, v = small_system()
    nst, dt = 12, 20.0
    field = S.oc_field(nst, dt, seed=1, amp=0.02)
    psi0 = v[:, 0].astype(complex)
    psi0 /= np.linalg.norm(psi0)
    target = v[:, 2].astype(complex)
    target /= np.linalg.norm(target)
    g = OC.gradient_exact(H0, M, field, dt, psi0, target)
    h = 1e-6
    for n in (0, 5, 11):
        fp, fm = field.copy(), field.copy()
        fp[n] += h
        fm[n] -= h
        jp, _ = OC.objective(H0, M, fp, dt, psi0, target)
        jm, _ = OC.objective(H0, M, fm, dt, psi0, target)
        fd = (jp - jm) / (2 * h)
        assert abs(fd - g[n]) <= 1e-7 * np.abs(g).max() + 1e-12


@pytest.mark.parametrize("dt", [4.0, 2.0])
def test_continuous_gradient_is_the_small_step_limit(dt):
    # symmetric H (nb == nq): the build_field direction integrated over a step tends to the
    # discrete gradient as O(dt^3) per step
    sp, H0, M, w, v = small_system(nb=4, nq=4)
    T = 200.0
    nst = int(T / dt)
    field = S.oc_field(nst, dt, seed=2, amp=0.02)
    psi0 = v[:, 0].astype(complex)
    target = v[:, 1].astype(complex)
    g = OC.gradient_exact(H0, M, field, dt, psi0, target)
    r = OC.gradient_continuous(H0, M, field, dt, psi0, target)
    trap = 0.5 * dt * (r[:-1] + r[1:])
    err = np.abs(trap - g).max() / np.abs(g).max()
    assert err < 5e-4 * (dt / 4.0) ** 2
