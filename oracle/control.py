"""Optimal-control oracle: exact propagation and gradients on small dense problems.

TEST INFRASTRUCTURE ONLY (tests/ import it; the product library never does).

The operators come from the C++ oracle (``OracleProblem.dense`` with the field term off,
and the dipole alone), so H0 and mu are the reference's OpPsi restated.  The control
problem is the one of sub_Opt_control (Source_ElVibRot/sub_propagation/sub_control.f90:290):

* H(t) = H0 - E(t) mu (fcn_field, sub_module_propa_march.f90:1494-1503), here with a
  piecewise-constant field E_n on step n, so U_n = expm(-i (H0 - E_n mu) dt) exactly;
* J = |<target|psi(T)>|^2 (calc_fidelity, sub_control.f90:1007-1050);
* the reference's field-update direction (build_field, sub_control.f90:955-975),
  E_new = -Im(<psi|chi><chi|mu|psi>)/alpha with chi the target propagated backwards,
  which is (1/(2 alpha)) dJ/dE(t) of the continuous-time problem.

``gradient_exact`` is dJ/dE_n of the discrete problem from the Frechet derivative of the
matrix exponential, independent of any Chebyshev recurrence.
"""
from __future__ import annotations

import numpy as np
import scipy.linalg as sla


def operators(op):
    """(H0, mu) as dense matrices of an OracleProblem whose spec carries a dipole."""
    op.set_field(1.0, 0.0, True)
    H0 = op.dense()
    op.set_field(0.0, 1.0, False)
    M = op.dense()
    op.set_field(1.0, 0.0, True)
    return H0, M


def propagators(H0, M, field, dt):
    return [sla.expm(-1j * (H0 - e * M) * dt) for e in field]


def forward(U, psi0):
    """States psi_0..psi_N."""
    out = [np.asarray(psi0, dtype=np.complex128)]
    for u in U:
        out.append(u @ out[-1])
    return out


def backward(U, target):
    """chi_n = U_{n+1}^+ ... U_N^+ target for n = 0..N."""
    chi = [None] * (len(U) + 1)
    chi[-1] = np.asarray(target, dtype=np.complex128)
    for n in range(len(U), 0, -1):
        chi[n - 1] = U[n - 1].conj().T @ chi[n]
    return chi


def objective(H0, M, field, dt, psi0, target):
    psi = forward(propagators(H0, M, field, dt), psi0)
    c = np.vdot(target, psi[-1])
    return abs(c) ** 2, c


def gradient_exact(H0, M, field, dt, psi0, target):
    """dJ/dE_n = 2 Re(conj(c) <chi_n| dU_n/dE_n |psi_{n-1}>), dU/dE = Frechet derivative of
    expm at -i (H0 - E mu) dt in the direction +i mu dt."""
    U = propagators(H0, M, field, dt)
    psi = forward(U, psi0)
    chi = backward(U, target)
    c = np.vdot(target, psi[-1])
    g = np.zeros(len(field))
    for n in range(1, len(field) + 1):
        A = -1j * (H0 - field[n - 1] * M) * dt
        dU = sla.expm_frechet(A, 1j * M * dt, compute_expm=False)
        g[n - 1] = 2.0 * np.real(np.conj(c) * np.vdot(chi[n], dU @ psi[n - 1]))
    return g


def gradient_continuous(H0, M, field, dt, psi0, target):
    """The build_field quantity -2 Im(<psi(t_n)|chi(t_n)><chi(t_n)|mu|psi(t_n)>), n = 0..N."""
    U = propagators(H0, M, field, dt)
    psi = forward(U, psi0)
    chi = backward(U, target)
    return np.array([-2.0 * np.imag(np.vdot(p, x) * np.vdot(x, M @ p)) for p, x in zip(psi, chi)])
