"""Gaussian filter diagonalisation oracle: the reference's algorithm restated in numpy.

TEST INFRASTRUCTURE ONLY (tests/ import it; the product library never does).

Restates sub_GaussianFilterDiagonalization
(Source_ElVibRot/sub_propagation/sub_module_Filter.f90:70-520) with its helpers, on an
H.psi callable (the C++ oracle's OpPsi, or a dense matrix):

* spectral scaling: Hmin/Hmax widened by 1 % of their range, E0 = centre, Esc = half range
  (:155-170); the window [LambdaMin, LambdaMax] with LambdaMin = max(ZPE, E0_filter - W/2),
  ZPE = the Hmin given (:178-190);
* L Gaussian filters exp(-((x - El)/sigma)^2), sigma = W/Esc/L, centred at
  LambdaMin + (l-1) W/(L-1) in scaled energy (:300-345, f_filter :2581-2645), projected on
  the Chebyshev polynomials by the Gauss-Chebyshev rule of gauss_chebyWeight
  (Source_Lib/sub_communf90/sub_math/sub_integration.f90:195-214) with the weight factor
  sqw = (1 - x^2)^(-1/4) sqrt(2/pi) and the kernel damping factor KDF (:2538-2579);
* the series length: nq = int(pi/|acos(B) - acos(A)|/3) for the central window cell, then
  grown by 10 % (integer arithmetic) until the mean of |f| over the last four coefficients
  (sum/3) of the central filter is below 1e-8 or the length exceeds M_filter (:199-283).
  Where the reference's nb*11/10 would not grow nb (nb < 10) it grows by one here: the
  reference loops forever there.  The cell's edges are clamped to [-1, 1] (acos) and the
  start value is at least 4 (the tail test reads four coefficients);
* the Chebyshev recursion T_0 = q1, T_1 = Hs q1, T_n = 2 Hs T_(n-1) - T_(n-2)
  (sub_chebychev_recursion :2221-2298), z_l = sum_n f(n, l) T_n (sub_newZ_vectors_withf
  :2441-2505);
* sub_Lowdin (Source_ElVibRot/sub_WP/sub_module_psi_Op.f90): z normalised, S = <z_i|z_j>
  diagonalised (eigenvalues in decreasing order), z_i <- normalised sum_j V_ji z_j, the S
  eigenvalue kept as the vector's weight; then sub_Schmidt (Gram-Schmidt from the second
  vector on, renormalised);
* the vectors with weight above 1e-9 span the subspace (:375); H_ij = <z_i|H z_j>,
  non_hermitic = max|H - H^T|/2 and H symmetrised (sub_hermitic_H,
  sub_inactive/sub_ana_HS.f90), eigenvalues ascending, residual norms of
  g_j = sum_i (H z_i - E_j z_i) V_ij (:405-470), convergence below
  max(conv_resi, non_hermitic), counts in the window.
"""
from __future__ import annotations

import numpy as np


def gauss_cheby_weight(n: int):
    """Nodes and weights of gauss_chebyWeight (the weights include sqrt(1 - x^2))."""
    step = np.pi / n
    x = np.cos(-0.5 * step + step * np.arange(1, n + 1))
    return x, step * np.sqrt(1.0 - x * x)


def kdf(j: int, nb: int) -> float:
    """Kernel damping factor of coefficient j (1-based) of a series of nb terms."""
    if j < 2:
        return 1.0
    r0 = np.pi / (nb - 1)
    r = np.pi * (j - 1) / (nb - 1)
    return (np.cos(r) * (nb - j) + np.sin(r) * np.sin(r0) / np.cos(r0)) / (nb - 1)


def cheby_coefficients(centres, sigma: float, nb: int) -> np.ndarray:
    """f(n, l), n < nb: the Gaussian filters centred at the scaled energies `centres`."""
    x, w = gauss_cheby_weight(nb)
    sqw = 1.0 / np.sqrt(np.sqrt(1.0 - x * x)) * np.sqrt(2.0 / np.pi)
    f = np.zeros((nb, len(centres)))
    for l, el in enumerate(centres):
        wfl = np.exp(-(((x - el) / sigma) ** 2)) * w
        p0 = np.ones(nb)
        f[0, l] = np.dot(wfl, p0 * sqw / np.sqrt(2.0))
        if nb > 1:
            p1 = x.copy()
            f[1, l] = np.dot(wfl, p1 * sqw) * kdf(2, nb)
        for j in range(3, nb + 1):
            p2 = 2.0 * x * p1 - p0
            f[j - 1, l] = np.dot(wfl, p2 * sqw) * kdf(j, nb)
            p0, p1 = p1, p2
    return f


def setup(hmin, hmax, e0_filter, width, n_filters, max_order):
    """Scaling, window, filter centres and series length as the reference derives them."""
    zpe = hmin
    d = hmax - hmin
    lo, hi = hmin - 0.01 * d, hmax + 0.01 * d
    E0, Esc = lo + 0.5 * (hi - lo), 0.5 * (hi - lo)
    dlam = width / (n_filters - 1)
    lmin = max(zpe, e0_filter - 0.5 * width)
    lmax = lmin + width
    sigma = width / Esc / n_filters
    el = (e0_filter - E0) / Esc
    a = min(1.0, max(-1.0, el - dlam / Esc / 2.0))
    b = min(1.0, max(-1.0, el + dlam / Esc / 2.0))
    nb = max(4, int(np.pi / abs(np.arccos(b) - np.arccos(a)) / 3.0))
    while True:
        nb = max(nb * 11 // 10, nb + 1)
        f = cheby_coefficients([el], sigma, nb)
        err = np.abs(f[nb - 4:nb, 0]).sum() / 3.0
        if err < 1e-8 or nb > max_order:
            break
    centres = [((lmin + l * dlam) - E0) / Esc for l in range(n_filters)]
    return dict(E0=E0, Esc=Esc, lmin=lmin, lmax=lmax, sigma=sigma, nb=nb,
                f=cheby_coefficients(centres, sigma, nb))


def filter_diag(hpsi, q1, hmin, hmax, e0_filter, width, n_filters, max_order, conv_resi=1e-6):
    """The reference's filter diagonalisation on start vectors q1 (N x ns, one set of L
    filtered vectors per column).  hpsi: callable on N x k blocks."""
    q1 = np.asarray(q1, dtype=np.float64)
    if q1.ndim == 1:
        q1 = q1[:, None]
    st = setup(hmin, hmax, e0_filter, width, n_filters, max_order)
    E0, Esc, f, nb = st["E0"], st["Esc"], st["f"], st["nb"]
    L = n_filters
    ns = q1.shape[1]
    Z = np.zeros((q1.shape[0], ns * L))

    def acc(T, n):
        for s in range(ns):
            Z[:, s * L:(s + 1) * L] += np.outer(T[:, s], f[n])

    t0 = q1.copy()
    acc(t0, 0)
    t1 = (hpsi(t0) - E0 * t0) / Esc
    acc(t1, 1)
    for n in range(2, nb):
        t2 = 2.0 * (hpsi(t1) - E0 * t1) / Esc - t0
        acc(t2, n)
        t0, t1 = t1, t2
    # sub_Lowdin, then sub_Schmidt
    Z /= np.linalg.norm(Z, axis=0)
    S = Z.T @ Z
    s, V = np.linalg.eigh(S)
    order = np.argsort(-s, kind="stable")
    s, V = s[order], V[:, order]
    Z = Z @ V
    Z /= np.linalg.norm(Z, axis=0)
    for i in range(1, Z.shape[1]):
        for j in range(i):
            Z[:, i] -= np.dot(Z[:, j], Z[:, i]) * Z[:, j]
        Z[:, i] /= np.linalg.norm(Z[:, i])
    keep = int((np.abs(s) > 1e-9).sum())
    Z = Z[:, :keep]
    HZ = hpsi(Z)
    H = Z.T @ HZ
    nonh = 0.5 * np.abs(H - H.T).max()
    H = 0.5 * (H + H.T)
    e, vec = np.linalg.eigh(H)
    G = HZ @ vec - (Z @ vec) * e
    resid = np.linalg.norm(G, axis=0)
    conv = resid < max(conv_resi, nonh)
    inwin = (e >= st["lmin"]) & (e <= st["lmax"])
    return dict(eig=e, resid=resid, conv=conv, vec=Z @ vec, nb=nb, keep=keep, non_hermitic=nonh,
                in_window=int(inwin.sum()), conv_in_window=int((inwin & conv).sum()), lmin=st["lmin"],
                lmax=st["lmax"], f=f, E0=E0, Esc=Esc)
