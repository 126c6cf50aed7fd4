"""ctypes front end of the CPU oracle (oracle/evr_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()`` and by
the ``cpu_baseline`` / ``--impl reference`` legs of ``bench.py``.  The product
library never imports this module.

The oracle restates the reference's OpPsi on SG4 and direct-product bases
(Source_ElVibRot/sub_Operator/sub_OpPsi_SG4.f90:678-1668 and the basis set-up it
depends on); see the header of evr_oracle.cpp for the golden files that pin it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libevr_oracle.so")
SRC = os.path.join(HERE, "evr_oracle.cpp")

_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle shared library (g++ -O3 -fopenmp)."""
    os.makedirs(BUILD, exist_ok=True)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        cmd = ["g++", "-O3", "-std=c++17", "-fopenmp", "-shared", "-fPIC", "-o", LIB + ".tmp", SRC]
        subprocess.check_call(cmd)
        os.replace(LIB + ".tmp", LIB)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        vp, ip, dp, lp = C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_double), C.POINTER(C.c_longlong)
        L.or_create.restype = vp
        L.or_create.argtypes = [C.c_int] * 5 + [ip] * 6 + [dp, dp]
        L.or_destroy.argtypes = [vp]
        L.or_sizes.argtypes = [vp, lp]
        L.or_tables.argtypes = [vp, ip, dp, ip, ip]
        L.or_basis.argtypes = [vp, C.c_int, C.c_int, ip] + [dp] * 8
        L.or_gauss_hermite.argtypes = [C.c_int, dp, dp]
        L.or_set_potential.argtypes = [vp, C.c_int, dp, ip, ip]
        L.or_set_keo.argtypes = [vp, C.c_int, dp, dp]
        L.or_vgrid.argtypes = [vp, dp]
        L.or_set_dipole.argtypes = [vp, C.c_int, dp, ip, ip]
        L.or_set_field.argtypes = [vp, C.c_double, C.c_double, C.c_int]
        L.or_set_metric.argtypes = [vp, dp, dp, dp]
        L.or_hpsi.argtypes = [vp, dp, C.c_longlong, dp, C.c_longlong, C.c_int, C.c_int]
        _lib = L
    return _lib


def _i(a):
    a = np.ascontiguousarray(a, dtype=np.int32)
    return a, a.ctypes.data_as(C.POINTER(C.c_int))


def _d(a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a, a.ctypes.data_as(C.POINTER(C.c_double))


def gauss_hermite(n: int):
    x = np.zeros(n)
    w = np.zeros(n)
    lib().or_gauss_hermite(n, x.ctypes.data_as(C.POINTER(C.c_double)), w.ctypes.data_as(C.POINTER(C.c_double)))
    return x, w


class OracleProblem:
    """One SG4 or direct-product problem with its operator, evaluated on the CPU."""

    def __init__(self, spec):
        self.spec = spec
        L = lib()
        D = spec.D
        z = np.zeros(D, dtype=np.int32)
        keep = []
        Aq, pAq = _i(spec.Aq if spec.kind == "sg4" else z)
        Bq, pBq = _i(spec.Bq if spec.kind == "sg4" else z)
        Ab, pAb = _i(spec.Ab if spec.kind == "sg4" else z)
        Bb, pBb = _i(spec.Bb if spec.kind == "sg4" else z)
        nq, pnq = _i(spec.nq_dp if spec.kind == "dp" else z)
        nb, pnb = _i(spec.nb_dp if spec.kind == "dp" else z)
        s, ps = _d(spec.scaleQ)
        q0, pq0 = _d(spec.Q0)
        keep += [Aq, Bq, Ab, Bb, nq, nb, s, q0]
        kind = 0 if spec.kind == "sg4" else 1
        self.h = L.or_create(kind, D, spec.nb0, spec.LG, spec.LB, pAq, pBq, pAb, pBb, pnq, pnb, ps, pq0)
        if not self.h:
            raise ValueError("oracle: bad problem description")
        sz = np.zeros(6, dtype=np.int64)
        L.or_sizes(self.h, sz.ctypes.data_as(C.POINTER(C.c_longlong)))
        self.Np, self.nterm, self.sum_nb, self.sum_nq, self.max_nb, self.max_nq = (int(v) for v in sz)
        coef, pc = _d(spec.mono_coef)
        idx, pidx = _i(spec.mono_idx)
        el, pel = _i(spec.mono_elec)
        if L.or_set_potential(self.h, len(coef), pc, pidx, pel) != 0:
            raise ValueError("oracle: bad potential")
        G0, pG0 = _d(np.asfortranarray(spec.G0).ravel(order="F"))
        g, pg = _d(np.asfortranarray(spec.g).ravel(order="F"))
        if L.or_set_keo(self.h, spec.keo_type, pG0, pg) != 0:
            raise ValueError("oracle: bad KEO")
        if getattr(spec, "dip_coef", None) is not None:
            dc, pdc = _d(spec.dip_coef)
            di, pdi = _i(spec.dip_idx)
            de, pde = _i(spec.dip_elec)
            if L.or_set_dipole(self.h, len(dc), pdc, pdi, pde) != 0:
                raise ValueError("oracle: bad dipole")

    def set_metric(self, jac=None, rho=None, G=None):
        """Type 10: Jacobian and rho per grid point (whole-grid order; None: 1) and G(Q)
        (sum_nq x D x D; None: G0 + g.Q), the values Tnum's get_d0GG gives per point."""
        D = self.spec.D
        dp = C.POINTER(C.c_double)
        keep = []

        def arr(a, shape):
            if a is None:
                return None
            a = np.ascontiguousarray(np.asarray(a, dtype=np.float64).reshape(shape))
            keep.append(a)
            return a.ctypes.data_as(dp)

        Gc = None if G is None else np.asarray(G, dtype=np.float64).reshape(self.sum_nq, D, D).transpose(0, 2, 1)
        rc = lib().or_set_metric(self.h, arr(jac, (self.sum_nq,)), arr(rho, (self.sum_nq,)),
                                 arr(Gc, (self.sum_nq, D, D)))
        if rc != 0:
            raise ValueError("oracle: Jacobian and rho must be positive")

    def set_field(self, vw: float = 1.0, mw: float = 0.0, keo: bool = True):
        """Grid operator vw*V + mw*mu (+ kinetic part) of later hpsi calls (H - E mu: vw=1, mw=-E)."""
        lib().or_set_field(self.h, float(vw), float(mw), 1 if keo else 0)

    def __del__(self):
        if getattr(self, "h", None):
            lib().or_destroy(self.h)
            self.h = None

    @property
    def N(self):
        return self.Np * self.spec.nb0

    def tables(self):
        D = self.spec.D
        term_l = np.zeros((self.nterm, D), dtype=np.int32)
        weight = np.zeros(self.nterm)
        mp = np.zeros(self.sum_nb, dtype=np.int32)
        packed = np.zeros((self.Np, D), dtype=np.int32)
        lib().or_tables(self.h, term_l.ctypes.data_as(C.POINTER(C.c_int)), weight.ctypes.data_as(C.POINTER(C.c_double)),
                        mp.ctypes.data_as(C.POINTER(C.c_int)), packed.ctypes.data_as(C.POINTER(C.c_int)))
        return dict(term_l=term_l, weight=weight, map=mp, packed=packed)

    def basis(self, mode: int, level: int):
        n = 64 * 64
        bufs = [np.zeros(n) for _ in range(8)]
        nbq = np.zeros(2, dtype=np.int32)
        ptrs = [b.ctypes.data_as(C.POINTER(C.c_double)) for b in bufs]
        if lib().or_basis(self.h, mode, level, nbq.ctypes.data_as(C.POINTER(C.c_int)), *ptrs) != 0:
            raise IndexError("no such basis")
        nb, nq = int(nbq[0]), int(nbq[1])
        x, w, d0, d1, d2, bgw, g1, g2 = bufs
        f = lambda a, r, c: a[: r * c].reshape((r, c), order="F").copy()
        return dict(nb=nb, nq=nq, x=x[:nq].copy(), w=w[:nq].copy(), d0b=f(d0, nq, nb), d1b=f(d1, nq, nb),
                    d2b=f(d2, nq, nb), bgw=f(bgw, nb, nq), d1gg=f(g1, nq, nq), d2gg=f(g2, nq, nq))

    def vgrid(self):
        v = np.zeros(self.sum_nq * self.spec.nb0 ** 2)
        lib().or_vgrid(self.h, v.ctypes.data_as(C.POINTER(C.c_double)))
        return v

    def hpsi(self, psi: np.ndarray, nthreads: int = 0) -> np.ndarray:
        """H applied to the columns of psi (N x nvec, any order)."""
        psi = np.asfortranarray(psi, dtype=np.float64)
        if psi.ndim == 1:
            psi = psi[:, None]
        N, nvec = psi.shape
        assert N == self.N
        out = np.zeros((N, nvec), order="F")
        rc = lib().or_hpsi(self.h, psi.ctypes.data_as(C.POINTER(C.c_double)), N,
                           out.ctypes.data_as(C.POINTER(C.c_double)), N, nvec, nthreads)
        if rc != 0:
            raise RuntimeError("oracle hpsi failed")
        return out

    def dense(self, nthreads: int = 0) -> np.ndarray:
        return self.hpsi(np.eye(self.N), nthreads)
