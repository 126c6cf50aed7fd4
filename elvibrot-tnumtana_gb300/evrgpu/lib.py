"""ctypes binding of libevrgpu.so (include/evr_gpu.h) and the host-side mirror of the
reference's OpPsi / Davidson / propagation call surface.

``Problem`` plays the role of the reference's ``para_Op`` for the H.psi path: it is
created once from a ``ProblemSpec`` and then applies H to blocks of vectors
(``hpsi`` ~ ``sub_TabOpPsi``, Source_ElVibRot/sub_Operator/sub_OpPsi.f90:701),
computes levels (``davidson`` ~ ``sub_propagation_Davidson``,
sub_propagation/sub_module_Davidson.f90:54) and propagates packets
(``chebyshev`` ~ ``march_cheby``, sub_propagation/sub_module_propa_march.f90:4142).
Errors come back as ``EvrError`` carrying the library's status and message; there is
no CPU fallback: without the compiled library or a GPU the calls fail.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

EVR_OK, EVR_EINVAL, EVR_ENOMEM, EVR_ETIMEDOUT, EVR_EDEVICE, EVR_ENOCONV = 0, 22, 12, 110, 1001, 1002
PREC = {"fp64": 0, "fp32": 1}
LAYOUT_COLMAJOR, LAYOUT_INTERLEAVED = 0, 1

_ip = C.POINTER(C.c_int)
_dp = C.POINTER(C.c_double)
_lp = C.POINTER(C.c_int64)


class EvrError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"evr error {code}: {msg}")
        self.code = code


class Basis1D(C.Structure):
    _fields_ = [("nq", C.c_int), ("nb", C.c_int), ("x", _dp), ("w", _dp), ("d0b", _dp), ("d1b", _dp),
                ("d2b", _dp)]


class ProblemDesc(C.Structure):
    _fields_ = [("kind", C.c_int), ("D", C.c_int), ("nb0", C.c_int), ("LG", C.c_int), ("LB", C.c_int),
                ("Aq", _ip), ("Bq", _ip), ("Ab", _ip), ("Bb", _ip), ("nq_dp", _ip), ("nb_dp", _ip),
                ("scaleQ", _dp), ("Q0", _dp), ("n_mono", C.c_int), ("mono_coef", _dp), ("mono_idx", _ip),
                ("mono_elec", _ip), ("keo_type", C.c_int), ("G0", _dp), ("g", _dp),
                ("bases", C.POINTER(Basis1D))]


class Sizes(C.Structure):
    _fields_ = [("Np", C.c_int64), ("N", C.c_int64), ("n_terms", C.c_int64), ("sum_nb", C.c_int64),
                ("sum_nq", C.c_int64), ("max_nq_term", C.c_int64), ("flop_per_hpsi", C.c_double)]


class DavidsonOpts(C.Structure):
    _fields_ = [("n_levels", C.c_int), ("block", C.c_int), ("max_dim", C.c_int), ("max_it", C.c_int),
                ("conv_resi", C.c_double), ("conv_ene", C.c_double), ("prec", C.c_int), ("n_guess", C.c_int),
                ("sym", C.c_int)]


class FilterOpts(C.Structure):
    _fields_ = [("hmin", C.c_double), ("hmax", C.c_double), ("e0", C.c_double), ("width", C.c_double),
                ("n_filters", C.c_int), ("max_order", C.c_int), ("nstart", C.c_int), ("prec", C.c_int),
                ("conv_resi", C.c_double), ("seed", C.c_ulonglong)]


class LanczosOpts(C.Structure):
    _fields_ = [("nev", C.c_int), ("ncv", C.c_int), ("max_restarts", C.c_int), ("tol", C.c_double), ("sym", C.c_int),
                ("seed", C.c_ulonglong)]


class OcOpts(C.Structure):
    _fields_ = [("nsteps", C.c_int), ("dt", C.c_double), ("emin", C.c_double), ("emax", C.c_double),
                ("poly_tol", C.c_double), ("checkpoint", C.c_int), ("prec", C.c_int)]


EXPORTS = ["evr_create", "evr_destroy", "evr_last_error", "evr_sizes", "evr_get_tables", "evr_get_basis",
           "evr_get_vgrid", "evr_hpsi_host", "evr_hpsi_device", "evr_set_operator", "evr_set_kernel_path",
           "evr_last_launch_count",
           "evr_last_kernel_ms",
           "evr_davidson",
           "evr_cheby_propagate", "evr_fma_peak", "evr_hpsi_noalloc", "evr_set_dipole", "evr_set_field",
           "evr_oc_forward", "evr_oc_backward", "evr_create_batch", "evr_batch_offsets", "evr_batch_davidson", "evr_autotune",
           "evr_psi_write", "evr_psi_read", "evr_set_vgrid", "evr_set_dipole_grid", "evr_set_ggrid",
           "evr_sil_propagate", "evr_restart_write", "evr_restart_read", "evr_autocorr_write",
           "evr_autocorr_read", "evr_tc_selftest", "evr_set_tensor_cores", "evr_set_jacobian", "evr_filter_diag", "evr_lanczos"]
VGRID_LAYOUT = {"terms": 0, "ref": 1}
WP_FORMAT = {"v0": 0, "v1": 1, "unformatted": 2, "sparse": 3}

_lib = None
_build_error = None  # a failed build is reported once per process, not retried by every call


def library_path() -> str:
    return _build.LIB


def load(build: bool = True):
    """Load (building first if needed) libevrgpu.so and declare its signatures."""
    global _lib, _build_error
    if _lib is not None:
        return _lib
    if _build_error is not None:
        raise EvrError(EVR_EDEVICE, f"libevrgpu.so failed to build earlier in this process: {_build_error}")
    if build:
        try:
            _build.build()
        except Exception as e:
            _build_error = str(e)[-2000:]
            raise
    if not os.path.exists(_build.LIB):
        raise EvrError(EVR_EDEVICE, f"{_build.LIB} is missing: build the CUDA library first")
    L = C.CDLL(_build.LIB)
    vp = C.c_void_p
    L.evr_create.argtypes = [C.POINTER(vp), C.POINTER(ProblemDesc), C.c_int]
    L.evr_destroy.argtypes = [vp]
    L.evr_last_error.argtypes = [vp]
    L.evr_last_error.restype = C.c_char_p
    L.evr_sizes.argtypes = [vp, C.POINTER(Sizes)]
    L.evr_get_tables.argtypes = [vp, _ip, _dp, _ip, _ip]
    L.evr_get_basis.argtypes = [vp, C.c_int, C.c_int, _ip] + [_dp] * 8
    L.evr_get_vgrid.argtypes = [vp, _dp]
    L.evr_set_vgrid.argtypes = [vp, _dp, C.c_int]
    L.evr_set_dipole_grid.argtypes = [vp, _dp, C.c_int]
    L.evr_set_ggrid.argtypes = [vp, _dp]
    L.evr_set_jacobian.argtypes = [vp, _dp, _dp]
    L.evr_hpsi_host.argtypes = [vp, _dp, C.c_int64, _dp, C.c_int64, C.c_int, C.c_int, C.c_int]
    L.evr_hpsi_device.argtypes = [vp, vp, C.c_int64, vp, C.c_int64, C.c_int, C.c_int, C.c_int, vp]
    L.evr_last_launch_count.argtypes = [vp, _lp, _lp]
    L.evr_last_kernel_ms.argtypes = [vp, C.POINTER(C.c_float), C.POINTER(C.c_float)]
    L.evr_set_operator.argtypes = [vp, C.c_int]
    L.evr_set_kernel_path.argtypes = [vp, C.c_int]
    L.evr_set_tensor_cores.argtypes = [vp, C.c_int, C.c_int]
    L.evr_fma_peak.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_double)]
    L.evr_hpsi_noalloc.argtypes = [vp, vp, C.c_int64, vp, C.c_int64, C.c_int, vp]
    L.evr_autotune.argtypes = [vp, C.c_int, C.c_int, _ip, _dp]
    L.evr_create_batch.argtypes = [C.POINTER(vp), C.POINTER(ProblemDesc), C.c_int, C.c_int]
    L.evr_batch_offsets.argtypes = [vp, _lp]
    L.evr_batch_davidson.argtypes = [vp, C.POINTER(DavidsonOpts), _dp, _lp]
    L.evr_set_dipole.argtypes = [vp, C.c_int, _dp, _ip, _ip]
    L.evr_set_field.argtypes = [vp, C.c_double, C.c_double, C.c_int]
    L.evr_oc_forward.argtypes = [vp, C.POINTER(OcOpts), _dp, _dp, _dp, _dp, _dp, _lp]
    L.evr_oc_backward.argtypes = [vp, _dp, _dp, _lp]
    L.evr_psi_write.argtypes = [vp, C.c_char_p, C.c_int, _dp, C.c_int64, C.c_int, C.c_int, C.c_double]
    L.evr_psi_read.argtypes = [vp, C.c_char_p, _dp, C.c_int64, C.c_int, C.c_int, _ip, _lp]
    L.evr_restart_write.argtypes = [vp, C.c_char_p, C.c_double, _dp, C.c_int64, C.c_int]
    L.evr_restart_read.argtypes = [vp, C.c_char_p, _dp, _dp, C.c_int64, C.c_int, _ip]
    L.evr_autocorr_write.argtypes = [C.c_char_p, _dp, _dp, C.c_int, C.c_int]
    L.evr_autocorr_read.argtypes = [C.c_char_p, _dp, _dp, C.c_int, _ip]
    if hasattr(L, "evr_davidson"):
        L.evr_davidson.argtypes = [vp, C.POINTER(DavidsonOpts), _dp, _dp, _dp, _lp]
    if hasattr(L, "evr_cheby_propagate"):
        L.evr_cheby_propagate.argtypes = [vp, _dp, C.c_int, C.c_double, C.c_int, C.c_double, C.c_double,
                                          C.c_double, C.c_int, _dp, _dp, _lp]
    _fp = C.POINTER(C.c_float)
    L.evr_tc_selftest.argtypes = [C.c_int] * 6 + [_fp, _fp, _fp, C.c_float, C.c_int, C.c_int]
    L.evr_sil_propagate.argtypes = [vp, _dp, C.c_int, C.c_double, C.c_int, C.c_int, C.c_double, C.c_int, _dp, _dp,
                                    _lp]
    L.evr_filter_diag.argtypes = [vp, C.POINTER(FilterOpts), _dp, _dp, _dp, _dp, C.POINTER(C.c_int), _dp, _lp]
    L.evr_lanczos.argtypes = [vp, C.POINTER(LanczosOpts), _dp, _dp, _dp, _dp, _lp]
    _lib = L
    return L


def fma_peak(device: int = 0, prec: str = "fp64") -> float:
    """Measured FMA issue rate (TFLOP/s) of the CUDA-core pipe for prec."""
    t = C.c_double()
    rc = load().evr_fma_peak(device, PREC[prec], C.byref(t))
    if rc != 0:
        raise EvrError(rc, "evr_fma_peak failed")
    return t.value


def tc_selftest(inp, mat, A, K, M, B, Vt, alpha=1.0, out=None, threads=512, device=0):
    """One tensor-core mode contraction (evr_tc_selftest) on float32 host arrays: in of
    shape (B, K, A, Vt), mat (K, ldm) with ldm = 4*ceil(M/4); returns out (B, M, A, Vt),
    accumulated onto `out` when given."""
    f = C.POINTER(C.c_float)
    inp = np.ascontiguousarray(inp, dtype=np.float32)
    mat = np.ascontiguousarray(mat, dtype=np.float32)
    acc = out is not None
    o = np.ascontiguousarray(out if acc else np.zeros((B, M, A, Vt)), dtype=np.float32).copy()
    rc = load().evr_tc_selftest(device, A, K, M, B, Vt, inp.ctypes.data_as(f), o.ctypes.data_as(f),
                                mat.ctypes.data_as(f), float(alpha), 1 if acc else 0, threads)
    if rc != 0:
        raise EvrError(rc, "evr_tc_selftest failed")
    return o


def _iarr(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _darr(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _p(a, t):
    return None if a is None else a.ctypes.data_as(t)


def _describe(spec, keep):
    """ProblemDesc of a spec; the arrays it points to are appended to `keep`."""
    def I(a):
        if a is None:
            return None
        a = _iarr(a)
        keep.append(a)
        return _p(a, _ip)

    def F(a):
        if a is None:
            return None
        a = _darr(a)
        keep.append(a)
        return _p(a, _dp)

    d = ProblemDesc()
    d.kind = 0 if spec.kind == "sg4" else 1
    d.D, d.nb0, d.LG, d.LB = spec.D, spec.nb0, spec.LG, spec.LB
    d.Aq, d.Bq, d.Ab, d.Bb = I(spec.Aq), I(spec.Bq), I(spec.Ab), I(spec.Bb)
    d.nq_dp, d.nb_dp = I(spec.nq_dp), I(spec.nb_dp)
    d.scaleQ, d.Q0 = F(spec.scaleQ), F(spec.Q0)
    d.n_mono = len(spec.mono_coef)
    d.mono_coef, d.mono_idx, d.mono_elec = F(spec.mono_coef), I(spec.mono_idx), I(spec.mono_elec)
    d.keo_type = spec.keo_type
    d.G0 = F(np.asarray(spec.G0).ravel(order="F"))
    d.g = F(np.asarray(spec.g).ravel(order="F"))
    if getattr(spec, "bases", None) is not None:
        # host tables of the primitive bases, (mode, level) order: dicts with x, w and the
        # nq x nb arrays d0b, d1b, d2b
        arr = (Basis1D * len(spec.bases))()
        for k, t in enumerate(spec.bases):
            d0 = np.asarray(t["d0b"])
            arr[k].nq, arr[k].nb = int(d0.shape[0]), int(d0.shape[1])
            arr[k].x, arr[k].w = F(t["x"]), F(t["w"])
            arr[k].d0b = F(np.asarray(t["d0b"]).ravel(order="F"))
            arr[k].d1b = F(np.asarray(t["d1b"]).ravel(order="F"))
            arr[k].d2b = F(np.asarray(t["d2b"]).ravel(order="F"))
        keep.append(arr)
        d.bases = C.cast(arr, C.POINTER(Basis1D))
    return d


def write_autocorr(path, t, cdot, append=False):
    """Autocorrelation lines "AutoCor T Re Im |C|" (Write_AutoCorr)."""
    t = _darr(t)
    c = np.ascontiguousarray(np.asarray(cdot, dtype=np.complex128))
    rc = load().evr_autocorr_write(os.fsencode(path), _p(t, _dp), c.ctypes.data_as(_dp), len(t), 1 if append else 0)
    if rc != 0:
        raise EvrError(rc, f"evr_autocorr_write: cannot write {path}")


def read_autocorr(path, n_max=1 << 20):
    """(t, cdot) of an autocorrelation file (Read_AutoCorr)."""
    t = np.zeros(n_max)
    c = np.zeros(n_max, dtype=np.complex128)
    n = C.c_int()
    rc = load().evr_autocorr_read(os.fsencode(path), _p(t, _dp), c.ctypes.data_as(_dp), n_max, C.byref(n))
    if rc != 0:
        raise EvrError(rc, f"evr_autocorr_read: cannot read {path}")
    return t[: n.value].copy(), c[: n.value].copy()


class Problem:
    """One H.psi problem on one GPU (device=-1: host tables only)."""

    def __init__(self, spec, device: int = 0):
        L = load()
        self.spec = spec
        self._keep = []
        d = _describe(spec, self._keep)
        h = C.c_void_p()
        rc = L.evr_create(C.byref(h), C.byref(d), device)
        self._finish(h, rc, device)
        if getattr(spec, "dip_coef", None) is not None and device >= 0:
            self.set_dipole(spec.dip_coef, spec.dip_idx, spec.dip_elec)

    def _finish(self, h, rc, device):
        L = load()
        self.h = h
        if rc != 0:
            msg = L.evr_last_error(h).decode() if h else ""
            self.close()
            raise EvrError(rc, msg)
        s = Sizes()
        L.evr_sizes(self.h, C.byref(s))
        self.Np, self.N, self.nterm = s.Np, s.N, s.n_terms
        self.sum_nb, self.sum_nq, self.max_nq = s.sum_nb, s.sum_nq, s.max_nq_term
        self.flop_per_hpsi = s.flop_per_hpsi
        self.device = device

    def close(self):
        if getattr(self, "h", None):
            load().evr_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc != 0:
            raise EvrError(rc, load().evr_last_error(self.h).decode())

    # ---- tables -------------------------------------------------------------------
    def tables(self):
        D = self.spec.D
        term_l = np.zeros((self.nterm, D), dtype=np.int32)
        weight = np.zeros(self.nterm)
        mp = np.zeros(self.sum_nb, dtype=np.int32)
        packed = np.zeros((self.Np, D), dtype=np.int32)
        self._check(load().evr_get_tables(self.h, _p(term_l, _ip), _p(weight, _dp), _p(mp, _ip), _p(packed, _ip)))
        return dict(term_l=term_l, weight=weight, map=mp, packed=packed)

    def basis(self, mode, level):
        bufs = [np.zeros(64 * 64) for _ in range(8)]
        nbq = np.zeros(2, dtype=np.int32)
        self._check(load().evr_get_basis(self.h, mode, level, _p(nbq, _ip), *[_p(b, _dp) for b in bufs]))
        nb, nq = int(nbq[0]), int(nbq[1])
        x, w, d0, d1, d2, bgw, g1, g2 = bufs
        f = lambda a, r, c: a[: r * c].reshape((r, c), order="F").copy()
        return dict(nb=nb, nq=nq, x=x[:nq].copy(), w=w[:nq].copy(), d0b=f(d0, nq, nb), d1b=f(d1, nq, nb),
                    d2b=f(d2, nq, nb), bgw=f(bgw, nb, nq), d1gg=f(g1, nq, nq), d2gg=f(g2, nq, nq))

    def vgrid(self):
        v = np.zeros(self.sum_nq * self.spec.nb0 ** 2)
        self._check(load().evr_get_vgrid(self.h, _p(v, _dp)))
        return v

    def set_vgrid(self, v, layout="terms"):
        """Potential given as grid values (a host's calcN_op grid cache) in place of the one
        evaluated from the monomials; layout "terms" (as vgrid()) or "ref" (the reference's
        OpGrid%Grid(sum_nq, nb0, nb0), column-major)."""
        v = _darr(np.asarray(v, dtype=np.float64).ravel(order="F"))
        if v.size != self.sum_nq * self.spec.nb0 ** 2:
            raise EvrError(EVR_EINVAL, f"V grid has {v.size} values, expected {self.sum_nq * self.spec.nb0 ** 2}")
        self._check(load().evr_set_vgrid(self.h, _p(v, _dp), VGRID_LAYOUT[layout]))

    # ---- wave-packet files ------------------------------------------------------------
    def write_psi(self, path, psi, fmt="v0", epsi=0.0):
        """Packets (columns of psi, N x npsi, real or complex) to a file in the reference's
        save format (sub_save_psi, Source_ElVibRot/sub_WP/sub_module_psi_io.f90:365):
        fmt "v0" (its default), "v1", "unformatted" or "sparse" (entries of modulus >= epsi)."""
        psi = np.asarray(psi)
        if psi.ndim == 1:
            psi = psi[:, None]
        cplx = np.iscomplexobj(psi)
        a = np.asfortranarray(psi, dtype=np.complex128 if cplx else np.float64)
        if a.shape[0] != self.N:
            raise EvrError(EVR_EINVAL, f"psi has {a.shape[0]} rows, expected {self.N}")
        ptr = a.ctypes.data_as(_dp)
        self._check(load().evr_psi_write(self.h, os.fsencode(path), WP_FORMAT[fmt], ptr, self.N, a.shape[1],
                                         1 if cplx else 0, float(epsi)))

    def read_psi(self, path, npsi_max=64, cplx=False, renorm=False):
        """Packets of a file in any of the reference's save formats, mapped onto this basis by
        their tuples (sub_read_psi0, sub_module_psi_io.f90:55).  Returns (psi N x npsi,
        dropped entries).  renorm=True normalises each packet as sub_read_psi0 does."""
        a = np.zeros((self.N, max(npsi_max, 1)), dtype=np.complex128 if cplx else np.float64, order="F")
        n = C.c_int()
        dropped = C.c_int64()
        self._check(load().evr_psi_read(self.h, os.fsencode(path), a.ctypes.data_as(_dp), self.N, npsi_max,
                                        1 if cplx else 0, C.byref(n), C.byref(dropped)))
        a = a[:, : n.value]
        if renorm:
            nrm = np.sqrt(np.sum(np.abs(a) ** 2, axis=0))
            a = a / np.where(nrm > 0, nrm, 1.0)
        return a, dropped.value

    def write_restart(self, path, t, psi):
        """Propagation restart file (SaveWP_restart): time t and complex packets psi (N x npsi)."""
        a = np.asfortranarray(np.asarray(psi, dtype=np.complex128).reshape(self.N, -1))
        self._check(load().evr_restart_write(self.h, os.fsencode(path), float(t), a.ctypes.data_as(_dp), self.N,
                                             a.shape[1]))

    def read_restart(self, path, npsi):
        """(t, packets N x npsi) of a restart file, or (0.0, None) when it holds no restart."""
        a = np.zeros((self.N, npsi), dtype=np.complex128, order="F")
        t, found = C.c_double(), C.c_int()
        self._check(load().evr_restart_read(self.h, os.fsencode(path), C.byref(t), a.ctypes.data_as(_dp), self.N,
                                            npsi, C.byref(found)))
        return (t.value, a) if found.value else (0.0, None)

    # ---- H.psi ----------------------------------------------------------------------
    def hpsi(self, psi, prec: str = "fp64"):
        """H applied to the columns of a HOST array psi (N x nvec); copies in and out."""
        psi = np.asfortranarray(psi, dtype=np.float64)
        if psi.ndim == 1:
            psi = psi[:, None]
        N, nvec = psi.shape
        if N != self.N:
            raise EvrError(EVR_EINVAL, f"psi has {N} rows, expected {self.N}")
        out = np.zeros((N, nvec), order="F")
        self._check(load().evr_hpsi_host(self.h, _p(psi, _dp), N, _p(out, _dp), N, nvec, LAYOUT_COLMAJOR,
                                         PREC[prec]))
        return out

    def hpsi_host_ptr(self, psi_ptr, ld_psi, hpsi_ptr, ld_hpsi, nvec, layout, prec="fp64"):
        """Raw host-pointer entry point (pinned buffers for the end-to-end timing)."""
        self._check(load().evr_hpsi_host(self.h, C.cast(psi_ptr, _dp), ld_psi, C.cast(hpsi_ptr, _dp), ld_hpsi, nvec,
                                         layout, PREC[prec]))

    def hpsi_device(self, psi_ptr, ld_psi, hpsi_ptr, ld_hpsi, nvec, layout=LAYOUT_INTERLEAVED, prec="fp64",
                    stream=None):
        """H.psi on DEVICE pointers (e.g. torch tensor data_ptr()), stream-ordered."""
        self._check(load().evr_hpsi_device(self.h, C.c_void_p(psi_ptr), ld_psi, C.c_void_p(hpsi_ptr), ld_hpsi, nvec,
                                           layout, PREC[prec], C.c_void_p(stream) if stream else None))

    def hpsi_noalloc(self, psi_ptr, ld_psi, hpsi_ptr, ld_hpsi, nvec, stream=None):
        """FP64 H.psi on DEVICE pointers (interleaved) using only the library's fixed
        scratch array: no device allocation (see evr_hpsi_noalloc in include/evr_gpu.h)."""
        self._check(load().evr_hpsi_noalloc(self.h, C.c_void_p(psi_ptr), ld_psi, C.c_void_p(hpsi_ptr), ld_hpsi, nvec,
                                            C.c_void_p(stream) if stream else None))

    def last_launch_count(self):
        k = C.c_int64()
        it = C.c_int64()
        self._check(load().evr_last_launch_count(self.h, C.byref(k), C.byref(it)))
        return k.value, it.value

    def last_kernel_ms(self):
        a, b = C.c_float(), C.c_float()
        self._check(load().evr_last_kernel_ms(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value

    # ---- drivers ------------------------------------------------------------------
    def davidson(self, n_levels, block=None, max_dim=None, max_it=200, conv_resi=1e-7, conv_ene=1e-10,
                 prec="fp64", guess=None, want_vectors=False, sym=-1):
        L = load()
        o = DavidsonOpts()
        o.n_levels = n_levels
        o.block = block or n_levels
        o.max_dim = max_dim or max(4 * n_levels, n_levels + 3 * o.block)
        o.max_it = max_it
        o.conv_resi, o.conv_ene = conv_resi, conv_ene
        o.prec = PREC[prec]
        o.sym = sym
        g = None
        if guess is not None:
            g = np.asfortranarray(guess, dtype=np.float64)
            o.n_guess = g.shape[1]
        eig = np.zeros(n_levels)
        vec = np.zeros((self.N, n_levels), order="F") if want_vectors else None
        info = np.zeros(4, dtype=np.int64)
        rc = L.evr_davidson(self.h, C.byref(o), _p(g, _dp), _p(eig, _dp), _p(vec, _dp), _p(info, _lp))
        stats = dict(iterations=int(info[0]), hpsi_fp64=int(info[1]), hpsi_fp32=int(info[2]),
                     converged=bool(info[3]))
        if rc not in (0, EVR_ENOCONV):
            self._check(rc)
        return eig, vec, stats

    # ---- field coupling and optimal control ---------------------------------------
    def set_dipole(self, coef, idx, elec=None):
        """Dipole mu(Q) from monomials (coef[m], idx[m, 0:4] with -1 unused, elec[m] = (a, b))."""
        coef = _darr(coef)
        idx = _iarr(np.asarray(idx).reshape(-1, 4))
        elec = _iarr(np.zeros((len(coef), 2)) if elec is None else np.asarray(elec).reshape(-1, 2))
        self._check(load().evr_set_dipole(self.h, len(coef), _p(coef, _dp), _p(idx, _ip), _p(elec, _ip)))

    def set_ggrid(self, G):
        """Kinetic metric G(Q) per grid point (sum_nq x D x D, the reference's point order) in
        place of G0 + g.Q (type-10 contexts)."""
        D = self.spec.D
        G = np.ascontiguousarray(np.asarray(G, dtype=np.float64).reshape(self.sum_nq, D, D).transpose(0, 2, 1))
        self._check(load().evr_set_ggrid(self.h, _p(G, _dp)))

    def set_jacobian(self, jac=None, rho=None):
        """Jacobian and rho per grid point (the reference's whole-grid order) of a type-10
        operator; None, None removes them (Jac = rho = 1)."""
        if jac is None and rho is None:
            self._check(load().evr_set_jacobian(self.h, None, None))
            return
        j = _darr(np.asarray(jac, dtype=np.float64).ravel())
        r = _darr(np.asarray(rho, dtype=np.float64).ravel())
        if j.size != self.sum_nq or r.size != self.sum_nq:
            raise EvrError(EVR_EINVAL, f"Jacobian / rho need {self.sum_nq} values")
        self._check(load().evr_set_jacobian(self.h, _p(j, _dp), _p(r, _dp)))

    def set_dipole_grid(self, mu, layout="terms"):
        """Dipole mu(Q) as grid values (layouts of set_vgrid) instead of monomials."""
        mu = _darr(np.asarray(mu, dtype=np.float64).ravel(order="F"))
        if mu.size != self.sum_nq * self.spec.nb0 ** 2:
            raise EvrError(EVR_EINVAL, f"dipole grid has {mu.size} values, expected {self.sum_nq * self.spec.nb0 ** 2}")
        self._check(load().evr_set_dipole_grid(self.h, _p(mu, _dp), VGRID_LAYOUT[layout]))

    def set_field(self, vw=1.0, mw=0.0, keo=True):
        """Grid operator vw*V + mw*mu (+ kinetic part) of later H.psi / Davidson / Chebyshev calls."""
        self._check(load().evr_set_field(self.h, float(vw), float(mw), 1 if keo else 0))

    def oc_forward(self, field, psi0, target, dt, emin, emax, poly_tol=1e-14, checkpoint=0, prec="fp64",
                   want_psi=False):
        """J = |<target|psi(T)>|^2 under H0 - E_n mu; returns (J, overlap, psiT or None, info)."""
        field = _darr(field)
        o = OcOpts()
        o.nsteps, o.dt, o.emin, o.emax = len(field), dt, emin, emax
        o.poly_tol, o.checkpoint, o.prec = poly_tol, checkpoint, PREC[prec]
        p0 = _darr(np.stack([np.real(psi0), np.imag(psi0)], axis=1))
        tg = _darr(np.stack([np.real(target), np.imag(target)], axis=1))
        out3 = np.zeros(3)
        psiT = np.zeros((self.N, 2)) if want_psi else None
        info = np.zeros(3, dtype=np.int64)
        self._check(load().evr_oc_forward(self.h, C.byref(o), _p(field, _dp), _p(p0, _dp), _p(tg, _dp),
                                          _p(out3, _dp), _p(psiT, _dp), _p(info, _lp)))
        psi = psiT[:, 0] + 1j * psiT[:, 1] if want_psi else None
        return out3[0], complex(out3[1], out3[2]), psi, dict(order=int(info[0]), columns=int(info[1]),
                                                              checkpoints=int(info[2]))

    def oc_backward(self, nsteps, want_ref=True):
        """dJ/dE_n of the last oc_forward, and the continuous-time gradient at t_n = n dt."""
        grad = np.zeros(nsteps)
        ref = np.zeros(nsteps + 1) if want_ref else None
        info = np.zeros(3, dtype=np.int64)
        self._check(load().evr_oc_backward(self.h, _p(grad, _dp), _p(ref, _dp), _p(info, _lp)))
        return grad, ref, dict(columns=int(info[0]), checkpoints=int(info[1]), segment=int(info[2]))

    def autotune(self, nvec=64, prec="fp64"):
        """Choose the work decomposition by timing; returns (slab cap, general cap,
        small-term threshold, ms), and for FP32 the tensor-core threshold (-1: CUDA cores)
        before the time."""
        caps = np.zeros(4, dtype=np.int32)
        ms = np.zeros(1)
        self._check(load().evr_autotune(self.h, nvec, PREC[prec], _p(caps, _ip), _p(ms, _dp)))
        if prec == "fp32":
            return int(caps[0]), int(caps[1]), int(caps[2]), int(caps[3]), float(ms[0])
        return int(caps[0]), int(caps[1]), int(caps[2]), float(ms[0])

    def set_kernel_path(self, path):
        """1 or True (default): stage kernels for single-term problems, else small terms in the
        general kernel, the slab kernel for the other terms that fit and the general kernel
        for the rest; 2: the slab kernel for every term that fits (small ones included), no
        stage kernels; 0 or False: general kernel only.  Names "auto", "slab", "general" work too."""
        names = {"auto": 1, "stages": 1, "slab": 2, "general": 0}
        v = names[path] if isinstance(path, str) else (1 if path is True else 0 if path is False else int(path))
        self._check(load().evr_set_kernel_path(self.h, v))

    def set_tensor_cores(self, on=True, min_km=64):
        """FP32 H.psi: mode contractions of the slab kernel on tcgen05 tensor cores (on) or on
        the CUDA cores (off); contractions with K*M < min_km stay on the CUDA cores."""
        self._check(load().evr_set_tensor_cores(self.h, 1 if on else 0, int(min_km)))

    def set_operator(self, form):
        """'H' (the reference's OpPsi), 'HT' (its transpose) or 'HSYM' ((H+H^T)/2)."""
        self._check(load().evr_set_operator(self.h, {"H": 0, "HT": 1, "HSYM": 2}[form]))

    def lanczos(self, nev, ncv=0, max_restarts=300, tol=0.0, v0=None, sym=-1, seed=1, want_vectors=False):
        """Restarted Lanczos for the lowest nev levels (the reference's ARPACK path,
        sub_propagation_Arpack_Sym); returns (eig, vectors or None, rel_resid, stats)."""
        L = load()
        o = LanczosOpts()
        o.nev, o.ncv, o.max_restarts, o.tol, o.sym, o.seed = nev, ncv, max_restarts, tol, sym, seed
        v = None if v0 is None else np.ascontiguousarray(v0, dtype=np.float64).reshape(self.N)
        eig, rres = np.zeros(nev), np.zeros(nev)
        vec = np.zeros((self.N, nev), order="F") if want_vectors else None
        info = np.zeros(4, dtype=np.int64)
        rc = L.evr_lanczos(self.h, C.byref(o), _p(v, _dp), _p(eig, _dp), _p(vec, _dp), _p(rres, _dp), _p(info, _lp))
        stats = dict(restarts=int(info[0]), hpsi=int(info[1]), converged=int(info[2]), ncv=int(info[3]))
        if rc not in (0, EVR_ENOCONV):
            self._check(rc)
        return eig, vec, rres, stats

    def filter_diag(self, hmin, hmax, e0, width, n_filters, max_order=2000, q0=None, nstart=1, prec="fp64",
                    conv_resi=1e-6, seed=1, want_vectors=False):
        """Gaussian filter diagonalisation (sub_GaussianFilterDiagonalization) of the levels
        in the window of `width` au around e0; q0: optional start vectors (N x nstart).
        Returns dict(eig, resid, vec, lambda_min, lambda_max, non_hermitic, order, hpsi,
        kept, in_window, converged_in_window)."""
        L = load()
        o = FilterOpts()
        o.hmin, o.hmax, o.e0, o.width = hmin, hmax, e0, width
        o.n_filters, o.max_order, o.prec, o.conv_resi, o.seed = n_filters, max_order, PREC[prec], conv_resi, seed
        q = None
        if q0 is not None:
            q = np.asfortranarray(np.asarray(q0, dtype=np.float64).reshape(self.N, -1))
            nstart = q.shape[1]
        o.nstart = nstart
        K = n_filters * nstart
        eig, resid = np.zeros(K), np.zeros(K)
        vec = np.zeros((self.N, K), order="F") if want_vectors else None
        nout = C.c_int(0)
        win = np.zeros(3)
        info = np.zeros(5, dtype=np.int64)
        self._check(L.evr_filter_diag(self.h, C.byref(o), _p(q, _dp), _p(eig, _dp), _p(resid, _dp), _p(vec, _dp),
                                      C.byref(nout), _p(win, _dp), _p(info, _lp)))
        k = nout.value
        return dict(eig=eig[:k], resid=resid[:k], vec=None if vec is None else vec[:, :k], lambda_min=win[0],
                    lambda_max=win[1], non_hermitic=win[2], order=int(info[0]), hpsi=int(info[1]), kept=int(info[2]),
                    in_window=int(info[3]), converged_in_window=int(info[4]))

    def sil(self, psi0, dt, nsteps, npoly=64, poly_tol=1e-10, prec="fp64", want_psi=False):
        """Short-iterative-Lanczos propagation (march_SIL) of complex packets psi0 (N x npsi);
        returns (autocorr (nsteps+1) x npsi, final packets or None, info)."""
        psi0 = np.asarray(psi0, dtype=np.complex128)
        if psi0.ndim == 1:
            psi0 = psi0[:, None]
        N, npsi = psi0.shape
        buf = np.ascontiguousarray(psi0.T).view(np.float64)
        ac = np.zeros((nsteps + 1) * npsi * 2)
        out = np.zeros(npsi * 2 * N) if want_psi else None
        info = np.zeros(3, dtype=np.int64)
        self._check(load().evr_sil_propagate(self.h, _p(buf, _dp), npsi, dt, nsteps, npoly, poly_tol, PREC[prec],
                                             _p(ac, _dp), _p(out, _dp), _p(info, _lp)))
        autocorr = ac.view(np.complex128).reshape(nsteps + 1, npsi)
        psi = out.view(np.complex128).reshape(npsi, N).T.copy() if want_psi else None
        return autocorr, psi, dict(krylov_dim=int(info[0]), hpsi=int(info[1]), status=int(info[2]))

    def chebyshev(self, psi0, dt, nsteps, emin, emax, poly_tol=1e-10, prec="fp64", want_psi=False):
        """Chebyshev propagation of complex packets psi0 (N x npsi, complex128)."""
        L = load()
        psi0 = np.asarray(psi0, dtype=np.complex128)
        if psi0.ndim == 1:
            psi0 = psi0[:, None]
        N, npsi = psi0.shape
        buf = np.ascontiguousarray(psi0.T).view(np.float64)  # packet p: 2N doubles (re, im per element)
        ac = np.zeros((nsteps + 1) * npsi * 2)
        out = np.zeros(npsi * 2 * N) if want_psi else None
        info = np.zeros(3, dtype=np.int64)
        self._check(L.evr_cheby_propagate(self.h, _p(buf, _dp), npsi, dt, nsteps, emin, emax, poly_tol, PREC[prec],
                                          _p(ac, _dp), _p(out, _dp), _p(info, _lp)))
        autocorr = ac.view(np.complex128).reshape(nsteps + 1, npsi)
        psi = out.view(np.complex128).reshape(npsi, N).T.copy() if want_psi else None
        return autocorr, psi, dict(max_order=int(info[0]), hpsi=int(info[1]), status=int(info[2]))


class BatchProblem(Problem):
    """Independent problems stacked in one context (evr_create_batch): vectors hold every
    problem's packed functions (problem s in rows offsets[s]:offsets[s+1]); H.psi applies
    the block-diagonal H in one launch; ``davidson`` runs all problems in lock-step."""

    def __init__(self, specs, device: int = 0):
        L = load()
        self.specs = list(specs)
        self.spec = self.specs[0]
        self._keep = []
        arr = (ProblemDesc * len(self.specs))(*[_describe(sp, self._keep) for sp in self.specs])
        self._keep.append(arr)
        h = C.c_void_p()
        rc = L.evr_create_batch(C.byref(h), arr, len(self.specs), device)
        self._finish(h, rc, device)
        off = np.zeros(len(self.specs) + 1, dtype=np.int64)
        self._check(L.evr_batch_offsets(self.h, _p(off, _lp)))
        self.offsets = off

    def davidson(self, n_levels, block=None, max_dim=None, max_it=200, conv_resi=1e-7, conv_ene=1e-10,
                 prec="fp64", sym=-1):
        L = load()
        o = DavidsonOpts()
        o.n_levels = n_levels
        o.block = block or n_levels
        o.max_dim = max_dim or 64
        o.max_it = max_it
        o.conv_resi, o.conv_ene = conv_resi, conv_ene
        o.prec = PREC[prec]
        o.sym = sym
        eig = np.zeros((len(self.specs), n_levels))
        info = np.zeros(4, dtype=np.int64)
        rc = L.evr_batch_davidson(self.h, C.byref(o), _p(eig, _dp), _p(info, _lp))
        stats = dict(iterations=int(info[0]), hpsi_fp64=int(info[1]), hpsi_fp32=int(info[2]),
                     converged=bool(info[3]))
        if rc not in (0, EVR_ENOCONV):
            self._check(rc)
        return eig, stats
