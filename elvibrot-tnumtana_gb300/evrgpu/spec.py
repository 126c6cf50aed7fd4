"""Problem descriptions for the H.psi path: bases, Smolyak rules and operators.

A ``ProblemSpec`` carries exactly what the reference's input namelists fix for the
OpPsi path (``&basis_nD`` with ``L_TO_nq_A/B``, ``L_SparseGrid``, ``L_SparseBasis``,
``Q0``, ``scaleQ``; the potential plugin ``calcN_op``; the KEO form selected by
``Type_HamilOp``), in plain arrays:

* ``kind = "sg4"``: Smolyak SparseGrid_type=4 basis, nq(l) = Aq + Bq*l and
  nb(l) = Ab + Bb*l per mode (Source_ElVibRot/sub_Basis/sub_module_Basis_LTO_n.f90:443),
  levels 0..LG, packed basis restricted by sum l(n_i) <= LB.
* ``kind = "dp"``: direct-product basis with nb_dp/nq_dp per mode.

The potential is a polynomial in Q given as monomials (coef, up to four mode
indices, electronic element) -- the values the reference caches on the grid with
``Save_MemGrid`` (sub_OpPsi_SG4.f90:2642-2668).  The KEO is either type 10,
-1/2 sum_ij d_i G_ij(Q) d_j with G(Q) = G0 + sum_k g_ijk Q_k
(sub_OpPsi_SG4.f90:1548-1650), or type 1 with a constant G0 (F2 = -G0/2,
sub_OpPsi_SG4.f90:1490-1546).

The seeded workload generators reproduce the shapes and value distributions of the
benchmark workloads; all random draws use ``numpy.random.default_rng(seed)``.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from itertools import combinations_with_replacement

import numpy as np


# --- CODATA 2006 constants, as the reference derives them
# (Source_PhysicalConstants/sub_module_constant.f90:274-318, :786-804)
def _codata2006():
    c = 299792458.0
    mu0 = math.pi * 4.0e-7
    h = 6.62606896e-34
    e = 1.602176487e-19
    me = 9.10938215e-31
    eps0 = 1.0 / (mu0 * c * c)
    hb = h / (2.0 * math.pi)
    a0 = (hb / e) ** 2 / me * 4.0 * math.pi * eps0
    Eh = (e * e / a0) / (4.0 * math.pi * eps0)
    Ta = hb / Eh
    au_to_cm = 1.0 / (Ta * 2.0 * math.pi * c * 100.0)
    au_to_ev = Eh / e
    fs_to_au = 1.0e-15 / Ta
    return au_to_cm, au_to_ev, fs_to_au


AU_TO_CM, AU_TO_EV, FS_TO_AU = _codata2006()


@dataclass
class ProblemSpec:
    kind: str                      # "sg4" or "dp"
    D: int
    nb0: int = 1
    LG: int = 0
    LB: int = 0
    Aq: np.ndarray = None
    Bq: np.ndarray = None
    Ab: np.ndarray = None
    Bb: np.ndarray = None
    nq_dp: np.ndarray = None
    nb_dp: np.ndarray = None
    scaleQ: np.ndarray = None
    Q0: np.ndarray = None
    mono_coef: np.ndarray = None   # (M,)
    mono_idx: np.ndarray = None    # (M,4) int, -1 = unused
    mono_elec: np.ndarray = None   # (M,2) int (ib0, jb0)
    keo_type: int = 10
    G0: np.ndarray = None          # (D,D)
    g: np.ndarray = None           # (D,D,D), g[i,j,k] multiplies Q_k
    dip_coef: np.ndarray = None    # optional dipole mu(Q), monomials like the potential
    dip_idx: np.ndarray = None
    dip_elec: np.ndarray = None
    # optional host tables of the primitive bases ((mode, level) order: dicts with x, w,
    # d0b, d1b, d2b on the grid); None: HO bases on Gauss-Hermite grids
    bases: list = None
    name: str = ""
    extra: dict = field(default_factory=dict)

    def __post_init__(self):
        D = self.D
        if self.scaleQ is None:
            self.scaleQ = np.ones(D)
        if self.Q0 is None:
            self.Q0 = np.zeros(D)
        if self.G0 is None:
            self.G0 = np.eye(D)
        if self.g is None:
            self.g = np.zeros((D, D, D))
        if self.mono_elec is None and self.mono_coef is not None:
            self.mono_elec = np.zeros((len(self.mono_coef), 2), dtype=np.int32)
        if self.dip_elec is None and self.dip_coef is not None:
            self.dip_elec = np.zeros((len(self.dip_coef), 2), dtype=np.int32)
        for k in ("Aq", "Bq", "Ab", "Bb", "nq_dp", "nb_dp"):
            v = getattr(self, k)
            if v is not None:
                setattr(self, k, np.asarray(v, dtype=np.int32))
        self.scaleQ = np.asarray(self.scaleQ, dtype=np.float64)
        self.Q0 = np.asarray(self.Q0, dtype=np.float64)


class Poly:
    """Accumulates polynomial monomials for the potential."""

    def __init__(self):
        self.coef, self.idx, self.elec = [], [], []

    def add(self, c, modes, ib0=0, jb0=0):
        m = list(modes) + [-1] * (4 - len(modes))
        assert len(m) == 4
        self.coef.append(float(c))
        self.idx.append(m)
        self.elec.append([ib0, jb0])

    def arrays(self):
        return (np.array(self.coef, dtype=np.float64), np.array(self.idx, dtype=np.int32).reshape(-1, 4),
                np.array(self.elec, dtype=np.int32).reshape(-1, 2))


# ------------------------------------------------------------------------------------
# Reference golden-test systems
# ------------------------------------------------------------------------------------
def henon_heiles(D: int = 6, L: int = 3, lam: float = 0.111803) -> ProblemSpec:
    """D-mode Henon-Heiles on SG4 with nb = nq = 1 + 2l ("Hm" bases, L_TO_nq_A=1,
    L_TO_nq_B=2), type-1 KEO with G = 1 (Gcte): the 6D_Davidson_S0 golden test
    (Working_tests/MPI_tests/6D_Davidson_S0/shell_run, sub_system_HenonHeiles.f:24-41)."""
    p = Poly()
    for i in range(D):
        p.add(0.5, [i, i])
    for i in range(D - 1):
        p.add(lam, [i, i, i + 1])
        p.add(-lam / 3.0, [i + 1, i + 1, i + 1])
    c, idx, el = p.arrays()
    one = np.ones(D, dtype=np.int32)
    return ProblemSpec(kind="sg4", D=D, LG=L, LB=L, Aq=one, Bq=2 * one, Ab=one, Bb=2 * one,
                       mono_coef=c, mono_idx=idx, mono_elec=el, keo_type=1, name=f"HH{D}D_L{L}")


PYRAZINE_W = [0.09357, 0.0740, 0.1273, 0.1568, 0.1347, 0.3431, 0.1157, 0.3242, 0.3621, 0.2673, 0.3052, 0.0968]
PYRAZINE_K1 = [0.0, -0.0964, 0.0470, 0.1594, 0.0308, 0.0782, 0.0261, 0.0717, 0.0560, 0.0625, 0.0780, 0.0188]
PYRAZINE_K2 = [0.0, 0.1194, 0.2012, 0.0484, -0.0308, -0.0782, -0.0261, -0.0717, -0.0560, -0.0625, -0.0780, -0.0188]


def pyrazine_12d(L: int = 1) -> ProblemSpec:
    """12-D two-state pyrazine vibronic model on SG4 (12D_propagation_S0 golden test):
    nb = nq = 1 + B_i l with B = 3,3,2,2,2,... (shell_run), V from sub_system_pyrazine.f
    (in eV, converted with the reference's CODATA-2006 eV), analytic type-1 KEO
    F2(i,i) = -w_i/2 (calc_f2_f1Q.f90)."""
    return pyrazine_vibronic(PYRAZINE_W, PYRAZINE_K1, PYRAZINE_K2, 0.46165, 0.1825, [3, 3, 2, 2] + [2] * 8, L)


def pyrazine_vibronic(w, k1, k2, delta, lam, B, L, name="pyrazine") -> ProblemSpec:
    """Two-state pyrazine vibronic model of the reference's propagation tests for any number
    of modes (sub_system_pyrazine.f): V11 = 1/2 sum w_i Q_i^2 - delta + sum k1_i Q_i,
    V22 = 1/2 sum w_i Q_i^2 + delta + sum k2_i Q_i, V12 = lam Q_1 (eV), analytic type-1 KEO
    F2(i,i) = -w_i/2, HO bases nb = nq = 1 + B_i l on SG4 level L."""
    D = len(w)
    ev = 1.0 / AU_TO_EV
    w = np.asarray(w, dtype=np.float64)
    p = Poly()
    for e in (0, 1):
        for i in range(D):
            p.add(0.5 * w[i] * ev, [i, i], e, e)
    p.add(-delta * ev, [], 0, 0)
    p.add(delta * ev, [], 1, 1)
    for i in range(D):
        if k1[i] != 0.0:
            p.add(k1[i] * ev, [i], 0, 0)
        if k2[i] != 0.0:
            p.add(k2[i] * ev, [i], 1, 1)
    p.add(lam * ev, [0], 0, 1)
    p.add(lam * ev, [0], 1, 0)
    c, idx, el = p.arrays()
    B = np.asarray(B, dtype=np.int32)
    one = np.ones(D, dtype=np.int32)
    return ProblemSpec(kind="sg4", D=D, nb0=2, LG=L, LB=L, Aq=one, Bq=B, Ab=one, Bb=B,
                       mono_coef=c, mono_idx=idx, mono_elec=el, keo_type=1, G0=np.diag(w * ev),
                       name=f"{name}{D}D_L{L}")


# ------------------------------------------------------------------------------------
# Synthetic benchmark workloads (seeded)
# ------------------------------------------------------------------------------------
def anharmonic_poly(D, omega, rng, cubic_sigma, quartic_sigma, g_amp, cubic_window=None):
    """V = sum 1/2 w_i^2 Q_i^2 + sum_{i<=j<=k} c_ijk q_i q_j q_k + sum_{i<=j<=k<=l} d_ijkl q_i q_j q_k q_l,
    G_ij = delta_ij + sum_k g_ijk q_k (g ~ U(-g_amp, g_amp), symmetrised in i,j), with
    q = sqrt(w) Q the dimensionless normal coordinates of the harmonic reference
    (Q is the unit-mass coordinate of the kinetic operator)."""
    omega = np.asarray(omega, dtype=np.float64)
    s = np.sqrt(omega)
    p = Poly()
    for i in range(D):
        p.add(0.5 * omega[i] ** 2, [i, i])
    for (i, j, k) in combinations_with_replacement(range(D), 3):
        if cubic_window is not None and k - i > cubic_window:
            continue
        c = rng.normal(0.0, cubic_sigma)
        p.add(c * s[i] * s[j] * s[k], [i, j, k])
    if quartic_sigma > 0:
        for (i, j, k, l) in combinations_with_replacement(range(D), 4):
            d = rng.normal(0.0, quartic_sigma)
            p.add(d * s[i] * s[j] * s[k] * s[l], [i, j, k, l])
    g = np.zeros((D, D, D))
    if g_amp > 0:
        g = rng.uniform(-g_amp, g_amp, size=(D, D, D))
        g = 0.5 * (g + g.transpose(1, 0, 2))
        g = g * s[None, None, :]
    c, idx, el = p.arrays()
    return c, idx, el, g


def config_dp3(seed: int = 0, nb: int = 20, nq: int = 24) -> ProblemSpec:
    """Direct product D=3, HO nb=20 on GH nq=24, w = [0.010, 0.0092, 0.0035] Eh,
    type-10 KEO with G = 1 + g.q, cubic and quartic couplings."""
    D = 3
    omega = np.array([0.010, 0.0092, 0.0035])
    rng = np.random.default_rng(seed)
    c, idx, el, g = anharmonic_poly(D, omega, rng, 1e-5, 1e-6, 0.01)
    return ProblemSpec(kind="dp", D=D, nq_dp=[nq] * D, nb_dp=[nb] * D, scaleQ=np.sqrt(omega),
                       mono_coef=c, mono_idx=idx, mono_elec=el, keo_type=10, g=g, name="DP3_nb20_nq24")


def config_sg4(D: int = 6, L: int = 8, seed: int = 1, wlo=0.003, whi=0.015, nq_A=3, cubic_sigma=1e-5,
               quartic_sigma=1e-6, g_amp=0.01, cubic_window=None) -> ProblemSpec:
    """SG4 D modes, level L, HO bases nb(l) = 2l+1, nq(l) = nq_A + 2l, w ~ U(wlo, whi),
    type-10 KEO with G = 1 + g.q and the anharmonic couplings of ``anharmonic_poly``."""
    rng = np.random.default_rng(seed)
    omega = rng.uniform(wlo, whi, size=D)
    c, idx, el, g = anharmonic_poly(D, omega, rng, cubic_sigma, quartic_sigma, g_amp, cubic_window)
    one = np.ones(D, dtype=np.int32)
    return ProblemSpec(kind="sg4", D=D, LG=L, LB=L, Aq=nq_A * one, Bq=2 * one, Ab=one, Bb=2 * one,
                       scaleQ=np.sqrt(omega), mono_coef=c, mono_idx=idx, mono_elec=el, keo_type=10, g=g,
                       name=f"SG4_D{D}_L{L}_nq{nq_A}+2l", extra=dict(omega=omega))


def config_sg4_6d_l8(seed: int = 1) -> ProblemSpec:
    """The D=6 Smolyak SG4 level-8 workload: nb(l)=2l+1, nq(l)=2l+3, w ~ U(0.003,0.015)."""
    return config_sg4(6, 8, seed)


def config_sg4_12d_l6(seed: int = 3) -> ProblemSpec:
    """The D=12 SG4 level-6 propagation workload: nb = nq = 2l+1, w ~ U(0.002, 0.02),
    cubic couplings only between modes within a window of three neighbours, G = 1."""
    return config_sg4(12, 6, seed, wlo=0.002, whi=0.02, nq_A=1, cubic_sigma=5e-6, quartic_sigma=0.0,
                      g_amp=0.0, cubic_window=2)


def dipole_poly(D, omega, rng, mu0=0.1, a_sigma=0.1, b_sigma=0.01):
    """mu = mu0 + sum_i a_i q_i + sum_{i<=j} b_ij q_i q_j, a ~ N(0, a_sigma), b ~ N(0, b_sigma),
    on the dimensionless q = sqrt(w) Q of ``anharmonic_poly``."""
    s = np.sqrt(np.asarray(omega, dtype=np.float64))
    p = Poly()
    p.add(mu0, [])
    for i in range(D):
        p.add(rng.normal(0.0, a_sigma) * s[i], [i])
    for (i, j) in combinations_with_replacement(range(D), 2):
        p.add(rng.normal(0.0, b_sigma) * s[i] * s[j], [i, j])
    return p.arrays()


def config_oc(seed: int = 0, nb: int = 20, nq: int = 24, D: int = 3, omega=(0.010, 0.0092, 0.0035)) -> ProblemSpec:
    """The optimal-control system: the direct-product system of ``config_dp3`` (D=3, nb=20,
    nq=24) with a dipole mu(Q) = mu0 + sum a_i q_i + sum b_ij q_i q_j, a ~ N(0, 0.1),
    b ~ N(0, 0.01).  Smaller nb/nq/D give the test-size versions."""
    omega = np.asarray(omega[:D], dtype=np.float64)
    rng = np.random.default_rng(seed)
    c, idx, el, g = anharmonic_poly(D, omega, rng, 1e-5, 1e-6, 0.01)
    dc, di, de = dipole_poly(D, omega, rng)
    return ProblemSpec(kind="dp", D=D, nq_dp=[nq] * D, nb_dp=[nb] * D, scaleQ=np.sqrt(omega),
                       mono_coef=c, mono_idx=idx, mono_elec=el, keo_type=10, g=g, dip_coef=dc, dip_idx=di,
                       dip_elec=de, name=f"OC_DP{D}_nb{nb}_nq{nq}", extra=dict(omega=omega))


def oc_field(nsteps: int = 4000, dt: float = 5.0, seed: int = 0, n_sin: int = 8, amp: float = 0.005,
             wlo: float = 0.002, whi: float = 0.03) -> np.ndarray:
    """Control field E_n = sum_k amp sin(w_k t_n + phi_k) at the step midpoints
    t_n = (n + 1/2) dt, w_k ~ U(wlo, whi), phi_k ~ U(0, 2 pi)."""
    rng = np.random.default_rng(seed)
    w = rng.uniform(wlo, whi, size=n_sin)
    ph = rng.uniform(0.0, 2.0 * np.pi, size=n_sin)
    t = (np.arange(nsteps) + 0.5) * dt
    return (amp * np.sin(np.outer(t, w) + ph[None, :])).sum(axis=1)


def displaced_gaussian(spec: ProblemSpec, problem, modes, shift: float) -> np.ndarray:
    """Harmonic ground state displaced by `shift` (dimensionless q) in `modes`, on the packed
    basis of `problem`: product of coherent-state amplitudes e^{-a^2/2} a^k / sqrt(k!),
    a = shift/sqrt(2), restricted to the packed functions and normalised (complex128)."""
    packed = problem.tables()["packed"] - 1          # HO quantum numbers, Np x D
    a = shift / math.sqrt(2.0)
    kmax = int(packed.max()) + 1
    lf = np.array([math.lgamma(k + 1.0) for k in range(kmax)])
    amp = np.exp(-0.5 * a * a + np.arange(kmax) * math.log(a) - 0.5 * lf)
    c = np.ones(len(packed))
    for i in range(spec.D):
        k = packed[:, i]
        c *= amp[k] if i in modes else (k == 0).astype(float)
    c = np.tile(c, spec.nb0) if spec.nb0 > 1 else c
    return (c / np.linalg.norm(c)).astype(np.complex128)


def spectral_bounds(spec: ProblemSpec, margin: float = 0.1):
    """Bounds [emin, emax] of a harmonic-dominated SG4 Hamiltonian from its frequencies:
    zero-point energy and the largest number of quanta of the packed basis (nb(l)-1 per
    mode, sum of levels <= LB), widened by `margin` for the anharmonic couplings."""
    w = np.asarray(spec.extra.get("omega", np.ones(spec.D)))
    zpe = 0.5 * w.sum()
    quanta = max(int(spec.Ab[i] + spec.Bb[i] * spec.LB) - 1 for i in range(spec.D))
    top = zpe + quanta * w.max()
    return zpe * (1.0 - margin), top * (1.0 + margin)


def batched_systems(n: int = 256, seed: int = 2):
    """Uneven batch: D ~ U{3..6}, L ~ U{4..8}, each system seeded from ``seed``."""
    rng = np.random.default_rng(seed)
    out = []
    for s in range(n):
        D = int(rng.integers(3, 7))
        L = int(rng.integers(4, 9))
        out.append(config_sg4(D, L, seed=int(rng.integers(0, 2**31 - 1))))
    return out
