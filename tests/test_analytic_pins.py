"""Pins of the headline operator that depend on neither the oracle nor the library: exact
matrix elements of H in harmonic-oscillator bases (``galerkin.py``, ladder operators).

The type-10 operator with nq > nb takes its grid derivative from the pseudo-inverse of the
basis on the grid (d1gg = d1b . pinv(d0b), sub_dnGB_TO_dnGG,
Source_ElVibRot/sub_Basis/sub_module_basis.f90:2195-2460).  That derivative is exact on
grid values of functions inside the basis span, so for a basis function n whose chain
d_j -> G(Q) -> d_i stays inside the span of every mode (n_i <= nb - 3 with a Q-dependent G,
nb - 2 with a constant one) and Gauss-Hermite rules of nq >= nb + 2 points, the column
H[:, n] is the exact Galerkin column.  On a Smolyak basis the combination technique gives
H[m, n] = c(m, n) <m|H|n> with c the summed weights of the terms holding both m and n
(``galerkin.pair_weights``).  What these tests fix, independently of the restatement:

* the direct-product benchmark operator (D=3, nb=20, nq=24, cubic + quartic V,
  G(Q) = 1 + g.q): every checked column to 1e-12 relative;
* a Smolyak type-10 operator with a Q-dependent G, non-diagonal G0 and anharmonic V
  (nb(l) = 3 + 3l, nq(l) = 5 + 3l), same bound;
* a separable harmonic Smolyak operator (type 1, nq > nb) is diagonal with the harmonic
  energies sum_i w_i (n_i + 1/2): Davidson levels to 1e-10 au, FP64 and mixed;
* with a constant non-diagonal G0, the type-10 operator equals the type-1 operator on the
  columns inside the span (an identity between the library's two code paths), 1e-12.

The CPU tests check the oracle against the same answers; the GPU tests the library through
the C ABI.
"""
import numpy as np
import pytest

import galerkin as GK
from evrgpu import spec as S
from evrgpu import lib as E
from oracle import oracle as O

TOL = 1e-12       # relative, max norm over the checked columns
LEVEL_TOL = 1e-10  # au


def sg4_deep(D, L, seed=4, keo=10, g_amp=0.01, harmonic=False):
    """Smolyak operator with nb(l) = 3 + 3l and nq(l) = 5 + 3l: the functions n = 0, 3, 6,
    ... of each mode lie two functions below the top of their own level's basis."""
    rng = np.random.default_rng(seed)
    om = rng.uniform(0.003, 0.015, size=D)
    if harmonic:
        p = S.Poly()
        for i in range(D):
            p.add(0.5 * om[i] ** 2, [i, i])
        c, idx, el = p.arrays()
        g = None
        G0 = np.eye(D)
    else:
        c, idx, el, g = S.anharmonic_poly(D, om, rng, 1e-5, 1e-6, g_amp)
        G0 = np.eye(D) + 0.05 * rng.uniform(-1.0, 1.0, (D, D))
        G0 = 0.5 * (G0 + G0.T)
    one = np.ones(D, dtype=np.int32)
    return S.ProblemSpec(kind="sg4", D=D, LG=L, LB=L, Aq=5 * one, Bq=3 * one, Ab=3 * one, Bb=3 * one,
                         scaleQ=np.sqrt(om), mono_coef=c, mono_idx=idx, mono_elec=el, keo_type=keo, G0=G0,
                         g=g if keo == 10 else None, name=f"SG4deep_D{D}_L{L}_type{keo}", extra=dict(omega=om))


def harmonic_sg4(D, L, seed=3, keo=1):
    """Separable harmonic V on SG4 with nb(l) = 2l+1, nq(l) = 2l+3 (the benchmark's rules)."""
    rng = np.random.default_rng(seed)
    om = rng.uniform(0.003, 0.015, size=D)
    p = S.Poly()
    for i in range(D):
        p.add(0.5 * om[i] ** 2, [i, i])
    c, idx, el = p.arrays()
    one = np.ones(D, dtype=np.int32)
    return S.ProblemSpec(kind="sg4", D=D, LG=L, LB=L, Aq=3 * one, Bq=2 * one, Ab=one, Bb=2 * one,
                         scaleQ=np.sqrt(om), mono_coef=c, mono_idx=idx, mono_elec=el, keo_type=keo,
                         name=f"harmonic_SG4_D{D}_L{L}", extra=dict(omega=om))


def const_g0(spec, keo):
    """The same operator with G(Q) = G0 constant and non-diagonal, as type `keo`."""
    D = spec.D
    i = np.arange(D)
    G0 = np.eye(D) + 0.08 * (-1.0) ** np.add.outer(i, i) * (1 - np.eye(D))
    return S.ProblemSpec(kind=spec.kind, D=D, LG=spec.LG, LB=spec.LB, Aq=spec.Aq, Bq=spec.Bq, Ab=spec.Ab,
                         Bb=spec.Bb, nq_dp=spec.nq_dp, nb_dp=spec.nb_dp, scaleQ=spec.scaleQ,
                         mono_coef=spec.mono_coef, mono_idx=spec.mono_idx, mono_elec=spec.mono_elec,
                         keo_type=keo, G0=G0, name=spec.name + f"_G0_type{keo}")


def inside(spec, packed, margin):
    """Packed functions whose quantum numbers lie `margin` below the top of their own
    level's basis (direct product: of the mode's basis) in every mode."""
    if spec.kind == "dp":
        return np.all(packed <= np.asarray(spec.nb_dp) - margin, axis=1)
    Ab, Bb = np.asarray(spec.Ab), np.asarray(spec.Bb)
    return np.all(packed <= Ab + Bb * GK.level_of(packed, Ab, Bb) - margin, axis=1)


def exact_columns(spec, packed, cols, nmax):
    """Exact H[:, n] on the packed basis for the packed indices `cols`."""
    gk = GK.Galerkin(spec, nmax)
    gal = gk.columns([tuple(packed[n]) for n in cols])
    ref = np.zeros((len(packed), len(cols)))
    for c, n in enumerate(cols):
        v = gal[tuple(packed.T) + (c,)]
        if spec.kind == "sg4":
            v = v * GK.pair_weights(spec, packed, packed[n])
        ref[:, c] = v
    return ref


def unit_block(N, cols):
    psi = np.zeros((N, len(cols)))
    psi[cols, np.arange(len(cols))] = 1.0
    return psi


def rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


GALERKIN_CASES = {
    # name: (spec builder, truncation of the ladder algebra, columns checked (None = all))
    "dp3_benchmark_nb20_nq24": (lambda: S.config_dp3(), 26, 48),
    "dp3_nb9_nq12": (lambda: S.config_dp3(nb=9, nq=12), 14, None),
    "sg4_d3_l3_type10_gq": (lambda: sg4_deep(3, 3), 18, None),
    "sg4_d4_l3_type10_gq": (lambda: sg4_deep(4, 3, seed=5), 18, None),
    "sg4_d3_l3_type1": (lambda: sg4_deep(3, 3, keo=1), 18, None),
}


def galerkin_case(name):
    build, nmax, ncols = GALERKIN_CASES[name]
    spec = build()
    packed = E.Problem(spec, device=-1).tables()["packed"] - 1
    cols = np.nonzero(inside(spec, packed, 3))[0]
    if ncols is not None and ncols < len(cols):
        cols = np.sort(np.random.default_rng(0).choice(cols, size=ncols, replace=False))
    return spec, packed, cols, exact_columns(spec, packed, cols, nmax)


@pytest.mark.parametrize("name", list(GALERKIN_CASES))
def test_oracle_columns_equal_exact_matrix_elements(name):
    spec, packed, cols, ref = galerkin_case(name)
    assert len(cols) > 0
    out = O.OracleProblem(spec).hpsi(unit_block(len(packed), cols))
    assert rel(out, ref) <= TOL


def test_oracle_harmonic_smolyak_operator_is_diagonal():
    spec = harmonic_sg4(4, 4)
    packed = E.Problem(spec, device=-1).tables()["packed"] - 1
    H = O.OracleProblem(spec).dense()
    e = (packed + 0.5) @ spec.extra["omega"]
    assert np.abs(H - np.diag(e)).max() <= 1e-15


@pytest.mark.parametrize("spec_fn", [lambda: S.config_dp3(nb=8, nq=10), lambda: sg4_deep(3, 3)],
                         ids=["dp3", "sg4"])
def test_oracle_type10_equals_type1_for_constant_g0(spec_fn):
    base = spec_fn()
    a, b = const_g0(base, 10), const_g0(base, 1)
    packed = E.Problem(a, device=-1).tables()["packed"] - 1
    cols = np.nonzero(inside(a, packed, 2))[0]
    psi = unit_block(len(packed), cols)
    ha, hb = O.OracleProblem(a).hpsi(psi), O.OracleProblem(b).hpsi(psi)
    assert rel(ha, hb) <= TOL


# ---------------------------------------------------------------- GPU (through the C ABI)
@pytest.mark.gpu
@pytest.mark.parametrize("path", [1, 2, 0], ids=["auto", "slab", "general"])
@pytest.mark.parametrize("name", list(GALERKIN_CASES))
def test_gpu_columns_equal_exact_matrix_elements(name, path):
    spec, packed, cols, ref = galerkin_case(name)
    pg = E.Problem(spec, device=0)
    pg.set_kernel_path(path)
    psi = unit_block(pg.N, cols)
    assert rel(pg.hpsi(psi, prec="fp64"), ref) <= TOL
    # random combinations of the same columns (a block of 64 vectors)
    w = np.random.default_rng(1).standard_normal((len(cols), 64))
    assert rel(pg.hpsi(psi @ w, prec="fp64"), ref @ w) <= TOL
    assert rel(pg.hpsi(psi @ w, prec="fp32"), ref @ w) <= 2e-5


@pytest.mark.gpu
def test_gpu_sg4_l4_type10_columns_through_the_slab_kernel():
    # a larger Smolyak case whose big terms run in the slab-streaming kernel
    spec = sg4_deep(4, 4, seed=6)
    packed = E.Problem(spec, device=-1).tables()["packed"] - 1
    cols = np.nonzero(inside(spec, packed, 3))[0]
    ref = exact_columns(spec, packed, cols, 20)
    pg = E.Problem(spec, device=0)
    assert rel(pg.hpsi(unit_block(pg.N, cols), prec="fp64"), ref) <= TOL


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_gpu_harmonic_levels_are_the_harmonic_energies(prec):
    spec = harmonic_sg4(6, 5)
    pg = E.Problem(spec, device=0)
    packed = pg.tables()["packed"] - 1
    exact = np.sort((packed + 0.5) @ spec.extra["omega"])[:30]
    eig, _, st = pg.davidson(30, block=16, conv_resi=1e-9, conv_ene=1e-13, prec=prec)
    assert st["converged"], st
    assert np.abs(eig - exact).max() <= LEVEL_TOL


@pytest.mark.gpu
@pytest.mark.parametrize("spec_fn", [lambda: S.config_dp3(nb=10, nq=13), lambda: sg4_deep(4, 3, seed=7)],
                         ids=["dp3", "sg4"])
def test_gpu_type10_equals_type1_for_constant_g0(spec_fn):
    base = spec_fn()
    a, b = const_g0(base, 10), const_g0(base, 1)
    pa, pb = E.Problem(a, device=0), E.Problem(b, device=0)
    packed = pa.tables()["packed"] - 1
    cols = np.nonzero(inside(a, packed, 2))[0]
    psi = unit_block(pa.N, cols)
    assert rel(pa.hpsi(psi), pb.hpsi(psi)) <= TOL
