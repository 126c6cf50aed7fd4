"""Host-side tables of the product library against the oracle (no GPU needed)."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from evrgpu import spec as S
from evrgpu import lib as E
from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_library_exports_every_declared_symbol():
    L = E.load()
    with open(os.path.join(ROOT, "include", "evr_gpu.h")) as f:
        hdr = f.read()
    declared = set(re.findall(r"^\s*(?:int|const char \*)\s*(evr_\w+)\s*\(", hdr, flags=re.M))
    assert declared, "no declarations parsed"
    for name in sorted(declared):
        assert hasattr(L, name), name
    assert set(E.EXPORTS) <= declared


@pytest.mark.parametrize("mk", [lambda: S.henon_heiles(6, 3), lambda: S.pyrazine_12d(1),
                                lambda: S.config_dp3(), lambda: S.config_sg4(4, 5, seed=5),
                                lambda: S.config_sg4(3, 4, seed=7, nq_A=1), lambda: S.henon_heiles(21, 2)])
def test_tables_match_oracle(mk):
    spec = mk()
    pg = E.Problem(spec, device=-1)
    po = O.OracleProblem(spec)
    assert (pg.Np, pg.nterm, pg.sum_nb, pg.sum_nq) == (po.Np, po.nterm, po.sum_nb, po.sum_nq)
    tg, to = pg.tables(), po.tables()
    for k in ("term_l", "weight", "map", "packed"):
        assert np.array_equal(tg[k], to[k]), k
    levels = range(spec.LG + 1) if spec.kind == "sg4" else [0]
    for d in range(spec.D):
        for l in levels:
            bg, bo = pg.basis(d, l), po.basis(d, l)
            assert (bg["nb"], bg["nq"]) == (bo["nb"], bo["nq"])
            for k in ("x", "w", "d0b", "d1b", "d2b", "bgw", "d1gg", "d2gg"):
                scale = max(1.0, np.abs(bo[k]).max())
                assert np.abs(bg[k] - bo[k]).max() <= 1e-11 * scale, (d, l, k)


def test_sg4_6d_l8_sizes_and_flops():
    pg = E.Problem(S.config_sg4_6d_l8(), device=-1)
    assert (pg.nterm, pg.Np, pg.sum_nb, pg.sum_nq) == (2975, 40081, 860455, 37769167)
    assert 5e9 < pg.flop_per_hpsi < 2e10


def test_bad_descriptions_are_rejected():
    spec = S.henon_heiles(3, 2)
    spec.LB = 5  # LB > LG
    with pytest.raises(E.EvrError) as ei:
        E.Problem(spec, device=-1)
    assert ei.value.code == E.EVR_EINVAL
    spec = S.henon_heiles(3, 2)
    spec.mono_idx = spec.mono_idx.copy()
    spec.mono_idx[0, 0] = 7  # mode out of range
    with pytest.raises(E.EvrError):
        E.Problem(spec, device=-1)


def test_device_calls_fail_loudly_on_host_only_context():
    pg = E.Problem(S.henon_heiles(3, 2), device=-1)
    with pytest.raises(E.EvrError) as ei:
        pg.hpsi(np.ones(pg.N))
    assert ei.value.code == E.EVR_EDEVICE


def test_set_vgrid_argument_checks():
    pg = E.Problem(S.henon_heiles(3, 2), device=-1)
    v = np.zeros(pg.sum_nq)
    with pytest.raises(E.EvrError) as ei:  # the table lives on the device
        pg.set_vgrid(v)
    assert ei.value.code == E.EVR_EDEVICE
    L = E.load()
    assert L.evr_set_vgrid(pg.h, v.ctypes.data_as(E._dp), 7) == E.EVR_EINVAL
    assert L.evr_set_vgrid(pg.h, None, 0) == E.EVR_EINVAL
    with pytest.raises(E.EvrError) as ei:
        pg.set_vgrid(v[:-1])
    assert ei.value.code == E.EVR_EINVAL
    with pytest.raises(E.EvrError) as ei:
        pg.set_dipole_grid(v)
    assert ei.value.code == E.EVR_EDEVICE
    assert L.evr_set_dipole_grid(pg.h, v.ctypes.data_as(E._dp), -1) == E.EVR_EINVAL
    # non-finite grid values are rejected before any upload, naming the value
    for bad in (np.nan, np.inf):
        vb = v.copy()
        vb[7] = bad
        for setter in (pg.set_vgrid, pg.set_dipole_grid):
            with pytest.raises(E.EvrError) as ei:
                setter(vb)
            assert ei.value.code == E.EVR_EINVAL and "value 7" in str(ei.value)


def test_sil_needs_a_device():
    pg = E.Problem(S.henon_heiles(3, 2), device=-1)
    with pytest.raises(E.EvrError) as ei:
        pg.sil(np.ones(pg.N, dtype=complex), 1.0, 1)
    assert ei.value.code == E.EVR_EDEVICE


def test_pyrazine_builders_agree():
    """pyrazine_12d is the general vibronic builder on the 12-D parameters: same monomials,
    KEO and bases (the 24-D oracle pin builds its model with the same function)."""
    a = S.pyrazine_12d(1)
    b = S.pyrazine_vibronic(S.PYRAZINE_W, S.PYRAZINE_K1, S.PYRAZINE_K2, 0.46165, 0.1825, [3, 3, 2, 2] + [2] * 8, 1)
    for k in ("D", "nb0", "LG", "LB", "Aq", "Bq", "Ab", "Bb", "mono_coef", "mono_idx", "mono_elec", "keo_type",
              "G0", "g"):
        assert np.array_equal(np.asarray(getattr(a, k)), np.asarray(getattr(b, k))), k


def test_set_ggrid_argument_checks():
    pt = E.Problem(S.config_sg4(3, 2, seed=1), device=-1)  # type 10
    with pytest.raises(E.EvrError) as ei:
        pt.set_ggrid(np.zeros((pt.sum_nq, 3, 3)))
    assert ei.value.code == E.EVR_EDEVICE
    p1 = E.Problem(S.henon_heiles(3, 2), device=-1)  # type 1: no G table to set
    with pytest.raises(E.EvrError) as ei:
        p1.set_ggrid(np.zeros((p1.sum_nq, 3, 3)))
    assert ei.value.code == E.EVR_EINVAL
    # G(Q) must be symmetric: one asymmetric point is named in the error, before any upload
    G = np.tile(np.eye(3), (pt.sum_nq, 1, 1))
    G[5, 0, 2] += 1e-6
    with pytest.raises(E.EvrError) as ei:
        pt.set_ggrid(G)
    assert ei.value.code == E.EVR_EINVAL and "grid point 5" in str(ei.value)
    G = np.tile(np.eye(3), (pt.sum_nq, 1, 1))
    G[3, 1, 1] = np.nan  # a diagonal NaN passes the symmetry test; the finiteness test catches it
    with pytest.raises(E.EvrError) as ei:
        pt.set_ggrid(G)
    assert ei.value.code == E.EVR_EINVAL and "not finite" in str(ei.value)


def test_set_jacobian_argument_checks():
    pt = E.Problem(S.config_sg4(3, 2, seed=1), device=-1)  # type 10
    one = np.ones(pt.sum_nq)
    bad = one.copy()
    bad[3] = -1.0
    with pytest.raises(E.EvrError) as ei:
        pt.set_jacobian(one, bad)
    assert ei.value.code == E.EVR_EINVAL and "grid point 3" in str(ei.value)
    with pytest.raises(E.EvrError) as ei:
        pt.set_jacobian(one, one)
    assert ei.value.code == E.EVR_EDEVICE  # valid values, but a host-only context
    p1 = E.Problem(S.henon_heiles(3, 2), device=-1)  # type 1: no Jacobian factors
    with pytest.raises(E.EvrError) as ei:
        p1.set_jacobian(np.ones(p1.sum_nq), np.ones(p1.sum_nq))
    assert ei.value.code == E.EVR_EINVAL


def grid_points(pg, spec):
    """Coordinates Q (sum_nq x D) of every grid point in the reference's order: terms in
    order, first mode fastest inside a term, at the scaled nodes of each (mode, level)."""
    term_l = pg.tables()["term_l"]
    out = []
    for t in range(pg.nterm):
        xs = [pg.basis(d, int(term_l[t, d]))["x"] for d in range(spec.D)]
        idx = np.indices([len(x) for x in xs]).reshape(spec.D, -1, order="F")
        out.append(np.stack([xs[d][idx[d]] for d in range(spec.D)], axis=1))
    return np.concatenate(out)


def test_grid_points_reproduce_the_oracle_potential_grid():
    """The coordinates the G-table GPU test evaluates G(Q) at are the grid's: the potential's
    monomials at them give the oracle's V grid."""
    for spec in (S.config_sg4(4, 5, seed=5), S.config_dp3(nb=6, nq=8)):
        pg = E.Problem(spec, device=-1)
        Q = grid_points(pg, spec)
        v = np.zeros(len(Q))
        for c, ix in zip(spec.mono_coef, np.asarray(spec.mono_idx).reshape(-1, 4)):
            term = np.full(len(Q), c)
            for i in ix:
                if i >= 0:
                    term = term * Q[:, i]
            v += term
        ref = O.OracleProblem(spec).vgrid()
        assert np.abs(v - ref).max() <= 1e-13 * np.abs(ref).max()
