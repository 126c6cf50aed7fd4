"""Batched problems (evr_create_batch): stacked tables on the host (CPU), stacked H.psi and
the lock-step batched Davidson against one context per problem (GPU)."""
import numpy as np
import pytest

from evrgpu import spec as S
from evrgpu import lib as E

SMALL = [(3, 4, 11), (4, 4, 12), (3, 6, 13), (5, 4, 14), (4, 5, 15), (6, 4, 16)]


def specs():
    return [S.config_sg4(D, L, seed=sd) for (D, L, sd) in SMALL]


def test_batch_tables_on_host():
    sp = specs()
    b = E.BatchProblem(sp, device=-1)
    singles = [E.Problem(x, device=-1) for x in sp]
    assert b.N == sum(p.N for p in singles)
    assert b.nterm == sum(p.nterm for p in singles)
    assert b.sum_nq == sum(p.sum_nq for p in singles)
    assert list(b.offsets) == list(np.concatenate([[0], np.cumsum([p.N for p in singles])]))
    assert abs(b.flop_per_hpsi - sum(p.flop_per_hpsi for p in singles)) <= 1e-9 * b.flop_per_hpsi


def test_batch_merged_tables_match_single_problems():
    # the stacked map and weights (host tables built on several threads) equal the single
    # problems' tables with the packed indices shifted by each problem's row offset
    sp = specs()
    for _ in range(2):
        b = E.BatchProblem(sp, device=-1)
        tb = b.tables()
        singles = [E.Problem(x, device=-1) for x in sp]
        ts = [p.tables() for p in singles]
        w = np.concatenate([t["weight"] for t in ts])
        m = np.concatenate([np.where(t["map"] >= 0, t["map"] + off, -1) for t, off in zip(ts, b.offsets[:-1])])
        assert np.array_equal(tb["weight"], w)
        assert np.array_equal(tb["map"], m)


def test_batch_reports_the_first_invalid_problem():
    import dataclasses
    sp = specs()
    bad = dataclasses.replace(sp[2], scaleQ=-np.abs(np.asarray(sp[2].scaleQ)))  # scaleQ must be > 0
    sp[2] = bad
    sp[4] = dataclasses.replace(sp[4], scaleQ=-np.abs(np.asarray(sp[4].scaleQ)))
    with pytest.raises(E.EvrError) as ei:
        E.BatchProblem(sp, device=-1)
    assert ei.value.code == E.EVR_EINVAL
    assert "problem 2:" in str(ei.value)


def test_batch_rejects_mixed_state_counts():
    sp = specs()[:2] + [S.pyrazine_12d(1)]
    with pytest.raises(E.EvrError) as ei:
        E.BatchProblem(sp, device=-1)
    assert ei.value.code == E.EVR_EINVAL


def rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.mark.gpu
@pytest.mark.parametrize("path", [1, 0], ids=["auto", "general"])
def test_batch_hpsi_equals_single_problems(path):
    sp = specs()
    b = E.BatchProblem(sp, device=0)
    b.set_kernel_path(path)
    rng = np.random.default_rng(4)
    x = rng.standard_normal((b.N, 5))
    y64 = b.hpsi(x)
    y32 = b.hpsi(x, prec="fp32")
    for q, s1 in enumerate(sp):
        p = E.Problem(s1, device=0)
        lo, hi = b.offsets[q], b.offsets[q + 1]
        ref = p.hpsi(x[lo:hi])
        assert rel(y64[lo:hi], ref) <= 1e-12
        assert rel(y32[lo:hi], ref) <= 2e-5


@pytest.mark.gpu
def test_batch_davidson_equals_single_problems():
    sp = specs()
    b = E.BatchProblem(sp, device=0)
    nlev = 6
    e64, st = b.davidson(nlev, block=8, conv_resi=1e-8, conv_ene=1e-11)
    assert st["converged"]
    for q, s1 in enumerate(sp):
        p = E.Problem(s1, device=0)
        e1, _, _ = p.davidson(nlev, block=8, conv_resi=1e-8, conv_ene=1e-11)
        assert np.abs(e64[q] - e1).max() <= 1e-9
    e32, st32 = b.davidson(nlev, block=8, conv_resi=1e-8, conv_ene=1e-11, prec="fp32")
    assert st32["converged"]
    assert st32["hpsi_fp32"] > 0
    # mixed form: within 1e-4 cm-1 of the FP64 levels
    assert np.abs(e32 - e64).max() * S.AU_TO_CM <= 1e-4


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_batch_davidson_matches_oracle_dense_spectra(prec):
    # every problem of a batch against the oracle's dense spectrum of the same operator (its
    # symmetric part, the operator the Davidson uses when nq > nb), 1e-9 au, in FP64 and in
    # the mixed form (per-problem FP32 phase, FP64 continuation)
    from oracle import oracle as O

    sp = specs()[:4]
    b = E.BatchProblem(sp, device=0)
    nlev = 6
    e, st = b.davidson(nlev, block=8, conv_resi=1e-8, conv_ene=1e-11, prec=prec)
    assert st["converged"], st
    if prec == "fp32":
        assert st["hpsi_fp32"] > 0 and st["hpsi_fp64"] > 0
    for q, s1 in enumerate(sp):
        H = O.OracleProblem(s1).dense()
        ref = np.linalg.eigvalsh(0.5 * (H + H.T))[:nlev]
        assert np.abs(e[q] - ref).max() <= 1e-9, q
