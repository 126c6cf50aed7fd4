"""The tensor-core mode contraction (tcgen05, three TF32 products of split operands, FP32
accumulation in tensor memory) against the same contraction in float64 on the host.

Tolerance: 2e-6 relative to the largest output (the split keeps about 21 bits of each
product; the FP32 H.psi path's own tolerance against the oracle is 2e-5)."""
import numpy as np
import pytest

from evrgpu import lib as E

pytestmark = pytest.mark.gpu

TOL = 2e-6

SHAPES = [  # A, K, M, B, Vt
    (1, 17, 19, 37, 4),
    (19, 17, 19, 5, 4),
    (7, 3, 3, 11, 2),
    (5, 24, 24, 3, 1),
    (3, 9, 32, 50, 1),
    (11, 13, 7, 1, 8),
    (1, 1, 1, 300, 1),
]


def reference(inp, mat, M, alpha, out0):
    # out[b, m, a, v] = alpha * sum_k mat[k, m] * in[b, k, a, v]
    r = alpha * np.einsum("km,bkav->bmav", mat[:, :M].astype(np.float64), inp.astype(np.float64))
    return r if out0 is None else r + out0.astype(np.float64)


@pytest.mark.parametrize("threads", [512, 256, 128])
@pytest.mark.parametrize("shape", SHAPES, ids=lambda s: "x".join(map(str, s)))
def test_tc_contraction_matches_host(shape, threads):
    A, K, M, B, Vt = shape
    rng = np.random.default_rng(sum(shape))
    inp = rng.standard_normal((B, K, A, Vt)).astype(np.float32)
    ldm = (M + 3) // 4 * 4
    mat = rng.standard_normal((K, ldm)).astype(np.float32)
    out = E.tc_selftest(inp, mat, A, K, M, B, Vt, alpha=-0.5, threads=threads)
    ref = reference(inp, mat, M, -0.5, None)
    assert np.abs(out - ref).max() <= TOL * np.abs(ref).max()
    # accumulation onto an existing output
    out0 = rng.standard_normal((B, M, A, Vt)).astype(np.float32)
    out2 = E.tc_selftest(inp, mat, A, K, M, B, Vt, alpha=1.5, out=out0, threads=threads)
    ref2 = reference(inp, mat, M, 1.5, out0)
    assert np.abs(out2 - ref2).max() <= TOL * np.abs(ref2).max()


def test_tc_rejects_sizes_beyond_the_tile():
    x = np.zeros((1, 25, 1, 1), dtype=np.float32)
    with pytest.raises(E.EvrError) as ei:
        E.tc_selftest(x, np.zeros((25, 4), dtype=np.float32), 1, 25, 4, 1, 1)
    assert ei.value.code == E.EVR_EINVAL


def test_fp32_hpsi_tensor_cores_on_and_off_match_oracle():
    # D=6 L=6 on 32 vectors (every slab-kernel mode in FP32): the tensor-core contractions
    # (default, and with every contraction routed to them) and the CUDA-core ones against
    # the oracle at the FP32 tolerance of the H.psi tests
    from evrgpu import spec as S
    from oracle import oracle as O

    spec = S.config_sg4(6, 6, seed=1)
    pg = E.Problem(spec, device=0)
    rng = np.random.default_rng(13)
    psi = rng.standard_normal((pg.N, 32))
    ref = O.OracleProblem(spec).hpsi(psi)
    outs = {}
    for name, on, km in (("tc", True, 64), ("tc_all", True, 0), ("cuda_cores", False, 64)):
        pg.set_tensor_cores(on, km)
        outs[name] = pg.hpsi(psi, prec="fp32")
        assert np.abs(outs[name] - ref).max() <= 2e-5 * np.abs(ref).max(), name
    pg.set_tensor_cores(True, 64)


def test_fp32_autotune_keeps_results():
    # the autotuner also chooses between CUDA-core and tensor-core contractions in FP32;
    # whatever it keeps computes the same operator
    from evrgpu import spec as S
    from oracle import oracle as O

    spec = S.config_sg4(5, 5, seed=3)
    pg = E.Problem(spec, device=0)
    cs, ci, thr, km, ms = pg.autotune(nvec=16, prec="fp32")
    assert km == -1 or km in (64, 160, 288)
    assert ms > 0
    psi = np.random.default_rng(8).standard_normal((pg.N, 16))
    ref = O.OracleProblem(spec).hpsi(psi)
    assert np.abs(pg.hpsi(psi, prec="fp32") - ref).max() <= 2e-5 * np.abs(ref).max()
