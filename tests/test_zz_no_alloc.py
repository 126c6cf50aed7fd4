"""evr_hpsi_noalloc: the H.psi entry point for callers that cannot let the library allocate
device memory (a host that owns all device buffers through its own pool, or code that must
stay out of the CUDA allocator).  Its output must equal evr_hpsi_device's on the same
inputs, call after call, although every call reuses the same fixed scratch array.

This file is collected last on purpose, so that a failure here comes after every other test.
"""
import numpy as np
import pytest

from evrgpu import spec as S
from evrgpu import lib as E

pytestmark = pytest.mark.gpu

TOL = 1e-12  # relative, max norm (the FP64 tolerance of the other H.psi tests)


def _rel(a, b):
    return float((a - b).abs().max() / b.abs().max())


def test_noalloc_matches_device_entry_point_twice():
    torch = pytest.importorskip("torch")
    p = E.Problem(S.config_sg4(4, 5, seed=5), device=0)
    nvec, ld = 6, 8
    g = torch.Generator(device="cuda").manual_seed(7)
    x = torch.randn((p.N, ld), dtype=torch.float64, device="cuda", generator=g)
    ref = torch.zeros_like(x)
    out1 = torch.full_like(x, 3.0)
    out2 = torch.full_like(x, -5.0)
    stream = torch.cuda.Stream()
    torch.cuda.synchronize()
    p.hpsi_device(x.data_ptr(), ld, ref.data_ptr(), ld, nvec, layout=E.LAYOUT_INTERLEAVED, stream=stream.cuda_stream)
    p.hpsi_noalloc(x.data_ptr(), ld, out1.data_ptr(), ld, nvec, stream=stream.cuda_stream)
    p.hpsi_noalloc(x.data_ptr(), ld, out2.data_ptr(), ld, nvec, stream=stream.cuda_stream)
    stream.synchronize()
    assert _rel(out1[:, :nvec], ref[:, :nvec]) <= TOL
    assert _rel(out2[:, :nvec], ref[:, :nvec]) <= TOL
    assert torch.all(out1[:, nvec:] == 3.0) and torch.all(out2[:, nvec:] == -5.0)


def test_noalloc_rejects_problems_beyond_the_static_scratch():
    torch = pytest.importorskip("torch")
    p = E.Problem(S.config_dp3(), device=0)  # 24^3-point grid: per-CTA buffers exceed 32 MiB in total
    x = torch.ones((p.N, 1), dtype=torch.float64, device="cuda")
    y = torch.zeros_like(x)
    with pytest.raises(E.EvrError) as ei:
        p.hpsi_noalloc(x.data_ptr(), 1, y.data_ptr(), 1, 1)
    assert ei.value.code == E.EVR_EINVAL and "scratch" in str(ei.value)
    torch.cuda.synchronize()
