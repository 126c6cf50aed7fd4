"""The host side of bench.py's propagation workload on CPU: a stand-in problem with the
library's call surface (hpsi, chebyshev, set_tensor_cores) checks the record the workload
writes into the bench line: the FP64 form on all 2000 steps, the FP32 legs on the shorter
count with their extrapolation, and the autocorrelation comparison over the common
steps."""
import argparse

import numpy as np


class _StandIn:
    """H = 0.1 (a multiple of the identity): e^{-iH t} keeps the norm and the energy."""

    N, nterm = 40, 3

    def __init__(self, spec, device=0):
        self.calls = []

    def hpsi(self, v, prec="fp64"):
        return 0.1 * np.asarray(v)

    def set_tensor_cores(self, on, min_km=64):
        pass

    def chebyshev(self, psi0, dt, nsteps, emin, emax, poly_tol=1e-10, prec="fp64", want_psi=False):
        self.calls.append((nsteps, prec))
        t = dt * np.arange(nsteps + 1)
        a = np.exp(-0.1j * t)[:, None]
        x = (np.asarray(psi0) * np.exp(-0.1j * t[-1]))[:, None]
        return a, x, {"max_order": 11}


def test_prop12d_record(monkeypatch):
    import bench
    import evrgpu.lib as L
    import evrgpu.spec as S

    made = []

    def problem(spec, device=0):
        made.append(_StandIn(spec, device))
        return made[-1]

    monkeypatch.setattr(L, "Problem", problem)
    monkeypatch.setattr(S, "config_sg4_12d_l6", lambda: None)
    monkeypatch.setattr(S, "displaced_gaussian", lambda sp, p, modes, d: np.ones(p.N, complex) / np.sqrt(p.N))
    out = bench.bench_prop12d(argparse.Namespace(prop_steps=200, autotune=False))
    assert out["fp64"]["steps"] == 2000 and "s_2000_steps_extrapolated" not in out["fp64"]
    for key in ("fp32", "fp32_tensor_cores"):
        assert out[key]["steps"] == 200
        assert out[key]["s_2000_steps_extrapolated"] == 10 * out[key]["s"]
        assert abs(out[key]["norm_final_minus_1"]) < 1e-12 and abs(out[key]["energy_drift_au"]) < 1e-12
    assert out["autocorr_max_abs_diff_fp32_vs_fp64"] < 1e-12
    assert (2000, "fp64") in made[0].calls and (200, "fp32") in made[0].calls
