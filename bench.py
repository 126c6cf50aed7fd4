#!/usr/bin/env python
"""H.psi throughput of the Smolyak SG4 D=6 L=8 workload on one GB300.

One step = one H.psi block: H applied to 64 FP64 vectors of the D=6, L=8 Smolyak basis
(nb(l)=2l+1, nq(l)=2l+3, 2975 terms, 40,081 packed functions, 37.8 M grid points),
type-10 KEO with G(Q) = 1 + g.q and a cubic+quartic potential, all drawn from a fixed
seed (synthetic inputs with the benchmark's shapes and distributions).

  value  : FP64 H.psi/s with the vectors resident in HBM (device entry point)
  e2e    : FP64 H.psi/s through the host entry point evr_hpsi_host with pinned host
           buffers (copies in and out inside the timed region)
  mixed  : the FP32-contraction path on the same block, with its error against FP64
  roofline: the term-pipeline kernels (slab + general) against the FP64 FMA rate of this
           GPU measured in this run (evr_fma_peak: independent FMA chains; the FP64 work of
           the contractions runs on the CUDA-core FMA pipe)
  davidson: time to converge the lowest 50 levels (residual 1e-7 au) in FP64 and in the
           mixed form (FP32 contractions, FP64 residuals / Gram-Schmidt / Rayleigh-Ritz,
           FP64 refinement), with the largest eigenvalue difference in cm-1
  cpu_baseline / --impl reference: the CPU oracle (C++/OpenMP restatement of the
           reference's OpPsi) on the host cores, bounded to a sample of the block.
  configs: the other workloads, one compact result each (wall clock around the library
           call, device-resident data):
           dp3_davidson  D=3 direct product nb=20 nq=24, lowest 20 levels to 1e-6 cm-1, FP64
                         and mixed, against a dense diagonalisation of the same operator;
           batch         256 uneven Smolyak problems (D 3..6, L 4..8), lowest 10 levels each,
                         lock-step batched Davidson, FP64 and mixed;
           prop12d       D=12 Smolyak L=6 Chebyshev propagation (dt = 10 au) timed on 200
                         steps in complex128 and complex64-contraction form (CUDA cores
                         and tcgen05 tensor cores); the 2000-step
                         time of the workload is extrapolated from them (labelled so); the
                         FP32 - FP64 autocorrelation difference and an FP64 norm / energy
                         check of the final packets;
           control       optimal-control gradient D=3 nb=20 nq=24, 4000 steps of 5 au:
                         forward and backward times, and the adjoint gradient against a
                         central difference (h = 1e-7) at one step.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference] [--no-configs]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for p in (ROOT, os.path.join(ROOT, "elvibrot-tnumtana_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)

import numpy as np  # noqa: E402

METRIC = "H.psi/s (OpPsi on SG4 D=6 L=8, 64-vector block)"
UNIT = "Hpsi/s"
NVEC = 64


def workload_config(n, terms, grid_points):
    """The workload's description, printed alike by both arms (the GPU library's problem and
    the oracle's give the same sizes)."""
    return {"workload": "OpPsi block: SG4 D=6 L=8, nb(l)=2l+1, nq(l)=2l+3, type-10 KEO, 64 vectors",
            "nvec": NVEC, "seed": 1, "l2": "flushed between timed steps (512 MB write)",
            "N": int(n), "terms": int(terms), "grid_points": int(grid_points)}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.out = ""

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        rows = [r.split(",") for r in self.out.strip().splitlines() if r.count(",") >= 8]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for r in rows for n, v in zip(names, r[5:9]) if "Active" in v and "Not" not in v})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": reasons, "samples": len(rows)}


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(x: float, device) -> float:
    """The largest x over the ranks of the default process group (x itself on one rank)."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def hbm_roofline(traffic_bytes: float, kernel_s: float, peaks_path: str = None) -> dict:
    """The DRAM side of the dominant kernel: its measured bytes per launch over its
    event-timed duration, against the measured copy bandwidth of the GB300s (the
    fallback figure when the peaks file is absent).  It shows how far HBM is from bounding
    the kernel."""
    peaks_path = peaks_path or os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(peaks_path) as f:
            peak, src = float(json.load(f)["hbm_gbs"]), "measured (hbm_gbs)"
    except (OSError, KeyError, TypeError, ValueError):
        peak, src = 6800.0, "fallback"
    achieved = traffic_bytes / kernel_s / 1e9
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": traffic_bytes, "peak_source": src}


def job_rate(units_per_rank: float, seconds_max: float, world: int) -> float:
    """Whole-job throughput: the units of every rank over the slowest rank's time."""
    return world * units_per_rank / seconds_max


def cpu_oracle_rate(spec, nvec_sample, threads):
    """Oracle H.psi/s on the host cores for a bounded sample of the block."""
    from oracle import oracle as O

    op = O.OracleProblem(spec)
    rng = np.random.default_rng(0)
    psi = rng.standard_normal((op.N, nvec_sample))
    op.hpsi(psi[:, :1], nthreads=threads)  # grid set-up outside the timing
    t0 = time.perf_counter()
    op.hpsi(psi, nthreads=threads)
    dt = time.perf_counter() - t0
    return nvec_sample / dt, dt


def run_reference(args):
    rank, world, _ = dist_info()
    if rank != 0:
        return 0
    from evrgpu import spec as S

    from oracle import oracle as O

    spec = S.config_sg4_6d_l8()
    threads = os.cpu_count() or 1
    op = O.OracleProblem(spec)
    cfg = workload_config(op.N, op.nterm, op.sum_nq)
    del op
    rates = []
    for i in range(args.warmup + args.steps):
        r, _ = cpu_oracle_rate(spec, 1, threads)
        if i >= args.warmup:
            rates.append(r)
    v = statistics.median(rates)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 / v, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
            "config": cfg,
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": "1 vector of the 64-vector block per step (the reference's Fortran "
                                       "cannot be built here: no Fortran compiler)"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def run_profile(args):
    """A handful of H.psi launches (FP64 then FP32) for ncu captures: D=6 Smolyak level 6
    (small case) or level 8 (the benchmark workload) on 64 vectors, the D=3 direct
    product (stage kernels) on 16 vectors, or the D=12 level-6 propagation workload on the
    two vectors of one complex packet."""
    import torch
    from evrgpu import Problem, spec as S
    import evrgpu.lib as E

    nvec = NVEC
    if args.profile == "dp3":  # direct product D=3 nb=20 nq=24: the stage kernels, 16 vectors
        spec, nvec = S.config_dp3(), 16
    elif args.profile == "sg4_12d_l6":  # the propagation workload: one complex packet, 2 vectors
        spec, nvec = S.config_sg4_12d_l6(), 2
    else:
        spec = S.config_sg4(6, 6, seed=1) if args.profile == "sg4_6d_l6" else S.config_sg4_6d_l8()
    p = Problem(spec, device=0)
    if args.tc:
        p.set_tensor_cores(True, 64)
    x = torch.randn((p.N, nvec), dtype=torch.float64, device="cuda")
    y = torch.empty_like(x)
    st = torch.cuda.Stream()
    torch.cuda.set_stream(st)
    out, launches = {}, {}
    for prec in (("fp64", "fp32") if args.prec == "both" else (args.prec,)):
        for _ in range(args.steps):
            p.hpsi_device(x.data_ptr(), nvec, y.data_ptr(), nvec, nvec, layout=E.LAYOUT_INTERLEAVED, prec=prec,
                          stream=st.cuda_stream)
        torch.cuda.synchronize()
        out[prec] = p.last_kernel_ms()[0]
        launches[prec] = p.last_launch_count()
    print(json.dumps({"profile": args.profile, "N": p.N, "terms": p.nterm, "gflop_per_hpsi": p.flop_per_hpsi / 1e9,
                      "items_ms": out, "kernels_items": launches}))
    return 0


# DRAM bytes (read + write) of one FP64 64-vector launch of the term kernels: a one-pass ncu
# capture of the D=6 L=6 launch (`--profile sg4_6d_l6 --prec fp64`, metrics
# dram__bytes_read.sum and dram__bytes_write.sum of both term kernels: slab kernel 1.338 GB
# read + 0.571 GB written, general kernel 0.009 GB + 0.033 GB; the reads are dominated by
# the per-point G table and V, the writes are staged tensors leaving L2) scaled to the L=8
# grid by the grid points (37.77 M / 6.49 M)
TRAFFIC_PER_LAUNCH = (1338332416 + 571358464 + 9097728 + 33347072) * 37.769167 / 6.487975
DAV_LEVELS, DAV_BLOCK, DAV_RESI = 50, 64, 1e-7


def davidson_legs(p, S):
    """Lowest 50 levels in FP64 and in the mixed form, timed end to end (host call)."""
    out = {"levels": DAV_LEVELS, "block": DAV_BLOCK, "conv_resi_au": DAV_RESI}
    res = {}
    for prec in ("fp64", "fp32"):
        t0 = time.perf_counter()
        e, _, st = p.davidson(DAV_LEVELS, block=DAV_BLOCK, max_it=400, conv_resi=DAV_RESI, conv_ene=1e-10,
                              prec=prec)
        res[prec] = (e, time.perf_counter() - t0, st)
    e64, t64, s64 = res["fp64"]
    e32, t32, s32 = res["fp32"]
    out.update({"fp64_s": t64, "mixed_s": t32, "speedup": t64 / t32,
                "max_abs_diff_cm": float(np.abs(e64 - e32).max() * S.AU_TO_CM),
                "fp64": {k: v for k, v in s64.items()}, "mixed": {k: v for k, v in s32.items()},
                "e0_cm": float(e64[0] * S.AU_TO_CM), "e49_cm": float(e64[-1] * S.AU_TO_CM)})
    return out


def bench_dp3(args):
    """D=3 direct product nb=20 nq=24 (type-10 KEO, G(Q) = 1 + g.q): lowest 20 levels with 16
    start vectors to the workload's 1e-6 cm-1 (energy change below 1e-6 cm-1 and residuals
    below 1e-8 au), FP64 and mixed, against a dense diagonalisation of the same operator
    ((H + H^T)/2, assembled from the library's H.psi on unit blocks, torch eigvalsh)."""
    import torch
    from evrgpu import spec as S
    from evrgpu.lib import Problem

    p = Problem(S.config_dp3(), device=0)
    tol_ene = 1e-6 / S.AU_TO_CM
    out = {"N": int(p.N), "levels": 20, "block": 16, "conv_ene_cm": 1e-6, "conv_resi_au": 1e-8}
    p.davidson(20, block=16, conv_resi=1e-8, conv_ene=tol_ene)  # warm-up (work decompositions)
    lev = {}
    for prec in ("fp64", "fp32"):
        t0 = time.perf_counter()
        e, _, st = p.davidson(20, block=16, conv_resi=1e-8, conv_ene=tol_ene, prec=prec)
        out[prec if prec == "fp64" else "mixed"] = {"s": time.perf_counter() - t0, **st}
        lev[prec] = e
    # dense operator from unit blocks (64 columns per call)
    N = p.N
    H = np.zeros((N, N))
    eye = np.eye(N)
    for c0 in range(0, N, 64):
        H[:, c0:c0 + 64] = p.hpsi(eye[:, c0:c0 + 64])
    Hs = torch.from_numpy(0.5 * (H + H.T)).cuda()
    dense = torch.linalg.eigvalsh(Hs)[:20].cpu().numpy()
    del Hs
    out["fp64"]["max_abs_err_vs_dense_cm"] = float(np.abs(lev["fp64"] - dense).max() * S.AU_TO_CM)
    out["mixed"]["max_abs_err_vs_dense_cm"] = float(np.abs(lev["fp32"] - dense).max() * S.AU_TO_CM)
    out["speedup_mixed"] = out["fp64"]["s"] / out["mixed"]["s"]
    out["levels_cm"] = [float(x * S.AU_TO_CM) for x in lev["fp64"][:3]]
    return out


def bench_batch(args):
    """256 uneven problems (D ~ U{3..6}, L ~ U{4..8}): lowest 10 levels of every problem to
    residual 1e-7 au, lock-step batched Davidson in FP64 and in the mixed form."""
    from evrgpu import spec as S
    from evrgpu.lib import BatchProblem

    t0 = time.perf_counter()
    b = BatchProblem(S.batched_systems(args.batch_n, seed=2), device=0)
    out = {"problems": args.batch_n, "N": int(b.N), "terms": int(b.nterm), "create_s": time.perf_counter() - t0}
    out["autotune"] = b.autotune(nvec=10, prec="fp32")
    res = {}
    out["conv_resi_au"] = args.batch_tol
    runs = [("fp64", "fp64", args.batch_tol), ("mixed", "fp32", args.batch_tol)]
    if args.batch_check:  # a tighter FP64 solve as the reference of both
        runs.append(("fp64_tight", "fp64", args.batch_tol * 1e-2))
    for name, prec, tol in runs:
        t0 = time.perf_counter()
        e, st = b.davidson(10, block=10, conv_resi=tol, conv_ene=tol * 1e-3, prec=prec, max_it=200)
        res[name] = e
        out[name] = {"s": time.perf_counter() - t0, **st}
    out["speedup_mixed"] = out["fp64"]["s"] / out["mixed"]["s"]
    d = np.abs(res["fp64"] - res["mixed"]) * S.AU_TO_CM
    out["max_abs_diff_cm"] = float(d.max())
    out["levels_above_1e-4_cm"] = int((d > 1e-4).sum())
    if args.batch_check:
        for name in ("fp64", "mixed"):
            out[name]["max_abs_diff_vs_tight_cm"] = float((np.abs(res[name] - res["fp64_tight"]) * S.AU_TO_CM).max())
    return out


def bench_prop12d(args):
    """D=12 Smolyak L=6 (nb = nq = 2l+1), Gaussian displaced by 1.0 in modes 1-3, Chebyshev
    dt = 10 au in complex128 and with FP32 contractions (complex64 arithmetic in the
    contractions, FP64 recurrence, autocorrelation and norm), the latter on the CUDA cores
    and on the tcgen05 tensor cores."""
    from evrgpu import spec as S
    from evrgpu.lib import Problem

    sp = S.config_sg4_12d_l6()
    p = Problem(sp, device=0)
    psi0 = S.displaced_gaussian(sp, p, [0, 1, 2], 1.0)
    # spectral bounds of the Smolyak operator by power iterations on H and on (shift - H):
    # the negative combination weights can put eigenvalues outside the harmonic estimate
    rng = np.random.default_rng(0)
    v = rng.standard_normal((p.N, 1))
    for _ in range(150):
        hv = p.hpsi(v)
        top = float(np.vdot(v, hv).real / np.vdot(v, v).real)
        v = hv / np.linalg.norm(hv)
    shift = 1.02 * abs(top)
    v = rng.standard_normal((p.N, 1))
    for _ in range(150):
        hv = shift * v - p.hpsi(v)
        low = shift - float(np.vdot(v, hv).real / np.vdot(v, v).real)
        v = hv / np.linalg.norm(hv)
    span = top - low
    emin, emax = low - 0.05 * span, top + 0.05 * span
    out = {"N": int(p.N), "terms": int(p.nterm), "dt_au": 10.0}
    for attempt in range(4):  # widen the bounds if the series meets a spectrum beyond them
        try:
            p.chebyshev(psi0, 10.0, 2, emin, emax)
            break
        except Exception:
            emin, emax = emin - 0.1 * (emax - emin), emax + 0.2 * (emax - emin)
    out.update({"emin": emin, "emax": emax})
    if args.autotune:
        out["autotune"] = p.autotune(nvec=2, prec="fp64")
    e0 = float(np.vdot(psi0, p.hpsi(psi0.real[:, None])[:, 0]).real)  # psi0 is real
    ac, fin = {}, {}
    # the plain FP64 form runs the workload's 2000 steps; the FP32 legs run prop_steps (their
    # norm drifts by about 7e-4 over 2000 steps, close to the 1e-3 guard of the FP32 form)
    full, steps32 = 2000, args.prop_steps
    for key, prec, tc, steps in (("fp64", "fp64", False, full), ("fp32", "fp32", False, steps32),
                                 ("fp32_tensor_cores", "fp32", True, steps32)):
        p.set_tensor_cores(tc, 64)
        p.chebyshev(psi0, 10.0, 2, emin, emax, prec=prec)
        t0 = time.perf_counter()
        a, psiT, st = p.chebyshev(psi0, 10.0, steps, emin, emax, prec=prec, want_psi=True)
        dt = time.perf_counter() - t0
        ac[key] = a[:, 0]
        # FP64 checks of the final packet: norm and energy <psi|H|psi> (FP64 H.psi)
        x = psiT[:, 0]
        hx = p.hpsi(np.stack([x.real, x.imag], axis=1))
        en = float((np.vdot(x.real, hx[:, 0]) + np.vdot(x.imag, hx[:, 1])).real / np.vdot(x, x).real)
        out[key] = {"steps": steps, "s": dt, "s_per_step": dt / steps, "order": st["max_order"],
                    "norm_final_minus_1": float(np.vdot(x, x).real - 1.0), "energy_drift_au": en - e0}
        if steps < full:
            out[key]["s_2000_steps_extrapolated"] = full * dt / steps
    p.set_tensor_cores(False)
    n32 = len(ac["fp32"])  # the FP32 legs against the first n32 values of the FP64 series
    out["autocorr_max_abs_diff_fp32_vs_fp64"] = float(np.abs(ac["fp32"] - ac["fp64"][:n32]).max())
    out["autocorr_max_abs_diff_fp32_tensor_cores_vs_fp64"] = float(
        np.abs(ac["fp32_tensor_cores"] - ac["fp64"][:n32]).max())
    out["autocorr_last"] = [float(ac["fp64"][-1].real), float(ac["fp64"][-1].imag)]
    out["note"] = (f"fp64 timed on all {full} steps; the FP32 legs on {steps32} of them, "
                   f"s_2000_steps_extrapolated = {full} x measured s per step")
    return out


def bench_control(args):
    """Optimal control on D=3 nb=20 nq=24 with the dipole: ground state -> level 5, 4000 steps
    of 5 au, dJ/dE by the adjoint, checked against a central difference at one step."""
    from evrgpu import spec as S
    from evrgpu.lib import Problem

    sp = S.config_oc(seed=0)
    p = Problem(sp, device=0)
    e, vec, _ = p.davidson(8, block=16, conv_resi=1e-9, conv_ene=1e-12, want_vectors=True, sym=0)
    rng = np.random.default_rng(0)
    v = rng.standard_normal((p.N, 1))
    for _ in range(200):
        hv = p.hpsi(v)
        lam = float(np.linalg.norm(hv))
        v = hv / lam
    psi0 = vec[:, 0] / np.linalg.norm(vec[:, 0]) + 0j
    tgt = vec[:, 5] / np.linalg.norm(vec[:, 5]) + 0j
    field = S.oc_field(4000, 5.0, seed=0)
    emin, emax = e[0] - 0.01, 1.05 * lam
    t0 = time.perf_counter()
    J, _, _, info = p.oc_forward(field, psi0, tgt, 5.0, emin, emax)
    tf = time.perf_counter() - t0
    t0 = time.perf_counter()
    g, ref, binfo = p.oc_backward(len(field))
    tb = time.perf_counter() - t0
    n, h = 2000, 1e-7
    fp, fm = field.copy(), field.copy()
    fp[n] += h
    fm[n] -= h
    fd = (p.oc_forward(fp, psi0, tgt, 5.0, emin, emax)[0] - p.oc_forward(fm, psi0, tgt, 5.0, emin, emax)[0]) / (2 * h)
    return {"steps": 4000, "J": J, "forward_s": tf, "backward_s": tb, "order": info["order"],
            "checkpoints": info["checkpoints"],
            "fd_step": n, "fd_h": h, "fd_rel_err": float(abs(fd - g[n]) / np.abs(g).max()),
            "ref_vs_grad": float(np.abs(0.5 * 5.0 * (ref[:-1] + ref[1:]) - g).max() / np.abs(g).max())}


CONFIGS = {"dp3": bench_dp3, "batch": bench_batch, "prop12d": bench_prop12d, "control": bench_control}


def run_suite(args):
    """The other workloads, one JSON line each."""
    which = list(CONFIGS) if args.suite == "all" else [args.suite]
    for w in which:
        print(json.dumps({"suite": w, **CONFIGS[w](args)}))
    return 0


def measure_dgemm_tflops(torch, dtype, n=4096, reps=5):
    a = torch.randn(n, n, dtype=dtype, device="cuda")
    b = torch.randn(n, n, dtype=dtype, device="cuda")
    torch.matmul(a, b)
    torch.cuda.synchronize()
    best = 1e30
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1) / 1e3)
    del a, b
    return 2.0 * n ** 3 / best / 1e12


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-davidson", action="store_true", help="skip the Davidson time-to-tolerance legs")
    ap.add_argument("--no-configs", action="store_true", help="skip the other workloads' compact results")
    ap.add_argument("--autotune", action="store_true", help="tune the work decomposition before timing")
    ap.add_argument("--profile", default=None, choices=["sg4_6d_l6", "sg4_6d_l8", "dp3", "sg4_12d_l6"],
                    help="profiling mode: a few H.psi launches of the named workload, nothing else")
    ap.add_argument("--prec", default="both", choices=["both", "fp64", "fp32"], help="precision(s) in profiling mode")
    ap.add_argument("--tc", action="store_true", help="profiling mode: FP32 contractions on the tensor cores")
    ap.add_argument("--suite", default=None, choices=["dp3", "batch", "prop12d", "control", "all"],
                    help="the other workloads (one JSON line each): direct-product Davidson, 256 batched "
                         "problems, D=12 Chebyshev propagation, optimal-control gradient")
    ap.add_argument("--batch-n", type=int, default=256, help="problems in the batch workload")
    ap.add_argument("--batch-tol", type=float, default=1e-7, help="residual tolerance of the batch Davidson (au)")
    ap.add_argument("--batch-check", action="store_true",
                    help="also solve the batch in FP64 at 1/100 of the tolerance and compare both against it")
    ap.add_argument("--prop-steps", type=int, default=200,
                    help="time steps timed in the FP32 legs of the propagation workload (FP64: all 2000)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        return run_reference(args)
    if args.profile:
        return run_profile(args)
    if args.suite:
        return run_suite(args)

    import torch

    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    from evrgpu import Problem, spec as S
    import evrgpu.lib as E

    spec = S.config_sg4_6d_l8()
    p = Problem(spec, device=local)
    N = p.N
    g = torch.Generator(device="cuda").manual_seed(1234 + rank)
    x = torch.randn((N, NVEC), dtype=torch.float64, device="cuda", generator=g)
    y = torch.empty_like(x)
    y32 = torch.empty_like(x)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    # a dedicated stream: the library launches on it and the CUDA events are recorded on it
    torch_stream = torch.cuda.Stream()
    torch.cuda.set_stream(torch_stream)
    stream = torch_stream.cuda_stream

    def step(prec, out):
        p.hpsi_device(x.data_ptr(), NVEC, out.data_ptr(), NVEC, NVEC, layout=E.LAYOUT_INTERLEAVED, prec=prec,
                      stream=stream)

    tuned = p.autotune(nvec=NVEC, prec="fp64") if args.autotune else None

    for _ in range(args.warmup):
        step("fp64", y)
        step("fp32", y32)
    torch.cuda.synchronize()

    def timed(prec, out):
        times, kms = [], []
        for _ in range(args.steps):
            flush.fill_(1.0)
            if world > 1:
                torch.distributed.barrier()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            step(prec, out)
            e1.record()
            e1.synchronize()
            times.append(e0.elapsed_time(e1) / 1e3)
            kms.append(p.last_kernel_ms())
        return times, kms

    with ClockSampler(local) as clk:
        t64, k64 = timed("fp64", y)
        launches = p.last_launch_count()[0] * args.steps
        t32, k32 = timed("fp32", y32)
        launches += p.last_launch_count()[0] * args.steps
    # the FP32 contractions of the slab kernel on the tcgen05 tensor cores (3xTF32), same block
    ytc = torch.empty_like(x)
    p.set_tensor_cores(True, 64)
    for _ in range(args.warmup):
        step("fp32", ytc)
    ttc, ktc = timed("fp32", ytc)
    p.set_tensor_cores(False)
    total64 = max_over_ranks(sum(t64), "cuda")
    value = job_rate(NVEC * args.steps, total64, world)
    mixed = NVEC * args.steps / sum(t32)
    err32 = float((y32 - y).abs().max() / y.abs().max())
    errtc = float((ytc - y).abs().max() / y.abs().max())
    itc = statistics.mean(k[0] for k in ktc)

    # end to end through the host entry point with pinned buffers (column-major, as the
    # Fortran host passes TabPsi(:)%RvecB)
    hx = torch.empty((NVEC, N), dtype=torch.float64).pin_memory()
    hx.copy_(x.t().cpu())
    hy = torch.empty((NVEC, N), dtype=torch.float64).pin_memory()
    p.hpsi_host_ptr(hx.data_ptr(), N, hy.data_ptr(), N, NVEC, E.LAYOUT_COLMAJOR)
    te = []
    for _ in range(args.steps):
        flush.fill_(1.0)
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        p.hpsi_host_ptr(hx.data_ptr(), N, hy.data_ptr(), N, NVEC, E.LAYOUT_COLMAJOR)
        te.append(time.perf_counter() - t0)
    e2e = job_rate(NVEC * args.steps, max_over_ranks(sum(te), "cuda"), world)
    e2e_err = float((hy.t().cuda() - y).abs().max() / y.abs().max())

    # roofline of the dominant kernel: algorithmic FLOPs of one 64-vector launch over the
    # measured FP64 FMA rate
    items_ms = statistics.mean(k[0] for k in k64)
    flop_launch = p.flop_per_hpsi * NVEC
    achieved = flop_launch / (items_ms / 1e3) / 1e12
    fma64 = E.fma_peak(local, "fp64")
    fma32 = E.fma_peak(local, "fp32")
    dgemm = measure_dgemm_tflops(torch, torch.float64)
    items32 = statistics.mean(k[0] for k in k32)

    dav = None
    if not args.no_davidson:
        dav = davidson_legs(p, S)
    cfg = workload_config(p.N, p.nterm, p.sum_nq)
    configs = None
    if not args.no_configs and rank == 0:
        p.close()  # the D=6 L=8 tables (about 11 GB) make room for the other workloads
        configs = {}
        for name, fn in CONFIGS.items():
            t0 = time.perf_counter()
            try:
                configs[name] = fn(args)
            except Exception as e:  # a failed workload is reported, the headline line still prints
                configs[name] = {"error": f"{type(e).__name__}: {e}"}
            configs[name]["wall_s"] = time.perf_counter() - t0

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * total64 / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
            "config": cfg,
            "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": int(N * NVEC * 8),
                    "d2h_bytes_per_step": int(N * NVEC * 8), "rel_err_vs_device": e2e_err},
            "mixed": {"value": mixed, "unit": UNIT, "dtype": "f32 contractions, f64 reduction",
                      "rel_err_vs_fp64": err32, "items_kernel_ms": items32,
                      "achieved_tflops": flop_launch / (items32 / 1e3) / 1e12, "fp32_fma_peak_tflops": fma32,
                      "frac_of_fp32_fma": flop_launch / (items32 / 1e3) / 1e12 / fma32,
                      "contractions": "CUDA cores (default; the autotuner's choice on this workload)",
                      "tensor_cores": {"value": NVEC * args.steps / sum(ttc), "unit": UNIT,
                                       "contractions": "tcgen05 kind::tf32, 3 products of split operands, "
                                                       "FP32 accumulation in TMEM, K*M >= 64",
                                       "rel_err_vs_fp64": errtc, "items_kernel_ms": itc}},
            "roofline": {"bound": "fp64-fma", "achieved": achieved, "peak": fma64, "unit": "TFLOP/s",
                         "frac": achieved / fma64, "traffic": TRAFFIC_PER_LAUNCH,
                         "kernel": "hpsi_slab_kernel<double> + hpsi_items_kernel<double>", "items_kernel_ms": items_ms,
                         "algorithmic_flop_per_launch": flop_launch, "dgemm_tflops": dgemm,
                         "peak_source": "FP64 FMA issue rate measured in this run (evr_fma_peak); no FP64 figure "
                                        "in the measured-peaks file"},
            "roofline_hbm": hbm_roofline(TRAFFIC_PER_LAUNCH, items_ms / 1e3),
            "davidson": dav,
            "configs": configs,
            "autotune": tuned,
            "gpu_launches": launches,
            "clocks": clk.summary()}
    if rank == 0 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        r, dt = cpu_oracle_rate(spec, 1, threads)
        line["cpu_baseline"] = {"value": r, "unit": UNIT, "cores": threads, "kind": "port",
                                "sample": f"1 vector of the block ({dt:.1f} s), CPU oracle with OpenMP over terms"}
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
