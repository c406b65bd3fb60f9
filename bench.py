"""Benchmark of the MOCCa mesh hot path on GB300.

Workload (the 24^3 configuration the headline metric is quoted on): N=Z=28,
24^3 stored EV8 mesh (48^3 full box), dx=0.8 fm, nwt=160 spinors (80 n +
80 p), SLy4, time-reversal invariant, HFB pairing (G=1250 MeV fm^3,
alpha=1), seeded harmonic-oscillator start, imaginary-time step dt=0.010
with momentum 0.3.  A step is one pass of the Evolve loop body
(src/Main.f90:255-328): GradDesc with Gram-Schmidt, the HFB pairing step,
DeriveAll, densities, moments, potentials with the Coulomb CG, energy.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--precision mixed|fp64] [--accuracy-iters A] [--breakdown] [--no-micro]
                  [--no-batch] [--no-large]

One JSON line on rank 0.  `value` is the headline form (mixed precision by
default): K steps with every input resident in HBM (CUDA events on the
library's stream, barrier + synchronize on both sides, max over ranks).
`fp64` is the plain FP64 path timed the same way in the same job, and
`accuracy` compares A iterations of the mixed form (the last 20 in FP64)
with A iterations of the FP64 path: |dE_total| in MeV.  `e2e` times the same
steps through the C ABI with the spinors uploaded from pinned host memory and
the spinors plus the energy read back every step.  The working set
(spinors, derivatives, updates: ~0.7 GB) is larger than the 129 MB L2, so
no flush is needed between steps.  Multi-GPU runs are independent replicas
(weak scaling).  `microbench_32c_200` times DeriveAll and h.psi of 200
spinors on the 32^3 symmetry-free box in both precisions, `poisson_64c`
one Coulomb solve on a 64^3 mesh, and `batched_64_uneven` 64 independent
Q20-constrained HFB instances of uneven size run concurrently through the
batch API (after its schedule autotuner) and one after another, and
`large_36c_300` 200 iterations of N=50, Z=40 on a 36^3 mesh with nwt=300,
mixed (last 20 in FP64) against FP64, and `c1_mg24_readme` the README Mg24
run (100 iterations, FP64) on the GPU beside the oracle.
"""
from __future__ import annotations

import argparse
import ctypes as C
import dataclasses
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

WORKLOAD = dict(nx=24, ny=24, nz=24, dx=0.8, nwt=160, neutrons=28.0, protons=28.0)
DT, MOMENTUM = 0.010, 0.3
POLISH = 20   # final FP64 iterations of the mixed form
# Iterations each timed arm runs from the HO start before its warm-up (untimed,
# like resuming from a restart file), so that the timed steps sample the
# converging phase of a 300-iteration run rather than only its first steps.
PREPARE = 100
METRIC = "HFB iter/s at 24^3, nwt=160: mixed vs FP64 GPU at |dE|<=1e-5 MeV"
# DRAM traffic of one mixed DeriveBasis (the three k_deriv_tc passes, nwt=160,
# 24^3) from ncu dram__bytes_read.sum + dram__bytes_write.sum, and the tensor
# pipe's active share over those launches, weighted by their durations
# (profiles/deriv_tc_24c_nwt160_full.md)
DERIV_TC_TRAFFIC = 610.3e6
DERIV_TC_TENSOR_ACTIVE = 0.103


def _params(precision):
    from mocca_gb300 import MG_FP64, MG_MIXED, MG_PAIRING_HFB, RunParams
    return RunParams(**WORKLOAD, precision=MG_MIXED if precision == "mixed" else MG_FP64,
                     pairing=MG_PAIRING_HFB)


def _config(precision, world):
    return {"workload": "N=Z=28 HO start (seed 1234), 24^3 EV8 stored mesh, dx=0.8, nwt=160, "
                        "SLy4, TRC, HFB pairing G=1250 alpha=1 (surface delta, 5 MeV cutoff), "
                        "dt=0.010, momentum 0.3, MixingScheme 0 (DampingParam 0.75)",
            **WORKLOAD, "precision": precision, "dt": DT, "momentum": MOMENTUM,
            "l2": "working set ~0.7 GB > 129 MB L2, no flush",
            "start": f"state after {PREPARE} iterations of the same form from the HO start "
                     "(prepared untimed), then the warm-up, then the timed steps",
            "parallelism": f"replicas x{world}"}


def _start_state(p, seed):
    from mocca_gb300 import synthetic
    return synthetic.ho_basis(p, p.nwt // 2, seed=seed)


def _make(precision, seed, stream=None):
    from mocca_gb300 import SLY4
    from mocca_gb300.mesh import MeshState
    p = _params(precision)
    psi, qn, en = _start_state(p, seed)
    g = MeshState(p, SLY4, stream=stream)
    g.set_spinors(psi, qn)
    g.set_energies(en)
    g.set_pairing()
    g.Start()
    return p, g


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except FileNotFoundError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            self.proc.wait(timeout=5)
            self.t.join(timeout=2)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4)
                          if len(r) > 2 + i and r[2 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.rows)}


def max_over_ranks(x, device="cuda"):
    """The slowest rank's time (replicas: the whole job ends with it)."""
    import torch
    if not (torch.distributed.is_available() and torch.distributed.is_initialized()):
        return x
    t = torch.tensor([x], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(world, steps, seconds):
    """Weak scaling: every rank runs `steps` iterations of its own replica."""
    return world * steps / seconds


def measured_peaks():
    try:
        return json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
    except Exception:
        return {}


def fp64_dgemm_peak(torch):
    """Measured FP64 throughput of a cuBLAS DGEMM (denominator for FP64-equivalent rates)."""
    n = 4096
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
    for _ in range(2):
        torch.matmul(a, b)
    torch.cuda.synchronize()
    best = 1e9
    for _ in range(3):
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        torch.matmul(a, b)
        e.record()
        torch.cuda.synchronize()
        best = min(best, s.elapsed_time(e) / 1e3)
    return 2 * n ** 3 / best / 1e12


def _oracle_state(timing=True, threads=1):
    """The oracle at the bench start.  timing=True: the -O3 OpenMP build (the
    CPU baseline) on `threads` host threads; False: the parity build."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle as O
    from mocca_gb300 import SLY4
    p = _params("fp64")
    psi, qn, en = _start_state(p, 1234)
    o = O.OracleState(p, SLY4, timing=timing)
    used = o.lib.orc_set_threads(threads)
    o.set_spinors(psi, qn)
    o.set_energies(en)
    o.set_pairing()
    o.Start()
    return o, used


def _host_threads():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def cpu_baseline(sample_steps=8, single_steps=1):
    """The FP64 oracle (C++ restatement of the reference's algorithms, -O3,
    OpenMP over spinors and spinor pairs) on a bounded sample of the
    workload: all host threads, and one thread beside it."""
    o, cores = _oracle_state(True, _host_threads())
    t = time.perf_counter()
    o.Evolve(sample_steps, DT, MOMENTUM)
    dt = time.perf_counter() - t
    o.close()
    o1, _ = _oracle_state(True, 1)
    t = time.perf_counter()
    o1.Evolve(single_steps, DT, MOMENTUM)
    dt1 = time.perf_counter() - t
    o1.close()
    return {"value": sample_steps / dt, "unit": "iter/s", "cores": cores, "kind": "port",
            "sample": f"{sample_steps} HFB iterations of the full 24^3 nwt=160 workload after its "
                      f"start, oracle (C++ FP64 restatement, -O3, OpenMP, {cores} threads), "
                      f"{dt:.1f} s",
            "single_thread": {"value": single_steps / dt1, "unit": "iter/s", "cores": 1,
                              "sample": f"{single_steps} iteration(s), {dt1:.1f} s"}}


def run_reference(args, rank, world):
    """--impl reference: the reference's CPU path (oracle port, -O3 OpenMP
    build on every host thread; no Fortran compiler exists to build the
    reference itself)."""
    if rank != 0:
        return None
    steps = max(1, min(args.steps, 30))
    warm = max(0, min(args.warmup, 1))
    o, cores = _oracle_state(True, _host_threads())
    if warm:
        o.Evolve(warm, DT, MOMENTUM)
    t = time.perf_counter()
    o.Evolve(steps, DT, MOMENTUM)
    dt = time.perf_counter() - t
    o.close()
    val = steps / dt
    return {
        "metric": METRIC, "value": val, "unit": "iter/s", "impl": "reference",
        "n_gpus": world, "steps": steps, "warmup": warm, "ms_per_step": dt / steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": _config(args.precision, world),
        "cpu_baseline": {"value": val, "unit": "iter/s", "cores": cores, "kind": "port",
                         "sample": f"{steps} full HFB iteration(s) (at most 30 to bound the run) "
                                   f"on {cores} host threads; the reference is Fortran without "
                                   "OpenMP and no Fortran compiler exists here or on the GPU "
                                   "host, so its C++ FP64 restatement is timed (-O3, OpenMP "
                                   "over spinors and spinor pairs)"},
        "e2e": {"value": val, "unit": "iter/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def _timed_steps(g, torch, stream, steps, barrier, clk_index=None):
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    l0 = g.launch_count()
    if clk_index is not None:
        with ClockSampler(clk_index) as clk:
            ev0.record(stream)
            last = g.Evolve(steps, DT, MOMENTUM)
            ev1.record(stream)
            barrier()
        clocks = clk.summary()
    else:
        ev0.record(stream)
        last = g.Evolve(steps, DT, MOMENTUM)
        ev1.record(stream)
        barrier()
        clocks = None
    return ev0.elapsed_time(ev1) / 1e3, last, g.launch_count() - l0, clocks


def state_errors(gm, gf):
    """Mixed-against-FP64 differences of the final states: the single-particle
    energies <psi|h|psi> of the HF basis (GradDesc's, energy-ordered), max
    |de| in MeV (compared as sorted lists per isospin), and the density L2
    norm, |rho_m - rho_f| / |rho_f|.  The canonical basis is not used for the
    energies: inside a cluster of equal occupations its states may rotate
    freely, which moves their individual energies but not the density."""
    import numpy as np
    from mocca_gb300 import _abi
    out = {}
    em, ef = gm.get_energies(_abi.MG_HF_BASIS)[0], gf.get_energies(_abi.MG_HF_BASIS)[0]
    half = len(em) // 2   # both starts: the first half neutrons, the second protons
    de = max(np.abs(np.sort(em[:half]) - np.sort(ef[:half])).max(),
             np.abs(np.sort(em[half:]) - np.sort(ef[half:])).max())
    rm, rf = gm.get_densities()["rho"], gf.get_densities()["rho"]
    out["d_sp_energy_max_MeV"] = float(de)
    out["density_l2_rel"] = float(np.linalg.norm(rm - rf) / np.linalg.norm(rf))
    return out


def whole_run(iters, seed, torch, stream):
    """The 24^3 configuration as defined: `iters` iterations from the HO
    start, the mixed form's last POLISH of them in FP64, against `iters`
    FP64 iterations from the same start; each whole run timed with CUDA
    events on the library's stream (the identical Start of both is outside).
    Reports both rates, their ratio, |dE_total|, the single-particle energies
    and the density L2 difference.  The FP64 GPU path stands for the FP64
    oracle here (tests/test_gpu_bench_configs.py holds it to the oracle at
    1e-8 MeV on this workload); a 300-iteration oracle run would take ~9
    minutes of CPU."""
    from mocca_gb300 import MG_FP64
    out = {"iterations": iters, "fp64_polish": POLISH,
           "start": "HO start (seed %d), Start() untimed" % seed}
    ev = lambda: torch.cuda.Event(enable_timing=True)  # noqa: E731
    states = {}
    for name in ("mixed", "fp64"):
        with torch.cuda.stream(stream):
            _, g = _make(name, seed, stream=stream.cuda_stream)
        a, b, c = ev(), ev(), ev()
        torch.cuda.synchronize()
        a.record(stream)
        if name == "mixed":
            em = g.Evolve(iters - POLISH, DT, MOMENTUM)["total"]
            b.record(stream)
            g.set_precision(MG_FP64)
            e = g.Evolve(POLISH, DT, MOMENTUM)["total"]
        else:
            e = g.Evolve(iters, DT, MOMENTUM)["total"]
            em = None
        c.record(stream)
        torch.cuda.synchronize()
        t = a.elapsed_time(c) / 1e3
        out[name] = {"value": iters / t, "unit": "iter/s", "seconds": t, "E_total": e}
        if em is not None:
            out[name]["E_before_polish"] = em
            out[name]["seconds_mixed_part"] = a.elapsed_time(b) / 1e3
        states[name] = g
    out["speedup_vs_fp64"] = out["fp64"]["seconds"] / out["mixed"]["seconds"]
    out["dE_total_MeV"] = out["mixed"]["E_total"] - out["fp64"]["E_total"]
    out.update(state_errors(states["mixed"], states["fp64"]))
    out["pass"] = abs(out["dE_total_MeV"]) <= 1e-5
    for g in states.values():
        g.close()
    return out


def microbench_c2(torch, stream, reps=5):
    """Mesh-kernel microbench on the 32^3 full (symmetry-free) box: 200
    Gaussian x Hermite spinors (seed 42) in Woods-Saxon fields; d/dx,y,z +
    Laplacian of every spinor (DeriveAll) and h.psi, FP64 and mixed."""
    import numpy as np
    from mocca_gb300 import MG_FP64, MG_MIXED, SLY4, RunParams, synthetic
    from mocca_gb300.mesh import MeshState
    out = {"workload": "32^3 full box (no symmetries, unfolded Lagrange matrices), dx=0.8, "
                       "200 spinors, Woods-Saxon U/B/W (R=3.5, a=0.65)"}
    for name, prec in (("fp64", MG_FP64), ("mixed", MG_MIXED)):
        p = RunParams(nx=32, ny=32, nz=32, dx=0.8, pc=0, sc=0, tsc=0, trc=1, nwt=200,
                      neutrons=8, protons=8, coulomb_solver=0, precision=prec)
        psi = synthetic.gaussian_hermite_spinors(p, p.nwt, seed=42)
        qn = np.tile(np.array([-1, 0, 0, 0], dtype=np.int32), (p.nwt, 1))
        qn[p.nwt // 2:, 0] = 1
        with torch.cuda.stream(stream):
            g = MeshState(p, SLY4, stream=stream.cuda_stream)
        g.set_spinors(psi, qn)
        g.set_energies(np.zeros(p.nwt))
        U, B, nB, W, dW = synthetic.woods_saxon_fields(p)
        g.set_potentials(U=U, B=B, nablaB=nB, W=W, divW=dW)
        g.DeriveBasis(0)
        g.hPsi(want_spinors=False)
        torch.cuda.synchronize()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        ev[0].record(stream)
        for _ in range(reps):
            g.DeriveBasis(0)
        ev[1].record(stream)
        for _ in range(reps):
            g.hPsi(want_spinors=False)
        ev[2].record(stream)
        torch.cuda.synchronize()
        t_d = ev[0].elapsed_time(ev[1]) / 1e3 / reps
        t_h = ev[1].elapsed_time(ev[2]) / 1e3 / reps
        V = p.V
        out[name] = {"derive_ms": t_d * 1e3,
                     "derive_gflops": 48.0 * 32 * V * p.nwt / t_d / 1e9,
                     "derive_gbs": 160.0 * V * p.nwt / t_d / 1e9,
                     "hpsi_ms": t_h * 1e3,
                     "hpsi_gbs": 192.0 * V * p.nwt / t_h / 1e9}
        g.close()
    return out


def poisson_64c(torch, stream):
    """Coulomb problem on the 64^3 stored EV8 mesh (128^3 full box), dx=0.8: a
    deformed Gaussian proton density (Z=40, axes 1:1:1.3, width 3 fm),
    multipole boundary values; one cold solve from the uniform-sphere guess,
    each solver to a relative residual of 1e-10: the FP64 CG (the
    reference's algorithm), the FP32 multigrid V-cycles inside the FP64
    conjugate-gradient iteration (CoulombSolver = 2), and the direct
    separable solve with two FP64 refinement rounds (the mixed form's
    default).  Best of two timed solves after one that sets the solver up."""
    import numpy as np
    from mocca_gb300 import MG_FP64, MG_MIXED, SLY4, RunParams, synthetic
    from mocca_gb300.mesh import MeshState
    out = {"workload": "64^3 EV8 stored (128^3 box), dx=0.8, Gaussian rho_p Z=40, "
                       "axes 1:1:1.3, width 3 fm; every solver to |b - L phi| <= 1e-10 |b|"}
    for name, prec, solver in (("fp64_cg", MG_FP64, 1), ("fp32_multigrid_fp64_pcg", MG_FP64, 2),
                               ("direct_fp64_refinement", MG_MIXED, 1)):
        p = RunParams(nx=64, ny=64, nz=64, dx=0.8, nwt=2, neutrons=40, protons=40,
                      precision=prec, coulomb_solver=solver, coulomb_prec=1e-10)
        x, y, z = synthetic.mesh_axes(p)
        X, Y, Z = np.meshgrid(x, y, z, indexing="ij")
        rp = np.exp(-(X ** 2 + Y ** 2) / 9.0 - Z ** 2 / (9.0 * 1.69)).transpose(2, 1, 0)
        rp *= 40.0 / (rp.sum() * p.dv)
        rho = np.concatenate([rp.reshape(-1), rp.reshape(-1)])
        with torch.cuda.stream(stream):
            g = MeshState(p, SLY4, stream=stream.cuda_stream)
        g.set_densities(rho=rho)
        g.CalculateAllMoments()
        g.SolveCoulomb()   # first call: setup (hierarchy, eigenvectors, graph)
        best = None
        for rep in range(2):
            g.set_densities(rho=rho)
            g.CalculateAllMoments()
            g.reset_coulomb_guess()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            it = g.SolveCoulomb()
            e1.record(stream)
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1)
            if best is None or ms < best["ms"]:
                best = {"ms": ms, "iterations": it, "residual_rel": g.CoulombResidual()}
        g.close()
        out[name] = best
    return out


def run_ours(args, rank, world, local_rank):
    import torch
    from mocca_gb300 import _abi

    torch.cuda.set_device(local_rank)
    stream = torch.cuda.Stream()
    dist = world > 1
    seed = 1234 + rank

    def barrier():
        if dist:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    with torch.cuda.stream(stream):
        p, g = _make(args.precision, seed, stream=stream.cuda_stream)
    if PREPARE > 0:
        g.Evolve(PREPARE, DT, MOMENTUM)
    g.Evolve(max(3, args.warmup), DT, MOMENTUM)
    torch.cuda.synchronize()

    # ---- device-resident throughput of the headline form --------------------------
    t_dev, last, launches, clocks = _timed_steps(g, torch, stream, args.steps, barrier, local_rank)
    t_dev = max_over_ranks(t_dev)

    # ---- end-to-end through the C ABI with host buffers --------------------------------
    host_psi = torch.empty((p.nwt, 4 * p.V), dtype=torch.float64, pin_memory=True)
    host_psi.copy_(torch.from_numpy(g.get_spinors().reshape(p.nwt, -1)))
    out_psi = torch.empty_like(host_psi).pin_memory()
    nwt = p.nwt
    up = (C.c_void_p * nwt)(*[host_psi[i].data_ptr() for i in range(nwt)])
    dn = (C.c_void_p * nwt)(*[out_psi[i].data_ptr() for i in range(nwt)])
    e_terms = _abi.MgEnergyTerms()
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        _abi.check("mg_upload_spinors", g.lib.mg_upload_spinors(g.h, 0, up, None, 0, nwt))
        _abi.check("mg_iterate", g.lib.mg_iterate(g.h, 1, DT, MOMENTUM, C.byref(e_terms)), True)
        _abi.check("mg_download_spinors", g.lib.mg_download_spinors(g.h, 0, dn, 0, nwt))
        host_psi, out_psi = out_psi, host_psi
        up, dn = dn, up
    barrier()
    t_e2e = max_over_ranks(time.perf_counter() - t0)

    # ---- dominant kernel pair: the Lagrange derivatives of one basis ------------------
    reps = 5
    k0, k1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    k0.record(stream)
    for _ in range(reps):
        g.DeriveBasis(0)
    k1.record(stream)
    torch.cuda.synchronize()
    t_der = k0.elapsed_time(k1) / 1e3 / reps
    flops = 48.0 * p.nx * p.V * p.nwt     # 4 comps x 6 line contractions x 2 n flops per point
    bytes_ = 160.0 * p.V * p.nwt          # FP64 psi in, 3 first derivatives + Laplacian out

    # ---- h.psi of the canonical basis (energies only): psi, 3 derivatives and the
    # Laplacian in (5 x 4V values of 8 bytes per spwf), the isospins' 17 fields once
    torch.cuda.synchronize()
    k0.record(stream)
    for _ in range(reps):
        _abi.check("mg_hpsi", g.lib.mg_hpsi(g.h, 1, None, None, None))
    k1.record(stream)
    torch.cuda.synchronize()
    t_hpsi = k0.elapsed_time(k1) / 1e3 / reps
    bytes_hpsi = 160.0 * p.V * p.nwt + 2 * 17 * 8.0 * p.V

    breakdown = stage_breakdown(g, torch, stream) if args.breakdown else None
    g.close()

    # ---- the plain FP64 path on the same workload (same job, same GPU) ------------------
    fp64 = None
    if args.precision == "mixed":
        with torch.cuda.stream(stream):
            _, g64 = _make("fp64", seed, stream=stream.cuda_stream)
        if PREPARE > 0:
            g64.Evolve(PREPARE, DT, MOMENTUM)
        g64.Evolve(max(3, args.warmup), DT, MOMENTUM)
        t64, _, _, _ = _timed_steps(g64, torch, stream, args.steps, barrier)
        t64 = max_over_ranks(t64)
        g64.close()
        fp64 = {"value": whole_job_rate(world, args.steps, t64), "unit": "iter/s",
                "ms_per_step": t64 / args.steps * 1e3}

    accuracy = None
    if rank == 0 and args.precision == "mixed" and args.accuracy_iters > POLISH:
        accuracy = whole_run(args.accuracy_iters, seed, torch, stream)
    micro = microbench_c2(torch, stream) if rank == 0 and args.micro else None
    poisson = poisson_64c(torch, stream) if rank == 0 and args.micro else None
    batched = batched_64_uneven(torch) if rank == 0 and args.batch else None
    large = large_36c_300(torch) if rank == 0 and args.large else None
    c1 = c1_mg24_readme(torch) if rank == 0 and args.micro else None

    if rank != 0:
        return None
    peaks = measured_peaks()
    hbm = peaks.get("hbm_gbs", 6800.0)
    fp64_peak = fp64_dgemm_peak(torch)
    mixed = args.precision == "mixed"
    value = whole_job_rate(world, args.steps, t_dev)
    res = {
        "metric": METRIC,
        "value": value,
        "unit": "iter/s",
    }
    # the configuration's comparison first: whole 300-iteration runs (mixed
    # with its FP64 polish against FP64), then the K-step window ratio
    if accuracy:
        res["speedup_vs_fp64"] = accuracy["speedup_vs_fp64"]
        res["whole_run"] = {k: accuracy[k] for k in
                            ("iterations", "fp64_polish", "speedup_vs_fp64", "dE_total_MeV",
                             "d_sp_energy_max_MeV", "density_l2_rel", "pass")}
        res["whole_run"]["mixed_iter_s"] = accuracy["mixed"]["value"]
        res["whole_run"]["fp64_iter_s"] = accuracy["fp64"]["value"]
    if fp64:
        res["fp64"] = fp64
        res["speedup_vs_fp64_window"] = value / fp64["value"]
    res.update({
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t_dev / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": ("f64 (exact BF16-digit tensor-core and double-float mesh kernels)" if mixed
                  else "f64"),
        "data": "synthetic",
        "config": _config(args.precision, world),
        "e2e": {"value": whole_job_rate(world, args.steps, t_e2e), "unit": "iter/s",
                "h2d_bytes_per_step": int(host_psi.numel() * 8),
                "d2h_bytes_per_step": int(out_psi.numel() * 8 + C.sizeof(e_terms))},
        "roofline": {"kernel": ("k_deriv_tc x3 (x, y, z passes)" if mixed else
                                "k_deriv_xy + k_deriv_z") + " (DeriveBasis, HF basis)",
                     "bound": "hbm", "achieved": bytes_ / t_der / 1e9, "peak": hbm,
                     "unit": "GB/s", "frac": bytes_ / t_der / 1e9 / hbm,
                     "traffic": DERIV_TC_TRAFFIC if mixed else None,
                     "tensor_pipe_active_ncu": DERIV_TC_TENSOR_ACTIVE if mixed else None,
                     "peak_source": "MEASURED_PEAKS.json hbm_gbs (copy, burst)",
                     "fp64_equivalent": {"achieved_tflops": flops / t_der / 1e12,
                                         "dgemm_tflops_measured": fp64_peak,
                                         "frac_of_dgemm": flops / t_der / 1e12 / fp64_peak},
                     "ms_per_derive": t_der * 1e3},
        "roofline_hpsi": {"kernel": ("k_hpsi_df" if mixed else "k_hpsi") + " (h.psi of the "
                                     "canonical basis, energies only, with its field staging "
                                     "and energy reduction; each call ends with a host "
                                     "synchronisation, so this is a lower bound)",
                          "bound": "hbm", "achieved": bytes_hpsi / t_hpsi / 1e9, "peak": hbm,
                          "unit": "GB/s", "frac": bytes_hpsi / t_hpsi / 1e9 / hbm,
                          "ms_per_call": t_hpsi * 1e3},
        "cpu_baseline": cpu_baseline(),
        "clocks": clocks,
        "gpu_launches": int(launches),
        "energy_last": last["total"],
    })
    if accuracy:
        res["accuracy"] = accuracy
    if breakdown:
        res["breakdown_ms"] = breakdown
    if micro:
        res["microbench_32c_200"] = micro
    if poisson:
        res["poisson_64c"] = poisson
    if batched:
        res["batched_64_uneven"] = batched
    if large:
        res["large_36c_300"] = large
    if c1:
        res["c1_mg24_readme"] = c1
    return res


def batched_64_uneven(torch, rounds=190, seq_rounds=5):
    """64 independent Q20-constrained HFB instances of uneven size (mixed
    precision), run concurrently through mg_batch_* after the schedule
    autotuner, then driven one after another (one worker) for comparison.
    With the tuner's passes (probe 1: one alone plus one per candidate worker
    count) and 2 warm-up rounds, the default 190 timed rounds make 200
    iterations per instance.
    A round is one Evolve pass of every instance; the rate is instance
    iterations per second (host clock around each batch call, which returns
    when every instance's work is complete)."""
    from mocca_gb300 import SLY4, synthetic
    from mocca_gb300.mesh import Batch, MeshState
    inst = synthetic.uneven_instances(64, seed=7)
    states = []
    t_setup = time.perf_counter()
    for d in inst:
        p = d["params"]
        psi, qn, en = synthetic.ho_basis(p, d["n_neutron"], seed=d["seed"])
        g = MeshState(p, SLY4)
        g.set_spinors(psi, qn)
        g.set_energies(en)
        g.set_pairing()
        g.add_constraint(2, 0, d["q20"])
        g.Start()
        states.append(g)
    torch.cuda.synchronize()
    t_setup = time.perf_counter() - t_setup
    b = Batch(states)
    t_tune = time.perf_counter()
    workers = b.tune(1, DT, MOMENTUM)
    t_tune = time.perf_counter() - t_tune
    hw = os.cpu_count() or 1
    cands = [w for w in (1, 2, 4, 8, 16, 32, 64) if w <= min(64, 4 * hw)]
    if 64 <= 4 * hw and cands[-1] != 64:
        cands.append(64)
    tuner_passes = 1 + len(cands)
    b.Evolve(2, DT, MOMENTUM)
    t0 = time.perf_counter()
    out = b.Evolve(rounds, DT, MOMENTUM)
    t_batch = time.perf_counter() - t0
    b.set_workers(1)
    t0 = time.perf_counter()
    b.Evolve(seq_rounds, DT, MOMENTUM)
    t_seq = time.perf_counter() - t0
    q20 = [sum(s.get_constraint(0)["value"]) for s in states]
    rate = 64 * rounds / t_batch
    rate_seq = 64 * seq_rounds / t_seq
    # INITWF's Nilsson start of the same 64 instances built on the device
    # (mg_nilsson_start, into the finished states), against the numpy
    # restatement with its upload for the first four (the batch itself
    # starts from the HO states)
    b.close()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for d, s in zip(inst, states):
        s.NilssonStart(d["n_neutron"], amplitude=1e-3, seed=d["seed"])
    torch.cuda.synchronize()
    t_nil_dev = time.perf_counter() - t0
    t0 = time.perf_counter()
    for d, s in zip(inst[:4], states[:4]):
        psi, qn, en = synthetic.nilsson_basis(d["params"], d["n_neutron"], seed=d["seed"])
        s.set_spinors(psi, qn)
        s.set_energies(en)
    t_nil_host = (time.perf_counter() - t0) / 4
    nilsson = {"device_ms_per_instance": t_nil_dev / 64 * 1e3,
               "host_numpy_ms_per_instance": t_nil_host * 1e3,
               "host_sample": "instances 0-3 (numpy restatement + upload)"}
    res = {
        "workload": "64 HFB instances, seed 7: beta2 ~ U[-0.3, 0.5] (Q20 constraint, alternating "
                    "kind, always on), N, Z even in [8, 40], n^3 EV8 stored meshes n in [12, 28] "
                    "(box holds the nucleus), nwt = round(1.4 A) in [20, 200]; SLy4, HFB "
                    "G=1250 alpha=1, mixed precision, dt=0.010, momentum 0.3",
        "meshes": sorted(d["params"].nx for d in inst),
        "nwt_total": int(sum(d["params"].nwt for d in inst)),
        "workers_tuned": workers,
        "value": rate, "unit": "instance-iter/s",
        "ms_per_round": t_batch / rounds * 1e3,
        "sequential": {"value": rate_seq, "unit": "instance-iter/s",
                       "ms_per_round": t_seq / seq_rounds * 1e3},
        "speedup_vs_sequential": rate / rate_seq,
        "rounds_timed": rounds, "iterations_per_instance": rounds + 2 + tuner_passes,
        "setup_s": t_setup, "tune_s": t_tune,
        "energies_finite": bool(all(math.isfinite(o["total"]) for o in out)),
        "q20_rel_dev_max": float(max(abs(q - d["q20"]) / max(1.0, abs(d["q20"]))
                                     for q, d in zip(q20, inst))),
        "nilsson_start": nilsson,
    }
    for s in states:
        s.close()
    return res


def large_36c_300(torch, iters=200, polish=POLISH):
    """N=50, Z=40 on a 36^3 EV8 stored mesh with nwt=300 (150 n + 150 p),
    HFB, from the seeded HO start: `iters` iterations of the mixed form
    (the last `polish` in FP64) and `iters` of the FP64 path, each timed
    whole with CUDA events; |dE_total| between them."""
    from mocca_gb300 import MG_FP64, MG_MIXED, SLY4, RunParams, _abi, synthetic
    from mocca_gb300.mesh import MeshState
    p = RunParams(nx=36, ny=36, nz=36, dx=0.8, nwt=300, neutrons=50.0, protons=40.0,
                  pairing=_abi.MG_PAIRING_HFB)
    psi, qn, en = synthetic.ho_basis(p, 150, seed=1234)
    stream = torch.cuda.Stream()
    out = {"workload": "N=50, Z=40, 36^3 EV8 stored mesh, dx=0.8, nwt=300 (150 n + 150 p), "
                       "SLy4, HFB G=1250 alpha=1, HO start (seed 1234), dt=0.010, momentum 0.3",
           "iterations": iters, "fp64_polish": polish}
    states = {}
    for name, prec in (("mixed", MG_MIXED), ("fp64", MG_FP64)):
        with torch.cuda.stream(stream):
            g = MeshState(dataclasses.replace(p, precision=prec), SLY4,
                          stream=stream.cuda_stream)
        g.set_spinors(psi, qn)
        g.set_energies(en)
        g.set_pairing()
        g.Start()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record(stream)
        if prec == MG_MIXED:
            g.Evolve(iters - polish, DT, MOMENTUM)
            g.set_precision(MG_FP64)
            e = g.Evolve(polish, DT, MOMENTUM)
        else:
            e = g.Evolve(iters, DT, MOMENTUM)
        b.record(stream)
        torch.cuda.synchronize()
        t = a.elapsed_time(b) / 1e3
        out[name] = {"value": iters / t, "unit": "iter/s", "ms_per_iter": t / iters * 1e3,
                     "E_total": e["total"]}
        states[name] = g
    out["speedup_vs_fp64"] = out["mixed"]["value"] / out["fp64"]["value"]
    out["dE_total_MeV"] = out["mixed"]["E_total"] - out["fp64"]["E_total"]
    out.update(state_errors(states["mixed"], states["fp64"]))
    for g in states.values():
        g.close()
    return out


def c1_mg24_readme(torch):
    """The reference README's Mg24 run (the CPU-runnable configuration):
    10^3 stored EV8 mesh, nwt=40, N=Z=12, SLy4, HFB (GuessKappa), Nilsson
    start + seeded 1e-3 perturbation, MixingScheme 2, ParameterEstimation 1,
    a Q20 constraint of 50 fm^2 for 10 iterations, 100 iterations, FP64.
    The GPU runs it with the reference's Fermi search (fermi_solver = 1) and
    with the library's Newton search; the oracle (1 thread) runs it beside;
    |dE_total| of the first against the oracle after the 100 iterations."""
    sys.path[:0] = [str(ROOT / "tests" / "golden"), str(ROOT / "oracle")]
    import make_golden
    import oracle as O
    from mocca_gb300 import SLY4, _abi
    from mocca_gb300.mesh import MeshState
    p, psi, qn, en = make_golden.c1_state()
    n = 100
    out = {"workload": "README Mg24 run: N=Z=12, 10^3 EV8 stored mesh, dx=0.8, nwt=40, SLy4, "
                       "HFB G=1250 alpha=1 GuessKappa, Nilsson start + 1e-3 perturbation (seed "
                       "1234), MixingScheme 2, ParameterEstimation 1, Q20 constraint 50 fm^2 "
                       "for 10 iterations, FP64", "iterations": n}
    for name, solver in (("gpu_reference_search", 1), ("gpu_newton_search", 0)):
        g = MeshState(p, SLY4)
        pp = _abi.MgPairingParams.defaults()
        pp.fermi_solver = solver
        g.set_spinors(psi, qn)
        g.set_energies(en)
        g.set_pairing(pp)
        g.add_constraint(2, 0, 50.0, 0.0, 10)
        g.Start()
        torch.cuda.synchronize()
        t = time.perf_counter()
        e = g.Evolve(n, DT, MOMENTUM)
        torch.cuda.synchronize()
        t = time.perf_counter() - t
        out[name] = {"value": n / t, "unit": "iter/s", "E_total": e["total"]}
        g.close()
    o = O.OracleState(p, SLY4)
    o.set_spinors(psi, qn)
    o.set_energies(en)
    o.set_pairing()
    o.add_constraint(2, 0, 50.0, 0.0, 10)
    o.Start()
    t = time.perf_counter()
    e = o.Evolve(n, DT, MOMENTUM)
    t = time.perf_counter() - t
    out["cpu_oracle"] = {"value": n / t, "unit": "iter/s", "E_total": e["total"], "cores": 1,
                         "kind": "port"}
    out["dE_total_MeV"] = out["gpu_reference_search"]["E_total"] - e["total"]
    return out


def stage_breakdown(g, torch, stream):
    out = {}
    ev = lambda: torch.cuda.Event(enable_timing=True)  # noqa: E731

    def t(name, fn, reps=3):
        a, b = ev(), ev()
        torch.cuda.synchronize()
        a.record(stream)
        for _ in range(reps):
            fn()
        b.record(stream)
        torch.cuda.synchronize()
        out[name] = a.elapsed_time(b) / reps

    t("grad_desc(hpsi+gs)", lambda: g.GradDesc(DT, MOMENTUM))
    t("gram_schmidt", g.GramSchmidt)
    t("solve_pairing", g.SolvePairing, reps=1)
    t("derive_all", g.DeriveAll)
    t("densities", g.UpdateDensities)
    t("moments", g.CalculateAllMoments)
    t("construct_potentials", g.ConstructPotentials)
    t("energy", g.CompEnergy)
    return out


def _profile_state(workload, precision, stream):
    """A prepared context for --profile-iteration: the headline workload, the
    36^3 nwt=300 one, or the 10^3 Mg24-type HFB start with a Q20 constraint
    (50 fm^2, on for the first 10 iterations) and ParameterEstimation = 1."""
    from mocca_gb300 import MG_FP64, MG_MIXED, SLY4, RunParams, _abi, synthetic
    from mocca_gb300.mesh import MeshState
    prec = MG_MIXED if precision == "mixed" else MG_FP64
    if workload == "headline":
        _, g = _make(precision, 1234, stream=stream.cuda_stream)
        return g, PREPARE
    if workload == "large":
        p = RunParams(nx=36, ny=36, nz=36, dx=0.8, nwt=300, neutrons=50.0, protons=40.0,
                      pairing=_abi.MG_PAIRING_HFB, precision=prec)
        psi, qn, en = synthetic.ho_basis(p, 150, seed=1234)
        prepare = 5
    else:
        p = RunParams(nx=10, ny=10, nz=10, dx=0.8, nwt=40, neutrons=12.0, protons=12.0,
                      pairing=_abi.MG_PAIRING_HFB, precision=prec, parameter_estimation=1)
        psi, qn, en = synthetic.ho_basis(p, 20, seed=1234)
        prepare = 2
    g = MeshState(p, SLY4, stream=stream.cuda_stream)
    g.set_spinors(psi, qn)
    g.set_energies(en)
    g.set_pairing()
    if workload == "c1q20":
        g.add_constraint(2, 0, 50.0, 0.0, 10)
    g.Start()
    return g, prepare


def profile_iteration(precision, workload="headline"):
    """The state after the workload's preparation iterations (plus 3 warm-up
    steps), then one HFB iteration between cudaProfilerStart and
    cudaProfilerStop, for `ncu --profile-from-start off` (launch lists and
    kernel captures)."""
    import torch
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        g, prepare = _profile_state(workload, precision, stream)
    if prepare > 0:
        g.Evolve(prepare, DT, MOMENTUM)
    g.Evolve(3, DT, MOMENTUM)
    torch.cuda.synchronize()
    torch.cuda.profiler.start()
    g.Evolve(1, DT, MOMENTUM)
    torch.cuda.synchronize()
    torch.cuda.profiler.stop()
    g.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--accuracy-iters", type=int, default=300)
    ap.add_argument("--breakdown", action="store_true")
    ap.add_argument("--no-micro", dest="micro", action="store_false",
                    help="skip the 32^3 mesh-kernel and 64^3 Poisson lines")
    ap.add_argument("--no-batch", dest="batch", action="store_false",
                    help="skip the 64-instance batched line")
    ap.add_argument("--no-large", dest="large", action="store_false",
                    help="skip the 36^3, nwt=300 line")
    ap.add_argument("--profile-workload", default="headline",
                    choices=["headline", "large", "c1q20"],
                    help="state that --profile-iteration prepares: the headline 24^3 "
                         "workload, the 36^3 nwt=300 one, or the 10^3 Q20-constrained start")
    ap.add_argument("--profile-iteration", action="store_true",
                    help="run one iteration of --precision between profiler start/stop "
                         "(for ncu --profile-from-start off) and exit")
    args = ap.parse_args()
    if args.profile_iteration:
        import __graft_entry__
        __graft_entry__.build()
        profile_iteration(args.precision, args.profile_workload)
        print("profiled one iteration")
        return
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        res = run_reference(args, rank, world)
    else:
        import __graft_entry__
        __graft_entry__.build()
        if world > 1:
            import torch
            torch.distributed.init_process_group("nccl")
        res = run_ours(args, rank, world, local_rank)
        if world > 1:
            import torch
            torch.distributed.destroy_process_group()
    if res is not None and rank == 0:
        print(json.dumps(res))


if __name__ == "__main__":
    main()
