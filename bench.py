"""Benchmark of the MOCCa mesh hot path on GB300.

Workload (the 24^3 configuration the headline metric is quoted on): N=Z=28,
24^3 stored EV8 mesh (48^3 full box), dx=0.8 fm, nwt=160 spinors (80 n +
80 p), SLy4, time-reversal invariant, seeded harmonic-oscillator start.  A
step is one pass of the Evolve loop body (src/Main.f90:255-328): GradDesc
with Gram-Schmidt, the pairing step, DeriveAll, densities, moments,
potentials with the Coulomb CG, energy.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--precision fp64|mixed] [--breakdown]

One JSON line on rank 0.  `value` times K steps with every input resident in
HBM (CUDA events on the library's stream, barrier + synchronize on both
sides, max over ranks); `e2e` times the same steps through the C ABI with
the spinors uploaded from pinned host memory and the spinors plus the
energy read back every step.  The working set (spinors, derivatives,
updates: ~0.7 GB) is larger than the 129 MB L2, so no flush is needed
between steps.  Multi-GPU runs are independent replicas (weak scaling).
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

import numpy as np  # noqa: E402

WORKLOAD = dict(nx=24, ny=24, nz=24, dx=0.8, nwt=160, neutrons=28.0, protons=28.0)
DT, MOMENTUM = 0.010, 0.3
METRIC = "HFB iter/s at 24^3, nwt=160: mixed vs FP64 GPU at |dE|<=1e-5 MeV"


def _params(precision):
    from mocca_gb300 import MG_FP64, MG_MIXED, MG_PAIRING_HFB, RunParams
    return RunParams(**WORKLOAD, precision=MG_MIXED if precision == "mixed" else MG_FP64,
                     pairing=MG_PAIRING_HFB)


def _start_state(p, seed):
    from mocca_gb300 import synthetic
    return synthetic.ho_basis(p, p.nwt // 2, seed=seed)


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
                 "--format=csv,noheader,nounits", "-lms", "200"],
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


def measured_peaks():
    try:
        return json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
    except Exception:
        return {}


def fp64_dgemm_peak(torch):
    """Measured FP64 throughput of a cuBLAS DGEMM (denominator for the FP64 kernels)."""
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


def cpu_baseline(sample_steps=1):
    """The FP64 oracle (single-threaded C++ port) on a bounded sample of the workload."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle as O
    from mocca_gb300 import SLY4
    p = _params("fp64")
    psi, qn, en = _start_state(p, 1234)
    o = O.OracleState(p, SLY4)
    o.set_spinors(psi, qn)
    o.set_energies(en)
    o.set_pairing()
    o.Start()
    t = time.perf_counter()
    o.Evolve(sample_steps, DT, MOMENTUM)
    dt = time.perf_counter() - t
    o.close()
    return {"value": sample_steps / dt, "unit": "iter/s", "cores": 1, "kind": "port",
            "sample": f"{sample_steps} HFB iteration(s) of the full 24^3 nwt=160 workload, "
                      f"oracle (C++ FP64 restatement, 1 thread), {dt:.1f} s"}


def run_reference(args, rank, world):
    """--impl reference: the reference's CPU path (oracle port; Fortran build unavailable)."""
    if rank != 0:
        return None
    steps = max(1, args.steps)
    warm = max(0, min(args.warmup, 1))
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle as O
    from mocca_gb300 import SLY4
    p = _params("fp64")
    psi, qn, en = _start_state(p, 1234)
    o = O.OracleState(p, SLY4)
    o.set_spinors(psi, qn)
    o.set_energies(en)
    o.set_pairing()
    o.Start()
    if warm:
        o.Evolve(warm, DT, MOMENTUM)
    per_step = 1  # one full iteration per step keeps K steps within minutes
    t = time.perf_counter()
    o.Evolve(steps * per_step, DT, MOMENTUM)
    dt = time.perf_counter() - t
    val = steps * per_step / dt
    return {
        "metric": METRIC, "value": val, "unit": "iter/s", "impl": "reference",
        "n_gpus": world, "steps": steps, "warmup": warm, "ms_per_step": dt / steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": {"workload": "Mg-like HO start, N=Z=28, 24^3 EV8, "
                                        "nwt=160, SLy4, HFB (G=1250, alpha=1)", **WORKLOAD},
        "cpu_baseline": {"value": val, "unit": "iter/s", "cores": 1, "kind": "port",
                         "sample": f"{steps} full iteration(s); the reference is single-threaded "
                                   "Fortran (no OpenMP) and no Fortran compiler exists here or on "
                                   "the GPU host, so its C++ FP64 restatement is timed"},
        "e2e": {"value": val, "unit": "iter/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def run_ours(args, rank, world, local_rank):
    import torch
    from mocca_gb300 import SLY4, _abi
    from mocca_gb300.mesh import MeshState

    torch.cuda.set_device(local_rank)
    stream = torch.cuda.Stream()
    p = _params(args.precision)
    psi, qn, en = _start_state(p, 1234 + rank)
    with torch.cuda.stream(stream):
        g = MeshState(p, SLY4, stream=stream.cuda_stream)
    g.set_spinors(psi, qn)
    g.set_energies(en)
    g.set_pairing()
    g.Start()
    g.Evolve(max(3, args.warmup), DT, MOMENTUM)
    torch.cuda.synchronize()
    dist = world > 1

    def barrier():
        if dist:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    def launches():
        n = C.c_longlong(0)
        g.lib.mg_launch_count(g.h, C.byref(n))
        return n.value

    # ---- device-resident throughput --------------------------------------------------
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    l0 = launches()
    with ClockSampler(local_rank) as clk:
        ev0.record(stream)
        last = g.Evolve(args.steps, DT, MOMENTUM)
        ev1.record(stream)
        barrier()
    l1 = launches()
    t_dev = ev0.elapsed_time(ev1) / 1e3
    if dist:
        t = torch.tensor([t_dev], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        t_dev = float(t.item())

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
    t_e2e = time.perf_counter() - t0
    if dist:
        t = torch.tensor([t_e2e], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        t_e2e = float(t.item())

    # ---- dominant kernel: the Lagrange derivative kernels of DeriveAll ------------------
    reps = 5
    k0, k1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    k0.record(stream)
    for _ in range(reps):
        g.DeriveBasis(0)
    k1.record(stream)
    torch.cuda.synchronize()
    t_der = k0.elapsed_time(k1) / 1e3 / reps
    n_line = p.nx  # line length
    flops = 48.0 * n_line * p.V * p.nwt          # 4 comps x 6 line-GEMMs x 2 n flops per point
    bytes_ = 160.0 * p.V * p.nwt                 # psi in + 3 der + lap out, FP64

    breakdown = None
    if args.breakdown:
        breakdown = stage_breakdown(g, torch, stream)

    if rank != 0:
        g.close()
        return None
    peaks = measured_peaks()
    hbm = peaks.get("hbm_gbs", 6800.0)
    fp64_peak = fp64_dgemm_peak(torch)
    res = {
        "metric": METRIC,
        "value": world * args.steps / t_dev,
        "unit": "iter/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t_dev / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if args.precision == "fp64" else "f64+tf32",
        "data": "synthetic",
        "config": {"workload": "N=Z=28 HO start (seed 1234), 24^3 EV8 stored mesh, dx=0.8, "
                               "nwt=160, SLy4, TRC, HFB pairing G=1250 alpha=1 "
                               "(surface delta, 5 MeV cutoff)",
                   **WORKLOAD, "precision": args.precision, "dt": DT, "momentum": MOMENTUM,
                   "l2": "working set ~0.7 GB > 129 MB L2, no flush",
                   "parallelism": f"replicas x{world}"},
        "e2e": {"value": world * args.steps / t_e2e, "unit": "iter/s",
                "h2d_bytes_per_step": int(host_psi.numel() * 8),
                "d2h_bytes_per_step": int(out_psi.numel() * 8 + C.sizeof(e_terms))},
        "roofline": {"kernel": "k_deriv_xy + k_deriv_z (DeriveAll, HF basis)",
                     "bound": "hbm", "achieved": bytes_ / t_der / 1e9, "peak": hbm,
                     "unit": "GB/s", "frac": bytes_ / t_der / 1e9 / hbm,
                     "traffic": None,
                     "fp64": {"achieved_tflops": flops / t_der / 1e12,
                              "peak_tflops_dgemm": fp64_peak,
                              "frac": flops / t_der / 1e12 / fp64_peak},
                     "ms_per_launch_pair": t_der * 1e3},
        "cpu_baseline": cpu_baseline(1) if world == 1 or rank == 0 else None,
        "clocks": clk.summary(),
        "gpu_launches": int(l1 - l0),
        "energy_last": last["total"],
    }
    if breakdown:
        res["breakdown_ms"] = breakdown
    g.close()
    return res


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


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"])
    ap.add_argument("--breakdown", action="store_true")
    args = ap.parse_args()
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
