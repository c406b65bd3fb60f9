"""Regenerate the golden fixtures of tests/golden from the FP64 oracle.

The reference is Fortran and cannot be built in this container (no Fortran
compiler), so these fixtures are the oracle's own FP64 numbers on seeded
synthetic inputs: they pin the oracle against regressions and give the GPU
tests a reference that needs no oracle run.  Run from the repo root:
    python tests/golden/make_golden.py
"""
import json
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[2]
sys.path[:0] = [str(ROOT), str(ROOT / "oracle")]

import oracle as O  # noqa: E402
from mocca_gb300 import SLY4, RunParams, synthetic  # noqa: E402


def mg24_hf():
    p = RunParams(nx=10, ny=10, nz=10, dx=0.8, nwt=40, neutrons=12, protons=12)
    psi, qn, en = synthetic.ho_basis(p, 20, seed=1234)
    o = O.OracleState(p, SLY4)
    o.set_spinors(psi, qn)
    o.set_energies(en)
    o.Start()
    e0 = o.CompEnergy()
    n, dt, mom = 8, 0.010, 0.3
    e = o.Evolve(n, dt, mom)
    sp, disp = o.get_energies()
    return {
        "config": "Mg24 (N=Z=12), EV8+TRC, 10^3 stored mesh, dx=0.8, nwt=40, SLy4, HF filling, "
                  "HO start seed 1234 amplitude 1e-3, MixingScheme 0 (DampingParam 0.75)",
        "iterations": n, "dt": dt, "momentum": mom,
        "E_start": e0["total"], "E_final": e["total"],
        "kinetic_final": e["kinetic"], "coulomb_final": e["coulomb"],
        "sp_energies": sp.tolist(), "dispersions": disp.tolist(),
    }


C1_CHECKPOINTS = (1, 10, 11, 20, 50, 100)


def c1_state():
    """The Mg24 run of the reference README (the CPU-runnable configuration):
    10^3 stored EV8 mesh, dx=0.8, nwt=40 (20 n + 20 p) from the Nilsson
    guess plus a seeded uniform perturbation of 1e-3, SLy4, HFB (G=1250,
    alpha=1, GuessKappa), MixingScheme 2, ParameterEstimation 1, a Q20
    constraint of 50 fm^2 for the first 10 iterations."""
    from mocca_gb300 import _abi
    p = RunParams(nx=10, ny=10, nz=10, dx=0.8, nwt=40, neutrons=12, protons=12,
                  pairing=_abi.MG_PAIRING_HFB, mixing_scheme=2, parameter_estimation=1)
    psi, qn, en = synthetic.nilsson_basis(p, 20, seed=1234)
    return p, psi, qn, en


def mg24_c1():
    p, psi, qn, en = c1_state()
    o = O.OracleState(p, SLY4)
    o.set_spinors(psi, qn)
    o.set_energies(en)
    o.set_pairing()
    o.add_constraint(2, 0, 50.0, 0.0, 10)
    o.Start()
    rows = []
    for k in range(1, C1_CHECKPOINTS[-1] + 1):
        e = o.Evolve(1, 0.010, 0.3)
        if k in C1_CHECKPOINTS:
            dt, mom = o.StepParameters()
            rows.append({"iteration": k, "E_total": e["total"], "pairing": e["pairing"],
                         "q20": sum(o.get_constraint(0)["value"]), "dt": dt, "momentum": mom})
    return {
        "config": "Mg24 README run: N=Z=12, EV8+TRC, 10^3 stored mesh, dx=0.8, nwt=40, SLy4, "
                  "HFB G=1250 alpha=1 GuessKappa, Nilsson start (6 even + 5 odd shells, "
                  "m omega/hbar=0.2) + uniform perturbation 1e-3 seed 1234, MixingScheme 2, "
                  "ParameterEstimation 1 (dt 0.010, momentum 0.3 seed the estimation), "
                  "Q20 constraint 50 fm^2 for 10 iterations, 100 iterations",
        "checkpoints": rows,
    }


if __name__ == "__main__":
    here = Path(__file__).resolve().parent
    (here / "mg24_hf.json").write_text(json.dumps(mg24_hf(), indent=1))
    (here / "mg24_c1.json").write_text(json.dumps(mg24_c1(), indent=1))
    print(here)
