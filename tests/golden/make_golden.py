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


if __name__ == "__main__":
    out = Path(__file__).resolve().parent / "mg24_hf.json"
    out.write_text(json.dumps(mg24_hf(), indent=1))
    print(out)
