"""ParameterEstimation = 1 on the GPU against the oracle.

IterativeEstimation (src/ImaginaryTime.f90:28-211) runs a gradient ascent of
one extra spwf (maxspwf) from a fixed-seed start before every GradDesc and
sets dt and the momentum from its largest-eigenvalue estimate and the
spectrum's smallest gap (HF) or quasiparticle energy (HFB).  The GPU and the
oracle start from the same splitmix64 stream, so their estimates and the
iterations that use them agree to FP64 rounding.
"""
import numpy as np
import pytest

import oracle as O
from mocca_gb300 import SLY4, RunParams, _abi, synthetic
from mocca_gb300.mesh import MeshState

pytestmark = pytest.mark.gpu


def _pair(p, seed, hfb):
    psi, qn, en = synthetic.ho_basis(p, p.nwt // 2, seed=seed)
    g = MeshState(p, SLY4)
    o = O.OracleState(p, SLY4)
    for s in (g, o):
        s.set_spinors(psi, qn)
        s.set_energies(en)
        if hfb:
            s.set_pairing()
    return g, o


@pytest.mark.parametrize("n,pairing,precision", [
    (10, _abi.MG_PAIRING_HF, _abi.MG_FP64),
    (10, _abi.MG_PAIRING_HFB, _abi.MG_FP64),
    (10, _abi.MG_PAIRING_HFB, _abi.MG_MIXED),
    (24, _abi.MG_PAIRING_HF, _abi.MG_FP64),
])
def test_estimated_step_parameters_match_oracle(built, n, pairing, precision):
    """dt and momentum after each of 3 iterations within 1e-9 (relative) of
    the oracle's, and E_total within 1e-8 MeV (1e-7 MeV with the
    tensor-core paths, whose rounding moves the estimate's stopping step by
    at most one)."""
    p = RunParams(nx=n, ny=n, nz=n, dx=0.8, nwt=40, neutrons=12, protons=12,
                  pairing=pairing, precision=precision, parameter_estimation=1)
    hfb = pairing == _abi.MG_PAIRING_HFB
    g, o = _pair(p, seed=7, hfb=hfb)
    g.Start()
    o.Start()
    for _ in range(3):
        eg = g.Evolve(1, 0.010, 0.3)
        eo = o.Evolve(1, 0.010, 0.3)
        dg, mg = g.StepParameters()
        do, mo = o.StepParameters()
        assert dg == pytest.approx(do, rel=1e-9, abs=0), (dg, do)
        assert mg == pytest.approx(mo, rel=1e-9, abs=0), (mg, mo)
    tol = 1e-8 if precision == _abi.MG_FP64 else 1e-7
    assert abs(eg["total"] - eo["total"]) < tol, (eg["total"], eo["total"])
    assert 0.0 < mg < 1.0 and dg > 0.0
    g.close()


def test_fixed_step_parameters_are_reported(built):
    """With ParameterEstimation = 0 the step parameters are the caller's."""
    p = RunParams(nx=10, ny=10, nz=10, dx=0.8, nwt=40, neutrons=12, protons=12)
    g, _ = _pair(p, seed=7, hfb=False)
    g.Start()
    g.Evolve(1, 0.0125, 0.25)
    assert g.StepParameters() == (0.0125, 0.25)
    g.close()
