"""The Evolve loop with its convergence exit (mg_evolve, ConvergenceCheck
src/Main.f90:358-397) on the GPU against the oracle: the HF Mg24 run with
ParameterEstimation 1 stops at the same iteration with the same energy."""
import pytest

import oracle as O
from mocca_gb300 import SLY4, RunParams, _abi, synthetic
from mocca_gb300.mesh import MeshState

pytestmark = pytest.mark.gpu


def test_evolve_stops_where_the_oracle_does(built):
    p = RunParams(nx=10, ny=10, nz=10, dx=0.8, nwt=40, neutrons=12, protons=12,
                  parameter_estimation=1)
    psi, qn, en = synthetic.ho_basis(p, 20, seed=1234)
    P = _abi.MgConvergence(1e-7, 1e-4, 1e-4)
    o = O.OracleState(p, SLY4)
    g = MeshState(p, SLY4)
    for s in (g, o):
        s.set_spinors(psi, qn)
        s.set_energies(en)
        s.Start()
    k = 0
    while k < 400:
        k += 1
        eo = o.Evolve(1, 0.010, 0.3)
        if o.ConvergenceCheck(P):
            break
    eg, n, conv = g.EvolveUntilConverged(400, 0.010, 0.3, P)
    assert conv and n == k, (n, k)
    assert abs(eg["total"] - eo["total"]) < 1e-8
    assert g.ConvergenceCheck(P)
    g.close()
