"""SymmetryOperators (mg_symmetry_operators) on the GPU against the oracle:
the EV8 box (quantum numbers and RMS radii of a 10^3 HO basis) and the
symmetry-free box (the expectation values of the mirror actions of
Gaussian x Hermite spinors on 16^3), within 1e-12."""
import numpy as np
import pytest

import oracle as O
from mocca_gb300 import SLY4, RunParams, synthetic
from mocca_gb300.mesh import MeshState

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("full", [False, True])
def test_symmetry_operators_against_oracle(built, full):
    if full:
        p = RunParams(nx=16, ny=16, nz=16, dx=0.8, pc=0, sc=0, tsc=0, trc=1, nwt=24,
                      neutrons=8, protons=8, coulomb_solver=0)
        psi = synthetic.gaussian_hermite_spinors(p, p.nwt, seed=42)
        qn = np.tile(np.array([-1, 0, 0, 0], dtype=np.int32), (p.nwt, 1))
        qn[p.nwt // 2:, 0] = 1
    else:
        p = RunParams(nx=10, ny=10, nz=10, dx=0.8, nwt=40, neutrons=12, protons=12)
        psi, qn, _ = synthetic.ho_basis(p, 20, seed=1234)
    g, o = MeshState(p, SLY4), O.OracleState(p, SLY4)
    for s in (g, o):
        s.set_spinors(psi, qn)
    sg, so = g.SymmetryOperators(), o.SymmetryOperators()
    assert np.abs(sg - so).max() <= 1e-12, np.abs(sg - so).max()
    if full:
        assert np.abs(so[:, 1:5]).max() > 1e-3   # computed, not quantum numbers
    g.close()
    o.close()
