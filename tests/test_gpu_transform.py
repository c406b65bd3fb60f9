"""mg_break_symmetries: an EV8 state unfolded onto the symmetry-free box.

The unfolded grids equal the restatement of BreakParity, BreakSignature and
BreakTimeSimplex applied in TransformInput's order (oracle/transform.py)
bit for bit.  The unfolded state is the same state: on the full box (no
Coulomb on either side) its densities on the positive octant equal the EV8
densities, its single-particle energies and total energy the EV8 ones
(1e-10 relative: the full line's Lagrange matrices against the folded
ones, and eight octants summed against one).
"""
import numpy as np
import pytest

import transform as T
from conftest import rel
from mocca_gb300 import SLY4, RunParams, _abi, synthetic
from mocca_gb300.mesh import MeshState

pytestmark = pytest.mark.gpu


def test_unfolded_state(built):
    n, nwt = 8, 20
    p = RunParams(nx=n, ny=n, nz=n, dx=0.8, nwt=nwt, neutrons=6, protons=6, coulomb_solver=0)
    psi, qn, en = synthetic.ho_basis(p, nwt // 2, seed=3)
    a = MeshState(p, SLY4)
    a.set_spinors(psi, qn)
    a.set_energies(en)
    a.Start()
    a.Evolve(3, 0.010, 0.3)
    q = RunParams(nx=2 * n, ny=2 * n, nz=2 * n, dx=0.8, nwt=nwt, neutrons=6, protons=6,
                  pc=0, sc=0, tsc=0, trc=1, coulomb_solver=0)
    b = MeshState(q, SLY4)
    a.BreakSymmetries(b)
    pa, pb = a.get_spinors(), b.get_spinors()
    for i in range(nwt):
        assert np.array_equal(pb[i], T.break_all(pa[i], int(qn[i, 1]))), i
    assert np.array_equal(b.get_occupations(), a.get_occupations())
    assert np.array_equal(b.get_energies()[0], a.get_energies()[0])
    # the same state on both boxes
    for s in (a, b):
        s.DeriveAll()
        s.UpdateDensities()
        s.ConstructPotentials()
    da, db = a.get_densities(), b.get_densities()
    for k in ("rho", "tau", "nablaj"):
        fa = da[k].reshape(2, n, n, n)
        fb = db[k].reshape(2, 2 * n, 2 * n, 2 * n)[:, n:, n:, n:]
        assert rel(fb, fa) < 1e-12, k
    ea, eb = a.CompEnergy()["total"], b.CompEnergy()["total"]
    assert abs(ea - eb) < 1e-10 * abs(ea), (ea, eb)
    _, e1, _ = a.hPsi(want_spinors=False)
    _, e2, _ = b.hPsi(want_spinors=False)
    assert np.abs(e1 - e2).max() < 1e-10 * np.abs(e1).max()
    a.close()
    b.close()


def test_refuses_wrong_shapes(built):
    p = RunParams(nx=8, ny=8, nz=8, dx=0.8, nwt=4, neutrons=2, protons=2, coulomb_solver=0)
    psi, qn, en = synthetic.ho_basis(p, 2, seed=3)
    a = MeshState(p, SLY4)
    a.set_spinors(psi, qn)
    q = RunParams(nx=12, ny=16, nz=16, dx=0.8, nwt=4, neutrons=2, protons=2, pc=0, sc=0, tsc=0,
                  coulomb_solver=0)
    b = MeshState(q, SLY4)
    with pytest.raises(_abi.MgError):
        a.BreakSymmetries(b)
    a.close()
    b.close()
