"""GPU parity of the FP64 path against the CPU oracle, through the C ABI.

Tolerances of the plain FP64 form: h.psi and densities within 1e-12
relative (norm-wise), total energy within 1e-8 MeV after a fixed number of
iterations.  Derivatives, potentials and Gram-Schmidt use the same 1e-12
norm-wise bar; single-particle energies 1e-9 MeV.
"""
import json
from pathlib import Path

import numpy as np
import pytest

import oracle as O
from conftest import rel
from mocca_gb300 import SLY4, RunParams, synthetic
from mocca_gb300.mesh import MeshState

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"


def _pair(p, psi, qn, en):
    g = MeshState(p, SLY4)
    o = O.OracleState(p, SLY4)
    for s in (g, o):
        s.set_spinors(psi, qn)
        s.set_energies(en)
    return g, o


def _mg24(n=10, nwt=40, seed=1234):
    p = RunParams(nx=n, ny=n, nz=n, dx=0.8, nwt=nwt, neutrons=12, protons=12)
    return (p, *synthetic.ho_basis(p, nwt // 2, seed=seed))


@pytest.fixture(scope="module")
def mg24(built):
    return _mg24()


def test_derivatives_ev8(mg24):
    p, psi, qn, en = mg24
    g, o = _pair(p, psi, qn, en)
    g.DeriveAll()
    o.DeriveAll()
    dg, lg = g.get_derivatives()
    do, lo = o.get_derivatives()
    assert rel(dg, do) < 1e-12
    assert rel(lg, lo) < 1e-12
    g.close()


@pytest.mark.parametrize("n,nwt", [(12, 8), (24, 8)])
def test_derivatives_ev8_sizes(built, n, nwt):
    p, psi, qn, en = _mg24(n=n, nwt=nwt, seed=7)
    g, o = _pair(p, psi, qn, en)
    g.DeriveAll()
    o.DeriveAll()
    dg, lg = g.get_derivatives()
    do, lo = o.get_derivatives()
    assert rel(dg, do) < 1e-12 and rel(lg, lo) < 1e-12
    g.close()


def test_derivatives_and_hpsi_full_box(built):
    """Symmetry-free box with unfolded Lagrange matrices and Woods-Saxon fields."""
    p = RunParams(nx=12, ny=12, nz=12, dx=0.8, pc=0, sc=0, tsc=0, trc=1, nwt=6,
                  neutrons=8, protons=8, coulomb_solver=0)
    psi = synthetic.gaussian_hermite_spinors(p, p.nwt, seed=42)
    qn = np.tile(np.array([-1, 0, 0, 0], dtype=np.int32), (p.nwt, 1))
    qn[3:, 0] = 1
    g, o = _pair(p, psi, qn, np.zeros(p.nwt))
    U, B, nB, W, dW = synthetic.woods_saxon_fields(p)
    for s in (g, o):
        s.set_potentials(U=U, B=B, nablaB=nB, W=W, divW=dW)
        s.DeriveAll()
    dg, lg = g.get_derivatives()
    do, lo = o.get_derivatives()
    assert rel(dg, do) < 1e-12 and rel(lg, lo) < 1e-12
    hg, eg, sg = g.hPsi()
    ho, eo, so = o.hPsi()
    assert rel(hg, ho) < 1e-12
    assert np.allclose(eg, eo, rtol=0, atol=1e-9)
    g.close()


def test_start_densities_potentials_energy(mg24):
    p, psi, qn, en = mg24
    g, o = _pair(p, psi, qn, en)
    itg = g.Start()
    ito = o.Start()
    assert abs(itg - ito) <= 1
    assert np.array_equal(g.get_occupations(), o.get_occupations())
    dg, do = g.get_densities(), o.get_densities()
    for k in dg:
        assert rel(dg[k], do[k]) < 1e-12, k
    pg, po = g.get_potentials(), o.get_potentials()
    for k in ("U", "B", "nablaB", "W", "coulomb", "coulex"):
        assert rel(pg[k], po[k]) < 1e-11, k
    # div W is analytically zero for the B9 term: compare on the scale of W's derivatives
    assert np.abs(pg["divW"] - po["divW"]).max() < 1e-9
    eg, eo = g.CompEnergy(), o.CompEnergy()
    assert abs(eg["total"] - eo["total"]) < 1e-8
    assert abs(eg["coulomb"] - eo["coulomb"]) < 1e-8
    hg, e1, d1 = g.hPsi()
    ho, e2, d2 = o.hPsi()
    assert rel(hg, ho) < 1e-12
    assert np.allclose(e1, e2, rtol=0, atol=1e-9)
    g.close()


def test_gram_schmidt(mg24):
    p, psi, qn, en = mg24
    rng = np.random.default_rng(11)
    pert = psi + 0.02 * rng.normal(size=psi.shape)
    g, o = _pair(p, pert, qn, en + rng.normal(size=en.shape))
    g.GramSchmidt()
    o.GramSchmidt()
    qg, qo = g.get_spinors(), o.get_spinors()
    assert rel(qg, qo) < 1e-12
    q = qg.reshape(p.nwt, -1)
    S = q @ q.T * p.dv
    same = (qn[:, None, 0] == qn[None, :, 0]) & (qn[:, None, 1] == qn[None, :, 1])
    assert np.abs(S[same] - np.eye(p.nwt)[same]).max() < 1e-13
    g.close()


def test_hf_iterations_match_golden(mg24):
    """E_total after a fixed number of GradDesc + HF iterations: 1e-8 MeV."""
    gold = json.loads((GOLDEN / "mg24_hf.json").read_text())
    p, psi, qn, en = mg24
    g = MeshState(p, SLY4)
    g.set_spinors(psi, qn)
    g.set_energies(en)
    g.Start()
    assert abs(g.CompEnergy()["total"] - gold["E_start"]) < 1e-8
    e = g.Evolve(gold["iterations"], gold["dt"], gold["momentum"])
    assert abs(e["total"] - gold["E_final"]) < 1e-8, (e["total"], gold["E_final"])
    sp, _ = g.get_energies()
    assert np.allclose(sp, gold["sp_energies"], atol=1e-8, rtol=0)
    g.close()


def test_hf_iterations_match_oracle_24(built):
    """A few iterations at the 24^3 mesh with 40 spwfs against the oracle."""
    p = RunParams(nx=24, ny=24, nz=24, dx=0.8, nwt=40, neutrons=12, protons=12)
    psi, qn, en = synthetic.ho_basis(p, 20, seed=99)
    g, o = _pair(p, psi, qn, en)
    g.Start()
    o.Start()
    eg = g.Evolve(2, 0.010, 0.3)["total"]
    eo = o.Evolve(2, 0.010, 0.3)["total"]
    assert abs(eg - eo) < 1e-8, (eg, eo)
    g.close()


@pytest.mark.parametrize("precon_w", [0.0, 1.0])
def test_hf_iterations_precondition_scheme2(built, precon_w):
    """MixingScheme 2 (PreconditionPotential on the U update; with PreConW >
    0 on each W component's too) on the GPU against the oracle: 4
    iterations, E_total within 1e-8 MeV, U and W within 1e-10."""
    p = RunParams(nx=10, ny=10, nz=10, dx=0.8, nwt=40, neutrons=12, protons=12,
                  mixing_scheme=2, precon_w=precon_w)
    psi, qn, en = synthetic.ho_basis(p, 20, seed=1234)
    g, o = _pair(p, psi, qn, en)
    g.Start()
    o.Start()
    eg = g.Evolve(4, 0.010, 0.3)
    eo = o.Evolve(4, 0.010, 0.3)
    assert abs(eg["total"] - eo["total"]) < 1e-8, (eg["total"], eo["total"])
    pg, po = g.get_potentials(), o.get_potentials()
    assert rel(pg["U"], po["U"]) < 1e-10
    assert rel(pg["W"], po["W"]) < 1e-10
    g.close()
