"""The J^2 (tensor) terms of the functional on the GPU against the oracle:
SLy5colo (tensor te = 296, to = -136 MeV fm^5, J2Terms), time reversal
conserved.

Both sides compute, from the same spinors, the tensor density J_{mu nu}
(GetJMuNu), the spin-orbit field W with its J^2 parts and div W
(CalcWPot), h.psi and the energy with the J^2 terms 19, 20, 23-26 of
compSkyrme.  Bars as the FP64 parity tests: J_{mu nu}, W, div W and h.psi
within 1e-12 norm-wise at the start (U 1e-11 with the Coulomb solve), the
J^2 energy terms within 1e-10 relative, the total energy within 1e-8 MeV at
the start and after 4 iterations (HF and HFB), J_{mu nu} then within 1e-9;
the mixed form (20 mixed + 5 FP64 iterations) within 1e-6 MeV of 25 FP64
iterations.
"""
import numpy as np
import pytest

import oracle as O
import wf_format as WF
from conftest import rel
from mocca_gb300 import RunParams, _abi, synthetic
from mocca_gb300.forces import SLY5_TENSOR
from mocca_gb300.mesh import MeshState

pytestmark = pytest.mark.gpu


def _pair(pairing=_abi.MG_PAIRING_HF, seed=1234, precision=0):
    p = RunParams(nx=10, ny=10, nz=10, dx=0.8, nwt=40, neutrons=12, protons=12, pairing=pairing,
                  precision=precision)
    psi, qn, en = synthetic.ho_basis(p, 20, seed=seed)
    g = MeshState(p, SLY5_TENSOR)
    o = O.OracleState(p, SLY5_TENSOR)
    for s in (g, o):
        s.set_spinors(psi, qn)
        s.set_energies(en)
        if pairing == _abi.MG_PAIRING_HFB:
            s.set_pairing()
    return p, g, o


def test_tensor_start(built):
    p, g, o = _pair()
    g.Start()
    o.Start()
    jg, jo = g.get_jmunu(), o.get_jmunu()
    assert np.abs(jo).max() > 1e-5
    assert rel(jg, jo) < 1e-12
    pg, po = g.get_potentials(), o.get_potentials()
    for k in ("B", "W", "divW"):
        assert rel(pg[k], po[k]) < 1e-12, k
    assert rel(pg["U"], po["U"]) < 1e-11   # with the Coulomb solve, as the FP64 parity tests
    # the diagonal of W is the J^2 part alone (B9 makes W antisymmetric)
    W = pg["W"].reshape(2, 3, 3, -1)
    assert np.abs(W[:, [0, 1, 2], [0, 1, 2]]).max() > 1e-5
    hg, eg, _ = g.hPsi()
    ho, eo, _ = o.hPsi()
    assert rel(hg, ho) < 1e-12
    Eg, Eo = g.CompEnergy(), o.CompEnergy()
    for q in (18, 19, 22, 23, 24, 25):
        assert Eo["skyrme"][q] != 0.0, q
        assert abs(Eg["skyrme"][q] - Eo["skyrme"][q]) <= 1e-10 * abs(Eo["skyrme"][q]), q
    assert abs(Eg["total"] - Eo["total"]) < 1e-8
    g.close()


@pytest.mark.parametrize("pairing", [_abi.MG_PAIRING_HF, _abi.MG_PAIRING_HFB])
def test_tensor_iterations(built, pairing):
    p, g, o = _pair(pairing, seed=5)
    g.Start()
    o.Start()
    eg = g.Evolve(4, 0.010, 0.3)
    eo = o.Evolve(4, 0.010, 0.3)
    assert abs(eg["total"] - eo["total"]) < 1e-8, (eg["total"], eo["total"])
    # after 4 iterations the two trajectories carry their roundings (the
    # energy bar above is the parity bar of the iteration)
    assert rel(g.get_jmunu(), o.get_jmunu()) < 1e-9
    g.close()


def test_tensor_mixed_form(built):
    p, m, _ = _pair(precision=_abi.MG_MIXED, seed=7)
    _, f, _ = _pair(seed=7)
    for s in (m, f):
        s.Start()
    m.Evolve(20, 0.010, 0.3)
    m.set_precision(_abi.MG_FP64)
    em = m.Evolve(5, 0.010, 0.3)["total"]
    ef = f.Evolve(25, 0.010, 0.3)["total"]
    assert abs(em - ef) < 1e-6, (em, ef)
    m.close()
    f.close()


def test_tensor_density_in_wf(built, tmp_path):
    p, g, _ = _pair()
    g.Start()
    g.WriteMOCCa(tmp_path / "t.wf")
    w = WF.read_v1(tmp_path / "t.wf")
    assert w["has_jmunu"] == 1
    assert np.array_equal(w["jmunu"], g.get_jmunu())
    g.close()
