"""HFB blocks above 128 (the eigensolver's extended range, up to 160) inside
the pairing step: N=Z=40 on a 16^3 EV8 mesh with nwt=280 from the HO start
puts 70 spwfs in every (isospin, parity) block, N = 140.  At h = 70 > 64 the
mixed form also leaves the tensor-core pairing and Gram-Schmidt kernels for
their double-float / FP64 counterparts.  FP64 against the oracle through the
start and one iteration (rho, kappa and Delta of every block, 1e-9 at the
start; energies, 1e-7 MeV at the start and 1e-6 MeV after one iteration);
mixed iterations with an FP64 polish against the FP64 GPU path (1e-5 MeV).

From this start (HO energies, GuessKappa) the reference's Broyden Fermi
search stops at its cap short of the particle number; the GPU side runs
that same search (fermi_solver = 1) so that both follow its iterates.  The
start is ill-posed for any Fermi search: 40 particles per isospin in blocks
of 70 stored states leave whole degenerate HO shells unpaired (outside the
pairing window), and where such a shell crosses the Fermi energy N(lambda)
jumps (from 39.2 to 69.2 at lambda = 2.33 MeV for the neutrons, with the
window of the default start).  Searches that stop short of N0 on such a
function amplify rounding-level differences of N(lambda), which is why the
energy bars here are 1e-7 MeV at the start and 1e-6 MeV after one
iteration; on the regular benchmark starts the FP64 path meets 1e-8 MeV
(test_gpu_bench_configs.py)."""
import numpy as np
import pytest

import oracle as O
from conftest import rel
from mocca_gb300 import MG_FP64, MG_MIXED, SLY4, RunParams, _abi, synthetic
from mocca_gb300.mesh import MeshState

pytestmark = pytest.mark.gpu


def _params(precision=MG_FP64):
    return RunParams(nx=16, ny=16, nz=16, dx=0.8, nwt=280, neutrons=40, protons=40,
                     pairing=_abi.MG_PAIRING_HFB, precision=precision)


def _start(s, psi, qn, en, solver=0):
    pp = _abi.MgPairingParams.defaults()
    pp.fermi_solver = solver
    s.set_spinors(psi, qn)
    s.set_energies(en)
    s.set_pairing(pp)
    s.Start()


def test_large_blocks_fp64_against_oracle(built):
    p = _params()
    psi, qn, en = synthetic.ho_basis(p, 140, seed=21)
    g, o = MeshState(p, SLY4), O.OracleState(p, SLY4)
    for s in (g, o):
        _start(s, psi, qn, en, solver=1)
    assert g.get_hfb_block(0)[0].shape == (140, 140)
    for b in range(4):
        rg, kg, dg = g.get_hfb_block(b)
        ro, ko, do = o.get_hfb_block(b)
        assert rel(dg, do) < 1e-12, b
        assert rel(rg, ro) < 1e-9, b
        assert rel(kg, ko) < 1e-9, b
    ds = abs(g.CompEnergy()["total"] - o.CompEnergy()["total"])
    eg = g.Evolve(1, 0.010, 0.3)
    eo = o.Evolve(1, 0.010, 0.3)
    de = abs(eg["total"] - eo["total"])
    # the unconverged searches amplify rounding-level differences (measured:
    # 2e-8 MeV at the start, 1.1e-7 MeV after one iteration)
    assert ds < 1e-7 and de < 1e-6, (ds, de)
    for b in range(4):
        rg, kg, dg = g.get_hfb_block(b)
        ro, ko, do = o.get_hfb_block(b)
        assert rel(dg, do) < 1e-7, b
        assert rel(rg, ro) < 1e-6, b
    g.close()


def test_large_blocks_mixed_with_polish(built):
    psi, qn, en = synthetic.ho_basis(_params(), 140, seed=21)
    ref = MeshState(_params(MG_FP64), SLY4)
    _start(ref, psi, qn, en)
    e_ref = ref.Evolve(15, 0.010, 0.3)["total"]
    mix = MeshState(_params(MG_MIXED), SLY4)
    _start(mix, psi, qn, en)
    mix.Evolve(10, 0.010, 0.3)
    mix.set_precision(MG_FP64)
    e_mix = mix.Evolve(5, 0.010, 0.3)["total"]
    assert np.isfinite(e_mix)
    assert abs(e_mix - e_ref) <= 1e-5, (e_mix, e_ref)
    ref.close()
    mix.close()
