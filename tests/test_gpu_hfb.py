"""GPU parity of the HFB pairing step against the CPU oracle.

The oracle follows the reference's damped Broyden Fermi solver and its
EISPACK-style eigensolver; the GPU uses a Newton root finder (analytic
dN/dlambda) and its batched Jacobi + refinement eigensolver.  Both stop at |N - N0| < 1e-12, so the converged states
agree to ~1e-12: rho, kappa, Delta and the pairing field are compared
norm-wise at 1e-10, the canonical densities at 1e-10, energies at 1e-8 MeV.
rho and kappa are projector blocks of the positive quasiparticle space and
so do not depend on eigenvector signs or degenerate rotations.
"""
import numpy as np
import pytest

import oracle as O
from conftest import rel
from mocca_gb300 import SLY4, RunParams, _abi, synthetic
from mocca_gb300.mesh import MeshState

pytestmark = pytest.mark.gpu


def _hfb_pair(n=10, nwt=40, N=12, Z=12, seed=1234):
    p = RunParams(nx=n, ny=n, nz=n, dx=0.8, nwt=nwt, neutrons=N, protons=Z,
                  pairing=_abi.MG_PAIRING_HFB)
    psi, qn, en = synthetic.ho_basis(p, nwt // 2, seed=seed)
    g = MeshState(p, SLY4)
    o = O.OracleState(p, SLY4)
    for s in (g, o):
        s.set_spinors(psi, qn)
        s.set_energies(en)
        s.set_pairing()
    return p, g, o


def test_hfb_start(built):
    p, g, o = _hfb_pair()
    ig = g.SolvePairing()
    io = o.SolvePairing()
    assert ig["converged"] and io["converged"]
    for it in range(2):
        assert abs(ig["particles"][it] - (p.neutrons, p.protons)[it]) < 1e-11
        assert abs(ig["fermi"][it] - io["fermi"][it]) < 1e-9
        assert abs(ig["pairing_energy"][it] - io["pairing_energy"][it]) < 1e-9
    fg, fo = g.get_pairing_field(), o.get_pairing_field()
    assert rel(fg[0], fo[0]) < 1e-12
    assert np.abs(fg[1] - fo[1]).max() <= 1e-12 * np.abs(fo[0]).max()
    for b in range(4):
        rg, kg, dg = g.get_hfb_block(b)
        ro, ko, do = o.get_hfb_block(b)
        assert rel(dg, do) < 1e-11, b
        assert rel(rg, ro) < 1e-10, b
        assert rel(kg, ko) < 1e-10, b
    og = np.sort(g.get_occupations(_abi.MG_CAN_BASIS))
    oo = np.sort(o.get_occupations(_abi.MG_CAN_BASIS))
    assert np.allclose(og, oo, atol=1e-10, rtol=0)
    assert abs(og.sum() - (p.neutrons + p.protons)) < 1e-9
    g.close()


def test_hfb_start_densities_energy(built):
    p, g, o = _hfb_pair()
    g.Start()
    o.Start()
    dg, do = g.get_densities(), o.get_densities()
    for k in dg:
        assert rel(dg[k], do[k]) < 1e-10, k
    eg, eo = g.CompEnergy(), o.CompEnergy()
    assert abs(eg["total"] - eo["total"]) < 1e-8
    assert abs(sum(eg["pairing"]) - sum(eo["pairing"])) < 1e-8
    g.close()


def test_hfb_iterations(built):
    p, g, o = _hfb_pair(seed=5)
    g.Start()
    o.Start()
    eg = g.Evolve(4, 0.010, 0.3)
    eo = o.Evolve(4, 0.010, 0.3)
    assert abs(eg["total"] - eo["total"]) < 1e-8, (eg["total"], eo["total"])
    assert abs(sum(eg["pairing"]) - sum(eo["pairing"])) < 1e-8
    g.close()


def test_hfb_iterations_first_order_finish(built):
    """Iterations long enough for the Fermi search to finish its last Newton
    step to first order (steps of at most 2e-7 MeV: rho and kappa move along
    d rho / d lambda, d kappa / d lambda of the last evaluation) against the
    oracle, whose Broyden search evaluates every step: 1e-8 MeV."""
    p, g, o = _hfb_pair(seed=5)
    g.Start()
    o.Start()
    pre, window = 30, 15
    g.Evolve(pre, 0.010, 0.3)
    used = 0
    for _ in range(window):   # the steps of mg_iterate, one by one
        g.GradDesc(0.010, 0.3)
        used += g.SolvePairing()["first_order"]
        g.DeriveAll()
        g.lib.mg_hpsi(g.h, 1, None, None, None)
        g.UpdateDensities()
        g.MixDensities()
        g.CalculateAllMoments()
        g.ConstructPotentials()
    eg = g.CompEnergy()
    eo = o.Evolve(pre + window, 0.010, 0.3)
    assert used > 0
    assert abs(eg["total"] - eo["total"]) < 1e-8, (eg["total"], eo["total"])
    assert abs(sum(eg["pairing"]) - sum(eo["pairing"])) < 1e-8
    g.close()


def test_bisection_fermi_solver(built):
    """FermiSolver 'BISECTION' (fermi_solver = 3: bracketing by growing
    steps from the stored Fermi energies, then Brent's method to fermi_prec
    on lambda) against the oracle's restatement: Fermi energies within 1e-9
    MeV at the first pairing step (from the module's -10 MeV start, tens of
    bracketing evaluations) and the energies of 4 iterations within 1e-8
    MeV; its root is the Newton search's within 1e-9 MeV."""
    p, g, o = _hfb_pair(seed=5)
    pp = _abi.MgPairingParams.defaults()
    pp.fermi_solver = 3
    g.set_pairing(pp)
    o.set_pairing(pp)
    ig, io = g.SolvePairing(), o.SolvePairing()
    assert ig["converged"] and io["converged"]
    assert ig["evaluations"] > 10
    for it in range(2):
        assert abs(ig["fermi"][it] - io["fermi"][it]) < 1e-9, (ig["fermi"], io["fermi"])
        assert abs(ig["particles"][it] - (p.neutrons, p.protons)[it]) < 1e-9
    _, n, _ = _hfb_pair(seed=5)
    inew = n.SolvePairing()
    for it in range(2):
        assert abs(ig["fermi"][it] - inew["fermi"][it]) < 1e-9
    n.close()
    g.Start()
    o.Start()
    eg = g.Evolve(4, 0.010, 0.3)
    eo = o.Evolve(4, 0.010, 0.3)
    assert abs(eg["total"] - eo["total"]) < 1e-8, (eg["total"], eo["total"])
    g.close()
    o.close()


def test_unknown_fermi_solver_is_rejected(built):
    p = RunParams(nx=10, ny=10, nz=10, dx=0.8, nwt=40, neutrons=12, protons=12,
                  pairing=_abi.MG_PAIRING_HFB)
    g = MeshState(p, SLY4)
    pp = _abi.MgPairingParams.defaults()
    pp.fermi_solver = 4
    with pytest.raises(_abi.MgError):
        g.set_pairing(pp)
    pp.fermi_solver = 1
    g.set_pairing(pp)
    g.close()


def test_phase_timer_and_side_derive(built):
    """mg_set_phase_timing / mg_get_phase_times over HFB passes: every phase
    of the pass is timed, the side-stream HF DeriveAll too, and the timed
    passes land on the same energies as untimed ones (the timer only records
    events); the HF-basis derivatives forked inside the pairing step equal
    a DeriveAll of the same spinors afterwards."""
    p, g, o = _hfb_pair()
    o.close()
    g.Start()
    ref = MeshState(p, SLY4)
    psi, qn, en = synthetic.ho_basis(p, p.nwt // 2, seed=1234)
    ref.set_spinors(psi, qn)
    ref.set_energies(en)
    ref.set_pairing()
    ref.Start()
    g.set_phase_timing(True)
    e1 = g.Evolve(3, 0.01, 0.3)["total"]
    t = g.phase_times()
    e0 = ref.Evolve(3, 0.01, 0.3)["total"]
    assert e1 == e0
    assert t["passes"] == 3
    for k in g.PHASES:
        if k != "moments":
            assert t[k] > 0.0, (k, t)
    d_side = g.get_derivatives(_abi.MG_HF_BASIS)
    g.DeriveAll()
    d_again = g.get_derivatives(_abi.MG_HF_BASIS)
    for a, b in zip(d_side, d_again):
        assert np.array_equal(a, b)
    g.set_phase_timing(False)
    g.Evolve(1, 0.01, 0.3)
    assert g.phase_times()["passes"] == 0
    g.close()
    ref.close()
