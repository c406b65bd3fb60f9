"""The FP64 GPU path against the oracle at the benchmark configurations.

- 24^3 EV8 mesh, nwt=160, N=Z=28, HFB (the headline workload, same HO start
  as the benchmark): the start and 5 iterations.
- 36^3 EV8 mesh, nwt=300, N=50, Z=40, HFB (the large-mesh workload): the
  start and 1 iteration.
- One Q20-constrained instance of the 64-instance uneven batch: the start
  and 5 iterations.

Both sides run the reference's Fermi search (damped Broyden,
fermi_solver = 1).  The Fermi energies start at the root of the first
pairing step, found by a probe context with the library's Newton search, so
that Broyden converges to FermiPrec in every step on both sides: from the
module default of -10 MeV it stops at its iteration cap in the first steps,
and an unconverged search amplifies rounding-level differences of N(lambda)
into ~1e-7 MeV.

Bars (the benchmark spec's): total energy within 1e-8 MeV at the start and after
every compared iteration.  h.psi and the densities within 1e-12, norm-wise
and pointwise (max |a - b| / max |b| over the whole field), computed by both
sides from the same inputs: the GPU state after the iterations (spinors,
occupations and potentials) is loaded into the oracle.  Along the
trajectories the densities are compared too, at the level the energy bar
implies (1e-9).
"""
import numpy as np
import pytest

import oracle as O
from conftest import rel
from mocca_gb300 import SLY4, RunParams, _abi, synthetic
from mocca_gb300.mesh import MeshState

pytestmark = pytest.mark.gpu
DT, MOM = 0.010, 0.3


def prel(a, b):
    """Pointwise relative difference: max |a - b| over max |b|."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    m = np.abs(b).max()
    return float(np.abs(a - b).max() / (m if m > 0 else 1.0))


def converging_pairing(p, psi, qn, en):
    """Pairing parameters with the reference's search started at a root of
    the first pairing step.  The root depends on the start through the
    pairing cutoffs (a window centred on the Fermi energy the step starts
    from), so probe contexts with the Newton search are run from their own
    result until the root reproduces itself.  On a start with degenerate
    unpaired shells the first probe can stop on a jump of N(lambda) (such a
    shell crossing the Fermi energy), where N0 is met only through an
    arbitrary split of zero-energy modes; the next probe, with the window
    moved there, leaves it."""
    def root(start):
        pp = _abi.MgPairingParams.defaults()
        pp.fermi_start[0], pp.fermi_start[1] = start
        probe = MeshState(p, SLY4)
        probe.set_spinors(psi, qn)
        probe.set_energies(en)
        probe.set_pairing(pp)
        info = probe.SolvePairing()
        probe.close()
        return np.array(info["fermi"]), info["converged"]

    # fixed-point steps lam <- root(lam), then a secant on root(lam) - lam
    # per isospin (the windows and particle numbers of the isospins are
    # independent)
    # (a probe whose search fails ends the iteration at the last good root)
    r, ok = root(np.array([-10.0, -10.0]))
    assert ok
    lam, best = r, r
    hist = []
    for k in range(30):
        r, ok = root(lam)
        if not ok:
            break
        best = r
        F = r - lam
        if np.abs(F).max() < 1e-9:
            break
        hist.append((lam.copy(), F))
        if k < 2:
            lam = r
        else:
            (l0, F0), (l1, F1) = hist[-2], hist[-1]
            den = np.where(F1 != F0, F1 - F0, 1.0)
            lam = np.where(F1 != F0, l1 - F1 * (l1 - l0) / den, r)
    lam = best
    pp = _abi.MgPairingParams.defaults()
    pp.fermi_solver = 1
    pp.fermi_start[0], pp.fermi_start[1] = lam
    return pp


def start_pair(p, psi, qn, en, constraint=None):
    pp = converging_pairing(p, psi, qn, en)
    g, o = MeshState(p, SLY4), O.OracleState(p, SLY4)
    for s in (g, o):
        s.set_spinors(psi, qn)
        s.set_energies(en)
        s.set_pairing(pp)
        if constraint is not None:
            s.add_constraint(*constraint)
        s.Start()
    return g, o


def compare_trajectory(g, o, iters, bar=1e-8):
    de = [abs(g.CompEnergy()["total"] - o.CompEnergy()["total"])]
    for _ in range(iters):
        eg = g.Evolve(1, DT, MOM)["total"]
        eo = o.Evolve(1, DT, MOM)["total"]
        de.append(abs(eg - eo))
    assert max(de) <= bar, de
    dg, do = g.get_densities(), o.get_densities()
    for k in ("rho", "tau", "nablaj"):
        assert rel(dg[k], do[k]) <= 1e-9, (k, rel(dg[k], do[k]))
    return de


def compare_kernels_same_inputs(g, o, p):
    """h.psi of the HF basis and the densities of the canonical basis from
    the GPU's current state, loaded into the oracle: 1e-12 norm-wise and
    pointwise."""
    qn = None
    o.set_spinors(g.get_spinors(_abi.MG_HF_BASIS), qn, _abi.MG_HF_BASIS)
    pot = g.get_potentials()
    o.set_potentials(**{k: pot[k] for k in ("U", "B", "nablaB", "W", "divW")})
    for s in (g, o):
        s.DeriveBasis(_abi.MG_HF_BASIS)
    hg, eg, _ = g.hPsi(_abi.MG_HF_BASIS)
    ho, eo, _ = o.hPsi(_abi.MG_HF_BASIS)
    assert rel(hg, ho) <= 1e-12 and prel(hg, ho) <= 1e-12, (rel(hg, ho), prel(hg, ho))
    assert np.abs(eg - eo).max() <= 1e-9
    o.set_spinors(g.get_spinors(_abi.MG_CAN_BASIS), None, _abi.MG_CAN_BASIS)
    o.set_occupations(g.get_occupations(_abi.MG_CAN_BASIS), _abi.MG_CAN_BASIS)
    for s in (g, o):
        s.DeriveBasis(_abi.MG_CAN_BASIS)
        s.UpdateDensities()
    dg, do = g.get_densities(), o.get_densities()
    for k in ("rho", "tau", "nablaj", "derrho", "laprho"):
        assert rel(dg[k], do[k]) <= 1e-12, (k, rel(dg[k], do[k]))
        assert prel(dg[k], do[k]) <= 1e-12, (k, prel(dg[k], do[k]))


def test_headline_24c_nwt160_fp64_against_oracle(built):
    p = RunParams(nx=24, ny=24, nz=24, dx=0.8, nwt=160, neutrons=28.0, protons=28.0,
                  pairing=_abi.MG_PAIRING_HFB)
    psi, qn, en = synthetic.ho_basis(p, 80, seed=1234)
    g, o = start_pair(p, psi, qn, en)
    compare_trajectory(g, o, 5)
    compare_kernels_same_inputs(g, o, p)
    g.close()
    o.close()


def test_large_36c_nwt300_fp64_against_oracle(built):
    p = RunParams(nx=36, ny=36, nz=36, dx=0.8, nwt=300, neutrons=50.0, protons=40.0,
                  pairing=_abi.MG_PAIRING_HFB)
    psi, qn, en = synthetic.ho_basis(p, 150, seed=1234)
    g, o = start_pair(p, psi, qn, en)
    compare_trajectory(g, o, 1)
    compare_kernels_same_inputs(g, o, p)
    g.close()
    o.close()


def test_constrained_batch_instance_against_oracle(built):
    """A Q20-constrained instance of the 64-instance uneven batch (seed 7;
    the alternating kind, always on): N=Z=10 on a 16^3 mesh with nwt=28
    (measured: |dE| <= 3.7e-9 MeV over the start and 5 iterations).  The
    smallest instance of the batch (N=12, Z=18 on 13^3, proton Fermi energy
    above zero from the second step on) amplifies rounding-level differences
    ~3000x per iteration in the oracle alone (a 1e-14 perturbation of the
    start gives 3e-11 MeV after one iteration), so there the GPU-oracle
    difference reaches 4.6e-8 MeV after 4 iterations and no 1e-8 bar
    applies."""
    inst = synthetic.uneven_instances(64, seed=7)
    d = sorted(inst, key=lambda x: x["params"].V * x["params"].nwt)[2]
    p = d["params"]
    assert (p.nx, p.nwt, p.neutrons, p.protons) == (16, 28, 10.0, 10.0)
    psi, qn, en = synthetic.ho_basis(p, d["n_neutron"], seed=d["seed"])
    g, o = start_pair(p, psi, qn, en, constraint=(2, 0, d["q20"]))
    compare_trajectory(g, o, 5)
    cg, co = g.get_constraint(0), o.get_constraint(0)
    assert abs(sum(cg["value"]) - sum(co["value"])) <= 1e-9 * max(1.0, abs(sum(co["value"])))
    g.close()
    o.close()
