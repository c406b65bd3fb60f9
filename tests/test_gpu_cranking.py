"""The time-odd path on the GPU (time reversal broken, cranking about z,
HF, FP64) against the oracle: the 10^3 EV8 start of 40 HO states and their
time-reversed partners, N=Z=12, Omega_z = 0.5.

Bars (the benchmark spec's): the time-odd densities (vecj, vecs, their curls), the
A and S fields with their cranking parts, div A and h.psi within 1e-12
norm-wise and pointwise (max |a - b| / max |b|), both sides computing them
from the same spinors; the total energy within 1e-8 MeV at the start and
after each of 4 iterations.  With Omega = 0 the
time-reversal-broken GPU run reproduces the 40-spwf time-reversal-invariant
one (energies within 1e-9 MeV)."""
import numpy as np
import pytest

import oracle as O
from conftest import rel
from mocca_gb300 import SLY4, _abi
from mocca_gb300.mesh import MeshState
from test_oracle_time_odd import cranked_start

pytestmark = pytest.mark.gpu


def prel(a, b):
    m = np.abs(b).max()
    return float(np.abs(a - b).max() / (m if m > 0 else 1.0))


def _pair(p, psi, qn, en):
    g, o = MeshState(p, SLY4), O.OracleState(p, SLY4)
    for s in (g, o):
        s.set_spinors(psi, qn)
        s.set_energies(en)
        s.Start()
    return g, o


def test_cranked_fields_and_hpsi_against_oracle(built):
    """After one iteration (the start's states are exact time-reversal
    pairs, whose currents vanish), the GPU's spinors and occupations go into
    the oracle and both recompute derivatives, densities, moments (the
    cutoff) and potentials from them."""
    _, _, p, s80 = cranked_start(0.5)
    g, o = _pair(p, *s80)
    g.Evolve(1, 0.010, 0.3)
    o.Evolve(1, 0.010, 0.3)
    o.set_spinors(g.get_spinors(_abi.MG_HF_BASIS), None, _abi.MG_HF_BASIS)
    o.set_occupations(g.get_occupations(_abi.MG_HF_BASIS), _abi.MG_HF_BASIS)
    for s in (g, o):
        s.DeriveAll()
        s.UpdateDensities()
        s.CalculateAllMoments()
        s.ConstructPotentials()
    tg, to = g.get_time_odd(), o.get_time_odd()
    for k in ("vecj", "vecs", "rotj", "rots", "A", "S", "divA"):
        assert np.abs(to[k]).max() > 1e-6, k
        assert rel(tg[k], to[k]) <= 1e-12 and prel(tg[k], to[k]) <= 1e-12, \
            (k, rel(tg[k], to[k]), prel(tg[k], to[k]))
    hg, eg, _ = g.hPsi(_abi.MG_HF_BASIS)
    ho, eo, _ = o.hPsi(_abi.MG_HF_BASIS)
    assert rel(hg, ho) <= 1e-12 and prel(hg, ho) <= 1e-12, (rel(hg, ho), prel(hg, ho))
    assert np.abs(eg - eo).max() <= 1e-9
    g.close()
    o.close()


def test_cranked_iterations_against_oracle(built):
    _, _, p, s80 = cranked_start(0.5)
    g, o = _pair(p, *s80)
    de = [abs(g.CompEnergy()["total"] - o.CompEnergy()["total"])]
    for _ in range(4):
        de.append(abs(g.Evolve(1, 0.010, 0.3)["total"] - o.Evolve(1, 0.010, 0.3)["total"]))
    assert max(de) <= 1e-8, de
    g.close()
    o.close()


def test_time_reversal_broken_without_cranking_on_the_gpu(built):
    base, s40, p, s80 = cranked_start(0.0)
    out = []
    for params, st in ((base, s40), (p, s80)):
        g = MeshState(params, SLY4)
        g.set_spinors(st[0], st[1])
        g.set_energies(st[2])
        g.Start()
        out.append([g.Evolve(1, 0.010, 0.3)["total"] for _ in range(3)])
        g.close()
    assert np.abs(np.array(out[0]) - np.array(out[1])).max() <= 1e-9, out
