"""The time-odd tensor terms on the GPU (time reversal broken, cranking
about z, HF, FP64, SLy5colo with J2Terms: B14..B21 all nonzero) against
the oracle, on the 10^3 EV8 start of 40 HO states and their time-reversed
partners (N = Z = 12), Omega_z = 0.5.

Bars (the benchmark spec's): lap s, grad div s, the C and D fields, div D, the
other time-odd densities and fields and h.psi within 1e-12 norm-wise and
pointwise (max |a - b| / max |b|), T and F within 1e-12 of max tau (the size
of their terms, which time-reversed partners cancel), both sides computing
them from the same spinors; the total energy within 1e-8 MeV at the start and after each of 4
iterations, with the fixed step, with ParameterEstimation = 1 (whose
probe takes the C and D actions too) and with MixingScheme 2 (the S update
preconditioned like U's).  With Omega = 0 the 80-spwf run
reproduces the 40-spwf time-reversal-invariant one (1e-9 MeV)."""
import dataclasses

import numpy as np
import pytest

import oracle as O
from conftest import rel
from mocca_gb300 import _abi
from mocca_gb300.forces import SLY5_TENSOR
from mocca_gb300.mesh import MeshState
from test_oracle_time_odd import cranked_start

pytestmark = pytest.mark.gpu


def prel(a, b):
    m = np.abs(b).max()
    return float(np.abs(a - b).max() / (m if m > 0 else 1.0))


def _pair(p, psi, qn, en):
    g, o = MeshState(p, SLY5_TENSOR), O.OracleState(p, SLY5_TENSOR)
    for s in (g, o):
        s.set_spinors(psi, qn)
        s.set_energies(en)
        s.Start()
    return g, o


def test_tensor_odd_fields_and_hpsi_against_oracle(built):
    """After one iteration the GPU's spinors and occupations go into the
    oracle and both recompute derivatives, densities, moments (the cutoff)
    and potentials from them."""
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
    # T and F are sums of products of derivatives whose time-reversed
    # partners cancel to ~1e-6 of the terms, so the last-bit differences of
    # the two sides' derivatives stand out in the net values: their bar is
    # relative to the size of the terms (max tau, the same products
    # uncancelled)
    tau = o.get_densities()["tau"]
    for tg, to in ((g.get_time_odd(), o.get_time_odd()),
                   (g.get_time_odd_tensor(), o.get_time_odd_tensor())):
        for k in to:
            assert np.abs(to[k]).max() > 1e-7, k
            if k in ("T", "F"):
                err = np.abs(tg[k] - to[k]).max() / np.abs(tau).max()
                assert err <= 1e-12, (k, err)
                continue
            assert rel(tg[k], to[k]) <= 1e-12 and prel(tg[k], to[k]) <= 1e-12, \
                (k, rel(tg[k], to[k]), prel(tg[k], to[k]))
    hg, eg, _ = g.hPsi(_abi.MG_HF_BASIS)
    ho, eo, _ = o.hPsi(_abi.MG_HF_BASIS)
    assert rel(hg, ho) <= 1e-12 and prel(hg, ho) <= 1e-12, (rel(hg, ho), prel(hg, ho))
    assert np.abs(eg - eo).max() <= 1e-9
    eg, eo = g.CompEnergy(), o.CompEnergy()
    for k in (20, 21, 26, 27, 28, 29):
        assert abs(eg["skyrme"][k] - eo["skyrme"][k]) <= 1e-10, (k + 1, eg["skyrme"][k],
                                                                 eo["skyrme"][k])
    assert abs(eg["total"] - eo["total"]) <= 1e-8
    g.close()
    o.close()


@pytest.mark.parametrize("estimate,mixing", [(0, 0), (1, 0), (0, 2)])
def test_tensor_odd_iterations_against_oracle(built, estimate, mixing):
    """mixing 2: MixingScheme 2 preconditions the U update and, without
    time reversal, each component of the S update."""
    _, _, p, s80 = cranked_start(0.5)
    p = dataclasses.replace(p, parameter_estimation=estimate, mixing_scheme=mixing)
    g, o = _pair(p, *s80)
    de = [abs(g.CompEnergy()["total"] - o.CompEnergy()["total"])]
    for _ in range(4):
        de.append(abs(g.Evolve(1, 0.010, 0.3)["total"] - o.Evolve(1, 0.010, 0.3)["total"]))
        if estimate:
            (dg, mg), (do, mo) = g.StepParameters(), o.StepParameters()
            assert dg == pytest.approx(do, rel=1e-9, abs=0) and mg == pytest.approx(mo, rel=1e-9,
                                                                                   abs=0)
    assert max(de) <= 1e-8, de
    g.close()
    o.close()


def test_uncranked_pairs_reproduce_the_invariant_run_on_the_gpu(built):
    base, s40, p, s80 = cranked_start(0.0)
    out = []
    for params, st in ((base, s40), (p, s80)):
        g = MeshState(params, SLY5_TENSOR)
        g.set_spinors(st[0], st[1])
        g.set_energies(st[2])
        g.Start()
        out.append([g.Evolve(1, 0.010, 0.3)["total"] for _ in range(3)])
        g.close()
    assert np.abs(np.array(out[0]) - np.array(out[1])).max() <= 1e-9, out
