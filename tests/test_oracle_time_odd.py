"""The oracle's time-odd path (time reversal broken, cranking about z)
against its own time-reversal-invariant path: with Omega = 0 a run on the
EV8 box whose 80 stored spwfs are 40 HO states and their time-reversed
partners (TimeReverse, src/Spinor.f90:371-389: (c3, -c4, -c1, c2)) keeps
every time-odd density at rounding level and reproduces the energies of
the 40-spwf time-reversal-invariant run; with Omega_z = 0.5 the currents,
spin densities and the A and S fields are nonzero and the energy moves."""
import numpy as np
import pytest

import oracle as O
from mocca_gb300 import SLY4, RunParams, synthetic


def cranked_start(omega):
    base = RunParams(nx=10, ny=10, nz=10, dx=0.8, nwt=40, neutrons=12, protons=12)
    psi, qn, en = synthetic.ho_basis(base, 20, seed=1234)
    en = np.asarray(en) + np.random.default_rng(5).uniform(-0.2, 0.2, size=len(en))
    p4 = psi.reshape(40, 4, -1)
    tr = np.stack([p4[:, 2], -p4[:, 3], -p4[:, 0], p4[:, 1]], axis=1)
    psi2 = np.concatenate([p4, tr]).reshape(80, -1)
    qn2 = np.concatenate([qn, qn])
    qn2[40:, 2] = -qn2[40:, 2]
    p = RunParams(nx=10, ny=10, nz=10, dx=0.8, nwt=80, neutrons=12, protons=12, trc=0,
                  omega=(0.0, 0.0, omega))
    return base, (psi, qn, en), p, (psi2, qn2, np.concatenate([en, en]))


@pytest.fixture(scope="module")
def built_oracle():
    O.build_oracle()
    return True


def _run(p, psi, qn, en, iters=3):
    o = O.OracleState(p, SLY4)
    o.set_spinors(psi, qn)
    o.set_energies(en)
    o.Start()
    es = [o.Evolve(1, 0.010, 0.3)["total"] for _ in range(iters)]
    odd = o.get_time_odd() if not p.trc else None
    o.close()
    return es, odd


def test_time_reversal_broken_without_cranking_reproduces_the_invariant_run(built_oracle):
    base, s40, p, s80 = cranked_start(0.0)
    e40, _ = _run(base, *s40)
    e80, odd = _run(p, *s80)
    assert np.abs(np.array(e40) - np.array(e80)).max() <= 1e-9, (e40, e80)
    for k, v in odd.items():
        assert np.abs(v).max() <= 1e-12, k


def test_cranking_makes_time_odd_fields(built_oracle):
    base, s40, p, s80 = cranked_start(0.5)
    e0, _ = _run(base, *s40)
    e1, odd = _run(p, *s80)
    for k in ("vecj", "vecs", "rotj", "rots", "A", "S", "divA"):
        assert np.abs(odd[k]).max() > 1e-5, k
    assert abs(e1[-1] - e0[-1]) > 1e-3
