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


def _full_box_state(builders):
    """Normalised spinors on a 12^3 symmetry-free box from (component,
    function of x, y, z) pairs."""
    p = RunParams(nx=12, ny=12, nz=12, dx=0.8, pc=0, sc=0, tsc=0, nwt=len(builders),
                  neutrons=2, protons=0)
    c = (np.arange(12) + 0.5) * 0.8 - 12 / 2 * 0.8
    Z, Y, X = np.meshgrid(c, c, c, indexing="ij")
    psi = np.zeros((p.nwt, 4, 12, 12, 12))
    for i, (comp, f) in enumerate(builders):
        psi[i, comp] = f(X, Y, Z)
    psi /= np.sqrt((psi ** 2).sum(axis=(1, 2, 3, 4)) * p.dv)[:, None, None, None, None]
    qn = np.tile(np.array([-1, 0, 0, 0], dtype=np.int32), (p.nwt, 1))
    return p, psi.reshape(p.nwt, -1), qn


def test_symmetry_operators_known_answers(built_oracle):
    """SymmetryOperators on the symmetry-free box for states of known
    symmetry: a spin-up s wave (parity, signature and time simplex +1,
    x-simplex 0), a spin-up p_x wave (parity -1, signature -1, time simplex
    +1), a spin-up p_y wave (time simplex -1), and the RMS radius of a
    Gaussian, sqrt(3/2) times its width parameter."""
    g = lambda X, Y, Z: np.exp(-(X ** 2 + Y ** 2 + Z ** 2) / 4.0)  # noqa: E731
    p, psi, qn = _full_box_state([(0, g), (0, lambda X, Y, Z: X * g(X, Y, Z)),
                                  (0, lambda X, Y, Z: Y * g(X, Y, Z))])
    o = O.OracleState(p, SLY4)
    o.set_spinors(psi, qn)
    s = o.SymmetryOperators()
    o.close()
    assert np.allclose(s[0, 1:5], [1.0, 1.0, 1.0, 0.0], atol=1e-12), s[0]
    assert np.allclose(s[1, 1:4], [-1.0, -1.0, 1.0], atol=1e-12), s[1]
    assert abs(s[2, 3] + 1.0) <= 1e-12, s[2]
    # <r^2> of exp(-r^2/4)^2 = exp(-r^2/2): 3 (variance 1); the mesh sum is
    # the exact integral to ~1e-6 at dx = 0.8 for this width
    assert abs(s[0, 5] - np.sqrt(3.0)) <= 1e-4, s[0, 5]
