"""The Nilsson start on the device (mg_nilsson_start) against the numpy
restatement of INITWF / nil8 used by the harness (synthetic.nilsson_basis).

Without perturbation both build the same states: quantum numbers equal,
Nilsson energies within 1e-12 MeV, and on a triaxial oscillator (no
degenerate levels among the stored states) every spinor within 1e-12 of
the restatement's up to its sign.  On the spherical oscillator of the
README's Mg24 start the levels of a j-multiplet are degenerate, so the two
eigensolvers may rotate within a multiplet: there each multiplet's two
sets of spinors span the same space (their overlap matrix orthogonal to
1e-12) and the per-isospin density sum |psi|^2 agrees (1e-12).
The perturbation is deterministic in the seed, bounded by its amplitude
and leaves every spwf normalised.
"""
import numpy as np
import pytest

from mocca_gb300 import SLY4, RunParams, _abi, synthetic
from mocca_gb300.mesh import MeshState

pytestmark = pytest.mark.gpu


def _params(n=10, nz=None, nwt=40, N=12, Z=12):
    return RunParams(nx=n, ny=n, nz=nz or n, dx=0.8, nwt=nwt, neutrons=N, protons=Z)


def _device(p, n_neutron, **kw):
    g = MeshState(p, SLY4)
    g.NilssonStart(n_neutron, **kw)
    return g


def test_triaxial_states_match_restatement(built):
    p = _params(n=12, nz=14, nwt=44, N=14, Z=12)
    ho = (0.18, 0.21, 0.25)
    g = _device(p, 22, ho=ho, amplitude=0.0)
    psi, qn, en = synthetic.nilsson_basis(p, 22, amplitude=0.0, ho=ho)
    e_dev, _ = g.get_energies()
    assert np.abs(e_dev - en).max() < 1e-12
    gp = g.get_spinors()
    gaps = np.diff(np.sort(en[:22])).min(), np.diff(np.sort(en[22:])).min()
    assert min(gaps) > 1e-6                      # no degenerate levels stored
    for i in range(p.nwt):
        s = np.sign(np.sum(gp[i] * psi[i]))
        assert np.abs(gp[i] - s * psi[i]).max() < 1e-12 * np.abs(psi[i]).max(), i
    g.close()


def test_spherical_start_matches_restatement(built):
    p = _params()
    g = _device(p, 20, amplitude=0.0)
    psi, qn, en = synthetic.nilsson_basis(p, 20, amplitude=0.0)
    e_dev, _ = g.get_energies()
    assert np.abs(e_dev - en).max() < 1e-12
    gp = g.get_spinors()
    dv = 8 * p.dx ** 3
    # each degenerate multiplet (isospin, parity, energy) spans the same
    # space: the overlap matrix of the two sets of spinors is orthogonal
    seen = 0
    for sl in (slice(0, 20), slice(20, 40)):
        idx = np.arange(p.nwt)[sl]
        groups = []
        for par in (1, -1):
            sel = sorted((i for i in idx if qn[i, 1] == par), key=lambda i: en[i])
            for i in sel:
                if groups and groups[-1][0] == par and en[i] - en[groups[-1][1][-1]] < 1e-8:
                    groups[-1][1].append(i)
                else:
                    groups.append((par, [i]))
        for _, members in groups:
            A = gp[members].reshape(len(members), -1)
            B = psi[members].reshape(len(members), -1)
            G = (A @ B.T) * dv
            assert np.abs(G.T @ G - np.eye(len(members))).max() < 1e-12, members
            seen += len(members)
        rd = np.sum(gp[sl] ** 2, axis=(0, 1))
        rp = np.sum(psi[sl] ** 2, axis=(0, 1))
        assert np.abs(rd - rp).max() < 1e-12 * rp.max()
    assert seen == p.nwt
    g.close()


def test_perturbation(built):
    p = _params()
    a = _device(p, 20, amplitude=0.0)
    b = _device(p, 20, amplitude=1e-3, seed=7)
    c = _device(p, 20, amplitude=1e-3, seed=7)
    d = _device(p, 20, amplitude=1e-3, seed=8)
    pa, pb, pc, pd = (s.get_spinors() for s in (a, b, c, d))
    assert np.array_equal(pb, pc)
    assert not np.array_equal(pb, pd)
    dv = 8 * p.dx ** 3
    for i in range(p.nwt):
        assert abs(np.sum(pb[i] ** 2) * dv - 1.0) < 1e-12
        # nil8's states come normalised, so the renormalisation is ~1 and
        # the difference is the perturbation: within the amplitude (plus
        # the small rescaling), nonzero, centred
        delta = pb[i] - pa[i]
        assert 2e-4 < np.abs(delta).max() < 1.5e-3, (i, np.abs(delta).max())
        assert abs(delta.mean()) < 5e-5
    for s in (a, b, c, d):
        s.close()


def test_refuses_non_ev8(built):
    q = RunParams(nx=16, ny=16, nz=16, dx=0.8, nwt=8, neutrons=4, protons=4, pc=0, sc=0, tsc=0)
    g = MeshState(q, SLY4)
    with pytest.raises(_abi.MgError):
        g.NilssonStart(4)
    g.close()
