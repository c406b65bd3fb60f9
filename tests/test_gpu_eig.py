"""The batched symmetric eigensolver (mg_eigh_batched) against LAPACK.

It replaces diagoncr8 (src/HFB.f90:5880-6087) for the HFB matrices and the
density matrix.  Bars: eigenvalues within 1e-13 |A|, residual
|A Z - Z diag(w)| within 1e-12 |A|, orthonormality within 1e-13, on random
spectra, on clustered spectra (splittings 1e-3 ... 1e-10 and exact
degeneracies) and on HFB-shaped matrices [[e, D], [D, -e]].
"""
import numpy as np
import pytest

from mocca_gb300 import _abi

pytestmark = pytest.mark.gpu


def _run(mats):
    nb = len(mats)
    ld = max(m.shape[0] for m in mats)
    a = np.zeros((nb, ld, ld))
    n = np.array([m.shape[0] for m in mats], dtype=np.int32)
    for b, m in enumerate(mats):
        a[b, :m.shape[0], :m.shape[0]] = m
    w = np.zeros((nb, ld))
    z = np.zeros((nb, ld, ld))
    st = _abi.load().mg_eigh_batched(nb, n.ctypes.data_as(_abi._I), ld, a.ctypes.data_as(_abi._D),
                                     w.ctypes.data_as(_abi._D), z.ctypes.data_as(_abi._D))
    assert st == 0, st
    return [(w[b, :k], z[b, :k, :k]) for b, k in enumerate(n)]


def _check(m, w, z):
    nrm = np.linalg.norm(m)
    ref = np.linalg.eigvalsh(m)
    assert np.abs(np.sort(w) - ref).max() <= 1e-13 * nrm
    assert np.linalg.norm(m @ z - z * w) <= 1e-12 * nrm
    assert np.abs(z.T @ z - np.eye(len(w))).max() <= 1e-13


def _sym(rng, n, spectrum):
    q, _ = np.linalg.qr(rng.normal(size=(n, n)))
    return (q * spectrum) @ q.T


def test_random_spectra(built):
    rng = np.random.default_rng(1)
    mats = []
    for n in (10, 37, 80, 128):
        x = rng.normal(size=(n, n))
        mats.append(x + x.T)
    for m, (w, z) in zip(mats, _run(mats)):
        _check(m, w, z)


@pytest.mark.parametrize("split", [1e-3, 1e-6, 1e-8, 1e-10, 0.0])
def test_clustered_spectra(built, split):
    rng = np.random.default_rng(2)
    mats = []
    for n in (20, 40, 80):
        base = np.repeat(np.linspace(0.0, 1.0, n // 4), 4)
        spec = base + split * rng.uniform(-1, 1, size=n)
        mats.append(_sym(rng, n, spec))
    for m, (w, z) in zip(mats, _run(mats)):
        _check(m, w, z)


def test_hfb_shaped(built):
    rng = np.random.default_rng(3)
    mats = []
    for h in (10, 40, 64):
        e = np.sort(rng.uniform(-30, 30, size=h))
        d = rng.normal(scale=1.5, size=(h, h))
        d = 0.5 * (d + d.T)
        mats.append(np.block([[np.diag(e), d], [d.T, -np.diag(e)]]))
    for m, (w, z) in zip(mats, _run(mats)):
        _check(m, w, z)


def test_large_blocks(built):
    """Matrices above 128 (up to the solver's 160): the HFB blocks of a
    300-spwf run (h up to 80), random, HFB-shaped and clustered, odd sizes
    included."""
    rng = np.random.default_rng(4)
    mats = []
    for n in (129, 151, 160):
        x = rng.normal(size=(n, n))
        mats.append(x + x.T)
    for h in (75, 80):
        e = np.sort(rng.uniform(-30, 30, size=h))
        d = rng.normal(scale=1.5, size=(h, h))
        d = 0.5 * (d + d.T)
        mats.append(np.block([[np.diag(e), d], [d.T, -np.diag(e)]]))
    base = np.repeat(np.linspace(0.0, 1.0, 40), 4)
    mats.append(_sym(rng, 160, base + 1e-9 * rng.uniform(-1, 1, size=160)))
    # a density-matrix-like spectrum: occupations clustered at 1 and 0
    occ = np.concatenate([1.0 - 1e-9 * rng.uniform(0, 1, 60), 1e-9 * rng.uniform(0, 1, 90),
                          rng.uniform(0, 1, 10)])
    mats.append(_sym(rng, 160, occ))
    for m, (w, z) in zip(mats, _run(mats)):
        _check(m, w, z)


def test_batch_of_64(built):
    """The largest batch both entry points accept (nb = 64) at a small
    leading dimension: every matrix of the batch is solved to the same bars."""
    rng = np.random.default_rng(5)
    mats = []
    for b in range(64):
        n = 4 + (b % 13)
        x = rng.normal(size=(n, n))
        mats.append(x + x.T)
    for m, (w, z) in zip(mats, _run(mats)):
        _check(m, w, z)


def test_density_matrix_with_near_one_cluster(built):
    """A density-matrix block of an HFB start whose occupations near one lie
    within 3e-8 of each other (0.999999935, 0.999999964 twice) and near zero
    within 3e-12: the refinement leaves that cluster unrotated, and the
    polish must start from vectors orthonormal to FP64 rounding, or its
    eigenvalues miss by the non-orthogonality (1.4e-7 was seen, above one)."""
    rng = np.random.default_rng(8)
    occ = np.array([2.13e-12, 2.41e-12, 2.55e-12, 2.93e-12, 3.04e-12, 3.56e-12, 3.56e-12,
                    3.96e-12, 4.60e-12, 4.94e-12, 0.999999935, 0.999999964, 0.999999964])
    mats = [_sym(rng, 13, occ) for _ in range(3)]
    for m, (w, z) in zip(mats, _run(mats)):
        _check(m, w, z)
        assert w.max() <= 1.0


def test_density_matrix_of_an_hfb_start(built):
    """The rho_++ blocks of the first pairing step of the perturbed-HO 10^3
    start (oracle), one of which has that near-one cluster: eigenvalues to
    the usual bars, none above one."""
    import oracle as O
    from mocca_gb300 import SLY4
    from test_gpu_gradient_hfb import _start
    p, psi, qn, en, pp = _start()
    pp.fermi_solver = 1
    o = O.OracleState(p, SLY4)
    o.set_spinors(psi, qn)
    o.set_energies(en)
    o.set_pairing(pp)
    o.SolvePairing()
    mats = []
    for b in range(4):
        r = o.get_hfb_block(b)[0]
        h = r.shape[0] // 2
        mats.append(np.ascontiguousarray(r[:h, :h]))
    o.close()
    for m, (w, z) in zip(mats, _run(mats)):
        _check(m, w, z)
        assert w.max() <= 1.0 + 1e-13
