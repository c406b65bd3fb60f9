"""Mixed-precision path (MG_MIXED): derivative contractions on the tensor
cores (exact BF16 digit products, line lengths up to 32) or as double-float
(FP32 pair) sums (longer lines, n = 36 below), stored as double-float pairs,
checked against the FP64 oracle; and the mixed iterations followed by an FP64
polish checked against the plain FP64 GPU path.

Bars: derivatives and Laplacians within 1e-11 relative (norm-wise).  The
tensor-core form rounds each line and each matrix row to 47-bit integers
(scaled by powers of two) and sums their digit products exactly, so its error
is a few units of 2^-47 of the line's largest terms; the double-float form
carries 48 significant bits with (hi, lo) sums.  After mixed iterations and an FP64 polish the total energy agrees
with the all-FP64 run to 1e-5 MeV.
"""
import numpy as np
import pytest

import oracle as O
from conftest import rel
from mocca_gb300 import MG_FP64, MG_MIXED, SLY4, RunParams, _abi, synthetic
from mocca_gb300.mesh import MeshState

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,nwt", [(10, 8), (13, 6), (24, 8), (36, 4)])
def test_mixed_derivatives_ev8(built, n, nwt):
    p = RunParams(nx=n, ny=n, nz=n, dx=0.8, nwt=nwt, neutrons=8, protons=8, precision=MG_MIXED)
    psi, qn, en = synthetic.ho_basis(p, nwt // 2, seed=5)
    g = MeshState(p, SLY4)
    o = O.OracleState(p, SLY4)
    for s in (g, o):
        s.set_spinors(psi, qn)
        s.set_energies(en)
    g.DeriveAll()
    o.DeriveAll()
    dg, lg = g.get_derivatives()
    do, lo = o.get_derivatives()
    assert rel(dg, do) < 1e-11
    assert rel(lg, lo) < 1e-11
    assert rel(dg, do) > 1e-15   # the double-float kernels ran, not the FP64 ones
    g.set_precision(MG_FP64)
    g.DeriveAll()
    dg, lg = g.get_derivatives()
    assert rel(dg, do) < 1e-12 and rel(lg, lo) < 1e-12
    g.close()


def test_mixed_derivatives_full_box(built):
    p = RunParams(nx=12, ny=12, nz=12, dx=0.8, pc=0, sc=0, tsc=0, trc=1, nwt=6,
                  neutrons=8, protons=8, coulomb_solver=0, precision=MG_MIXED)
    psi = synthetic.gaussian_hermite_spinors(p, p.nwt, seed=42)
    qn = np.tile(np.array([-1, 0, 0, 0], dtype=np.int32), (p.nwt, 1))
    qn[3:, 0] = 1
    g = MeshState(p, SLY4)
    o = O.OracleState(p, SLY4)
    for s in (g, o):
        s.set_spinors(psi, qn)
        s.set_energies(np.zeros(p.nwt))
    g.DeriveAll()
    o.DeriveAll()
    dg, lg = g.get_derivatives()
    do, lo = o.get_derivatives()
    assert rel(dg, do) < 1e-11
    assert rel(lg, lo) < 1e-11
    g.close()


def test_mixed_hpsi_full_box(built):
    """h.psi with Woods-Saxon fields in double-float against the FP64 oracle."""
    p = RunParams(nx=12, ny=12, nz=12, dx=0.8, pc=0, sc=0, tsc=0, trc=1, nwt=6,
                  neutrons=8, protons=8, coulomb_solver=0, precision=MG_MIXED)
    psi = synthetic.gaussian_hermite_spinors(p, p.nwt, seed=42)
    qn = np.tile(np.array([-1, 0, 0, 0], dtype=np.int32), (p.nwt, 1))
    qn[3:, 0] = 1
    g = MeshState(p, SLY4)
    o = O.OracleState(p, SLY4)
    U, B, nB, W, dW = synthetic.woods_saxon_fields(p)
    for s in (g, o):
        s.set_spinors(psi, qn)
        s.set_energies(np.zeros(p.nwt))
        s.set_potentials(U=U, B=B, nablaB=nB, W=W, divW=dW)
        s.DeriveAll()
    hg, eg, _ = g.hPsi()
    ho, eo, _ = o.hPsi()
    assert rel(hg, ho) < 1e-11
    assert np.allclose(eg, eo, rtol=0, atol=1e-9)
    g.close()


def test_mixed_start_densities_energy(built):
    """HF start of the Mg24 case with every mesh kernel in double-float.

    The mixed form solves the Coulomb problem directly (separable eigenbasis +
    FP64 refinement) while the oracle, like the reference, stops its CG at
    sum r^2 <= 1e-9 / (dx^3 V): U (which holds the Coulomb potential) and the
    energy then differ by the CG truncation, ~1e-9 relative and ~1e-7 MeV.
    """
    p = RunParams(nx=10, ny=10, nz=10, dx=0.8, nwt=40, neutrons=12, protons=12,
                  precision=MG_MIXED)
    psi, qn, en = synthetic.ho_basis(p, 20, seed=1234)
    g = MeshState(p, SLY4)
    o = O.OracleState(p, SLY4)
    for s in (g, o):
        s.set_spinors(psi, qn)
        s.set_energies(en)
    g.Start()
    o.Start()
    dg, do = g.get_densities(), o.get_densities()
    for k in dg:
        assert rel(dg[k], do[k]) < 1e-11, k
    pg, po = g.get_potentials(), o.get_potentials()
    for k in ("B", "nablaB", "W"):
        assert rel(pg[k], po[k]) < 1e-10, k
    assert rel(pg["U"], po["U"]) < 1e-8
    assert rel(pg["coulomb"], po["coulomb"]) < 1e-8
    eg, eo = g.CompEnergy(), o.CompEnergy()
    assert abs(eg["total"] - eo["total"]) < 1e-6
    assert abs(eg["kinetic"][0] - eo["kinetic"][0]) < 1e-9
    hg, e1, _ = g.hPsi()
    ho, e2, _ = o.hPsi()
    assert rel(hg, ho) < 1e-9
    assert np.allclose(e1, e2, rtol=0, atol=1e-7)
    g.close()


def test_mixed_coulomb_direct_residual(built):
    """The direct Coulomb solve leaves a residual far below the CG tolerance:
    the FP64 CG started from its solution stops after at most a few steps."""
    p = RunParams(nx=10, ny=10, nz=10, dx=0.8, nwt=40, neutrons=12, protons=12,
                  precision=MG_MIXED)
    psi, qn, en = synthetic.ho_basis(p, 20, seed=1234)
    g = MeshState(p, SLY4)
    g.set_spinors(psi, qn)
    g.set_energies(en)
    g.Start()
    g.set_precision(MG_FP64)
    assert g.SolveCoulomb() <= 2
    g.close()


def test_mixed_hfb_start(built):
    """Pairing field and gaps (double-float mesh kernels) and the canonical
    basis (tensor-core block apply), the latter through the densities it
    builds (invariant under sign and degenerate-subspace choices)."""
    p = RunParams(nx=10, ny=10, nz=10, dx=0.8, nwt=40, neutrons=12, protons=12,
                  pairing=_abi.MG_PAIRING_HFB, precision=MG_MIXED)
    psi, qn, en = synthetic.ho_basis(p, 20, seed=1234)
    g = MeshState(p, SLY4)
    o = O.OracleState(p, SLY4)
    for s in (g, o):
        s.set_spinors(psi, qn)
        s.set_energies(en)
        s.set_pairing()
    ig = g.SolvePairing()
    io = o.SolvePairing()
    assert ig["converged"] and io["converged"]
    fg, fo = g.get_pairing_field(), o.get_pairing_field()
    for a, b in zip(fg, fo):
        assert rel(a, b) < 1e-10
    assert abs(sum(ig["pairing_energy"]) - sum(io["pairing_energy"])) < 1e-9
    for s in (g, o):
        s.DeriveAll()
        s.UpdateDensities()
    dg, do = g.get_densities(), o.get_densities()
    for k in ("rho", "tau", "nablaj"):
        assert rel(dg[k], do[k]) < 1e-10, k
    g.close()


def _hfb(precision):
    p = RunParams(nx=10, ny=10, nz=10, dx=0.8, nwt=40, neutrons=12, protons=12,
                  pairing=_abi.MG_PAIRING_HFB, precision=precision)
    psi, qn, en = synthetic.ho_basis(p, 20, seed=1234)
    g = MeshState(p, SLY4)
    g.set_spinors(psi, qn)
    g.set_energies(en)
    g.set_pairing()
    g.Start()
    return g


def test_mixed_iterations_with_fp64_polish(built):
    ref = _hfb(MG_FP64)
    e_ref = ref.Evolve(40, 0.01, 0.3)["total"]
    mix = _hfb(MG_MIXED)
    e_mid = mix.Evolve(30, 0.01, 0.3)["total"]
    mix.set_precision(MG_FP64)
    e_mix = mix.Evolve(10, 0.01, 0.3)["total"]
    assert np.isfinite(e_mid)
    assert abs(e_mix - e_ref) <= 1e-5, (e_mix, e_ref)
    ref.close()
    mix.close()


@pytest.mark.parametrize("n,nwt", [(10, 40), (24, 160), (10, 224), (10, 300)])
def test_mixed_gram_schmidt(built, n, nwt):
    """Tensor-core Gram-Schmidt (overlap and apply as exact digit products)
    against the FP64 oracle: 1e-11 relative on the spinors, orthonormal to
    5e-12 within each (isospin, parity) block.  Block sizes 34/46 (nwt=160),
    62/50 (224: K groups 7 and 8 of the apply) and 70/80 (300: 512 TMEM
    columns, one CTA per SM).  The apply rounds each point's
    spinor values to 47 bits of the point's largest one and this basis is far
    from orthonormal (2% noise), so R^-1 amplifies that rounding a little."""
    p = RunParams(nx=n, ny=n, nz=n, dx=0.8, nwt=nwt, neutrons=nwt // 4, protons=nwt // 4,
                  precision=MG_MIXED)
    psi, qn, en = synthetic.ho_basis(p, nwt // 2, seed=7)
    rng = np.random.default_rng(11)
    pert = psi + 0.02 * rng.normal(size=psi.shape) * np.abs(psi).max()
    en = en + rng.normal(size=en.shape)
    g = MeshState(p, SLY4)
    o = O.OracleState(p, SLY4)
    for s in (g, o):
        s.set_spinors(pert, qn)
        s.set_energies(en)
    g.GramSchmidt()
    o.GramSchmidt()
    qg, qo = g.get_spinors(), o.get_spinors()
    assert rel(qg, qo) < 1e-11
    assert rel(qg, qo) > 1e-16   # the tensor-core kernels ran, not the FP64 ones
    q = qg.reshape(p.nwt, -1)
    S = q @ q.T * p.dv
    same = (qn[:, None, 0] == qn[None, :, 0]) & (qn[:, None, 1] == qn[None, :, 1])
    assert np.abs(S[same] - np.eye(p.nwt)[same]).max() < 5e-12
    g.close()


@pytest.mark.parametrize("nwt,nz", [(224, 60), (300, 66)])
def test_mixed_hfb_large_blocks(built, nwt, nz):
    """Pairing field, gaps and canonical-basis transform on the tensor cores
    for HFB blocks of 50-62 (nwt=224) and 70-80 spinors (nwt=300), against the
    FP64 GPU path from the same start (the FP64 path is held to the oracle by
    the parity tests; both run the same Newton Fermi search): pairing field
    within 1e-10 of its scale, rho and tau within 1e-10, div J within 5e-10,
    pairing energies within 1e-8 MeV.  N = Z = nz keeps the pairing alive on this start (pairing energies of
    -18 and -31 MeV; at N = Z = nwt / 4 it collapses and the field is zero)."""
    out = {}
    for prec in (MG_FP64, MG_MIXED):
        p = RunParams(nx=10, ny=10, nz=10, dx=0.8, nwt=nwt, neutrons=nz, protons=nz,
                      pairing=_abi.MG_PAIRING_HFB, precision=prec)
        psi, qn, en = synthetic.ho_basis(p, nwt // 2, seed=1234)
        g = MeshState(p, SLY4)
        g.set_spinors(psi, qn)
        g.set_energies(en)
        g.set_pairing()
        info = g.SolvePairing()
        assert info["converged"]
        field = g.get_pairing_field()
        g.DeriveAll()
        g.UpdateDensities()
        out[prec] = (info, field, g.get_densities())
        g.close()
    (i64, f64, d64), (imx, fmx, dmx) = out[MG_FP64], out[MG_MIXED]
    # real and imaginary parts against the field's scale (the imaginary part
    # vanishes with time reversal up to rounding), the density factor relative
    scale = np.abs(f64[0]).max()
    for k in (0, 1):
        assert np.abs(fmx[k] - f64[k]).max() < 1e-10 * scale, k
    assert rel(fmx[2], f64[2]) < 1e-12
    for it in range(2):
        assert abs(imx["pairing_energy"][it] - i64["pairing_energy"][it]) < 1e-8
    # rho and tau within 1e-10; div J, a difference of derivative products
    # summed over the canonical states, measured 1.8e-10 at nwt=224
    for k, bar in (("rho", 1e-10), ("tau", 1e-10), ("nablaj", 5e-10)):
        assert rel(dmx[k], d64[k]) < bar, k
