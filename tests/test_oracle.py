"""CPU checks of the FP64 oracle against known answers.

The reference ships no golden outputs, so the oracle is pinned by
self-derived known-answer tests from the formulas it restates:
Lagrange-mesh derivatives exact on the anti-periodic half-integer Fourier
modes of the full line (Baye-Heenen, src/Derivatives.f90:899-973), folded
EV8 matrices equal to the unfolded line operator applied to mirror-extended
lines (reduceLag, :975-1078), the SLy4 coupling constants, orthonormality
after Gram-Schmidt, the Coulomb potential of a uniform sphere, and the
committed golden fixture produced by tests/golden/make_golden.py.
"""
import json
import math
from pathlib import Path

import numpy as np
import pytest

import oracle as O
from conftest import rel
from mocca_gb300 import SLY4, RunParams, _abi, synthetic

GOLDEN = Path(__file__).resolve().parent / "golden"


@pytest.mark.parametrize("n", [6, 10, 24])
def test_lagrange_exact_on_half_integer_modes(n):
    dx = 0.8
    d1, d2 = O.lagrange_matrices(n, dx, True)
    x = dx / 2 + dx * np.arange(n)
    L = 2 * n * dx
    for k in range(n):
        w = math.pi * (2 * k + 1) / L
        assert np.abs(d1[1] @ np.cos(w * x) + w * np.sin(w * x)).max() < 1e-12 * w * 50
        assert np.abs(d1[0] @ np.sin(w * x) - w * np.cos(w * x)).max() < 1e-12 * w * 50
        assert np.abs(d2[1] @ np.cos(w * x) + w * w * np.cos(w * x)).max() < 1e-12 * w * w * 50
        assert np.abs(d2[0] @ np.sin(w * x) + w * w * np.sin(w * x)).max() < 1e-12 * w * w * 50


@pytest.mark.parametrize("n", [5, 12])
def test_folded_equals_unfolded_on_mirrored_line(n):
    dx = 0.7
    d1, d2 = O.lagrange_matrices(n, dx, True)
    u1, u2 = O.lagrange_matrices(2 * n, dx, False)
    rng = np.random.default_rng(3)
    half = rng.normal(size=n)
    for s, slot in ((1.0, 1), (-1.0, 0)):
        # full line ordered -x_n..-x_1, x_1..x_n with f(-x) = s f(x)
        full = np.concatenate([s * half[::-1], half])
        assert np.allclose((u1[0] @ full)[n:], d1[slot] @ half, atol=1e-12, rtol=0)
        assert np.allclose((u2[0] @ full)[n:], d2[slot] @ half, atol=1e-11, rtol=0)


def test_sly4_coefficients():
    b = _abi.MgSkyrmeB()
    st = O.load().orc_skyrme_coefficients(SLY4.to_c(), 1, b)
    assert st == 0
    t0, x0, t1, x1, t2, x2, t3, x3 = -2488.913, 0.834, 486.818, -0.344, -546.395, -1.0, 13777.0, 1.354
    assert b.B1 == pytest.approx(t0 / 2 * (1 + x0 / 2))
    assert b.B2 == pytest.approx(-t0 / 2 * (x0 + 0.5))
    assert b.B3 == pytest.approx((t1 * (1 + x1 / 2) + t2 * (1 + x2 / 2)) / 4)
    assert b.B7a == pytest.approx(t3 / 12 * (1 + x3 / 2))
    assert b.B9 == pytest.approx(-123.0 / 2)
    assert b.B16 == 0.0 and b.B17 == 0.0


def _mg24(nwt=40):
    p = RunParams(nx=10, ny=10, nz=10, dx=0.8, nwt=nwt, neutrons=12, protons=12)
    psi, qn, en = synthetic.ho_basis(p, nwt // 2, seed=1234)
    return p, psi, qn, en


def test_gram_schmidt_orthonormal():
    p, psi, qn, en = _mg24()
    o = O.OracleState(p, SLY4)
    rng = np.random.default_rng(5)
    o.set_spinors(psi + 0.05 * rng.normal(size=psi.shape), qn)
    o.set_energies(en)
    o.GramSchmidt()
    q = o.get_spinors().reshape(p.nwt, -1)
    S = q @ q.T * p.dv
    same = (qn[:, None, 0] == qn[None, :, 0]) & (qn[:, None, 1] == qn[None, :, 1])
    assert np.abs(S[same] - np.eye(p.nwt)[same]).max() < 1e-13


def test_uniform_sphere_coulomb():
    """Coulomb of a uniform proton sphere against Q/R (3 - r^2/R^2)/2 inside."""
    p = RunParams(nx=16, ny=16, nz=16, dx=0.8, nwt=2, neutrons=20, protons=20)
    o = O.OracleState(p, SLY4)
    x, y, z = synthetic.mesh_axes(p)
    Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
    r = np.sqrt(X ** 2 + Y ** 2 + Z ** 2)
    R = 5.0
    rho0 = 20.0 / (4.0 / 3.0 * math.pi * R ** 3)
    # smooth the edge so the FD Laplacian sees a resolvable profile
    prof = rho0 / (1.0 + np.exp((r - R) / 0.3))
    prof *= 20.0 / (prof.sum() * p.dv)
    rho = np.stack([prof, prof]).reshape(2, -1)
    o.set_densities(rho=rho)
    o.CalculateAllMoments()
    it = o.SolveCoulomb()
    assert 0 < it < 500
    pot = o.get_potentials()["coulomb"].reshape(p.nz, p.ny, p.nx)
    e2 = SLY4.e2
    # radial quadrature of the same (renormalised) profile:
    # V(r) = 4 pi e2 [ (1/r) int_0^r rho r'^2 dr' + int_r^inf rho r' dr' ]
    scale = prof.max() / (rho0 / (1.0 + np.exp(-R / 0.3)))
    s = np.linspace(0.0, 30.0, 300001)
    f = scale * rho0 / (1.0 + np.exp((s - R) / 0.3))
    ds = s[1] - s[0]
    q_in = np.concatenate([[0.0], np.cumsum((f[1:] * s[1:] ** 2 + f[:-1] * s[:-1] ** 2) / 2 * ds)])
    g = f * s
    tail = np.concatenate([np.cumsum(((g[1:] + g[:-1]) / 2 * ds)[::-1])[::-1], [0.0]])
    with np.errstate(divide="ignore", invalid="ignore"):
        Vr = 4 * math.pi * e2 * (np.where(s > 0, q_in / np.where(s > 0, s, 1), 0.0) + tail)
    ana = np.interp(r, s, Vr)
    assert np.abs(pot - ana).max() / ana.max() < 2e-3


def test_hf_iterations_lower_the_energy():
    p, psi, qn, en = _mg24()
    o = O.OracleState(p, SLY4)
    o.set_spinors(psi, qn)
    o.set_energies(en)
    o.Start()
    e0 = o.CompEnergy()["total"]
    e = o.Evolve(5, 0.010, 0.0)["total"]
    assert e < e0 - 5.0


def test_golden_fixture():
    """The oracle reproduces the committed golden numbers (make_golden.py)."""
    g = json.loads((GOLDEN / "mg24_hf.json").read_text())
    p, psi, qn, en = _mg24()
    o = O.OracleState(p, SLY4)
    o.set_spinors(psi, qn)
    o.set_energies(en)
    o.Start()
    assert o.CompEnergy()["total"] == pytest.approx(g["E_start"], abs=1e-9)
    e = o.Evolve(g["iterations"], g["dt"], g["momentum"])
    assert e["total"] == pytest.approx(g["E_final"], abs=1e-9)
    sp, _ = o.get_energies()
    assert np.allclose(sp, g["sp_energies"], atol=1e-9, rtol=0)


def test_precondition_potential_scheme2():
    """MixingScheme 2 (PreconditionPotential): the oracle's CG solves
    (1 - preconu Lap) x = dU to sum(r^2) dv < 1e-8, and the run still
    lowers the energy."""
    p = RunParams(nx=10, ny=10, nz=10, dx=0.8, nwt=40, neutrons=12, protons=12,
                  mixing_scheme=2)
    psi, qn, en = synthetic.ho_basis(p, 20, seed=1234)
    o = O.OracleState(p, SLY4)
    o.set_spinors(psi, qn)
    o.set_energies(en)
    o.Start()
    e1 = o.Evolve(2, 0.010, 0.3)["total"]
    e2 = o.Evolve(4, 0.010, 0.3)["total"]
    assert e2 < e1


def test_mix_densities_scheme0():
    """MixingScheme 0: after UpdateDensities + MixDensities every density is
    (1 - 0.75) new + 0.75 previous."""
    p = RunParams(nx=8, ny=8, nz=8, dx=0.8, nwt=16, neutrons=4, protons=4)
    psi, qn, en = synthetic.ho_basis(p, 8, seed=3)
    o = O.OracleState(p, SLY4)
    o.set_spinors(psi, qn)
    o.set_energies(en)
    o.Start()
    prev = o.get_densities()
    o.GradDesc(0.01, 0.0)
    o.HFFill()
    o.DeriveAll()
    o.UpdateDensities()
    new = o.get_densities()
    o.MixDensities()
    mixed = o.get_densities()
    for k in mixed:
        np.testing.assert_allclose(mixed[k], 0.25 * new[k] + 0.75 * prev[k], rtol=0, atol=1e-14)


def _hf_gap(occ, e, iso):
    """relE of IterativeEstimation's HF branch (src/ImaginaryTime.f90:110-129)."""
    rel_e = 10000.0
    for i in range(len(e)):
        if abs(occ[i]) < 0.5:
            continue
        for k in range(len(e)):
            if abs(occ[k]) > 0.5 or iso[k] != iso[i]:
                continue
            if e[k] - e[i] > 0.0:
                rel_e = min(rel_e, e[k] - e[i])
    return max(rel_e, 0.1)


def test_iterative_estimation_step_parameters():
    """ParameterEstimation = 1 (src/ImaginaryTime.f90:28-211): the momentum
    gives kappa = relE / (maxE - min e) back, and dt must then equal
    0.9 * 4 hbar / (sqrt(maxE - min e) + sqrt(relE))^2 with relE the HF gap of
    the energies the estimation saw; the largest eigenvalue of h on a 0.8 fm
    mesh lies between 100 MeV and 5 GeV, and repeated runs agree bit for bit."""
    p, psi, qn, en = _mg24()
    p.parameter_estimation = 1
    runs = []
    for _ in range(2):
        o = O.OracleState(p, SLY4)
        o.set_spinors(psi, qn)
        o.set_energies(en)
        o.Start()
        o.Evolve(1, 0.010, 0.3)
        occ = o.get_occupations()
        e, _ = o.get_energies()
        o.GradDesc(0.010, 0.3)
        runs.append(o.StepParameters())
    assert runs[0] == runs[1]
    dt, mom = runs[0]
    assert 0.0 < mom < 1.0 and dt > 0.0
    rel_e = _hf_gap(occ, e, qn[:, 0])
    sk = (1.0 - math.sqrt(mom)) / (1.0 + math.sqrt(mom))
    max_e = rel_e / sk ** 2
    assert 100.0 < max_e + e.min() < 5000.0
    want = 0.9 * 4.0 * SLY4.hbar / (math.sqrt(max_e) + math.sqrt(rel_e)) ** 2
    assert dt == pytest.approx(want, rel=1e-12, abs=0)


def _rutz_numpy(rho, n, dx, dv):
    """RutzCutOff (src/Moments.f90:2703-2871) restated with numpy on an
    n^3 EV8 stored mesh: the oracle's loop form must agree with it."""
    x = dx / 2 + dx * np.arange(n)
    out = np.zeros_like(rho)
    for it in range(2):
        r = rho[it].reshape(n, n, n)            # [k][j][i], x fastest
        if dv * r.sum() < 1e-10:
            continue
        tr = r.max() / 10.0
        a = r[:-1, :-1, :-1]
        Z, Y, X = np.meshgrid(x[:-1], x[:-1], x[:-1], indexing="ij")
        pts = []
        for b, axis in ((r[:-1, :-1, 1:], 0), (r[:-1, 1:, :-1], 1), (r[1:, :-1, :-1], 2)):
            m = ((a >= tr) & (b <= tr)) | ((a <= tr) & (b >= tr))
            p = [X[m], Y[m], Z[m]]
            p[axis] = p[axis] + dx * (tr - a[m]) / (b[m] - a[m])
            pts.append(np.stack(p, axis=1))
        s = np.concatenate(pts)
        Zg, Yg, Xg = np.meshgrid(x, x, x, indexing="ij")
        g = np.stack([Xg.ravel(), Yg.ravel(), Zg.ravel()], axis=1)
        d = ((g[:, None, 0] - s[None, :, 0]) ** 2 + (g[:, None, 1] - s[None, :, 1]) ** 2
             + (g[:, None, 2] - s[None, :, 2]) ** 2).min(axis=1)
        sig = np.where(r.ravel() > tr, -1.0, 1.0)
        out[it] = 1.0 / (1.0 + np.exp((sig * np.sqrt(d) - 4.0) / 0.4))
    return out


def _constrained_start(iteration=10, target=50.0, n=10):
    p = RunParams(nx=n, ny=n, nz=n, dx=0.8, nwt=40, neutrons=12, protons=12,
                  pairing=_abi.MG_PAIRING_HFB)
    psi, qn, en = synthetic.ho_basis(p, 20, seed=1234)
    o = O.OracleState(p, SLY4)
    o.set_spinors(psi, qn)
    o.set_energies(en)
    o.set_pairing()
    k = o.add_constraint(2, 0, target, 0.0, iteration)
    o.Start()
    return p, o, k


def test_rutz_cutoff_matches_numpy_restatement():
    p, o, _ = _constrained_start()
    rho = o.get_densities()["rho"].reshape(2, -1)
    cut, field = o.get_constraint_fields()
    ref = _rutz_numpy(rho, p.nx, p.dx, 8 * p.dx ** 3)
    assert np.abs(cut.reshape(2, -1) - ref).max() < 1e-13
    assert 0.0 <= cut.min() and cut.max() <= 1.0 and cut.max() > 0.99
    # the intensity is estimated on the first readjustment: no field at the start
    assert np.abs(field).max() == 0.0


def test_q20_constraint_moves_the_moment_then_switches_off():
    """A Q20 constraint (alternating kind) for 4 iterations: the
    alternate steps and the constraint field push <Q20> from ~0 towards
    the target; afterwards the constraint is inactive and its field zero."""
    p, o, k = _constrained_start(iteration=4)
    q0 = sum(o.get_constraint(k)["value"])
    assert abs(q0) < 0.1
    o.Evolve(1, 0.010, 0.3)
    st = o.get_constraint(k)
    # Readjust: Intensity = 2 / sum(Squared), halved under momentum
    assert st["intensity"] == pytest.approx(0.5 * 2.0 / sum(st["squared"]), rel=1e-12)
    o.Evolve(3, 0.010, 0.3)
    st = o.get_constraint(k)
    assert st["active"] and sum(st["value"]) > 20.0
    assert np.abs(o.get_constraint_fields()[1]).max() > 0.0
    o.Evolve(2, 0.010, 0.3)     # iteration 5 switches it off, 6 has no field
    st = o.get_constraint(k)
    assert not st["active"]
    assert np.abs(o.get_constraint_fields()[1]).max() == 0.0


def test_nilsson_start():
    """The restated Nilsson guess (nil8 via INITWF): orthonormal inside every
    (isospin, parity) block, proton levels those of the neutrons scaled by
    the proton oscillator factor, positive parity first within each isospin,
    the s1/2 level at 1.5 hbar omega above the -50 MeV shift."""
    p = RunParams(nx=10, ny=10, nz=10, dx=0.8, nwt=40, neutrons=12, protons=12)
    psi, qn, en = synthetic.nilsson_basis(p, 20, amplitude=0.0)
    S = np.einsum("iczyx,jczyx->ij", psi, psi) * p.dv
    same = (qn[:, 0][:, None] == qn[:, 0][None, :]) & (qn[:, 1][:, None] == qn[:, 1][None, :])
    assert np.abs((S - np.eye(40)) * same).max() < 1e-13
    # N = Z: the proton oscillator is scaled by ca = 0.986 (src/nil8.f90:124, :271-274)
    assert np.allclose(en[20:] + 50.0, 0.986 * (en[:20] + 50.0), atol=1e-12)
    for iso in (-1, 1):
        par = qn[qn[:, 0] == iso, 1]
        assert np.all(np.diff(par) <= 0) and par[0] == 1
    # the lowest level is the s1/2 state, 1.5 hbar omega above -50 MeV minus
    # the l^2 shift (none for kappa mu = 0 below 50 particles)
    hw = 0.2 * 6.58218 ** 2 / 1.044673
    assert en[0] == pytest.approx(-50.0 + 1.5 * hw, abs=1e-9)
    # the perturbed start keeps the same shapes and quantum numbers
    psi2, qn2, en2 = synthetic.nilsson_basis(p, 20, seed=1234)
    assert np.array_equal(qn2, qn) and np.array_equal(en2, en)
    assert 0 < np.abs(psi2 - psi).max() < 2e-2


def test_golden_c1_fixture():
    """The README Mg24 run (Nilsson start, HFB, MixingScheme 2,
    ParameterEstimation 1, Q20 constraint for 10 iterations, 100 iterations)
    in the oracle reproduces the committed checkpoints (make_golden.py; the
    Nilsson start is rebuilt here with the same numpy)."""
    import sys
    sys.path.insert(0, str(GOLDEN))
    import make_golden
    g = json.loads((GOLDEN / "mg24_c1.json").read_text())
    d = make_golden.mg24_c1()
    for a, b in zip(d["checkpoints"], g["checkpoints"]):
        assert a["iteration"] == b["iteration"]
        assert a["E_total"] == pytest.approx(b["E_total"], abs=1e-9), a["iteration"]
        assert a["q20"] == pytest.approx(b["q20"], abs=1e-9)
        assert a["dt"] == pytest.approx(b["dt"], rel=1e-12)


def _hf_pe_run():
    p = RunParams(nx=10, ny=10, nz=10, dx=0.8, nwt=40, neutrons=12, protons=12,
                  parameter_estimation=1)
    psi, qn, en = synthetic.ho_basis(p, 20, seed=1234)
    o = O.OracleState(p, SLY4)
    o.set_spinors(psi, qn)
    o.set_energies(en)
    o.Start()
    return o


def test_convergence_check():
    """ConvergenceCheck in the oracle: an HF run (ParameterEstimation 1)
    stops once E_total changed by at most EnergyPrec (relative) against each
    of the last 7 iterations; an HFB run never passes, because ConverFermi
    compares the Fermi energies with a history the reference never fills."""
    P = _abi.MgConvergence(1e-7, 1e-4, 1e-4)
    o = _hf_pe_run()
    k = 0
    while k < 400:
        k += 1
        e = o.Evolve(1, 0.010, 0.3)
        if o.ConvergenceCheck(P):
            break
    assert k == 261, k
    assert e["total"] == pytest.approx(-195.69968851824, abs=1e-8)
    # HFB: not even a loose energy bar passes
    p = RunParams(nx=10, ny=10, nz=10, dx=0.8, nwt=40, neutrons=12, protons=12,
                  pairing=_abi.MG_PAIRING_HFB)
    psi, qn, en = synthetic.ho_basis(p, 20, seed=1234)
    h = O.OracleState(p, SLY4)
    h.set_spinors(psi, qn)
    h.set_energies(en)
    h.set_pairing()
    h.Start()
    loose = _abi.MgConvergence(1.0, 1.0, 1e-4)
    for _ in range(9):
        h.Evolve(1, 0.010, 0.3)
        assert not h.ConvergenceCheck(loose)


def test_bisection_fermi_search_finds_the_broyden_root():
    """The oracle's FermiSolver 'BISECTION' (bracketing by steps of 0.01 MeV
    times the attempt, then Brent's method to fermi_prec on lambda) lands on
    the root of its damped Broyden search (1e-10 MeV) with the particle
    numbers within 1e-9, after more evaluations (the bracket from -10 MeV)."""
    from mocca_gb300 import SLY4 as F
    p = RunParams(nx=10, ny=10, nz=10, dx=0.8, nwt=40, neutrons=12, protons=12,
                  pairing=_abi.MG_PAIRING_HFB)
    psi, qn, en = synthetic.ho_basis(p, 20, seed=5)
    out = {}
    for solver in (1, 3):
        o = O.OracleState(p, F)
        o.set_spinors(psi, qn)
        o.set_energies(en)
        pp = _abi.MgPairingParams.defaults()
        pp.fermi_solver = solver
        o.set_pairing(pp)
        out[solver] = o.SolvePairing()
        o.close()
    a, b = out[1], out[3]
    assert a["converged"] and b["converged"]
    assert b["evaluations"] > 2 * a["evaluations"] > 0
    for it in range(2):
        assert abs(a["fermi"][it] - b["fermi"][it]) < 1e-10
        assert abs(b["particles"][it] - 12.0) < 1e-9
