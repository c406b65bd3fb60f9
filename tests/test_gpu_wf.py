"""GPU checks of the .wf bridge (mg_wf_from_context / mg_wf_to_context) and
of DiagAng's <J> (mg_angular_momentum).

Files written from a device context are parsed by the oracle's restatement
of ReadMOCCa_v1 (oracle/wf_format.py) and compared with what the context
reports through its other entry points: spinors, densities, occupations,
energies and the HFB blocks bit-exact; <J> against the oracle's
restatement of DiagAng on the downloaded derivatives (1e-12 relative);
the HF file's kappa against GuessHFBMatrices(0)'s loop.  The HFB matrices
are checked for the structure the reference's routines give them: U and V
columns chosen by HFBColumns orthonormal (1e-12) and reproducing
rho_++ = rho_-- = V V^T of the first pairing step (no mixing yet; 1e-6,
the first-order finish of the Fermi search moves rho by up to ~1e-7 after
the last evaluation); CanTransfo's columns the eigenvectors of the block
rho in DiagonaliseRhoHFB's order (1e-10).  An HF restart from the file
reproduces the writer's energy (1e-7 MeV) and then runs exactly as a
context handed the same state through the other entry points; an HFB
restart starts from the file's kappa and Fermi energies.  Without time
reversal the time-odd density records are written and read back.
"""
import numpy as np
import pytest

import wf_format as WF
from mocca_gb300 import SLY4, RunParams, _abi, synthetic
from mocca_gb300.mesh import MeshState
from mocca_gb300.wf import WavefunctionFile

pytestmark = pytest.mark.gpu


def _state(pairing=_abi.MG_PAIRING_HF, n=10, nwt=40, N=12, Z=12, seed=1234, precision=0,
           guess_kappa=True):
    p = RunParams(nx=n, ny=n, nz=n, dx=0.8, nwt=nwt, neutrons=N, protons=Z, pairing=pairing,
                  precision=precision)
    psi, qn, en = synthetic.ho_basis(p, nwt // 2, seed=seed)
    g = MeshState(p, SLY4)
    g.set_spinors(psi, qn)
    g.set_energies(en)
    if pairing == _abi.MG_PAIRING_HFB:
        g.set_pairing(_abi.MgPairingParams.defaults(guess_kappa=guess_kappa))
    return p, g


def _coords(p):
    x = 0.5 * p.dx + p.dx * np.arange(p.nx)
    y = 0.5 * p.dx + p.dx * np.arange(p.ny)
    z = 0.5 * p.dx + p.dx * np.arange(p.nz)
    Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
    return X.ravel(), Y.ravel(), Z.ravel()


def _blocks(w):
    m = w["hfb_size"]
    c = lambda a, nb: (a.reshape(nb, -1, m, 2)[..., 0] + 1j * a.reshape(nb, -1, m, 2)[..., 1])
    U = c(w["U"], 4)     # [b][col][row]
    V = c(w["V"], 4)
    R = c(w["rhohfb"], 4)
    K = c(w["kappahfb"], 4)
    T = c(w["cantransfo"], w["can_blocks"])
    cols = w["columns"].reshape(-1, m)
    return U, V, R, K, T, cols


def test_hf_file_matches_the_context(built, tmp_path):
    p, g = _state()
    g.Start()
    e = g.Evolve(6, 0.010, 0.3)
    path = tmp_path / "hf.wf"
    g.WriteMOCCa(path)
    w = WF.read_v1(path)
    V = p.nx * p.ny * p.nz
    assert w["nwt"] == p.nwt and w["trc"] == 1 and w["pc"] == 1 and w["pairing_type"] == 0
    assert w["force"] == "SLy4" and w["fd_order"] == -1 and w["coulomb_lap_order"] == 2
    assert w["energy"] == e["total"]
    psi = g.get_spinors()
    assert np.array_equal(w["grids"], psi.ravel())
    d = g.get_densities()
    assert np.array_equal(w["rho"], d["rho"].ravel())
    assert np.array_equal(w["tau"], d["tau"].ravel())
    assert np.array_equal(w["nablaj"], d["nablaj"].ravel())
    assert np.array_equal(w["derrho"], d["derrho"].ravel())
    assert np.array_equal(w["laprho"], d["laprho"].ravel())
    assert w["jmunu"].size == 0 and w["odd_records"] == 0 and w["cutoffs"].size == 0
    sr = w["spwf_real"].reshape(-1, 7)
    si = w["spwf_int"].reshape(-1, 5)
    occ = g.get_occupations()
    en, disp = g.get_energies()
    assert np.array_equal(sr[:, 0], occ) and np.array_equal(sr[:, 1], en)
    assert np.array_equal(sr[:, 2], disp)
    assert np.abs(sr[:, 3] - 1.0).max() < 1e-12          # <psi|psi> after Gram-Schmidt
    assert np.all(si[:, 4] == 1) and np.all(si[:, 1] == 1) and np.all(si[:, 3] == 1)
    # DiagAng's <J> against the restatement on the downloaded derivatives
    der, _ = g.get_derivatives()
    X, Y, Z = _coords(p)
    dv = 8 * p.dx ** 3
    for i in range(p.nwt):
        J = WF.diag_ang(psi[i].reshape(4, V), der[i].reshape(3, 4, V), X, Y, Z, dv, True, True)
        assert np.abs(sr[i, 4:7] - J).max() <= 1e-12 * max(1.0, np.abs(J).max()), i
    assert np.abs(sr[:, 6]).max() > 0.1      # Omega = Jz of the HO start is not zero
    # GuessHFBMatrices(0): blocks (P, it) of stored spwfs then their partners
    par = si[:, 2]
    iso = si[:, 0]
    sigs = []
    for b in range(4):
        P, it = b % 2, b // 2
        k = int(np.sum((par == 2 * P - 1) & (iso == 2 * it - 1)))
        sigs.append([1] * k + [-1] * k)
        assert w["blocksizes"][b] == 2 * k
    assert np.array_equal(w["kappahfb"], WF.guess_hf_kappa(sigs, w["hfb_size"]))
    assert w["can_blocks"] == 4 and not w["cantransfo"].any() and not w["U"].any()
    g.close()


def test_hfb_file_structure(built, tmp_path):
    p, g = _state(_abi.MG_PAIRING_HFB, seed=5)
    g.Start()                       # the first pairing step: rho not mixed yet
    path = tmp_path / "hfb.wf"
    g.WriteMOCCa(path)
    w = WF.read_v1(path)
    assert w["pairing_type"] == 2 and w["has_cutoffs"] and w["cutoffs"].size == p.nwt
    assert np.all(w["cutoffs"] > 0) and np.all(w["cutoffs"] <= 1)
    U, V, R, K, T, cols = _blocks(w)
    for M in (U, V, R, K, T):
        assert not M.imag.any()
    for b in range(4):
        N = int(w["blocksizes"][b])
        h = N // 2
        rho, kap, _ = g.get_hfb_block(b)
        assert np.array_equal(R[b][:N, :N].real.T, rho)       # [col][row] -> row-major
        assert np.array_equal(K[b][:N, :N].real.T, kap)
        # HFBColumns with signature: 2N, 2N-1, ..., then h+1 ... N
        c = cols[b]
        assert list(c[:h]) == [2 * N - i for i in range(h)]
        assert list(c[h:N]) == list(range(h + 1, N + 1)) and not c[N:].any()
        sel = c[:N] - 1
        Ub = U[b][sel, :N].real.T              # rows x chosen columns
        Vb = V[b][sel, :N].real.T
        A = np.vstack([Ub, Vb])
        assert np.abs(A.T @ A - np.eye(N)).max() < 1e-12, b
        rv = Vb @ Vb.T
        assert np.abs(rv - rho).max() < 1e-6, (b, np.abs(rv - rho).max())
        # CanTransfo: negative-signature eigenvectors first, then positive,
        # each ascending; both halves share the vectors under time reversal
        Tb = T[b][:N, :N].real.T               # rows x columns
        assert np.array_equal(Tb[h:, :h], Tb[:h, h:]) and not Tb[:h, :h].any()
        Q = Tb[:h, h:]
        occ = np.diag(Q.T @ rho[:h, :h] @ Q)
        assert np.abs(rho[:h, :h] @ Q - Q * occ).max() < 1e-10, b
        assert np.abs(Q.T @ Q - np.eye(h)).max() < 1e-10
        assert np.all(np.diff(occ) >= -1e-12)
    g.close()


def test_hf_restart(built, tmp_path):
    """The file carries everything the restart needs: a restart from it runs
    exactly as a context given the writer's spinors, quantum numbers,
    energies, occupations and densities through the other entry points.
    Neither keeps the writer's GradDesc momentum history (the reference's
    file has none), so both leave the writer's own trajectory."""
    p, a = _state(seed=7)
    a.Start()
    a.Evolve(20, 0.010, 0.3)
    ea = a.CompEnergy()["total"]
    path = tmp_path / "r.wf"
    a.WriteMOCCa(path)
    _, b = _state(seed=99)              # other spinors, replaced by the file's
    hdr = b.ReadMOCCa(path)
    assert hdr["energy"] == ea
    b.Start(recalc=False)
    eb = b.CompEnergy()["total"]
    assert abs(eb - ea) < 1e-7, (ea, eb)
    c = MeshState(p, SLY4)
    qn = WF.read_v1(path)["spwf_int"].reshape(-1, 5)[:, [0, 2, 3, 1]].astype(np.int32)
    c.set_spinors(a.get_spinors(), qn)
    c.set_energies(a.get_energies()[0])
    c.set_occupations(a.get_occupations())
    d = a.get_densities()
    c.set_densities(**d)
    c.Start(recalc=False)
    assert c.CompEnergy()["total"] == eb
    fb = b.Evolve(10, 0.010, 0.3)["total"]
    fc = c.Evolve(10, 0.010, 0.3)["total"]
    fa = a.Evolve(10, 0.010, 0.3)["total"]
    print("restart HF", ea, eb, fa, fb, fc)
    assert fb == fc, (fb, fc)
    assert fb < eb and abs(fa - fb) < 0.5, (fa, fb)
    for s in (a, b, c):
        s.close()


def test_hfb_restart(built, tmp_path):
    """The pairing step after the restart is the writer's next pairing step:
    the same kappa and Fermi energies (the file's), the same spinors and
    densities.  Only the rho mixing differs, as in the reference: the
    restarted context has no history yet (OldRhoHFB = 0 until its first
    step), so rho_writer = mix rho_restart + (1 - mix) rho_file."""
    p, a = _state(_abi.MG_PAIRING_HFB, seed=5)
    a.Start()
    a.Evolve(20, 0.010, 0.3)
    path = tmp_path / "r.wf"
    a.WriteMOCCa(path)
    w = WF.read_v1(path)
    _, b = _state(_abi.MG_PAIRING_HFB, seed=11, guess_kappa=False)
    b.ReadMOCCa(path)
    ia, ib = a.SolvePairing(), b.SolvePairing()
    assert ia["converged"] and ib["converged"]
    for it in range(2):
        assert abs(ia["fermi"][it] - ib["fermi"][it]) < 1e-9, (ia["fermi"], ib["fermi"])
        assert abs(ia["pairing_energy"][it] - ib["pairing_energy"][it]) < 1e-8
    mix = _abi.MgPairingParams.defaults().mix
    _, _, R, _, _, _ = _blocks(w)
    for k in range(4):
        ra, ka, _ = a.get_hfb_block(k)
        rb, kb, _ = b.get_hfb_block(k)
        N = ra.shape[0]
        assert np.abs(ka - kb).max() < 1e-9, k
        rf = R[k][:N, :N].real.T
        assert np.abs(ra - (mix * rb + (1 - mix) * rf)).max() < 1e-9, k
    # and the restarted run goes on from there
    _, c = _state(_abi.MG_PAIRING_HFB, seed=11, guess_kappa=False)
    c.ReadMOCCa(path)
    c.Start(recalc=False)
    ec = c.CompEnergy()["total"]
    fa = a.Evolve(10, 0.010, 0.3)["total"]
    fc = c.Evolve(10, 0.010, 0.3)["total"]
    print("restart HFB", w["energy"], ec, fa, fc)
    assert abs(fa - fc) < 0.5, (fa, fc)
    # a context whose pairing step already ran takes no restart
    with pytest.raises(_abi.MgError):
        WavefunctionFile.load(path).to_state(a)
    for s_ in (a, b, c):
        s_.close()


def test_restart_refuses_another_mesh(built, tmp_path):
    p, a = _state()
    a.Start()
    a.WriteMOCCa(tmp_path / "m.wf")
    q = RunParams(nx=12, ny=12, nz=12, dx=0.8, nwt=40, neutrons=12, protons=12)
    b = MeshState(q, SLY4)
    with pytest.raises(_abi.MgError):
        b.ReadMOCCa(tmp_path / "m.wf")
    a.close()
    b.close()


def test_angular_momentum_mixed_derivatives(built):
    """<J> from the double-float derivatives of the mixed form agrees with
    the FP64 path to the double-float rounding."""
    p, g = _state(precision=_abi.MG_MIXED)
    g.Start()
    g.Evolve(3, 0.010, 0.3)
    jm = g.AngularMomentum()
    g.set_precision(_abi.MG_FP64)
    jd = g.AngularMomentum()
    assert np.abs(jm - jd).max() < 1e-9 * max(1.0, np.abs(jd).max())
    assert np.abs(jd[:, :2]).max() == 0.0      # signature conserved: Jx = Jy = 0
    g.close()


@pytest.mark.parametrize("tensor", [False, True])
def test_time_odd_records(built, tmp_path, tensor):
    """Without time reversal (cranked about z) the file carries the time-odd
    density records WriteDensity writes: j and rot j; s, rot s and DerS;
    with SLy5colo's tensor terms also lap s, div s (zero: the reference
    never assigns it) and grad div s, T and F; each bit-exact with the
    context's read-outs.  DerS is zero after SLy4's linearly mixed
    iteration (the mixing carries it only beside lap s) and d_a s_m of the
    current s (1e-12 against the oracle's Lagrange derivative) with lap s.
    A restart from the file takes every time-odd density back bit-exact."""
    import oracle as O
    from mocca_gb300.forces import SLY5_TENSOR
    from test_oracle_time_odd import cranked_start
    force = SLY5_TENSOR if tensor else SLY4
    _, _, p, (psi, qn, en) = cranked_start(0.5)
    a = MeshState(p, force)
    a.set_spinors(psi, qn)
    a.set_energies(en)
    a.Start()
    a.Evolve(3, 0.010, 0.3)
    V = a.V
    path = tmp_path / "odd.wf"
    a.WriteMOCCa(path)
    with WavefunctionFile.load(path) as w:
        h, arr = w.header, w.arrays()
    t = a.get_time_odd()
    assert h["odd_records"] == (31 if tensor else 3)
    assert np.array_equal(arr["odd1"], np.concatenate([t["vecj"], t["rotj"]]))
    assert np.array_equal(arr["odd2"][:12 * V], np.concatenate([t["vecs"], t["rots"]]))
    ders = arr["odd2"][12 * V:].reshape(2, 3, 3, V)
    if tensor:
        tt = a.get_time_odd_tensor()
        assert np.array_equal(arr["odd3"], np.concatenate([tt["lapS"], np.zeros(2 * V),
                                                           tt["gradDivS"]]))
        assert np.array_equal(arr["odd4"], tt["T"])
        assert np.array_equal(arr["odd5"], tt["F"])
        o = O.OracleState(p, force)
        s = t["vecs"].reshape(2, 3, V)
        for it in range(2):
            for m in range(3):
                for d in range(3):
                    r = o.derive_grid(s[it, m], d, 1, 1 if m == 2 else -1, 1,
                                      2 if m == 1 else 1).reshape(-1)
                    err = np.abs(ders[it, m, d] - r).max() / np.abs(r).max()
                    assert err <= 1e-12, (it, m, d, err)
        o.close()
    else:
        assert not ders.any() and arr["odd3"].size == arr["odd4"].size == arr["odd5"].size == 0
    b = MeshState(p, force)
    b.set_spinors(psi, qn)
    b.ReadMOCCa(path)
    tb = b.get_time_odd()
    for k in ("vecj", "vecs", "rotj", "rots"):
        assert np.array_equal(tb[k], t[k]), k
    if tensor:
        ttb = b.get_time_odd_tensor()
        for k in ("T", "F", "lapS", "gradDivS"):
            assert np.array_equal(ttb[k], tt[k]), k
    a.close()
    b.close()
