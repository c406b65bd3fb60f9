"""Host-side mirror of the reference's module procedures for the hot path.

`MeshState` owns one libmocca_gpu context.  Its methods carry the names of
the Fortran procedures they replace, with the same argument meaning, and
every one of them runs on the GPU through the C ABI:

    DeriveAll          src/SpwfStorage.f90:586-604
    hPsi               src/ImaginaryTime.f90:213-304   (whole basis)
    GradDesc           src/ImaginaryTime.f90:439-500
    GramSchmidt        src/SpwfStorage.f90:372-480
    HFFill             src/HartreeFock.f90:177-260     (NaiveFill)
    UpdateDensities    src/Densities.f90:406-550
    CalculateAllMoments src/Moments.f90:2250-2334      (electric moments)
    SolveCoulomb       src/Coulomb.f90:255-346
    ConstructPotentials src/PotentialMixing.f90:17-201
    CompEnergy         src/Energy.f90:62-179
    Evolve             src/Main.f90:255-328            (n passes of the loop body)
    WriteMOCCa         src/InOut.f90:905-1046          (.wf version 1)
    ReadMOCCa          src/InOut.f90:1050-1416         (restart from .wf)

`Batch` runs many independent instances (one MeshState each) concurrently
through mg_batch_*.

A non-zero status raises `MgError` (the reference stops through stp()).
Arrays follow the reference's memory order: a spinor batch is
[nwt, 4, nz, ny, nx] float64, fields are [it, ..., nz, ny, nx].
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi
from .forces import Force, RunParams


def _dptr(a: np.ndarray | None):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_abi._D)


class MeshState:
    def __init__(self, params: RunParams, force: Force, stream=None):
        self.lib = _abi.load()
        self.p = params
        self.force = force
        self._cp = params.to_c()
        self._cf = force.to_c()
        h = C.c_void_p()
        st = self.lib.mg_create(C.byref(self._cp), C.byref(self._cf),
                                C.c_void_p(stream) if stream else None, C.byref(h))
        _abi.check("mg_create", st)
        self.h = h

    # ---- lifetime -----------------------------------------------------------
    def close(self):
        if getattr(self, "h", None):
            self.lib.mg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def launch_count(self) -> int:
        """Kernels this context has launched (mg_launch_count)."""
        n = C.c_longlong(0)
        self._call("mg_launch_count", C.byref(n))
        return n.value

    PHASES = ("grad_desc", "pairing_mesh", "fermi", "canonical", "derive", "hpsi_can",
              "densities", "moments", "potentials", "energy", "side_derive")

    def set_phase_timing(self, on: bool = True):
        """Per-phase CUDA-event timing of the following Evolve passes
        (mg_set_phase_timing; clears the totals)."""
        self._call("mg_set_phase_timing", 1 if on else 0)

    def phase_times(self) -> dict:
        """Average device ms per timed pass of each phase (mg_get_phase_times);
        side_derive overlaps the pairing phases on the side stream."""
        ms = np.zeros(len(self.PHASES))
        n = C.c_longlong(0)
        self._call("mg_get_phase_times", _dptr(ms), len(ms), C.byref(n))
        out = {k: float(v) / max(1, n.value) for k, v in zip(self.PHASES, ms)}
        out["passes"] = n.value
        return out

    def set_precision(self, precision: int):
        """MG_FP64 or MG_MIXED for the following calls (mixed iterations, FP64 polish)."""
        self._call("mg_set_precision", precision)

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def V(self) -> int:
        return self.p.V

    def _call(self, name, *args, allow_not_converged=False):
        return _abi.check(name, getattr(self.lib, name)(self.h, *args), allow_not_converged)

    def synchronize(self):
        self._call("mg_synchronize")

    # ---- transfers ---------------------------------------------------------------
    def set_spinors(self, psi: np.ndarray, qn: np.ndarray | None = None,
                    basis: int = _abi.MG_HF_BASIS):
        psi = np.ascontiguousarray(psi, dtype=np.float64).reshape(self.p.nwt, -1)
        ptrs = (C.c_void_p * self.p.nwt)(*[psi[i].ctypes.data for i in range(self.p.nwt)])
        q = None
        if qn is not None:
            qn = np.ascontiguousarray(qn, dtype=np.int32).reshape(-1)
            q = qn.ctypes.data_as(_abi._I)
        self._keep = psi
        self._call("mg_upload_spinors", basis, ptrs, q, 0, self.p.nwt)
        self.synchronize()

    def get_spinors(self, basis: int = _abi.MG_HF_BASIS) -> np.ndarray:
        out = np.empty((self.p.nwt, 4 * self.V))
        ptrs = (C.c_void_p * self.p.nwt)(*[out[i].ctypes.data for i in range(self.p.nwt)])
        self._call("mg_download_spinors", basis, ptrs, 0, self.p.nwt)
        return out.reshape(self.p.nwt, 4, self.p.nz, self.p.ny, self.p.nx)

    def get_derivatives(self, basis: int = _abi.MG_HF_BASIS):
        n = self.p.nwt
        der = np.empty((n, 12 * self.V))
        lap = np.empty((n, 4 * self.V))
        dp = (C.c_void_p * n)(*[der[i].ctypes.data for i in range(n)])
        lp = (C.c_void_p * n)(*[lap[i].ctypes.data for i in range(n)])
        self._call("mg_download_derivatives", basis, dp, lp, 0, n)
        s = (self.p.nz, self.p.ny, self.p.nx)
        return der.reshape(n, 3, 4, *s), lap.reshape(n, 4, *s)

    def set_occupations(self, occ, basis: int = _abi.MG_HF_BASIS):
        occ = np.ascontiguousarray(occ, dtype=np.float64)
        self._call("mg_set_occupations", basis, _dptr(occ))

    def get_occupations(self, basis: int = _abi.MG_HF_BASIS) -> np.ndarray:
        out = np.empty(self.p.nwt)
        self._call("mg_get_occupations", basis, _dptr(out))
        return out

    def set_energies(self, e, basis: int = _abi.MG_HF_BASIS):
        e = np.ascontiguousarray(e, dtype=np.float64)
        self._call("mg_set_energies", basis, _dptr(e))

    def get_energies(self, basis: int = _abi.MG_HF_BASIS):
        e = np.empty(self.p.nwt)
        d = np.empty(self.p.nwt)
        self._call("mg_get_energies", basis, _dptr(e), _dptr(d))
        return e, d

    def get_densities(self) -> dict:
        V = self.V
        out = {k: np.empty(n * V) for k, n in
               (("rho", 2), ("tau", 2), ("nablaj", 2), ("derrho", 6), ("laprho", 2))}
        self._call("mg_get_densities", *(_dptr(out[k]) for k in
                                         ("rho", "tau", "nablaj", "derrho", "laprho")))
        return out

    def get_jmunu(self) -> np.ndarray:
        """J_{mu nu} [it][nu][mu][V] (forces with J^2 terms only)."""
        out = np.empty(18 * self.V)
        self._call("mg_get_jmunu", _dptr(out))
        return out

    def set_densities(self, rho=None, tau=None, nablaj=None, derrho=None, laprho=None):
        arrs = [None if a is None else np.ascontiguousarray(a, dtype=np.float64).reshape(-1)
                for a in (rho, tau, nablaj, derrho, laprho)]
        self._call("mg_set_densities", *(_dptr(a) for a in arrs))

    def get_potentials(self) -> dict:
        V = self.V
        out = {k: np.empty(n * V) for k, n in
               (("U", 2), ("B", 2), ("nablaB", 6), ("W", 18), ("divW", 6), ("coulomb", 1),
                ("coulex", 1))}
        self._call("mg_get_potentials", *(_dptr(out[k]) for k in
                                          ("U", "B", "nablaB", "W", "divW", "coulomb", "coulex")))
        return out

    def SymmetryOperators(self, basis: int = _abi.MG_HF_BASIS) -> np.ndarray:
        """Per spwf: isospin, signature, parity, time simplex, x-simplex
        expectation values and the RMS radius (mg_symmetry_operators)."""
        out = np.empty((self.p.nwt, 6))
        self._call("mg_symmetry_operators", int(basis), _dptr(out))
        return out

    def get_time_odd(self) -> dict:
        """Time-odd densities and fields without time reversal (mg_get_time_odd):
        vecj, vecs, rotj, rots, A, S as [it][m][V], divA as [it][V]."""
        V = self.V
        out = {k: np.empty(6 * V) for k in ("vecj", "vecs", "rotj", "rots", "A", "S")}
        out["divA"] = np.empty(2 * V)
        self._call("mg_get_time_odd", *(_dptr(out[k]) for k in
                                         ("vecj", "vecs", "rotj", "rots", "A", "S", "divA")))
        return out

    TENSOR_ODD = ("T", "F", "lapS", "gradDivS", "C", "D", "divD")

    def get_time_odd_tensor(self) -> dict:
        """Time-odd tensor densities and fields without time reversal
        (mg_get_time_odd_tensor): T, F, lap s, grad div s, C, D as [it][m][V],
        div D as [it][V]."""
        V = self.V
        out = {k: np.empty((2 if k == "divD" else 6) * V) for k in self.TENSOR_ODD}
        self._call("mg_get_time_odd_tensor", *(_dptr(out[k]) for k in self.TENSOR_ODD))
        return out

    def set_potentials(self, U=None, B=None, nablaB=None, W=None, divW=None):
        arrs = [None if a is None else np.ascontiguousarray(a, dtype=np.float64).reshape(-1)
                for a in (U, B, nablaB, W, divW)]
        self._call("mg_set_potentials", *(_dptr(a) for a in arrs))

    # ---- reference procedures ----------------------------------------------------
    def DeriveAll(self):
        self._call("mg_derive_all")

    def DeriveBasis(self, basis: int = _abi.MG_HF_BASIS):
        self._call("mg_derive_basis", basis)

    def hPsi(self, basis: int = _abi.MG_HF_BASIS, want_spinors: bool = True):
        e = np.empty(self.p.nwt)
        d = np.empty(self.p.nwt)
        h = np.empty((self.p.nwt, 4 * self.V)) if want_spinors else None
        self._call("mg_hpsi", basis, _dptr(h), _dptr(e), _dptr(d))
        if h is not None:
            h = h.reshape(self.p.nwt, 4, self.p.nz, self.p.ny, self.p.nx)
        return h, e, d

    def GradDesc(self, dt: float, momentum: float = 0.0):
        self._call("mg_grad_desc", C.c_double(dt), C.c_double(momentum))

    def StepParameters(self) -> tuple[float, float]:
        """(dt, momentum) of the last GradDesc: IterativeEstimation's estimate
        (src/ImaginaryTime.f90:28-211) when ParameterEstimation = 1."""
        dt, mom = C.c_double(), C.c_double()
        self._call("mg_get_step_parameters", C.byref(dt), C.byref(mom))
        return dt.value, mom.value

    def GramSchmidt(self):
        self._call("mg_gram_schmidt")

    def HFFill(self):
        self._call("mg_hf_fill")

    def UpdateDensities(self):
        self._call("mg_update_densities")

    def MixDensities(self):
        self._call("mg_mix_densities")

    def CalculateAllMoments(self):
        self._call("mg_calculate_moments")

    def add_constraint(self, l: int, m: int, constraint: float, intensity: float = 0.0,
                       iteration: int = -1) -> int:
        """&MomentConstraint l, m, Constraint, Intensity, iteration (alternating kind)."""
        mc = _abi.MgMomentConstraint(l, m, constraint, intensity, iteration)
        k = self.lib.mg_add_constraint(self.h, C.byref(mc))
        if k < 0:
            raise _abi.MgError("mg_add_constraint", k)
        return k

    def get_constraint(self, k: int = 0) -> dict:
        st = _abi.MgConstraintState()
        self._call("mg_get_constraint", int(k), C.byref(st))
        return st.as_dict()

    def get_constraint_fields(self):
        cut, fld = np.empty(2 * self.V), np.empty(2 * self.V)
        self._call("mg_get_constraint_fields", _dptr(cut), _dptr(fld))
        return cut, fld

    def AlternateStep(self):
        self._call("mg_alternate_step")

    def ReadjustAllMoments(self, iteration: int):
        self._call("mg_readjust_moments", int(iteration))

    def SolveCoulomb(self) -> int:
        it = C.c_int(0)
        self._call("mg_solve_coulomb", C.byref(it), allow_not_converged=True)
        return it.value

    def reset_coulomb_guess(self):
        """The Coulomb potential back to InitialGuess (mg_coulomb_reset)."""
        self._call("mg_coulomb_reset")

    def CoulombResidual(self) -> float:
        """|b - L phi| / |b| of the last Coulomb solve (mg_coulomb_residual)."""
        r = C.c_double(0.0)
        self._call("mg_coulomb_residual", C.byref(r))
        return r.value

    def ConstructPotentials(self) -> int:
        it = C.c_int(0)
        self._call("mg_construct_potentials", C.byref(it), allow_not_converged=True)
        return it.value

    def CompEnergy(self) -> dict:
        e = _abi.MgEnergyTerms()
        self._call("mg_energy", C.byref(e))
        return e.as_dict()

    def Evolve(self, n_iter: int, dt: float, momentum: float = 0.0) -> dict:
        e = _abi.MgEnergyTerms()
        self._call("mg_iterate", int(n_iter), C.c_double(dt), C.c_double(momentum), C.byref(e),
                   allow_not_converged=True)
        return e.as_dict()

    def ConvergenceCheck(self, prec=None) -> bool:
        """ConvergenceCheck (src/Main.f90:358-397); prec: MgConvergence or None."""
        conv = C.c_int(0)
        self._call("mg_convergence_check", C.byref(prec) if prec is not None else None,
                   C.byref(conv))
        return bool(conv.value)

    def EvolveUntilConverged(self, max_iter: int, dt: float, momentum: float = 0.0,
                             prec=None):
        """The Evolve loop with its convergence exit (mg_evolve): returns
        (energy terms, iterations run, converged)."""
        e = _abi.MgEnergyTerms()
        n, conv = C.c_int(0), C.c_int(0)
        self._call("mg_evolve", int(max_iter), C.c_double(dt), C.c_double(momentum),
                   C.byref(prec) if prec is not None else None, C.byref(n), C.byref(conv),
                   C.byref(e), allow_not_converged=True)
        return e.as_dict(), n.value, bool(conv.value)

    def set_pairing(self, pp=None):
        """&Pairing values of an HFB run (defaults: the Mg24 example input of the reference's README.md)."""
        pp = pp if pp is not None else _abi.MgPairingParams.defaults()
        self._call("mg_set_pairing", C.byref(pp))

    def SolvePairing(self) -> dict:
        info = _abi.MgPairingInfo()
        self._call("mg_solve_pairing", C.byref(info), allow_not_converged=True)
        return info.as_dict()

    def get_hfb_block(self, b: int):
        N = self.lib.mg_get_hfb_block(self.h, b, None, None, None)
        if N < 0:
            raise _abi.MgError("mg_get_hfb_block", N)
        r, k, d = (np.empty(N * N) for _ in range(3))
        self.lib.mg_get_hfb_block(self.h, b, _dptr(r), _dptr(k), _dptr(d))
        return r.reshape(N, N), k.reshape(N, N), d.reshape(N, N)

    def get_pairing_field(self):
        V = self.V
        re, im, df = np.empty(2 * V), np.empty(2 * V), np.empty(2 * V)
        self._call("mg_get_pairing_field", _dptr(re), _dptr(im), _dptr(df))
        return re, im, df

    def NilssonStart(self, n_neutron: int, meven: int = 6, modd: int = 5, ho=(0.2, 0.2, 0.2),
                     amplitude: float = 0.0, seed: int = 1234):
        """INITWF's Nilsson states (src/InOut.f90:1418-1473, src/nil8.f90:16-546)
        built on the device, plus a seeded uniform perturbation of the given
        amplitude and the normalisation of every spwf."""
        npar = _abi.MgNilssonParams()
        npar.n_neutron, npar.meven, npar.modd = n_neutron, meven, modd
        for k in range(3):
            npar.ho[k] = float(ho[k])
        npar.amplitude, npar.seed = float(amplitude), int(seed)
        self._call("mg_nilsson_start", C.byref(npar))

    def BreakSymmetries(self, full: "MeshState"):
        """BreakParity, BreakSignature, BreakTimeSimplex (src/Transform.f90:
        187-366) of this EV8 state's HF spwfs into `full`, a symmetry-free
        state with twice the points per axis."""
        self._call("mg_break_symmetries", full.h)

    def AngularMomentum(self, basis: int = _abi.MG_HF_BASIS) -> np.ndarray:
        """DiagAng's <J> (src/Spwf.f90:976-1085) per spwf, [nwt, 3]."""
        out = np.empty(3 * self.p.nwt)
        self._call("mg_angular_momentum", basis, _dptr(out))
        return out.reshape(self.p.nwt, 3)

    def WriteMOCCa(self, path, force_name: str | None = None):
        """WriteMOCCa_v1 (src/InOut.f90:905-1046): this state as a version-1
        .wf file."""
        from .wf import WavefunctionFile
        with WavefunctionFile.from_state(self, force_name) as w:
            w.save(path)

    def ReadMOCCa(self, path) -> dict:
        """ReadMOCCa_v1 + Input (src/InOut.f90:1050-1416, :123-192): restart
        from a .wf file with this state's mesh, symmetries and nwt (under HFB
        after set_pairing, before the first pairing step); returns the file's
        header.  Follow with Start()."""
        from .wf import WavefunctionFile
        with WavefunctionFile.load(path) as w:
            w.to_state(self)
            return w.header

    def Start(self, recalc: bool = True):
        """Iteration-0 preparation of Evolve (src/Main.f90:177-231) for a run
        started from spinors with given energies: pairing step (HF filling or
        HFB), derivatives, densities, moments, potentials and, under HFB, the
        canonical single-particle energies.  recalc=False keeps the densities
        already set (a restart from a .wf file without Recalc,
        src/Main.f90:213-215)."""
        hfb = self.p.pairing == _abi.MG_PAIRING_HFB
        if hfb:
            self.SolvePairing()
        else:
            self.HFFill()
        self.DeriveAll()
        if recalc:
            self.UpdateDensities()
        # three times, as the reference does (src/Main.f90:219-221): the
        # moments' OldValue history then holds the start value thrice
        for _ in range(3):
            self.CalculateAllMoments()
        it = self.ConstructPotentials()
        self.CompEnergy()   # src/Main.f90:223: the energy history starts here
        if hfb:
            self.hPsi(_abi.MG_CAN_BASIS, want_spinors=False)
        return it


class Batch:
    """Independent instances run concurrently (mg_batch_*): each MeshState
    keeps its own mesh, spwf count, particle numbers and constraints; host
    worker threads drive them, each on its own streams.  The states stay
    owned by the caller and must be prepared (spinors, pairing, constraints,
    Start) before they are batched."""

    def __init__(self, states: list[MeshState]):
        self.lib = _abi.load()
        self.states = list(states)
        arr = (C.c_void_p * len(self.states))(*[s.h.value for s in self.states])
        h = C.c_void_p()
        _abi.check("mg_batch_create", self.lib.mg_batch_create(len(self.states), arr, C.byref(h)))
        self.h = h

    def _vec(self, x) -> np.ndarray:
        a = np.ascontiguousarray(np.broadcast_to(np.asarray(x, dtype=np.float64),
                                                 (len(self.states),)))
        return a

    def tune(self, probe: int, dt, momentum) -> int:
        """Schedule autotuner (mg_batch_tune); its passes advance every
        instance.  Returns the chosen worker count."""
        d, m = self._vec(dt), self._vec(momentum)
        w = C.c_int(0)
        _abi.check("mg_batch_tune", self.lib.mg_batch_tune(self.h, int(probe), _dptr(d), _dptr(m),
                                                            C.byref(w)))
        return w.value

    def set_workers(self, workers: int) -> int:
        w = self.lib.mg_batch_set_workers(self.h, int(workers))
        if w < 0:
            raise _abi.MgError("mg_batch_set_workers", w)
        return w

    def Evolve(self, n_iter: int, dt, momentum, allow_failures: bool = False) -> list[dict]:
        """n_iter passes of every instance; a failed instance is skipped from
        then on (see status()); with allow_failures the call returns instead
        of raising when one fails."""
        d, m = self._vec(dt), self._vec(momentum)
        out = (_abi.MgEnergyTerms * len(self.states))()
        st = self.lib.mg_batch_iterate(self.h, int(n_iter), _dptr(d), _dptr(m), out)
        if st < 0 and not allow_failures:
            raise _abi.MgError("mg_batch_iterate", st)
        return [e.as_dict() for e in out]

    def status(self) -> list[int]:
        """Per-instance status after the last call (negative: failed, skipped)."""
        st = np.zeros(len(self.states), dtype=np.int32)
        _abi.check("mg_batch_status", self.lib.mg_batch_status(self.h, st.ctypes.data_as(_abi._I)))
        return st.tolist()

    def close(self):
        if getattr(self, "h", None):
            self.lib.mg_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
