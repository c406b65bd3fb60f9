"""ctypes wrapper of the CPU FP64 oracle (oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's cpu_baseline leg, never by the product package.  `OracleState`
exposes the same methods as mocca_gb300.mesh.MeshState so a parity test
drives both with one script.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

from mocca_gb300 import _abi
from mocca_gb300.forces import Force, RunParams

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liboracle.so"
# -O3 OpenMP build of the same sources: timing of the CPU baseline only
LIB_OMP = HERE / "_build" / "liboracle_omp.so"

_D = _abi._D
_I = _abi._I
_P = C.c_void_p

_SIG = {
    "orc_skyrme_coefficients": ([C.POINTER(_abi.MgForce), C.c_int, C.POINTER(_abi.MgSkyrmeB)], C.c_int),
    "orc_lagrange_matrices": ([C.c_int, C.c_double, C.c_int, _D, _D], C.c_int),
    "orc_create": ([C.POINTER(_abi.MgParams), C.POINTER(_abi.MgForce)], _P),
    "orc_destroy": ([_P], None),
    "orc_set_spinors": ([_P, C.c_int, _D, _I], C.c_int),
    "orc_get_spinors": ([_P, C.c_int, _D], C.c_int),
    "orc_get_qn": ([_P, C.c_int, _I], C.c_int),
    "orc_get_derivatives": ([_P, C.c_int, _D, _D], C.c_int),
    "orc_set_occupations": ([_P, C.c_int, _D], C.c_int),
    "orc_get_occupations": ([_P, C.c_int, _D], C.c_int),
    "orc_set_energies": ([_P, C.c_int, _D], C.c_int),
    "orc_get_energies": ([_P, C.c_int, _D, _D], C.c_int),
    "orc_derive_grid": ([_P, _D, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _D], C.c_int),
    "orc_derive_basis": ([_P, C.c_int], C.c_int),
    "orc_derive_all": ([_P], C.c_int),
    "orc_hpsi": ([_P, C.c_int, _D, _D, _D], C.c_int),
    "orc_grad_desc": ([_P, C.c_double, C.c_double], C.c_int),
    "orc_get_step_parameters": ([_P, _D, _D], C.c_int),
    "orc_gram_schmidt": ([_P], C.c_int),
    "orc_hf_fill": ([_P], C.c_int),
    "orc_update_densities": ([_P], C.c_int),
    "orc_mix_densities": ([_P], C.c_int),
    "orc_get_densities": ([_P, _D, _D, _D, _D, _D], C.c_int),
    "orc_set_densities": ([_P, _D, _D, _D, _D, _D], C.c_int),
    "orc_get_jmunu": ([_P, _D], C.c_int),
    "orc_calculate_moments": ([_P], C.c_int),
    "orc_get_moments": ([_P, _D, _I, C.c_int], C.c_int),
    "orc_add_constraint": ([_P, C.POINTER(_abi.MgMomentConstraint)], C.c_int),
    "orc_get_constraint": ([_P, C.c_int, C.POINTER(_abi.MgConstraintState)], C.c_int),
    "orc_get_constraint_fields": ([_P, _D, _D], C.c_int),
    "orc_alternate_step": ([_P], C.c_int),
    "orc_readjust_moments": ([_P, C.c_int], C.c_int),
    "orc_convergence_check": ([_P, C.POINTER(_abi.MgConvergence), C.POINTER(C.c_int)], C.c_int),
    "orc_solve_coulomb": ([_P, _I], C.c_int),
    "orc_construct_potentials": ([_P, _I], C.c_int),
    "orc_get_potentials": ([_P, _D, _D, _D, _D, _D, _D, _D], C.c_int),
    "orc_set_potentials": ([_P, _D, _D, _D, _D, _D], C.c_int),
    "orc_energy": ([_P, C.POINTER(_abi.MgEnergyTerms)], C.c_int),
    "orc_iterate": ([_P, C.c_int, C.c_double, C.c_double, C.POINTER(_abi.MgEnergyTerms)], C.c_int),
    "orc_set_pairing": ([_P, C.POINTER(_abi.MgPairingParams)], C.c_int),
    "orc_solve_pairing": ([_P, C.POINTER(_abi.MgPairingInfo)], C.c_int),
    "orc_get_hfb_block": ([_P, C.c_int, _D, _D, _D], C.c_int),
    "orc_get_pairing_field": ([_P, _D, _D, _D], C.c_int),
    "orc_eigh": ([C.c_int, _D, _D, _D], C.c_int),
    "orc_set_threads": ([C.c_int], C.c_int),
    "orc_get_time_odd": ([_P, _D, _D, _D, _D, _D, _D, _D], C.c_int),
    "orc_get_time_odd_tensor": ([_P, _D, _D, _D, _D, _D, _D, _D], C.c_int),
    "orc_tensor_odd_action": ([_P, C.c_int, C.c_int, _D, _D], C.c_int),
    "orc_symmetry_operators": ([_P, C.c_int, _D], C.c_int),
}

_libs = {}


def build_oracle() -> Path:
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB


def load(timing: bool = False):
    """The parity build, or with timing=True the -O3 OpenMP build."""
    path = LIB_OMP if timing else LIB
    if path not in _libs:
        if not path.exists():
            build_oracle()
        lib = C.CDLL(str(path))
        for name, (args, res) in _SIG.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = res
        _libs[path] = lib
    return _libs[path]


def _d(a):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_D)


def lagrange_matrices(n: int, dx: float, folded: bool):
    d1 = np.empty(2 * n * n)
    d2 = np.empty(2 * n * n)
    st = load().orc_lagrange_matrices(n, dx, int(folded), _d(d1), _d(d2))
    _abi.check("orc_lagrange_matrices", st)
    return d1.reshape(2, n, n), d2.reshape(2, n, n)


class OracleState:
    def __init__(self, params: RunParams, force: Force, timing: bool = False):
        self.lib = load(timing)
        self.p = params
        self._cp = params.to_c()
        self._cf = force.to_c()
        self.h = self.lib.orc_create(C.byref(self._cp), C.byref(self._cf))
        if not self.h:
            raise ValueError("oracle does not support these parameters")

    def close(self):
        if getattr(self, "h", None):
            self.lib.orc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def V(self):
        return self.p.V

    def _call(self, name, *args, allow_not_converged=False):
        return _abi.check(name, getattr(self.lib, name)(self.h, *args), allow_not_converged)

    def set_spinors(self, psi, qn=None, basis=_abi.MG_HF_BASIS):
        psi = np.ascontiguousarray(psi, dtype=np.float64).reshape(-1)
        q = None
        if qn is not None:
            qn = np.ascontiguousarray(qn, dtype=np.int32).reshape(-1)
            q = qn.ctypes.data_as(_I)
        self._call("orc_set_spinors", basis, _d(psi), q)

    def get_spinors(self, basis=_abi.MG_HF_BASIS):
        out = np.empty(self.p.nwt * 4 * self.V)
        self._call("orc_get_spinors", basis, _d(out))
        return out.reshape(self.p.nwt, 4, self.p.nz, self.p.ny, self.p.nx)

    def get_derivatives(self, basis=_abi.MG_HF_BASIS):
        n = self.p.nwt
        der = np.empty(n * 12 * self.V)
        lap = np.empty(n * 4 * self.V)
        self._call("orc_get_derivatives", basis, _d(der), _d(lap))
        s = (self.p.nz, self.p.ny, self.p.nx)
        return der.reshape(n, 3, 4, *s), lap.reshape(n, 4, *s)

    def set_occupations(self, occ, basis=_abi.MG_HF_BASIS):
        self._call("orc_set_occupations", basis, _d(np.ascontiguousarray(occ, dtype=np.float64)))

    def get_occupations(self, basis=_abi.MG_HF_BASIS):
        out = np.empty(self.p.nwt)
        self._call("orc_get_occupations", basis, _d(out))
        return out

    def set_energies(self, e, basis=_abi.MG_HF_BASIS):
        self._call("orc_set_energies", basis, _d(np.ascontiguousarray(e, dtype=np.float64)))

    def get_energies(self, basis=_abi.MG_HF_BASIS):
        e = np.empty(self.p.nwt)
        d = np.empty(self.p.nwt)
        self._call("orc_get_energies", basis, _d(e), _d(d))
        return e, d

    def derive_grid(self, grid, direction, P, S, TS, comp):
        g = np.ascontiguousarray(grid, dtype=np.float64).reshape(-1)
        out = np.empty_like(g)
        self._call("orc_derive_grid", _d(g), direction, P, S, TS, comp, _d(out))
        return out.reshape(self.p.nz, self.p.ny, self.p.nx)

    def get_densities(self):
        V = self.V
        out = {k: np.empty(n * V) for k, n in
               (("rho", 2), ("tau", 2), ("nablaj", 2), ("derrho", 6), ("laprho", 2))}
        self._call("orc_get_densities", *(_d(out[k]) for k in
                                          ("rho", "tau", "nablaj", "derrho", "laprho")))
        return out

    def get_jmunu(self) -> np.ndarray:
        out = np.empty(18 * self.V)
        self._call("orc_get_jmunu", _d(out))
        return out

    def set_densities(self, rho=None, tau=None, nablaj=None, derrho=None, laprho=None):
        arrs = [None if a is None else np.ascontiguousarray(a, dtype=np.float64).reshape(-1)
                for a in (rho, tau, nablaj, derrho, laprho)]
        self._call("orc_set_densities", *(_d(a) for a in arrs))

    def get_potentials(self):
        V = self.V
        out = {k: np.empty(n * V) for k, n in
               (("U", 2), ("B", 2), ("nablaB", 6), ("W", 18), ("divW", 6), ("coulomb", 1),
                ("coulex", 1))}
        self._call("orc_get_potentials", *(_d(out[k]) for k in
                                           ("U", "B", "nablaB", "W", "divW", "coulomb", "coulex")))
        return out

    def SymmetryOperators(self, basis=_abi.MG_HF_BASIS):
        out = np.empty((self.p.nwt, 6))
        self._call("orc_symmetry_operators", basis, _d(out))
        return out

    def get_time_odd(self):
        V = self.V
        out = {k: np.empty(6 * V) for k in ("vecj", "vecs", "rotj", "rots", "A", "S")}
        out["divA"] = np.empty(2 * V)
        self._call("orc_get_time_odd", *(_d(out[k]) for k in
                                          ("vecj", "vecs", "rotj", "rots", "A", "S", "divA")))
        return out

    TENSOR_ODD = ("T", "F", "lapS", "gradDivS", "C", "D", "divD")

    def get_time_odd_tensor(self):
        """T, F, lap s, grad div s, C, D as [it][m][V] and div D as [it][V]."""
        V = self.V
        out = {k: np.empty((2 if k == "divD" else 6) * V) for k in self.TENSOR_ODD}
        self._call("orc_get_time_odd_tensor", *(_d(out[k]) for k in self.TENSOR_ODD))
        return out

    def tensor_odd_action(self, i, basis=_abi.MG_HF_BASIS):
        """ActionOfC and ActionOfD of spwf i (4V each)."""
        xc, xd = np.empty(4 * self.V), np.empty(4 * self.V)
        self._call("orc_tensor_odd_action", basis, i, _d(xc), _d(xd))
        return xc, xd

    def set_potentials(self, U=None, B=None, nablaB=None, W=None, divW=None):
        arrs = [None if a is None else np.ascontiguousarray(a, dtype=np.float64).reshape(-1)
                for a in (U, B, nablaB, W, divW)]
        self._call("orc_set_potentials", *(_d(a) for a in arrs))

    def get_moments(self):
        vals = np.empty(2 * 64)
        lm = np.empty(2 * 64, dtype=np.int32)
        n = self.lib.orc_get_moments(self.h, _d(vals), lm.ctypes.data_as(_I), 64)
        return vals[:2 * n].reshape(n, 2), lm[:2 * n].reshape(n, 2)

    def DeriveAll(self):
        self._call("orc_derive_all")

    def DeriveBasis(self, basis=_abi.MG_HF_BASIS):
        self._call("orc_derive_basis", basis)

    def hPsi(self, basis=_abi.MG_HF_BASIS, want_spinors=True):
        e = np.empty(self.p.nwt)
        d = np.empty(self.p.nwt)
        h = np.empty(self.p.nwt * 4 * self.V) if want_spinors else None
        self._call("orc_hpsi", basis, _d(h), _d(e), _d(d))
        if h is not None:
            h = h.reshape(self.p.nwt, 4, self.p.nz, self.p.ny, self.p.nx)
        return h, e, d

    def GradDesc(self, dt, momentum=0.0):
        self._call("orc_grad_desc", C.c_double(dt), C.c_double(momentum))

    def StepParameters(self):
        """(dt, momentum) of the last GradDesc: IterativeEstimation's when
        ParameterEstimation = 1."""
        dt, mom = C.c_double(), C.c_double()
        self._call("orc_get_step_parameters", C.byref(dt), C.byref(mom))
        return dt.value, mom.value

    def GramSchmidt(self):
        self._call("orc_gram_schmidt")

    def HFFill(self):
        self._call("orc_hf_fill")

    def UpdateDensities(self):
        self._call("orc_update_densities")

    def MixDensities(self):
        self._call("orc_mix_densities")

    def CalculateAllMoments(self):
        self._call("orc_calculate_moments")

    def add_constraint(self, l, m, constraint, intensity=0.0, iteration=-1):
        mc = _abi.MgMomentConstraint(l, m, constraint, intensity, iteration)
        k = self.lib.orc_add_constraint(self.h, C.byref(mc))
        if k < 0:
            raise _abi.MgError("orc_add_constraint", k)
        return k

    def get_constraint(self, k=0):
        st = _abi.MgConstraintState()
        self._call("orc_get_constraint", int(k), C.byref(st))
        return st.as_dict()

    def get_constraint_fields(self):
        cut, fld = np.empty(2 * self.V), np.empty(2 * self.V)
        self._call("orc_get_constraint_fields", _d(cut), _d(fld))
        return cut, fld

    def AlternateStep(self):
        self._call("orc_alternate_step")

    def ConvergenceCheck(self, prec=None) -> bool:
        conv = C.c_int(0)
        self._call("orc_convergence_check", C.byref(prec) if prec is not None else None,
                   C.byref(conv))
        return bool(conv.value)

    def ReadjustAllMoments(self, iteration):
        self._call("orc_readjust_moments", int(iteration))

    def SolveCoulomb(self):
        it = C.c_int(0)
        self._call("orc_solve_coulomb", C.byref(it), allow_not_converged=True)
        return it.value

    def ConstructPotentials(self):
        it = C.c_int(0)
        self._call("orc_construct_potentials", C.byref(it), allow_not_converged=True)
        return it.value

    def CompEnergy(self):
        e = _abi.MgEnergyTerms()
        self._call("orc_energy", C.byref(e))
        return e.as_dict()

    def Evolve(self, n_iter, dt, momentum=0.0):
        e = _abi.MgEnergyTerms()
        self._call("orc_iterate", int(n_iter), C.c_double(dt), C.c_double(momentum), C.byref(e),
                   allow_not_converged=True)
        return e.as_dict()

    def set_pairing(self, pp=None):
        pp = pp if pp is not None else _abi.MgPairingParams.defaults()
        self._call("orc_set_pairing", C.byref(pp))

    def SolvePairing(self):
        info = _abi.MgPairingInfo()
        self._call("orc_solve_pairing", C.byref(info), allow_not_converged=True)
        return info.as_dict()

    def get_hfb_block(self, b):
        N = self.lib.orc_get_hfb_block(self.h, b, None, None, None)
        if N < 0:
            raise RuntimeError("no HFB state")
        r, k, d = (np.empty(N * N) for _ in range(3))
        self.lib.orc_get_hfb_block(self.h, b, _d(r), _d(k), _d(d))
        return r.reshape(N, N), k.reshape(N, N), d.reshape(N, N)

    def get_pairing_field(self):
        V = self.V
        re, im, df = np.empty(2 * V), np.empty(2 * V), np.empty(2 * V)
        self._call("orc_get_pairing_field", _d(re), _d(im), _d(df))
        return re, im, df

    def Start(self):
        """Iteration-0 preparation of Evolve (src/Main.f90:177-231)."""
        hfb = self.p.pairing == _abi.MG_PAIRING_HFB
        if hfb:
            self.SolvePairing()
        else:
            self.HFFill()
        self.DeriveAll()
        self.UpdateDensities()
        # three times, as the reference does (src/Main.f90:219-221): the
        # moments' OldValue history then holds the start value thrice
        for _ in range(3):
            self.CalculateAllMoments()
        it = self.ConstructPotentials()
        self.CompEnergy()   # src/Main.f90:223: the energy history starts here
        if hfb:
            _, e, d = self.hPsi(_abi.MG_CAN_BASIS, want_spinors=False)
            self.set_energies(e, _abi.MG_CAN_BASIS)
        return it


def eigh(a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    n = a.shape[0]
    w = np.empty(n)
    z = np.empty((n, n))
    st = load().orc_eigh(n, _d(a), _d(w), _d(z))
    _abi.check("orc_eigh", st)
    return w, z
