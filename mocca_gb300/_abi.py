"""ctypes declarations of the C ABI in include/mocca_gpu.h and include/mocca_wf.h.

The structures mirror the header field by field; `load()` opens the in-tree
libmocca_gpu.so and declares every entry point's signature.  No compute
happens here and nothing falls back to another implementation: when the
library is missing, `load()` raises.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

MG_OK = 0
MG_NOT_CONVERGED = 1
MG_ERR_ARG = -1
MG_ERR_CUDA = -2
MG_ERR_STATE = -3
MG_ERR_TIMEOUT = -4
MG_ERR_NAN = -5
MG_ERR_IO = -6

MG_FP64 = 0
MG_MIXED = 1
MG_HF_BASIS = 0
MG_CAN_BASIS = 1
MG_PAIRING_HF = 0
MG_PAIRING_HFB = 2

STATUS_NAMES = {
    MG_OK: "ok", MG_NOT_CONVERGED: "not converged", MG_ERR_ARG: "invalid argument",
    MG_ERR_CUDA: "CUDA error", MG_ERR_STATE: "call out of order",
    MG_ERR_TIMEOUT: "device wait timed out", MG_ERR_NAN: "NaN detected",
    MG_ERR_IO: "wavefunction file missing, unreadable or not version 1",
}


class MgParams(C.Structure):
    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
        ("dx", C.c_double),
        ("pc", C.c_int), ("sc", C.c_int), ("tsc", C.c_int), ("trc", C.c_int),
        ("nwt", C.c_int),
        ("neutrons", C.c_double), ("protons", C.c_double),
        ("precision", C.c_int),
        ("pairing", C.c_int),
        ("coulomb_max", C.c_int),
        ("max_l_coul", C.c_int),
        ("coulomb_solver", C.c_int),
        ("mixing_scheme", C.c_int),
        ("damping", C.c_double),
        ("precon_u", C.c_double),
        ("parameter_estimation", C.c_int),
        ("coulomb_prec", C.c_double),
        ("omega", C.c_double * 3),
        ("precon_w", C.c_double),
    ]


class MgForce(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "t0", "x0", "t1", "x1", "t2", "x2", "t3a", "x3a", "yt3a", "t3b", "x3b", "yt3b",
        "te", "to", "wso", "wsoq", "hbm", "e2", "hbar")] + [
        ("nucleonmass", C.c_double * 2),
        ("com1body", C.c_int), ("com2body", C.c_int), ("cexchange", C.c_int),
        ("j2terms", C.c_int), ("coupling", C.c_int),
    ]


class MgSkyrmeB(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "B1", "B2", "B3", "B4", "B5", "B6", "B7a", "B7b", "B8a", "B8b", "byt3a", "byt3b",
        "B9", "B9q", "B10", "B11", "B12a", "B12b", "B13a", "B13b", "B14", "B15", "B16",
        "B17", "B18", "B19", "B20", "B21")]


class MgPairingParams(C.Structure):
    _fields_ = [
        ("strength", C.c_double * 2), ("alpha", C.c_double * 2), ("rhosat", C.c_double),
        ("cut", C.c_double * 2), ("mu", C.c_double * 2), ("mix", C.c_double),
        ("fermi_prec", C.c_double), ("max_iter", C.c_int), ("guess_kappa", C.c_int),
        ("fermi_start", C.c_double * 2), ("fermi_solver", C.c_int),
    ]

    @classmethod
    def defaults(cls, strength=1250.0, alpha=1.0, guess_kappa=True):
        """The &Pairing values of the Mg24 example input in the reference's README.md, with the reference's defaults."""
        p = cls()
        p.strength[0] = p.strength[1] = strength
        p.alpha[0] = p.alpha[1] = alpha
        p.rhosat = 0.16
        p.cut[0] = p.cut[1] = 5.0
        p.mu[0] = p.mu[1] = 0.5
        p.mix = 0.1
        p.fermi_prec = 1e-12
        p.max_iter = 50
        p.guess_kappa = int(guess_kappa)
        p.fermi_start[0] = p.fermi_start[1] = -10.0
        p.fermi_solver = 0
        return p


class MgPairingInfo(C.Structure):
    _fields_ = [
        ("fermi", C.c_double * 2), ("particles", C.c_double * 2), ("evaluations", C.c_int),
        ("converged", C.c_int), ("pairing_energy", C.c_double * 2), ("dispersion", C.c_double * 2),
        ("first_order", C.c_int),
    ]

    def as_dict(self) -> dict:
        return {"fermi": list(self.fermi), "particles": list(self.particles),
                "evaluations": self.evaluations, "converged": bool(self.converged),
                "pairing_energy": list(self.pairing_energy), "dispersion": list(self.dispersion),
                "first_order": bool(self.first_order)}


class MgEnergyTerms(C.Structure):
    _fields_ = [
        ("total", C.c_double),
        ("kinetic", C.c_double * 2),
        ("skyrme", C.c_double * 36),
        ("coulomb", C.c_double),
        ("coulomb_exchange", C.c_double),
        ("com", (C.c_double * 2) * 2),
        ("pairing", C.c_double * 2),
        ("sp_energy", C.c_double),
    ]

    def as_dict(self) -> dict:
        return {
            "total": self.total,
            "kinetic": list(self.kinetic),
            "skyrme": list(self.skyrme),
            "coulomb": self.coulomb,
            "coulomb_exchange": self.coulomb_exchange,
            "com": [list(r) for r in self.com],
            "pairing": list(self.pairing),
            "sp_energy": self.sp_energy,
        }


class MgMomentConstraint(C.Structure):
    _fields_ = [("l", C.c_int), ("m", C.c_int), ("constraint", C.c_double),
                ("intensity", C.c_double), ("iteration", C.c_int)]


class MgConstraintState(C.Structure):
    _fields_ = [("value", C.c_double * 2), ("squared", C.c_double * 2),
                ("constraint", C.c_double), ("intensity", C.c_double), ("active", C.c_int)]

    def as_dict(self) -> dict:
        return {"value": list(self.value), "squared": list(self.squared),
                "constraint": self.constraint, "intensity": self.intensity,
                "active": bool(self.active)}


class MgConvergence(C.Structure):
    _fields_ = [("energy_prec", C.c_double), ("moment_prec", C.c_double),
                ("pairing_prec", C.c_double)]


class MgNilssonParams(C.Structure):
    _fields_ = [("n_neutron", C.c_int), ("meven", C.c_int), ("modd", C.c_int),
                ("ho", C.c_double * 3), ("amplitude", C.c_double), ("seed", C.c_int)]


class MgWfHeader(C.Structure):
    _fields_ = [
        ("version", C.c_int),
        ("energy", C.c_double), ("denergy", C.c_double),
        ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
        ("dx", C.c_double),
        ("trc", C.c_int), ("pc", C.c_int), ("sc", C.c_int), ("tsc", C.c_int), ("ic", C.c_int),
        ("nwt", C.c_int),
        ("neutrons", C.c_double), ("protons", C.c_double),
        ("fd_order", C.c_int), ("fd_lap_order", C.c_int), ("coulomb_lap_order", C.c_int),
        ("force", C.c_char * 208),
        ("skyrme", C.c_double * 14),
        ("hbar", C.c_double), ("hbm", C.c_double * 2),
        ("com1body", C.c_int), ("com2body", C.c_int),
        ("coef", C.c_double * 28),
        ("pairing_type", C.c_int),
        ("pairing_strength", C.c_double * 2), ("pairing_alpha", C.c_double * 2),
        ("pairing_cut", C.c_double * 2),
        ("fermi", C.c_double * 2), ("ln_lambda", C.c_double * 2),
        ("omega", C.c_double * 3), ("crank_values", C.c_double * 3),
        ("hfb_size", C.c_int), ("pindex", C.c_int), ("iindex", C.c_int),
        ("can_blocks", C.c_int), ("has_cutoffs", C.c_int), ("has_jmunu", C.c_int),
        ("odd_records", C.c_int), ("n_moments", C.c_int),
    ]


# MG_WF_* field ids of include/mocca_wf.h, in order
WF_FIELDS = ("grids", "spwf_real", "spwf_int", "rho", "derrho", "laprho", "tau", "nablaj",
             "jmunu", "odd1", "odd2", "odd3", "odd4", "odd5", "cutoffs", "blocksizes", "U",
             "V", "columns", "rhohfb", "kappahfb", "cantransfo", "moment_int", "moment_real")
WF_INT_FIELDS = {"spwf_int", "blocksizes", "columns", "moment_int"}


_P = C.c_void_p
_D = C.POINTER(C.c_double)
_I = C.POINTER(C.c_int)
_PP = C.POINTER(C.c_void_p)

# name -> argtypes (every function returns int status)
SIGNATURES = {
    "mg_skyrme_coefficients": [C.POINTER(MgForce), C.c_int, C.POINTER(MgSkyrmeB)],
    "mg_lagrange_matrices": [C.c_int, C.c_double, C.c_int, _D, _D],
    "mg_create": [C.POINTER(MgParams), C.POINTER(MgForce), _P, C.POINTER(_P)],
    "mg_destroy": [_P],
    "mg_synchronize": [_P],
    "mg_set_precision": [_P, C.c_int],
    "mg_upload_spinors": [_P, C.c_int, _PP, _I, C.c_int, C.c_int],
    "mg_download_spinors": [_P, C.c_int, _PP, C.c_int, C.c_int],
    "mg_download_derivatives": [_P, C.c_int, _PP, _PP, C.c_int, C.c_int],
    "mg_set_occupations": [_P, C.c_int, _D],
    "mg_get_occupations": [_P, C.c_int, _D],
    "mg_set_energies": [_P, C.c_int, _D],
    "mg_get_energies": [_P, C.c_int, _D, _D],
    "mg_derive_basis": [_P, C.c_int],
    "mg_derive_all": [_P],
    "mg_hpsi": [_P, C.c_int, _D, _D, _D],
    "mg_grad_desc": [_P, C.c_double, C.c_double],
    "mg_gram_schmidt": [_P],
    "mg_hf_fill": [_P],
    "mg_update_densities": [_P],
    "mg_get_step_parameters": [_P, _D, _D],
    "mg_mix_densities": [_P],
    "mg_get_densities": [_P, _D, _D, _D, _D, _D],
    "mg_set_densities": [_P, _D, _D, _D, _D, _D],
    "mg_get_jmunu": [_P, _D],
    "mg_set_jmunu": [_P, _D],
    "mg_calculate_moments": [_P],
    "mg_add_constraint": [_P, C.POINTER(MgMomentConstraint)],
    "mg_get_constraint": [_P, C.c_int, C.POINTER(MgConstraintState)],
    "mg_get_constraint_fields": [_P, _D, _D],
    "mg_alternate_step": [_P],
    "mg_readjust_moments": [_P, C.c_int],
    "mg_solve_coulomb": [_P, _I],
    "mg_coulomb_residual": [_P, _D],
    "mg_coulomb_reset": [_P],
    "mg_get_time_odd": [_P, _D, _D, _D, _D, _D, _D, _D],
    "mg_get_time_odd_tensor": [_P, _D, _D, _D, _D, _D, _D, _D],
    "mg_symmetry_operators": [_P, C.c_int, _D],
    "mg_construct_potentials": [_P, _I],
    "mg_get_potentials": [_P, _D, _D, _D, _D, _D, _D, _D],
    "mg_set_potentials": [_P, _D, _D, _D, _D, _D],
    "mg_energy": [_P, C.POINTER(MgEnergyTerms)],
    "mg_iterate": [_P, C.c_int, C.c_double, C.c_double, C.POINTER(MgEnergyTerms)],
    "mg_launch_count": [_P, C.POINTER(C.c_longlong)],
    "mg_set_phase_timing": [_P, C.c_int],
    "mg_get_phase_times": [_P, _D, C.c_int, C.POINTER(C.c_longlong)],
    "mg_convergence_check": [_P, C.POINTER(MgConvergence), _I],
    "mg_evolve": [_P, C.c_int, C.c_double, C.c_double, C.POINTER(MgConvergence), _I, _I,
                  C.POINTER(MgEnergyTerms)],
    "mg_batch_create": [C.c_int, _PP, C.POINTER(_P)],
    "mg_batch_destroy": [_P],
    "mg_batch_tune": [_P, C.c_int, _D, _D, _I],
    "mg_batch_set_workers": [_P, C.c_int],
    "mg_batch_status": [_P, _I],
    "mg_batch_iterate": [_P, C.c_int, _D, _D, C.POINTER(MgEnergyTerms)],
    "mg_eigh_batched": [C.c_int, _I, C.c_int, _D, _D, _D],
    "mg_eigh_batched_noalloc": [C.c_int, _I, C.c_int, _P, _P, _P, _P, _P],
    "mg_set_pairing": [_P, C.POINTER(MgPairingParams)],
    "mg_solve_pairing": [_P, C.POINTER(MgPairingInfo)],
    "mg_get_hfb_block": [_P, C.c_int, _D, _D, _D],
    "mg_get_pairing_field": [_P, _D, _D, _D],
    "mg_wf_load": [C.c_char_p, C.POINTER(_P)],
    "mg_wf_new": [C.POINTER(MgWfHeader), C.POINTER(_P)],
    "mg_wf_save": [_P, C.c_char_p],
    "mg_wf_free": [_P],
    "mg_wf_get_header": [_P, C.POINTER(MgWfHeader)],
    "mg_wf_set_scalars": [_P, C.POINTER(MgWfHeader)],
    "mg_wf_field": [_P, C.c_int, C.POINTER(_P), C.POINTER(C.c_longlong)],
    "mg_wf_from_context": [_P, C.c_char_p, C.POINTER(_P)],
    "mg_wf_to_context": [_P, _P],
    "mg_angular_momentum": [_P, C.c_int, _D],
    "mg_nilsson_start": [_P, C.POINTER(MgNilssonParams)],
    "mg_break_symmetries": [_P, _P],
}

LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libmocca_gpu.so"
_lib = None


def load(path: Path | None = None):
    """Open libmocca_gpu.so (built by mocca_gb300.build) and bind signatures."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(
            f"{p} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`"
            " (there is no CPU fallback)")
    lib = C.CDLL(str(p))
    for name, args in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = C.c_int
    if path is None:
        _lib = lib
    return lib


class MgError(RuntimeError):
    def __init__(self, fn: str, status: int):
        super().__init__(f"{fn} returned {status} ({STATUS_NAMES.get(status, 'unknown')})")
        self.status = status


def check(fn: str, status: int, allow_not_converged: bool = False) -> int:
    if status < 0 or (status > 0 and not allow_not_converged):
        raise MgError(fn, status)
    return status
