"""CPU checks of the C ABI boundary (no device work).

* libmocca_gpu.so loads and exports every function include/mocca_gpu.h
  declares, and the ctypes table in mocca_gb300/_abi.py covers them all;
* the host-only helpers (Lagrange matrices, Skyrme coefficients) agree with
  the oracle's independent restatement;
* the product package never imports or links the oracle.
"""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

import oracle as O
from mocca_gb300 import SLY4, RunParams, _abi

ROOT = Path(__file__).resolve().parents[1]


def header_functions(pattern: str = "*.h"):
    names = []
    for h in sorted((ROOT / "include").glob(pattern)):
        txt = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names += re.findall(r"^\s*int\s+(mg_\w+)\s*\(", txt, flags=re.M)
    return names


def test_every_declared_symbol_is_exported(built):
    names = header_functions()
    assert len(names) >= 25
    lib = C.CDLL(str(_abi.LIB_PATH))
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert set(names) <= set(_abi.SIGNATURES), set(names) - set(_abi.SIGNATURES)


@pytest.mark.parametrize("n,folded", [(10, True), (24, True), (32, False), (7, False)])
def test_lagrange_matrices_match_oracle(built, n, folded):
    lib = _abi.load()
    d1 = np.empty(2 * n * n)
    d2 = np.empty(2 * n * n)
    assert lib.mg_lagrange_matrices(n, 0.8, int(folded), d1.ctypes.data_as(_abi._D),
                                    d2.ctypes.data_as(_abi._D)) == 0
    o1, o2 = O.lagrange_matrices(n, 0.8, folded)
    assert np.array_equal(d1.reshape(2, n, n), o1)
    assert np.array_equal(d2.reshape(2, n, n), o2)


def test_invalid_arguments_are_rejected(built):
    lib = _abi.load()
    d = np.empty(8)
    assert lib.mg_lagrange_matrices(0, 0.8, 1, d.ctypes.data_as(_abi._D),
                                    d.ctypes.data_as(_abi._D)) == _abi.MG_ERR_ARG
    assert lib.mg_lagrange_matrices(2, -1.0, 1, d.ctypes.data_as(_abi._D),
                                    d.ctypes.data_as(_abi._D)) == _abi.MG_ERR_ARG
    assert lib.mg_destroy(None) == _abi.MG_ERR_ARG
    # ParameterEstimation takes 0 or 1; the check comes before any CUDA call
    params = RunParams(nx=10, ny=10, nz=10, parameter_estimation=2).to_c()
    ctx = C.c_void_p()
    assert lib.mg_create(C.byref(params), SLY4.to_c(), None, C.byref(ctx)) == _abi.MG_ERR_ARG
    assert not ctx.value


@pytest.mark.parametrize("force", ["SLY4", "SLY5_TENSOR"])
@pytest.mark.parametrize("trc", [1, 0])
def test_skyrme_coefficients_match_oracle(built, force, trc):
    import mocca_gb300.forces as F
    f = getattr(F, force).to_c()
    a, b = _abi.MgSkyrmeB(), _abi.MgSkyrmeB()
    assert _abi.load().mg_skyrme_coefficients(f, trc, a) == 0
    assert O.load().orc_skyrme_coefficients(f, trc, b) == 0
    for name, _ in _abi.MgSkyrmeB._fields_:
        assert getattr(a, name) == pytest.approx(getattr(b, name), rel=1e-15, abs=0), name


def test_tensor_coefficients():
    """CalcEDFCoef's J^2 coefficients (src/Force.f90:526-537) for SLy5colo
    (t1, x1, t2, x2 and te = 296, to = -136 MeV fm^5 of forces.param):
    B14 = -(t1 x1 + t2 x2)/8 + (te + to)/4, B15 = (t1 - t2)/8 - (te - to)/4,
    B16 = -3 (te + to)/8, B17 = 3 (te - to)/8; without J2Terms only B16, B17."""
    import dataclasses
    from mocca_gb300.forces import SLY5_TENSOR as T
    a = _abi.MgSkyrmeB()
    assert _abi.load().mg_skyrme_coefficients(T.to_c(), 1, a) == 0
    assert a.B14 == pytest.approx(-(T.t1 * T.x1 + T.t2 * T.x2) / 8 + (T.te + T.to) / 4, rel=1e-14)
    assert a.B15 == pytest.approx((T.t1 - T.t2) / 8 - (T.te - T.to) / 4, rel=1e-14)
    assert a.B16 == pytest.approx(-3 * (T.te + T.to) / 8, rel=1e-14)
    assert a.B17 == pytest.approx(3 * (T.te - T.to) / 8, rel=1e-14)
    b = _abi.MgSkyrmeB()
    assert _abi.load().mg_skyrme_coefficients(dataclasses.replace(T, j2terms=False).to_c(), 1,
                                              b) == 0
    assert b.B14 == 0.0 and b.B15 == 0.0 and b.B16 == a.B16 and b.B17 == a.B17


def test_time_odd_tensor_coefficients():
    """CalcEDFCoef's time-odd tensor coefficients (src/Force.f90:539-551):
    with broken time reversal B18 = -(3 t1 x1 - t2 x2)/32 + (3 te - to)/16,
    B19 = (3 t1 + t2)/32 - (3 te + to)/16 (J2Terms only), B20 = 3 (3 te -
    to)/16, B21 = -3 (3 te + to)/16 (te, to alone); all four zero with time
    reversal."""
    import dataclasses
    from mocca_gb300.forces import SLY5_TENSOR as T
    lib = _abi.load()
    a, b, c = _abi.MgSkyrmeB(), _abi.MgSkyrmeB(), _abi.MgSkyrmeB()
    assert lib.mg_skyrme_coefficients(T.to_c(), 0, a) == 0
    assert a.B18 == pytest.approx(-(3 * T.t1 * T.x1 - T.t2 * T.x2) / 32 + (3 * T.te - T.to) / 16,
                                  rel=1e-14)
    assert a.B19 == pytest.approx((3 * T.t1 + T.t2) / 32 - (3 * T.te + T.to) / 16, rel=1e-14)
    assert a.B20 == pytest.approx(3 * (3 * T.te - T.to) / 16, rel=1e-14)
    assert a.B21 == pytest.approx(-3 * (3 * T.te + T.to) / 16, rel=1e-14)
    assert lib.mg_skyrme_coefficients(dataclasses.replace(T, j2terms=False).to_c(), 0, b) == 0
    assert b.B18 == 0.0 and b.B19 == 0.0 and b.B20 == a.B20 and b.B21 == a.B21
    assert lib.mg_skyrme_coefficients(T.to_c(), 1, c) == 0
    assert c.B18 == c.B19 == c.B20 == c.B21 == 0.0


@pytest.mark.parametrize("name,b14,b15", [
    ("SLy4T", 15.0, -120.0), ("sly4tmin", 15.0, -120.0),
    ("UNEDF2", -54.4333635973721002 + 65.9030310445938028, -65.9030310445938028 * 2.0)])
def test_named_coupling_overrides(built, name, b14, b15):
    """CalcEDFCoef overrides B14..B17 for the SLy4T, SLy4Tmin and UNEDF2
    parameterizations, by name, case-insensitively (src/Force.f90:552-597);
    the library and the oracle agree, other names keep the relations."""
    import dataclasses
    f = dataclasses.replace(SLY4, j2terms=True, name=name)
    for trc in (1, 0):
        a, b = _abi.MgSkyrmeB(), _abi.MgSkyrmeB()
        assert _abi.load().mg_skyrme_coefficients(f.to_c(), trc, a) == 0
        assert O.load().orc_skyrme_coefficients(f.to_c(), trc, b) == 0
        assert (a.B14, a.B15, a.B16, a.B17) == (b14, b15, 0.0, 0.0)
        for n, _ in _abi.MgSkyrmeB._fields_:
            assert getattr(a, n) == getattr(b, n), n
    c = _abi.MgSkyrmeB()
    assert _abi.load().mg_skyrme_coefficients(dataclasses.replace(f, name="SLy4").to_c(), 1,
                                              c) == 0
    assert c.B14 == pytest.approx(-(SLY4.t1 * SLY4.x1 + SLY4.t2 * SLY4.x2) / 8, rel=1e-14)


def test_coupling_selector_is_checked(built):
    lib = _abi.load()
    f = SLY4.to_c()
    f.coupling = 4
    params = RunParams(nx=10, ny=10, nz=10).to_c()
    ctx = C.c_void_p()
    assert lib.mg_create(C.byref(params), f, None, C.byref(ctx)) == _abi.MG_ERR_ARG
    assert not ctx.value


def test_product_does_not_use_the_oracle():
    for p in list((ROOT / "mocca_gb300").rglob("*.py")) + list((ROOT / "mocca_gb300").rglob("*.cu")):
        txt = p.read_text()
        assert "import oracle" not in txt and "liboracle" not in txt and "orc_" not in txt, p


def test_fortran_module_matches_header():
    """include/mocca_gpu.f90 (the reference-side binding) declares exactly the
    entry points of mocca_gpu.h and one bind(C) type per header struct.  The
    .wf layer (mocca_wf.h) serves C and Python hosts; a Fortran host writes
    its files with its own WriteMOCCa_v1."""
    f90 = (ROOT / "include" / "mocca_gpu.f90").read_text()
    fns = set(re.findall(r"function\s+(mg_\w+)\s*\(", f90))
    assert fns == set(header_functions("mocca_gpu.h"))
    hdr = re.sub(r"/\*.*?\*/", "", (ROOT / "include" / "mocca_gpu.h").read_text(), flags=re.S)
    structs = set(re.findall(r"typedef struct (\w+) \{", hdr))
    types = set(re.findall(r"type, bind\(C\) :: (\w+)", f90))
    assert types == structs
    for name in fns:
        assert f'bind(C, name="{name}")' in f90, name
    # and it is what include/make_fortran_module.py writes from the header
    import importlib.util
    spec = importlib.util.spec_from_file_location("mfm", ROOT / "include" / "make_fortran_module.py")
    mfm = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mfm)
    assert mfm.module_text((ROOT / "include" / "mocca_gpu.h").read_text()) == f90
    # free-form Fortran: at most 132 characters per line
    assert max(len(line) for line in f90.splitlines()) <= 132


def test_new_entry_points_reject_bad_arguments(built):
    """Argument checks that return before any device work: NULL contexts and
    outputs, eigensolver sizes beyond its 160 limit, empty batches."""
    lib = _abi.load()
    one = np.zeros(1)
    d = one.ctypes.data_as(_abi._D)
    n = np.array([161], dtype=np.int32)
    big = np.zeros(1)
    assert lib.mg_eigh_batched(1, n.ctypes.data_as(_abi._I), 161, big.ctypes.data_as(_abi._D),
                               d, d) == _abi.MG_ERR_ARG
    assert lib.mg_eigh_batched(65, n.ctypes.data_as(_abi._I), 8, d, d, d) == _abi.MG_ERR_ARG
    conv = C.c_int(0)
    assert lib.mg_convergence_check(None, None, C.byref(conv)) == _abi.MG_ERR_ARG
    assert lib.mg_evolve(None, 1, 0.01, 0.3, None, None, None, None) == _abi.MG_ERR_ARG
    assert lib.mg_coulomb_residual(None, d) == _abi.MG_ERR_ARG
    assert lib.mg_add_constraint(None, None) == _abi.MG_ERR_ARG
    assert lib.mg_alternate_step(None) == _abi.MG_ERR_ARG
    assert lib.mg_readjust_moments(None, 1) == _abi.MG_ERR_ARG
    assert lib.mg_batch_iterate(None, 1, d, d, None) == _abi.MG_ERR_ARG
    assert lib.mg_batch_status(None, None) == _abi.MG_ERR_ARG
    assert lib.mg_batch_set_workers(None, 2) == _abi.MG_ERR_ARG


def test_time_odd_and_solver_parameters_are_checked(built):
    """mg_create refuses, before any device work: cranking with time
    reversal, OmegaX with signature or OmegaY with time simplex, the
    time-odd path off the EV8 box, in mixed precision or with HFB, an
    unknown Coulomb solver or a negative Coulomb tolerance."""
    lib = _abi.load()
    ctx = C.c_void_p()
    bad = [dict(trc=1, omega=(0.0, 0.0, 0.5)), dict(trc=0, omega=(0.5, 0.0, 0.0)),
           dict(trc=0, omega=(0.0, 0.5, 0.0)), dict(trc=0, precision=_abi.MG_MIXED),
           dict(trc=0, pairing=_abi.MG_PAIRING_HFB), dict(trc=0, pc=0, sc=0, tsc=0),
           dict(coulomb_solver=3), dict(coulomb_prec=-1.0)]
    for kw in bad:
        p = RunParams(nx=10, ny=10, nz=10, nwt=8, **kw).to_c()
        assert lib.mg_create(C.byref(p), SLY4.to_c(), None, C.byref(ctx)) == _abi.MG_ERR_ARG, kw
    assert lib.mg_get_time_odd(None, None, None, None, None, None, None, None) == _abi.MG_ERR_ARG
    assert lib.mg_coulomb_reset(None) == _abi.MG_ERR_ARG
