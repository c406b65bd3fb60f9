"""CPU checks of the .wf file layer (include/mocca_wf.h, host code only).

The native loader and writer are compared with the oracle's independent
restatement of WriteMOCCa_v1 / ReadMOCCa_v1 (oracle/wf_format.py): every
field bit-exact, files byte-identical, the committed fixture
tests/golden/wf_small_v1.wf parsed to the content its script defines, and
the error cases of ReadMOCCa_v1 (missing file, wrong version, a record too
short, a bad isospin, a file cut inside a record) refused with MG_ERR_IO.
No device work: the file layer never touches the GPU.
"""
import hashlib
import sys
from pathlib import Path

import numpy as np
import pytest

import wf_format as WF
from mocca_gb300 import _abi
from mocca_gb300.wf import WavefunctionFile

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT / "tests" / "golden"))
import make_wf_fixture  # noqa: E402

FIXTURE = ROOT / "tests" / "golden" / "wf_small_v1.wf"
FIXTURE_SHA256 = "07160e065b69d5bc692ec1beb735d464ebac7762dee6ee633b92aa64e3a18f9a"

SCALARS = ("energy", "denergy", "nx", "ny", "nz", "dx", "trc", "pc", "sc", "tsc", "ic", "nwt",
           "neutrons", "protons", "fd_order", "fd_lap_order", "coulomb_lap_order", "force",
           "skyrme", "hbar", "hbm", "com1body", "com2body", "coef", "pairing_type",
           "pairing_strength", "pairing_alpha", "pairing_cut", "fermi", "ln_lambda", "omega",
           "crank_values", "hfb_size", "pindex", "iindex", "can_blocks", "has_cutoffs",
           "has_jmunu", "odd_records", "n_moments")


def random_content(seed=3, trc=1, pc=1, nwt=3, jmunu=1, odd=0b10101, cutoffs=1, moments=1,
                   can_blocks=0, n=(3, 4, 5)):
    rng = np.random.default_rng(seed)
    h = dict(energy=rng.normal() * 100, denergy=rng.normal() * 1e-6, nx=n[0], ny=n[1], nz=n[2],
             dx=0.8, trc=trc, pc=pc, sc=1, tsc=1, ic=1, nwt=nwt, neutrons=8.0, protons=6.0,
             fd_order=-1, fd_lap_order=-1, coulomb_lap_order=2, force="SkM*",
             skyrme=rng.normal(size=14), hbar=6.58211928, hbm=rng.normal(size=2) + 41,
             com1body=2, com2body=1, coef=rng.normal(size=28), pairing_type=2,
             pairing_strength=rng.normal(size=2), pairing_alpha=rng.normal(size=2),
             pairing_cut=rng.normal(size=2), fermi=rng.normal(size=2),
             ln_lambda=rng.normal(size=2), omega=rng.normal(size=3),
             crank_values=rng.normal(size=3), has_cutoffs=cutoffs, has_jmunu=jmunu,
             odd_records=odd, n_moments=moments, can_blocks=can_blocks)
    w = WF.empty(h)
    for name in WF.FIELDS:
        a = w[name]
        if name in WF.INT_FIELDS:
            a[:] = rng.integers(-50, 50, size=a.size)
        else:
            a[:] = rng.normal(size=a.size) * 10.0 ** rng.integers(-3, 3)
    w["spwf_int"][0::5] = rng.choice([-1, 1], size=nwt)
    if moments:
        w["moment_int"][4::5] = 0
    return w


def assert_same(w: dict, f: WavefunctionFile):
    h = f.header
    for k in SCALARS:
        a, b = np.asarray(h[k]), np.asarray(w[k])
        if k == "force":
            assert str(h[k]) == str(w[k])
        else:
            assert np.array_equal(a, b.astype(a.dtype)), k
    for name in WF.FIELDS:
        got = f.field(name)
        exp = np.asarray(w[name])
        assert got.shape == exp.shape, name
        assert np.array_equal(got, exp.astype(got.dtype)), name


def test_fixture_is_the_committed_one():
    assert hashlib.sha256(FIXTURE.read_bytes()).hexdigest() == FIXTURE_SHA256


def test_fixture_parses_to_its_content(built, tmp_path):
    exp = WF.read_v1(FIXTURE)
    ref = make_wf_fixture.content()
    for k in WF.FIELDS:
        assert np.array_equal(exp[k], ref[k]), k
    with WavefunctionFile.load(FIXTURE) as f:
        assert_same(exp, f)
        assert f.header["can_blocks"] == 4 and f.header["pindex"] == 1
        f.save(tmp_path / "again.wf")
    assert (tmp_path / "again.wf").read_bytes() == FIXTURE.read_bytes()


@pytest.mark.parametrize("trc,pc,jmunu,odd,cutoffs,moments", [
    (1, 1, 1, 0b10101, 1, 1), (1, 1, 0, 0, 0, 0), (0, 1, 0, 0b11111, 1, 3), (0, 0, 1, 0b00010, 0, 0)])
def test_oracle_file_loads_and_saves_identically(built, tmp_path, trc, pc, jmunu, odd, cutoffs,
                                                  moments):
    w = random_content(trc=trc, pc=pc, jmunu=jmunu, odd=odd, cutoffs=cutoffs, moments=moments)
    p = tmp_path / "o.wf"
    WF.write_v1(p, w)
    with WavefunctionFile.load(p) as f:
        assert_same(w, f)
        f.save(tmp_path / "n.wf")
    assert (tmp_path / "n.wf").read_bytes() == p.read_bytes()


def test_native_file_reads_back_in_the_oracle(built, tmp_path):
    w = random_content(seed=11, moments=2)
    hdr = {k: w[k] for k in SCALARS if k not in ("hfb_size", "pindex", "iindex")}
    with WavefunctionFile.new(hdr) as f:
        for name in WF.FIELDS:
            f.field(name)[:] = w[name]
        f.save(tmp_path / "n.wf")
    back = WF.read_v1(tmp_path / "n.wf")
    for k in WF.FIELDS:
        assert np.array_equal(back[k], w[k]), k
    for k in ("energy", "force", "skyrme", "coef", "fermi", "n_moments", "odd_records"):
        assert np.array_equal(np.asarray(back[k]), np.asarray(w[k])), k


@pytest.mark.parametrize("max_sub", [8, 100, 1000])
def test_subrecords(built, tmp_path, max_sub):
    """Records split into subrecords (the layout gfortran uses above
    2**31 - 9 bytes) read back as the same records."""
    w = random_content(seed=5)
    p = tmp_path / "s.wf"
    WF.write_v1(p, w, max_sub=max_sub)
    assert WF.read_v1(p)["grids"].tobytes() == w["grids"].tobytes()
    with WavefunctionFile.load(p) as f:
        assert_same(w, f)


def test_longer_records_are_accepted(built, tmp_path):
    """A Fortran READ ignores the rest of a record: extra bytes after the
    items are skipped, not an error."""
    w = random_content(seed=7)
    recs = WF.payloads(w)
    recs[2] += b"\0" * 8            # nx, ny, nz, dx
    recs[-4] += b"\1" * 24          # CanTransfo: tail of a partial block
    recs[-3] += b"\2" * 16          # Omega, CrankValues
    p = tmp_path / "l.wf"
    p.write_bytes(WF.encode_records(recs))
    with WavefunctionFile.load(p) as f:
        assert_same(w, f)


def _status(path) -> int:
    lib = _abi.load()
    import ctypes as C
    h = C.c_void_p()
    st = lib.mg_wf_load(str(path).encode(), C.byref(h))
    if h.value:
        lib.mg_wf_free(h)
    return st


def test_bad_files_are_refused(built, tmp_path):
    w = random_content(seed=9)
    assert _status(tmp_path / "missing.wf") == _abi.MG_ERR_IO
    recs = WF.payloads(w)
    # version 2
    bad = list(recs)
    bad[0] = np.int32(2).tobytes()
    (tmp_path / "v.wf").write_bytes(WF.encode_records(bad))
    assert _status(tmp_path / "v.wf") == _abi.MG_ERR_IO
    # a grid record one double short
    bad = list(recs)
    bad[5] = bad[5][:-8]
    (tmp_path / "g.wf").write_bytes(WF.encode_records(bad))
    assert _status(tmp_path / "g.wf") == _abi.MG_ERR_IO
    # isospin 0 (ReadSpwf stops on it)
    w2 = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in w.items()}
    w2["spwf_int"][5] = 0
    WF.write_v1(tmp_path / "i.wf", w2)
    assert _status(tmp_path / "i.wf") == _abi.MG_ERR_IO
    # cut inside a record, and damaged markers
    data = WF.encode_records(recs)
    (tmp_path / "t.wf").write_bytes(data[:len(data) // 2])
    assert _status(tmp_path / "t.wf") == _abi.MG_ERR_IO
    (tmp_path / "m.wf").write_bytes(data[:4] + np.int32(999).tobytes() + data[8:])
    assert _status(tmp_path / "m.wf") == _abi.MG_ERR_IO
    # a moment's second record missing at the end of the file
    (tmp_path / "e.wf").write_bytes(WF.encode_records(recs[:-1]))
    assert _status(tmp_path / "e.wf") == _abi.MG_ERR_IO
    # the intact file still loads
    WF.write_v1(tmp_path / "ok.wf", w)
    assert _status(tmp_path / "ok.wf") == _abi.MG_OK


def test_guess_hf_kappa_restatement():
    """GuessHFBMatrices(0)'s loop order: the later of the two writes wins,
    leaving +0.1 above and -0.1 below the diagonal between opposite
    signatures."""
    sig = [[1, 1, -1, -1]]
    K = WF.guess_hf_kappa(sig + [[], [], []], 4).reshape(2, 2, 4, 4, 2)[0, 0, :, :, 0].T
    exp = np.array([[0, 0, .1, .1], [0, 0, .1, .1], [-.1, -.1, 0, 0], [-.1, -.1, 0, 0]])
    assert np.array_equal(K, exp)
