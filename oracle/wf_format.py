"""CPU restatement of MOCCa's version-1 wavefunction file (.wf), for tests.

TEST INFRASTRUCTURE: the checker of libmocca_gpu's file layer
(include/mocca_wf.h).  Only tests/ and the fixture script under
tests/golden/ use it; the product never imports it.

It writes and reads the records in the order of the reference's
WriteMOCCa_v1 (src/InOut.f90:905-1046) and ReadMOCCa_v1 (:1050-1416), one
record per WRITE statement, with the per-spwf records of WriteSpwf
(src/Spwf.f90:2246-2261), the density records of WriteDensity
(src/Densities.f90:1189-1240) and the moment records of WriteMoment
(src/Moments.f90:3330-3363).  Records use gfortran's unformatted sequential
layout: int32 little-endian byte counts around each payload; a payload
longer than `max_sub` bytes (gfortran: 2**31 - 9) is split into subrecords
whose leading marker (all but the last) and trailing marker (all but the
first) are negated.

Parity is unpinned by reference artefacts: the reference ships no .wf file
and cannot be built here (no Fortran compiler), so this restatement follows
the source text of those WRITE statements only.

A file is a dict: the scalars of mg_wf_header by name, and numpy arrays
under the MG_WF_* field names (float64 or int32, flat, Fortran element
order).  Optional records are absent arrays of length 0.
"""
from __future__ import annotations

import struct

import numpy as np

MAX_SUB = 2**31 - 9
FORCE_LEN = 200           # character(len=200) :: afor (src/Force.f90:23)
ODD_V = (12, 30, 14, 6, 6)  # time-odd density records, doubles per mesh point

FIELDS = ("grids", "spwf_real", "spwf_int", "rho", "derrho", "laprho", "tau", "nablaj",
          "jmunu", "odd1", "odd2", "odd3", "odd4", "odd5", "cutoffs", "blocksizes", "U",
          "V", "columns", "rhohfb", "kappahfb", "cantransfo", "moment_int", "moment_real")
INT_FIELDS = {"spwf_int", "blocksizes", "columns", "moment_int"}


# ---- records -----------------------------------------------------------------

def encode_records(payloads: list[bytes], max_sub: int = MAX_SUB) -> bytes:
    out = bytearray()
    for p in payloads:
        chunks = [p[i:i + max_sub] for i in range(0, len(p), max_sub)] or [b""]
        for k, c in enumerate(chunks):
            n = len(c)
            lead = n if k == len(chunks) - 1 else -n
            trail = n if k == 0 else -n
            out += struct.pack("<i", lead) + c + struct.pack("<i", trail)
    return bytes(out)


def decode_records(data: bytes) -> list[bytes]:
    recs, pos, cur, first = [], 0, bytearray(), True
    while pos < len(data):
        (lead,) = struct.unpack_from("<i", data, pos)
        n = abs(lead)
        cur += data[pos + 4:pos + 4 + n]
        (trail,) = struct.unpack_from("<i", data, pos + 4 + n)
        if abs(trail) != n or (trail < 0) == first:
            raise ValueError("damaged record markers")
        pos += 8 + n
        first = False
        if lead >= 0:
            recs.append(bytes(cur))
            cur, first = bytearray(), True
    if not first:
        raise ValueError("file ends inside a record")
    return recs


# ---- shapes --------------------------------------------------------------------

def shapes(h: dict) -> dict:
    """Element counts of every field (src/Pairing.f90:400-405 for HFBSize,
    PrepareHFBModule src/HFB.f90:254-255 for Pindex / Iindex)."""
    V = h["nx"] * h["ny"] * h["nz"]
    n = h["nwt"]
    m = 2 * n if h["trc"] else n
    pi, ii = (2 if h["pc"] else 1), (2 if h["ic"] else 1)
    cb = h.get("can_blocks") or pi * ii
    c = {"grids": n * 4 * V, "spwf_real": n * 7, "spwf_int": n * 5,
         "rho": 2 * V, "derrho": 6 * V, "laprho": 2 * V, "tau": 2 * V, "nablaj": 2 * V,
         "jmunu": 18 * V if h.get("has_jmunu") else 0,
         "cutoffs": n if h.get("has_cutoffs") else 0,
         "blocksizes": pi * ii, "U": 2 * m * 2 * m * 4, "V": 2 * m * 2 * m * 4,
         "columns": m * pi * ii, "rhohfb": 2 * m * m * 4, "kappahfb": 2 * m * m * 4,
         "cantransfo": 2 * m * m * cb, "moment_int": 5 * h.get("n_moments", 0),
         "moment_real": 22 * h.get("n_moments", 0)}
    for k in range(5):
        c[f"odd{k + 1}"] = ODD_V[k] * V if (h.get("odd_records", 0) >> k) & 1 else 0
    return c


def empty(h: dict) -> dict:
    """A file dict with the header's scalars and zero arrays."""
    w = dict(h)
    w["hfb_size"] = 2 * h["nwt"] if h["trc"] else h["nwt"]
    w["pindex"], w["iindex"] = (2 if h["pc"] else 1), (2 if h["ic"] else 1)
    w["can_blocks"] = h.get("can_blocks") or w["pindex"] * w["iindex"]
    for k, n in shapes(w).items():
        w[k] = np.zeros(n, dtype=np.int32 if k in INT_FIELDS else np.float64)
    return w


# ---- write -----------------------------------------------------------------------

def _d(*xs) -> bytes:
    return b"".join(np.asarray(x, dtype="<f8").ravel(order="C").tobytes() for x in xs)


def _i(*xs) -> bytes:
    return b"".join(np.asarray(x, dtype="<i4").ravel(order="C").tobytes() for x in xs)


def _name(s: str) -> bytes:
    b = s.encode("ascii")[:FORCE_LEN]
    return b + b" " * (FORCE_LEN - len(b))


def payloads(w: dict) -> list[bytes]:
    """The records of WriteMOCCa_v1, in order."""
    V = w["nx"] * w["ny"] * w["nz"]
    rec = [_i(1),
           _d(w["energy"], w["denergy"]),
           _i(w["nx"], w["ny"], w["nz"]) + _d(w["dx"]),
           _i(*[1 if w[k] else 0 for k in ("trc", "pc", "sc", "tsc", "ic")]),
           _i(w["nwt"]) + _d(w["neutrons"], w["protons"])]
    for k in range(w["nwt"]):
        rec.append(_d(w["grids"][k * 4 * V:(k + 1) * 4 * V]))
        rec.append(_d(w["spwf_real"][7 * k:7 * k + 7]) + _i(w["spwf_int"][5 * k:5 * k + 5]))
    rec.append(_d(w["rho"], w["derrho"], w["laprho"]))
    rec.append(_d(w["tau"]))
    rec.append(_d(w["nablaj"]))
    rec.append(_d(w["jmunu"]))
    for k in range(5):
        rec.append(_d(w[f"odd{k + 1}"]))
    rec.append(_i(w["fd_order"], w["fd_lap_order"], w["coulomb_lap_order"]))
    rec.append(_name(w["force"]))
    rec.append(_d(w["skyrme"]))
    rec.append(_name(w["force"]) + _d(w["hbar"], w["hbm"]) + _i(w["com1body"], w["com2body"]))
    rec.append(_d(w["coef"]))
    rec.append(_i(w["pairing_type"]) + _d(w["pairing_strength"], w["pairing_alpha"],
                                          w["pairing_cut"]))
    rec.append(_d(w["cutoffs"]))
    rec.append(_d(w["fermi"], w["ln_lambda"]))
    rec.append(_i(w["blocksizes"]))
    rec.append(_d(w["U"], w["V"]))
    rec.append(_i(w["columns"]))
    rec.append(_d(w["rhohfb"], w["kappahfb"]))
    rec.append(_d(w["cantransfo"]))
    rec.append(_d(w["omega"], w["crank_values"]))
    for k in range(w.get("n_moments", 0)):
        mi = w["moment_int"][5 * k:5 * k + 5]
        rec.append(_i(mi[0], mi[1], mi[2], mi[3], 1 if mi[4] else 0))
        rec.append(_d(w["moment_real"][22 * k:22 * k + 22]))
    return rec


def write_v1(path, w: dict, max_sub: int = MAX_SUB) -> None:
    with open(path, "wb") as f:
        f.write(encode_records(payloads(w), max_sub))


# ---- read ------------------------------------------------------------------------

def read_v1(path) -> dict:
    """ReadMOCCa_v1's parse; records shorter than their items raise,
    longer ones keep only the items (a Fortran READ ignores the rest)."""
    with open(path, "rb") as f:
        recs = decode_records(f.read())
    it = iter(recs)

    def nxt(need: int) -> bytes:
        r = next(it)
        if len(r) < need:
            raise ValueError("record too short")
        return r

    h: dict = {}
    if struct.unpack("<i", nxt(4)[:4])[0] != 1:
        raise ValueError("version")
    h["energy"], h["denergy"] = struct.unpack("<2d", nxt(16)[:16])
    r = nxt(20)
    h["nx"], h["ny"], h["nz"] = struct.unpack("<3i", r[:12])
    (h["dx"],) = struct.unpack("<d", r[12:20])
    flags = struct.unpack("<5i", nxt(20)[:20])
    for k, v in zip(("trc", "pc", "sc", "tsc", "ic"), flags):
        h[k] = int(v != 0)
    r = nxt(20)
    (h["nwt"],) = struct.unpack("<i", r[:4])
    h["neutrons"], h["protons"] = struct.unpack("<2d", r[4:20])
    V = h["nx"] * h["ny"] * h["nz"]
    n = h["nwt"]
    grids, sr, si = [], [], []
    for _ in range(n):
        grids.append(np.frombuffer(nxt(32 * V)[:32 * V], "<f8"))
        r = nxt(76)
        sr.append(np.frombuffer(r[:56], "<f8"))
        si.append(np.frombuffer(r[56:76], "<i4"))
        if si[-1][0] not in (1, -1):
            raise ValueError("isospin")
    w = {"grids": np.concatenate(grids) if n else np.zeros(0),
         "spwf_real": np.concatenate(sr) if n else np.zeros(0),
         "spwf_int": np.concatenate(si).astype(np.int32) if n else np.zeros(0, np.int32)}
    a = np.frombuffer(nxt(80 * V)[:80 * V], "<f8")
    w["rho"], w["derrho"], w["laprho"] = a[:2 * V], a[2 * V:8 * V], a[8 * V:10 * V]
    w["tau"] = np.frombuffer(nxt(16 * V)[:16 * V], "<f8")
    w["nablaj"] = np.frombuffer(nxt(16 * V)[:16 * V], "<f8")
    r = next(it)
    h["has_jmunu"] = int(len(r) >= 144 * V)
    w["jmunu"] = np.frombuffer(r[:144 * V], "<f8") if h["has_jmunu"] else np.zeros(0)
    h["odd_records"] = 0
    for k in range(5):
        r = next(it)
        nb = ODD_V[k] * V * 8
        if len(r) >= nb:
            h["odd_records"] |= 1 << k
            w[f"odd{k + 1}"] = np.frombuffer(r[:nb], "<f8")
        else:
            w[f"odd{k + 1}"] = np.zeros(0)
    h["fd_order"], h["fd_lap_order"], h["coulomb_lap_order"] = struct.unpack("<3i", nxt(12)[:12])
    h["force"] = nxt(FORCE_LEN)[:FORCE_LEN].decode("ascii").rstrip(" \0")
    h["skyrme"] = np.frombuffer(nxt(112)[:112], "<f8")
    r = nxt(FORCE_LEN + 32)
    h["hbar"], hb0, hb1 = struct.unpack("<3d", r[FORCE_LEN:FORCE_LEN + 24])
    h["hbm"] = np.array([hb0, hb1])
    h["com1body"], h["com2body"] = struct.unpack("<2i", r[FORCE_LEN + 24:FORCE_LEN + 32])
    h["coef"] = np.frombuffer(nxt(224)[:224], "<f8")
    r = nxt(52)
    (h["pairing_type"],) = struct.unpack("<i", r[:4])
    v = np.frombuffer(r[4:52], "<f8")
    h["pairing_strength"], h["pairing_alpha"], h["pairing_cut"] = v[0:2], v[2:4], v[4:6]
    r = next(it)
    h["has_cutoffs"] = int(n > 0 and len(r) >= 8 * n)
    w["cutoffs"] = np.frombuffer(r[:8 * n], "<f8") if h["has_cutoffs"] else np.zeros(0)
    v = np.frombuffer(nxt(32)[:32], "<f8")
    h["fermi"], h["ln_lambda"] = v[0:2], v[2:4]
    m = 2 * n if h["trc"] else n
    pi, ii = (2 if h["pc"] else 1), (2 if h["ic"] else 1)
    w["blocksizes"] = np.frombuffer(nxt(4 * pi * ii)[:4 * pi * ii], "<i4")
    nu = 2 * m * 2 * m * 4
    r = nxt(16 * nu)
    w["U"] = np.frombuffer(r[:8 * nu], "<f8")
    w["V"] = np.frombuffer(r[8 * nu:16 * nu], "<f8")
    w["columns"] = np.frombuffer(nxt(4 * m * pi * ii)[:4 * m * pi * ii], "<i4")
    nr = 2 * m * m * 4
    r = nxt(16 * nr)
    w["rhohfb"] = np.frombuffer(r[:8 * nr], "<f8")
    w["kappahfb"] = np.frombuffer(r[8 * nr:16 * nr], "<f8")
    r = nxt(16 * m * m * pi * ii)
    blk = 16 * m * m
    h["can_blocks"] = max(pi * ii, min(4, len(r) // blk)) if blk else pi * ii
    w["cantransfo"] = np.frombuffer(r[:blk * h["can_blocks"]], "<f8")
    v = np.frombuffer(nxt(48)[:48], "<f8")
    h["omega"], h["crank_values"] = v[0:3], v[3:6]
    mi, mr = [], []
    for r in it:
        if len(r) < 20:
            raise ValueError("moment record")
        mi.append(np.frombuffer(r[:20], "<i4"))
        r2 = next(it, None)
        if r2 is None or len(r2) < 176:
            raise ValueError("moment record")
        mr.append(np.frombuffer(r2[:176], "<f8"))
    h["n_moments"] = len(mi)
    w["moment_int"] = np.concatenate(mi).astype(np.int32) if mi else np.zeros(0, np.int32)
    w["moment_real"] = np.concatenate(mr) if mr else np.zeros(0)
    h["hfb_size"], h["pindex"], h["iindex"] = m, pi, ii
    h["version"] = 1
    w.update(h)
    return w


# ---- reference algorithms the file carries ---------------------------------------

def guess_hf_kappa(blocksignatures: list[list[int]], m: int) -> np.ndarray:
    """KappaHFB of GuessHFBMatrices(0) (src/HFB.f90:3686-3718): the double
    loop over (j, i) sets kappa(i, j) = 0.1, kappa(j, i) = -0.1 for indices
    of opposite (or undefined) signature; later iterations overwrite earlier
    ones.  Returns the complex array flattened as (re, im) pairs, blocks
    (P, it) in Fortran order, 2 x 2 blocks."""
    K = np.zeros((2, 2, m, m), dtype=np.complex128)   # [it][P][j][i]
    for b, sig in enumerate(blocksignatures):
        P, it = b % 2, b // 2
        N = len(sig)
        for j in range(N):
            for i in range(N):
                if sig[j] * sig[i] > 0:
                    continue
                K[it, P, j, i] = 0.1
                K[it, P, i, j] = -0.1
    return np.stack([K.real, K.imag], axis=-1).ravel()


def diag_ang(psi: np.ndarray, der: np.ndarray, X, Y, Z, dv: float, sc: bool, tsc: bool):
    """<J> of DiagAng (src/Spwf.f90:976-1085) for one spwf: psi [4][V],
    der [3][4][V] (d/dx, d/dy, d/dz), mesh coordinates X, Y, Z [V]."""
    p1, p2, p3, p4 = psi
    dx_, dy_, dz_ = der
    J = np.zeros(3)
    if not sc:
        J[0] = np.sum(0.5 * (p1 * p3 + p2 * p4 + p3 * p1 + p4 * p2)
                      + p2 * Z * dy_[0] - p2 * Y * dz_[0] - p1 * Z * dy_[1] + p1 * Y * dz_[1]
                      + p4 * Z * dy_[2] - p4 * Y * dz_[2] - p3 * Z * dy_[3] + p3 * Y * dz_[3])
    if not (sc or tsc):
        J[1] = np.sum(0.5 * (p1 * p4 - p2 * p3 - p3 * p2 + p4 * p1)
                      + p2 * X * dz_[0] - p2 * Z * dx_[0] - p1 * X * dz_[1] + p1 * Z * dx_[1]
                      + p4 * X * dz_[2] - p4 * Z * dx_[2] - p3 * X * dz_[3] + p3 * Z * dx_[3])
    J[2] = np.sum(0.5 * (p1 * p1 + p2 * p2 - p3 * p3 - p4 * p4)
                  + p2 * Y * dx_[0] - p2 * X * dy_[0] - p1 * Y * dx_[1] + p1 * X * dy_[1]
                  + p4 * Y * dx_[2] - p4 * X * dy_[2] - p3 * Y * dx_[3] + p3 * X * dy_[3])
    return J * dv
