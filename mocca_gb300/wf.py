"""MOCCa wavefunction files (.wf, format version 1) through libmocca_gpu.

`WavefunctionFile` holds one file's content in the library's host memory
(include/mocca_wf.h): `load` parses a file as ReadMOCCa_v1 does
(src/InOut.f90:1050-1416), `save` writes WriteMOCCa_v1's records
(src/InOut.f90:905-1046), `header` gives the scalars and `field(name)` a
numpy view of an array (Fortran element order, writable).  `from_state`
gathers a MeshState's device state into a file; `to_state` restarts a
MeshState from one.

All parsing and writing happens in the native library; a missing library
raises, there is no Python fallback.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import _abi

FIELD_IDS = {name: k for k, name in enumerate(_abi.WF_FIELDS)}


def _header_dict(h: _abi.MgWfHeader) -> dict:
    out = {}
    for name, typ in _abi.MgWfHeader._fields_:
        v = getattr(h, name)
        if name == "force":
            v = v.decode("ascii", "replace")
        elif hasattr(typ, "_length_"):
            v = np.array(v[:], dtype=np.float64)
        out[name] = v
    return out


def _header_struct(d: dict) -> _abi.MgWfHeader:
    h = _abi.MgWfHeader()
    for name, typ in _abi.MgWfHeader._fields_:
        if name not in d:
            continue
        v = d[name]
        if name == "force":
            setattr(h, name, str(v).encode("ascii")[:207])
        elif hasattr(typ, "_length_"):
            arr = getattr(h, name)
            for k, x in enumerate(np.asarray(v, dtype=np.float64).ravel()[:typ._length_]):
                arr[k] = float(x)
        elif typ is C.c_int:
            setattr(h, name, int(v))
        else:
            setattr(h, name, float(v))
    return h


class WavefunctionFile:
    """One version-1 .wf file held by the native library."""

    def __init__(self, handle: C.c_void_p):
        self.lib = _abi.load()
        self.h = handle

    # ---- construction --------------------------------------------------------
    @classmethod
    def load(cls, path: str | Path) -> "WavefunctionFile":
        lib = _abi.load()
        h = C.c_void_p()
        _abi.check("mg_wf_load", lib.mg_wf_load(str(path).encode(), C.byref(h)))
        return cls(h)

    @classmethod
    def new(cls, header: dict) -> "WavefunctionFile":
        """Zero arrays shaped by header's nx, ny, nz, nwt, symmetries and the
        optional-record flags (has_cutoffs, has_jmunu, odd_records,
        n_moments, can_blocks)."""
        lib = _abi.load()
        h = C.c_void_p()
        hs = _header_struct(header)
        _abi.check("mg_wf_new", lib.mg_wf_new(C.byref(hs), C.byref(h)))
        return cls(h)

    @classmethod
    def from_state(cls, state, force_name: str | None = None) -> "WavefunctionFile":
        """The state WriteMOCCa_v1 writes, gathered from a MeshState."""
        lib = _abi.load()
        h = C.c_void_p()
        name = (force_name if force_name is not None else getattr(state.force, "name", ""))
        _abi.check("mg_wf_from_context",
                   lib.mg_wf_from_context(state.h, str(name).encode(), C.byref(h)))
        return cls(h)

    def to_state(self, state) -> None:
        """Restart a MeshState from this file (before its first pairing step;
        under HFB after set_pairing)."""
        _abi.check("mg_wf_to_context", self.lib.mg_wf_to_context(state.h, self.h))

    # ---- access --------------------------------------------------------------
    def save(self, path: str | Path) -> None:
        _abi.check("mg_wf_save", self.lib.mg_wf_save(self.h, str(path).encode()))

    @property
    def header(self) -> dict:
        hs = _abi.MgWfHeader()
        _abi.check("mg_wf_get_header", self.lib.mg_wf_get_header(self.h, C.byref(hs)))
        return _header_dict(hs)

    def set_scalars(self, **values) -> None:
        d = self.header
        d.update(values)
        hs = _header_struct(d)
        _abi.check("mg_wf_set_scalars", self.lib.mg_wf_set_scalars(self.h, C.byref(hs)))

    def field(self, name: str) -> np.ndarray:
        """A writable view of one array (valid while this object lives)."""
        ptr = C.c_void_p()
        n = C.c_longlong()
        _abi.check("mg_wf_field",
                   self.lib.mg_wf_field(self.h, FIELD_IDS[name], C.byref(ptr), C.byref(n)))
        is_int = name in _abi.WF_INT_FIELDS
        if n.value == 0:
            return np.zeros(0, dtype=np.int32 if is_int else np.float64)
        ct = C.c_int if is_int else C.c_double
        arr = np.ctypeslib.as_array(C.cast(ptr, C.POINTER(ct)), shape=(n.value,))
        arr.flags.writeable = True
        return arr

    def arrays(self) -> dict:
        return {name: self.field(name).copy() for name in _abi.WF_FIELDS}

    # ---- lifetime ------------------------------------------------------------
    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.mg_wf_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
