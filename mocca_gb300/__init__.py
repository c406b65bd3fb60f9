"""GB300-native (sm_103a) implementation of MOCCa's per-iteration mesh hot path.

The compute lives in libmocca_gpu.so (C ABI: include/mocca_gpu.h); this
package holds the ctypes binding (`_abi`), the reference-shaped host mirror
(`mesh.MeshState`), the .wf wavefunction files (`wf.WavefunctionFile`, C
ABI include/mocca_wf.h), Skyrme parameter sets (`forces`) and seeded
synthetic inputs (`synthetic`).  There is no CPU fallback: without the library every
entry point raises.
"""
from ._abi import (MG_CAN_BASIS, MG_FP64, MG_HF_BASIS, MG_MIXED, MG_PAIRING_HF,  # noqa: F401
                   MG_PAIRING_HFB, MgError)
from .forces import SLY4, Force, RunParams  # noqa: F401


def build(force: bool = False, verbose: bool = False):
    from .build import build as _build
    return _build(force=force, verbose=verbose)


def MeshState(*args, **kwargs):  # noqa: N802 - mirrors the class it returns
    from .mesh import MeshState as _MS
    return _MS(*args, **kwargs)
