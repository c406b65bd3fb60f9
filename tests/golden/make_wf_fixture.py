"""Write tests/golden/wf_small_v1.wf, a small version-1 MOCCa wavefunction file.

The reference ships no .wf file and cannot be built here (no Fortran
compiler), so this fixture comes from the oracle's restatement of
WriteMOCCa_v1 (oracle/wf_format.py) on deterministic content: a 3 x 4 x 5
mesh with time reversal, 4 spwfs, every optional record present (JMuNu,
the five time-odd records, cutoffs, two constrained moments) and
CanTransfo with the 2 x 2 blocks GuessHFBMatrices allocates.  It pins the
record layout of the native file layer against regressions.  Run from the
repo root:
    python tests/golden/make_wf_fixture.py
"""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path[:0] = [str(ROOT), str(ROOT / "oracle")]

import wf_format as WF  # noqa: E402

PATH = Path(__file__).resolve().parent / "wf_small_v1.wf"


def content() -> dict:
    h = dict(energy=-198.765432109876, denergy=-3.25e-9, nx=3, ny=4, nz=5, dx=0.8,
             trc=1, pc=0, sc=1, tsc=1, ic=1, nwt=4, neutrons=12.0, protons=10.0,
             fd_order=-1, fd_lap_order=-1, coulomb_lap_order=2, force="SLy4",
             skyrme=np.arange(14) * 1.5 - 7.0, hbar=6.58211928, hbm=np.array([41.4710382] * 2),
             com1body=2, com2body=0, coef=np.linspace(-1.0, 1.0, 28), pairing_type=2,
             pairing_strength=np.array([-1250.0, -1250.0]), pairing_alpha=np.array([1.0, 1.0]),
             pairing_cut=np.array([5.0, 5.0]), fermi=np.array([-8.25, -6.5]),
             ln_lambda=np.array([0.0, 0.0]), omega=np.array([0.0, 0.0, 0.125]),
             crank_values=np.array([0.0, 0.0, 2.0]),
             has_cutoffs=1, has_jmunu=1, odd_records=31, n_moments=2, can_blocks=4)
    w = WF.empty(h)
    for k, name in enumerate(WF.FIELDS):
        a = w[name]
        if a.size == 0:
            continue
        if name in WF.INT_FIELDS:
            a[:] = (np.arange(a.size) * 7 + 3 * k) % 23 - 11
        else:
            a[:] = np.sin(np.arange(a.size) * 0.37 + k) * 10.0 ** (k % 5 - 2)
    w["spwf_int"][0::5] = [1, 1, -1, -1]      # isospins must be +-1
    w["moment_int"][:] = [2, 1, 2, 0, 0, 2, 1, 4, 2, 0]
    return w


if __name__ == "__main__":
    WF.write_v1(PATH, content())
    print(PATH, PATH.stat().st_size, "bytes")
