"""CPU restatement of the reference's symmetry-breaking transforms, for tests.

TEST INFRASTRUCTURE: the checker of mg_break_symmetries.  Only tests/ use
it; the product never imports it.

BreakParity, BreakSignature and BreakTimeSimplex (src/Transform.f90:187-366)
applied one after another, in TransformInput's order (:83-99), to one EV8
spinor [4][nz][ny][nx]: each doubles one axis, keeps the stored values on
the positive side and puts the reversed line times CompSignExtension's sign
(src/Derivatives.f90:348-439, with the symmetries conserved at that step)
on the negative side.
"""
from __future__ import annotations

import numpy as np


def sign_extension(direction: int, parity: int, signature: int, timesimplex: int,
                   component: int) -> int:
    """CompSignExtension (src/Derivatives.f90:348-439); component 1..4."""
    if direction == 1:
        if signature == 0:
            return 0
        if timesimplex != 0:
            return {1: 1, 2: -1, 3: -1, 4: 1}[component] * signature * timesimplex
        return signature if component in (1, 2) else -signature
    if direction == 2:
        if timesimplex == 0:
            return 0
        return timesimplex if component in (1, 3) else -timesimplex
    if parity == 0:
        return 0
    if signature != 0:
        return signature * parity if component in (1, 2) else -signature * parity
    if timesimplex != 0:
        return parity * timesimplex if component in (1, 3) else -parity * timesimplex
    return parity


def break_all(psi: np.ndarray, parity: int, signature: int = 1, timesimplex: int = 1):
    """psi [4][nz][ny][nx] of an EV8 spwf -> [4][2nz][2ny][2nx]."""
    out = np.asarray(psi, dtype=np.float64)
    # BreakParity: z doubles; signature and time simplex still conserved
    # (LineExtensionCoulombZ reads the same (x, y) line)
    s = [sign_extension(3, parity, signature, timesimplex, c) for c in (1, 2, 3, 4)]
    out = np.concatenate([np.stack([s[c] * out[c, ::-1] for c in range(4)]), out], axis=1)
    # BreakSignature: x doubles; time simplex still conserved
    s = [sign_extension(1, 0, signature, timesimplex, c) for c in (1, 2, 3, 4)]
    out = np.concatenate([np.stack([s[c] * out[c, :, :, ::-1] for c in range(4)]), out], axis=3)
    # BreakTimeSimplex: y doubles
    s = [sign_extension(2, 0, 0, timesimplex, c) for c in (1, 2, 3, 4)]
    out = np.concatenate([np.stack([s[c] * out[c, :, ::-1, :] for c in range(4)]), out], axis=2)
    return out
