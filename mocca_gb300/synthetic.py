"""Seeded synthetic inputs with the shapes of the benchmark configurations.

The reference ships no wavefunction files and no datasets, so these stand in
for them:

* `ho_basis` -- harmonic-oscillator start for an EV8 + time-reversal run:
  one stored spwf per Cartesian HO orbital (nx, ny, nz), signature +1 and
  time simplex +1 as the reference's from-scratch guess uses
  (src/InOut.f90:1418-1473), placed in the spinor component whose mirror
  parities match the orbital (the sign rules of
  src/Derivatives.f90:348-439), plus a seeded uniform perturbation.
* `nilsson_basis` -- the reference's own from-scratch guess (INITWF with the
  Nilsson-model routine of nil8), restated with numpy, plus a seeded uniform
  perturbation.
* `uneven_instances` -- the batched workload: quadrupole-constrained HFB
  runs with random deformation targets, particle numbers, meshes and spwf
  counts.
* `gaussian_hermite_spinors` / `woods_saxon_fields` -- the mesh microbench
  (32^3 full box, 200 spinors): Gaussian envelopes of random width and
  centre times random Hermite polynomials, and Woods-Saxon U, B, W fields.
"""
from __future__ import annotations

import math

import numpy as np

from .forces import RunParams


def mesh_axes(p: RunParams):
    """Stored mesh coordinates (Mesh.f90:49-73)."""
    def axis(n, conserved):
        x = p.dx / 2.0 + p.dx * np.arange(n)
        return x if conserved else x - n / 2.0 * p.dx
    return axis(p.nx, p.sc), axis(p.ny, p.tsc), axis(p.nz, p.pc)


def _hermite(n: int, x: np.ndarray) -> np.ndarray:
    h0, h1 = np.ones_like(x), 2 * x
    if n == 0:
        return h0
    for k in range(1, n):
        h0, h1 = h1, 2 * x * h1 - 2 * k * h0
    return h1


def ho_orbitals(count: int):
    """Cartesian HO orbitals (nx,ny,nz) by shell, then lexicographic."""
    out = []
    N = 0
    while len(out) < count:
        for a in range(N, -1, -1):
            for b in range(N - a, -1, -1):
                out.append((a, b, N - a - b))
        N += 1
    return out[:count]


# spinor component (0..3) holding an orbital with x/y parities (odd?) for
# signature +1: (even,even)->Re up, (odd,odd)->Im up, (odd,even)->Re down,
# (even,odd)->Im down; the spwf parity follows from nz.
_COMP = {(0, 0): 0, (1, 1): 1, (1, 0): 2, (0, 1): 3}


def ho_basis(p: RunParams, n_neutron: int, seed: int = 1234, amplitude: float = 1e-3,
             b_osc: float | None = None):
    """HO start for an EV8 run: returns (psi[nwt,4,nz,ny,nx], qn[nwt,4], energies)."""
    if not (p.pc and p.sc and p.tsc):
        raise ValueError("ho_basis builds EV8 (all spatial symmetries conserved) states")
    nwt = p.nwt
    n_proton = nwt - n_neutron
    A = p.neutrons + p.protons
    hw = 41.0 * A ** (-1.0 / 3.0)
    if b_osc is None:
        b_osc = math.sqrt(41.47 / hw)  # hbar^2/m / (hbar omega), fm^2
    x, y, z = mesh_axes(p)
    rng = np.random.default_rng(seed)
    psi = np.zeros((nwt, 4, p.nz, p.ny, p.nx))
    qn = np.zeros((nwt, 4), dtype=np.int32)
    en = np.zeros(nwt)
    k = 0
    for iso, count in ((-1, n_neutron), (1, n_proton)):
        for (a, b, c) in ho_orbitals(count):
            comp = _COMP[(a % 2, b % 2)]
            parity = (-1) ** c if comp in (0, 1) else -((-1) ** c)
            fx = _hermite(a, x / b_osc) * np.exp(-0.5 * (x / b_osc) ** 2)
            fy = _hermite(b, y / b_osc) * np.exp(-0.5 * (y / b_osc) ** 2)
            fz = _hermite(c, z / b_osc) * np.exp(-0.5 * (z / b_osc) ** 2)
            g = fz[:, None, None] * fy[None, :, None] * fx[None, None, :]
            psi[k, comp] = g
            psi[k] += amplitude * rng.uniform(-1.0, 1.0, size=psi[k].shape) * np.abs(g).max()
            nrm = math.sqrt(float(np.sum(psi[k] ** 2)) * p.dv)
            psi[k] /= nrm
            qn[k] = (iso, parity, 1, 1)
            en[k] = -50.0 + hw * (a + b + c + 1.5)
            k += 1
    return psi, qn, en


def gaussian_hermite_spinors(p: RunParams, count: int, seed: int = 42):
    """Microbench spinors on the full (symmetry-free) box."""
    x, y, z = mesh_axes(p)
    rng = np.random.default_rng(seed)
    out = np.zeros((count, 4, p.nz, p.ny, p.nx))
    for i in range(count):
        for l in range(4):
            w = rng.uniform(1.5, 3.0)
            c = rng.uniform(-3.0, 3.0, size=3)
            d = rng.integers(0, 4, size=3)
            fx = _hermite(int(d[0]), (x - c[0]) / w) * np.exp(-0.5 * ((x - c[0]) / w) ** 2)
            fy = _hermite(int(d[1]), (y - c[1]) / w) * np.exp(-0.5 * ((y - c[1]) / w) ** 2)
            fz = _hermite(int(d[2]), (z - c[2]) / w) * np.exp(-0.5 * ((z - c[2]) / w) ** 2)
            out[i, l] = fz[:, None, None] * fy[None, :, None] * fx[None, None, :]
        out[i] /= math.sqrt(float(np.sum(out[i] ** 2)) * p.dv)
    return out


def woods_saxon_fields(p: RunParams, R: float = 3.5, a: float = 0.65, u0: float = -50.0,
                       b0: float = 20.7, w0: float = 120.0):
    """U, B, grad B, W, div W of Woods-Saxon form, both isospins equal.

    U = u0 f, B = b0 f, W_mn = -eps_kmn w0 d_k f, f = 1/(1+exp((r-R)/a)).
    """
    x, y, z = mesh_axes(p)
    Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
    r = np.sqrt(X ** 2 + Y ** 2 + Z ** 2)
    f = 1.0 / (1.0 + np.exp((r - R) / a))
    df = -f * (1 - f) / a
    rs = np.where(r > 0, r, 1.0)
    grad = [df * X / rs, df * Y / rs, df * Z / rs]
    V = p.V
    U = np.stack([u0 * f, u0 * f]).reshape(2, V)
    B = np.stack([b0 * f, b0 * f]).reshape(2, V)
    nablaB = np.stack([np.stack([b0 * g for g in grad])] * 2).reshape(2, 3, V)
    W = np.zeros((2, 3, 3, V))
    eps = np.zeros((3, 3, 3))
    eps[0, 1, 2] = eps[1, 2, 0] = eps[2, 0, 1] = 1
    eps[0, 2, 1] = eps[2, 1, 0] = eps[1, 0, 2] = -1
    for n in range(3):
        for m in range(3):
            acc = np.zeros(V)
            for k in range(3):
                acc -= eps[k, m, n] * w0 * grad[k].reshape(V)
            W[:, n, m] = acc
    divW = np.zeros((2, 3, V))
    return U, B, nablaB, W, divW


def beta2_to_q20(beta2: float, A: float) -> float:
    """<Q20> (fm^2) of a deformation beta2, inverting CalcBeta
    (src/Moments.f90:3472-3494): beta = 4 pi Q / (3 A R^2), R = 1.2 A^(1/3)."""
    R = 1.2 * A ** (1.0 / 3.0)
    return beta2 * 3.0 * A * R * R / (4.0 * math.pi)


def uneven_instances(count: int = 64, seed: int = 7, n_range=(12, 28), dx: float = 0.8,
                     precision: int = 1, pairing: int = 2):
    """Seeded independent constrained-HFB instances of uneven size.

    Per instance: beta2 ~ U[-0.3, 0.5]; N, Z even in [8, 40]; stored mesh n
    uniform in [n_min(A), 28] with n_min(A) = max(12, ceil((1.2 A^(1/3) + 6) /
    dx)) so the box holds the nucleus; nwt = round(1.4 (N + Z)) clipped to
    [20, 200] and made even, split between neutrons and protons in
    proportion to N and Z.  Returns a list of dicts with the RunParams, the
    neutron spwf count, the Q20 target and the start seed.
    """
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        beta2 = float(rng.uniform(-0.3, 0.5))
        N = int(rng.integers(4, 21)) * 2
        Z = int(rng.integers(4, 21)) * 2
        A = N + Z
        n_min = max(n_range[0], math.ceil((1.2 * A ** (1.0 / 3.0) + 6.0) / dx))
        n = int(rng.integers(min(n_min, n_range[1]), n_range[1] + 1))
        nwt = int(min(200, max(20, round(1.4 * A))))
        nwt += nwt % 2
        n_neutron = max(N // 2 + 2, min(nwt - Z // 2 - 2, round(nwt * N / A)))
        p = RunParams(nx=n, ny=n, nz=n, dx=dx, nwt=nwt, neutrons=float(N), protons=float(Z),
                      precision=precision, pairing=pairing)
        out.append({"params": p, "n_neutron": int(n_neutron), "beta2": beta2,
                    "q20": beta2_to_q20(beta2, A), "seed": seed * 1000 + i})
    return out


def _nilsson_shell_states(meven: int, modd: int):
    """Cartesian HO states (nx, ny, nz) of the first `meven` even and `modd`
    odd major shells in nil8's order (src/nil8.f90:162-268): per shell the
    four sub-blocks (x, y parities) one after another; returns the states,
    the shell start offsets and the sub-block sizes of each shell."""
    states, starts, subs = [], [0], []
    shells = [2 * (ni - 1) for ni in range(1, meven + 1)] + [2 * ni - 1 for ni in range(1, modd + 1)]
    for n in shells:
        ni = n // 2 + 1 if n % 2 == 0 else (n + 1) // 2
        blocks = []
        if n % 2 == 0:
            blocks.append([(2 * (i - 1), 2 * (j - 1)) for i in range(1, ni + 1)
                           for j in range(1, ni - i + 2)])
            if ni > 1:
                blocks.append([(2 * (i - 1) + 1, 2 * (j - 1) + 1) for i in range(1, ni)
                               for j in range(1, ni - i + 1)])
                blocks.append([(2 * (i - 1) + 1, 2 * (j - 1)) for i in range(1, ni)
                               for j in range(1, ni - i + 1)])
                blocks.append([(2 * (i - 1), 2 * (j - 1) + 1) for i in range(1, ni)
                               for j in range(1, ni - i + 1)])
            else:
                blocks += [[], [], []]
        else:
            blocks.append([(2 * (i - 1), 2 * (j - 1)) for i in range(1, ni + 1)
                           for j in range(1, ni - i + 2)])
            blocks.append([(2 * i - 1, 2 * j - 1) for i in range(1, ni) for j in range(1, ni - i + 1)])
            blocks.append([(2 * i - 1, 2 * (j - 1)) for i in range(1, ni + 1)
                           for j in range(1, ni - i + 2)])
            blocks.append([(2 * (i - 1), 2 * j - 1) for i in range(1, ni + 1)
                           for j in range(1, ni - i + 2)])
        subs.append([len(b) for b in blocks])
        for b in blocks:
            states += [(a, c, n - a - c) for (a, c) in b]
        starts.append(len(states))
    return states, starts, subs


def _nilsson_block_matrix(states, x, y, ax, ay, az):
    """Nilsson Hamiltonian of one major shell in units of hbar omega0, with
    stretched l.s (strength kappa = x) and l^2 (x mu = x y) terms
    (src/nil8.f90:383-433)."""
    n = len(states)
    h = np.zeros((n, n))
    for i in range(n):
        nx1, ny1, nz1 = states[i]
        nb = nx1 + ny1 + nz1
        x1 = 1 - 2 * ((nb - nz1) % 2)
        x2 = 1 - 2 * (ny1 % 2)
        for j in range(i, n):
            nx2, ny2, nz2 = states[j]
            if j == i:
                v = (ax * (nx1 + 0.5) + ay * (ny1 + 0.5) + az * (nz1 + 0.5)
                     - x * y * ((nb * (nb + 1)) / 2.0 - nx1 ** 2 - ny1 ** 2 - nz1 ** 2))
            elif nx1 == nx2:
                v = 0.0
                an, am = float(ny2), float(ny1)
                if ny2 == ny1 + 1: v = x * math.sqrt(an * nz1)
                if ny2 == ny1 - 1: v = x * math.sqrt(am * nz2)
                if ny2 == ny1 + 2: v = -x * y * math.sqrt(an * (ny2 - 1) * nz1 * (nz1 - 1))
                if ny2 == ny1 - 2: v = -x * y * math.sqrt(am * (ny1 - 1) * nz2 * (nz2 - 1))
            elif nz1 == nz2:
                v = 0.0
                am, an = float(nx1), float(nx2)
                if nx2 == nx1 + 1: v = -x * x1 * math.sqrt(an * ny1)
                if nx2 == nx1 - 1: v = -x * x1 * math.sqrt(am * ny2)
                if nx2 == nx1 + 2: v = -x * y * math.sqrt(an * (nx2 - 1) * ny1 * (ny1 - 1))
                if nx2 == nx1 - 2: v = -x * y * math.sqrt(am * (nx1 - 1) * ny2 * (ny2 - 1))
            else:
                v = 0.0
                if ny1 == ny2:
                    x3 = 1.0 - 2.0 * (nx1 % 2)
                    x4 = 1.0 - 2.0 * (nx2 % 2)
                    an, am = float(nx2), float(nx1)
                    if nz2 == nz1 + 1: v = -x * x2 * x3 * math.sqrt(am * nz2)
                    if nz2 == nz1 - 1: v = -x * x2 * x4 * math.sqrt(an * nz1)
                    if nz2 == nz1 + 2: v = x * y * math.sqrt(nz2 * (nz2 - 1) * am * (nx1 - 1))
                    if nz2 == nz1 - 2: v = x * y * math.sqrt(nz1 * (nz1 - 1) * an * (nx2 - 1))
            h[i, j] = h[j, i] = v
    return h


def _nilsson_hermite(nfun: int, npts: int, xho: float, dx: float) -> np.ndarray:
    """The 1-D oscillator functions of nil8 on the stored half line
    (src/nil8.f90:283-339): x^k exp(-x^2/2) built by multiplication,
    orthogonalised against the lower functions of the same parity and
    normalised on the mirrored full line."""
    he = np.zeros((nfun, npts))
    xs = xho * (np.arange(1, npts + 1) - 0.5)
    for j in range(1, nfun // 2 + 1):
        a, b = 2 * j - 2, 2 * j - 1
        if j == 1:
            he[0] = np.exp(-xs * xs / 2.0)
            he[1] = xs * he[0]
        else:
            x2 = xs * xs
            he[a] = he[a - 2] * x2
            he[b] = he[b - 2] * x2
            for k in range(1, j):
                c, d = 2 * k - 2, 2 * k - 1
                s1 = float(np.sum(he[a] * he[c])) * dx * 2.0
                s2 = float(np.sum(he[b] * he[d])) * dx * 2.0
                he[a] = he[a] - s1 * he[c]
                he[b] = he[b] - s2 * he[d]
        he[a] *= math.sqrt(0.5 / (dx * float(np.sum(he[a] ** 2))))
        he[b] *= math.sqrt(0.5 / (dx * float(np.sum(he[b] ** 2))))
    return he


def nilsson_basis(p: RunParams, n_neutron: int, seed: int = 1234, amplitude: float = 1e-3,
                  meven: int = 6, modd: int = 5, ho=(0.2, 0.2, 0.2)):
    """The reference's from-scratch guess for an EV8 run: INITWF
    (src/InOut.f90:1418-1473) calling the Nilsson routine of nil8
    (src/nil8.f90:16-546) with 6 even and 5 odd shells and m omega / hbar =
    0.2 fm^-2 on every axis, then a seeded uniform perturbation of the given
    absolute amplitude on every spinor value (each spwf renormalised).

    Returns (psi[nwt,4,nz,ny,nx], qn[nwt,4], energies) like `ho_basis`:
    neutrons first (n_neutron of them), positive parity first within each
    isospin, signature and time simplex +1.  The block diagonalisation uses
    numpy's symmetric eigensolver, so inside an exactly degenerate Nilsson
    level the eigenvectors may differ from the reference's diagoncr8 by a
    rotation (and any vector by its sign).
    """
    if not (p.pc and p.sc and p.tsc):
        raise ValueError("nilsson_basis builds EV8 (all spatial symmetries conserved) states")
    if max(p.nx, p.ny) > p.nz:
        raise ValueError("nil8 needs nz >= nx, ny")
    nwt = p.nwt
    n_proton = nwt - n_neutron
    hox, hoy, hoz = ho
    # the reference passes floor(neutrons) as npp and floor(protons) as npn
    npp, npn = math.floor(p.neutrons), math.floor(p.protons)
    xk = (0.08, 0.08, 0.0637, 0.0637)
    xmu = (0.0, 0.0, 0.42, 0.60)
    hbm = 6.58218 ** 2 / 1.044673
    xis = (npn - npp) / (npn + npp)
    cf = (1.0 + 0.14 * xis, 0.986 - 0.14 * xis)
    states, starts, subs = _nilsson_shell_states(meven, modd)
    nvec = len(states)
    nmax = max(meven, modd)
    rng = np.random.default_rng(seed)
    psi = np.zeros((nwt, 4, p.nz, p.ny, p.nx))
    qn = np.zeros((nwt, 4), dtype=np.int32)
    en = np.zeros(nwt)
    w = 0
    for it, (iso, nw) in enumerate(((-1, n_neutron), (1, n_proton))):
        nn = max(p.nx, p.ny, p.nz)
        he = [_nilsson_hermite(2 * nmax, nn, math.sqrt(h) * p.dx * math.sqrt(cf[it]), p.dx)
              for h in (hox, hoy, hoz)]
        ho0 = (hox * hoy * hoz) ** (1.0 / 3.0)
        ax, ay, az = hox / ho0, hoy / ho0, hoz / ho0
        ho0 = ho0 * hbm * cf[it]
        npart = npn if it == 0 else npp
        x, y = (xk[it], xmu[it]) if npart <= 50 else (xk[it + 2], xmu[it + 2])
        e = np.zeros(nvec)
        vecs = []
        for b in range(len(starts) - 1):
            h = _nilsson_block_matrix(states[starts[b]:starts[b + 1]], x, y, ax, ay, az)
            d, s = np.linalg.eigh(h)
            vecs.append(s)
            e[starts[b]:starts[b + 1]] = d * ho0 - 50.0
        # exchange sort of nil8 (src/nil8.f90:437-449): ties keep its order
        nor = list(range(nvec))
        ev = e.copy()
        for i in range(nvec - 1):
            for j in range(i + 1, nvec):
                if ev[j] < ev[i]:
                    ev[i], ev[j] = ev[j], ev[i]
                    nor[i], nor[j] = nor[j], nor[i]
        npa = [1 - 2 * (sum(states[nor[i]]) % 2) for i in range(nvec)]
        order = [i for i in range(nw) if npa[i] != -1] + [i for i in range(nw) if npa[i] != 1]
        for i in order:
            j = nor[i]
            b = next(k for k in range(len(starts) - 1) if j < starts[k + 1])
            s = vecs[b][:, j - starts[b]]
            g = np.zeros((4, p.nz, p.ny, p.nx))
            off = 0
            for k in range(4):
                flip = 3 if k in (0, 2) else 0
                for q in range(off, off + subs[b][k]):
                    a1, a2, a3 = states[starts[b] + q]
                    xph = s[q]
                    if (a2 + 1) % 4 == flip:
                        xph = -xph
                    g[k] += xph * (he[2][a3, :p.nz][:, None, None] * he[1][a2, :p.ny][None, :, None]
                                   * he[0][a1, :p.nx][None, None, :])
                off += subs[b][k]
            g += amplitude * rng.uniform(-1.0, 1.0, size=g.shape)
            g /= math.sqrt(float(np.sum(g ** 2)) * p.dv)
            psi[w] = g
            qn[w] = (iso, npa[i], 1, 1)
            en[w] = ev[i]
            w += 1
    return psi, qn, en
