"""CPU pin of the oracle's tensor density J_{mu nu} (no reference artefact
holds one).

The vector part of the tensor density, J_k = eps_{k mu nu} J_{mu nu} with
J_{mu nu} = Im(psi^+ sigma_nu d_mu psi) (GetJMuNu, src/Spwf.f90:2186-2204),
is the spin-orbit current, whose divergence is the density of GetNablaJ
(src/Spwf.f90:2206-2243): div J = eps_{k mu nu} Im(d_k psi^+ sigma_nu d_mu psi),
the second-derivative part cancelling by symmetry.  On the mesh the Lagrange
derivative of the product J_k and the product of derivatives agree to the
discretisation error, so the oracle's J_{mu nu} and nabla J must satisfy
div(eps J) = nabla J up to that error; an exchanged (mu, nu)
convention flips the sign and misses by ~2.  Full box (unfolded Lagrange
matrices), Gaussian-Hermite spinors (their tails reach the box edge, which
leaves the mesh forms ~1-6% apart): the oracle's convention must land within
0.2, the exchanged one beyond 1.5.
"""
import numpy as np

import oracle as O
from mocca_gb300 import RunParams, synthetic
from mocca_gb300.forces import SLY5_TENSOR


def test_vector_part_of_jmunu_has_the_spin_orbit_divergence(built):
    p = RunParams(nx=24, ny=24, nz=24, dx=0.8, pc=0, sc=0, tsc=0, trc=1, nwt=6, neutrons=6,
                  protons=6, coulomb_solver=0)
    psi = synthetic.gaussian_hermite_spinors(p, p.nwt, seed=11)
    qn = np.tile(np.array([-1, 0, 0, 0], dtype=np.int32), (p.nwt, 1))
    qn[3:, 0] = 1
    o = O.OracleState(p, SLY5_TENSOR)
    o.set_spinors(psi, qn)
    o.set_occupations(np.full(p.nwt, 2.0))
    o.DeriveAll()
    o.UpdateDensities()
    V = p.nx * p.ny * p.nz
    J = o.get_jmunu().reshape(2, 3, 3, V)   # [it][nu][mu]
    nj = o.get_densities()["nablaj"].reshape(2, V)
    eps = np.zeros((3, 3, 3))
    eps[0, 1, 2] = eps[1, 2, 0] = eps[2, 0, 1] = 1
    eps[0, 2, 1] = eps[2, 1, 0] = eps[1, 0, 2] = -1
    for it in range(2):
        assert np.abs(nj[it]).max() > 1e-4
        errs = []
        for swap in (False, True):
            div = np.zeros(V)
            for k in range(3):
                Jk = sum(eps[k, mu, nu] * (J[it, mu, nu] if swap else J[it, nu, mu])
                         for mu in range(3) for nu in range(3))
                div += o.derive_grid(Jk.reshape(p.nz, p.ny, p.nx), k, 0, 0, 0, 1).ravel()
            errs.append(np.linalg.norm(div - nj[it]) / np.linalg.norm(nj[it]))
        assert errs[0] < 0.2 and errs[1] > 1.5, (it, errs)
