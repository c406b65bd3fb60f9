"""Skyrme parameter sets and run parameters.

`SLY4` restates the &skf group "Sly4" of the reference's forces.param
(forces.param:9-15) together with the constants that ReadForce leaves at
their defaults (src/Force.f90:103-105, :170-176): e2, hbar, the nucleon
masses averaged when averagemass (src/Force.f90:243-244) and hbm = 2 x
20.73551910 (src/Force.f90:246).
"""
from __future__ import annotations

from dataclasses import dataclass, field

from . import _abi


@dataclass
class Force:
    t0: float = 0.0
    x0: float = 0.0
    t1: float = 0.0
    x1: float = 0.0
    t2: float = 0.0
    x2: float = 0.0
    t3a: float = 0.0
    x3a: float = 0.0
    yt3a: float = 0.0
    t3b: float = 0.0
    x3b: float = 0.0
    yt3b: float = 0.0
    te: float = 0.0
    to: float = 0.0
    wso: float = 0.0
    wsoq: float = 0.0
    hbm: float = 2.0 * 20.73551910
    e2: float = 1.43996446
    hbar: float = 6.58211928
    nucleonmass: tuple = (939.565379, 938.272046)
    averagemass: bool = True
    com1body: int = 0
    com2body: int = 0
    cexchange: int = 2
    j2terms: bool = False     # J2Terms: J^2 terms in B14, B15 (tensor te, to)
    name: str = ""            # afor, the &skf group's name (written to .wf files)

    def to_c(self) -> _abi.MgForce:
        f = _abi.MgForce()
        for name in ("t0", "x0", "t1", "x1", "t2", "x2", "t3a", "x3a", "yt3a", "t3b", "x3b",
                     "yt3b", "te", "to", "wso", "wsoq", "hbm", "e2", "hbar"):
            setattr(f, name, float(getattr(self, name)))
        m = self.nucleonmass
        if self.averagemass:
            avg = (m[0] + m[1]) / 2
            m = (avg, avg)
        f.nucleonmass[0], f.nucleonmass[1] = m
        f.com1body, f.com2body, f.cexchange = self.com1body, self.com2body, self.cexchange
        f.j2terms = int(bool(self.j2terms))
        f.coupling = COUPLING_OVERRIDES.get(self.name.strip().upper(), 0)
        return f


# CalcEDFCoef overrides B14..B17 for these names (src/Force.f90:552-597)
COUPLING_OVERRIDES = {"SLY4T": 1, "SLY4TMIN": 2, "UNEDF2": 3}


# &skf "SLy5colo" (forces.param:145-154): SLy5 with the tensor te = 296,
# to = -136 MeV fm^5 and J2Terms = T.
SLY5_TENSOR = Force(t0=-2484.880, x0=0.778, t1=483.130, x1=-0.328, t2=-549.400, x2=-1.0,
                    t3a=13763.0, x3a=1.267, yt3a=0.1666666666666667, wso=126.0, wsoq=126.0,
                    te=296.0, to=-136.0, j2terms=True, com1body=2, name="SLy5colo")

SLY4 = Force(t0=-2488.913, x0=0.834, t1=486.818, x1=-0.344, t2=-546.395, x2=-1.0,
             t3a=13777.0, x3a=1.354, yt3a=0.166666666666666666667, t3b=0.0, x3b=0.0,
             yt3b=0.0, wso=123.0, wsoq=123.0, com1body=2, name="SLy4")


@dataclass
class RunParams:
    """&GenInfo / &SpwfStorage / &Coulomb values of one run."""
    nx: int
    ny: int
    nz: int
    dx: float = 0.8
    pc: int = 1
    sc: int = 1
    tsc: int = 1
    trc: int = 1
    nwt: int = 40
    neutrons: float = 12.0
    protons: float = 12.0
    precision: int = _abi.MG_FP64
    pairing: int = _abi.MG_PAIRING_HF
    coulomb_max: int = 500
    max_l_coul: int = 10
    coulomb_solver: int = 1
    mixing_scheme: int = 0      # MixingScheme: 0 linear density mixing, 2 preconditioned U
    damping: float = 0.75       # DampingParam
    precon_u: float = 1.0       # preconu
    precon_w: float = 0.0       # PreConW: > 0 preconditions the W update too (MixingScheme 2)
    parameter_estimation: int = 0   # ParameterEstimation: 1 estimates dt, momentum every step
    coulomb_prec: float = 0.0   # > 0: relative residual of the CG / multigrid Coulomb solves
    omega: tuple = (0.0, 0.0, 0.0)  # cranking OmegaX, OmegaY, OmegaZ (needs trc = 0)
    extra: dict = field(default_factory=dict)

    @property
    def V(self) -> int:
        return self.nx * self.ny * self.nz

    @property
    def dv(self) -> float:
        return self.dx ** 3 * 2.0 ** (self.pc + self.sc + self.tsc)

    def to_c(self) -> _abi.MgParams:
        p = _abi.MgParams()
        for name, _ in _abi.MgParams._fields_:
            if name == "omega":
                for k in range(3):
                    p.omega[k] = float(self.omega[k])
            else:
                setattr(p, name, getattr(self, name))
        return p
