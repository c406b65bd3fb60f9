// oracle.cpp -- CPU FP64 restatement of MOCCa's mesh hot path.
//
// TEST INFRASTRUCTURE ONLY: the parity checker for the CUDA library.  Only
// tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg load it.
//
// Each routine cites the reference routine (path:line inside the MOCCa
// sources) it restates.  Loops keep the reference's summation order where it
// fixes the rounding (matmul over j ascending, spwf sums in index order,
// Laplacian = (X + Y) + Z).
#include "oracle.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

const double kPi = 4.0 * std::atan2(1.0, 1.0);  // src/GenInfo.f90:47

struct Basis {
    std::vector<double> psi, der, lap;  // nwt*4V, nwt*12V, nwt*4V
    std::vector<int> qn;                // nwt*4: isospin, parity, signature, timesimplex
    std::vector<double> occ, e, disp;
};

struct Moment {  // one electric multipole moment (src/Moments.f90:372-582)
    int l, m, im;
    std::vector<double> sh;  // SpherHarm on the stored mesh
    double value[2] = {0.0, 0.0};
};

// One constrained moment: the fields of type Moment that the alternating
// (ConstraintType 2), isoscalar (Isoswitch 1), non-total constraint uses
// (src/Moments.f90:146-200).
struct Constraint {
    int l, m, mom;              // mom: index in orc_ctx::moments
    int type = 2;               // ConstraintType; TurnOffConstraints sets 0
    int iteration = -1;         // last iteration with the constraint
    double constraint = 0.0;    // Constraint(1): the readjusted target
    double true_constraint = 0.0;
    double intensity = 0.0;     // Intensity(1); 0 = estimate on first Readjust
    double value[2] = {0.0, 0.0}, squared[2] = {0.0, 0.0};
    double old_value[7] = {0, 0, 0, 0, 0, 0, 0};   // sums of OldValue(:, 1..7)
    bool started = false;       // first CalculateAllMoments seen (src/Moments.f90:2277)
};

}  // namespace

struct orc_ctx {
    mg_params p;
    mg_force f;
    mg_skyrme_b B;
    int nx, ny, nz;
    long V;
    double dx, dv;
    bool folded;
    // Lagrange matrices per axis: [s][i*n+j], s=0 odd, s=1 even
    std::vector<double> D[3][2], L[3][2];
    Basis bas[2];
    std::vector<double> updates;
    // densities (src/Densities.f90:39-94) and the previous iteration's
    // (DensityHistory(1), src/Densities.f90:406-429)
    std::vector<double> rho, tau, nablaj, derrho, laprho;
    std::vector<double> hrho, htau, hnablaj, hderrho, hlaprho;
    std::vector<double> Uold;   // UpotOld (src/PotentialMixing.f90:115)
    // time-odd densities without time reversal (src/Densities.f90:39-94):
    // vecj, vecs, their curls [it][m][V], and their history for the mixing
    std::vector<double> vecj, vecs, rotj, rots, hvecj, hvecs, hrotj, hrots;
    // the tensor density J_{mu nu} [it][nu][mu][V] (src/Densities.f90:148)
    // when B14..B17 are not all zero, and its history
    bool tensor = false;
    std::vector<double> jmunu, hjmunu;
    // time-odd fields (src/MeanFields.f90:79-85): A, S [it][m][V], div A [it][V]
    std::vector<double> Apot, Spot, divA;
    // time-odd tensor terms without time reversal (B14..B21 not all zero):
    // the densities T, F, lap s, grad div s [it][m][V] (src/Densities.f90:
    // 55-64; each stays zero when no coefficient uses it, as the reference
    // leaves it unallocated) and their history; the fields C, D [it][m][V],
    // the derivatives of D [it][m][n][V] (d_n D_m) and div D [it][V]
    // (src/MeanFields.f90:84-87)
    bool todd = false;
    std::vector<double> vecT, vecF, lapS, gdivS, hvecT, hvecF, hlapS, hgdivS;
    std::vector<double> Cpot, Dpot, dD, divD;
    // potentials (src/MeanFields.f90:79-85)
    std::vector<double> U, Bp, nablaB, W, divW;
    // Coulomb (src/Coulomb.f90:20-105)
    int mx, my, mz;
    std::vector<double> cpot_complete, source, bc, rext, coulomb, coulex;
    std::vector<double> sh_ext;  // [moment][mx*my*mz]
    std::vector<Moment> moments;
    bool coulomb_init = false;

    // HFB pairing (src/HFB.f90, src/PairingInteraction.f90).  Blocks are the
    // (isospin, parity) blocks b = it*2 + (parity+1)/2; a block lists HFB
    // indices 0..2nwt-1 (stored spwfs first, then their time-reversed
    // partners, as PrepareHFBModule orders them).  All matrices are real
    // (time simplex conserved) and row-major [i*N + j].
    mg_pairing_params pp{};
    bool hfb_ready = false;
    std::vector<int> bidx[4];
    std::vector<double> rho_h[4], kappa_h[4], oldrho[4], oldkappa[4], delta[4];
    std::vector<double> Um[4], Vm[4], qe[4], cantr[4], occs[4];
    double fermi[2] = {-10.0, -10.0};
    // HFBFermiGradient (src/GradientHFB.f90): GradU, GradV of every block
    // (N x N, the N columns the CR8 choice keeps) and the positive-signature
    // column count SigBlocks
    bool ghfb_ready = false;
    std::vector<double> GU[4], GV[4];
    int gsig[4] = {0, 0, 0, 0};
    std::vector<double> pcut, dfac, pf_re, pf_im;
    double epair[2] = {0.0, 0.0};
    double pdisp[2] = {0.0, 0.0};
    bool fermi_hist[7] = {false, false, false, false, false, false, false};
    int last_evals = 0;

    // IterativeEstimation (src/ImaginaryTime.f90:28-211): maxspwf and the step
    // parameters in use
    Basis est;
    int est_iter = 0;
    bool step_set = false;
    double step_dt = 0.0, step_mom = 0.0;

    // Multipole constraints (src/Moments.f90:146-200, :2250-2531, :2929-3058)
    // with the Rutz cutoff (:2703-2871) and the alternate step
    // (src/ImaginaryTime.f90:306-437); the Evolve iteration counter of
    // TurnOffConstraints (src/Main.f90:256-304)
    std::vector<Constraint> cons;
    std::vector<double> cutoff, cons_energy;   // Cutoff(:,:,:,it), ConstraintEnergy
    bool alternate_check = false;              // AlternateCheck, src/Main.f90:247, :274
    int iteration = 0;
    // OldEnergy(7) and TotalEnergy (src/Energy.f90:34), for ConvergenceCheck
    double old_energy[7] = {0, 0, 0, 0, 0, 0, 0};
    double total_energy = 0.0;
};

// --------------------------------------------------------------------------
// Force coefficients: CalcEDFCoef, src/Force.f90:467-560
// --------------------------------------------------------------------------
extern "C" int orc_skyrme_coefficients(const mg_force* f, int trc, mg_skyrme_b* B) {
    if (!f || !B) return MG_ERR_ARG;
    std::memset(B, 0, sizeof(*B));
    const double t0 = f->t0, x0 = f->x0, t1 = f->t1, x1 = f->x1, t2 = f->t2, x2 = f->x2;
    B->B1 = t0 * (1.0 + 1 / 2.0 * x0) / 2.0;
    B->B2 = -t0 * (1 / 2.0 + x0) / 2.0;
    B->B3 = (t1 * (1 + 1 / 2.0 * x1) + t2 * (1 + 1 / 2.0 * x2)) / 4.0;
    B->B4 = -(t1 * (1 / 2.0 + x1) - t2 * (1 / 2.0 + x2)) / 4.0;
    B->B5 = -(3.0 * t1 * (1 + x1 / 2.0) - t2 * (1 + x2 / 2.0)) / 16.0;
    B->B6 = (3.0 * t1 * (x1 + 1 / 2.0) + t2 * (x2 + 1 / 2.0)) / 16.0;
    B->B7a = f->t3a * (1 + f->x3a / 2.0) / 12.0;
    B->B8a = -f->t3a * (f->x3a + 1 / 2.0) / 12.0;
    B->B7b = f->t3b * (1 + f->x3b / 2.0) / 12.0;
    B->B8b = -f->t3b * (f->x3b + 1 / 2.0) / 12.0;
    B->B9 = -f->wso / 2.0;
    B->B9q = -f->wsoq / 2.0;
    B->byt3a = f->yt3a;
    B->byt3b = f->yt3b;
    if (!trc) {
        B->B10 = t0 * x0 / 4.0;
        B->B11 = -t0 / 4.0;
        B->B12a = f->t3a * f->x3a / 24.0;
        B->B13a = -f->t3a / 24.0;
        B->B12b = f->t3b * f->x3b / 24.0;
        B->B13b = -f->t3b / 24.0;
    }
    if (f->j2terms) {
        // central J^2 terms of t1, t2 plus the tensor part
        const double C14 = -(1.0 / 8.0) * (f->t1 * f->x1 + f->t2 * f->x2);
        const double C15 = (1.0 / 8.0) * (f->t1 - f->t2);
        const double T14 = (1.0 / 4.0) * (f->te + f->to);
        const double T15 = -(1.0 / 4.0) * (f->te - f->to);
        B->B14 = C14 + T14;
        B->B15 = C15 + T15;
    }
    B->B16 = -(3.0 / 8.0) * (f->te + f->to);
    B->B17 = (3.0 / 8.0) * (f->te - f->to);
    if (f->j2terms && !trc) {
        // s . lap s terms: central part of t1, t2 plus the tensor part
        const double C18 = -(1.0 / 32.0) * (3 * f->t1 * f->x1 - f->t2 * f->x2);
        const double C19 = (1.0 / 32.0) * (3 * f->t1 + f->t2);
        const double T18 = (1.0 / 16.0) * (3 * f->te - f->to);
        const double T19 = -(1.0 / 16.0) * (3 * f->te + f->to);
        B->B18 = C18 + T18;
        B->B19 = C19 + T19;
    }
    if (!trc) {
        B->B20 = (3.0 / 16.0) * (3 * f->te - f->to);
        B->B21 = -(3.0 / 16.0) * (3 * f->te + f->to);
    }
    // parameterizations whose tensor couplings the relations above cannot
    // give, selected by the force's name
    if (f->coupling == MG_COUPLING_SLY4T || f->coupling == MG_COUPLING_SLY4TMIN) {
        B->B14 = 15.0;
        B->B15 = -120.0;
        B->B16 = 0.0;
        B->B17 = 0.0;
    } else if (f->coupling == MG_COUPLING_UNEDF2) {
        B->B14 = -54.4333635973721002 + 65.9030310445938028;
        B->B15 = -65.9030310445938028 * 2.0;
        B->B16 = 0.0;
        B->B17 = 0.0;
    }
    return MG_OK;
}

// --------------------------------------------------------------------------
// Lagrange coefficients: IniLag src/Derivatives.f90:899-973,
// folded matrices: reduceLag src/Derivatives.f90:975-1078,
// unfolded: DerLag_1D / SecondDerLag src/Derivatives.f90:1177-1312.
// --------------------------------------------------------------------------
static void ini_lag(int N, double dx, std::vector<double>& c1, std::vector<double>& c2,
                    double& diag) {
    c1.assign(N + 1, 0.0);
    c2.assign(N + 1, 0.0);
    double factor = kPi / N;
    double dxf = factor / dx;
    diag = -(kPi * kPi) / (3.0 * (dx * dx)) * (1.0 - 1.0 / double(N * N));
    for (int k = 1; k <= N - 1; ++k) {
        double s = std::sin(factor * k), c = std::cos(factor * k);
        double sg_k = (k % 2 == 0) ? 1.0 : -1.0;
        double sg_k1 = -sg_k;
        c1[k] = dxf * sg_k / s;
        c2[k] = sg_k1 * 2.0 * (dxf * dxf) * c / (s * s);
    }
}

extern "C" int orc_lagrange_matrices(int n, double dx, int folded, double* d1, double* d2) {
    if (n <= 0 || dx <= 0 || !d1 || !d2) return MG_ERR_ARG;
    std::vector<double> C, Lc;
    double diag;
    const long nn = (long)n * n;
    if (folded) {
        ini_lag(2 * n, dx, C, Lc, diag);
        for (int i = 1; i <= n; ++i) {
            for (int j = 1; j <= n; ++j) {
                double m1, m2, l1, l2;
                if (j < i) {
                    m2 = C[i - j] + C[i + j - 1];
                    m1 = C[i - j] - C[i + j - 1];
                    l2 = Lc[i - j] + Lc[i + j - 1];
                    l1 = Lc[i - j] - Lc[i + j - 1];
                } else if (j == i) {
                    l1 = diag - Lc[2 * i - 1];
                    l2 = diag + Lc[2 * i - 1];
                    m1 = -C[2 * i - 1];
                    m2 = +C[2 * i - 1];
                } else {
                    m2 = -C[j - i] + C[i + j - 1];
                    m1 = -C[j - i] - C[i + j - 1];
                    l2 = Lc[j - i] + Lc[i + j - 1];
                    l1 = Lc[j - i] - Lc[i + j - 1];
                }
                long o = (long)(i - 1) * n + (j - 1);
                d1[o] = m1; d1[nn + o] = m2;
                d2[o] = l1; d2[nn + o] = l2;
            }
        }
    } else {
        ini_lag(n, dx, C, Lc, diag);
        for (int i = 1; i <= n; ++i)
            for (int j = 1; j <= n; ++j) {
                long o = (long)(i - 1) * n + (j - 1);
                double m, l;
                if (i == j) { m = 0.0; l = diag; }
                else { m = (i > j ? 1.0 : -1.0) * C[std::abs(i - j)]; l = Lc[std::abs(i - j)]; }
                d1[o] = d1[nn + o] = m;
                d2[o] = d2[nn + o] = l;
            }
    }
    return MG_OK;
}

// Extension sign selection of Opt_LAG{X,Y,Z}_EV8 / Lapla_LAG_EV8
// (src/OptimizedDerivatives.f90:115-148, :306-338, :432-464, :551-615):
// returns the matrix slot, 1 = even (Fortran index 2), 0 = odd (index 1).
static int lag_slot(int dir, int P, int S, int TS, int comp) {
    int s = 0;
    if (dir == 0) s = (comp == 1 || comp == 4) ? S * TS : -S * TS;
    else if (dir == 1) s = (comp == 1 || comp == 3) ? TS : -TS;
    else s = (comp == 1 || comp == 2) ? S * P : -S * P;
    return s > 0 ? 1 : 0;
}

// out(i along dir) = sum_j M(i,j) in(j along dir); j ascending (matmul)
static void apply_axis(const orc_ctx* c, const double* M, int dir, const double* in,
                       double* out) {
    const int nx = c->nx, ny = c->ny, nz = c->nz;
    if (dir == 0) {
        for (int k = 0; k < nz; ++k)
            for (int j = 0; j < ny; ++j) {
                const double* line = in + (long)nx * (j + (long)ny * k);
                double* o = out + (long)nx * (j + (long)ny * k);
                for (int i = 0; i < nx; ++i) {
                    double s = 0.0;
                    for (int q = 0; q < nx; ++q) s += M[(long)i * nx + q] * line[q];
                    o[i] = s;
                }
            }
    } else if (dir == 1) {
        for (int k = 0; k < nz; ++k)
            for (int x = 0; x < nx; ++x)
                for (int i = 0; i < ny; ++i) {
                    double s = 0.0;
                    for (int q = 0; q < ny; ++q)
                        s += M[(long)i * ny + q] * in[x + (long)nx * (q + (long)ny * k)];
                    out[x + (long)nx * (i + (long)ny * k)] = s;
                }
    } else {
        for (int y = 0; y < ny; ++y)
            for (int x = 0; x < nx; ++x)
                for (int i = 0; i < nz; ++i) {
                    double s = 0.0;
                    for (int q = 0; q < nz; ++q)
                        s += M[(long)i * nz + q] * in[x + (long)nx * (y + (long)ny * q)];
                    out[x + (long)nx * (y + (long)ny * i)] = s;
                }
    }
}

// DeriveX/Y/Z (dir 0..2) or Laplacian (dir 3) of one real grid.
static void derive_grid(const orc_ctx* c, const double* g, int dir, int P, int S, int TS,
                        int comp, double* out) {
    if (dir < 3) {
        apply_axis(c, c->D[dir][lag_slot(dir, P, S, TS, comp)].data(), dir, g, out);
        return;
    }
    std::vector<double> a(c->V), b(c->V), d(c->V);
    apply_axis(c, c->L[0][lag_slot(0, P, S, TS, comp)].data(), 0, g, a.data());
    apply_axis(c, c->L[1][lag_slot(1, P, S, TS, comp)].data(), 1, g, b.data());
    apply_axis(c, c->L[2][lag_slot(2, P, S, TS, comp)].data(), 2, g, d.data());
    for (long v = 0; v < c->V; ++v) out[v] = a[v] + b[v] + d[v];
}

extern "C" int orc_derive_grid(orc_ctx* c, const double* g, int dir, int P, int S, int TS,
                               int comp, double* out) {
    if (!c || !g || !out || dir < 0 || dir > 3) return MG_ERR_ARG;
    derive_grid(c, g, dir, P, S, TS, comp, out);
    return MG_OK;
}

// --------------------------------------------------------------------------
// Context
// --------------------------------------------------------------------------
extern "C" orc_ctx* orc_create(const mg_params* p, const mg_force* f) {
    if (!p || !f || p->nx <= 0 || p->ny <= 0 || p->nz <= 0 || p->nwt <= 0) return nullptr;
    bool ev8 = p->pc && p->sc && p->tsc;
    bool full = !p->pc && !p->sc && !p->tsc;
    if (!ev8 && !full) return nullptr;
    orc_ctx* c = new orc_ctx();
    c->p = *p;
    c->f = *f;
    orc_skyrme_coefficients(f, p->trc, &c->B);
    c->nx = p->nx; c->ny = p->ny; c->nz = p->nz;
    c->V = (long)p->nx * p->ny * p->nz;
    c->dx = p->dx;
    // dv = dx^3 * 2^(number of conserved spatial symmetries), src/GenInfo.f90:296
    int nsym = (p->pc ? 1 : 0) + (p->sc ? 1 : 0) + (p->tsc ? 1 : 0);
    c->dv = p->dx * p->dx * p->dx * std::pow(2.0, nsym);
    c->folded = ev8;
    int ns[3] = {p->nx, p->ny, p->nz};
    for (int d = 0; d < 3; ++d) {
        long nn = (long)ns[d] * ns[d];
        std::vector<double> d1(2 * nn), d2(2 * nn);
        orc_lagrange_matrices(ns[d], p->dx, ev8 ? 1 : 0, d1.data(), d2.data());
        for (int s = 0; s < 2; ++s) {
            c->D[d][s].assign(d1.begin() + s * nn, d1.begin() + (s + 1) * nn);
            c->L[d][s].assign(d2.begin() + s * nn, d2.begin() + (s + 1) * nn);
        }
    }
    for (int b = 0; b < 2; ++b) {
        Basis& B = c->bas[b];
        B.psi.assign(p->nwt * 4 * c->V, 0.0);
        B.der.assign(p->nwt * 12 * c->V, 0.0);
        B.lap.assign(p->nwt * 4 * c->V, 0.0);
        B.qn.assign(p->nwt * 4, 1);
        B.occ.assign(p->nwt, 0.0);
        B.e.assign(p->nwt, 0.0);
        B.disp.assign(p->nwt, 0.0);
    }
    c->updates.assign(p->nwt * 4 * c->V, 0.0);
    long V = c->V;
    c->rho.assign(2 * V, 0); c->tau.assign(2 * V, 0); c->nablaj.assign(2 * V, 0);
    c->derrho.assign(6 * V, 0); c->laprho.assign(2 * V, 0);
    c->U.assign(2 * V, 0); c->Bp.assign(2 * V, 0); c->nablaB.assign(6 * V, 0);
    c->W.assign(18 * V, 0); c->divW.assign(6 * V, 0);
    c->tensor = c->B.B14 != 0.0 || c->B.B15 != 0.0 || c->B.B16 != 0.0 || c->B.B17 != 0.0;
    if (c->tensor) c->jmunu.assign(18 * V, 0.0);
    c->coulomb.assign(V, 0); c->coulex.assign(V, 0);
    if (!p->trc)
        for (auto* x : {&c->vecj, &c->vecs, &c->rotj, &c->rots, &c->Apot, &c->Spot})
            x->assign(6 * V, 0.0);
    if (!p->trc) c->divA.assign(2 * V, 0.0);
    const mg_skyrme_b& B = c->B;
    c->todd = !p->trc && (c->tensor || B.B18 != 0.0 || B.B19 != 0.0 || B.B20 != 0.0 ||
                          B.B21 != 0.0);
    if (c->todd) {
        for (auto* x : {&c->vecT, &c->vecF, &c->lapS, &c->gdivS, &c->Cpot, &c->Dpot})
            x->assign(6 * V, 0.0);
        c->dD.assign(18 * V, 0.0);
        c->divD.assign(2 * V, 0.0);
    }
    return c;
}

static bool cranking(const orc_ctx* c) {
    return c->p.omega[0] != 0.0 || c->p.omega[1] != 0.0 || c->p.omega[2] != 0.0;
}

extern "C" void orc_destroy(orc_ctx* c) { delete c; }

extern "C" int orc_set_spinors(orc_ctx* c, int b, const double* psi, const int* qn) {
    if (!c || b < 0 || b > 1) return MG_ERR_ARG;
    Basis& B = c->bas[b];
    if (psi) std::memcpy(B.psi.data(), psi, B.psi.size() * sizeof(double));
    if (qn) std::memcpy(B.qn.data(), qn, B.qn.size() * sizeof(int));
    return MG_OK;
}
extern "C" int orc_get_spinors(orc_ctx* c, int b, double* psi) {
    if (!c || b < 0 || b > 1 || !psi) return MG_ERR_ARG;
    std::memcpy(psi, c->bas[b].psi.data(), c->bas[b].psi.size() * sizeof(double));
    return MG_OK;
}
extern "C" int orc_get_qn(orc_ctx* c, int b, int* qn) {
    if (!c || b < 0 || b > 1 || !qn) return MG_ERR_ARG;
    std::memcpy(qn, c->bas[b].qn.data(), c->bas[b].qn.size() * sizeof(int));
    return MG_OK;
}
extern "C" int orc_get_derivatives(orc_ctx* c, int b, double* der, double* lap) {
    if (!c || b < 0 || b > 1) return MG_ERR_ARG;
    if (der) std::memcpy(der, c->bas[b].der.data(), c->bas[b].der.size() * sizeof(double));
    if (lap) std::memcpy(lap, c->bas[b].lap.data(), c->bas[b].lap.size() * sizeof(double));
    return MG_OK;
}
extern "C" int orc_set_occupations(orc_ctx* c, int b, const double* occ) {
    if (!c || b < 0 || b > 1 || !occ) return MG_ERR_ARG;
    std::copy(occ, occ + c->p.nwt, c->bas[b].occ.begin());
    return MG_OK;
}
extern "C" int orc_get_occupations(orc_ctx* c, int b, double* occ) {
    if (!c || b < 0 || b > 1 || !occ) return MG_ERR_ARG;
    std::copy(c->bas[b].occ.begin(), c->bas[b].occ.end(), occ);
    return MG_OK;
}
extern "C" int orc_set_energies(orc_ctx* c, int b, const double* e) {
    if (!c || b < 0 || b > 1 || !e) return MG_ERR_ARG;
    std::copy(e, e + c->p.nwt, c->bas[b].e.begin());
    return MG_OK;
}
extern "C" int orc_get_energies(orc_ctx* c, int b, double* e, double* disp) {
    if (!c || b < 0 || b > 1) return MG_ERR_ARG;
    if (e) std::copy(c->bas[b].e.begin(), c->bas[b].e.end(), e);
    if (disp) std::copy(c->bas[b].disp.begin(), c->bas[b].disp.end(), disp);
    return MG_OK;
}

// --------------------------------------------------------------------------
// CompDer / DeriveSpinor / LapSpinor, src/Spwf.f90:778-792,
// src/Spinor.f90:516-552, :661-687; DeriveAll src/SpwfStorage.f90:586-604
// --------------------------------------------------------------------------
extern "C" int orc_derive_basis(orc_ctx* c, int b) {
    if (!c || b < 0 || b > 1) return MG_ERR_ARG;
    Basis& B = c->bas[b];
    const long V = c->V;
#pragma omp parallel for schedule(dynamic, 1)
    for (int i = 0; i < c->p.nwt; ++i) {
        int P = B.qn[4 * i + 1], S = B.qn[4 * i + 2], TS = B.qn[4 * i + 3];
        const double* psi = &B.psi[(long)i * 4 * V];
        for (int l = 0; l < 4; ++l) {
            for (int d = 0; d < 3; ++d)
                derive_grid(c, psi + l * V, d, P, S, TS, l + 1,
                            &B.der[((long)i * 12 + d * 4 + l) * V]);
            derive_grid(c, psi + l * V, 3, P, S, TS, l + 1, &B.lap[((long)i * 4 + l) * V]);
        }
    }
    return MG_OK;
}

extern "C" int orc_derive_all(orc_ctx* c) {
    if (!c) return MG_ERR_ARG;
    orc_derive_basis(c, MG_HF_BASIS);
    if (c->p.pairing == MG_PAIRING_HFB) orc_derive_basis(c, MG_CAN_BASIS);
    return MG_OK;
}

// --------------------------------------------------------------------------
// Spinor helpers (src/Spinor.f90)
// --------------------------------------------------------------------------
// Pauli(Psi, dir) at one point, src/Spinor.f90:113-157
static inline void pauli(const double* p, int dir, double* o) {
    if (dir == 1) { o[0] = p[2]; o[1] = p[3]; o[2] = p[0]; o[3] = p[1]; }
    else if (dir == 2) { o[0] = p[3]; o[1] = -p[2]; o[2] = -p[1]; o[3] = p[0]; }
    else { o[0] = p[0]; o[1] = p[1]; o[2] = -p[2]; o[3] = -p[3]; }
}
// InproductSpinorReal, src/Spinor.f90:715-731
static double inprod_real(const orc_ctx* c, const double* a, const double* b) {
    double s = 0.0;
    for (long i = 0; i < 4 * c->V; ++i) s += a[i] * b[i];
    return s * c->dv;
}

static double reduced_mass(const orc_ctx* c, int it) {
    // ActionOfBNew, src/MeanFields.f90:829-833
    if (c->f.com1body == 2)
        return 1.0 - c->f.nucleonmass[it] /
                         (c->p.neutrons * c->f.nucleonmass[0] + c->p.protons * c->f.nucleonmass[1]);
    return 1.0;
}

// ActionOfC and ActionOfD (src/MeanFields.f90:1149-1255) of spwf i into xc,
// xd (4V each):
//   C psi = sum_n d_n [-sum_m C_m sigma_m d_n psi]
//   D psi = -1/2 [div D sigma.grad psi + sum_mn d_n D_m sigma_n d_m psi
//                 + 2 sum_mn D_m sigma_n d_m d_n psi]
// The outer derivatives take the symmetries of d_n psi: (-P, -S, TS) for
// x, (-P, -S, -TS) for y, (-P, S, TS) for z; d_m d_n psi is d_m of the
// stored d_n psi.
static void tensor_odd_action(const orc_ctx* c, const Basis& Bs, int i, double* xc,
                              double* xd) {
    const long V = c->V;
    const mg_skyrme_b& B = c->B;
    const int it = (Bs.qn[4 * i] + 3) / 2 - 1;
    const int P = Bs.qn[4 * i + 1], S = Bs.qn[4 * i + 2], TS = Bs.qn[4 * i + 3];
    const double* der = &Bs.der[(long)i * 12 * V];
    const int sp[3][2] = {{-S, TS}, {-S, -TS}, {S, TS}};
    std::fill(xc, xc + 4 * V, 0.0);
    std::fill(xd, xd + 4 * V, 0.0);
    if (B.B14 != 0.0 || B.B15 != 0.0) {
        std::vector<double> tmp(4 * V), dt(V);
        for (int n = 0; n < 3; ++n) {
            for (long v = 0; v < V; ++v) {
                double dn[4], t[4] = {0.0, 0.0, 0.0, 0.0};
                for (int l = 0; l < 4; ++l) dn[l] = der[(n * 4 + l) * V + v];
                for (int m = 0; m < 3; ++m) {
                    double sg[4];
                    pauli(dn, m + 1, sg);
                    const double cm = c->Cpot[(it * 3 + m) * V + v];
                    for (int l = 0; l < 4; ++l) t[l] = t[l] - cm * sg[l];
                }
                for (int l = 0; l < 4; ++l) tmp[l * V + v] = t[l];
            }
            for (int l = 0; l < 4; ++l) {
                derive_grid(c, &tmp[l * V], n, -P, sp[n][0], sp[n][1], l + 1, dt.data());
                for (long v = 0; v < V; ++v) xc[l * V + v] = xc[l * V + v] + dt[v];
            }
        }
    }
    if (B.B16 != 0.0 || B.B17 != 0.0) {
        std::vector<double> dd(36 * V);   // [a][n][l][V] = d_a (d_n psi)_l
        for (int n = 0; n < 3; ++n)
            for (int l = 0; l < 4; ++l)
                for (int a = 0; a < 3; ++a)
                    derive_grid(c, &der[(n * 4 + l) * V], a, -P, sp[n][0], sp[n][1], l + 1,
                                &dd[((a * 3 + n) * 4 + l) * V]);
        for (long v = 0; v < V; ++v) {
            double d[3][4];
            for (int m = 0; m < 3; ++m)
                for (int l = 0; l < 4; ++l) d[m][l] = der[(m * 4 + l) * V + v];
            double t1[4] = {0, 0, 0, 0}, t2[4] = {0, 0, 0, 0}, t3[4] = {0, 0, 0, 0};
            for (int m = 0; m < 3; ++m) {
                double sg[4];
                pauli(d[m], m + 1, sg);
                for (int l = 0; l < 4; ++l) t1[l] = t1[l] + sg[l];
            }
            const double dvD = c->divD[it * V + v];
            for (int l = 0; l < 4; ++l) t1[l] = dvD * t1[l];
            for (int m = 0; m < 3; ++m)
                for (int n = 0; n < 3; ++n) {
                    double sg[4];
                    pauli(d[m], n + 1, sg);
                    const double g = c->dD[((it * 3 + m) * 3 + n) * V + v];
                    for (int l = 0; l < 4; ++l) t2[l] = t2[l] + g * sg[l];
                }
            for (int m = 0; m < 3; ++m)
                for (int n = 0; n < 3; ++n) {
                    double q[4], sg[4];
                    for (int l = 0; l < 4; ++l) q[l] = dd[((m * 3 + n) * 4 + l) * V + v];
                    pauli(q, n + 1, sg);
                    const double Dm = c->Dpot[(it * 3 + m) * V + v];
                    for (int l = 0; l < 4; ++l) t3[l] = t3[l] + Dm * sg[l];
                }
            for (int l = 0; l < 4; ++l) xd[l * V + v] = -0.5 * (t1[l] + t2[l] + 2.0 * t3[l]);
        }
    }
}

// hPsi for one spwf: B (ActionOfBNew) + U + W, src/ImaginaryTime.f90:213-304,
// src/MeanFields.f90:792-851, :1029-1065; without time reversal S and A, and
// with the time-odd tensor terms C and D.
static void hpsi_one(const orc_ctx* c, const Basis& B, int i, double* out) {
    const long V = c->V;
    std::vector<double> xc, xd;
    if (c->todd) {
        xc.resize(4 * V);
        xd.resize(4 * V);
        tensor_odd_action(c, B, i, xc.data(), xd.data());
    }
    const int it = (B.qn[4 * i] + 3) / 2 - 1;
    const double* psi = &B.psi[(long)i * 4 * V];
    const double* der = &B.der[(long)i * 12 * V];
    const double* lap = &B.lap[(long)i * 4 * V];
    const double kin = c->f.hbm / 2.0 * reduced_mass(c, it);
    const double* Bq = &c->Bp[it * V];
    const double* Uq = &c->U[it * V];
    for (long v = 0; v < V; ++v) {
        double p[4], d[3][4], L[4];
        for (int l = 0; l < 4; ++l) {
            p[l] = psi[l * V + v];
            L[l] = lap[l * V + v];
            for (int m = 0; m < 3; ++m) d[m][l] = der[(m * 4 + l) * V + v];
        }
        double b[4], u[4], w[4] = {0, 0, 0, 0};
        for (int l = 0; l < 4; ++l) {
            double t = -(Bq[v] * L[l]);
            t = t - kin * L[l];
            double sd = c->nablaB[(it * 3 + 0) * V + v] * d[0][l] +
                        c->nablaB[(it * 3 + 1) * V + v] * d[1][l];
            sd = sd + c->nablaB[(it * 3 + 2) * V + v] * d[2][l];
            b[l] = t - sd;
            u[l] = Uq[v] * p[l];
        }
        // ActionOfW: sum_mu sum_nu W(mu,nu) sigma_nu d_mu psi + 1/2 sum_nu divW(nu) sigma_nu psi
        for (int mu = 0; mu < 3; ++mu)
            for (int nu = 0; nu < 3; ++nu) {
                double s[4];
                pauli(d[mu], nu + 1, s);
                double wv = c->W[((it * 3 + nu) * 3 + mu) * V + v];
                for (int l = 0; l < 4; ++l) w[l] = w[l] + wv * s[l];
            }
        for (int nu = 0; nu < 3; ++nu) {
            double s[4];
            pauli(p, nu + 1, s);
            double hv = 0.5 * c->divW[(it * 3 + nu) * V + v];
            for (int l = 0; l < 4; ++l) w[l] = w[l] + hv * s[l];
        }
        // (-1) * MultiplyI(w): (w1,w2,w3,w4) -> (w2,-w1,w4,-w3)
        double wf[4] = {w[1], -w[0], w[3], -w[2]};
        double h[4];
        for (int l = 0; l < 4; ++l) h[l] = (b[l] + u[l]) + wf[l];
        if (!c->p.trc) {
            // ActionOfS: sum_m S_m sigma_m psi; ActionOfA: -i (sum_m A_m d_m psi
            // + 1/2 div A psi) (src/MeanFields.f90:1107-1147)
            double sa[4] = {0, 0, 0, 0}, aa[4] = {0, 0, 0, 0};
            for (int m = 0; m < 3; ++m) {
                double sg[4];
                pauli(p, m + 1, sg);
                const double sm = c->Spot[(it * 3 + m) * V + v], am = c->Apot[(it * 3 + m) * V + v];
                for (int l = 0; l < 4; ++l) {
                    sa[l] = sa[l] + sm * sg[l];
                    aa[l] = aa[l] + am * d[m][l];
                }
            }
            const double hd = 0.5 * c->divA[it * V + v];
            for (int l = 0; l < 4; ++l) aa[l] = aa[l] + hd * p[l];
            const double af[4] = {aa[1], -aa[0], aa[3], -aa[2]};
            for (int l = 0; l < 4; ++l) h[l] = (h[l] + sa[l]) + af[l];
        }
        if (c->todd)
            for (int l = 0; l < 4; ++l) h[l] = (h[l] + xc[l * V + v]) + xd[l * V + v];
        for (int l = 0; l < 4; ++l) out[l * V + v] = h[l];
    }
}

extern "C" int orc_hpsi(orc_ctx* c, int b, double* hpsi, double* e, double* disp) {
    if (!c || b < 0 || b > 1) return MG_ERR_ARG;
    const Basis& B = c->bas[b];
    const long V4 = 4 * c->V;
#pragma omp parallel for schedule(dynamic, 1)
    for (int i = 0; i < c->p.nwt; ++i) {
        std::vector<double> h(V4);
        hpsi_one(c, B, i, h.data());
        double en = inprod_real(c, &B.psi[i * V4], h.data());
        double hh = inprod_real(c, h.data(), h.data());
        if (hpsi) std::memcpy(hpsi + i * V4, h.data(), V4 * sizeof(double));
        if (e) e[i] = en;
        if (disp) disp[i] = hh - en * en;
    }
    return MG_OK;
}

// --------------------------------------------------------------------------
// GramSchmidt, src/SpwfStorage.f90:372-480 (TSC, SC conserved branch);
// OrderSpwfsISO src/SpwfStorage.f90:795-848 (stable ascending insertion sort)
// --------------------------------------------------------------------------
static std::vector<int> order_iso(const Basis& B, int nwt, int iso) {
    std::vector<int> idx;
    for (int i = 0; i < nwt; ++i)
        if (B.qn[4 * i] == iso) idx.push_back(i);
    std::stable_sort(idx.begin(), idx.end(), [&](int a, int b2) { return B.e[a] < B.e[b2]; });
    return idx;
}

extern "C" int orc_gram_schmidt(orc_ctx* c) {
    if (!c) return MG_ERR_ARG;
    Basis& B = c->bas[MG_HF_BASIS];
    const long V4 = 4 * c->V;
    for (int it = 1; it <= 2; ++it) {
        std::vector<int> idx = order_iso(B, c->p.nwt, it * 2 - 3);
        for (size_t k = 0; k < idx.size(); ++k) {
            int nw = idx[k];
            double* pn = &B.psi[nw * V4];
            double norm = inprod_real(c, pn, pn);
            double sc = 1.0 / std::sqrt(norm);
            for (long v = 0; v < V4; ++v) pn[v] = sc * pn[v];
#pragma omp parallel for schedule(dynamic, 1)
            for (size_t l = k + 1; l < idx.size(); ++l) {
                int mw = idx[l];
                if (B.qn[4 * mw] != B.qn[4 * nw] || B.qn[4 * mw + 1] != B.qn[4 * nw + 1] ||
                    B.qn[4 * mw + 2] != B.qn[4 * nw + 2])
                    continue;
                double* pm = &B.psi[mw * V4];
                double me = inprod_real(c, pm, pn);  // InProduct(HFBasis(mw), HFBasis(nw))
                for (long v = 0; v < V4; ++v) pm[v] = pm[v] - me * pn[v];
            }
        }
    }
    return MG_OK;
}

// --------------------------------------------------------------------------
// IterativeEstimation, src/ImaginaryTime.f90:28-211.  The reference fills
// the start with an unseeded random_number; this restatement (like the GPU
// path) uses a fixed-seed splitmix64 stream so that runs repeat.
// --------------------------------------------------------------------------
static double est_start_value(unsigned long long k) {
    unsigned long long z = 0x2545F4914F6CDD1Dull + (k + 1) * 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}

static void est_derive(orc_ctx* c) {
    Basis& E = c->est;
    const long V = c->V;
    const int P = E.qn[1], S = E.qn[2], TS = E.qn[3];
    for (int l = 0; l < 4; ++l) {
        for (int d = 0; d < 3; ++d)
            derive_grid(c, &E.psi[l * V], d, P, S, TS, l + 1, &E.der[(d * 4 + l) * V]);
        derive_grid(c, &E.psi[l * V], 3, P, S, TS, l + 1, &E.lap[l * V]);
    }
}

static int iterative_estimation(orc_ctx* c) {
    Basis& B = c->bas[MG_HF_BASIS];
    Basis& E = c->est;
    const long V = c->V, V4 = 4 * V;
    const int nwt = c->p.nwt;
    ++c->est_iter;
    if (c->est_iter == 1) {
        // maxspwf = HFBasis(nwt) (HFBasis(nwn) without protons), random start
        int iw = nwt - 1;
        if (c->p.protons < 1e-9)
            for (int i = 0; i < nwt; ++i)
                if (B.qn[4 * i] == -1) iw = i;
        E.qn.assign(B.qn.begin() + 4 * iw, B.qn.begin() + 4 * iw + 4);
        E.psi.assign(V4, 0.0);
        E.der.assign(12 * V, 0.0);
        E.lap.assign(V4, 0.0);
        double norm = 0.0;
        for (long k = 0; k < V4; ++k) {
            E.psi[k] = est_start_value((unsigned long long)k);
            norm += E.psi[k] * E.psi[k];
        }
        const double sc = 1.0 / std::sqrt(norm * c->dv);
        for (long k = 0; k < V4; ++k) E.psi[k] *= sc;
        est_derive(c);
    }
    std::vector<double> up(V4, 0.0), h(V4);
    const double fac = c->step_dt / c->f.hbar, mom = c->step_mom;
    double maxE = 0.0, prev = NAN, con = NAN;
    for (int it = 0; it < 500; ++it) {
        hpsi_one(c, E, 0, h.data());
        maxE = inprod_real(c, E.psi.data(), h.data());
        con = prev - maxE;
        prev = maxE;
        double norm = 0.0;
        for (long k = 0; k < V4; ++k) {
            up[k] = fac * (h[k] - maxE * E.psi[k]) + mom * up[k];
            E.psi[k] = E.psi[k] + up[k];
            norm += E.psi[k] * E.psi[k];
        }
        const double sc = 1.0 / std::sqrt(norm * c->dv);
        for (long k = 0; k < V4; ++k) E.psi[k] *= sc;
        est_derive(c);
        if (std::fabs(con) < 1e-2) break;
    }
    if (std::isnan(maxE)) return MG_ERR_NAN;
    double relE = 10000.0;
    if (c->p.pairing == MG_PAIRING_HFB && c->hfb_ready) {
        // the columns the HFB solution keeps (HFBcolumns) carry the upper
        // half of each block's ascending spectrum
        for (int b = 0; b < 4; ++b) {
            const size_t N = c->qe[b].size() / 2;
            for (size_t k = N / 2; k < N; ++k)
                if (c->qe[b][k] > 0.0) relE = std::min(relE, std::fabs(c->qe[b][k]));
        }
    } else {
        for (int i = 0; i < nwt; ++i) {
            if (std::fabs(B.occ[i]) < 0.5) continue;
            for (int k = 0; k < nwt; ++k) {
                if (std::fabs(B.occ[k]) > 0.5 || B.qn[4 * k] != B.qn[4 * i]) continue;
                const double d = B.e[k] - B.e[i];
                if (d > 0.0) relE = std::min(relE, d);
            }
        }
        if (relE < 0.1) relE = 0.1;
    }
    double minh = 10000.0;
    for (int i = 0; i < nwt; ++i) minh = std::min(minh, B.e[i]);
    maxE -= minh;
    const double kappa = relE / maxE;
    c->step_mom = std::pow((std::sqrt(kappa) - 1.0) / (std::sqrt(kappa) + 1.0), 2.0);
    c->step_dt = 4.0 / (maxE + relE + 2.0 * std::sqrt(maxE * relE)) * c->f.hbar * 0.90;
    return MG_OK;
}

extern "C" int orc_get_step_parameters(orc_ctx* c, double* dt, double* momentum) {
    if (!c || !dt || !momentum) return MG_ERR_ARG;
    *dt = c->step_dt;
    *momentum = c->step_mom;
    return MG_OK;
}

// --------------------------------------------------------------------------
// GradDesc, src/ImaginaryTime.f90:439-500 (no InverseKineticDamping), with
// IterativeEstimation first when ParameterEstimation = 1 (:465)
// --------------------------------------------------------------------------
extern "C" int orc_grad_desc(orc_ctx* c, double dt, double momentum) {
    if (!c) return MG_ERR_ARG;
    Basis& B = c->bas[MG_HF_BASIS];
    const long V4 = 4 * c->V;
    if (!c->step_set || c->p.parameter_estimation != 1) {
        c->step_dt = dt;
        c->step_mom = momentum;
        c->step_set = true;
    }
    if (c->p.parameter_estimation == 1) {
        const int st = iterative_estimation(c);
        if (st != MG_OK) return st;
    }
    dt = c->step_dt;
    momentum = c->step_mom;
    const double fac = dt / c->f.hbar;
#pragma omp parallel for schedule(dynamic, 1)
    for (int i = 0; i < c->p.nwt; ++i) {
        std::vector<double> h(V4);
        double* cur = &B.psi[i * V4];
        hpsi_one(c, B, i, h.data());
        double en = inprod_real(c, cur, h.data());
        double ds = inprod_real(c, h.data(), h.data()) - en * en;
        double* up = &c->updates[i * V4];
        for (long v = 0; v < V4; ++v) {
            double a = -fac * h[v] + momentum * up[v];
            up[v] = cur[v];
            cur[v] = cur[v] + a;
        }
        B.e[i] = en;
        B.disp[i] = ds;
    }
    orc_gram_schmidt(c);
    for (int i = 0; i < c->p.nwt; ++i)
        for (long v = 0; v < V4; ++v) c->updates[i * V4 + v] = B.psi[i * V4 + v] - c->updates[i * V4 + v];
    return MG_OK;
}

// --------------------------------------------------------------------------
// NaiveFill, src/HartreeFock.f90:177-260 (no blocking)
// --------------------------------------------------------------------------
extern "C" int orc_hf_fill(orc_ctx* c) {
    if (!c) return MG_ERR_ARG;
    Basis& B = c->bas[MG_HF_BASIS];
    const int nwt = c->p.nwt;
    std::fill(B.occ.begin(), B.occ.end(), 0.0);
    int pub = c->p.trc ? (int)std::floor(c->p.protons / 2) : (int)std::floor(c->p.protons);
    int nub = c->p.trc ? (int)std::floor(c->p.neutrons / 2) : (int)std::floor(c->p.neutrons);
    std::vector<int> order(nwt);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b2) { return B.e[a] < B.e[b2]; });
    int n = 0, pp = 0;
    for (int i = 0; i < nwt && pp < pub; ++i) {
        int j = order[i];
        if (B.occ[j] == 0.0 && B.qn[4 * j] == 1) { B.occ[j] = 1.0; ++pp; }
    }
    for (int i = 0; i < nwt && n < nub; ++i) {
        int j = order[i];
        if (B.occ[j] == 0.0 && B.qn[4 * j] == -1) { B.occ[j] = 1.0; ++n; }
    }
    if (c->p.trc)
        for (int i = 0; i < nwt; ++i) B.occ[i] = 2.0 * B.occ[i];
    return MG_OK;
}

// --------------------------------------------------------------------------
// ComputeDensity, src/Densities.f90:431-550 (TRC, no tensor / N2LO):
// rho (GetDensity src/Spwf.f90:536-546), tau (GetTau :1897-1909),
// NablaJ (GetNablaJ :2206-2243), then DerRho and LapRho.
// --------------------------------------------------------------------------
static inline double imag_mult(const double* a, const double* b) {
    // ImagMultiplySpinor, src/Spinor.f90:264-281
    return a[0] * b[1] - a[1] * b[0] + a[2] * b[3] - a[3] * b[2];
}

// Curls of vecj and vecs with the symmetry arguments of Table V of
// Hellemans et al. (src/Densities.f90:1004-1106): d_y j_x, d_z j_x with
// (-P, -S, TS, 2); d_x j_y, d_z j_y with (-P, -S, TS, 1); d_x j_z, d_y j_z
// with (-P, S, TS, 2); d s_x with (P, -S, TS, 1), d s_y with (P, -S, TS, 2),
// d s_z with (P, S, TS, 1).
static void time_odd_curls(orc_ctx* c) {
    const long V = c->V;
    const int P = c->p.pc, S = c->p.sc, TS = c->p.tsc;
    std::vector<double> d[3][3];   // d[axis][component]
    for (int it = 0; it < 2; ++it) {
        for (int pass = 0; pass < 2; ++pass) {
            const std::vector<double>& f = pass == 0 ? c->vecj : c->vecs;
            std::vector<double>& rot = pass == 0 ? c->rotj : c->rots;
            for (int m = 0; m < 3; ++m)
                for (int a = 0; a < 3; ++a) {
                    d[a][m].assign(V, 0.0);
                    if (a == m) continue;
                    int pp, ss, comp;
                    if (pass == 0) {
                        pp = -P;
                        ss = m == 2 ? S : -S;
                        comp = m == 1 ? 1 : 2;
                    } else {
                        pp = P;
                        ss = m == 2 ? S : -S;
                        comp = m == 1 ? 2 : 1;
                    }
                    derive_grid(c, &f[(it * 3 + m) * V], a, pp, ss, TS, comp, d[a][m].data());
                }
            for (long v = 0; v < V; ++v) {
                rot[(it * 3 + 0) * V + v] = d[1][2][v] - d[2][1][v];
                rot[(it * 3 + 1) * V + v] = d[2][0][v] - d[0][2][v];
                rot[(it * 3 + 2) * V + v] = d[0][1][v] - d[1][0][v];
            }
        }
    }
}

extern "C" int orc_update_densities(orc_ctx* c) {
    if (!c) return MG_ERR_ARG;
    const long V = c->V;
    // UpdateDensities(0): DensityHistory(1) = Density before recomputing
    c->hrho = c->rho; c->htau = c->tau; c->hnablaj = c->nablaj;
    c->hderrho = c->derrho; c->hlaprho = c->laprho;
    c->hvecj = c->vecj; c->hvecs = c->vecs; c->hrotj = c->rotj; c->hrots = c->rots;
    c->hjmunu = c->jmunu;
    c->hvecT = c->vecT; c->hvecF = c->vecF; c->hlapS = c->lapS; c->hgdivS = c->gdivS;
    if (c->tensor) std::fill(c->jmunu.begin(), c->jmunu.end(), 0.0);
    const bool odd = !c->p.trc;
    if (odd) {
        std::fill(c->vecj.begin(), c->vecj.end(), 0.0);
        std::fill(c->vecs.begin(), c->vecs.end(), 0.0);
    }
    // T with B14 or B15, F with B16 or B17 (src/Densities.f90:502-510)
    const mg_skyrme_b& Bc = c->B;
    const bool wantT = c->todd && (Bc.B14 != 0.0 || Bc.B15 != 0.0);
    const bool wantF = c->todd && (Bc.B16 != 0.0 || Bc.B17 != 0.0);
    if (c->todd) {
        std::fill(c->vecT.begin(), c->vecT.end(), 0.0);
        std::fill(c->vecF.begin(), c->vecF.end(), 0.0);
    }
    const Basis& B = c->bas[c->p.pairing == MG_PAIRING_HFB ? MG_CAN_BASIS : MG_HF_BASIS];
    std::fill(c->rho.begin(), c->rho.end(), 0.0);
    std::fill(c->tau.begin(), c->tau.end(), 0.0);
    std::fill(c->nablaj.begin(), c->nablaj.end(), 0.0);
    // (i,j,k, LeviCivita) in the reference's order
    static const int trip[6][4] = {{1, 2, 3, 1}, {1, 3, 2, -1}, {3, 2, 1, -1},
                                   {3, 1, 2, 1}, {2, 1, 3, -1}, {2, 3, 1, 1}};
    for (int i = 0; i < c->p.nwt; ++i) {
        double occ = B.occ[i];
        if (occ == 0.0) continue;
        int it = (B.qn[4 * i] + 3) / 2 - 1;
        const double* psi = &B.psi[(long)i * 4 * V];
        const double* der = &B.der[(long)i * 12 * V];
        for (long v = 0; v < V; ++v) {
            double p[4], d[3][4];
            for (int l = 0; l < 4; ++l) {
                p[l] = psi[l * V + v];
                for (int m = 0; m < 3; ++m) d[m][l] = der[(m * 4 + l) * V + v];
            }
            double den = p[0] * p[0] + p[1] * p[1] + p[2] * p[2] + p[3] * p[3];
            c->rho[it * V + v] = c->rho[it * V + v] + occ * den;
            double t = 0.0;
            for (int m = 0; m < 3; ++m)
                t = t + (d[m][0] * d[m][0] + d[m][1] * d[m][1] + d[m][2] * d[m][2] + d[m][3] * d[m][3]);
            c->tau[it * V + v] = c->tau[it * V + v] + occ * t;
            double nj = 0.0;
            for (int q = 0; q < 6; ++q) {
                double s[4];
                pauli(d[trip[q][1] - 1], trip[q][2], s);
                nj = nj + double(trip[q][3]) * imag_mult(d[trip[q][0] - 1], s);
            }
            c->nablaj[it * V + v] = c->nablaj[it * V + v] + occ * nj;
            if (c->tensor) {
                // GetJMuNu (src/Spwf.f90:2186-2204): Im(psi^+ sigma_nu d_mu psi)
                for (int nu = 0; nu < 3; ++nu)
                    for (int mu = 0; mu < 3; ++mu) {
                        double s[4];
                        pauli(d[mu], nu + 1, s);
                        double& J = c->jmunu[((it * 3 + nu) * 3 + mu) * V + v];
                        J = J + occ * imag_mult(p, s);
                    }
            }
            if (odd) {
                // GetVecj: Im(psi^+ d_m psi); GetVecs: Re(psi^+ sigma_m psi)
                // (src/Spwf.f90:2034-2085)
                for (int m = 0; m < 3; ++m) {
                    double s[4];
                    pauli(p, m + 1, s);
                    const double sm = p[0] * s[0] + p[1] * s[1] + p[2] * s[2] + p[3] * s[3];
                    c->vecj[(it * 3 + m) * V + v] = c->vecj[(it * 3 + m) * V + v] + occ * imag_mult(p, d[m]);
                    c->vecs[(it * 3 + m) * V + v] = c->vecs[(it * 3 + m) * V + v] + occ * sm;
                }
                // GetVecT: T_m = sum_l Re(d_l psi^+ sigma_m d_l psi); GetVecF:
                // F_m = Re(d_m psi^+ sum_n sigma_n d_n psi) (src/Spwf.f90:2087-2180)
                auto re_mult = [](const double* a, const double* b) {
                    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2] + a[3] * b[3];
                };
                if (wantT)
                    for (int m = 0; m < 3; ++m) {
                        double t = 0.0;
                        for (int l = 0; l < 3; ++l) {
                            double sg[4];
                            pauli(d[l], m + 1, sg);
                            t = t + re_mult(d[l], sg);
                        }
                        double& T = c->vecT[(it * 3 + m) * V + v];
                        T = T + occ * t;
                    }
                if (wantF) {
                    double sd[4] = {0.0, 0.0, 0.0, 0.0};
                    for (int n = 0; n < 3; ++n) {
                        double sg[4];
                        pauli(d[n], n + 1, sg);
                        for (int l = 0; l < 4; ++l) sd[l] = sd[l] + sg[l];
                    }
                    for (int m = 0; m < 3; ++m) {
                        double& F = c->vecF[(it * 3 + m) * V + v];
                        F = F + occ * re_mult(d[m], sd);
                    }
                }
            }
        }
    }
    const int P = c->p.pc, S = c->p.sc, TS = c->p.tsc;
    for (int it = 0; it < 2; ++it) {
        for (int d = 0; d < 3; ++d)
            derive_grid(c, &c->rho[it * V], d, P, S, TS, 1, &c->derrho[(it * 3 + d) * V]);
        derive_grid(c, &c->rho[it * V], 3, P, S, TS, 1, &c->laprho[it * V]);
    }
    if (odd) time_odd_curls(c);
    if (c->todd && (Bc.B18 != 0.0 || Bc.B19 != 0.0 || Bc.B20 != 0.0 || Bc.B21 != 0.0)) {
        // lap s with the symmetries of the s components (P, -S, TS, 1),
        // (P, -S, TS, 2), (P, S, TS, 1); grad div s as the reference forms
        // it (src/Densities.f90:1055-1185): its divergence accumulator adds
        // each d_i s_i to the never-assigned DivS field, so only d_z s_z
        // survives, and the gradient takes (-P, S, TS, 1)
        std::vector<double> dz(V);
        for (int it = 0; it < 2; ++it) {
            for (int m = 0; m < 3; ++m)
                derive_grid(c, &c->vecs[(it * 3 + m) * V], 3, P, m == 2 ? S : -S, TS,
                            m == 1 ? 2 : 1, &c->lapS[(it * 3 + m) * V]);
            derive_grid(c, &c->vecs[(it * 3 + 2) * V], 2, P, S, TS, 1, dz.data());
            for (int a = 0; a < 3; ++a)
                derive_grid(c, dz.data(), a, -P, S, TS, 1, &c->gdivS[(it * 3 + a) * V]);
        }
    }
    return MG_OK;
}

// MixDensities, src/DensityMixing.f90:22-86: scheme 0 mixes every density
// (the time-odd ones too: the DensityVector operators combine all fields),
// Density = (1 - DampingParam) Density + DampingParam DensityHistory(1);
// scheme 2 leaves the densities (the U update is preconditioned instead).
extern "C" int orc_mix_densities(orc_ctx* c) {
    if (!c) return MG_ERR_ARG;
    if (c->p.mixing_scheme == 2) return MG_OK;
    if (c->p.mixing_scheme != 0) return MG_ERR_ARG;
    const double d = c->p.damping;
    auto mix = [d](std::vector<double>& x, const std::vector<double>& h) {
        if (h.size() != x.size()) return;
        for (size_t k = 0; k < x.size(); ++k) x[k] = (1.0 - d) * x[k] + d * h[k];
    };
    mix(c->rho, c->hrho); mix(c->tau, c->htau); mix(c->nablaj, c->hnablaj);
    mix(c->derrho, c->hderrho); mix(c->laprho, c->hlaprho);
    mix(c->vecj, c->hvecj); mix(c->vecs, c->hvecs); mix(c->rotj, c->hrotj); mix(c->rots, c->hrots);
    mix(c->jmunu, c->hjmunu);
    mix(c->vecT, c->hvecT); mix(c->vecF, c->hvecF); mix(c->lapS, c->hlapS);
    mix(c->gdivS, c->hgdivS);
    return MG_OK;
}

// SymmetryOperators + CalcRMSRadius, src/Spwf.f90:2289-2347, with the
// mirror actions of src/Spinor.f90:391-490 on the symmetry-free box and the
// mesh of IniMesh (src/Mesh.f90:40-85).  out[6 i ..]: isospin, signature,
// parity, time simplex, x-simplex, RMS radius.
extern "C" int orc_symmetry_operators(orc_ctx* c, int b, double* out) {
    if (!c || !out || b < 0 || b > 1) return MG_ERR_ARG;
    const Basis& B = c->bas[b];
    const long V = c->V;
    const int nx = c->nx, ny = c->ny, nz = c->nz;
    const double dx = c->dx;
    const double ox = c->p.sc ? 0.0 : nx / 2.0 * dx, oy = c->p.tsc ? 0.0 : ny / 2.0 * dx,
                 oz = c->p.pc ? 0.0 : nz / 2.0 * dx;
    auto at = [&](const double* p, int l, int x, int y, int z) {
        return p[l * V + x + (long)nx * (y + (long)ny * z)];
    };
    for (int i = 0; i < c->p.nwt; ++i) {
        const double* p = &B.psi[(long)i * 4 * V];
        const int* qn = &B.qn[4 * i];
        double r2 = 0, par = 0, sig = 0, ts = 0, xs = 0;
        for (int z = 0; z < nz; ++z)
            for (int y = 0; y < ny; ++y)
                for (int x = 0; x < nx; ++x) {
                    double a[4];
                    for (int l = 0; l < 4; ++l) a[l] = at(p, l, x, y, z);
                    const double X = dx / 2.0 + dx * x - ox, Y = dx / 2.0 + dx * y - oy,
                                 Z = dx / 2.0 + dx * z - oz;
                    r2 += (X * X + Y * Y + Z * Z) * (a[0] * a[0] + a[1] * a[1] + a[2] * a[2] + a[3] * a[3]);
                    if (c->folded) continue;
                    const int mx = nx - 1 - x, my = ny - 1 - y, mz = nz - 1 - z;
                    for (int l = 0; l < 4; ++l) par += a[l] * at(p, l, mx, my, mz);
                    {   // ActionOfSignature: MultiplyI(Pauli_z(psi(-x,-y,z)))
                        const double c1 = at(p, 0, mx, my, z), c2 = at(p, 1, mx, my, z),
                                     c3 = at(p, 2, mx, my, z), c4 = at(p, 3, mx, my, z);
                        const double t[4] = {-c2, c1, c4, -c3};
                        sig += t[1] * a[0] - t[0] * a[1] + t[3] * a[2] - t[2] * a[3];
                    }
                    {   // ActionOfTimeSimplex: Conj(psi(x,-y,z))
                        const double t[4] = {at(p, 0, x, my, z), -at(p, 1, x, my, z),
                                             at(p, 2, x, my, z), -at(p, 3, x, my, z)};
                        for (int l = 0; l < 4; ++l) ts += a[l] * t[l];
                    }
                    {   // ActionOfXSimplex: -MultiplyI(spin-swapped psi(-x,y,z))
                        const double c1 = at(p, 0, mx, y, z), c2 = at(p, 1, mx, y, z),
                                     c3 = at(p, 2, mx, y, z), c4 = at(p, 3, mx, y, z);
                        const double t[4] = {c4, -c3, c2, -c1};
                        xs += t[1] * a[0] - t[0] * a[1] + t[3] * a[2] - t[2] * a[3];
                    }
                }
        double* o = out + 6 * i;
        o[0] = qn[0];
        o[1] = qn[2] != 0 ? qn[2] : sig * c->dv;
        o[2] = qn[1] != 0 ? qn[1] : par * c->dv;
        o[3] = qn[3] != 0 ? qn[3] : ts * c->dv;
        o[4] = qn[2] != 0 ? 0.0 : xs * c->dv;
        o[5] = std::sqrt(r2 * c->dv);
    }
    return MG_OK;
}

// Time-odd densities and fields ([it][m][V] vectors, div A [it][V]); any may be NULL.
extern "C" int orc_get_time_odd(orc_ctx* c, double* vecj, double* vecs, double* rotj,
                                double* rots, double* apot, double* spot, double* diva) {
    if (!c || c->p.trc) return MG_ERR_ARG;
    auto cp = [](double* dst, const std::vector<double>& s) {
        if (dst) std::memcpy(dst, s.data(), s.size() * sizeof(double));
    };
    cp(vecj, c->vecj); cp(vecs, c->vecs); cp(rotj, c->rotj); cp(rots, c->rots);
    cp(apot, c->Apot); cp(spot, c->Spot); cp(diva, c->divA);
    return MG_OK;
}

// ActionOfC and ActionOfD of spwf i of basis b, each 4V (test access).
extern "C" int orc_tensor_odd_action(orc_ctx* c, int b, int i, double* xc, double* xd) {
    if (!c || !c->todd || b < 0 || b > 1 || i < 0 || i >= c->p.nwt || !xc || !xd)
        return MG_ERR_ARG;
    tensor_odd_action(c, c->bas[b], i, xc, xd);
    return MG_OK;
}

// Time-odd tensor densities and fields ([it][m][V] vectors, div D [it][V]).
extern "C" int orc_get_time_odd_tensor(orc_ctx* c, double* vect, double* vecf, double* laps,
                                       double* graddivs, double* cpot, double* dpot,
                                       double* divd) {
    if (!c || !c->todd) return MG_ERR_ARG;
    auto cp = [](double* dst, const std::vector<double>& s) {
        if (dst) std::memcpy(dst, s.data(), s.size() * sizeof(double));
    };
    cp(vect, c->vecT); cp(vecf, c->vecF); cp(laps, c->lapS); cp(graddivs, c->gdivS);
    cp(cpot, c->Cpot); cp(dpot, c->Dpot); cp(divd, c->divD);
    return MG_OK;
}

extern "C" int orc_get_densities(orc_ctx* c, double* rho, double* tau, double* nablaj,
                                 double* derrho, double* laprho) {
    if (!c) return MG_ERR_ARG;
    auto cp = [](double* dst, const std::vector<double>& s) {
        if (dst) std::memcpy(dst, s.data(), s.size() * sizeof(double));
    };
    cp(rho, c->rho); cp(tau, c->tau); cp(nablaj, c->nablaj); cp(derrho, c->derrho); cp(laprho, c->laprho);
    return MG_OK;
}
extern "C" int orc_get_jmunu(orc_ctx* c, double* jmunu) {
    if (!c || !jmunu || !c->tensor) return MG_ERR_ARG;
    std::copy(c->jmunu.begin(), c->jmunu.end(), jmunu);
    return MG_OK;
}

extern "C" int orc_set_densities(orc_ctx* c, const double* rho, const double* tau,
                                 const double* nablaj, const double* derrho, const double* laprho) {
    if (!c) return MG_ERR_ARG;
    auto cp = [](std::vector<double>& d, const double* s) {
        if (s) std::memcpy(d.data(), s, d.size() * sizeof(double));
    };
    cp(c->rho, rho); cp(c->tau, tau); cp(c->nablaj, nablaj); cp(c->derrho, derrho); cp(c->laprho, laprho);
    return MG_OK;
}

// --------------------------------------------------------------------------
// Multipole moments for the Coulomb boundary.
// legendre_pnm src/Mesh.f90:96-262, SphericalHarmonics src/Moments.f90:584-691
// (QuantisationAxis 3, SecondaryAxis 1), IniMoments src/Moments.f90:372-582,
// Calculate_Multipole src/Moments.f90:1907-1966.
// --------------------------------------------------------------------------
static void legendre_pnm(int n, int m, double x, double* cx) {
    for (int i = 0; i < m; ++i) cx[i] = 0.0;
    cx[m] = 1.0;
    double somx2 = std::sqrt(1.0 - x * x), fact = 1.0;
    for (int i = 1; i <= m; ++i) { cx[m] = -cx[m] * fact * somx2; fact += 2.0; }
    if (m == n) return;
    cx[m + 1] = x * double(2 * m + 1) * cx[m];
    for (int i = m + 2; i <= n; ++i)
        cx[i] = (double(2 * i - 1) * x * cx[i - 1] - double(i + m - 1) * cx[i - 2]) / double(i - m);
}

static double ipow(double x, int n) {
    double r = 1.0;
    for (int i = 0; i < n; ++i) r *= x;
    return r;
}

// r^l Y_lm (real part if im==0) at (X,Y,Z), as SphericalHarmonics
static double spher_harm(int l, int m, int im, double X, double Y, double Z, int maxl) {
    double r = std::sqrt(X * X + Y * Y + Z * Z);
    double cost = Z / r;
    double phi = std::atan2(Y, X);
    std::vector<double> leg(maxl + 1);
    legendre_pnm(maxl, m, cost, leg.data());
    double fq = 1.0;
    for (int q = 1; q <= 2 * m; ++q) fq = fq / double(l + m - q + 1);
    double fac = ((m % 2) ? -1.0 : 1.0) * std::sqrt(fq) * ipow(r, l);
    fac = fac * std::sqrt(double(2 * l + 1) / (4 * kPi));
    double ang = im ? std::sin(m * phi) : std::cos(m * phi);
    return fac * leg[l] * ang;
}

// Electric moments allowed for EV8 with quantisation axis z
// (NewMoment_Electric: odd l removed by parity, imaginary parts by time
// simplex, odd m by signature).
static void init_moments(orc_ctx* c) {
    const int maxl = 10;  // MaxMoment default, src/Moments.f90:229
    c->moments.clear();
    Moment root;
    root.l = 0; root.m = 0; root.im = 0;
    root.sh.assign(c->V, 1.0 / std::sqrt(4.0 * kPi));
    c->moments.push_back(root);
    for (int l = 1; l <= maxl; ++l)
        for (int m = 0; m <= l; ++m)
            for (int im = 0; im <= 1; ++im) {
                if (c->p.pc && (l % 2)) continue;
                if (c->p.tsc && im == 1) continue;
                if (c->p.sc && (m % 2)) continue;
                if (m == 0 && im == 1) continue;
                Moment mo;
                mo.l = l; mo.m = m; mo.im = im;
                mo.sh.resize(c->V);
                for (int k = 0; k < c->nz; ++k)
                    for (int j = 0; j < c->ny; ++j)
                        for (int i = 0; i < c->nx; ++i) {
                            double X = c->dx / 2.0 + c->dx * i, Y = c->dx / 2.0 + c->dx * j,
                                   Z = c->dx / 2.0 + c->dx * k;
                            mo.sh[i + c->nx * (j + (long)c->ny * k)] = spher_harm(l, m, im, X, Y, Z, maxl);
                        }
                c->moments.push_back(mo);
            }
}

// --------------------------------------------------------------------------
// Multipole constraints: alternating-direction kind (ConstraintType 2, the
// &MomentConstraint default), Isoswitch 1, Total false, CutoffType 0,
// Damping 0 (src/Moments.f90:258, :280).
// --------------------------------------------------------------------------
static const double kRadd = 4.0, kAcut = 0.4;  // src/Moments.f90:258
// d0 = 0.1 is a default-kind (single precision) literal assigned to a
// real(dp) variable (src/Moments.f90:258): its value is 0.1f widened.
static const double kD0 = (double)0.1f;

// RutzCutOff, src/Moments.f90:2703-2871: distance DeltaR from each mesh
// point to the surface rho = max(rho)/10 (linear interpolation between
// neighbours of the stored box, negative inside), then
// Cutoff = 1 / (1 + exp((DeltaR - radd) / acut)).
static void rutz_cutoff(orc_ctx* c) {
    const long V = c->V;
    const int nx = c->nx, ny = c->ny, nz = c->nz;
    const double dx = c->dx;
    c->cutoff.assign(2 * V, 0.0);
    auto mesh = [&](int i) { return dx / 2.0 + dx * i; };   // src/Mesh.f90:50
    for (int it = 0; it < 2; ++it) {
        const double* r = &c->rho[it * V];
        double s = 0.0;
        for (long v = 0; v < V; ++v) s += r[v];
        if (c->dv * s < 0.0000000001) continue;   // no particles: Cutoff = 0
        double mx = r[0];
        for (long v = 1; v < V; ++v) mx = std::max(mx, r[v]);
        const double tr = mx / 10.0;
        auto R = [&](int i, int j, int k) { return r[i + (long)nx * (j + (long)ny * k)]; };
        std::vector<double> sx, sy, sz;
        for (int k = 0; k < nz - 1; ++k)
            for (int j = 0; j < ny - 1; ++j)
                for (int i = 0; i < nx - 1; ++i) {
                    const double X = mesh(i), Y = mesh(j), Z = mesh(k);
                    const double r0 = R(i, j, k);
                    const double rx = R(i + 1, j, k), ry = R(i, j + 1, k), rz = R(i, j, k + 1);
                    if ((r0 >= tr && rx <= tr) || (r0 <= tr && rx >= tr)) {
                        sx.push_back(X + dx * (tr - r0) / (rx - r0)); sy.push_back(Y); sz.push_back(Z);
                    }
                    if ((r0 >= tr && ry <= tr) || (r0 <= tr && ry >= tr)) {
                        sx.push_back(X); sy.push_back(Y + dx * (tr - r0) / (ry - r0)); sz.push_back(Z);
                    }
                    if ((r0 >= tr && rz <= tr) || (r0 <= tr && rz >= tr)) {
                        sx.push_back(X); sy.push_back(Y); sz.push_back(Z + dx * (tr - r0) / (rz - r0));
                    }
                }
        const size_t T = sx.size();
        for (int k = 0; k < nz; ++k)
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nx; ++i) {
                    const double X = mesh(i), Y = mesh(j), Z = mesh(k);
                    double d = 1.0e12;
                    for (size_t l = 0; l < T; ++l) {
                        const double a = X - sx[l], b = Y - sy[l], e = Z - sz[l];
                        d = std::min(d, a * a + b * b + e * e);
                    }
                    const long v = i + (long)nx * (j + (long)ny * k);
                    const double sig = r[v] > tr ? -1.0 : 1.0;
                    const double delta = sig * std::sqrt(d);
                    c->cutoff[it * V + v] = 1.0 / (1.0 + std::exp((delta - kRadd) / kAcut));
                }
    }
}

// CalcConstraintEnergy, src/Moments.f90:2368-2486 (alternating constraints,
// Isoswitch 1, not Total; Damping 0 so the old field is dropped):
// ConstraintEnergy(it) += 2 I (<Q> - C) Q_lm Cutoff(it).
static void calc_constraint_energy(orc_ctx* c) {
    const long V = c->V;
    c->cons_energy.assign(2 * V, 0.0);
    for (const Constraint& k : c->cons) {
        if (k.type != 2) continue;
        const double factor = 2.0 * k.intensity;
        const double value = k.value[0] + k.value[1];
        const double a = factor * (value - k.constraint);
        const std::vector<double>& sh = c->moments[k.mom].sh;
        for (int it = 0; it < 2; ++it)
            for (long v = 0; v < V; ++v)
                c->cons_energy[it * V + v] += a * sh[v] * c->cutoff[it * V + v];
    }
}

// Readjust (alternating branch), src/Moments.f90:2994-3058, over the
// constrained moments as ReadjustAllMoments :2336-2366; then
// TurnOffConstraints :3516-3550.
static void readjust_moments(orc_ctx* c, int iteration) {
    for (Constraint& k : c->cons) {
        if (k.type != 2) continue;
        if (k.intensity == 0.0) {
            k.intensity = 2.0 / (k.squared[0] + k.squared[1]);
            if (c->step_mom != 0.0) k.intensity = 0.5 * k.intensity;
        }
        k.constraint = k.constraint - ((k.value[0] + k.value[1]) - k.true_constraint);
    }
    for (Constraint& k : c->cons)
        if (k.type != 0 && k.iteration > 0 && iteration > k.iteration) k.type = 0;
}

static bool any_alternating(const orc_ctx* c) {   // CheckForAlternateConstraints
    for (const Constraint& k : c->cons)
        if (k.type == 2) return true;
    return false;
}

// CalculateAllMoments, src/Moments.f90:2250-2334 (electric moments): the
// cutoff, every moment's value (Calculate_Multipole :1907-1966) and, for the
// constrained ones, the squares; the first call sets each constraint's
// running target to the current value (:2277-2297); then the constraint
// field.
extern "C" int orc_calculate_moments(orc_ctx* c) {
    if (!c) return MG_ERR_ARG;
    if (c->moments.empty()) init_moments(c);
    // CompCutoff runs in every CalculateAllMoments (src/Moments.f90:2267);
    // the constraints and the cranking fields use it
    if (!c->cons.empty() || cranking(c)) rutz_cutoff(c);
    for (Moment& mo : c->moments)
        for (int it = 0; it < 2; ++it) {
            double s = 0.0;
            for (long v = 0; v < c->V; ++v) s += mo.sh[v] * c->rho[it * c->V + v];
            mo.value[it] = s * c->dv;
        }
    if (c->cons.empty()) return MG_OK;
    for (Constraint& k : c->cons) {
        const std::vector<double>& sh = c->moments[k.mom].sh;
        // SaveOld = 1: OldValue shifts and takes the previous Value (:1921-1931)
        for (int i = 6; i > 0; --i) k.old_value[i] = k.old_value[i - 1];
        k.old_value[0] = k.value[0] + k.value[1];
        for (int it = 0; it < 2; ++it) {
            double s = 0.0;
            for (long v = 0; v < c->V; ++v) s += sh[v] * sh[v] * c->rho[it * c->V + v];
            k.value[it] = c->moments[k.mom].value[it];
            k.squared[it] = s * c->dv;
        }
        if (!k.started && k.type != 0) k.constraint = k.value[0] + k.value[1];
        k.started = true;
    }
    calc_constraint_energy(c);
    return MG_OK;
}

extern "C" int orc_add_constraint(orc_ctx* c, const mg_moment_constraint* mc) {
    if (!c || !mc || !c->folded || mc->l < 1) return MG_ERR_ARG;
    if (c->moments.empty()) init_moments(c);
    int mom = -1;
    for (size_t q = 0; q < c->moments.size(); ++q)
        if (c->moments[q].l == mc->l && c->moments[q].m == mc->m && c->moments[q].im == 0)
            mom = (int)q;
    if (mom < 0) return MG_ERR_ARG;
    Constraint k;
    k.l = mc->l; k.m = mc->m; k.mom = mom;
    k.iteration = mc->iteration;
    k.constraint = k.true_constraint = mc->constraint;   // src/Moments.f90:3719-3726
    k.intensity = mc->intensity;
    c->cons.push_back(k);
    c->alternate_check = true;
    if (c->cutoff.empty()) c->cutoff.assign(2 * c->V, 0.0);
    if (c->cons_energy.empty()) c->cons_energy.assign(2 * c->V, 0.0);
    return (int)c->cons.size() - 1;
}

extern "C" int orc_get_constraint(orc_ctx* c, int q, mg_constraint_state* out) {
    if (!c || !out || q < 0 || q >= (int)c->cons.size()) return MG_ERR_ARG;
    const Constraint& k = c->cons[q];
    for (int it = 0; it < 2; ++it) { out->value[it] = k.value[it]; out->squared[it] = k.squared[it]; }
    out->constraint = k.constraint;
    out->intensity = k.intensity;
    out->active = k.type != 0;
    return MG_OK;
}

extern "C" int orc_get_constraint_fields(orc_ctx* c, double* cutoff, double* field) {
    if (!c) return MG_ERR_ARG;
    const long V = c->V;
    for (long v = 0; v < 2 * V; ++v) {
        if (cutoff) cutoff[v] = c->cutoff.empty() ? 0.0 : c->cutoff[v];
        if (field) field[v] = c->cons_energy.empty() ? 0.0 : c->cons_energy[v];
    }
    return MG_OK;
}

extern "C" int orc_readjust_moments(orc_ctx* c, int iteration) {
    if (!c) return MG_ERR_ARG;
    readjust_moments(c, iteration);
    return MG_OK;
}

// AlternateStep, src/ImaginaryTime.f90:306-437 (no cranking):
// psi <- psi - multipole(it) psi with
// multipole(it) = sum 0.5 (<Q> - Q_target) / (<Q^2> + d0) Cutoff(it) Q_lm
// over the alternating constraints, then GramSchmidt.
extern "C" int orc_alternate_step(orc_ctx* c) {
    if (!c) return MG_ERR_ARG;
    const long V = c->V;
    if (!c->cons.empty()) rutz_cutoff(c);
    std::vector<double> mp(2 * V, 0.0);
    bool any = false;
    for (const Constraint& k : c->cons) {
        if (k.type != 2) continue;
        any = true;
        const double o2 = k.squared[0] + k.squared[1];
        const double value = k.value[0] + k.value[1];
        const double f = 0.5 * (value - k.true_constraint) / (o2 + kD0);
        const std::vector<double>& sh = c->moments[k.mom].sh;
        for (int it = 0; it < 2; ++it)
            for (long v = 0; v < V; ++v) mp[it * V + v] += f * c->cutoff[it * V + v] * sh[v];
    }
    if (any) {
        Basis& B = c->bas[MG_HF_BASIS];
        for (int i = 0; i < c->p.nwt; ++i) {
            const int it = (B.qn[4 * i] + 3) / 2 - 1;
            double* p = &B.psi[(long)i * 4 * V];
            for (int l = 0; l < 4; ++l)
                for (long v = 0; v < V; ++v) p[l * V + v] = p[l * V + v] - mp[it * V + v] * p[l * V + v];
        }
    }
    return orc_gram_schmidt(c);
}

extern "C" int orc_get_moments(orc_ctx* c, double* values, int* lm, int max_count) {
    if (!c) return MG_ERR_ARG;
    int n = (int)c->moments.size();
    for (int i = 0; i < n && i < max_count; ++i) {
        if (values) { values[2 * i] = c->moments[i].value[0]; values[2 * i + 1] = c->moments[i].value[1]; }
        if (lm) { lm[2 * i] = c->moments[i].l; lm[2 * i + 1] = c->moments[i].m; }
    }
    return n;
}

// --------------------------------------------------------------------------
// Coulomb: SetupCoulomb / InitialGuess / CoulombBound / ConjugGrad
// (src/Coulomb.f90:255-900) with CoulombLaplacian / Coulomb_1D
// (src/CoulombDerivatives.f90:144-281), CoulombLapOrder = 2, EV8 box.
// --------------------------------------------------------------------------
static void coulomb_setup(orc_ctx* c) {
    const int bcn = 2;
    c->mx = c->nx + bcn; c->my = c->ny + bcn; c->mz = c->nz + bcn;
    long M = (long)c->mx * c->my * c->mz;
    c->cpot_complete.assign(M, 0.0);
    c->source.assign(M, 0.0);
    c->bc.assign(M, 0.0);
    c->rext.assign(M, 0.0);
    for (int k = 0; k < c->mz; ++k)
        for (int j = 0; j < c->my; ++j)
            for (int i = 0; i < c->mx; ++i) {
                double X = (0.5 + i) * c->dx, Y = (0.5 + j) * c->dx, Z = (0.5 + k) * c->dx;
                c->rext[i + c->mx * (j + (long)c->my * k)] = std::sqrt(X * X + Y * Y + Z * Z);
            }
    if (c->moments.empty()) init_moments(c);
    c->sh_ext.assign(c->moments.size() * M, 0.0);
    for (size_t q = 0; q < c->moments.size(); ++q) {
        const Moment& mo = c->moments[q];
        for (int k = 0; k < c->mz; ++k)
            for (int j = 0; j < c->my; ++j)
                for (int i = 0; i < c->mx; ++i) {
                    double X = (0.5 + i) * c->dx, Y = (0.5 + j) * c->dx, Z = (0.5 + k) * c->dx;
                    c->sh_ext[q * M + i + c->mx * (j + (long)c->my * k)] =
                        spher_harm(mo.l, mo.m, mo.im, X, Y, Z, 10);
                }
    }
    // InitialGuess, src/Coulomb.f90:542-581
    double R = 1.25 * std::pow(c->p.neutrons + c->p.protons, 1.0 / 3.0);
    double charge = c->p.protons * c->f.e2, fac = charge / (2 * R);
    for (int k = 0; k < c->nz; ++k)
        for (int j = 0; j < c->ny; ++j)
            for (int i = 0; i < c->nx; ++i) {
                long o = i + c->mx * (j + (long)c->my * k);
                double r = c->rext[o];
                c->cpot_complete[o] = (r <= R) ? fac * (3 - r * r / (R * R)) : charge / r;
            }
    c->coulomb_init = true;
}

// 5-point FD Laplacian on the interior (1..n per axis) with an even mirror
// at the low end; zero outside the interior.
static void coulomb_laplacian(const orc_ctx* c, const double* g, double* out) {
    static const double cf[5] = {-1.0 / 12.0, 4.0 / 3.0, -5.0 / 2.0, 4.0 / 3.0, -1.0 / 12.0};
    const int mx = c->mx, my = c->my, mz = c->mz;
    const long M = (long)mx * my * mz;
    std::fill(out, out + M, 0.0);
    const double factor = 1.0 / (c->dx * c->dx);
    auto at = [&](int i, int j, int k) { return g[i + mx * (j + (long)my * k)]; };
    for (int k = 0; k < c->nz; ++k)
        for (int j = 0; j < c->ny; ++j)
            for (int i = 0; i < c->nx; ++i) {
                double dxl = 0.0, dyl = 0.0, dzl = 0.0;
                for (int q = -2; q <= 2; ++q) {
                    int ii = i + q;  // 0-based; mirror: -1 -> 0, -2 -> 1
                    dxl += cf[q + 2] * at(ii < 0 ? -ii - 1 : ii, j, k);
                    int jj = j + q;
                    dyl += cf[q + 2] * at(i, jj < 0 ? -jj - 1 : jj, k);
                    int kk = k + q;
                    dzl += cf[q + 2] * at(i, j, kk < 0 ? -kk - 1 : kk);
                }
                out[i + mx * (j + (long)my * k)] = dxl * factor + dyl * factor + dzl * factor;
            }
}

extern "C" int orc_solve_coulomb(orc_ctx* c, int* iters) {
    if (!c) return MG_ERR_ARG;
    if (!c->p.pc || !c->p.sc || !c->p.tsc) return MG_ERR_ARG;
    if (!c->coulomb_init) coulomb_setup(c);
    const int mx = c->mx, my = c->my, mz = c->mz;
    const long M = (long)mx * my * mz;
    // CoulombBound, src/Coulomb.f90:583-674
    std::fill(c->bc.begin(), c->bc.end(), 0.0);
    std::fill(c->source.begin(), c->source.end(), 0.0);
    for (int k = 0; k < c->nz; ++k)
        for (int j = 0; j < c->ny; ++j)
            for (int i = 0; i < c->nx; ++i)
                c->source[i + mx * (j + (long)my * k)] =
                    -4 * kPi * c->f.e2 * c->rho[c->V + i + c->nx * (j + (long)c->ny * k)];
    int maxl = c->p.max_l_coul > 0 ? c->p.max_l_coul : 10;
    for (size_t q = 0; q < c->moments.size(); ++q) {
        const Moment& mo = c->moments[q];
        if (mo.l > maxl) break;
        double value = mo.value[1] * (4 * kPi / (2 * mo.l + 1));
        for (int k = 0; k < mz; ++k)
            for (int j = 0; j < my; ++j)
                for (int i = 0; i < mx; ++i) {
                    if (i < c->nx && j < c->ny && k < c->nz) continue;
                    long o = i + mx * (j + (long)my * k);
                    c->bc[o] = c->bc[o] + value * c->sh_ext[q * M + o] * c->f.e2 /
                                              ipow(c->rext[o], 2 * mo.l + 1);
                }
    }
    for (long o = 0; o < M; ++o)
        if (c->bc[o] != 0.0) c->cpot_complete[o] = c->bc[o];
    // ConjugGrad, src/Coulomb.f90:755-900
    double prec = 1.0e-9 / (c->dx * c->dx * c->dx * c->nx * c->ny * c->nz);
    std::vector<double> res(M), p(M), t(M);
    double* sol = c->cpot_complete.data();
    coulomb_laplacian(c, sol, t.data());
    for (long o = 0; o < M; ++o) res[o] = -t[o] + c->source[o];
    p = res;
    double pnorm = 0.0;
    for (long o = 0; o < M; ++o) pnorm += res[o] * res[o];
    int maxit = c->p.coulomb_max > 0 ? c->p.coulomb_max : 500;
    int it = 0, status = MG_NOT_CONVERGED;
    for (it = 1; it <= maxit; ++it) {
        coulomb_laplacian(c, p.data(), t.data());
        double integral = 0.0;
        for (long o = 0; o < M; ++o) integral += res[o] * t[o];
        double a = pnorm / integral;
        for (long o = 0; o < M; ++o) sol[o] = sol[o] + a * p[o];
        for (long o = 0; o < M; ++o) res[o] = res[o] - a * t[o];
        double nn = 0.0;
        for (long o = 0; o < M; ++o) nn += res[o] * res[o];
        if (nn <= prec) { status = MG_OK; break; }
        double ck = nn / pnorm;
        pnorm = nn;
        for (long o = 0; o < M; ++o) p[o] = res[o] + ck * p[o];
    }
    if (iters) *iters = std::min(it, maxit);
    for (int k = 0; k < c->nz; ++k)
        for (int j = 0; j < c->ny; ++j)
            for (int i = 0; i < c->nx; ++i)
                c->coulomb[i + c->nx * (j + (long)c->ny * k)] = sol[i + mx * (j + (long)my * k)];
    double fac = -std::pow(3 / kPi, 1 / 3.0) * c->f.e2;
    for (long v = 0; v < c->V; ++v) c->coulex[v] = fac * std::pow(c->rho[c->V + v], 1 / 3.0);
    return status;
}

// --------------------------------------------------------------------------
// Potentials: CalcUPot src/MeanFields.f90:269-409, CalcWPot :494-597,
// CalcBPot :115-150; ConstructPotentials src/PotentialMixing.f90:17-201.
// --------------------------------------------------------------------------
// CalcAPot (src/MeanFields.f90:411-492) and CalcSPot (:618-712) for the
// functional without tensor, N2LO and J2 terms, with the cranking fields
// CrankAPot = -f_cut omega x r and CrankSPot = -f_cut omega / 2
// (src/Cranking.f90:234-334); div A with the symmetry arguments of :476-481.
static void time_odd_potentials(orc_ctx* c) {
    const long V = c->V;
    const mg_skyrme_b& B = c->B;
    const int P = c->p.pc, S = c->p.sc, TS = c->p.tsc;
    const double* om = c->p.omega;
    const bool crank = cranking(c);
    auto lc = [](int i, int j, int k) {
        if (i == j || j == k || k == i) return 0;
        if ((i == 0 && j == 1 && k == 2) || (i == 2 && j == 0 && k == 1) || (i == 1 && j == 2 && k == 0))
            return 1;
        return -1;
    };
    for (int it = 0; it < 2; ++it) {
        const int at = 1 - it;
        for (int m = 0; m < 3; ++m)
            for (long v = 0; v < V; ++v) {
                const long q = (it * 3 + m) * V + v, qa = (at * 3 + m) * V + v;
                double a = -2.0 * ((B.B3 + B.B4) * c->vecj[q] + B.B3 * c->vecj[qa]);
                a = a + ((B.B9 + B.B9q) * c->rots[q] + B.B9 * c->rots[qa]);
                c->Apot[q] = a;
                const double rt = c->rho[v] + c->rho[V + v];
                const double ra = std::pow(rt, B.byt3a);
                double sv = (B.B9 + B.B9q) * c->rotj[q] + B.B9 * c->rotj[qa] +
                            2.0 * ((B.B10 + B.B11) * c->vecs[q] + B.B10 * c->vecs[qa]) +
                            2.0 * ((B.B12a + B.B13a) * (ra * c->vecs[q]) + B.B12a * (ra * c->vecs[qa]));
                if (c->todd) {
                    // the time-odd tensor terms of CalcSPot (src/MeanFields.f90:651-670)
                    if (B.B14 != 0.0 || B.B15 != 0.0)
                        sv = sv - (B.B14 + B.B15) * c->vecT[q] - B.B14 * c->vecT[qa];
                    if (B.B16 != 0.0 || B.B17 != 0.0)
                        sv = sv - 2.0 * (B.B16 + B.B17) * c->vecF[q] - 2.0 * B.B16 * c->vecF[qa];
                    if (B.B18 != 0.0 || B.B19 != 0.0 || B.B20 != 0.0 || B.B21 != 0.0)
                        sv = sv + 2.0 * ((B.B18 + B.B19) * c->lapS[q] + B.B18 * c->lapS[qa]) -
                             2.0 * ((B.B20 + B.B21) * c->gdivS[q] - B.B20 * c->gdivS[qa]);
                }
                if (B.B12b != 0.0 || B.B13b != 0.0) {
                    const double rb = std::pow(rt, B.byt3b);
                    sv = sv + 2.0 * ((B.B12b + B.B13b) * (rb * c->vecs[q]) + B.B12b * (rb * c->vecs[qa]));
                }
                c->Spot[q] = sv;
            }
    }
    if (crank) {
        for (int it = 0; it < 2; ++it)
            for (int k = 0; k < 3; ++k)
                for (int j = 0; j < 3; ++j)
                    for (int i = 0; i < 3; ++i) {
                        const int e = lc(i, j, k);
                        for (int z = 0; z < c->nz; ++z)
                            for (int y = 0; y < c->ny; ++y)
                                for (int x = 0; x < c->nx; ++x) {
                                    const long v = x + (long)c->nx * (y + (long)c->ny * z);
                                    const double r[3] = {c->dx / 2.0 + c->dx * x, c->dx / 2.0 + c->dx * y,
                                                         c->dx / 2.0 + c->dx * z};
                                    double& a = c->Apot[(it * 3 + i) * V + v];
                                    a = a - e * om[j] * r[k] * c->cutoff[it * V + v];
                                }
                    }
        for (int it = 0; it < 2; ++it)
            for (int i = 0; i < 3; ++i)
                for (long v = 0; v < V; ++v) {
                    double& sv = c->Spot[(it * 3 + i) * V + v];
                    sv = sv - 1 / 2.0 * om[i] * c->cutoff[it * V + v];
                }
    }
    std::vector<double> t1(V), t2(V), t3(V);
    for (int it = 0; it < 2; ++it) {
        derive_grid(c, &c->Apot[(it * 3 + 0) * V], 0, -P, -S, TS, 2, t1.data());
        derive_grid(c, &c->Apot[(it * 3 + 1) * V], 1, -P, -S, TS, 1, t2.data());
        derive_grid(c, &c->Apot[(it * 3 + 2) * V], 2, -P, S, TS, 2, t3.data());
        for (long v = 0; v < V; ++v) c->divA[it * V + v] = t1[v] + t2[v] + t3[v];
    }
    if (!c->todd) return;
    // CalcCPot: C_q = -B14 s_t - B15 s_q; CalcDPot: D_q = -2 B16 s_t - 2 B17 s_q,
    // d_n D_m with the s symmetries, div D (src/MeanFields.f90:714-790)
    for (int it = 0; it < 2; ++it)
        for (int m = 0; m < 3; ++m)
            for (long v = 0; v < V; ++v) {
                const double st = c->vecs[m * V + v] + c->vecs[(3 + m) * V + v];
                const double sq = c->vecs[(it * 3 + m) * V + v];
                c->Cpot[(it * 3 + m) * V + v] = -(B.B14 * st) - B.B15 * sq;
                c->Dpot[(it * 3 + m) * V + v] = -(2 * B.B16 * st) - 2 * B.B17 * sq;
            }
    for (int it = 0; it < 2; ++it) {
        for (int m = 0; m < 3; ++m)
            for (int n = 0; n < 3; ++n)
                derive_grid(c, &c->Dpot[(it * 3 + m) * V], n, P, m == 2 ? S : -S, TS,
                            m == 1 ? 2 : 1, &c->dD[((it * 3 + m) * 3 + n) * V]);
        for (long v = 0; v < V; ++v)
            c->divD[it * V + v] = c->dD[((it * 3 + 0) * 3 + 0) * V + v] +
                                  c->dD[((it * 3 + 1) * 3 + 1) * V + v] +
                                  c->dD[((it * 3 + 2) * 3 + 2) * V + v];
    }
}

static void calc_potentials(orc_ctx* c) {
    const long V = c->V;
    const mg_skyrme_b& B = c->B;
    const double eps = 1.0e-20;
    const int P = c->p.pc, S = c->p.sc, TS = c->p.tsc;
    for (long v = 0; v < V; ++v) {
        double rn = c->rho[v], rp = c->rho[V + v];
        double rt = rn + rp;
        double njt = c->nablaj[v] + c->nablaj[V + v];
        double u[2];
        u[0] = (2.0 * B.B1 + 2.0 * B.B2) * rn + 2.0 * B.B1 * rp;
        u[1] = (2.0 * B.B1 + 2.0 * B.B2) * rp + 2.0 * B.B1 * rn;
        for (int it = 0; it < 2; ++it) {
            int at = 1 - it;
            double ri = c->rho[it * V + v], ra = c->rho[at * V + v];
            double x = u[it] + (B.B3 + B.B4) * c->tau[it * V + v] + B.B3 * c->tau[at * V + v] +
                       2.0 * ((B.B5 + B.B6) * c->laprho[it * V + v] + B.B5 * c->laprho[at * V + v]) +
                       (2 + B.byt3a) * B.B7a * std::pow(rt + eps, 1 + B.byt3a) +
                       B.B8a * (B.byt3a * std::pow(rt, B.byt3a) / (rt + eps) * (ri * ri + ra * ra) +
                                2.0 * std::pow(rt, B.byt3a) * ri) +
                       B.B9 * njt + B.B9q * c->nablaj[it * V + v];
            if (B.B7b != 0.0 || B.B8b != 0.0)
                x = x + (2 + B.byt3b) * B.B7b * std::pow(rt + eps, 1 + B.byt3b) +
                    B.B8b * (B.byt3b * std::pow(rt, B.byt3b) / (rt + eps) * (ri * ri + ra * ra) +
                             2.0 * std::pow(rt, B.byt3b) * ri);
            u[it] = x;
        }
        u[1] = u[1] + c->coulomb[v];
        if (c->f.cexchange == 2) u[1] = u[1] + c->coulex[v];
        // U = U + ConstraintEnergy (src/MeanFields.f90:403)
        if (!c->cons_energy.empty()) {
            u[0] = u[0] + c->cons_energy[v];
            u[1] = u[1] + c->cons_energy[V + v];
        }
        c->U[v] = u[0];
        c->U[V + v] = u[1];
    }
    // W: -sum_k eps_{kmn} ((B9+B9q) d_k rho_q + B9 d_k rho_q')
    std::fill(c->W.begin(), c->W.end(), 0.0);
    auto lc = [](int i, int j, int k) {
        if (i == j || j == k || k == i) return 0;
        if ((i == 1 && j == 2 && k == 3) || (i == 3 && j == 1 && k == 2) || (i == 2 && j == 3 && k == 1))
            return 1;
        return -1;
    };
    for (int it = 0; it < 2; ++it)
        for (int m = 1; m <= 3; ++m)
            for (int n = 1; n <= 3; ++n)
                for (int k = 1; k <= 3; ++k) {
                    int e = lc(k, m, n);
                    double* w = &c->W[((it * 3 + (n - 1)) * 3 + (m - 1)) * V];
                    const double* dq = &c->derrho[(it * 3 + k - 1) * V];
                    const double* dqa = &c->derrho[((1 - it) * 3 + k - 1) * V];
                    for (long v = 0; v < V; ++v)
                        w[v] = w[v] - e * ((B.B9 + B.B9q) * dq[v] + B.B9 * dqa[v]);
                }
    if (c->tensor) {
        // CalcWPot's J^2 parts (src/MeanFields.f90:531-556): B14, B15 on
        // J_{mu nu}; B16, B17 on J_{nu mu} and on the trace times delta
        const double* J = c->jmunu.data();
        auto jm = [&](int it, int m, int n, long v) {   // J(m, n, it), 1-based m, n
            return J[((it * 3 + (n - 1)) * 3 + (m - 1)) * V + v];
        };
        for (int it = 0; it < 2; ++it) {
            const int at = 1 - it;
            for (int m = 1; m <= 3; ++m)
                for (int n = 1; n <= 3; ++n) {
                    double* w = &c->W[((it * 3 + (n - 1)) * 3 + (m - 1)) * V];
                    if (B.B14 != 0.0 || B.B15 != 0.0)
                        for (long v = 0; v < V; ++v)
                            w[v] = w[v] + 2.0 * (B.B14 + B.B15) * jm(it, m, n, v) +
                                   2.0 * B.B14 * jm(at, m, n, v);
                }
            if (B.B16 != 0.0 || B.B17 != 0.0)
                for (int m = 1; m <= 3; ++m) {
                    for (int n = 1; n <= 3; ++n) {
                        double* w = &c->W[((it * 3 + (n - 1)) * 3 + (m - 1)) * V];
                        for (long v = 0; v < V; ++v)
                            w[v] = w[v] + 2.0 * (B.B16 + B.B17) * jm(it, n, m, v) +
                                   2.0 * B.B16 * jm(at, n, m, v);
                    }
                    double* w = &c->W[((it * 3 + (m - 1)) * 3 + (m - 1)) * V];
                    for (int k = 1; k <= 3; ++k)
                        for (long v = 0; v < V; ++v)
                            w[v] = w[v] + 2 * (B.B16 + B.B17) * jm(it, k, k, v) +
                                   2 * B.B16 * jm(at, k, k, v);
                }
        }
    }
    // div W with the symmetry arguments of src/MeanFields.f90:575-591
    std::vector<double> t1(V), t2(V), t3(V);
    struct Term { int dir, m, n, P, S, TS, comp; };
    static const Term terms[3][3] = {
        {{0, 1, 1, -1, 1, 1, 2}, {1, 2, 1, -1, 1, 1, 1}, {2, 3, 1, -1, -1, 1, 2}},
        {{0, 1, 2, -1, 1, 1, 1}, {1, 2, 2, -1, 1, 1, 2}, {2, 3, 2, -1, -1, 1, 1}},
        {{0, 1, 3, -1, -1, 1, 2}, {1, 2, 3, -1, -1, 1, 1}, {2, 3, 3, -1, 1, 1, 2}}};
    for (int it = 0; it < 2; ++it)
        for (int nu = 0; nu < 3; ++nu) {
            std::vector<double>* tv[3] = {&t1, &t2, &t3};
            for (int q = 0; q < 3; ++q) {
                const Term& T = terms[nu][q];
                const double* w = &c->W[((it * 3 + (T.n - 1)) * 3 + (T.m - 1)) * V];
                derive_grid(c, w, T.dir, T.P * P, T.S * S, T.TS * TS, T.comp, tv[q]->data());
            }
            for (long v = 0; v < V; ++v) c->divW[(it * 3 + nu) * V + v] = t1[v] + t2[v] + t3[v];
        }
    // B and grad B
    for (int it = 0; it < 2; ++it) {
        int at = 1 - it;
        for (long v = 0; v < V; ++v)
            c->Bp[it * V + v] = B.B3 * c->rho[at * V + v] + (B.B3 + B.B4) * c->rho[it * V + v];
        for (int d = 0; d < 3; ++d)
            derive_grid(c, &c->Bp[it * V], d, P, S, TS, 1, &c->nablaB[(it * 3 + d) * V]);
    }
    if (!c->p.trc) time_odd_potentials(c);
}

// PreconditionPotential + preconoperator, src/Damping.f90:158-228: per
// isospin, CG on (beta + alpha Lap) x = pot with alpha = -preconu, beta = 1,
// the Lagrange Laplacian with the potential's symmetry arguments, at most
// 300 steps, stop when sum(residual^2) dv < 1e-8.
static void precondition_potential(orc_ctx* c, const std::vector<double>& pot,
                                   std::vector<double>& inv, int P, int S, int TS, int comp) {
    const long V = c->V;
    const double alpha = -c->p.precon_u, beta = 1.0;
    inv.assign(2 * V, 0.0);
    std::vector<double> res(V), dir(V), upd(V), lap(V);
    for (int it = 0; it < 2; ++it) {
        for (long v = 0; v < V; ++v) res[v] = pot[it * V + v];
        dir = res;
        double nn = 0.0;
        for (long v = 0; v < V; ++v) nn = nn + dir[v] * dir[v];
        nn = nn * c->dv;
        if (nn == 0.0) continue;   // a zero update stays zero (0/0 otherwise)
        for (int iter = 1; iter <= 300; ++iter) {
            derive_grid(c, dir.data(), 3, P, S, TS, comp, lap.data());
            for (long v = 0; v < V; ++v) upd[v] = beta * dir[v] + alpha * lap[v];
            double dd = 0.0;
            for (long v = 0; v < V; ++v) dd = dd + dir[v] * upd[v];
            const double a = nn / (dd * c->dv);
            for (long v = 0; v < V; ++v) {
                inv[it * V + v] = inv[it * V + v] + a * dir[v];
                res[v] = res[v] - a * upd[v];
            }
            const double old = nn;
            nn = 0.0;
            for (long v = 0; v < V; ++v) nn = nn + res[v] * res[v];
            nn = nn * c->dv;
            const double b = nn / old;
            for (long v = 0; v < V; ++v) dir[v] = res[v] + b * dir[v];
            if (nn < 1e-8) break;
        }
    }
}

extern "C" int orc_construct_potentials(orc_ctx* c, int* iters) {
    if (!c) return MG_ERR_ARG;
    int st = MG_OK;
    c->Uold = c->U;   // UpotOld = Upot (src/PotentialMixing.f90:115)
    const std::vector<double> Sold = c->Spot;   // SpotOld = Spot (:122)
    const std::vector<double> Wold = c->W;      // WpotOld = Wpot (:117)
    if (c->p.coulomb_solver != 0) {
        st = orc_solve_coulomb(c, iters);
        if (st < 0) return st;
    } else {
        std::fill(c->coulomb.begin(), c->coulomb.end(), 0.0);
        std::fill(c->coulex.begin(), c->coulex.end(), 0.0);
        if (iters) *iters = 0;
    }
    calc_potentials(c);
    // MixingScheme 2: Upot = UpotOld + PreconditionPotential(Upot - UpotOld)
    // once UpotOld is not all zero (src/PotentialMixing.f90:143-154)
    bool have_old = false;
    for (double u : c->Uold) have_old = have_old || u != 0.0;
    if (c->p.mixing_scheme == 2 && have_old) {
        std::vector<double> du(c->U.size()), inv;
        for (size_t k = 0; k < du.size(); ++k) du[k] = c->U[k] - c->Uold[k];
        const int P = c->p.pc, S = c->p.sc, TS = c->p.tsc;
        precondition_potential(c, du, inv, P, S, TS, 1);
        for (size_t k = 0; k < du.size(); ++k) c->U[k] = c->Uold[k] + inv[k];
        if (!c->p.trc) {
            // each S component: (P, -S, TS, 1), (P, -S, TS, 2), (P, S, TS, 1)
            // (src/PotentialMixing.f90:156-168)
            const long V = c->V;
            for (int m = 0; m < 3; ++m) {
                std::vector<double> ds(2 * V);
                for (int it = 0; it < 2; ++it)
                    for (long v = 0; v < V; ++v)
                        ds[it * V + v] = c->Spot[(it * 3 + m) * V + v] - Sold[(it * 3 + m) * V + v];
                precondition_potential(c, ds, inv, P, m == 2 ? S : -S, TS, m == 1 ? 2 : 1);
                for (int it = 0; it < 2; ++it)
                    for (long v = 0; v < V; ++v)
                        c->Spot[(it * 3 + m) * V + v] = Sold[(it * 3 + m) * V + v] + inv[it * V + v];
            }
        }
        if (c->p.precon_w > 0.0) {
            // each W (mu, nu) ([it][nu][mu]) with the symmetries of its class
            // (src/PotentialMixing.f90:169-210)
            const long V = c->V;
            for (int mu = 0; mu < 3; ++mu)
                for (int nu = 0; nu < 3; ++nu) {
                    int ss = S, comp = 2;
                    if (mu == nu) { ss = S; comp = 2; }
                    else if ((mu == 0 && nu == 1) || (mu == 1 && nu == 0)) { ss = S; comp = 1; }
                    else if ((mu == 0 && nu == 2) || (mu == 2 && nu == 0)) { ss = -S; comp = 2; }
                    else { ss = -S; comp = 1; }
                    std::vector<double> dw(2 * V);
                    for (int it = 0; it < 2; ++it)
                        for (long v = 0; v < V; ++v) {
                            const long q = ((it * 3 + nu) * 3 + mu) * V + v;
                            dw[it * V + v] = c->W[q] - Wold[q];
                        }
                    precondition_potential(c, dw, inv, -P, ss, TS, comp);
                    for (int it = 0; it < 2; ++it)
                        for (long v = 0; v < V; ++v) {
                            const long q = ((it * 3 + nu) * 3 + mu) * V + v;
                            c->W[q] = Wold[q] + inv[it * V + v];
                        }
                }
        }
    }
    return st;
}

extern "C" int orc_get_potentials(orc_ctx* c, double* u, double* b, double* nablab, double* w,
                                  double* divw, double* coul, double* coulex) {
    if (!c) return MG_ERR_ARG;
    auto cp = [](double* dst, const std::vector<double>& s) {
        if (dst) std::memcpy(dst, s.data(), s.size() * sizeof(double));
    };
    cp(u, c->U); cp(b, c->Bp); cp(nablab, c->nablaB); cp(w, c->W); cp(divw, c->divW);
    cp(coul, c->coulomb); cp(coulex, c->coulex);
    return MG_OK;
}
extern "C" int orc_set_potentials(orc_ctx* c, const double* u, const double* b,
                                  const double* nablab, const double* w, const double* divw) {
    if (!c) return MG_ERR_ARG;
    auto cp = [](std::vector<double>& d, const double* s) {
        if (s) std::memcpy(d.data(), s, d.size() * sizeof(double));
    };
    cp(c->U, u); cp(c->Bp, b); cp(c->nablaB, nablab); cp(c->W, w); cp(c->divW, divw);
    return MG_OK;
}

// --------------------------------------------------------------------------
// CompEnergy, src/Energy.f90:62-179: CompKinetic :1426-1456, compSkyrme
// :623-860 (TRC terms), CompCoulombEnergy / CompCoulombExchange
// src/Coulomb.f90:215-253, CompCOMCorrection src/Energy.f90:1608-1660,
// SpwfEnergy :1483-1554.
// --------------------------------------------------------------------------
extern "C" int orc_energy(orc_ctx* c, mg_energy_terms* out) {
    if (!c || !out) return MG_ERR_ARG;
    std::memset(out, 0, sizeof(*out));
    const long V = c->V;
    const mg_skyrme_b& B = c->B;
    const Basis& D = c->bas[c->p.pairing == MG_PAIRING_HFB ? MG_CAN_BASIS : MG_HF_BASIS];
    double kin[2] = {0, 0};
    for (int l = 0; l < c->p.nwt; ++l) {
        int it = (D.qn[4 * l] + 3) / 2 - 1;
        double ip = inprod_real(c, &D.psi[(long)l * 4 * V], &D.lap[(long)l * 4 * V]);
        kin[it] = kin[it] + D.occ[l] * ip;
    }
    for (int it = 0; it < 2; ++it) out->kinetic[it] = -kin[it] / 2.0 * c->f.hbm;
    double* t = out->skyrme;
    double s1 = 0, s2 = 0, s3 = 0, s4 = 0, s7 = 0, s8 = 0, s9 = 0, s10 = 0, s11 = 0, s12 = 0;
    double s33 = 0, s34 = 0;
    for (long v = 0; v < V; ++v) {
        double rt = c->rho[v] + c->rho[V + v];
        double tt = c->tau[v] + c->tau[V + v];
        double lt = c->laprho[v] + c->laprho[V + v];
        double jt = c->nablaj[v] + c->nablaj[V + v];
        s1 += rt * rt;
        s3 += rt * tt;
        s7 += rt * lt;
        s9 += std::pow(rt, 2 + B.byt3a);
        s11 += rt * jt;
        if (B.B7b != 0.0) s33 += std::pow(rt, 2 + B.byt3b);
    }
    for (int it = 0; it < 2; ++it) {
        double a2 = 0, a4 = 0, a8 = 0, a10 = 0, a12 = 0, a34 = 0;
        for (long v = 0; v < V; ++v) {
            double r = c->rho[it * V + v];
            double rt = c->rho[v] + c->rho[V + v];
            a2 += r * r;
            a4 += r * c->tau[it * V + v];
            a8 += r * c->laprho[it * V + v];
            a10 += r * r * std::pow(rt, B.byt3a);
            a12 += r * c->nablaj[it * V + v];
            if (B.B8b != 0.0) a34 += r * r * std::pow(rt, B.byt3b);
        }
        s2 += a2;
        s4 += B.B4 * a4;
        s8 += B.B6 * a8;
        s10 += B.B8a * a10;
        s12 += B.B9q * a12;
        s34 += B.B8b * a34;
    }
    if (!c->p.trc) {
        // time-odd terms 5, 6, 13-18, 35, 36 of compSkyrme (src/Energy.f90:623-860)
        double j2 = 0, jrs = 0, s2t = 0, s2a = 0, s2b = 0;
        double q6 = 0, q14 = 0, q16 = 0, q18 = 0, q36 = 0;
        for (int m = 0; m < 3; ++m)
            for (long v = 0; v < V; ++v) {
                const double jt = c->vecj[m * V + v] + c->vecj[(3 + m) * V + v];
                const double st = c->vecs[m * V + v] + c->vecs[(3 + m) * V + v];
                const double rs = c->rots[m * V + v] + c->rots[(3 + m) * V + v];
                const double rt = c->rho[v] + c->rho[V + v];
                j2 += jt * jt;
                jrs += jt * rs;
                s2t += st * st;
                s2a += std::pow(rt, B.byt3a) * (st * st);
                if (B.B12b != 0.0) s2b += std::pow(rt, B.byt3b) * (st * st);
            }
        for (int it = 0; it < 2; ++it) {
            double a6 = 0, a14 = 0, a16 = 0, a18 = 0, a36 = 0;
            for (int m = 0; m < 3; ++m)
                for (long v = 0; v < V; ++v) {
                    const long q = (it * 3 + m) * V + v;
                    const double rt = c->rho[v] + c->rho[V + v];
                    a6 += c->vecj[q] * c->vecj[q];
                    a14 += c->vecj[q] * c->rots[q];
                    a16 += c->vecs[q] * c->vecs[q];
                    a18 += std::pow(rt, B.byt3a) * (c->vecs[q] * c->vecs[q]);
                    if (B.B13b != 0.0) a36 += std::pow(rt, B.byt3b) * (c->vecs[q] * c->vecs[q]);
                }
            q6 = q6 - B.B4 * a6;
            q14 = q14 + B.B9q * a14;
            q16 = q16 + B.B11 * a16;
            q18 = q18 + B.B13a * a18;
            q36 = q36 + B.B13b * a36;
        }
        t[4] = -B.B3 * j2; t[5] = q6; t[12] = B.B9 * jrs; t[13] = q14;
        t[14] = B.B10 * s2t; t[15] = q16; t[16] = B.B12a * s2a; t[17] = q18;
        t[34] = B.B12b * s2b; t[35] = q36;
    }
    if (c->todd) {
        // time-odd tensor terms 21, 22, 27-32 of compSkyrme (src/Energy.f90:
        // 775-845); 31 and 32 square the divergence of s, which the
        // reference's density code never assigns (zero)
        double sT = 0, sF = 0, sL = 0, qT = 0, qF = 0, qL = 0;
        for (int m = 0; m < 3; ++m)
            for (long v = 0; v < V; ++v) {
                const double st = c->vecs[m * V + v] + c->vecs[(3 + m) * V + v];
                sT += st * (c->vecT[m * V + v] + c->vecT[(3 + m) * V + v]);
                sF += st * (c->vecF[m * V + v] + c->vecF[(3 + m) * V + v]);
                sL += st * (c->lapS[m * V + v] + c->lapS[(3 + m) * V + v]);
            }
        for (int it = 0; it < 2; ++it) {
            double aF = 0, aL = 0;
            for (int m = 0; m < 3; ++m)
                for (long v = 0; v < V; ++v) {
                    const long q = (it * 3 + m) * V + v;
                    qT += c->vecs[q] * c->vecT[q];
                    aF += c->vecs[q] * c->vecF[q];
                    aL += c->vecs[q] * c->lapS[q];
                }
            qF = qF - 2.0 * B.B17 * aF;
            qL = qL + B.B19 * aL;
        }
        t[20] = B.B14 != 0.0 ? -B.B14 * sT : 0.0;
        t[21] = B.B15 != 0.0 ? -B.B15 * qT : 0.0;
        t[26] = B.B16 != 0.0 ? -2.0 * B.B16 * sF : 0.0;
        t[27] = B.B17 != 0.0 ? qF : 0.0;
        t[28] = B.B18 != 0.0 ? B.B18 * sL : 0.0;
        t[29] = B.B19 != 0.0 ? qL : 0.0;
        t[30] = 0.0;
        t[31] = 0.0;
    }
    if (c->tensor) {
        // J^2 terms 19, 20, 23-26 of compSkyrme (src/Energy.f90:763-810)
        const double* J = c->jmunu.data();
        auto jm = [&](int it, int m, int n, long v) {
            return J[((it * 3 + n) * 3 + m) * V + v];
        };
        double s19 = 0, s20 = 0, s23 = 0, s24 = 0, s25 = 0, s26 = 0;
        for (long v = 0; v < V; ++v)
            for (int m = 0; m < 3; ++m)
                for (int n = 0; n < 3; ++n) {
                    const double jt = jm(0, m, n, v) + jm(1, m, n, v);
                    s19 += jt * jt;
                    s25 += jt * (jm(0, n, m, v) + jm(1, n, m, v));
                    for (int it = 0; it < 2; ++it) {
                        s20 += jm(it, m, n, v) * jm(it, m, n, v);
                        s26 += jm(it, m, n, v) * jm(it, n, m, v);
                    }
                }
        for (long v = 0; v < V; ++v) {
            double trt = 0.0;
            for (int it = 0; it < 2; ++it) {
                const double tr = jm(it, 0, 0, v) + jm(it, 1, 1, v) + jm(it, 2, 2, v);
                s24 += tr * tr;
                trt += tr;
            }
            s23 += trt * trt;
        }
        t[18] = B.B14 * s19; t[19] = B.B15 * s20; t[22] = B.B16 * s23;
        t[23] = B.B17 * s24; t[24] = B.B16 * s25; t[25] = B.B17 * s26;
    }
    t[0] = B.B1 * s1; t[1] = B.B2 * s2; t[2] = B.B3 * s3; t[3] = s4;
    t[6] = B.B5 * s7; t[7] = s8; t[8] = B.B7a * s9; t[9] = s10;
    t[10] = B.B9 * s11; t[11] = s12;
    t[32] = B.B7b * s33; t[33] = s34;
    for (int q = 0; q < 36; ++q) t[q] *= c->dv;
    double sk = 0;
    for (int q = 0; q < 36; ++q) sk += t[q];
    double ec = 0, ex = 0;
    if (c->p.coulomb_solver != 0) {
        for (long v = 0; v < V; ++v) ec += c->rho[V + v] * c->coulomb[v];
        ec = ec * c->dv * 0.5;
        if (c->f.cexchange >= 1) {
            double fac = -std::pow(3 / kPi, 1 / 3.0) * c->f.e2 * 0.75 * c->dv;
            for (long v = 0; v < V; ++v) ex += c->rho[V + v] * std::pow(c->rho[V + v], 1 / 3.0);
            ex = fac * ex;
        }
    }
    out->coulomb = ec;
    out->coulomb_exchange = ex;
    if (c->f.com1body > 0) {
        double mt = c->p.neutrons * c->f.nucleonmass[0] + c->p.protons * c->f.nucleonmass[1];
        for (int it = 0; it < 2; ++it) out->com[0][it] = -out->kinetic[it] * c->f.nucleonmass[it] / mt;
    }
    if (c->p.pairing == MG_PAIRING_HFB) {
        out->pairing[0] = c->epair[0];
        out->pairing[1] = c->epair[1];
    }
    double com = out->com[0][0] + out->com[1][0] + out->com[0][1] + out->com[1][1];
    out->total = sk + (out->kinetic[0] + out->kinetic[1]) + ec + com + ex +
                 (out->pairing[0] + out->pairing[1]);
    // OldEnergy shifts and takes the previous TotalEnergy (src/Energy.f90:93-98)
    for (int i = 6; i > 0; --i) c->old_energy[i] = c->old_energy[i - 1];
    c->old_energy[0] = c->total_energy;
    c->total_energy = out->total;
    // SpwfEnergy (TermByTerm)
    double sp = 0;
    for (int i = 0; i < c->p.nwt; ++i) sp += D.occ[i] * D.e[i];
    sp = 0.5 * (sp + (out->kinetic[0] + out->kinetic[1])) -
         0.5 * B.byt3a * ((t[8] + t[9]) + (t[16] + t[17])) -
         0.5 * B.byt3b * ((t[32] + t[33]) + (t[34] + t[35])) + ex / 3.0;
    sp = sp + (out->pairing[0] + out->pairing[1]);
    if (c->f.com1body > 0) sp = sp + (out->com[0][0] + out->com[0][1]) / 2.0;
    if (c->f.com2body == 1) sp = sp + (out->com[1][0] + out->com[1][1]);
    out->sp_energy = sp;
    return MG_OK;
}

// --------------------------------------------------------------------------
// Symmetric eigensolver: Householder tridiagonalisation followed by implicit
// QL with eigenvector accumulation (the published tred2 / tql2 algorithm of
// Martin, Reinsch and Wilkinson that diagoncr8, src/HFB.f90:5880-6087, also
// implements), eigenvalues sorted ascending with their vectors.
// a: n*n row-major symmetric input; w: eigenvalues; z: n*n, column k = vector k.
// --------------------------------------------------------------------------
// Host threads of the OpenMP build (the timing build of the CPU baseline);
// returns the count in use, 1 in the parity build (compiled without OpenMP).
extern "C" int orc_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
#else
    (void)n;
    return 1;
#endif
}

extern "C" int orc_eigh(int n, const double* a_in, double* w, double* z) {
    if (n <= 0) return MG_ERR_ARG;
    std::vector<double> A(a_in, a_in + (size_t)n * n), d(n), e(n);
    auto a = [&](int i, int j) -> double& { return A[(size_t)i * n + j]; };
    for (int i = n - 1; i > 0; --i) {
        const int l = i - 1;
        double h = 0.0, scale = 0.0;
        if (l > 0) {
            for (int k = 0; k <= l; ++k) scale += std::fabs(a(i, k));
            if (scale == 0.0) {
                e[i] = a(i, l);
            } else {
                for (int k = 0; k <= l; ++k) { a(i, k) /= scale; h += a(i, k) * a(i, k); }
                double f = a(i, l);
                double g = f >= 0.0 ? -std::sqrt(h) : std::sqrt(h);
                e[i] = scale * g;
                h -= f * g;
                a(i, l) = f - g;
                f = 0.0;
                for (int j = 0; j <= l; ++j) {
                    a(j, i) = a(i, j) / h;
                    g = 0.0;
                    for (int k = 0; k <= j; ++k) g += a(j, k) * a(i, k);
                    for (int k = j + 1; k <= l; ++k) g += a(k, j) * a(i, k);
                    e[j] = g / h;
                    f += e[j] * a(i, j);
                }
                const double hh = f / (h + h);
                for (int j = 0; j <= l; ++j) {
                    f = a(i, j);
                    e[j] = g = e[j] - hh * f;
                    for (int k = 0; k <= j; ++k) a(j, k) -= (f * e[k] + g * a(i, k));
                }
            }
        } else {
            e[i] = a(i, l);
        }
        d[i] = h;
    }
    d[0] = 0.0;
    e[0] = 0.0;
    for (int i = 0; i < n; ++i) {
        const int l = i - 1;
        if (d[i] != 0.0) {
            for (int j = 0; j <= l; ++j) {
                double g = 0.0;
                for (int k = 0; k <= l; ++k) g += a(i, k) * a(k, j);
                for (int k = 0; k <= l; ++k) a(k, j) -= g * a(k, i);
            }
        }
        d[i] = a(i, i);
        a(i, i) = 1.0;
        for (int j = 0; j <= l; ++j) a(j, i) = a(i, j) = 0.0;
    }
    for (int i = 1; i < n; ++i) e[i - 1] = e[i];
    e[n - 1] = 0.0;
    for (int l = 0; l < n; ++l) {
        int iter = 0, m;
        do {
            for (m = l; m < n - 1; ++m) {
                const double dd = std::fabs(d[m]) + std::fabs(d[m + 1]);
                if (std::fabs(e[m]) <= 2.2e-16 * dd) break;
            }
            if (m != l) {
                if (iter++ == 60) return MG_NOT_CONVERGED;
                double g = (d[l + 1] - d[l]) / (2.0 * e[l]);
                double r = std::hypot(g, 1.0);
                g = d[m] - d[l] + e[l] / (g + (g >= 0.0 ? std::fabs(r) : -std::fabs(r)));
                double s = 1.0, c = 1.0, p = 0.0;
                int i;
                for (i = m - 1; i >= l; --i) {
                    double f = s * e[i], b = c * e[i];
                    e[i + 1] = (r = std::hypot(f, g));
                    if (r == 0.0) {
                        d[i + 1] -= p;
                        e[m] = 0.0;
                        break;
                    }
                    s = f / r;
                    c = g / r;
                    g = d[i + 1] - p;
                    r = (d[i] - g) * s + 2.0 * c * b;
                    d[i + 1] = g + (p = s * r);
                    g = c * r - b;
                    for (int k = 0; k < n; ++k) {
                        f = a(k, i + 1);
                        a(k, i + 1) = s * a(k, i) + c * f;
                        a(k, i) = c * a(k, i) - s * f;
                    }
                }
                if (r == 0.0 && i >= l) continue;
                d[l] -= p;
                e[l] = g;
                e[m] = 0.0;
            }
        } while (m != l);
    }
    // selection sort ascending, as the last loop of diagoncr8
    for (int i = 0; i < n - 1; ++i) {
        int k = i;
        double p = d[i];
        for (int j = i + 1; j < n; ++j)
            if (d[j] < p) { k = j; p = d[j]; }
        if (k != i) {
            d[k] = d[i];
            d[i] = p;
            for (int j = 0; j < n; ++j) std::swap(a(j, i), a(j, k));
        }
    }
    std::copy(d.begin(), d.end(), w);
    std::copy(A.begin(), A.end(), z);
    return MG_OK;
}

// --------------------------------------------------------------------------
// HFB pairing step (PairingType 2, FermiSolver 'BROYDEN', PairingIter 1,
// no Lipkin-Nogami, no blocking, ULB density-dependent delta pairing).
// --------------------------------------------------------------------------
static const double kHFBNumCut = 1e-12;  // src/HFB.f90:46

extern "C" int orc_set_pairing(orc_ctx* c, const mg_pairing_params* pp) {
    if (!c || !pp || c->p.pairing != MG_PAIRING_HFB || !c->p.trc || !c->folded) return MG_ERR_ARG;
    c->pp = *pp;
    c->fermi[0] = pp->fermi_start[0];
    c->fermi[1] = pp->fermi_start[1];
    return MG_OK;
}

// PrepareHFBModule, src/HFB.f90:245-292
static void hfb_prepare(orc_ctx* c) {
    const Basis& B = c->bas[MG_HF_BASIS];
    const int nwt = c->p.nwt;
    for (int b = 0; b < 4; ++b) c->bidx[b].clear();
    for (int i = 0; i < 2 * nwt; ++i) {
        const int ii = i % nwt;
        const int P = (B.qn[4 * ii + 1] + 1) / 2, it = (B.qn[4 * ii] + 3) / 2 - 1;
        c->bidx[it * 2 + P].push_back(i);
    }
    for (int b = 0; b < 4; ++b) {
        const size_t N = c->bidx[b].size();
        for (auto* v : {&c->rho_h[b], &c->kappa_h[b], &c->oldrho[b], &c->oldkappa[b], &c->delta[b],
                        &c->cantr[b]})
            v->assign(N * N, 0.0);
        c->Um[b].assign(N * 2 * N, 0.0);
        c->Vm[b].assign(N * 2 * N, 0.0);
        c->qe[b].assign(2 * N, 0.0);
        c->occs[b].assign(N, 0.0);
    }
    c->pcut.assign(nwt, 0.0);
    c->dfac.assign(2 * c->V, 0.0);
    c->pf_re.assign(2 * c->V, 0.0);
    c->pf_im.assign(2 * c->V, 0.0);
    c->hfb_ready = true;
}

// sig of HFB index i (time-reversed partner flips the signature)
static int hfb_sig(const orc_ctx* c, int i) {
    const int nwt = c->p.nwt;
    const int s = c->bas[MG_HF_BASIS].qn[4 * (i % nwt) + 2];
    return i >= nwt ? -s : s;
}

// ComputePairingCutoffs + SymmetricFermi, src/PairingInteraction.f90:182-228
static void pairing_cutoffs(orc_ctx* c, const double* lambda) {
    const Basis& B = c->bas[MG_HF_BASIS];
    for (int i = 0; i < c->p.nwt; ++i) {
        const int it = (B.qn[4 * i] + 3) / 2 - 1;
        const double E = B.e[i];
        const double up = (E - lambda[it] - c->pp.cut[it]) / c->pp.mu[it];
        const double down = -(E - lambda[it] + c->pp.cut[it]) / c->pp.mu[it];
        double f = std::sqrt(std::sqrt(1.0 / (1.0 + std::exp(up))));
        f = f * std::sqrt(std::sqrt(1.0 / (1.0 + std::exp(down))));
        c->pcut[i] = f;
    }
}

// GetPairDensity, src/PairingInteraction.f90:101-180, at one point
static inline void pair_density(const double* l, const double* r, bool tr, double& re, double& im) {
    if (!tr) {
        re = l[0] * r[2] - l[1] * r[3] - l[2] * r[0] + l[3] * r[1];
        im = l[0] * r[3] + l[1] * r[2] - l[2] * r[1] - l[3] * r[0];
    } else {
        re = -l[0] * r[0] - l[1] * r[1] - l[2] * r[2] - l[3] * r[3];
        im = l[0] * r[1] - l[1] * r[0] + l[2] * r[3] - l[3] * r[2];
    }
}

// HFBPairingField, src/HFB.f90:350-518 (no LN), with CompDensityFactor (ULB)
static void pairing_field(orc_ctx* c) {
    const long V = c->V;
    const int nwt = c->p.nwt;
    const Basis& B = c->bas[MG_HF_BASIS];
    for (int it = 0; it < 2; ++it)
        for (long v = 0; v < V; ++v) {
            const double rho0 = c->rho[v] + c->rho[V + v];
            c->dfac[it * V + v] = -c->pp.strength[it] * (1.0 - c->pp.alpha[it] / c->pp.rhosat * rho0);
        }
    std::fill(c->pf_re.begin(), c->pf_re.end(), 0.0);
    std::fill(c->pf_im.begin(), c->pf_im.end(), 0.0);
    for (int b = 0; b < 4; ++b) {
        const int it = b / 2;
        const auto& idx = c->bidx[b];
        const int N = (int)idx.size();
        for (int j = 0; j < N; ++j) {
            const int jj = idx[j], jjj = jj % nwt;
            const int sig1 = hfb_sig(c, jj);
            const double c1 = c->pcut[jjj];
            if (c1 < kHFBNumCut) continue;
            for (int i = j + 1; i < N; ++i) {
                const int ii = idx[i], iii = ii % nwt;
                const int sig2 = hfb_sig(c, ii);
                if (sig1 != -sig2) continue;
                const double c2 = c->pcut[iii];
                const double kij = c->kappa_h[b][(size_t)i * N + j];
                if (c1 * c2 * std::fabs(kij) < kHFBNumCut) continue;
                const bool tr = (ii >= nwt || jj >= nwt) && !(ii >= nwt && jj >= nwt);
                const double factor = c1 * c2 * kij;
                const double* pl = &B.psi[(long)jjj * 4 * V];
                const double* pr = &B.psi[(long)iii * 4 * V];
#pragma omp parallel for schedule(static)
                for (long v = 0; v < V; ++v) {
                    const double l[4] = {pl[v], pl[V + v], pl[2 * V + v], pl[3 * V + v]};
                    const double r[4] = {pr[v], pr[V + v], pr[2 * V + v], pr[3 * V + v]};
                    double re, im;
                    pair_density(l, r, tr, re, im);
                    c->pf_re[it * V + v] = c->pf_re[it * V + v] - factor * re;
                    c->pf_im[it * V + v] = c->pf_im[it * V + v] - factor * im;
                }
            }
        }
    }
    for (int it = 0; it < 2; ++it)
        for (long v = 0; v < V; ++v) {
            c->pf_re[it * V + v] = c->pf_re[it * V + v] * c->dfac[it * V + v] * 1.0;
            c->pf_im[it * V + v] = c->pf_im[it * V + v] * c->dfac[it * V + v] * 1.0;
        }
}

// HFBGaps, src/HFB.f90:520-632
static void pairing_gaps(orc_ctx* c) {
    const long V = c->V;
    const int nwt = c->p.nwt;
    const Basis& B = c->bas[MG_HF_BASIS];
    for (int b = 0; b < 4; ++b) {
        const int it = b / 2;
        const auto& idx = c->bidx[b];
        const int N = (int)idx.size();
        std::fill(c->delta[b].begin(), c->delta[b].end(), 0.0);
#pragma omp parallel for schedule(dynamic, 1)
        for (int i = 0; i < N; ++i) {
            const int ii = idx[i], iii = ii % nwt;
            const int sig1 = hfb_sig(c, ii);
            const double c1 = c->pcut[iii];
            for (int j = i + 1; j < N; ++j) {
                const int jj = idx[j], jjj = jj % nwt;
                const int sig2 = hfb_sig(c, jj);
                if (sig1 != -sig2) continue;
                const double c2 = c->pcut[jjj];
                if (c1 * c2 < kHFBNumCut) continue;
                const bool tr = (ii >= nwt || jj >= nwt) && !(ii >= nwt && jj >= nwt);
                const double* pl = &B.psi[(long)iii * 4 * V];
                const double* pr = &B.psi[(long)jjj * 4 * V];
                double s1 = 0.0, s2 = 0.0;
                for (long v = 0; v < V; ++v) {
                    const double l[4] = {pl[v], pl[V + v], pl[2 * V + v], pl[3 * V + v]};
                    const double r[4] = {pr[v], pr[V + v], pr[2 * V + v], pr[3 * V + v]};
                    double re, im;
                    pair_density(l, r, tr, re, im);
                    s1 += re * c->pf_re[it * V + v];
                    s2 += im * c->pf_im[it * V + v];
                }
                const double d = c->dv * c1 * c2 * (s1 + s2);
                c->delta[b][(size_t)i * N + j] = d;
                c->delta[b][(size_t)j * N + i] = -d;
            }
        }
    }
}

// HFBNumberofParticles_ordinary (PfSolver off, SC conserved: the CR8 column
// choice), with ConstructHFBHamiltonian, DiagonaliseHFBHamiltonian_Signature,
// constructRhoHFB and ConstructKappaHFB (src/HFB.f90:810-1072, :2554-2786,
// :3128-3154, :3335-3359).  Returns Tr rho per isospin.
static int hfb_number(orc_ctx* c, const double* lambda, double* Nout) {
    const Basis& B = c->bas[MG_HF_BASIS];
    const int nwt = c->p.nwt;
    Nout[0] = Nout[1] = 0.0;
    for (int b = 0; b < 4; ++b) {
        const int it = b / 2;
        const auto& idx = c->bidx[b];
        const int N = (int)idx.size(), h = N / 2;
        if (N == 0) continue;
        std::vector<double> T((size_t)N * N, 0.0), w(N), X((size_t)N * N);
        for (int j = 0; j < h; ++j)
            for (int i = 0; i < h; ++i) {
                const double hij = (i == j) ? B.e[idx[i] % nwt] - lambda[it] : 0.0;
                const double hr = (i == j) ? -(B.e[idx[i + h] % nwt] - lambda[it]) : 0.0;
                T[(size_t)i * N + j] = hij;
                T[(size_t)j * N + i] = hij;
                T[(size_t)(i + h) * N + j + h] = hr;
                T[(size_t)(j + h) * N + i + h] = hr;
                const double dd = c->delta[b][(size_t)i * N + j + h];
                T[(size_t)i * N + j + h] = dd;
                T[(size_t)(j + h) * N + i] = dd;
            }
        if (orc_eigh(N, T.data(), w.data(), X.data()) != MG_OK) return MG_NOT_CONVERGED;
        std::vector<double>& U = c->Um[b];
        std::vector<double>& Vv = c->Vm[b];
        std::fill(U.begin(), U.end(), 0.0);
        std::fill(Vv.begin(), Vv.end(), 0.0);
        const int N2 = 2 * N;
        for (int k = 0; k < N; ++k) {
            for (int r = 0; r < h; ++r) {
                U[(size_t)r * N2 + k] = X[(size_t)r * N + k];
                Vv[(size_t)(h + r) * N2 + k] = X[(size_t)(h + r) * N + k];
                U[(size_t)(h + r) * N2 + N + k] = -X[(size_t)r * N + k];
                Vv[(size_t)r * N2 + N + k] = X[(size_t)(h + r) * N + k];
            }
            c->qe[b][k] = w[k];
            c->qe[b][N + k] = w[k];
        }
        std::vector<int> cols(N);
        for (int i = 0; i < h; ++i) cols[i] = 2 * N - 1 - i;
        for (int i = h; i < N; ++i) cols[i] = i;
        for (int j = 0; j < N; ++j)
            for (int i = 0; i < N; ++i) {
                double s = 0.0;
                for (int k = 0; k < N; ++k) s += Vv[(size_t)i * N2 + cols[k]] * Vv[(size_t)j * N2 + cols[k]];
                c->rho_h[b][(size_t)i * N + j] = s;
            }
        for (int j = 0; j < N; ++j)
            for (int i = j + 1; i < N; ++i) {
                double s = 0.0;
                for (int k = 0; k < N; ++k) s += Vv[(size_t)i * N2 + cols[k]] * U[(size_t)j * N2 + cols[k]];
                c->kappa_h[b][(size_t)i * N + j] = s;
                c->kappa_h[b][(size_t)j * N + i] = -s;
            }
        for (int i = 0; i < N; ++i) Nout[it] += c->rho_h[b][(size_t)i * N + i];
    }
    return MG_OK;
}

// HFBFindFermiEnergyBroyden, src/HFB.f90:1849-2161 (no LN, no dispersion
// constraint): damped (step 0.5) Broyden on N(lambda) - N0 per isospin.
static int fermi_broyden(orc_ctx* c, int* evals) {
    const double part[2] = {c->p.neutrons, c->p.protons};
    const double prec = c->pp.fermi_prec;
    double hist[2] = {c->fermi[0] + 0.01, c->fermi[1] + 0.01};
    bool conv[2] = {false, false};
    double N[2], NX[2], J[2], upd[2] = {0, 0}, norm[2] = {1, 1};
    int ne = 0, st;
    if ((st = hfb_number(c, c->fermi, N)) != MG_OK) return st;
    ++ne;
    for (int it = 0; it < 2; ++it) {
        N[it] -= part[it];
        if (std::fabs(N[it]) < prec) conv[it] = true;
    }
    if ((st = hfb_number(c, hist, NX)) != MG_OK) return st;
    ++ne;
    for (int it = 0; it < 2; ++it) {
        NX[it] -= part[it];
        J[it] = (N[it] - NX[it]) / (c->fermi[it] - hist[it]);
    }
    const double step = 0.5;
    for (int iter = 1; iter <= c->pp.max_iter; ++iter) {
        double invJ[2];
        for (int it = 0; it < 2; ++it)
            invJ[it] = std::fabs(J[it]) < 0.001 ? (J[it] >= 0 ? 0.99 : -0.99) : 1.0 / J[it];
        for (int it = 0; it < 2; ++it) {
            if (conv[it]) continue;
            upd[it] = -invJ[it] * N[it];
            norm[it] = upd[it] * upd[it];
        }
        for (int it = 0; it < 2; ++it) upd[it] = step * upd[it];
        for (int it = 0; it < 2; ++it) {
            if (conv[it]) continue;
            hist[it] = c->fermi[it];
            c->fermi[it] = c->fermi[it] + upd[it];
        }
        if ((st = hfb_number(c, c->fermi, N)) != MG_OK) return st;
        ++ne;
        for (int it = 0; it < 2; ++it) {
            N[it] -= part[it];
            if (std::fabs(N[it]) < prec) conv[it] = true;
        }
        if (conv[0] && conv[1]) break;
        if (iter > 1)
            for (int it = 0; it < 2; ++it) {
                if (conv[it]) continue;
                J[it] = J[it] + N[it] * upd[it] / norm[it];
            }
        for (int it = 0; it < 2; ++it)
            if (std::isnan(N[it])) return MG_ERR_NAN;
    }
    for (int i = 0; i < 6; ++i) c->fermi_hist[i] = c->fermi_hist[i + 1];
    c->fermi_hist[6] = std::fabs(N[0]) > 0.9 || std::fabs(N[1]) > 0.9;
    bool lost = true;
    for (int i = 0; i < 7; ++i) lost = lost && c->fermi_hist[i];
    if (evals) *evals = ne;
    if (lost) return MG_ERR_STATE;
    return (conv[0] && conv[1]) ? MG_OK : MG_NOT_CONVERGED;
}

// FermiBrent, src/HFB.f90:2273-2487: Brent's method per isospin on
// N(lambda) - N0 from the bracket [a, b] (a == b: nothing to search), both
// isospins evaluated together at b, tolerance prec on lambda.
static int fermi_brent(orc_ctx* c, double a[2], double b[2], double fa[2], double fb[2],
                       double prec, bool found[2], int* ne) {
    const double part[2] = {c->p.neutrons, c->p.protons};
    double cc[2], fc[2], d[2] = {0, 0}, e[2] = {0, 0}, N[2];
    for (int it = 0; it < 2; ++it) {
        found[it] = a[it] == b[it];
        if (!found[it] && fa[it] * fb[it] > 0.0) return MG_ERR_STATE;
        cc[it] = b[it];
        fc[it] = fb[it];
    }
    for (int iter = 0; iter < 100000 && !(found[0] && found[1]); ++iter) {
        for (int it = 0; it < 2; ++it) {
            if (found[it]) continue;
            if ((fb[it] > 0.0 && fc[it] > 0.0) || (fb[it] < 0.0 && fc[it] < 0.0)) {
                cc[it] = a[it];
                fc[it] = fa[it];
                d[it] = b[it] - a[it];
                e[it] = d[it];
            }
            if (std::fabs(fc[it]) < std::fabs(fb[it])) {
                a[it] = b[it]; fa[it] = fb[it];
                b[it] = cc[it]; fb[it] = fc[it];
                cc[it] = a[it]; fc[it] = fa[it];
            }
            const double tol = prec, xm = 0.5 * (cc[it] - b[it]);
            if (std::fabs(xm) <= tol) {
                found[it] = true;
                continue;
            }
            if (std::fabs(e[it]) >= tol && std::fabs(fa[it]) > std::fabs(fb[it])) {
                const double sv = fb[it] / fa[it];
                double p, q;
                if (a[it] == cc[it]) {
                    p = 2.0 * xm * sv;
                    q = 1.0 - sv;
                } else {
                    const double qa = fa[it] / fc[it], r = fb[it] / fc[it];
                    p = sv * (2.0 * xm * qa * (qa - r) - (b[it] - a[it]) * (r - 1.0));
                    q = (qa - 1.0) * (r - 1.0) * (sv - 1.0);
                }
                if (p > 0.0) q = -q;
                p = std::fabs(p);
                if (2.0 * p < std::min(3.0 * xm * q - std::fabs(tol * q), std::fabs(e[it] * q))) {
                    e[it] = d[it];
                    d[it] = p / q;
                } else {
                    d[it] = xm;
                    e[it] = d[it];
                }
            } else {
                d[it] = xm;
                e[it] = d[it];
            }
            a[it] = b[it];
            fa[it] = fb[it];
            b[it] = b[it] + (std::fabs(d[it]) > tol ? d[it] : std::copysign(tol, xm));
        }
        int st;
        if ((st = hfb_number(c, b, N)) != MG_OK) return st;
        ++*ne;
        for (int it = 0; it < 2; ++it) fb[it] = N[it] - part[it];
    }
    return MG_OK;
}

// HFBFindFermiEnergyBisection, src/HFB.f90:1074-1342 (no LN; the emergency
// handling is off in the reference): bracket the root by stepping the
// boundary on its side out by 0.01 MeV times the attempt, then FermiBrent.
static int fermi_bisection(orc_ctx* c, int* evals) {
    const double part[2] = {c->p.neutrons, c->p.protons};
    const double prec = c->pp.fermi_prec;
    int ne = 0, st;
    double N[2];
    for (int it = 0; it < 2; ++it)
        if (part[it] < 0.1) c->fermi[it] = -100.0;
    if ((st = hfb_number(c, c->fermi, N)) != MG_OK) return st;
    ++ne;
    for (int it = 0; it < 2; ++it) N[it] -= part[it];
    bool conv[2] = {std::fabs(N[0]) < prec, std::fabs(N[1]) < prec};
    if (!(conv[0] && conv[1])) {
        double br[2][2], fa[2], fb[2], X[2];
        int idir[2], sig[2];
        bool notfound[2] = {true, true};
        for (int it = 0; it < 2; ++it) {
            br[0][it] = br[1][it] = c->fermi[it];
            idir[it] = N[it] < 0.0 ? 1 : 0;
            sig[it] = N[it] < 0.0 ? 1 : -1;
        }
        for (int fail = 0;; ++fail) {
            for (int it = 0; it < 2; ++it)
                if (std::fabs(N[it]) < prec) notfound[it] = false;
            for (int it = 0; it < 2; ++it)
                if (notfound[it]) br[idir[it]][it] = br[idir[it]][it] + sig[it] * 0.01 * (fail + 1);
            if ((st = hfb_number(c, br[0], X)) != MG_OK) return st;
            for (int it = 0; it < 2; ++it) fa[it] = X[it] - part[it];
            if ((st = hfb_number(c, br[1], X)) != MG_OK) return st;
            for (int it = 0; it < 2; ++it) fb[it] = X[it] - part[it];
            ne += 2;
            for (int it = 0; it < 2; ++it)
                if (notfound[it] && fa[it] * fb[it] <= 0.0) notfound[it] = false;
            if (!notfound[0] && !notfound[1]) break;
            if (fail + 1 > 130) return MG_ERR_STATE;
            for (int it = 0; it < 2; ++it)
                if (notfound[it]) br[1 - idir[it]][it] = br[idir[it]][it];
        }
        bool found[2];
        if ((st = fermi_brent(c, br[0], br[1], fa, fb, prec, found, &ne)) != MG_OK) return st;
        for (int it = 0; it < 2; ++it) {
            c->fermi[it] = br[1][it];
            N[it] = fb[it];
            conv[it] = found[it];
        }
    }
    for (int i = 0; i < 6; ++i) c->fermi_hist[i] = c->fermi_hist[i + 1];
    c->fermi_hist[6] = std::fabs(N[0]) > 0.9 || std::fabs(N[1]) > 0.9;
    bool lost = true;
    for (int i = 0; i < 7; ++i) lost = lost && c->fermi_hist[i];
    if (evals) *evals = ne;
    if (lost) return MG_ERR_STATE;
    return (conv[0] && conv[1]) ? MG_OK : MG_NOT_CONVERGED;
}

// DiagonaliseRhoHFB + HFBOccupations, src/HFB.f90:3156-3284, :3361-3560:
// canonical basis from the eigenvectors of rho, occupations, rho / kappa mixing.
static int hfb_occupations(orc_ctx* c) {
    const int nwt = c->p.nwt;
    const long V4 = 4 * c->V;
    Basis& H = c->bas[MG_HF_BASIS];
    Basis& C = c->bas[MG_CAN_BASIS];
    std::fill(C.psi.begin(), C.psi.end(), 0.0);
    c->pdisp[0] = c->pdisp[1] = 0.0;
    int index = 0;
    for (int b = 0; b < 4; ++b) {
        const int it = b / 2;
        const auto& idx = c->bidx[b];
        const int N = (int)idx.size(), h = N / 2;
        if (N == 0) continue;
        std::vector<double> T(c->rho_h[b]), w(N), X((size_t)N * N);
        for (int i = 0; i < N; ++i)
            if (idx[i] >= nwt || hfb_sig(c, idx[i]) == -1) T[(size_t)i * N + i] -= 2.0;
        if (orc_eigh(N, T.data(), w.data(), X.data()) != MG_OK) return MG_NOT_CONVERGED;
        for (int k = 0; k < N; ++k) {
            double o = w[k];
            if (o < -0.1) o += 2.0;
            if (o < 0.0) o = 0.0;
            if (o > 1.0) o = 1.0;
            c->occs[b][k] = 2.0 * o;
        }
        for (size_t q = 0; q < X.size(); ++q)
            if (std::fabs(X[q]) < 1e-11) X[q] = 0.0;
        c->cantr[b] = X;
        for (int col = 0; col < N; ++col) {
            bool neg = false;
            for (int r = h; r < N; ++r) neg = neg || std::fabs(X[(size_t)r * N + col]) > kHFBNumCut;
            if (neg) continue;
            if (index >= nwt) return MG_ERR_STATE;
            int loc = 0;
            for (int r = 1; r < N; ++r)
                if (std::fabs(X[(size_t)r * N + col]) > std::fabs(X[(size_t)loc * N + col])) loc = r;
            const int dom = idx[loc] % nwt;
            C.qn[4 * index + 0] = 2 * it - 1;
            C.qn[4 * index + 1] = H.qn[4 * dom + 1];
            C.qn[4 * index + 2] = hfb_sig(c, idx[loc]);
            C.qn[4 * index + 3] = H.qn[4 * dom + 3];
            double* out = &C.psi[(long)index * V4];
            for (int r = 0; r < N; ++r) {
                const double ct = X[(size_t)r * N + col];
                if (std::fabs(ct) < kHFBNumCut) continue;
                const double* src = &H.psi[(long)(idx[r] % nwt) * V4];
                for (long q = 0; q < V4; ++q) out[q] = out[q] + ct * src[q];
            }
            const double o = c->occs[b][col];
            c->pdisp[it] += o * (2.0 - o);
            C.occ[index] = o;
            ++index;
        }
    }
    if (index != nwt) return MG_ERR_STATE;
    bool oldzero = true, kzero = true;
    for (int b = 0; b < 4; ++b) {
        for (double x : c->oldrho[b]) oldzero = oldzero && x == 0.0;
        for (double x : c->kappa_h[b]) kzero = kzero && x == 0.0;
    }
    const double m = c->pp.mix;
    for (int b = 0; b < 4; ++b) {
        if (!oldzero)
            for (size_t q = 0; q < c->rho_h[b].size(); ++q)
                c->rho_h[b][q] = m * c->rho_h[b][q] + (1.0 - m) * c->oldrho[b][q];
        if (!kzero)
            for (size_t q = 0; q < c->kappa_h[b].size(); ++q)
                c->kappa_h[b][q] = m * c->kappa_h[b][q] + (1.0 - m) * c->oldkappa[b][q];
        c->oldrho[b] = c->rho_h[b];
        c->oldkappa[b] = c->kappa_h[b];
    }
    return MG_OK;
}

// GuessHFBMatrices case(2), src/HFB.f90:3645-3835, time-reversal conserved:
// every stored spwf is paired with its own time-reversed partner.
static void guess_kappa(orc_ctx* c) {
    for (int b = 0; b < 4; ++b) {
        const int N = (int)c->bidx[b].size(), h = N / 2;
        std::fill(c->kappa_h[b].begin(), c->kappa_h[b].end(), 0.0);
        for (int i = 0; i < h; ++i) {
            c->kappa_h[b][(size_t)i * N + i + h] = -0.25;
            c->kappa_h[b][(size_t)(i + h) * N + i] = 0.25;
        }
    }
}

// HFBEnergy, src/HFB.f90:296-348
static void hfb_energy(orc_ctx* c) {
    c->epair[0] = c->epair[1] = 0.0;
    for (int b = 0; b < 4; ++b) {
        const int it = b / 2;
        const size_t n = c->delta[b].size();
        double e = 0.0;
        for (size_t q = 0; q < n; ++q) e = e - c->delta[b][q] * c->kappa_h[b][q];
        c->epair[it] += e;
    }
    c->epair[0] *= -0.5;
    c->epair[1] *= -0.5;
}

// SolvePairing, src/Pairing.f90:743-890
// --------------------------------------------------------------------------
// HFBFermiGradient, src/GradientHFB.f90:473-733 (FermiSolver 'GRADIENT',
// signature conserved: H20_sig :1014-1068, N20 :1070-1108, GradUpdate_sig
// :884-920, ortho_sig :1148-1222; HFBReduce off, no blocking, no
// Lipkin-Nogami, FermiMomentum off so step = 0.020 and mu = 0).  The U and V
// it starts from are GetUandV's (:108-186): the module's U and V, which the
// reference has from an earlier diagonalisation or a restart file; here the
// first call takes them from one diagonalisation at the Fermi energies the
// step starts from (hfb_number).  Later calls continue from the solver's own
// GradU, GradV.  Matrices are N x N row-major, 0-based.
// --------------------------------------------------------------------------
static void ghfb_matmul(const double* A, int lda, const double* B, int ldb, double* C, int ldc,
                        int m, int n, int k, bool ta) {
    // C(m x n) = op(A) B with op(A) = A or A^T, sums in index order
    for (int i = 0; i < m; ++i)
        for (int j = 0; j < n; ++j) {
            double x = 0.0;
            for (int q = 0; q < k; ++q)
                x += (ta ? A[(size_t)q * lda + i] : A[(size_t)i * lda + q]) * B[(size_t)q * ldb + j];
            C[(size_t)i * ldc + j] = x;
        }
}

static int fermi_gradient(orc_ctx* c, int* iters_out) {
    const Basis& B = c->bas[MG_HF_BASIS];
    const int nwt = c->p.nwt;
    if (!c->ghfb_ready) {
        double Nt[2];
        const int st = hfb_number(c, c->fermi, Nt);
        if (st != MG_OK) return st;
        for (int b = 0; b < 4; ++b) {
            const int N = (int)c->bidx[b].size(), h = N / 2, N2 = 2 * N;
            c->GU[b].assign((size_t)N * N, 0.0);
            c->GV[b].assign((size_t)N * N, 0.0);
            // the CR8 columns h..N-1 and 2N-h..2N-1, in increasing order
            int ind = 0;
            for (int j = 0; j < N2; ++j) {
                const bool in = (j >= h && j < N) || j >= N2 - h;
                if (!in) continue;
                for (int i = 0; i < N; ++i) {
                    c->GU[b][(size_t)i * N + ind] = c->Um[b][(size_t)i * N2 + j];
                    c->GV[b][(size_t)i * N + ind] = c->Vm[b][(size_t)i * N2 + j];
                }
                bool sig = false;
                for (int i = 0; i < h; ++i) sig = sig || std::fabs(c->GU[b][(size_t)i * N + ind]) > 1e-10;
                for (int i = h; i < N; ++i) sig = sig || std::fabs(c->GV[b][(size_t)i * N + ind]) > 1e-10;
                if (sig) ++c->gsig[b];
                ++ind;
            }
        }
        c->ghfb_ready = true;
    }
    const double prec = c->pp.fermi_prec;
    const int maxit = c->pp.max_iter > 0 ? c->pp.max_iter : 500;
    const double particles[2] = {c->p.neutrons, c->p.protons};
    const double step = 0.020;
    bool conv[2] = {false, false};
    double n20norm[2] = {0.0, 0.0}, par[2] = {0.0, 0.0};
    std::vector<double> grad[4], an20[4];
    double gnorm[4] = {0.0, 0.0, 0.0, 0.0};
    int iter = 0;
    for (iter = 1; iter <= maxit; ++iter) {
        for (int it = 0; it < 2; ++it) {
            if (conv[it]) continue;
            n20norm[it] = 0.0;
            for (int b = 2 * it; b < 2 * it + 2; ++b) {
                const int N = (int)c->bidx[b].size(), h = N / 2, S = c->gsig[b];
                const std::vector<double>& U = c->GU[b];
                const std::vector<double>& V = c->GV[b];
                const std::vector<double>& D = c->delta[b];
                std::vector<double> e(N);
                for (int i = 0; i < N; ++i) e[i] = B.e[c->bidx[b][i] % nwt];
                // H20_sig: hU, hV, DsV, DsU (only the halves the formula reads)
                std::vector<double> hU((size_t)N * N, 0.0), hV((size_t)N * N, 0.0),
                    DsV((size_t)N * N, 0.0), DsU((size_t)N * N, 0.0);
                for (int i = 0; i < h; ++i)
                    for (int j = 0; j < S; ++j) hU[(size_t)i * N + j] = e[i] * U[(size_t)i * N + j];
                for (int i = h; i < N; ++i)
                    for (int j = 0; j < S; ++j) hV[(size_t)i * N + j] = e[i] * V[(size_t)i * N + j];
                ghfb_matmul(&D[h], N, &V[(size_t)h * N], N, DsV.data(), N, h, S, N - h, false);
                ghfb_matmul(&D[(size_t)h * N], N, U.data(), N, &DsU[(size_t)h * N], N, N - h, S, h,
                            false);
                std::vector<double>& G = grad[b];
                G.assign((size_t)N * N, 0.0);
                const int m = N - S;
                std::vector<double> t1((size_t)m * S), t2((size_t)m * S), t3((size_t)m * S),
                    t4((size_t)m * S);
                ghfb_matmul(&U[(size_t)h * N + S], N, &hV[(size_t)h * N], N, t1.data(), S, m, S,
                            N - h, true);
                ghfb_matmul(&V[S], N, DsV.data(), N, t2.data(), S, m, S, h, true);
                ghfb_matmul(&U[(size_t)h * N + S], N, &DsU[(size_t)h * N], N, t3.data(), S, m, S,
                            N - h, true);
                ghfb_matmul(&V[S], N, hU.data(), N, t4.data(), S, m, S, h, true);
                for (int i = 0; i < m; ++i)
                    for (int j = 0; j < S; ++j) {
                        double x = t1[(size_t)i * S + j];
                        x = x - t2[(size_t)i * S + j];
                        x = x + t3[(size_t)i * S + j];
                        x = x - t4[(size_t)i * S + j];
                        G[(size_t)(S + i) * N + j] = x;
                        G[(size_t)j * N + S + i] = -x;
                    }
                // N20 with signature: N20(0:S, S:N) = U(0:h,0:S)^T V(0:h,S:N)
                //                                   - V(h:N,0:S)^T U(h:N,S:N)
                std::vector<double>& A = an20[b];
                A.assign((size_t)N * N, 0.0);
                std::vector<double> u1((size_t)S * m), u2((size_t)S * m);
                ghfb_matmul(U.data(), N, &V[S], N, u1.data(), m, S, m, h, true);
                ghfb_matmul(&V[(size_t)h * N], N, &U[(size_t)h * N + S], N, u2.data(), m, S, m,
                            N - h, true);
                for (int i = 0; i < S; ++i)
                    for (int j = 0; j < m; ++j) {
                        const double x = u1[(size_t)i * m + j] - u2[(size_t)i * m + j];
                        A[(size_t)i * N + S + j] = x;
                        A[(size_t)(S + j) * N + i] = -x;
                    }
                for (int j = 0; j < N; ++j)
                    for (int i = 0; i < N; ++i) n20norm[it] += A[(size_t)i * N + j] * A[(size_t)i * N + j];
            }
        }
        // Fermi energies from the particle numbers of the current V
        for (int it = 0; it < 2; ++it) {
            par[it] = 0.0;
            for (int b = 2 * it; b < 2 * it + 2; ++b) {
                const int N = (int)c->bidx[b].size();
                for (int i = 0; i < N; ++i)
                    for (int j = 0; j < N; ++j) par[it] += c->GV[b][(size_t)i * N + j] * c->GV[b][(size_t)i * N + j];
            }
            if (std::fabs(n20norm[it]) > 1e-10)
                c->fermi[it] = c->fermi[it] + (particles[it] - par[it]) / n20norm[it];
            else
                c->fermi[it] = c->fermi[it] + 0.1 * (particles[it] - par[it]);
        }
        // total gradient and convergence
        for (int it = 0; it < 2; ++it) {
            if (conv[it]) continue;
            bool ok = std::fabs(par[it] - particles[it]) < prec;
            for (int b = 2 * it; b < 2 * it + 2; ++b) {
                const int N = (int)c->bidx[b].size();
                for (size_t q = 0; q < (size_t)N * N; ++q) grad[b][q] = grad[b][q] - c->fermi[it] * an20[b][q];
                gnorm[b] = 0.0;
                for (int i = 0; i < N; ++i)
                    for (int j = 0; j < N; ++j) gnorm[b] += grad[b][(size_t)i * N + j] * grad[b][(size_t)j * N + i];
                ok = ok && std::sqrt(std::fabs(gnorm[b])) < prec;
            }
            conv[it] = ok;
        }
        // gradient step and orthonormalisation
        for (int it = 0; it < 2; ++it) {
            if (conv[it]) continue;
            for (int b = 2 * it; b < 2 * it + 2; ++b) {
                const int N = (int)c->bidx[b].size(), h = N / 2, S = c->gsig[b], m = N - S;
                std::vector<double>& U = c->GU[b];
                std::vector<double>& V = c->GV[b];
                const std::vector<double> tU = U, tV = V;
                const std::vector<double>& G = grad[b];
                std::vector<double> w;
                // U(0:h,0:S) -= step tV(0:h,S:N) G(S:N,0:S)
                w.assign((size_t)h * S, 0.0);
                ghfb_matmul(&tV[S], N, &G[(size_t)S * N], N, w.data(), S, h, S, m, false);
                for (int i = 0; i < h; ++i)
                    for (int j = 0; j < S; ++j) U[(size_t)i * N + j] = U[(size_t)i * N + j] - step * w[(size_t)i * S + j];
                // U(h:N,S:N) -= step tV(h:N,0:S) G(0:S,S:N)
                w.assign((size_t)(N - h) * m, 0.0);
                ghfb_matmul(&tV[(size_t)h * N], N, &G[S], N, w.data(), m, N - h, m, S, false);
                for (int i = 0; i < N - h; ++i)
                    for (int j = 0; j < m; ++j)
                        U[(size_t)(h + i) * N + S + j] = U[(size_t)(h + i) * N + S + j] - step * w[(size_t)i * m + j];
                // V(0:h,S:N) -= step tU(0:h,0:S) G(0:S,S:N)
                w.assign((size_t)h * m, 0.0);
                ghfb_matmul(tU.data(), N, &G[S], N, w.data(), m, h, m, S, false);
                for (int i = 0; i < h; ++i)
                    for (int j = 0; j < m; ++j) V[(size_t)i * N + S + j] = V[(size_t)i * N + S + j] - step * w[(size_t)i * m + j];
                // V(h:N,0:S) -= step tU(h:N,S:N) G(S:N,0:S)
                w.assign((size_t)(N - h) * S, 0.0);
                ghfb_matmul(&tU[(size_t)h * N + S], N, &G[(size_t)S * N], N, w.data(), S, N - h, S, m,
                            false);
                for (int i = 0; i < N - h; ++i)
                    for (int j = 0; j < S; ++j)
                        V[(size_t)(h + i) * N + j] = V[(size_t)(h + i) * N + j] - step * w[(size_t)i * S + j];
                // ortho_sig
                for (int j = 0; j < S; ++j) {
                    double ov = 0.0;
                    for (int i = 0; i < h; ++i) ov = ov + U[(size_t)i * N + j] * U[(size_t)i * N + j];
                    for (int i = h; i < N; ++i) ov = ov + V[(size_t)i * N + j] * V[(size_t)i * N + j];
                    ov = 1.0 / std::sqrt(ov);
                    for (int i = 0; i < h; ++i) U[(size_t)i * N + j] = U[(size_t)i * N + j] * ov;
                    for (int i = h; i < N; ++i) V[(size_t)i * N + j] = V[(size_t)i * N + j] * ov;
                    for (int i = j + 1; i < h; ++i) {
                        double o = 0.0;
                        for (int k = 0; k < h; ++k) o = o + U[(size_t)k * N + j] * U[(size_t)k * N + i];
                        for (int k = h; k < N; ++k) o = o + V[(size_t)k * N + j] * V[(size_t)k * N + i];
                        for (int k = 0; k < h; ++k) U[(size_t)k * N + i] = U[(size_t)k * N + i] - o * U[(size_t)k * N + j];
                        for (int k = h; k < N; ++k) V[(size_t)k * N + i] = V[(size_t)k * N + i] - o * V[(size_t)k * N + j];
                    }
                }
                for (int j = S; j < N; ++j) {
                    double ov = 0.0;
                    for (int i = 0; i < h; ++i) ov = ov + V[(size_t)i * N + j] * V[(size_t)i * N + j];
                    for (int i = h; i < N; ++i) ov = ov + U[(size_t)i * N + j] * U[(size_t)i * N + j];
                    ov = 1.0 / std::sqrt(ov);
                    for (int i = h; i < N; ++i) U[(size_t)i * N + j] = U[(size_t)i * N + j] * ov;
                    for (int i = 0; i < h; ++i) V[(size_t)i * N + j] = V[(size_t)i * N + j] * ov;
                    for (int i = j + 1; i < N; ++i) {
                        double o = 0.0;
                        for (int k = 0; k < h; ++k) o = o + V[(size_t)k * N + j] * V[(size_t)k * N + i];
                        for (int k = h; k < N; ++k) o = o + U[(size_t)k * N + j] * U[(size_t)k * N + i];
                        for (int k = h; k < N; ++k) U[(size_t)k * N + i] = U[(size_t)k * N + i] - o * U[(size_t)k * N + j];
                        for (int k = 0; k < h; ++k) V[(size_t)k * N + i] = V[(size_t)k * N + i] - o * V[(size_t)k * N + j];
                    }
                }
            }
        }
        if (conv[0] && conv[1]) break;
    }
    *iters_out = std::min(iter, maxit);
    // OutHFBModule: rho = V V^T, kappa(i > j) = sum_k V(i,k) U(j,k) over the
    // kept columns (constructRhoHFB / ConstructKappaHFB, src/HFB.f90:3128-3154,
    // :3335-3359)
    for (int b = 0; b < 4; ++b) {
        const int N = (int)c->bidx[b].size();
        const std::vector<double>& U = c->GU[b];
        const std::vector<double>& V = c->GV[b];
        for (int j = 0; j < N; ++j)
            for (int i = 0; i < N; ++i) {
                double x = 0.0;
                for (int k = 0; k < N; ++k) x += V[(size_t)i * N + k] * V[(size_t)j * N + k];
                c->rho_h[b][(size_t)i * N + j] = x;
            }
        for (int j = 0; j < N; ++j) {
            c->kappa_h[b][(size_t)j * N + j] = 0.0;
            for (int i = j + 1; i < N; ++i) {
                double x = 0.0;
                for (int k = 0; k < N; ++k) x += V[(size_t)i * N + k] * U[(size_t)j * N + k];
                c->kappa_h[b][(size_t)i * N + j] = x;
                c->kappa_h[b][(size_t)j * N + i] = -x;
            }
        }
    }
    return (conv[0] && conv[1]) ? MG_OK : MG_NOT_CONVERGED;
}

extern "C" int orc_solve_pairing(orc_ctx* c, mg_pairing_info* info) {
    if (!c || c->p.pairing != MG_PAIRING_HFB) return MG_ERR_ARG;
    if (!c->hfb_ready) {
        hfb_prepare(c);
        if (c->pp.guess_kappa) {
            guess_kappa(c);
            c->pp.guess_kappa = 0;
        }
    }
    bool oz = true;
    for (int b = 0; b < 4; ++b)
        for (double x : c->oldrho[b]) oz = oz && x == 0.0;
    if (oz)
        for (int b = 0; b < 4; ++b) {
            c->oldrho[b] = c->rho_h[b];
            c->oldkappa[b] = c->kappa_h[b];
        }
    pairing_cutoffs(c, c->fermi);
    pairing_field(c);
    pairing_gaps(c);
    int evals = 0;
    const int st = c->pp.fermi_solver == 2   ? fermi_gradient(c, &evals)
                   : c->pp.fermi_solver == 3 ? fermi_bisection(c, &evals)
                                             : fermi_broyden(c, &evals);
    if (st < 0 && st != MG_ERR_STATE) return st;
    double tr[2] = {0.0, 0.0};
    for (int b = 0; b < 4; ++b) {
        const int N = (int)c->bidx[b].size();
        for (int i = 0; i < N; ++i) tr[b / 2] += c->rho_h[b][(size_t)i * N + i];
    }
    pairing_cutoffs(c, c->fermi);
    const int so = hfb_occupations(c);
    if (so != MG_OK) return so < 0 ? so : MG_ERR_STATE;
    hfb_energy(c);
    if (info) {
        std::memset(info, 0, sizeof(*info));
        info->fermi[0] = c->fermi[0];
        info->fermi[1] = c->fermi[1];
        info->particles[0] = tr[0];
        info->particles[1] = tr[1];
        info->evaluations = evals;
        info->converged = st == MG_OK;
        info->pairing_energy[0] = c->epair[0];
        info->pairing_energy[1] = c->epair[1];
        info->dispersion[0] = c->pdisp[0];
        info->dispersion[1] = c->pdisp[1];
    }
    return st == MG_ERR_STATE ? MG_ERR_STATE : MG_OK;
}

extern "C" int orc_get_hfb_block(orc_ctx* c, int b, double* rho, double* kappa, double* delta) {
    if (!c || b < 0 || b > 3 || !c->hfb_ready) return MG_ERR_ARG;
    const size_t n = c->rho_h[b].size();
    if (rho) std::copy(c->rho_h[b].begin(), c->rho_h[b].end(), rho);
    if (kappa) std::copy(c->kappa_h[b].begin(), c->kappa_h[b].end(), kappa);
    if (delta) std::copy(c->delta[b].begin(), c->delta[b].end(), delta);
    return (int)std::lround(std::sqrt((double)n));
}

extern "C" int orc_get_pairing_field(orc_ctx* c, double* re, double* im, double* dfac) {
    if (!c || !c->hfb_ready) return MG_ERR_ARG;
    if (re) std::copy(c->pf_re.begin(), c->pf_re.end(), re);
    if (im) std::copy(c->pf_im.begin(), c->pf_im.end(), im);
    if (dfac) std::copy(c->dfac.begin(), c->dfac.end(), dfac);
    return MG_OK;
}

// --------------------------------------------------------------------------
// Evolve loop body, src/Main.f90:255-328, HF pairing type (SolvePairing =
// NaiveFill), no constraints, MixingScheme 0.
// --------------------------------------------------------------------------
extern "C" int orc_iterate(orc_ctx* c, int n_iter, double dt, double momentum,
                           mg_energy_terms* out) {
    if (!c) return MG_ERR_ARG;
    const bool hfb = c->p.pairing == MG_PAIRING_HFB;
    int st = MG_OK;
    for (int k = 0; k < n_iter; ++k) {
        ++c->iteration;
        if (c->alternate_check) orc_alternate_step(c);   // src/Main.f90:261-263
        st = orc_grad_desc(c, dt, momentum);
        if (st != MG_OK) return st;
        if (hfb) {
            const int sp = orc_solve_pairing(c, nullptr);
            if (sp < 0) return sp;
        } else {
            orc_hf_fill(c);
        }
        c->alternate_check = any_alternating(c);           // src/Main.f90:274
        orc_derive_all(c);
        if (hfb) orc_hpsi(c, MG_CAN_BASIS, nullptr, c->bas[MG_CAN_BASIS].e.data(),
                          c->bas[MG_CAN_BASIS].disp.data());
        orc_update_densities(c);
        orc_mix_densities(c);
        orc_calculate_moments(c);
        readjust_moments(c, c->iteration);                  // src/Main.f90:299-304
        st = orc_construct_potentials(c, nullptr);
        if (st < 0) return st;
        // CompEnergy every pass (src/Main.f90:309), which also keeps the
        // energy history of ConvergenceCheck
        mg_energy_terms e{};
        orc_energy(c, out ? out : &e);
    }
    return st;
}

// ConvergenceCheck, src/Main.f90:358-397: ConverMultipoleAll
// (src/Moments.f90:2628-2701), ConverEnergy (src/Energy.f90:1458-1481),
// ConverFermi (src/Pairing.f90:1048-1070; its FermiHistory is never written,
// so it stays zero), and the stop on a positive total energy.
extern "C" int orc_convergence_check(orc_ctx* c, const mg_convergence* prec, int* converged) {
    if (!c || !converged) return MG_ERR_ARG;
    const mg_convergence P = prec ? *prec : mg_convergence{(double)0.01e-8f, 1e-4, 1e-4};
    bool conv = true;
    for (const Constraint& k : c->cons) {
        if (k.type == 0) continue;
        const double C = k.constraint;
        const double v = k.value[0] + k.value[1];
        double d[8];
        if (k.true_constraint != 0.0) {
            d[0] = std::fabs((C - v) / C);
            for (int i = 1; i < 8; ++i) d[i] = std::fabs((C - k.old_value[i - 1]) / C);
        } else {
            d[0] = std::fabs(C - v);
            for (int i = 1; i < 8; ++i) d[i] = std::fabs(C - k.old_value[i - 1]);
        }
        for (int i = 0; i < 8; ++i)
            if (d[i] >= P.moment_prec) conv = false;
    }
    const double E = c->total_energy;
    for (int i = 0; i < 7; ++i)
        conv = conv && std::fabs((c->old_energy[i] - E) / E) <= P.energy_prec;
    if (c->p.pairing == MG_PAIRING_HFB)
        for (int it = 0; it < 2; ++it)
            if (std::fabs(c->fermi[it] - 0.0) > P.pairing_prec) conv = false;
    *converged = conv ? 1 : 0;
    return E >= 0.0 ? MG_ERR_STATE : MG_OK;
}
