// host.cu -- the extern "C" entry points of libmocca_gpu (include/mocca_gpu.h).
//
// Each entry point validates its arguments, enqueues its kernels on the
// context's stream and returns an int status; the Fortran shim turns a
// non-zero status into the reference's stp() (src/GenInfo.f90:84-177).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>

#include "mg_internal.cuh"

using namespace mg;

namespace {

const double kPi = 4.0 * std::atan2(1.0, 1.0);

bool valid_basis(const mg_ctx* c, int b) {
    if (b == MG_HF_BASIS) return true;
    return b == MG_CAN_BASIS && c->p.pairing == MG_PAIRING_HFB;
}

void free_all(mg_ctx* c) {
    auto F = [](void* p) { if (p) cudaFree(p); };
    F(c->mats);
    F(c->mats32);
    F(c->tcmats);
    F(c->tc_erow);
    F(c->tc_status);
    F(c->gs_Stc); F(c->gs_xd); F(c->gs_xe); F(c->can_xd); F(c->can_xe); F(c->gap_part); F(c->fields_df);
    F(c->field_y); F(c->field_xd); F(c->field_xe); F(c->field_ybase);
    F(c->est); F(c->est_jobs); F(c->est_qn);
    for (int b = 0; b < 2; ++b) {
        Basis& B = c->bas[b];
        F(B.psi); F(B.der); F(B.lap); F(B.qn); F(B.occ); F(B.e); F(B.disp); F(B.jobs);
    }
    F(c->updates); F(c->hbuf);
    F(c->rho); F(c->tau); F(c->nablaj); F(c->derrho); F(c->laprho);
    F(c->U); F(c->Bp); F(c->nablaB); F(c->W); F(c->divW); F(c->divw_tmp); F(c->field_jobs);
    F(c->gs_S); F(c->gs_R); F(c->gs_index);
    F(c->cpot); F(c->csource); F(c->cres); F(c->cp); F(c->ct); F(c->sh_ext); F(c->sh_mesh);
    F(c->coulomb); F(c->coulex); F(c->moment_values); F(c->rpow_ext); F(c->mfac);
    F(c->cg_bar); F(c->cg_status); F(c->red); F(c->flags); F(c->cfast); F(c->cguess);
    F(c->dhist); F(c->Uold); F(c->Sold); F(c->Wold); F(c->pc_buf); F(c->pc_jobs); F(c->jmunu); F(c->jmunu_hist);
    F(c->odd); F(c->odd_hist); F(c->Apot); F(c->Spot); F(c->divA); F(c->odd_der); F(c->odd_tmp);
    F(c->odd_jobs);
    F(c->Cpot); F(c->Dpot); F(c->dDpot); F(c->divD); F(c->todd_tmp); F(c->todd_work);
    F(c->todd_x); F(c->todd_jobs); F(c->todd_act_jobs);
    multigrid_free(c->mgrid);
    c->mgrid = nullptr;
    hfb_free(c);
    constraints_free(c);
    if (c->h_cg_status) cudaFreeHost(c->h_cg_status);
    if (c->h_tc_status) cudaFreeHost(c->h_tc_status);
    if (c->cfast_graph) cudaGraphExecDestroy(c->cfast_graph);
    if (c->ev_fork) cudaEventDestroy(c->ev_fork);
    if (c->ev_join) cudaEventDestroy(c->ev_join);
    for (cudaEvent_t e : c->ph.ev)
        if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : c->ph.side)
        if (e) cudaEventDestroy(e);
    if (c->side) cudaStreamDestroy(c->side);
    if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
}

}  // namespace

// ---------------------------------------------------------------------------
// Host helpers
// ---------------------------------------------------------------------------
extern "C" int mg_skyrme_coefficients(const mg_force* f, int trc, mg_skyrme_b* B) {
    // CalcEDFCoef, src/Force.f90:467-560
    if (!f || !B) return MG_ERR_ARG;
    std::memset(B, 0, sizeof(*B));
    B->B1 = f->t0 * (1.0 + 0.5 * f->x0) / 2.0;
    B->B2 = -f->t0 * (0.5 + f->x0) / 2.0;
    B->B3 = (f->t1 * (1 + 0.5 * f->x1) + f->t2 * (1 + 0.5 * f->x2)) / 4.0;
    B->B4 = -(f->t1 * (0.5 + f->x1) - f->t2 * (0.5 + f->x2)) / 4.0;
    B->B5 = -(3.0 * f->t1 * (1 + f->x1 / 2.0) - f->t2 * (1 + f->x2 / 2.0)) / 16.0;
    B->B6 = (3.0 * f->t1 * (f->x1 + 0.5) + f->t2 * (f->x2 + 0.5)) / 16.0;
    B->B7a = f->t3a * (1 + f->x3a / 2.0) / 12.0;
    B->B8a = -f->t3a * (f->x3a + 0.5) / 12.0;
    B->B7b = f->t3b * (1 + f->x3b / 2.0) / 12.0;
    B->B8b = -f->t3b * (f->x3b + 0.5) / 12.0;
    B->B9 = -f->wso / 2.0;
    B->B9q = -f->wsoq / 2.0;
    B->byt3a = f->yt3a;
    B->byt3b = f->yt3b;
    if (!trc) {
        B->B10 = f->t0 * f->x0 / 4.0;
        B->B11 = -f->t0 / 4.0;
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

extern "C" int mg_lagrange_matrices(int n, double dx, int folded, double* d1, double* d2) {
    // Baye-Heenen coefficients on the full line of N points (IniLag,
    // src/Derivatives.f90:899-973):
    //   C1(k) = pi/(N dx) (-1)^k / sin(pi k/N)
    //   C2(k) = (-1)^(k+1) 2 (pi/(N dx))^2 cos(pi k/N) / sin(pi k/N)^2
    //   diag  = -pi^2/(3 dx^2) (1 - 1/N^2)
    // folded (reduceLag, :975-1078): M_s(i,j) = sgn(i-j) C1(|i-j|) + s C1(i+j-1),
    // L_s(i,j) = C2(|i-j|) + s C2(i+j-1) (+ diag on i=j), s = -1 / +1.
    if (n <= 0 || n > kMaxN || !(dx > 0) || !d1 || !d2) return MG_ERR_ARG;
    const int N = folded ? 2 * n : n;
    std::vector<double> C1(N + 1, 0.0), C2(N + 1, 0.0);
    const double factor = kPi / N, dxf = factor / dx;
    const double diag = -(kPi * kPi) / (3.0 * (dx * dx)) * (1.0 - 1.0 / double(N * N));
    for (int k = 1; k < N; ++k) {
        const double s = std::sin(factor * k), c = std::cos(factor * k);
        const double sg = (k % 2 == 0) ? 1.0 : -1.0;
        C1[k] = dxf * sg / s;
        C2[k] = -sg * 2.0 * (dxf * dxf) * c / (s * s);
    }
    const long nn = (long)n * n;
    for (int i = 1; i <= n; ++i)
        for (int j = 1; j <= n; ++j) {
            const long o = (long)(i - 1) * n + (j - 1);
            const double sgn = i > j ? 1.0 : (i < j ? -1.0 : 0.0);
            const double t1 = i == j ? 0.0 : sgn * C1[std::abs(i - j)];
            const double t2 = i == j ? diag : C2[std::abs(i - j)];
            if (folded) {
                const double e1 = C1[i + j - 1], e2 = C2[i + j - 1];
                d1[o] = t1 - e1; d1[nn + o] = t1 + e1;
                d2[o] = t2 - e2; d2[nn + o] = t2 + e2;
            } else {
                d1[o] = d1[nn + o] = t1;
                d2[o] = d2[nn + o] = t2;
            }
        }
    return MG_OK;
}

// ---------------------------------------------------------------------------
// Context
// ---------------------------------------------------------------------------
extern "C" int mg_create(const mg_params* p, const mg_force* f, void* stream, mg_ctx** out) {
    if (!p || !f || !out) return MG_ERR_ARG;
    if (f->coupling < 0 || f->coupling > MG_COUPLING_UNEDF2) return MG_ERR_ARG;
    *out = nullptr;
    if (p->nx <= 0 || p->ny <= 0 || p->nz <= 0 || p->nx > kMaxN || p->ny > kMaxN ||
        p->nz > kMaxN || !(p->dx > 0) || p->nwt <= 0)
        return MG_ERR_ARG;
    const bool ev8 = p->pc && p->sc && p->tsc;
    const bool full = !p->pc && !p->sc && !p->tsc;
    if (!ev8 && !full) return MG_ERR_ARG;
    if (p->precision != MG_FP64 && p->precision != MG_MIXED) return MG_ERR_ARG;
    if ((p->parameter_estimation != 0 && p->parameter_estimation != 1) ||
        (p->mixing_scheme != 0 && p->mixing_scheme != 2) || !(p->damping >= 0.0) ||
        !(p->precon_w >= 0.0) ||
        p->damping > 1.0)
        return MG_ERR_ARG;
    if (p->pairing != MG_PAIRING_HF && p->pairing != MG_PAIRING_HFB) return MG_ERR_ARG;
    if (p->coulomb_solver < 0 || p->coulomb_solver > 2 || !(p->coulomb_prec >= 0.0))
        return MG_ERR_ARG;
    // time reversal broken: the time-odd fields (timeodd.cu) on the EV8 box,
    // HF filling, FP64; cranking only then, and with EV8 only about z (the
    // reference stops on OmegaX with signature, OmegaY with time simplex)
    const bool crank = p->omega[0] != 0.0 || p->omega[1] != 0.0 || p->omega[2] != 0.0;
    if (crank && p->trc) return MG_ERR_ARG;
    if ((p->sc && p->omega[0] != 0.0) || (p->tsc && p->omega[1] != 0.0)) return MG_ERR_ARG;
    if (!p->trc && (!ev8 || p->precision != MG_FP64 || p->pairing != MG_PAIRING_HF))
        return MG_ERR_ARG;
    int dev = 0;
    MG_CUDA(cudaGetDevice(&dev));
    mg_ctx* c = new mg_ctx();
    c->device = dev;
    c->p = *p;
    c->f = *f;
    mg_skyrme_coefficients(f, p->trc, &c->B);
    c->tensor = c->B.B14 != 0.0 || c->B.B15 != 0.0 || c->B.B16 != 0.0 || c->B.B17 != 0.0;
    // without time reversal the tensor terms have time-odd partners
    // (tensor_odd.cu): T, F, lap s and grad div s behind the time-odd densities
    c->todd = !p->trc && (c->tensor || c->B.B18 != 0.0 || c->B.B19 != 0.0 ||
                          c->B.B20 != 0.0 || c->B.B21 != 0.0);
    c->odd_len = c->todd ? 48 : 24;
    c->nx = p->nx; c->ny = p->ny; c->nz = p->nz;
    c->V = (long)p->nx * p->ny * p->nz;
    const int nsym = (p->pc ? 1 : 0) + (p->sc ? 1 : 0) + (p->tsc ? 1 : 0);
    c->dv = p->dx * p->dx * p->dx * std::pow(2.0, nsym);  // src/GenInfo.f90:296
    c->folded = ev8;
    int st = MG_OK;
    auto fail = [&](int s) { free_all(c); delete c; return s; };
    if (cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return fail(MG_ERR_CUDA);
    if (stream) {
        c->stream = (cudaStream_t)stream;
    } else {
        if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess)
            return fail(MG_ERR_CUDA);
        c->own_stream = true;
    }
    // side stream (lower priority) for the HF-basis derivatives, which run
    // while the latency-bound Fermi search of the pairing step occupies few SMs
    {
        int lo = 0, hi = 0;
        if (cudaDeviceGetStreamPriorityRange(&lo, &hi) != cudaSuccess ||
            cudaStreamCreateWithPriority(&c->side, cudaStreamNonBlocking, lo) != cudaSuccess ||
            cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming) != cudaSuccess)
            return fail(MG_ERR_CUDA);
    }
    const long V = c->V, nwt = p->nwt;
    auto A = [&](double** ptr, long n) {
        if (cudaMalloc(ptr, std::max(1L, n) * sizeof(double)) != cudaSuccess) return false;
        return cudaMemset(*ptr, 0, std::max(1L, n) * sizeof(double)) == cudaSuccess;
    };
    bool ok = true;
    const int nb = p->pairing == MG_PAIRING_HFB ? 2 : 1;
    for (int b = 0; b < nb && ok; ++b) {
        Basis& B = c->bas[b];
        ok = A(&B.psi, nwt * 4 * V) && A(&B.der, nwt * 12 * V) && A(&B.lap, nwt * 4 * V) &&
             A(&B.occ, nwt) && A(&B.e, nwt) && A(&B.disp, nwt) &&
             cudaMalloc(&B.qn, nwt * 4 * sizeof(int)) == cudaSuccess &&
             cudaMalloc(&B.jobs, nwt * 4 * sizeof(GridJob)) == cudaSuccess;
        B.h_qn.assign(nwt * 4, 1);
        B.h_occ.assign(nwt, 0.0);
        B.h_e.assign(nwt, 0.0);
        B.h_disp.assign(nwt, 0.0);
    }
    ok = ok && A(&c->updates, nwt * 4 * V) && A(&c->rho, 2 * V) && A(&c->tau, 2 * V) &&
         A(&c->nablaj, 2 * V) && A(&c->derrho, 6 * V) && A(&c->laprho, 2 * V) &&
         A(&c->U, 2 * V) && A(&c->Bp, 2 * V) && A(&c->nablaB, 6 * V) && A(&c->W, 18 * V) &&
         A(&c->divW, 6 * V) && A(&c->divw_tmp, 18 * V) && A(&c->coulomb, V) && A(&c->coulex, V);
    if (ok && c->tensor) ok = A(&c->jmunu, 18 * V) && A(&c->jmunu_hist, 18 * V);
    if (!ok) return fail(MG_ERR_CUDA);
    // reduction scratch: the largest of the per-kernel partial tables
    const long hp = nwt * div_up(V, 256) * 2;
    const long dens = (long)density_groups(c) * 6 * V;
    const long dots = 64 * nwt;
    const long en = 2L * c->num_sms * 26 + 4L * c->num_sms;
    c->red_len = (size_t)std::max(std::max(hp, dens), dots + en);   // energy uses both
    if (!A(&c->red, (long)c->red_len)) return fail(MG_ERR_CUDA);
    if (cudaMalloc(&c->flags, 16 * sizeof(int)) != cudaSuccess ||
        cudaMemset(c->flags, 0, 16 * sizeof(int)) != cudaSuccess ||
        cudaMallocHost(&c->h_cg_status, 4 * sizeof(int)) != cudaSuccess)
        return fail(MG_ERR_CUDA);
    c->cur_precision = p->precision;
    if ((st = upload_matrices(c)) != MG_OK) return fail(st);
    if ((st = build_field_jobs(c)) != MG_OK) return fail(st);
    if ((st = mixing_setup(c)) != MG_OK) return fail(st);
    if (!p->trc && (st = time_odd_setup(c)) != MG_OK) return fail(st);
    if (ev8 && p->coulomb_solver != 0) {
        if ((st = coulomb_setup(c)) != MG_OK) return fail(st);
    }
    *out = c;
    return MG_OK;
}

extern "C" int mg_set_precision(mg_ctx* c, int precision) {
    if (!c || (precision != MG_FP64 && precision != MG_MIXED)) return MG_ERR_ARG;
    if (!c->p.trc && precision != MG_FP64) return MG_ERR_ARG;   // time-odd path: FP64
    c->cur_precision = precision;
    return MG_OK;
}

extern "C" int mg_destroy(mg_ctx* c) {
    if (!c) return MG_ERR_ARG;
    if (c->stream) cudaStreamSynchronize(c->stream);
    free_all(c);
    delete c;
    return MG_OK;
}

extern "C" int mg_synchronize(mg_ctx* c) {
    if (!c) return MG_ERR_ARG;
    MG_CUDA(cudaStreamSynchronize(c->stream));
    return MG_OK;
}

// ---------------------------------------------------------------------------
// Transfers
// ---------------------------------------------------------------------------
extern "C" int mg_upload_spinors(mg_ctx* c, int b, const double* const* grids, const int* qn,
                                 int first, int count) {
    if (!c || !valid_basis(c, b) || first < 0 || count < 0 || first + count > c->p.nwt)
        return MG_ERR_ARG;
    Basis& B = c->bas[b];
    const long V4 = 4 * c->V;
    if (grids) {
        // one copy per run of spwfs whose host grids lie back to back (a
        // Fortran program allocates each Grid separately; a contiguous host
        // array becomes a single transfer instead of nwt small ones)
        for (int i = 0; i < count;) {
            if (!grids[i]) return MG_ERR_ARG;
            int j = i + 1;
            while (j < count && grids[j] == grids[j - 1] + V4) ++j;
            MG_CUDA(cudaMemcpyAsync(B.psi + (long)(first + i) * V4, grids[i],
                                    (size_t)(j - i) * V4 * sizeof(double), cudaMemcpyHostToDevice,
                                    c->stream));
            i = j;
        }
    }
    if (qn) {
        for (int i = 0; i < 4 * count; ++i) {
            const int q = qn[i];
            if ((i % 4 == 0 && q != 1 && q != -1) || q < -1 || q > 1) return MG_ERR_ARG;
            B.h_qn[4 * first + i] = q;
        }
        MG_CUDA(cudaMemcpyAsync(B.qn, B.h_qn.data(), B.h_qn.size() * sizeof(int),
                                cudaMemcpyHostToDevice, c->stream));
        if (first + count == c->p.nwt || B.have_qn) {
            B.have_qn = true;
            MG_TRY(build_basis_jobs(c, b));
            if (b == MG_HF_BASIS) c->gs_nblk = 0;  // rebuild Gram-Schmidt blocks
        }
    }
    return MG_OK;
}

extern "C" int mg_download_spinors(mg_ctx* c, int b, double* const* grids, int first, int count) {
    if (!c || !valid_basis(c, b) || !grids || first < 0 || count < 0 || first + count > c->p.nwt)
        return MG_ERR_ARG;
    const long V4 = 4 * c->V;
    for (int i = 0; i < count;) {
        if (!grids[i]) return MG_ERR_ARG;
        int j = i + 1;   // a run of back-to-back host grids: one transfer
        while (j < count && grids[j] == grids[j - 1] + V4) ++j;
        MG_CUDA(cudaMemcpyAsync(grids[i], c->bas[b].psi + (long)(first + i) * V4,
                                (size_t)(j - i) * V4 * sizeof(double), cudaMemcpyDeviceToHost,
                                c->stream));
        i = j;
    }
    MG_CUDA(cudaStreamSynchronize(c->stream));
    return MG_OK;
}

extern "C" int mg_download_derivatives(mg_ctx* c, int b, double* const* der, double* const* lap,
                                       int first, int count) {
    if (!c || !valid_basis(c, b) || first < 0 || count < 0 || first + count > c->p.nwt)
        return MG_ERR_ARG;
    const long V = c->V;
    for (int i = 0; i < count; ++i) {
        if (der && der[i])
            MG_CUDA(cudaMemcpyAsync(der[i], c->bas[b].der + (long)(first + i) * 12 * V,
                                    12 * V * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
        if (lap && lap[i])
            MG_CUDA(cudaMemcpyAsync(lap[i], c->bas[b].lap + (long)(first + i) * 4 * V,
                                    4 * V * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    }
    MG_CUDA(cudaStreamSynchronize(c->stream));
    if (c->bas[b].der_df) {
        // mixed form: {hi, lo} float pairs -> FP64 in place
        auto widen = [](double* p, long n) {
            for (long k = 0; k < n; ++k) {
                float hl[2];
                std::memcpy(hl, p + k, sizeof(hl));
                p[k] = (double)hl[0] + (double)hl[1];
            }
        };
        for (int i = 0; i < count; ++i) {
            if (der && der[i]) widen(der[i], 12 * V);
            if (lap && lap[i]) widen(lap[i], 4 * V);
        }
    }
    return MG_OK;
}

extern "C" int mg_set_occupations(mg_ctx* c, int b, const double* occ) {
    if (!c || !valid_basis(c, b) || !occ) return MG_ERR_ARG;
    std::copy(occ, occ + c->p.nwt, c->bas[b].h_occ.begin());
    MG_CUDA(cudaMemcpyAsync(c->bas[b].occ, c->bas[b].h_occ.data(), c->p.nwt * sizeof(double),
                            cudaMemcpyHostToDevice, c->stream));
    MG_CUDA(cudaStreamSynchronize(c->stream));
    return MG_OK;
}

extern "C" int mg_get_occupations(mg_ctx* c, int b, double* occ) {
    if (!c || !valid_basis(c, b) || !occ) return MG_ERR_ARG;
    MG_CUDA(cudaMemcpyAsync(occ, c->bas[b].occ, c->p.nwt * sizeof(double), cudaMemcpyDeviceToHost,
                            c->stream));
    MG_CUDA(cudaStreamSynchronize(c->stream));
    return MG_OK;
}

extern "C" int mg_set_energies(mg_ctx* c, int b, const double* e) {
    if (!c || !valid_basis(c, b) || !e) return MG_ERR_ARG;
    MG_CUDA(cudaMemcpyAsync(c->bas[b].e, e, c->p.nwt * sizeof(double), cudaMemcpyHostToDevice,
                            c->stream));
    MG_CUDA(cudaStreamSynchronize(c->stream));
    return MG_OK;
}

extern "C" int mg_get_energies(mg_ctx* c, int b, double* e, double* disp) {
    if (!c || !valid_basis(c, b)) return MG_ERR_ARG;
    if (e)
        MG_CUDA(cudaMemcpyAsync(e, c->bas[b].e, c->p.nwt * sizeof(double), cudaMemcpyDeviceToHost,
                                c->stream));
    if (disp)
        MG_CUDA(cudaMemcpyAsync(disp, c->bas[b].disp, c->p.nwt * sizeof(double),
                                cudaMemcpyDeviceToHost, c->stream));
    MG_CUDA(cudaStreamSynchronize(c->stream));
    return MG_OK;
}

// ---------------------------------------------------------------------------
// Compute
// ---------------------------------------------------------------------------
extern "C" int mg_derive_basis(mg_ctx* c, int b) {
    if (!c || !valid_basis(c, b)) return MG_ERR_ARG;
    return derive_basis(c, b);
}

extern "C" int mg_derive_all(mg_ctx* c) {
    if (!c) return MG_ERR_ARG;
    MG_TRY(derive_basis(c, MG_HF_BASIS));
    if (c->p.pairing == MG_PAIRING_HFB) MG_TRY(derive_basis(c, MG_CAN_BASIS));
    return tc_check(c);
}

extern "C" int mg_hpsi(mg_ctx* c, int b, double* hpsi, double* e, double* disp) {
    if (!c || !valid_basis(c, b)) return MG_ERR_ARG;
    const long total = (long)c->p.nwt * 4 * c->V;
    double* dev_out = nullptr;
    if (hpsi) {
        if (!c->hbuf) MG_CUDA(cudaMalloc(&c->hbuf, total * sizeof(double)));
        dev_out = c->hbuf;
    }
    MG_TRY(hpsi_basis(c, b, dev_out, false, 0.0, 0.0));
    if (hpsi)
        MG_CUDA(cudaMemcpyAsync(hpsi, c->hbuf, total * sizeof(double), cudaMemcpyDeviceToHost,
                                c->stream));
    return mg_get_energies(c, b, e, disp);
}

extern "C" int mg_grad_desc(mg_ctx* c, double dt, double momentum) {
    if (!c) return MG_ERR_ARG;
    if (!c->step_set || c->p.parameter_estimation != 1) {
        c->step_dt = dt;
        c->step_mom = momentum;
        c->step_set = true;
    }
    // ParameterEstimation = 1: IterativeEstimation first (src/ImaginaryTime.f90:465)
    if (c->p.parameter_estimation == 1) MG_TRY(estimate_parameters(c));
    MG_TRY(hpsi_basis(c, MG_HF_BASIS, nullptr, true, c->step_dt / c->f.hbar, c->step_mom));
    return gram_schmidt_impl(c, c->updates);
}

extern "C" int mg_get_step_parameters(mg_ctx* c, double* dt, double* momentum) {
    if (!c || !dt || !momentum) return MG_ERR_ARG;
    *dt = c->step_dt;
    *momentum = c->step_mom;
    return MG_OK;
}

extern "C" int mg_gram_schmidt(mg_ctx* c) {
    if (!c) return MG_ERR_ARG;
    return gram_schmidt(c);
}

extern "C" int mg_hf_fill(mg_ctx* c) {
    // NaiveFill, src/HartreeFock.f90:177-260 (no blocking)
    if (!c) return MG_ERR_ARG;
    Basis& B = c->bas[MG_HF_BASIS];
    const int nwt = c->p.nwt;
    std::vector<double> e(nwt);
    MG_CUDA(cudaMemcpyAsync(e.data(), B.e, nwt * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    MG_CUDA(cudaStreamSynchronize(c->stream));
    std::vector<int> order(nwt);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b2) { return e[a] < e[b2]; });
    std::vector<double> occ(nwt, 0.0);
    const int pub = c->p.trc ? (int)std::floor(c->p.protons / 2) : (int)std::floor(c->p.protons);
    const int nub = c->p.trc ? (int)std::floor(c->p.neutrons / 2) : (int)std::floor(c->p.neutrons);
    int np = 0, nn = 0;
    for (int i = 0; i < nwt && np < pub; ++i)
        if (occ[order[i]] == 0.0 && B.h_qn[4 * order[i]] == 1) { occ[order[i]] = 1.0; ++np; }
    for (int i = 0; i < nwt && nn < nub; ++i)
        if (occ[order[i]] == 0.0 && B.h_qn[4 * order[i]] == -1) { occ[order[i]] = 1.0; ++nn; }
    if (c->p.trc)
        for (double& o : occ) o = 2.0 * o;
    return mg_set_occupations(c, MG_HF_BASIS, occ.data());
}

extern "C" int mg_update_densities(mg_ctx* c) {
    if (!c) return MG_ERR_ARG;
    MG_TRY(save_density_history(c));
    return densities(c);
}

extern "C" int mg_mix_densities(mg_ctx* c) {
    if (!c) return MG_ERR_ARG;
    return mix_densities(c);
}

static int copy_out(mg_ctx* c, double* dst, const double* src, long n) {
    if (!dst) return MG_OK;
    MG_CUDA(cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    return MG_OK;
}
static int copy_in(mg_ctx* c, double* dst, const double* src, long n) {
    if (!src) return MG_OK;
    MG_CUDA(cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    return MG_OK;
}

extern "C" int mg_get_densities(mg_ctx* c, double* rho, double* tau, double* nablaj,
                                double* derrho, double* laprho) {
    if (!c) return MG_ERR_ARG;
    const long V = c->V;
    MG_TRY(copy_out(c, rho, c->rho, 2 * V));
    MG_TRY(copy_out(c, tau, c->tau, 2 * V));
    MG_TRY(copy_out(c, nablaj, c->nablaj, 2 * V));
    MG_TRY(copy_out(c, derrho, c->derrho, 6 * V));
    MG_TRY(copy_out(c, laprho, c->laprho, 2 * V));
    MG_CUDA(cudaStreamSynchronize(c->stream));
    return MG_OK;
}

extern "C" int mg_get_jmunu(mg_ctx* c, double* jmunu) {
    if (!c || !jmunu || !c->tensor) return MG_ERR_ARG;
    MG_TRY(copy_out(c, jmunu, c->jmunu, 18 * c->V));
    MG_CUDA(cudaStreamSynchronize(c->stream));
    return MG_OK;
}

extern "C" int mg_set_jmunu(mg_ctx* c, const double* jmunu) {
    if (!c || !jmunu || !c->tensor) return MG_ERR_ARG;
    MG_TRY(copy_in(c, c->jmunu, jmunu, 18 * c->V));
    MG_CUDA(cudaStreamSynchronize(c->stream));
    return MG_OK;
}

extern "C" int mg_set_densities(mg_ctx* c, const double* rho, const double* tau,
                                const double* nablaj, const double* derrho, const double* laprho) {
    if (!c) return MG_ERR_ARG;
    const long V = c->V;
    MG_TRY(copy_in(c, c->rho, rho, 2 * V));
    MG_TRY(copy_in(c, c->tau, tau, 2 * V));
    MG_TRY(copy_in(c, c->nablaj, nablaj, 2 * V));
    MG_TRY(copy_in(c, c->derrho, derrho, 6 * V));
    MG_TRY(copy_in(c, c->laprho, laprho, 2 * V));
    MG_CUDA(cudaStreamSynchronize(c->stream));
    return MG_OK;
}

extern "C" int mg_calculate_moments(mg_ctx* c) {
    if (!c) return MG_ERR_ARG;
    return moments(c);
}

extern "C" int mg_solve_coulomb(mg_ctx* c, int* iters) {
    if (!c || !c->folded) return MG_ERR_ARG;
    int it = 0;
    const int st = coulomb_solve(c, &it);
    if (iters) *iters = it;
    return st;
}

extern "C" int mg_coulomb_reset(mg_ctx* c) {
    if (!c || !c->folded) return MG_ERR_ARG;
    return coulomb_reset(c);
}

extern "C" int mg_coulomb_residual(mg_ctx* c, double* rel) {
    if (!c || !rel || !c->folded) return MG_ERR_ARG;
    return coulomb_residual(c, rel);
}

extern "C" int mg_construct_potentials(mg_ctx* c, int* iters) {
    if (!c) return MG_ERR_ARG;
    int st = MG_OK;
    if (c->p.coulomb_solver != 0) {
        if (!c->folded) return MG_ERR_ARG;
        int it = 0;
        st = coulomb_solve(c, iters ? &it : nullptr);
        if (st < 0) return st;
        if (iters) *iters = it;
    } else if (iters) {
        *iters = 0;
    }
    // UpotOld = Upot (src/PotentialMixing.f90:115); MixingScheme 2 then
    // preconditions the update once UpotOld is not all zero
    MG_CUDA(cudaMemcpyAsync(c->Uold, c->U, 2 * c->V * sizeof(double), cudaMemcpyDeviceToDevice,
                            c->stream));
    if (c->Wold)   // WpotOld = Wpot (src/PotentialMixing.f90:117)
        MG_CUDA(cudaMemcpyAsync(c->Wold, c->W, 18 * c->V * sizeof(double),
                                cudaMemcpyDeviceToDevice, c->stream));
    if (c->Sold)   // SpotOld = Spot (src/PotentialMixing.f90:122)
        MG_CUDA(cudaMemcpyAsync(c->Sold, c->Spot, 6 * c->V * sizeof(double),
                                cudaMemcpyDeviceToDevice, c->stream));
    MG_TRY(potentials(c));
    if (c->p.mixing_scheme == 2 && c->have_uold) MG_TRY(precondition_u(c));
    c->have_uold = true;
    return st;
}

extern "C" int mg_get_potentials(mg_ctx* c, double* u, double* b, double* nablab, double* w,
                                 double* divw, double* coul, double* coulex) {
    if (!c) return MG_ERR_ARG;
    const long V = c->V;
    MG_TRY(copy_out(c, u, c->U, 2 * V));
    MG_TRY(copy_out(c, b, c->Bp, 2 * V));
    MG_TRY(copy_out(c, nablab, c->nablaB, 6 * V));
    MG_TRY(copy_out(c, w, c->W, 18 * V));
    MG_TRY(copy_out(c, divw, c->divW, 6 * V));
    MG_TRY(copy_out(c, coul, c->coulomb, V));
    MG_TRY(copy_out(c, coulex, c->coulex, V));
    MG_CUDA(cudaStreamSynchronize(c->stream));
    return MG_OK;
}

extern "C" int mg_set_potentials(mg_ctx* c, const double* u, const double* b,
                                 const double* nablab, const double* w, const double* divw) {
    if (!c) return MG_ERR_ARG;
    const long V = c->V;
    MG_TRY(copy_in(c, c->U, u, 2 * V));
    if (u) c->have_uold = true;   // the next UpotOld is this U
    MG_TRY(copy_in(c, c->Bp, b, 2 * V));
    MG_TRY(copy_in(c, c->nablaB, nablab, 6 * V));
    MG_TRY(copy_in(c, c->W, w, 18 * V));
    MG_TRY(copy_in(c, c->divW, divw, 6 * V));
    MG_CUDA(cudaStreamSynchronize(c->stream));
    return MG_OK;
}

extern "C" int mg_energy(mg_ctx* c, mg_energy_terms* out) {
    if (!c || !out) return MG_ERR_ARG;
    return energy(c, out);
}

extern "C" int mg_set_pairing(mg_ctx* c, const mg_pairing_params* pp) {
    if (!c || !pp || c->p.pairing != MG_PAIRING_HFB || !c->p.trc || !c->folded) return MG_ERR_ARG;
    if (c->hfb.ready) return MG_ERR_STATE;
    if (!(pp->rhosat > 0) || pp->mu[0] <= 0 || pp->mu[1] <= 0 || pp->cut[0] <= 0 || pp->cut[1] <= 0)
        return MG_ERR_ARG;
    if (pp->fermi_solver < 0 || pp->fermi_solver > 3) return MG_ERR_ARG;
    c->hfb.pp = *pp;
    c->hfb.fermi[0] = pp->fermi_start[0];
    c->hfb.fermi[1] = pp->fermi_start[1];
    return MG_OK;
}

extern "C" int mg_solve_pairing(mg_ctx* c, mg_pairing_info* info) {
    if (!c || c->p.pairing != MG_PAIRING_HFB) return MG_ERR_ARG;
    if (!(c->hfb.pp.rhosat > 0)) return MG_ERR_STATE;  // mg_set_pairing first
    if (!c->bas[MG_HF_BASIS].have_qn) return MG_ERR_STATE;
    return hfb_solve(c, info);
}

extern "C" int mg_get_hfb_block(mg_ctx* c, int b, double* rho, double* kappa, double* delta) {
    if (!c || b < 0 || b > 3 || !c->hfb.ready) return MG_ERR_ARG;
    const Hfb& H = c->hfb;
    const int N = 2 * H.hsz_h[b];
    const long off = (long)b * H.nmax * H.nmax;
    if (rho) MG_CUDA(cudaMemcpyAsync(rho, H.rho + off, (size_t)N * N * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    if (kappa) MG_CUDA(cudaMemcpyAsync(kappa, H.kappa + off, (size_t)N * N * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    if (delta) MG_CUDA(cudaMemcpyAsync(delta, H.delta + off, (size_t)N * N * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    MG_CUDA(cudaStreamSynchronize(c->stream));
    return N;
}

extern "C" int mg_get_pairing_field(mg_ctx* c, double* re, double* im, double* dfac) {
    if (!c || !c->hfb.ready) return MG_ERR_ARG;
    const long V = c->V;
    MG_TRY(copy_out(c, re, c->hfb.fre, 2 * V));
    MG_TRY(copy_out(c, im, c->hfb.fim, 2 * V));
    MG_TRY(copy_out(c, dfac, c->hfb.dfac, 2 * V));
    MG_CUDA(cudaStreamSynchronize(c->stream));
    return MG_OK;
}

extern "C" int mg_launch_count(mg_ctx* c, long long* count) {
    if (!c || !count) return MG_ERR_ARG;
    *count = c->launches;
    return MG_OK;
}

// ---------------------------------------------------------------------------
// Phase timer
// ---------------------------------------------------------------------------
namespace mg {

// The HF-basis DeriveAll on the side stream, after the work queued so far on
// the main stream.  The persistent tensor-core kernel takes a whole SM per
// CTA, so on the side stream it keeps to two thirds of the SMs: the Fermi
// search's kernels find the rest free (measured at 24^3, nwt=160: caps of
// 1/4, 1/3, 1/2 and 2/3 of the SMs gave 3.376, 3.358, 3.353 and 3.325 ms per
// mixed iteration).  The caller joins on ev_join.
int side_derive_hf(mg_ctx* c) {
    c->side_derive_pending = false;
    MG_CUDA(cudaEventRecord(c->ev_fork, c->stream));
    MG_CUDA(cudaStreamWaitEvent(c->side, c->ev_fork, 0));
    if (c->ph.on && c->ph.n > 0) {
        MG_CUDA(cudaEventRecord(c->ph.side[0], c->side));
        c->ph.side_used = true;
    }
    cudaStream_t main = c->stream;
    c->stream = c->side;
    c->tc_grid_cap = c->num_sms * 2 / 3;
    const int sd = derive_basis(c, MG_HF_BASIS);
    c->tc_grid_cap = 0;
    c->stream = main;
    MG_TRY(sd);
    if (c->ph.side_used) MG_CUDA(cudaEventRecord(c->ph.side[1], c->side));
    MG_CUDA(cudaEventRecord(c->ev_join, c->side));
    return MG_OK;
}

int phase_begin(mg_ctx* c) {
    if (!c->ph.on) return MG_OK;
    c->ph.n = 0;
    c->ph.side_used = false;
    MG_CUDA(cudaEventRecord(c->ph.ev[0], c->stream));
    c->ph.id[0] = -1;
    c->ph.n = 1;
    return MG_OK;
}

void phase_mark(mg_ctx* c, int id) {
    if (!c->ph.on || c->ph.n == 0 || c->ph.n >= mg_ctx::PhaseTimer::kMarks) return;
    if (cudaEventRecord(c->ph.ev[c->ph.n], c->stream) != cudaSuccess) return;
    c->ph.id[c->ph.n++] = id;
}

int phase_end(mg_ctx* c) {
    if (!c->ph.on || c->ph.n == 0) return MG_OK;
    auto& P = c->ph;
    MG_CUDA(cudaEventSynchronize(P.ev[P.n - 1]));
    for (int i = 1; i < P.n; ++i) {
        float ms = 0.0f;
        MG_CUDA(cudaEventElapsedTime(&ms, P.ev[i - 1], P.ev[i]));
        P.ms[P.id[i]] += ms;
    }
    if (P.side_used) {
        float ms = 0.0f;
        MG_CUDA(cudaEventSynchronize(P.side[1]));
        MG_CUDA(cudaEventElapsedTime(&ms, P.side[0], P.side[1]));
        P.ms[MG_PH_SIDE_DERIVE] += ms;
    }
    ++P.passes;
    P.n = 0;
    return MG_OK;
}

}  // namespace mg

extern "C" int mg_set_phase_timing(mg_ctx* c, int on) {
    if (!c) return MG_ERR_ARG;
    auto& P = c->ph;
    if (on && !P.ev[0]) {
        for (cudaEvent_t& e : P.ev) MG_CUDA(cudaEventCreate(&e));
        for (cudaEvent_t& e : P.side) MG_CUDA(cudaEventCreate(&e));
    }
    P.on = on != 0;
    P.n = 0;
    P.passes = 0;
    for (double& m : P.ms) m = 0.0;
    return MG_OK;
}

extern "C" int mg_get_phase_times(mg_ctx* c, double* ms, int n, long long* passes) {
    if (!c || !ms || n < MG_PH_COUNT) return MG_ERR_ARG;
    for (int k = 0; k < MG_PH_COUNT; ++k) ms[k] = c->ph.ms[k];
    if (passes) *passes = c->ph.passes;
    return MG_OK;
}

extern "C" int mg_iterate(mg_ctx* c, int n_iter, double dt, double momentum,
                          mg_energy_terms* out) {
    // Evolve loop body, src/Main.f90:255-328 (HF: SolvePairing = NaiveFill)
    if (!c || n_iter < 0) return MG_ERR_ARG;
    const bool hfb = c->p.pairing == MG_PAIRING_HFB;
    int st = MG_OK;
    for (int k = 0; k < n_iter; ++k) {
        ++c->iteration;
        MG_TRY(phase_begin(c));
        // AlternateStep while an alternating constraint was active at the
        // last check (src/Main.f90:261-263)
        if (c->cons.alternate_check) MG_TRY(alternate_step(c));
        MG_TRY(mg_grad_desc(c, dt, momentum));
        phase_mark(c, MG_PH_GRAD_DESC);
        if (hfb) {
            // DeriveAll of the HF basis needs only the new HF spinors: it runs
            // on the side stream, forked by the pairing step once its mesh
            // contractions are done (side_derive_hf), beside the Fermi search
            // and the canonical basis; the canonical basis follows.
            c->side_derive_pending = true;
            const int sp = mg_solve_pairing(c, nullptr);
            if (c->side_derive_pending) MG_TRY(side_derive_hf(c));   // not forked
            MG_TRY(sp);
            MG_CUDA(cudaStreamWaitEvent(c->stream, c->ev_join, 0));
            MG_TRY(derive_basis(c, MG_CAN_BASIS));
        } else {
            MG_TRY(mg_hf_fill(c));
            phase_mark(c, MG_PH_CANONICAL);
            MG_TRY(mg_derive_all(c));
        }
        phase_mark(c, MG_PH_DERIVE);
        c->cons.alternate_check = any_alternating(c);   // src/Main.f90:274
        // canonical single-particle energies with the previous potentials
        // (src/Main.f90:282-289)
        if (hfb) MG_TRY(hpsi_basis(c, MG_CAN_BASIS, nullptr, false, 0.0, 0.0));
        phase_mark(c, MG_PH_HPSI_CAN);
        MG_TRY(save_density_history(c));
        MG_TRY(densities(c));
        MG_TRY(mix_densities(c));
        phase_mark(c, MG_PH_DENSITIES);
        MG_TRY(moments(c));
        readjust_moments(c, c->iteration);   // src/Main.f90:299-304
        phase_mark(c, MG_PH_MOMENTS);
        st = mg_construct_potentials(c, nullptr);
        if (st < 0) return st;
        phase_mark(c, MG_PH_POTENTIALS);
        // CompEnergy every pass (src/Main.f90:309): it also keeps the energy
        // history of the convergence check
        mg_energy_terms e{};
        // the tensor-core status word comes back with the energy's readback
        if (k == n_iter - 1) MG_TRY(tc_status_async(c));
        MG_TRY(energy(c, out ? out : &e));
        phase_mark(c, MG_PH_ENERGY);
        MG_TRY(phase_end(c));
    }
    MG_TRY(n_iter > 0 ? tc_status_result(c) : tc_check(c));
    return st;
}

// ---------------------------------------------------------------------------
// ConvergenceCheck and the Evolve loop
// ---------------------------------------------------------------------------
static mg_convergence default_convergence() {
    // &GenInfo defaults (src/GenInfo.f90:54-55); EnergyPrec = 0.01E-08 is a
    // default-kind (single precision) literal
    return mg_convergence{(double)0.01e-8f, 1e-4, 1e-4};
}

extern "C" int mg_convergence_check(mg_ctx* c, const mg_convergence* prec, int* converged) {
    if (!c || !converged) return MG_ERR_ARG;
    const mg_convergence P = prec ? *prec : default_convergence();
    bool conv = moments_converged(c, P.moment_prec);
    const double E = c->total_energy;
    for (int i = 0; i < 7 && conv; ++i)   // ConverEnergy, src/Energy.f90:1458-1481
        conv = conv && std::fabs((c->old_energy[i] - E) / E) <= P.energy_prec;
    if (c->p.pairing == MG_PAIRING_HFB)   // ConverFermi: the history stays zero
        for (int it = 0; it < 2; ++it)
            if (std::fabs(c->hfb.fermi[it] - 0.0) > P.pairing_prec) conv = false;
    *converged = conv ? 1 : 0;
    if (E >= 0.0) {
        fprintf(stderr, "mocca_gpu: positive total energy (%.6f MeV)\n", E);
        return MG_ERR_STATE;
    }
    return MG_OK;
}

extern "C" int mg_evolve(mg_ctx* c, int max_iter, double dt, double momentum,
                         const mg_convergence* prec, int* iterations, int* converged,
                         mg_energy_terms* out) {
    if (!c || max_iter < 0) return MG_ERR_ARG;
    mg_energy_terms e{};
    int st = MG_OK, conv = 0, k = 0;
    while (k < max_iter) {
        ++k;
        const int s = mg_iterate(c, 1, dt, momentum, &e);
        if (s < 0) { st = s; break; }
        st = std::max(st, s);
        const int sc = mg_convergence_check(c, prec, &conv);
        if (sc < 0) { st = sc; break; }
        if (conv) break;
    }
    if (iterations) *iterations = k;
    if (converged) *converged = conv;
    if (out) *out = e;
    return st;
}
