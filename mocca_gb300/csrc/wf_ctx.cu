// wf_ctx.cu -- a device context and a version-1 MOCCa wavefunction file
// (include/mocca_wf.h): the state WriteMOCCa_v1 writes
// (src/InOut.f90:905-1046), gathered from the device, and the restart of
// ReadMOCCa_v1 + Input (src/InOut.f90:123-192, :1050-1416) into a context.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <vector>

#include "mg_internal.cuh"
#include "wf_format.h"

namespace mg {

namespace {

// index of a complex element (r, s) of block k of an m x n x blocks array,
// in doubles (re; im follows)
inline size_t cidx(long r, long s, long k, long m, long n) {
    return (size_t)(((k * n + s) * m + r) * 2);
}

// Pindex / Iindex position of a stored spwf (PrepareHFBModule,
// src/HFB.f90:263-266): P = (parity + 3) / 2, it = (isospin + 3) / 2
int block_of(const mg_wf_header& h, const int* qn) {
    const int P = h.pc ? (qn[1] + 3) / 2 - 1 : 0;
    const int it = (qn[0] + 3) / 2 - 1;
    return P + h.pindex * it;
}

// The time-odd density records WriteDensity writes without time reversal
// (src/Densities.f90:1214-1238): 1 j and rot j, 2 s, rot s and DerS, then,
// where the functional allocates them (src/Densities.f90:163-178), 4 lap s,
// div s and grad div s, 8 T, 16 F.
int odd_record_mask(const mg_ctx* c) {
    if (c->p.trc || !c->odd) return 0;
    int rec = 1 | 2;
    if (c->todd) {
        const mg_skyrme_b& B = c->B;
        if (B.B18 != 0.0 || B.B19 != 0.0 || B.B20 != 0.0 || B.B21 != 0.0) rec |= 4;
        if (B.B14 != 0.0 || B.B15 != 0.0) rec |= 8;
        if (B.B16 != 0.0 || B.B17 != 0.0) rec |= 16;
    }
    return rec;
}

// DerS as the reference's Density holds it after the iteration: the mixing
// operators carry DerS only beside lap s (src/Densities.f90:262-266,
// :328-333), so MixDensities' scheme 0 leaves it zero unless lap s is
// allocated; otherwise it is d_a s_m of the current s (the mixed
// derivatives equal the derivatives of the mixed s by linearity), with
// the arguments (P, -S, TS, 1), (P, -S, TS, 2), (P, S, TS, 1) of the
// components.  out: [it][m][a][V].
int wf_ders(mg_ctx* c, bool with_laps, double* out) {
    const long V = c->V;
    if (c->p.mixing_scheme == 0 && !with_laps) {
        std::fill(out, out + 18 * V, 0.0);
        return MG_OK;
    }
    double* d = nullptr;
    GridJob* jd = nullptr;
    std::vector<GridJob> jobs(6);
    auto done = [&](int st) {
        if (d) cudaFree(d);
        if (jd) cudaFree(jd);
        return st;
    };
    if (cudaMalloc(&d, 18 * V * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&jd, jobs.size() * sizeof(GridJob)) != cudaSuccess)
        return done(MG_ERR_CUDA);
    for (int it = 0; it < 2; ++it)
        for (int m = 0; m < 3; ++m) {
            GridJob& J = jobs[it * 3 + m];
            J = GridJob{};
            J.in = c->odd + (6 + it * 3 + m) * V;
            double* o = d + (it * 3 + m) * 3 * V;
            J.dx = o;
            J.dy = o + V;
            J.dz = o + 2 * V;
            const int ss = m == 2 ? 1 : -1, comp = m == 1 ? 2 : 1;
            for (int a = 0; a < 3; ++a) J.slot[a] = (int8_t)lag_slot(a, 1, ss, 1, comp);
        }
    if (cudaMemcpy(jd, jobs.data(), jobs.size() * sizeof(GridJob), cudaMemcpyHostToDevice) !=
        cudaSuccess)
        return done(MG_ERR_CUDA);
    int st = run_jobs(c, jd, 6);
    if (st == MG_OK &&
        (cudaMemcpyAsync(out, d, 18 * V * sizeof(double), cudaMemcpyDeviceToHost, c->stream) !=
             cudaSuccess ||
         cudaStreamSynchronize(c->stream) != cudaSuccess))
        st = MG_ERR_CUDA;
    return done(st);
}

// GuessHFBMatrices(0) (src/HFB.f90:3686-3718): blocksizes of the HFB
// indices (stored spwfs, then their time-reversed partners with
// opposite signature) and kappa = +-0.1 between opposite signatures, in
// the order the double loop leaves it.
void guess_hf_matrices(mg_wf& w, const std::vector<int>& qn, int nwt) {
    mg_wf_header& h = w.h;
    const int m = h.hfb_size;
    std::vector<std::vector<int>> members(h.pindex * h.iindex);
    for (int i = 0; i < m; ++i) {
        const int ii = i % nwt;
        members[block_of(h, &qn[4 * ii])].push_back(i);
    }
    for (size_t b = 0; b < members.size(); ++b)
        w.i[MG_WF_BLOCKSIZES][b] = (int)members[b].size();
    double* K = w.d[MG_WF_KAPPAHFB].data();
    for (size_t b = 0; b < members.size(); ++b) {
        const std::vector<int>& mb = members[b];
        const int N = (int)mb.size();
        auto sig = [&](int k) {
            const int i = mb[k], ii = i % nwt;
            int s = h.sc ? qn[4 * ii + 2] : 0;
            return i != ii ? -s : s;
        };
        for (int j = 0; j < N; ++j)
            for (int i = 0; i < N; ++i) {
                if (sig(j) * sig(i) > 0) continue;
                K[cidx(i, j, (long)b, m, m)] = 0.1;
                K[cidx(j, i, (long)b, m, m)] = -0.1;
            }
    }
}

// The HFB matrices of the last pairing step in the file's layout.
int hfb_matrices(mg_ctx* c, mg_wf& w) {
    Hfb& H = c->hfb;
    const mg_wf_header& h = w.h;
    const int m = h.hfb_size, nm = H.nmax, hmax = H.hmax;
    std::vector<double> X((size_t)4 * nm * nm), rho((size_t)4 * nm * nm),
        kap((size_t)4 * nm * nm), can((size_t)4 * hmax * hmax);
    MG_CUDA(cudaMemcpyAsync(X.data(), H.eT.X, X.size() * sizeof(double), cudaMemcpyDeviceToHost,
                            c->stream));
    MG_CUDA(cudaMemcpyAsync(rho.data(), H.rho, rho.size() * sizeof(double),
                            cudaMemcpyDeviceToHost, c->stream));
    MG_CUDA(cudaMemcpyAsync(kap.data(), H.kappa, kap.size() * sizeof(double),
                            cudaMemcpyDeviceToHost, c->stream));
    MG_CUDA(cudaMemcpyAsync(can.data(), H.cantr, can.size() * sizeof(double),
                            cudaMemcpyDeviceToHost, c->stream));
    MG_CUDA(cudaStreamSynchronize(c->stream));
    double *U = w.d[MG_WF_U].data(), *Vm = w.d[MG_WF_V].data();
    double *R = w.d[MG_WF_RHOHFB].data(), *K = w.d[MG_WF_KAPPAHFB].data();
    double* T = w.d[MG_WF_CANTRANSFO].data();
    int* cols = w.i[MG_WF_COLUMNS].data();
    // block b = it * 2 + (parity + 1) / 2 is the file's (P, it) = b % 2, b / 2
    for (int b = 0; b < 4; ++b) {
        const int hb = H.hsz_h[b], N = 2 * hb;
        w.i[MG_WF_BLOCKSIZES][b] = N;
        const double* Xb = X.data() + (size_t)b * nm * nm;
        // DiagonaliseHFBHamiltonian_Signature: the first N columns hold the
        // eigenvectors of the signature-reduced matrix (upper half in U,
        // lower in V), the next N their time-reversed partners
        for (int col = 0; col < N; ++col)
            for (int r = 0; r < hb; ++r) {
                const double up = Xb[(size_t)r * nm + col], lo = Xb[(size_t)(hb + r) * nm + col];
                U[cidx(r, col, b, m, 2 * m)] = up;
                Vm[cidx(hb + r, col, b, m, 2 * m)] = lo;
                U[cidx(hb + r, N + col, b, m, 2 * m)] = -up;
                Vm[cidx(r, N + col, b, m, 2 * m)] = lo;
            }
        // HFBColumns with signature (src/HFB.f90:1008-1019), 1-based
        for (int i = 0; i < hb; ++i) cols[(size_t)b * m + i] = 2 * N - i;
        for (int i = hb; i < N; ++i) cols[(size_t)b * m + i] = i + 1;
        const double* Rb = rho.data() + (size_t)b * nm * nm;
        const double* Kb = kap.data() + (size_t)b * nm * nm;
        for (int r = 0; r < N; ++r)
            for (int s = 0; s < N; ++s) {
                R[cidx(r, s, b, m, m)] = Rb[(size_t)r * N + s];
                K[cidx(r, s, b, m, m)] = Kb[(size_t)r * N + s];
            }
        // DiagonaliseRhoHFB with signature: the negative-signature
        // eigenvectors (shifted by -2) first, then the positive ones, each
        // ascending; with time reversal both halves share the vectors
        const double* Cb = can.data() + (size_t)b * hmax * hmax;
        for (int k = 0; k < hb; ++k)
            for (int r = 0; r < hb; ++r) {
                const double x = Cb[(size_t)r * hb + k];
                T[cidx(hb + r, k, b, m, m)] = x;
                T[cidx(r, hb + k, b, m, m)] = x;
            }
    }
    return MG_OK;
}

int from_context(mg_ctx* c, const char* force_name, mg_wf& w) {
    Basis& B = c->bas[MG_HF_BASIS];
    if (!B.have_qn) return MG_ERR_STATE;
    const bool hfb = c->p.pairing == MG_PAIRING_HFB;
    if (hfb && !c->hfb.ready) return MG_ERR_STATE;   // no pairing step yet
    const int nwt = c->p.nwt;
    const long V = c->V;
    mg_wf_header& h = w.h;
    h = mg_wf_header{};
    h.energy = c->total_energy;
    h.denergy = c->total_energy - c->old_energy[1];
    h.nx = c->p.nx;
    h.ny = c->p.ny;
    h.nz = c->p.nz;
    h.dx = c->p.dx;
    h.trc = c->p.trc != 0;
    h.pc = c->p.pc != 0;
    h.sc = c->p.sc != 0;
    h.tsc = c->p.tsc != 0;
    h.ic = 1;
    h.nwt = nwt;
    h.neutrons = c->p.neutrons;
    h.protons = c->p.protons;
    // Lagrange derivatives (MaxFDOrder = MaxFDLapOrder = -1) and the
    // Coulomb Laplacian's default order 2 (src/Derivatives.f90:67)
    h.fd_order = -1;
    h.fd_lap_order = -1;
    h.coulomb_lap_order = 2;
    if (force_name) {
        std::strncpy(h.force, force_name, sizeof(h.force) - 1);
        h.force[sizeof(h.force) - 1] = '\0';
    }
    const mg_force& f = c->f;
    const double sk[14] = {f.t0, f.x0, f.t1, f.x1, f.t2, f.x2, f.t3a,
                           f.x3a, f.yt3a, f.t3b, f.x3b, f.yt3b, f.wso, f.wsoq};
    std::copy(sk, sk + 14, h.skyrme);
    h.hbar = f.hbar;
    h.hbm[0] = h.hbm[1] = f.hbm;
    h.com1body = f.com1body;
    h.com2body = f.com2body;
    // B1 ... B21 in the record's order
    static_assert(sizeof(mg_skyrme_b) == 28 * sizeof(double), "B1 ... B21");
    std::memcpy(h.coef, &c->B, sizeof(mg_skyrme_b));
    if (hfb) {
        const mg_pairing_params& pp = c->hfb.pp;
        h.pairing_type = 2;
        for (int k = 0; k < 2; ++k) {
            h.pairing_strength[k] = pp.strength[k];
            h.pairing_alpha[k] = pp.alpha[k];
            h.pairing_cut[k] = pp.cut[k];
        }
        h.has_cutoffs = 1;
    } else {
        // the pairing module's defaults (src/PairingInteraction.f90:23-94)
        h.pairing_type = 0;
        h.pairing_alpha[0] = h.pairing_alpha[1] = 1.0;
        h.pairing_cut[0] = h.pairing_cut[1] = 5.0;
    }
    h.fermi[0] = c->hfb.fermi[0];
    h.fermi[1] = c->hfb.fermi[1];
    for (int k = 0; k < 3; ++k) h.omega[k] = c->p.omega[k];
    h.odd_records = odd_record_mask(c);
    h.has_jmunu = c->tensor ? 1 : 0;
    h.n_moments = 0;
    for (const MomentConstraint& k : c->cons.list) h.n_moments += k.type != 0;
    // an HF context writes GuessHFBMatrices(0)'s CanTransfo(HFBSize,HFBSize,2,2)
    h.can_blocks = hfb ? 0 : 4;
    wf_derive_shapes(h);
    wf_allocate(w);
    // spwfs
    {
        std::vector<double*> ptr(nwt);
        for (int i = 0; i < nwt; ++i) ptr[i] = w.d[MG_WF_GRIDS].data() + (size_t)i * 4 * V;
        MG_TRY(mg_download_spinors(c, MG_HF_BASIS, ptr.data(), 0, nwt));
        std::vector<double> occ(nwt), e(nwt), disp(nwt), J(3 * (size_t)nwt);
        MG_TRY(mg_get_occupations(c, MG_HF_BASIS, occ.data()));
        MG_TRY(mg_get_energies(c, MG_HF_BASIS, e.data(), disp.data()));
        MG_TRY(mg_angular_momentum(c, MG_HF_BASIS, J.data()));
        for (int i = 0; i < nwt; ++i) {
            const double* g = ptr[i];
            double nrm = 0.0;
            for (long v = 0; v < 4 * V; ++v) nrm += g[v] * g[v];
            double* o = w.d[MG_WF_SPWF_REAL].data() + (size_t)i * 7;
            o[0] = occ[i];
            o[1] = e[i];
            o[2] = disp[i];
            o[3] = nrm * c->dv;
            o[4] = J[3 * (size_t)i];
            o[5] = J[3 * (size_t)i + 1];
            o[6] = J[3 * (size_t)i + 2];
            const int* q = &B.h_qn[4 * (size_t)i];
            int* n = w.i[MG_WF_SPWF_INT].data() + (size_t)i * 5;
            n[0] = q[0];   // isospin
            n[1] = q[3];   // time simplex
            n[2] = q[1];   // parity
            n[3] = q[2];   // signature
            n[4] = 1;      // time reversal (INITWF, src/InOut.f90:1465)
        }
    }
    // densities
    MG_TRY(mg_get_densities(c, w.d[MG_WF_RHO].data(), w.d[MG_WF_TAU].data(),
                            w.d[MG_WF_NABLAJ].data(), w.d[MG_WF_DERRHO].data(),
                            w.d[MG_WF_LAPRHO].data()));
    if (h.has_jmunu) MG_TRY(mg_get_jmunu(c, w.d[MG_WF_JMUNU].data()));
    if (h.odd_records & 1) {
        double* o1 = w.d[MG_WF_ODD1].data();
        double* o2 = w.d[MG_WF_ODD2].data();
        MG_TRY(mg_get_time_odd(c, o1, o2, o1 + 6 * V, o2 + 6 * V, nullptr, nullptr, nullptr));
        MG_TRY(wf_ders(c, (h.odd_records & 4) != 0, o2 + 12 * V));
    }
    if (h.odd_records & (4 | 8 | 16)) {
        // lap s, div s (never assigned by the reference: zero), grad div s; T; F
        double* o3 = (h.odd_records & 4) ? w.d[MG_WF_ODD3].data() : nullptr;
        if (o3) std::fill(o3 + 6 * V, o3 + 8 * V, 0.0);
        MG_TRY(mg_get_time_odd_tensor(c, (h.odd_records & 8) ? w.d[MG_WF_ODD4].data() : nullptr,
                                      (h.odd_records & 16) ? w.d[MG_WF_ODD5].data() : nullptr,
                                      o3, o3 ? o3 + 8 * V : nullptr, nullptr, nullptr, nullptr));
    }
    // pairing and the HFB matrices
    if (hfb) {
        MG_CUDA(cudaMemcpyAsync(w.d[MG_WF_CUTOFFS].data(), c->hfb.pcut, nwt * sizeof(double),
                                cudaMemcpyDeviceToHost, c->stream));
        MG_CUDA(cudaStreamSynchronize(c->stream));
        MG_TRY(hfb_matrices(c, w));
    } else {
        guess_hf_matrices(w, B.h_qn, nwt);
    }
    // constrained moments (WriteMoment, Isoswitch 1: scalars twice)
    int q = 0;
    for (const MomentConstraint& k : c->cons.list) {
        if (k.type == 0) continue;
        int* mi = w.i[MG_WF_MOMENT_INT].data() + (size_t)q * 5;
        mi[0] = k.type;
        mi[1] = 1;
        mi[2] = k.l;
        mi[3] = k.m;
        mi[4] = 0;
        double* mr = w.d[MG_WF_MOMENT_REAL].data() + (size_t)q * 22;
        mr[0] = mr[1] = k.intensity;
        mr[2] = mr[3] = k.constraint;
        mr[4] = mr[5] = k.true_constraint;
        mr[6] = k.value[0];
        mr[7] = k.value[1];
        for (int j = 0; j < 7; ++j) {
            mr[8 + 2 * j] = k.old_iso[j][0];
            mr[9 + 2 * j] = k.old_iso[j][1];
        }
        ++q;
    }
    return MG_OK;
}

int to_context(mg_ctx* c, const mg_wf& w) {
    const mg_wf_header& h = w.h;
    const mg_params& p = c->p;
    // the reference transforms other meshes, symmetries and nwt
    // (TransformInput, src/Transform.f90); this restart takes the same ones
    if (h.nx != p.nx || h.ny != p.ny || h.nz != p.nz || std::fabs(h.dx - p.dx) > 1e-12 * p.dx ||
        h.nwt != p.nwt || !h.trc != !p.trc || !h.pc != !p.pc || !h.sc != !p.sc ||
        !h.tsc != !p.tsc || !h.ic)
        return MG_ERR_ARG;
    const bool hfb = p.pairing == MG_PAIRING_HFB;
    if (hfb && (c->hfb.ready || !(c->hfb.pp.rhosat > 0))) return MG_ERR_STATE;
    const int nwt = p.nwt;
    const long V = c->V;
    std::vector<int> qn(4 * (size_t)nwt);
    std::vector<double> occ(nwt), e(nwt);
    std::vector<const double*> ptr(nwt);
    for (int i = 0; i < nwt; ++i) {
        const int* n = w.i[MG_WF_SPWF_INT].data() + (size_t)i * 5;
        qn[4 * i + 0] = n[0];
        qn[4 * i + 1] = n[2];
        qn[4 * i + 2] = n[3];
        qn[4 * i + 3] = n[1];
        const double* r = w.d[MG_WF_SPWF_REAL].data() + (size_t)i * 7;
        occ[i] = r[0];
        e[i] = r[1];
        ptr[i] = w.d[MG_WF_GRIDS].data() + (size_t)i * 4 * V;
    }
    // HFB matrices: checked against the blocks the quantum numbers give
    // before anything changes on the device
    int nb[4] = {0, 0, 0, 0};
    if (hfb) {
        for (int i = 0; i < nwt; ++i) {
            if (qn[4 * i + 1] == 0) return MG_ERR_ARG;   // HFB needs parity blocks
            nb[((qn[4 * i] + 1) / 2) * 2 + (qn[4 * i + 1] + 1) / 2] += 2;
        }
        for (int b = 0; b < 4; ++b)
            if (w.i[MG_WF_BLOCKSIZES][b] != nb[b]) return MG_ERR_ARG;
    }
    MG_TRY(mg_upload_spinors(c, MG_HF_BASIS, ptr.data(), qn.data(), 0, nwt));
    MG_TRY(mg_set_occupations(c, MG_HF_BASIS, occ.data()));
    MG_TRY(mg_set_energies(c, MG_HF_BASIS, e.data()));
    MG_TRY(mg_set_densities(c, w.d[MG_WF_RHO].data(), w.d[MG_WF_TAU].data(),
                            w.d[MG_WF_NABLAJ].data(), w.d[MG_WF_DERRHO].data(),
                            w.d[MG_WF_LAPRHO].data()));
    // the time-odd densities as ReadDensity takes them
    // (src/Densities.f90:1280-1340): from the records that are there, else
    // zero (DerS and div s are not kept: the next densities recompute them)
    if (!p.trc && c->odd) {
        std::vector<double> o((size_t)c->odd_len * V, 0.0);
        auto put = [&](int field, long src_off, long dst_off, long n) {
            if (w.d[field].size() >= (size_t)(src_off + n))
                std::copy(w.d[field].begin() + src_off, w.d[field].begin() + src_off + n,
                          o.begin() + dst_off);
        };
        put(MG_WF_ODD1, 0, 0, 6 * V);             // j
        put(MG_WF_ODD1, 6 * V, 12 * V, 6 * V);    // rot j
        put(MG_WF_ODD2, 0, 6 * V, 6 * V);         // s
        put(MG_WF_ODD2, 6 * V, 18 * V, 6 * V);    // rot s
        if (c->todd) {
            put(MG_WF_ODD4, 0, 24 * V, 6 * V);        // T
            put(MG_WF_ODD5, 0, 30 * V, 6 * V);        // F
            put(MG_WF_ODD3, 0, 36 * V, 6 * V);        // lap s
            put(MG_WF_ODD3, 8 * V, 42 * V, 6 * V);    // grad div s
        }
        MG_CUDA(cudaMemcpyAsync(c->odd, o.data(), o.size() * sizeof(double),
                                cudaMemcpyHostToDevice, c->stream));
        MG_CUDA(cudaStreamSynchronize(c->stream));
    }
    // JMuNu as ReadDensity takes it: from the file when there, else zero
    if (c->tensor) {
        std::vector<double> zero;
        const double* j = w.d[MG_WF_JMUNU].data();
        if (!h.has_jmunu) {
            zero.assign((size_t)18 * V, 0.0);
            j = zero.data();
        }
        MG_TRY(mg_set_jmunu(c, j));
    }
    if (hfb) {
        Hfb& H = c->hfb;
        const int m = h.hfb_size;
        for (int b = 0; b < 4; ++b) {
            const int N = nb[b];
            H.restart_n[b] = N;
            H.restart_rho[b].assign((size_t)N * N, 0.0);
            H.restart_kappa[b].assign((size_t)N * N, 0.0);
            for (int r = 0; r < N; ++r)
                for (int s = 0; s < N; ++s) {
                    H.restart_rho[b][(size_t)r * N + s] = w.d[MG_WF_RHOHFB][cidx(r, s, b, m, m)];
                    H.restart_kappa[b][(size_t)r * N + s] =
                        w.d[MG_WF_KAPPAHFB][cidx(r, s, b, m, m)];
                }
        }
        H.restart_pending = true;
        H.fermi[0] = H.fermi_prev[0] = h.fermi[0];
        H.fermi[1] = H.fermi_prev[1] = h.fermi[1];
    }
    // constrained moments matched by (l, m), as ReadMoment's FindMoment
    // (src/Moments.f90:3384-3386); the running targets continue
    // (ContinueMoment, src/Moments.f90:2277)
    for (int q = 0; q < h.n_moments; ++q) {
        const int* mi = w.i[MG_WF_MOMENT_INT].data() + (size_t)q * 5;
        const double* mr = w.d[MG_WF_MOMENT_REAL].data() + (size_t)q * 22;
        if (mi[4] != 0) continue;   // imaginary parts are not constrained here
        for (MomentConstraint& k : c->cons.list) {
            if (k.l != mi[2] || k.m != mi[3]) continue;
            k.type = mi[0] == 3 ? 2 : mi[0];   // legacy type 3 reads as 2
            k.intensity = mr[0];
            k.constraint = mr[2];
            k.true_constraint = mr[4];
            k.value[0] = mr[6];
            k.value[1] = mr[7];
            for (int j = 0; j < 7; ++j) {
                k.old_iso[j][0] = mr[8 + 2 * j];
                k.old_iso[j][1] = mr[9 + 2 * j];
                k.old_value[j] = mr[8 + 2 * j] + mr[9 + 2 * j];
            }
            k.started = true;
        }
    }
    return MG_OK;
}

}  // namespace

}  // namespace mg

extern "C" int mg_wf_from_context(mg_ctx* c, const char* force_name, mg_wf** out) {
    using namespace mg;
    if (!c || !out) return MG_ERR_ARG;
    *out = nullptr;
    std::unique_ptr<mg_wf> w(new (std::nothrow) mg_wf());
    if (!w) return MG_ERR_CUDA;
    const int st = from_context(c, force_name, *w);
    if (st != MG_OK) return st;
    *out = w.release();
    return MG_OK;
}

extern "C" int mg_wf_to_context(mg_ctx* c, const mg_wf* w) {
    using namespace mg;
    if (!c || !w) return MG_ERR_ARG;
    return to_context(c, *w);
}
