// energy.cu -- total energy, FP64 (CompEnergy, src/Energy.f90:62-179).
//
// Device side: per-spwf <psi|lap psi> of the density basis (CompKinetic,
// :1426-1456) and block partials of the mesh integrals of compSkyrme
// (:623-860, time-even terms, the J^2 ones included) and of the Coulomb
// direct / Slater exchange energies (src/Coulomb.f90:215-253).  Host side:
// the block partials are added in block order and combined exactly as
// CompEnergy / SpwfEnergy do.
#include <cmath>
#include <cstring>

#include "df.cuh"
#include "mg_internal.cuh"

namespace mg {

namespace {

constexpr int kThreads = 256;
constexpr int kTerms = 26;

// per-spwf dot products over 4V, block partials (b as double-float pairs when
// kBdf: the Laplacians of the mixed form)
template <bool kBdf>
__global__ void __launch_bounds__(kThreads)
k_dots(const double* __restrict__ a, const double* __restrict__ b, long V4,
       double* __restrict__ part) {
    const int i = blockIdx.y;
    double s = 0.0;
    if (kBdf) {
        // double-float products and sums (FP32 pipe), FP64 once per thread
        float sh = 0.f, sl = 0.f;
        const float2* bp = reinterpret_cast<const float2*>(b) + (long)i * V4;
        for (long o = (long)blockIdx.x * kThreads + threadIdx.x; o < V4;
             o += (long)gridDim.x * kThreads)
            df_acc(sh, sl, df_split(a[(long)i * V4 + o]), df_ld(bp + o));
        s = df_to_fast(df_norm(dfl{sh, sl}));
    } else {
        for (long o = (long)blockIdx.x * kThreads + threadIdx.x; o < V4;
             o += (long)gridDim.x * kThreads)
            s = fma(a[(long)i * V4 + o], b[(long)i * V4 + o], s);
    }
    __shared__ double red[kThreads / 32];
    for (int q = 16; q > 0; q >>= 1) s += __shfl_xor_sync(0xffffffffu, s, q);
    if (threadIdx.x % 32 == 0) red[threadIdx.x / 32] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int q = 0; q < kThreads / 32; ++q) t += red[q];
        part[(long)i * gridDim.x + blockIdx.x] = t;
    }
}

struct ECoef {
    double B4, B6, B8a, B8b, B9q, byt3a, byt3b, B7b;
};

__global__ void __launch_bounds__(kThreads)
k_energy_partial(const double* __restrict__ rho, const double* __restrict__ tau,
                 const double* __restrict__ laprho, const double* __restrict__ nablaj,
                 const double* __restrict__ coul, const double* __restrict__ jm, ECoef k, long V,
                 double* __restrict__ part) {
    double acc[kTerms];
#pragma unroll
    for (int q = 0; q < kTerms; ++q) acc[q] = 0.0;
    for (long v = (long)blockIdx.x * kThreads + threadIdx.x; v < V; v += (long)gridDim.x * kThreads) {
        const double rn = rho[v], rp = rho[V + v];
        const double rt = rn + rp;
        const double tt = tau[v] + tau[V + v];
        const double lt = laprho[v] + laprho[V + v];
        const double jt = nablaj[v] + nablaj[V + v];
        const double pa = pow(rt, k.byt3a);
        acc[0] += rt * rt;                 // B1
        acc[1] += rt * tt;                 // B3
        acc[2] += rt * lt;                 // B5
        acc[3] += pow(rt, 2 + k.byt3a);    // B7a
        acc[4] += rt * jt;                 // B9
        if (k.B7b != 0.0) acc[5] += pow(rt, 2 + k.byt3b);
#pragma unroll
        for (int it = 0; it < 2; ++it) {
            const double r = rho[it * V + v];
            acc[6 + it] += r * r;                       // B2
            acc[8 + it] += r * tau[it * V + v];         // B4
            acc[10 + it] += r * laprho[it * V + v];     // B6
            acc[12 + it] += r * r * pa;                 // B8a
            acc[14 + it] += r * nablaj[it * V + v];     // B9q
            if (k.B8b != 0.0) acc[16 + it] += r * r * pow(rt, k.byt3b);
        }
        acc[18] += rp * coul[v];                        // Coulomb direct
        acc[19] += rp * pow(rp, 1 / 3.0);               // Slater exchange
        if (jm) {
            // J^2 terms 19, 20, 23-26 (src/Energy.f90:763-810), J(m, n) of
            // isospin q at jm[((q * 3 + n) * 3 + m) * V]
            double tr[2] = {0.0, 0.0};
            for (int m = 0; m < 3; ++m)
                for (int n = 0; n < 3; ++n) {
                    const double j0 = jm[((0 * 3 + n) * 3 + m) * V + v];
                    const double j1 = jm[((1 * 3 + n) * 3 + m) * V + v];
                    const double t0 = jm[((0 * 3 + m) * 3 + n) * V + v];   // J(n, m)
                    const double t1 = jm[((1 * 3 + m) * 3 + n) * V + v];
                    const double jt = j0 + j1;
                    acc[20] += jt * jt;
                    acc[24] += jt * (t0 + t1);
                    acc[21] += j0 * j0 + j1 * j1;
                    acc[25] += j0 * t0 + j1 * t1;
                    if (m == n) { tr[0] += j0; tr[1] += j1; }
                }
            acc[22] += (tr[0] + tr[1]) * (tr[0] + tr[1]);
            acc[23] += tr[0] * tr[0] + tr[1] * tr[1];
        }
    }
    __shared__ double red[kThreads / 32];
    for (int q = 0; q < kTerms; ++q) {
        double s = acc[q];
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        __syncthreads();
        if (threadIdx.x % 32 == 0) red[threadIdx.x / 32] = s;
        __syncthreads();
        if (threadIdx.x == 0) {
            double t = 0.0;
            for (int w = 0; w < kThreads / 32; ++w) t += red[w];
            part[(long)blockIdx.x * kTerms + q] = t;
        }
    }
}

}  // namespace

static int dots_chunks(long V4) { return std::max(1, std::min(64, div_up(V4, kThreads * 8))); }

// block partials of the nwt dot products <a_i|b_i> into out[i * nch + chunk]
static int launch_dots(mg_ctx* c, const double* a, const double* b, bool b_df, double* out) {
    const long V4 = 4 * c->V;
    const int nch = dots_chunks(V4);
    if (b_df)
        k_dots<true><<<dim3(nch, c->p.nwt), kThreads, 0, c->stream>>>(a, b, V4, out);
    else
        k_dots<false><<<dim3(nch, c->p.nwt), kThreads, 0, c->stream>>>(a, b, V4, out);
    MG_LAUNCHED(c);
    return MG_OK;
}

// nwt dot products <a_i|b_i> * dv of a basis into host array out.
int basis_dots(mg_ctx* c, const double* a, const double* b, double* out, bool b_df) {
    const long V4 = 4 * c->V;
    const int nch = dots_chunks(V4);
    MG_TRY(launch_dots(c, a, b, b_df, c->red));
    std::vector<double> h((size_t)nch * c->p.nwt);
    MG_CUDA(cudaMemcpyAsync(h.data(), c->red, h.size() * sizeof(double), cudaMemcpyDeviceToHost,
                            c->stream));
    MG_CUDA(cudaStreamSynchronize(c->stream));
    for (int i = 0; i < c->p.nwt; ++i) {
        double s = 0.0;
        for (int q = 0; q < nch; ++q) s += h[(size_t)i * nch + q];
        out[i] = s * c->dv;
    }
    return MG_OK;
}

int energy(mg_ctx* c, mg_energy_terms* out) {
    std::memset(out, 0, sizeof(*out));
    const int db = c->p.pairing == MG_PAIRING_HFB ? MG_CAN_BASIS : MG_HF_BASIS;
    Basis& D = c->bas[db];
    const int nwt = c->p.nwt;
    const long V = c->V;
    const mg_skyrme_b& B = c->B;
    // the per-spwf <psi|lap psi> partials and the mesh-integral partials go
    // to two regions of the reduction table and come back in one read
    const long V4 = 4 * V;
    const int nch = dots_chunks(V4);
    const size_t ndots = (size_t)nch * nwt;
    launch_dots(c, D.psi, D.lap, D.der_df, c->red);
    std::vector<double> occ(nwt), e(nwt);
    MG_CUDA(cudaMemcpyAsync(occ.data(), D.occ, nwt * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    MG_CUDA(cudaMemcpyAsync(e.data(), D.e, nwt * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    const int nblk = std::max(1, std::min(2 * c->num_sms, div_up(V, kThreads)));
    if (ndots + (size_t)nblk * kTerms > c->red_len) return MG_ERR_STATE;
    ECoef k{B.B4, B.B6, B.B8a, B.B8b, B.B9q, B.byt3a, B.byt3b, B.B7b};
    k_energy_partial<<<nblk, kThreads, 0, c->stream>>>(c->rho, c->tau, c->laprho, c->nablaj,
                                                       c->coulomb,
                                                       c->tensor ? c->jmunu : nullptr, k, V,
                                                       c->red + ndots);
    MG_LAUNCHED(c);
    std::vector<double> all(ndots + (size_t)nblk * kTerms);
    MG_CUDA(cudaMemcpyAsync(all.data(), c->red, all.size() * sizeof(double),
                            cudaMemcpyDeviceToHost, c->stream));
    MG_CUDA(cudaStreamSynchronize(c->stream));
    std::vector<double> ip(nwt);
    for (int i = 0; i < nwt; ++i) {
        double s = 0.0;
        for (int q = 0; q < nch; ++q) s += all[(size_t)i * nch + q];
        ip[i] = s * c->dv;
    }
    const double* part = all.data() + ndots;
    double S[kTerms] = {0};
    for (int b = 0; b < nblk; ++b)
        for (int q = 0; q < kTerms; ++q) S[q] += part[(size_t)b * kTerms + q];

    double kin[2] = {0, 0};
    for (int l = 0; l < nwt; ++l) {
        const int it = (D.h_qn[4 * l] + 3) / 2 - 1;
        kin[it] = kin[it] + occ[l] * ip[l];
    }
    for (int it = 0; it < 2; ++it) out->kinetic[it] = -kin[it] / 2.0 * c->f.hbm;
    double* t = out->skyrme;
    t[0] = B.B1 * S[0];
    t[1] = B.B2 * (S[6] + S[7]);
    t[2] = B.B3 * S[1];
    t[3] = B.B4 * S[8] + B.B4 * S[9];
    t[6] = B.B5 * S[2];
    t[7] = B.B6 * S[10] + B.B6 * S[11];
    t[8] = B.B7a * S[3];
    t[9] = B.B8a * S[12] + B.B8a * S[13];
    t[10] = B.B9 * S[4];
    t[11] = B.B9q * S[14] + B.B9q * S[15];
    t[32] = B.B7b * S[5];
    t[33] = B.B8b * S[16] + B.B8b * S[17];
    if (c->tensor) {
        t[18] = B.B14 * S[20];
        t[19] = B.B15 * S[21];
        t[22] = B.B16 * S[22];
        t[23] = B.B17 * S[23];
        t[24] = B.B16 * S[24];
        t[25] = B.B17 * S[25];
    }
    if (!c->p.trc) MG_TRY(time_odd_energy(c, t));
    for (int q = 0; q < 36; ++q) t[q] *= c->dv;
    double sk = 0.0;
    for (int q = 0; q < 36; ++q) sk += t[q];
    const double pi = 4.0 * std::atan2(1.0, 1.0);
    double ec = 0.0, ex = 0.0;
    if (c->p.coulomb_solver != 0) {
        ec = S[18] * c->dv * 0.5;
        if (c->f.cexchange >= 1) ex = -std::pow(3 / pi, 1 / 3.0) * c->f.e2 * 0.75 * c->dv * S[19];
    }
    out->coulomb = ec;
    out->coulomb_exchange = ex;
    if (c->f.com1body > 0) {
        const double mt = c->p.neutrons * c->f.nucleonmass[0] + c->p.protons * c->f.nucleonmass[1];
        for (int it = 0; it < 2; ++it) out->com[0][it] = -out->kinetic[it] * c->f.nucleonmass[it] / mt;
    }
    out->pairing[0] = c->pairing_energy[0];
    out->pairing[1] = c->pairing_energy[1];
    const double com = out->com[0][0] + out->com[1][0] + out->com[0][1] + out->com[1][1];
    out->total = sk + (out->kinetic[0] + out->kinetic[1]) + ec + com + ex +
                 (out->pairing[0] + out->pairing[1]);
    // OldEnergy shifts and takes the previous TotalEnergy (src/Energy.f90:93-98)
    for (int i = 6; i > 0; --i) c->old_energy[i] = c->old_energy[i - 1];
    c->old_energy[0] = c->total_energy;
    c->total_energy = out->total;
    double sp = 0.0;
    for (int i = 0; i < nwt; ++i) sp += occ[i] * e[i];
    sp = 0.5 * (sp + (out->kinetic[0] + out->kinetic[1])) -
         0.5 * B.byt3a * ((t[8] + t[9]) + (t[16] + t[17])) -
         0.5 * B.byt3b * ((t[32] + t[33]) + (t[34] + t[35])) + ex / 3.0;
    sp = sp + (out->pairing[0] + out->pairing[1]);
    if (c->f.com1body > 0) sp = sp + (out->com[0][0] + out->com[0][1]) / 2.0;
    if (c->f.com2body == 1) sp = sp + (out->com[1][0] + out->com[1][1]);
    out->sp_energy = sp;
    return MG_OK;
}

}  // namespace mg
