// density.cu -- density accumulation over the density basis, FP64 (double-float
// in the mixed form).
//
// Replaces ComputeDensity (src/Densities.f90:431-550) for time-reversal
// invariant functionals without tensor / N2LO terms:
//   rho_q    += v^2 |psi|^2                      GetDensity src/Spwf.f90:536-546
//   tau_q    += v^2 sum_m |d_m psi|^2             GetTau     :1897-1909
//   divJ_q   += v^2 sum eps_ijk Im(d_i psi^+ sigma_k d_j psi)  GetNablaJ :2206-2243
// then grad rho and lap rho with the Lagrange kernels (deriv.cu).
// Grid = (point chunks) x (spwf groups): each thread walks its group's spwfs
// in index order for one mesh point (16 doubles per spwf, coalesced along
// x), writes six group partials, and k_dens_reduce adds the groups in order,
// so the result is deterministic.
#include "df.cuh"
#include "mg_internal.cuh"

namespace mg {

namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ void pauli(const double* p, int dir, double* o) {
    if (dir == 1) { o[0] = p[2]; o[1] = p[3]; o[2] = p[0]; o[3] = p[1]; }
    else if (dir == 2) { o[0] = p[3]; o[1] = -p[2]; o[2] = -p[1]; o[3] = p[0]; }
    else { o[0] = p[0]; o[1] = p[1]; o[2] = -p[2]; o[3] = -p[3]; }
}
__device__ __forceinline__ double imag_mult(const double* a, const double* b) {
    return a[0] * b[1] - a[1] * b[0] + a[2] * b[3] - a[3] * b[2];
}

__global__ void __launch_bounds__(kThreads)
k_dens_partial(const double* __restrict__ psi, const double* __restrict__ der,
               const double* __restrict__ occ, const int* __restrict__ qn, int nwt,
               int per_group, long V, double* __restrict__ part) {
    const long v = (long)blockIdx.x * kThreads + threadIdx.x;
    const int g = blockIdx.y;
    if (v >= V) return;
    double acc[2][3] = {{0, 0, 0}, {0, 0, 0}};
    const int i0 = g * per_group, i1 = min(nwt, i0 + per_group);
    for (int i = i0; i < i1; ++i) {
        const double o = occ[i];
        if (o == 0.0) continue;
        const int it = (qn[4 * i] + 3) / 2 - 1;
        const double* ps = psi + (long)i * 4 * V;
        const double* dr = der + (long)i * 12 * V;
        double p[4], d[3][4];
#pragma unroll
        for (int l = 0; l < 4; ++l) {
            p[l] = ps[l * V + v];
#pragma unroll
            for (int m = 0; m < 3; ++m) d[m][l] = dr[(m * 4 + l) * V + v];
        }
        const double den = p[0] * p[0] + p[1] * p[1] + p[2] * p[2] + p[3] * p[3];
        double t = 0.0;
#pragma unroll
        for (int m = 0; m < 3; ++m)
            t = t + (d[m][0] * d[m][0] + d[m][1] * d[m][1] + d[m][2] * d[m][2] + d[m][3] * d[m][3]);
        // (i, j, k, eps_ijk) in the order of GetNablaJ
        double nj = 0.0, s[4];
        pauli(d[1], 3, s); nj = nj + imag_mult(d[0], s);
        pauli(d[2], 2, s); nj = nj - imag_mult(d[0], s);
        pauli(d[1], 1, s); nj = nj - imag_mult(d[2], s);
        pauli(d[0], 2, s); nj = nj + imag_mult(d[2], s);
        pauli(d[0], 3, s); nj = nj - imag_mult(d[1], s);
        pauli(d[2], 1, s); nj = nj + imag_mult(d[1], s);
        acc[it][0] = fma(o, den, acc[it][0]);
        acc[it][1] = fma(o, t, acc[it][1]);
        acc[it][2] = fma(o, nj, acc[it][2]);
    }
    double* pg = part + (long)g * 6 * V;
#pragma unroll
    for (int it = 0; it < 2; ++it)
#pragma unroll
        for (int q = 0; q < 3; ++q) pg[(q * 2 + it) * V + v] = acc[it][q];
}

// Mixed form: the same sums in double-float from double-float derivatives
// (psi split from its FP64 bits); group partials leave as FP64.
__device__ __forceinline__ void imag_acc(float& sh, float& sl, const dfl* a, const dfl* b,
                                         float sgn) {
    // sgn * (a0 b1 - a1 b0 + a2 b3 - a3 b2)
    const dfl s{sgn, 0.0f}, m{-sgn, 0.0f};
    df_acc(sh, sl, df_mul(s, a[0]), b[1]);
    df_acc(sh, sl, df_mul(m, a[1]), b[0]);
    df_acc(sh, sl, df_mul(s, a[2]), b[3]);
    df_acc(sh, sl, df_mul(m, a[3]), b[2]);
}

__device__ __forceinline__ void pauli_df(const dfl* p, int dir, dfl* o) {
    if (dir == 1) { o[0] = p[2]; o[1] = p[3]; o[2] = p[0]; o[3] = p[1]; }
    else if (dir == 2) { o[0] = p[3]; o[1] = df_neg(p[2]); o[2] = df_neg(p[1]); o[3] = p[0]; }
    else { o[0] = p[0]; o[1] = p[1]; o[2] = df_neg(p[2]); o[3] = df_neg(p[3]); }
}

__global__ void __launch_bounds__(kThreads)
k_dens_partial_df(const double* __restrict__ psi, const float2* __restrict__ der,
                  const double* __restrict__ occ, const int* __restrict__ qn, int nwt,
                  int per_group, long V, double* __restrict__ part) {
    const long v = (long)blockIdx.x * kThreads + threadIdx.x;
    const int g = blockIdx.y;
    if (v >= V) return;
    // per isospin (n: 0, p: 1) accumulators of rho, tau, divJ; kept in named
    // registers (a runtime-indexed array would live in local memory)
    float nh[3] = {0.f, 0.f, 0.f}, nl[3] = {0.f, 0.f, 0.f};
    float ph[3] = {0.f, 0.f, 0.f}, pl[3] = {0.f, 0.f, 0.f};
    const int i0 = g * per_group, i1 = min(nwt, i0 + per_group);
    for (int i = i0; i < i1; ++i) {
        const double o64 = occ[i];
        if (o64 == 0.0) continue;
        const dfl o = df_split(o64);
        const int it = (qn[4 * i] + 3) / 2 - 1;
        const double* ps = psi + (long)i * 4 * V;
        const float2* dr = der + (long)i * 12 * V;
        dfl p[4], d[3][4];
#pragma unroll
        for (int l = 0; l < 4; ++l) {
            p[l] = df_split(ps[l * V + v]);
#pragma unroll
            for (int m = 0; m < 3; ++m) d[m][l] = df_ld(dr + (m * 4 + l) * V + v);
        }
        float dh = 0.f, dl = 0.f, th = 0.f, tl = 0.f, jh = 0.f, jl = 0.f;
#pragma unroll
        for (int l = 0; l < 4; ++l) df_acc(dh, dl, p[l], p[l]);
#pragma unroll
        for (int m = 0; m < 3; ++m)
#pragma unroll
            for (int l = 0; l < 4; ++l) df_acc(th, tl, d[m][l], d[m][l]);
        dfl s[4];
        pauli_df(d[1], 3, s); imag_acc(jh, jl, d[0], s, 1.0f);
        pauli_df(d[2], 2, s); imag_acc(jh, jl, d[0], s, -1.0f);
        pauli_df(d[1], 1, s); imag_acc(jh, jl, d[2], s, -1.0f);
        pauli_df(d[0], 2, s); imag_acc(jh, jl, d[2], s, 1.0f);
        pauli_df(d[0], 3, s); imag_acc(jh, jl, d[1], s, -1.0f);
        pauli_df(d[2], 1, s); imag_acc(jh, jl, d[1], s, 1.0f);
        const dfl q3[3] = {df_norm(dfl{dh, dl}), df_norm(dfl{th, tl}), df_norm(dfl{jh, jl})};
        if (it == 0) {
#pragma unroll
            for (int q = 0; q < 3; ++q) df_acc(nh[q], nl[q], o, q3[q]);
        } else {
#pragma unroll
            for (int q = 0; q < 3; ++q) df_acc(ph[q], pl[q], o, q3[q]);
        }
    }
    double* pg = part + (long)g * 6 * V;
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        pg[(q * 2 + 0) * V + v] = df_to(dfl{nh[q], nl[q]});
        pg[(q * 2 + 1) * V + v] = df_to(dfl{ph[q], pl[q]});
    }
}

__global__ void k_dens_reduce(const double* __restrict__ part, int ngroups, long V,
                              double* __restrict__ rho, double* __restrict__ tau,
                              double* __restrict__ nablaj) {
    const long v = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= V) return;
    double a[6] = {0, 0, 0, 0, 0, 0};
    for (int g = 0; g < ngroups; ++g)
#pragma unroll
        for (int q = 0; q < 6; ++q) a[q] += part[((long)g * 6 + q) * V + v];
    rho[v] = a[0]; rho[V + v] = a[1];
    tau[v] = a[2]; tau[V + v] = a[3];
    nablaj[v] = a[4]; nablaj[V + v] = a[5];
}

// The tensor density J_{mu nu}(it) = sum_i occ_i Im(psi_i^+ sigma_nu d_mu psi_i)
// (GetJMuNu, src/Spwf.f90:2186-2204, summed as ComputeDensity does,
// src/Densities.f90:486-490): one thread per mesh point, the spwfs in index
// order, the derivatives FP64 or double-float; out [it][nu][mu][V].
__device__ __forceinline__ double der_value(const double* p, long k, bool df) {
    if (!df) return p[k];
    const float2 hl = reinterpret_cast<const float2*>(p)[k];
    return (double)hl.x + (double)hl.y;
}

__global__ void __launch_bounds__(kThreads)
k_jmunu(const double* __restrict__ psi, const double* __restrict__ der, bool df,
        const double* __restrict__ occ, const int* __restrict__ qn, int nwt, long V,
        double* __restrict__ out) {
    const long v = (long)blockIdx.x * kThreads + threadIdx.x;
    if (v >= V) return;
    double J[2][3][3];
#pragma unroll
    for (int it = 0; it < 2; ++it)
#pragma unroll
        for (int nu = 0; nu < 3; ++nu)
#pragma unroll
            for (int mu = 0; mu < 3; ++mu) J[it][nu][mu] = 0.0;
    for (int i = 0; i < nwt; ++i) {
        const double o = occ[i];
        if (o == 0.0) continue;
        const bool prot = qn[4 * i] > 0;
        const double* p = psi + (long)i * 4 * V;
        const double* d = der + (long)i * 12 * V;
        const double a0 = p[v], a1 = p[V + v], a2 = p[2 * V + v], a3 = p[3 * V + v];
#pragma unroll
        for (int mu = 0; mu < 3; ++mu) {
            const double g0 = der_value(d, (mu * 4 + 0) * V + v, df);
            const double g1 = der_value(d, (mu * 4 + 1) * V + v, df);
            const double g2 = der_value(d, (mu * 4 + 2) * V + v, df);
            const double g3 = der_value(d, (mu * 4 + 3) * V + v, df);
            // sigma_x g = (g2, g3, g0, g1); sigma_y g = (g3, -g2, -g1, g0);
            // sigma_z g = (g0, g1, -g2, -g3); Im(a^+ b) = a0 b1 - a1 b0 + a2 b3 - a3 b2
            const double jx = a0 * g3 - a1 * g2 + a2 * g1 - a3 * g0;
            const double jy = a0 * -g2 - a1 * g3 + a2 * g0 - a3 * -g1;
            const double jz = a0 * g1 - a1 * g0 + a2 * -g3 - a3 * -g2;
            if (prot) {
                J[1][0][mu] += o * jx;
                J[1][1][mu] += o * jy;
                J[1][2][mu] += o * jz;
            } else {
                J[0][0][mu] += o * jx;
                J[0][1][mu] += o * jy;
                J[0][2][mu] += o * jz;
            }
        }
    }
#pragma unroll
    for (int it = 0; it < 2; ++it)
#pragma unroll
        for (int nu = 0; nu < 3; ++nu)
#pragma unroll
            for (int mu = 0; mu < 3; ++mu) out[((it * 3 + nu) * 3 + mu) * V + v] = J[it][nu][mu];
}

}  // namespace

int density_groups(const mg_ctx* c) {
    const int chunks = div_up(c->V, kThreads);
    int g = std::max(1, (4 * c->num_sms + chunks - 1) / chunks);
    return std::min(g, c->p.nwt);
}

int densities(mg_ctx* c) {
    const int b = c->p.pairing == MG_PAIRING_HFB ? MG_CAN_BASIS : MG_HF_BASIS;
    Basis& B = c->bas[b];
    if (!B.have_qn) return MG_ERR_STATE;
    const long V = c->V;
    const int ng = density_groups(c);
    const int per = div_up(c->p.nwt, ng);
    dim3 grid(div_up(V, kThreads), ng);
    if (B.der_df)
        k_dens_partial_df<<<grid, kThreads, 0, c->stream>>>(
            B.psi, reinterpret_cast<const float2*>(B.der), B.occ, B.qn, c->p.nwt, per, V, c->red);
    else
        k_dens_partial<<<grid, kThreads, 0, c->stream>>>(B.psi, B.der, B.occ, B.qn, c->p.nwt, per,
                                                         V, c->red);
    MG_LAUNCHED(c);
    k_dens_reduce<<<div_up(V, kThreads), kThreads, 0, c->stream>>>(c->red, ng, V, c->rho, c->tau,
                                                                   c->nablaj);
    MG_LAUNCHED(c);
    // grad rho, lap rho: the first two field jobs
    MG_TRY(run_jobs(c, c->field_jobs, 2));
    if (c->tensor) {
        k_jmunu<<<div_up(V, kThreads), kThreads, 0, c->stream>>>(B.psi, B.der, B.der_df, B.occ,
                                                                B.qn, c->p.nwt, V, c->jmunu);
        MG_LAUNCHED(c);
    }
    if (!c->p.trc) MG_TRY(time_odd_densities(c, B));
    return MG_OK;
}

}  // namespace mg
