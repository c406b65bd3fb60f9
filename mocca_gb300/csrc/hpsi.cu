// hpsi.cu -- action of the single-particle Hamiltonian, FP64, with the fused
// imaginary-time (GradDesc) update.
//
// h.psi = B + U + W (src/ImaginaryTime.f90:213-304, time-even fields):
//   B = -(B_q + hbm/2 mu_red) lap psi - sum_m d_m B_q d_m psi   ActionOfBNew
//                                                  src/MeanFields.f90:811-851
//   U = U_q psi                                    ActionOfU :792-809
//   W = -i [sum_mn W_mn sigma_n d_m psi + 1/2 sum_n (div W)_n sigma_n psi]
//                                                  ActionOfW :1029-1065
// One thread owns one mesh point of one spwf: it reads psi, Der(1:3), Lap at
// that point (20 doubles) and the isospin's fields (L2-resident), and writes
// either h.psi or, for a GradDesc step (src/ImaginaryTime.f90:467-491),
// psi <- psi - dt/hbar h.psi + mu*update and update <- psi_old in place, so
// h.psi never goes to HBM.  The per-spwf sums <psi|h psi> and <h psi|h psi>
// are reduced per block into a partial table and finished in block order
// (deterministic).
#include "df.cuh"
#include "mg_internal.cuh"

namespace mg {

namespace {

constexpr int kThreads = 256;

struct Fields {
    const double* U;
    const double* B;
    const double* nablaB;
    const double* W;
    const double* divW;
    // time-odd fields without time reversal ([it][m][V], div A [it][V]);
    // nullptr with time reversal
    const double* A = nullptr;
    const double* S = nullptr;
    const double* divA = nullptr;
    // the C and D actions of the time-odd tensor terms per spwf
    // ([i][2][l][V], tensor_odd.cu), or nullptr
    const double* X = nullptr;
};

__device__ __forceinline__ void pauli(const double* p, int dir, double* o) {
    if (dir == 1) { o[0] = p[2]; o[1] = p[3]; o[2] = p[0]; o[3] = p[1]; }
    else if (dir == 2) { o[0] = p[3]; o[1] = -p[2]; o[2] = -p[1]; o[3] = p[0]; }
    else { o[0] = p[0]; o[1] = p[1]; o[2] = -p[2]; o[3] = -p[3]; }
}

template <bool kGradStep>
__global__ void __launch_bounds__(kThreads)
k_hpsi(double* __restrict__ psi, const double* __restrict__ der,
       const double* __restrict__ lap, const int* __restrict__ qn, Fields F,
       double* __restrict__ hout, double* __restrict__ upd, double* __restrict__ partial,
       long V, double kin0, double kin1, double fac, double mom) {
    const int i = blockIdx.y;
    const long v = (long)blockIdx.x * kThreads + threadIdx.x;
    double s_eh = 0.0, s_hh = 0.0;
    if (v < V) {
        const int it = (qn[4 * i] + 3) / 2 - 1;
        const double kin = it == 0 ? kin0 : kin1;
        double* ps = psi + (long)i * 4 * V;
        const double* dr = der + (long)i * 12 * V;
        const double* lp = lap + (long)i * 4 * V;
        double p[4], d[3][4], L[4];
#pragma unroll
        for (int l = 0; l < 4; ++l) {
            p[l] = ps[l * V + v];
            L[l] = lp[l * V + v];
#pragma unroll
            for (int m = 0; m < 3; ++m) d[m][l] = dr[(m * 4 + l) * V + v];
        }
        const double Bq = F.B[it * V + v];
        const double Uq = F.U[it * V + v];
        const double nb0 = F.nablaB[(it * 3 + 0) * V + v];
        const double nb1 = F.nablaB[(it * 3 + 1) * V + v];
        const double nb2 = F.nablaB[(it * 3 + 2) * V + v];
        double w[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll
        for (int mu = 0; mu < 3; ++mu)
#pragma unroll
            for (int nu = 0; nu < 3; ++nu) {
                double s[4];
                pauli(d[mu], nu + 1, s);
                const double wv = F.W[((it * 3 + nu) * 3 + mu) * V + v];
#pragma unroll
                for (int l = 0; l < 4; ++l) w[l] = fma(wv, s[l], w[l]);
            }
#pragma unroll
        for (int nu = 0; nu < 3; ++nu) {
            double s[4];
            pauli(p, nu + 1, s);
            const double hv = 0.5 * F.divW[(it * 3 + nu) * V + v];
#pragma unroll
            for (int l = 0; l < 4; ++l) w[l] = fma(hv, s[l], w[l]);
        }
        const double wf[4] = {w[1], -w[0], w[3], -w[2]};
        double h[4];
#pragma unroll
        for (int l = 0; l < 4; ++l) {
            double t = -(Bq * L[l]);
            t = t - kin * L[l];
            double sd = fma(nb1, d[1][l], nb0 * d[0][l]);
            sd = fma(nb2, d[2][l], sd);
            const double b = t - sd;
            const double u = Uq * p[l];
            h[l] = (b + u) + wf[l];
        }
        if (F.A) {
            // ActionOfS: sum_m S_m sigma_m psi; ActionOfA: -i (sum_m A_m d_m psi
            // + 1/2 div A psi) (src/MeanFields.f90:1107-1147)
            double sa[4] = {0.0, 0.0, 0.0, 0.0}, aa[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll
            for (int m = 0; m < 3; ++m) {
                double sg[4];
                pauli(p, m + 1, sg);
                const double sm = F.S[(it * 3 + m) * V + v], am = F.A[(it * 3 + m) * V + v];
#pragma unroll
                for (int l = 0; l < 4; ++l) {
                    sa[l] = fma(sm, sg[l], sa[l]);
                    aa[l] = fma(am, d[m][l], aa[l]);
                }
            }
            const double hd = 0.5 * F.divA[it * V + v];
#pragma unroll
            for (int l = 0; l < 4; ++l) aa[l] = fma(hd, p[l], aa[l]);
            const double af[4] = {aa[1], -aa[0], aa[3], -aa[2]};
#pragma unroll
            for (int l = 0; l < 4; ++l) h[l] = (h[l] + sa[l]) + af[l];
        }
        if (F.X) {
            // ActionOfC, then ActionOfD (src/ImaginaryTime.f90:270-284)
            const double* x = F.X + (long)i * 8 * V;
#pragma unroll
            for (int l = 0; l < 4; ++l) h[l] = (h[l] + x[l * V + v]) + x[(4 + l) * V + v];
        }
#pragma unroll
        for (int l = 0; l < 4; ++l) {
            s_eh = fma(p[l], h[l], s_eh);
            s_hh = fma(h[l], h[l], s_hh);
        }
        if (kGradStep) {
            double* up = upd + (long)i * 4 * V;
#pragma unroll
            for (int l = 0; l < 4; ++l) {
                const double a = fma(-fac, h[l], mom * up[l * V + v]);
                up[l * V + v] = p[l];
                ps[l * V + v] = p[l] + a;
            }
        } else if (hout) {
            double* ho = hout + (long)i * 4 * V;
#pragma unroll
            for (int l = 0; l < 4; ++l) ho[l * V + v] = h[l];
        }
    }
    // block reduction of (s_eh, s_hh)
    __shared__ double red[2][kThreads / 32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        s_eh += __shfl_xor_sync(0xffffffffu, s_eh, o);
        s_hh += __shfl_xor_sync(0xffffffffu, s_hh, o);
    }
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    if (lane == 0) { red[0][warp] = s_eh; red[1][warp] = s_hh; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, b = 0.0;
        for (int q = 0; q < kThreads / 32; ++q) { a += red[0][q]; b += red[1][q]; }
        partial[((long)i * gridDim.x + blockIdx.x) * 2 + 0] = a;
        partial[((long)i * gridDim.x + blockIdx.x) * 2 + 1] = b;
    }
}

// Mixed precision: the same action in double-float arithmetic (df.cuh).  The
// derivatives arrive as double-float pairs, psi and the fields are split from
// their FP64 bits (no FP64 instructions); the GradDesc update and the
// per-point energy terms are double-float too, so the only FP64 work left is
// the final rounding of the new psi and the per-thread partial sums.
__device__ __forceinline__ void pauli_df(const dfl* p, int dir, dfl* o) {
    if (dir == 1) { o[0] = p[2]; o[1] = p[3]; o[2] = p[0]; o[3] = p[1]; }
    else if (dir == 2) { o[0] = p[3]; o[1] = df_neg(p[2]); o[2] = df_neg(p[1]); o[3] = p[0]; }
    else { o[0] = p[0]; o[1] = p[1]; o[2] = df_neg(p[2]); o[3] = df_neg(p[3]); }
}

// The isospin's fields as double-float, once per h.psi call (they are shared
// by every spwf of the isospin): per point, in order
//   -(B + hbm/2 mu_red), U, -dB/dx_m (3), W_nm (n-major, 9), (div W)_n / 2 (3).
constexpr int kNF = 17;

__global__ void k_fields_df(Fields F, long V, double kin0, double kin1, float2* __restrict__ out) {
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 2 * V) return;
    const int it = (int)(t / V);
    const long v = t % V;
    float2* o = out + (long)it * kNF * V + v;
    auto put = [&](int f, double x) {
        const dfl d = df_from(x);
        o[(long)f * V] = make_float2(d.h, d.l);
    };
    put(0, -(F.B[it * V + v] + (it == 0 ? kin0 : kin1)));
    put(1, F.U[it * V + v]);
    for (int m = 0; m < 3; ++m) put(2 + m, -F.nablaB[(it * 3 + m) * V + v]);
    for (int q = 0; q < 9; ++q) put(5 + q, F.W[(it * 9 + q) * V + v]);
    for (int n = 0; n < 3; ++n) put(14 + n, 0.5 * F.divW[(it * 3 + n) * V + v]);
}

template <bool kGradStep>
__global__ void __launch_bounds__(kThreads, 4)
k_hpsi_df(double* __restrict__ psi, const float2* __restrict__ der,
          const float2* __restrict__ lap, const int* __restrict__ qn,
          const float2* __restrict__ Fd, double* __restrict__ hout, double* __restrict__ upd,
          double* __restrict__ partial, long V, double fac, double mom) {
    const int i = blockIdx.y;
    const long v = (long)blockIdx.x * kThreads + threadIdx.x;
    // <psi|h psi> and <h psi|h psi> accumulate in double-float and become
    // FP64 once per thread
    float eh = 0.f, el = 0.f, hh = 0.f, hl = 0.f;
    if (v < V) {
        const int it = (qn[4 * i] + 3) / 2 - 1;
        const float2* fd = Fd + (long)it * kNF * V + v;
        double* ps = psi + (long)i * 4 * V;
        const float2* dr = der + (long)i * 12 * V;
        const float2* lp = lap + (long)i * 4 * V;
        // the spinor and the update history first; the derivatives one
        // direction at a time (each direction's values die after use, which
        // keeps the live registers low enough for more resident warps)
        double p64[4], u64[4];
        dfl p[4];
#pragma unroll
        for (int l = 0; l < 4; ++l) {
            p64[l] = ps[l * V + v];
            if (kGradStep) u64[l] = upd[(long)i * 4 * V + l * V + v];
        }
#pragma unroll
        for (int l = 0; l < 4; ++l) p[l] = df_split(p64[l]);
        // B, U: -(B + hbar^2/2m) lap psi + U psi
        float th[4] = {0.f, 0.f, 0.f, 0.f}, tl[4] = {0.f, 0.f, 0.f, 0.f};
        {
            const dfl nkB = df_ld(fd), Uq = df_ld(fd + V);
#pragma unroll
            for (int l = 0; l < 4; ++l) {
                df_acc(th[l], tl[l], nkB, df_ld(lp + l * V + v));
                df_acc(th[l], tl[l], Uq, p[l]);
            }
        }
        // per direction mu: -(d_mu B) d_mu psi and sum_nu W_{nu mu} sigma_nu d_mu psi
        float wh[4] = {0.f, 0.f, 0.f, 0.f}, wl[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
        for (int mu = 0; mu < 3; ++mu) {
            dfl dm[4];
#pragma unroll
            for (int l = 0; l < 4; ++l) dm[l] = df_ld(dr + (mu * 4 + l) * V + v);
            const dfl nb = df_ld(fd + (2 + mu) * V);
#pragma unroll
            for (int l = 0; l < 4; ++l) df_acc(th[l], tl[l], nb, dm[l]);
#pragma unroll
            for (int nu = 0; nu < 3; ++nu) {
                dfl sg[4];
                pauli_df(dm, nu + 1, sg);
                const dfl wv = df_ld(fd + (5 + nu * 3 + mu) * V);
#pragma unroll
                for (int l = 0; l < 4; ++l) df_acc(wh[l], wl[l], wv, sg[l]);
            }
        }
#pragma unroll
        for (int nu = 0; nu < 3; ++nu) {
            dfl sg[4];
            pauli_df(p, nu + 1, sg);
            const dfl hv = df_ld(fd + (14 + nu) * V);
#pragma unroll
            for (int l = 0; l < 4; ++l) df_acc(wh[l], wl[l], hv, sg[l]);
        }
        const dfl w[4] = {df_norm(dfl{wh[0], wl[0]}), df_norm(dfl{wh[1], wl[1]}),
                          df_norm(dfl{wh[2], wl[2]}), df_norm(dfl{wh[3], wl[3]})};
        const dfl wf[4] = {w[1], df_neg(w[0]), w[3], df_neg(w[2])};
        dfl h[4];
#pragma unroll
        for (int l = 0; l < 4; ++l) {
            h[l] = df_add(df_norm(dfl{th[l], tl[l]}), wf[l]);
            df_acc(eh, el, p[l], h[l]);
            df_acc(hh, hl, h[l], h[l]);
        }
        if (kGradStep) {
            // psi <- psi - fac h + mom update ; update <- psi_old (FP64 copy)
            const dfl nf = df_neg(df_split(fac)), mm = df_split(mom);
            double* up = upd + (long)i * 4 * V;
#pragma unroll
            for (int l = 0; l < 4; ++l) {
                float ah = 0.f, al = 0.f;
                df_acc(ah, al, nf, h[l]);
                df_acc(ah, al, mm, df_split(u64[l]));
                up[l * V + v] = p64[l];
                ps[l * V + v] = df_to_fast(df_add(p[l], df_norm(dfl{ah, al})));
            }
        } else if (hout) {
            double* ho = hout + (long)i * 4 * V;
#pragma unroll
            for (int l = 0; l < 4; ++l) ho[l * V + v] = df_to_fast(h[l]);
        }
    }
    // warp and block sums in double-float (FP32 pipe), FP64 once per block
    dfl se = df_norm(dfl{eh, el}), sh = df_norm(dfl{hh, hl});
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        se = df_add(se, dfl{__shfl_xor_sync(0xffffffffu, se.h, o),
                            __shfl_xor_sync(0xffffffffu, se.l, o)});
        sh = df_add(sh, dfl{__shfl_xor_sync(0xffffffffu, sh.h, o),
                            __shfl_xor_sync(0xffffffffu, sh.l, o)});
    }
    __shared__ float2 red[2][kThreads / 32];
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    if (lane == 0) {
        red[0][warp] = make_float2(se.h, se.l);
        red[1][warp] = make_float2(sh.h, sh.l);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        dfl a = {0.f, 0.f}, b = {0.f, 0.f};
        for (int q = 0; q < kThreads / 32; ++q) {
            a = df_add(a, df_ld(&red[0][q]));
            b = df_add(b, df_ld(&red[1][q]));
        }
        partial[((long)i * gridDim.x + blockIdx.x) * 2 + 0] = df_to_fast(a);
        partial[((long)i * gridDim.x + blockIdx.x) * 2 + 1] = df_to_fast(b);
    }
}

// e[i] = dv * sum <psi|h psi>, disp[i] = dv * sum <h psi|h psi> - e^2
__global__ void k_finish_energies(const double* __restrict__ partial, int nchunk, int nwt,
                                  double dv, double* __restrict__ e, double* __restrict__ disp) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nwt) return;
    double a = 0.0, b = 0.0;
    for (int q = 0; q < nchunk; ++q) {
        a += partial[((long)i * nchunk + q) * 2 + 0];
        b += partial[((long)i * nchunk + q) * 2 + 1];
    }
    const double en = a * dv;
    e[i] = en;
    disp[i] = b * dv - en * en;
}

double reduced_mass(const mg_ctx* c, int it) {
    if (c->f.com1body == 2)
        return 1.0 - c->f.nucleonmass[it] /
                         (c->p.neutrons * c->f.nucleonmass[0] + c->p.protons * c->f.nucleonmass[1]);
    return 1.0;
}

}  // namespace

// h.psi over a basis.  grad_step: GradDesc update of the HF basis in place
// (fac = dt/hbar, mom = momentum); otherwise h.psi goes to out (may be NULL).
// Energies and dispersions land in the basis' e / disp arrays.
int hpsi_basis(mg_ctx* c, int b, double* out, bool grad_step, double fac, double mom) {
    Basis& B = c->bas[b];
    if (!B.have_qn) return MG_ERR_STATE;
    const long V = c->V;
    const int nchunk = div_up(V, kThreads);
    Fields F{c->U, c->Bp, c->nablaB, c->W, c->divW, c->Apot, c->Spot, c->divA};
    const double kin0 = c->f.hbm / 2.0 * reduced_mass(c, 0);
    const double kin1 = c->f.hbm / 2.0 * reduced_mass(c, 1);
    dim3 grid(nchunk, c->p.nwt);
    if (c->todd) {
        // the time-odd tensor actions first (the time-odd path is FP64)
        if (B.der_df) return MG_ERR_STATE;
        if (!c->todd_x) MG_CUDA(cudaMalloc(&c->todd_x, 8 * (size_t)c->p.nwt * V * sizeof(double)));
        MG_TRY(tensor_odd_action(c, B.der, B.h_qn.data(), B.qn, c->p.nwt, c->todd_x));
        F.X = c->todd_x;
    }
    // the derivative format decides: double-float derivatives come from the
    // mixed kernels
    const bool mixed = B.der_df;
    const float2* der2 = reinterpret_cast<const float2*>(B.der);
    const float2* lap2 = reinterpret_cast<const float2*>(B.lap);
    if (mixed) {
        if (!c->fields_df) MG_CUDA(cudaMalloc(&c->fields_df, 2 * kNF * V * sizeof(float2)));
        k_fields_df<<<div_up(2 * V, kThreads), kThreads, 0, c->stream>>>(F, V, kin0, kin1,
                                                                         c->fields_df);
        MG_LAUNCHED(c);
    }
    if (grad_step && mixed)
        k_hpsi_df<true><<<grid, kThreads, 0, c->stream>>>(B.psi, der2, lap2, B.qn, c->fields_df,
                                                          nullptr, c->updates, c->red, V, fac,
                                                          mom);
    else if (mixed)
        k_hpsi_df<false><<<grid, kThreads, 0, c->stream>>>(B.psi, der2, lap2, B.qn,
                                                           c->fields_df, out, nullptr, c->red, V,
                                                           0.0, 0.0);
    else if (grad_step)
        k_hpsi<true><<<grid, kThreads, 0, c->stream>>>(B.psi, B.der, B.lap, B.qn, F, nullptr,
                                                       c->updates, c->red, V, kin0, kin1, fac, mom);
    else
        k_hpsi<false><<<grid, kThreads, 0, c->stream>>>(B.psi, B.der, B.lap, B.qn, F, out,
                                                        nullptr, c->red, V, kin0, kin1, 0.0, 0.0);
    MG_LAUNCHED(c);
    k_finish_energies<<<div_up(c->p.nwt, 128), 128, 0, c->stream>>>(c->red, nchunk, c->p.nwt,
                                                                     c->dv, B.e, B.disp);
    MG_LAUNCHED(c);
    return MG_OK;
}

// h.psi of one spinor outside the bases (FP64 kernel, FP64 derivatives), for
// IterativeEstimation: out = h psi, e_dev[0] = <psi|h psi> dv.
int hpsi_single(mg_ctx* c, double* psi, const double* der, const double* lap, const int* qn_dev,
                double* out, double* e_dev) {
    const long V = c->V;
    const int nchunk = div_up(V, kThreads);
    Fields F{c->U, c->Bp, c->nablaB, c->W, c->divW, c->Apot, c->Spot, c->divA};
    const double kin0 = c->f.hbm / 2.0 * reduced_mass(c, 0);
    const double kin1 = c->f.hbm / 2.0 * reduced_mass(c, 1);
    if (c->todd) {
        if (!c->todd_x) MG_CUDA(cudaMalloc(&c->todd_x, 8 * (size_t)c->p.nwt * V * sizeof(double)));
        MG_TRY(tensor_odd_action(c, der, c->est_h_qn, qn_dev, 1, c->todd_x));
        F.X = c->todd_x;
    }
    k_hpsi<false><<<dim3(nchunk, 1), kThreads, 0, c->stream>>>(psi, der, lap, qn_dev, F, out,
                                                               nullptr, c->red, V, kin0, kin1,
                                                               0.0, 0.0);
    MG_LAUNCHED(c);
    k_finish_energies<<<1, 128, 0, c->stream>>>(c->red, nchunk, 1, c->dv, e_dev, e_dev + 1);
    MG_LAUNCHED(c);
    return MG_OK;
}

}  // namespace mg
