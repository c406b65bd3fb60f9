// fields.cu -- mean-field potentials and multipole moments, FP64.
//
// Potentials (ConstructPotentials, src/PotentialMixing.f90:17-201 with
// MixingScheme 0):
//   U  CalcUPot  src/MeanFields.f90:269-409 (time-even Skyrme part, Coulomb
//      direct + Slater exchange on protons)
//   W  CalcWPot  src/MeanFields.f90:494-597 (the B9 spin-orbit part and the
//      J^2 parts of B14..B17) and div W
//      with the symmetry arguments of :575-591
//   B  CalcBPot  src/MeanFields.f90:115-150 and grad B
// One thread per mesh point computes U, B and the nine W components of both
// isospins; the derivatives go through the Lagrange job kernels.
// Moments: Calculate_Multipole (src/Moments.f90:1907-1966) for the electric
// moments the Coulomb boundary uses; the constrained moments, the cutoff and
// the constraint field (added to U here) come from constraints.cu.
#include <cmath>

#include "mg_internal.cuh"

namespace mg {

namespace {

constexpr int kThreads = 256;

struct Coef {
    double B1, B2, B3, B4, B5, B6, B7a, B7b, B8a, B8b, byt3a, byt3b, B9, B9q;
    int cexchange;
    double B14, B15, B16, B17;   // the J^2 terms (with jmunu)
};

__device__ __forceinline__ int levi(int i, int j, int k) {
    if (i == j || j == k || k == i) return 0;
    if ((i == 1 && j == 2 && k == 3) || (i == 3 && j == 1 && k == 2) || (i == 2 && j == 3 && k == 1))
        return 1;
    return -1;
}

__global__ void __launch_bounds__(kThreads)
k_potentials(const double* __restrict__ rho, const double* __restrict__ tau,
             const double* __restrict__ nablaj, const double* __restrict__ derrho,
             const double* __restrict__ laprho, const double* __restrict__ coul,
             const double* __restrict__ coulex, const double* __restrict__ cons,
             const double* __restrict__ jm, Coef B, long V, double* __restrict__ U,
             double* __restrict__ Bp, double* __restrict__ W) {
    const long v = (long)blockIdx.x * kThreads + threadIdx.x;
    if (v >= V) return;
    const double eps = 1.0e-20;
    const double rn = rho[v], rp = rho[V + v];
    const double rt = rn + rp;
    const double njt = nablaj[v] + nablaj[V + v];
    double u[2];
    u[0] = (2.0 * B.B1 + 2.0 * B.B2) * rn + 2.0 * B.B1 * rp;
    u[1] = (2.0 * B.B1 + 2.0 * B.B2) * rp + 2.0 * B.B1 * rn;
    const double pa = pow(rt, B.byt3a);
    const double pa1 = pow(rt + eps, 1 + B.byt3a);
    for (int it = 0; it < 2; ++it) {
        const int at = 1 - it;
        const double ri = rho[it * V + v], ra = rho[at * V + v];
        double x = u[it] + (B.B3 + B.B4) * tau[it * V + v] + B.B3 * tau[at * V + v] +
                   2.0 * ((B.B5 + B.B6) * laprho[it * V + v] + B.B5 * laprho[at * V + v]) +
                   (2 + B.byt3a) * B.B7a * pa1 +
                   B.B8a * (B.byt3a * pa / (rt + eps) * (ri * ri + ra * ra) + 2.0 * pa * ri) +
                   B.B9 * njt + B.B9q * nablaj[it * V + v];
        if (B.B7b != 0.0 || B.B8b != 0.0) {
            const double pb = pow(rt, B.byt3b);
            x = x + (2 + B.byt3b) * B.B7b * pow(rt + eps, 1 + B.byt3b) +
                B.B8b * (B.byt3b * pb / (rt + eps) * (ri * ri + ra * ra) + 2.0 * pb * ri);
        }
        u[it] = x;
    }
    u[1] = u[1] + coul[v];
    if (B.cexchange == 2) u[1] = u[1] + coulex[v];
    if (cons) {   // U = U + ConstraintEnergy (src/MeanFields.f90:403)
        u[0] = u[0] + cons[v];
        u[1] = u[1] + cons[V + v];
    }
    U[v] = u[0];
    U[V + v] = u[1];
    for (int it = 0; it < 2; ++it) {
        Bp[it * V + v] = B.B3 * rho[(1 - it) * V + v] + (B.B3 + B.B4) * rho[it * V + v];
        for (int n = 1; n <= 3; ++n)
            for (int m = 1; m <= 3; ++m) {
                double w = 0.0;
                for (int k = 1; k <= 3; ++k) {
                    const int e = levi(k, m, n);
                    w = w - e * ((B.B9 + B.B9q) * derrho[(it * 3 + k - 1) * V + v] +
                                 B.B9 * derrho[((1 - it) * 3 + k - 1) * V + v]);
                }
                if (jm) {
                    // CalcWPot's J^2 parts (src/MeanFields.f90:531-556) in its
                    // order: B14, B15 on J(m, n); B16, B17 on J(n, m), then
                    // on the traces along the diagonal
                    auto J = [&](int q, int a, int b) {   // J(a, b) of isospin q
                        return jm[((q * 3 + b - 1) * 3 + a - 1) * V + v];
                    };
                    const int at = 1 - it;
                    if (B.B14 != 0.0 || B.B15 != 0.0)
                        w = w + 2.0 * (B.B14 + B.B15) * J(it, m, n) + 2.0 * B.B14 * J(at, m, n);
                    if (B.B16 != 0.0 || B.B17 != 0.0) {
                        w = w + 2.0 * (B.B16 + B.B17) * J(it, n, m) + 2.0 * B.B16 * J(at, n, m);
                        if (m == n)
                            for (int k = 1; k <= 3; ++k)
                                w = w + 2 * (B.B16 + B.B17) * J(it, k, k) + 2 * B.B16 * J(at, k, k);
                    }
                }
                W[((it * 3 + n - 1) * 3 + m - 1) * V + v] = w;
            }
    }
}

// divW(nu) = t1 + t2 + t3 (the three derivative terms of src/MeanFields.f90:575-591)
__global__ void k_sum3(const double* __restrict__ t, long n, double* __restrict__ out) {
    const long v = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n) return;
    out[v] = t[v] + t[n + v] + t[2 * n + v];
}

// values[m][it] = dv * sum_v sh[m][v] rho[it][v]
__global__ void __launch_bounds__(kThreads)
k_moments(const double* __restrict__ sh, const double* __restrict__ rho, long V, double dv,
          double* __restrict__ values) {
    const int m = blockIdx.x;
    double a = 0.0, b = 0.0;
    for (long v = threadIdx.x; v < V; v += kThreads) {
        const double s = sh[(long)m * V + v];
        a = fma(s, rho[v], a);
        b = fma(s, rho[V + v], b);
    }
    __shared__ double red[2][kThreads / 32];
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, o);
        b += __shfl_xor_sync(0xffffffffu, b, o);
    }
    if (threadIdx.x % 32 == 0) { red[0][threadIdx.x / 32] = a; red[1][threadIdx.x / 32] = b; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double x = 0.0, y = 0.0;
        for (int q = 0; q < kThreads / 32; ++q) { x += red[0][q]; y += red[1][q]; }
        values[2 * m] = x * dv;
        values[2 * m + 1] = y * dv;
    }
}

}  // namespace

// Field derivative jobs: [0,1] rho_q -> grad rho, lap rho; [2,3] B_q -> grad B;
// [4..21] the 18 single-axis derivatives of W entering div W.
int build_field_jobs(mg_ctx* c) {
    const long V = c->V;
    const int P = c->p.pc, S = c->p.sc, TS = c->p.tsc;
    std::vector<GridJob> jobs;
    for (int it = 0; it < 2; ++it) {
        GridJob J{};
        J.in = c->rho + it * V;
        J.dx = c->derrho + (it * 3 + 0) * V;
        J.dy = c->derrho + (it * 3 + 1) * V;
        J.dz = c->derrho + (it * 3 + 2) * V;
        J.lap = c->laprho + it * V;
        for (int d = 0; d < 3; ++d) J.slot[d] = (int8_t)lag_slot(d, P, S, TS, 1);
        jobs.push_back(J);
    }
    for (int it = 0; it < 2; ++it) {
        GridJob J{};
        J.in = c->Bp + it * V;
        J.dx = c->nablaB + (it * 3 + 0) * V;
        J.dy = c->nablaB + (it * 3 + 1) * V;
        J.dz = c->nablaB + (it * 3 + 2) * V;
        for (int d = 0; d < 3; ++d) J.slot[d] = (int8_t)lag_slot(d, P, S, TS, 1);
        jobs.push_back(J);
    }
    // {dir, m, n, P sign, S sign, comp} of DivWpot, src/MeanFields.f90:575-591
    static const int T[3][3][6] = {
        {{0, 1, 1, -1, 1, 2}, {1, 2, 1, -1, 1, 1}, {2, 3, 1, -1, -1, 2}},
        {{0, 1, 2, -1, 1, 1}, {1, 2, 2, -1, 1, 2}, {2, 3, 2, -1, -1, 1}},
        {{0, 1, 3, -1, -1, 2}, {1, 2, 3, -1, -1, 1}, {2, 3, 3, -1, 1, 2}}};
    for (int it = 0; it < 2; ++it)
        for (int nu = 0; nu < 3; ++nu)
            for (int q = 0; q < 3; ++q) {
                const int* t = T[nu][q];
                GridJob J{};
                J.in = c->W + ((it * 3 + t[2] - 1) * 3 + t[1] - 1) * V;
                double* out = c->divw_tmp + ((long)q * 6 + it * 3 + nu) * V;
                if (t[0] == 0) J.dx = out;
                else if (t[0] == 1) J.dy = out;
                else J.dz = out;
                for (int d = 0; d < 3; ++d)
                    J.slot[d] = (int8_t)lag_slot(d, t[3] * P, t[4] * S, TS, t[5]);
                jobs.push_back(J);
            }
    c->n_field_jobs = (int)jobs.size();
    MG_CUDA(cudaMalloc(&c->field_jobs, jobs.size() * sizeof(GridJob)));
    MG_CUDA(cudaMemcpy(c->field_jobs, jobs.data(), jobs.size() * sizeof(GridJob),
                       cudaMemcpyHostToDevice));
    return MG_OK;
}

int potentials(mg_ctx* c) {
    const long V = c->V;
    Coef k{c->B.B1, c->B.B2, c->B.B3, c->B.B4, c->B.B5, c->B.B6, c->B.B7a, c->B.B7b, c->B.B8a,
           c->B.B8b, c->B.byt3a, c->B.byt3b, c->B.B9, c->B.B9q, c->f.cexchange,
           c->B.B14, c->B.B15, c->B.B16, c->B.B17};
    k_potentials<<<div_up(V, kThreads), kThreads, 0, c->stream>>>(
        c->rho, c->tau, c->nablaj, c->derrho, c->laprho, c->coulomb, c->coulex,
        c->cons.list.empty() ? nullptr : c->cons.field, c->tensor ? c->jmunu : nullptr, k, V,
        c->U, c->Bp, c->W);
    MG_LAUNCHED(c);
    MG_TRY(run_jobs(c, c->field_jobs + 2, c->n_field_jobs - 2));
    k_sum3<<<div_up(6 * V, kThreads), kThreads, 0, c->stream>>>(c->divw_tmp, 6 * V, c->divW);
    MG_LAUNCHED(c);
    if (!c->p.trc) MG_TRY(time_odd_potentials(c));
    return MG_OK;
}

int moments(mg_ctx* c) {
    if (c->n_moments > 0) {
        k_moments<<<c->n_moments, kThreads, 0, c->stream>>>(c->sh_mesh, c->rho, c->V, c->dv,
                                                            c->moment_values);
        MG_LAUNCHED(c);
    }
    MG_TRY(constraint_moments(c));   // constraints.cu (nothing without constraints)
    // the cranking fields need the cutoff too (CompCutoff runs in every
    // CalculateAllMoments, src/Moments.f90:2267)
    if (cranking(c) && c->cons.list.empty()) MG_TRY(cranking_cutoff(c));
    return MG_OK;
}

}  // namespace mg
