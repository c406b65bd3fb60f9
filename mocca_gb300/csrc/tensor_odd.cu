// tensor_odd.cu -- the time-odd partners of the J^2 (tensor) terms without
// time-reversal invariance (cranked, signature and time simplex conserved),
// FP64.
//
// Replaces, for B14..B21 not all zero:
//   ComputeDensity's T, F, lap s and grad div s (src/Densities.f90:502-510,
//   :1043-1185):
//     T_m = sum_l Re(d_l psi^+ sigma_m d_l psi)       GetVecT src/Spwf.f90:2087-2129
//     F_m = Re(d_m psi^+ sum_n sigma_n d_n psi)       GetVecF :2162-2180
//     lap s with the symmetries of the s components; grad div s as the
//     reference forms it: its divergence accumulator adds each d_i s_i to a
//     field that is never assigned, so only d_z s_z reaches the gradient;
//   CalcSPot's tensor terms (src/MeanFields.f90:651-670; in timeodd.cu's
//   field kernel), CalcCPot and CalcDPot (:714-790):
//     C_q = -B14 s_t - B15 s_q,   D_q = -2 B16 s_t - 2 B17 s_q,  d_n D_m, div D;
//   ActionOfC and ActionOfD (:1149-1255), added to h.psi by hpsi.cu:
//     C psi = sum_n d_n [-sum_m C_m sigma_m d_n psi]
//     D psi = -1/2 [div D sigma.grad psi + sum_mn d_n D_m sigma_n d_m psi
//                   + 2 sum_mn D_m sigma_n d_m d_n psi];
//   compSkyrme's terms 21, 22, 27-32 (src/Energy.f90:775-845); 31 and 32
//   square the never-assigned divergence of s and are zero.
// The densities sit behind timeodd.cu's in the same buffer and mix with
// them (the DensityVector operators combine every allocated field).
#include <cstring>
#include <vector>

#include "mg_internal.cuh"

namespace mg {

namespace {

constexpr int kThreads = 256;
constexpr int kTensorOddSums = 8;

__device__ __forceinline__ void pauli(const double* p, int dir, double* o) {
    if (dir == 1) { o[0] = p[2]; o[1] = p[3]; o[2] = p[0]; o[3] = p[1]; }
    else if (dir == 2) { o[0] = p[3]; o[1] = -p[2]; o[2] = -p[1]; o[3] = p[0]; }
    else { o[0] = p[0]; o[1] = p[1]; o[2] = -p[2]; o[3] = -p[3]; }
}
// Re(a^+ b), unfused, left to right
__device__ __forceinline__ double re_mult(const double* a, const double* b) {
    return __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(a[0], b[0]), __dmul_rn(a[1], b[1])),
                               __dmul_rn(a[2], b[2])),
                     __dmul_rn(a[3], b[3]));
}

// T and F at one point, summed over the density basis in index order.  The
// partners of a time-reversal pair cancel (both densities are time-odd), so
// products and sums stay unfused, in the reference's order, like timeodd.cu's
// vecj and vecs.
__global__ void __launch_bounds__(kThreads)
k_tensor_dens(const double* __restrict__ der, const double* __restrict__ occ,
              const int* __restrict__ qn, int nwt, long V, int wantT, int wantF,
              double* __restrict__ vt, double* __restrict__ vf) {
    const long v = (long)blockIdx.x * kThreads + threadIdx.x;
    if (v >= V) return;
    double T[2][3] = {{0, 0, 0}, {0, 0, 0}}, F[2][3] = {{0, 0, 0}, {0, 0, 0}};
    for (int i = 0; i < nwt; ++i) {
        const double o = occ[i];
        if (o == 0.0) continue;
        const int it = (qn[4 * i] + 3) / 2 - 1;
        const double* dr = der + (long)i * 12 * V;
        double d[3][4];
#pragma unroll
        for (int m = 0; m < 3; ++m)
#pragma unroll
            for (int l = 0; l < 4; ++l) d[m][l] = dr[(m * 4 + l) * V + v];
        if (wantT) {
#pragma unroll
            for (int m = 0; m < 3; ++m) {
                double t = 0.0;
#pragma unroll
                for (int l = 0; l < 3; ++l) {
                    double sg[4];
                    pauli(d[l], m + 1, sg);
                    t = __dadd_rn(t, re_mult(d[l], sg));
                }
                T[it][m] = __dadd_rn(T[it][m], __dmul_rn(o, t));
            }
        }
        if (wantF) {
            double sd[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll
            for (int n = 0; n < 3; ++n) {
                double sg[4];
                pauli(d[n], n + 1, sg);
#pragma unroll
                for (int l = 0; l < 4; ++l) sd[l] = __dadd_rn(sd[l], sg[l]);
            }
#pragma unroll
            for (int m = 0; m < 3; ++m) F[it][m] = __dadd_rn(F[it][m], __dmul_rn(o, re_mult(d[m], sd)));
        }
    }
#pragma unroll
    for (int it = 0; it < 2; ++it)
#pragma unroll
        for (int m = 0; m < 3; ++m) {
            vt[(it * 3 + m) * V + v] = T[it][m];
            vf[(it * 3 + m) * V + v] = F[it][m];
        }
}

// C and D at one point
__global__ void k_cd_fields(const double* __restrict__ vecs, double B14, double B15, double B16,
                            double B17, long V, double* __restrict__ C, double* __restrict__ D) {
    const long v = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= V) return;
#pragma unroll
    for (int m = 0; m < 3; ++m) {
        const double st = vecs[m * V + v] + vecs[(3 + m) * V + v];
#pragma unroll
        for (int it = 0; it < 2; ++it) {
            const double sq = vecs[(it * 3 + m) * V + v];
            C[(it * 3 + m) * V + v] = __dsub_rn(-(B14 * st), B15 * sq);
            D[(it * 3 + m) * V + v] = __dsub_rn(-(2 * B16 * st), 2 * B17 * sq);
        }
    }
}

// div D = d_x D_x + d_y D_y + d_z D_z from dD [it][m][n][V]
__global__ void k_div_d(const double* __restrict__ dD, long V, double* __restrict__ divD) {
    const long v = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const int it = blockIdx.y;
    if (v >= V) return;
    const double* b = dD + (long)it * 9 * V;
    divD[it * V + v] = b[0 * V + v] + b[4 * V + v] + b[8 * V + v];
}

// Temp(n) = -sum_m C_m sigma_m d_n psi of spwf i: tmp [i][n][l][V]
__global__ void __launch_bounds__(kThreads)
k_c_temp(const double* __restrict__ der, const int* __restrict__ qn,
         const double* __restrict__ C, long V, double* __restrict__ tmp) {
    const int i = blockIdx.y;
    const long v = (long)blockIdx.x * kThreads + threadIdx.x;
    if (v >= V) return;
    const int it = (qn[4 * i] + 3) / 2 - 1;
    const double* dr = der + (long)i * 12 * V;
    const double c0 = C[(it * 3 + 0) * V + v], c1 = C[(it * 3 + 1) * V + v],
                 c2 = C[(it * 3 + 2) * V + v];
#pragma unroll
    for (int n = 0; n < 3; ++n) {
        double dn[4], t[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll
        for (int l = 0; l < 4; ++l) dn[l] = dr[(n * 4 + l) * V + v];
        double sg[4];
        pauli(dn, 1, sg);
#pragma unroll
        for (int l = 0; l < 4; ++l) t[l] = t[l] - c0 * sg[l];
        pauli(dn, 2, sg);
#pragma unroll
        for (int l = 0; l < 4; ++l) t[l] = t[l] - c1 * sg[l];
        pauli(dn, 3, sg);
#pragma unroll
        for (int l = 0; l < 4; ++l) t[l] = t[l] - c2 * sg[l];
#pragma unroll
        for (int l = 0; l < 4; ++l) tmp[(((long)i * 3 + n) * 4 + l) * V + v] = t[l];
    }
}

// x [i][2][l][V]: the C action (the three outer derivatives dC [i][n][l][V]
// summed) and the D action (dd [i][a][n][l][V] = d_a d_n psi)
__global__ void __launch_bounds__(kThreads)
k_cd_action(const double* __restrict__ der, const int* __restrict__ qn,
            const double* __restrict__ dC, const double* __restrict__ dd,
            const double* __restrict__ D, const double* __restrict__ dD,
            const double* __restrict__ divD, long V, int withC, int withD,
            double* __restrict__ x) {
    const int i = blockIdx.y;
    const long v = (long)blockIdx.x * kThreads + threadIdx.x;
    if (v >= V) return;
    const int it = (qn[4 * i] + 3) / 2 - 1;
    double* xc = x + (long)i * 8 * V;
    double* xd = xc + 4 * V;
    if (withC) {
        const double* b = dC + (long)i * 12 * V;
#pragma unroll
        for (int l = 0; l < 4; ++l)
            xc[l * V + v] = (b[(0 * 4 + l) * V + v] + b[(1 * 4 + l) * V + v]) + b[(2 * 4 + l) * V + v];
    } else {
#pragma unroll
        for (int l = 0; l < 4; ++l) xc[l * V + v] = 0.0;
    }
    if (!withD) {
#pragma unroll
        for (int l = 0; l < 4; ++l) xd[l * V + v] = 0.0;
        return;
    }
    const double* dr = der + (long)i * 12 * V;
    double d[3][4];
#pragma unroll
    for (int m = 0; m < 3; ++m)
#pragma unroll
        for (int l = 0; l < 4; ++l) d[m][l] = dr[(m * 4 + l) * V + v];
    double t1[4] = {0, 0, 0, 0}, t2[4] = {0, 0, 0, 0}, t3[4] = {0, 0, 0, 0};
#pragma unroll
    for (int m = 0; m < 3; ++m) {
        double sg[4];
        pauli(d[m], m + 1, sg);
#pragma unroll
        for (int l = 0; l < 4; ++l) t1[l] = t1[l] + sg[l];
    }
    const double dv = divD[it * V + v];
#pragma unroll
    for (int l = 0; l < 4; ++l) t1[l] = dv * t1[l];
#pragma unroll
    for (int m = 0; m < 3; ++m)
#pragma unroll
        for (int n = 0; n < 3; ++n) {
            double sg[4];
            pauli(d[m], n + 1, sg);
            const double g = dD[((it * 3 + m) * 3 + n) * V + v];
#pragma unroll
            for (int l = 0; l < 4; ++l) t2[l] = fma(g, sg[l], t2[l]);
        }
    const double* q = dd + (long)i * 36 * V;
#pragma unroll
    for (int m = 0; m < 3; ++m) {
        const double Dm = D[(it * 3 + m) * V + v];
#pragma unroll
        for (int n = 0; n < 3; ++n) {
            double w[4], sg[4];
#pragma unroll
            for (int l = 0; l < 4; ++l) w[l] = q[((m * 3 + n) * 4 + l) * V + v];
            pauli(w, n + 1, sg);
#pragma unroll
            for (int l = 0; l < 4; ++l) t3[l] = fma(Dm, sg[l], t3[l]);
        }
    }
#pragma unroll
    for (int l = 0; l < 4; ++l) xd[l * V + v] = -0.5 * ((t1[l] + t2[l]) + 2.0 * t3[l]);
}

// block partials of s_t.T_t, s_t.F_t, s_t.lap s_t, sum_q s_q.T_q, and per
// isospin s_q.F_q, s_q.lap s_q
__global__ void __launch_bounds__(kThreads)
k_tensor_odd_energy(const double* __restrict__ vecs, const double* __restrict__ vt,
                    const double* __restrict__ vf, const double* __restrict__ ls, long V,
                    double* __restrict__ part) {
    __shared__ double red[kThreads / 32][kTensorOddSums];
    double acc[kTensorOddSums];
#pragma unroll
    for (int q = 0; q < kTensorOddSums; ++q) acc[q] = 0.0;
    for (long v = (long)blockIdx.x * kThreads + threadIdx.x; v < V;
         v += (long)gridDim.x * kThreads) {
#pragma unroll
        for (int m = 0; m < 3; ++m) {
            const double s0 = vecs[m * V + v], s1 = vecs[(3 + m) * V + v];
            const double T0 = vt[m * V + v], T1 = vt[(3 + m) * V + v];
            const double F0 = vf[m * V + v], F1 = vf[(3 + m) * V + v];
            const double L0 = ls[m * V + v], L1 = ls[(3 + m) * V + v];
            const double st = s0 + s1;
            acc[0] = fma(st, T0 + T1, acc[0]);
            acc[1] = fma(st, F0 + F1, acc[1]);
            acc[2] = fma(st, L0 + L1, acc[2]);
            acc[3] = fma(s0, T0, fma(s1, T1, acc[3]));
            acc[4] = fma(s0, F0, acc[4]);
            acc[5] = fma(s1, F1, acc[5]);
            acc[6] = fma(s0, L0, acc[6]);
            acc[7] = fma(s1, L1, acc[7]);
        }
    }
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
#pragma unroll
    for (int q = 0; q < kTensorOddSums; ++q) {
        double x = acc[q];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
        if (lane == 0) red[warp][q] = x;
    }
    __syncthreads();
    if (threadIdx.x < kTensorOddSums) {
        double t = 0.0;
        for (int w = 0; w < kThreads / 32; ++w) t += red[w][threadIdx.x];
        part[(long)blockIdx.x * kTensorOddSums + threadIdx.x] = t;
    }
}

bool want_lap(const mg_skyrme_b& B) {
    return B.B18 != 0.0 || B.B19 != 0.0 || B.B20 != 0.0 || B.B21 != 0.0;
}

}  // namespace

// Buffers and the fixed derivative jobs (mg_create): lap s (6 jobs), d_z s_z
// (2), its gradient (2), the derivatives of D (6).
int tensor_odd_setup(mg_ctx* c) {
    const long V = c->V;
    auto A = [&](double** p, long n) {
        return cudaMalloc(p, n * sizeof(double)) == cudaSuccess &&
               cudaMemset(*p, 0, n * sizeof(double)) == cudaSuccess;
    };
    if (!(A(&c->Cpot, 6 * V) && A(&c->Dpot, 6 * V) && A(&c->dDpot, 18 * V) &&
          A(&c->divD, 2 * V) && A(&c->todd_tmp, 2 * V)))
        return MG_ERR_CUDA;
    double* ls = c->odd + 36 * V;   // lap s
    double* gd = c->odd + 42 * V;   // grad div s
    const double* vs = c->odd + 6 * V;
    std::vector<GridJob> jobs(16);
    for (int it = 0; it < 2; ++it) {
        for (int m = 0; m < 3; ++m) {
            // the s components: (P, -S, TS, 1), (P, -S, TS, 2), (P, S, TS, 1)
            const int ss = m == 2 ? 1 : -1, comp = m == 1 ? 2 : 1;
            GridJob& L = jobs[it * 3 + m];
            L = GridJob{};
            L.in = vs + (it * 3 + m) * V;
            L.lap = ls + (it * 3 + m) * V;
            for (int a = 0; a < 3; ++a) L.slot[a] = (int8_t)lag_slot(a, 1, ss, 1, comp);
            GridJob& G = jobs[10 + it * 3 + m];
            G = GridJob{};
            G.in = c->Dpot + (it * 3 + m) * V;
            double* o = c->dDpot + (it * 3 + m) * 3 * V;
            G.dx = o;
            G.dy = o + V;
            G.dz = o + 2 * V;
            for (int a = 0; a < 3; ++a) G.slot[a] = (int8_t)lag_slot(a, 1, ss, 1, comp);
        }
        GridJob& Z = jobs[6 + it];
        Z = GridJob{};
        Z.in = vs + (it * 3 + 2) * V;
        Z.dz = c->todd_tmp + it * V;
        for (int a = 0; a < 3; ++a) Z.slot[a] = (int8_t)lag_slot(a, 1, 1, 1, 1);
        GridJob& D = jobs[8 + it];
        D = GridJob{};
        D.in = c->todd_tmp + it * V;
        D.dx = gd + (it * 3 + 0) * V;
        D.dy = gd + (it * 3 + 1) * V;
        D.dz = gd + (it * 3 + 2) * V;
        for (int a = 0; a < 3; ++a) D.slot[a] = (int8_t)lag_slot(a, -1, 1, 1, 1);
    }
    MG_CUDA(cudaMalloc(&c->todd_jobs, jobs.size() * sizeof(GridJob)));
    MG_CUDA(cudaMemcpy(c->todd_jobs, jobs.data(), jobs.size() * sizeof(GridJob),
                       cudaMemcpyHostToDevice));
    return MG_OK;
}

// T, F of the density basis; lap s and grad div s of the new vecs.
int tensor_odd_densities(mg_ctx* c, const Basis& D) {
    const long V = c->V;
    const mg_skyrme_b& B = c->B;
    const int wantT = B.B14 != 0.0 || B.B15 != 0.0, wantF = B.B16 != 0.0 || B.B17 != 0.0;
    k_tensor_dens<<<div_up(V, kThreads), kThreads, 0, c->stream>>>(
        D.der, D.occ, D.qn, c->p.nwt, V, wantT, wantF, c->odd + 24 * V, c->odd + 30 * V);
    MG_LAUNCHED(c);
    if (want_lap(B)) {
        MG_TRY(run_jobs(c, c->todd_jobs, 8));       // lap s, d_z s_z
        MG_TRY(run_jobs(c, c->todd_jobs + 8, 2));   // its gradient
    }
    return MG_OK;
}

// C, D, the derivatives of D and div D (after the S field).
int tensor_odd_fields(mg_ctx* c) {
    const long V = c->V;
    const mg_skyrme_b& B = c->B;
    k_cd_fields<<<div_up(V, kThreads), kThreads, 0, c->stream>>>(
        c->odd + 6 * V, B.B14, B.B15, B.B16, B.B17, V, c->Cpot, c->Dpot);
    MG_LAUNCHED(c);
    if (B.B16 != 0.0 || B.B17 != 0.0) {
        MG_TRY(run_jobs(c, c->todd_jobs + 10, 6));
        k_div_d<<<dim3(div_up(V, kThreads), 2), kThreads, 0, c->stream>>>(c->dDpot, V, c->divD);
        MG_LAUNCHED(c);
    }
    return MG_OK;
}

// ActionOfC and ActionOfD of count spwfs (derivatives der [i][d][l][V],
// quantum numbers h_qn on the host and d_qn on the device) into
// x [i][2][l][V].  The outer derivatives take the symmetries of d_n psi:
// (-P, -S, TS) for x, (-P, -S, -TS) for y, (-P, S, TS) for z.
int tensor_odd_action(mg_ctx* c, const double* der, const int* h_qn, const int* d_qn, int count,
                      double* x) {
    const long V = c->V;
    const mg_skyrme_b& B = c->B;
    const bool withC = B.B14 != 0.0 || B.B15 != 0.0, withD = B.B16 != 0.0 || B.B17 != 0.0;
    if (count <= 0) return MG_OK;
    if (count > c->p.nwt) return MG_ERR_ARG;
    const size_t per = 60 * (size_t)V;   // tmp 12V, dC 12V, dd 36V
    if (!c->todd_work) {
        MG_CUDA(cudaMalloc(&c->todd_work, per * c->p.nwt * sizeof(double)));
        MG_CUDA(cudaMalloc(&c->todd_act_jobs, 24 * (size_t)c->p.nwt * sizeof(GridJob)));
    }
    double* tmp = c->todd_work;
    double* dC = tmp + 12 * (size_t)count * V;
    double* dd = dC + 12 * (size_t)count * V;
    std::vector<GridJob> jobs;
    jobs.reserve(24 * (size_t)count);
    for (int i = 0; i < count; ++i) {
        const int P = h_qn[4 * i + 1], S = h_qn[4 * i + 2], TS = h_qn[4 * i + 3];
        const int sp[3][2] = {{-S, TS}, {-S, -TS}, {S, TS}};
        for (int n = 0; n < 3; ++n)
            for (int l = 0; l < 4; ++l) {
                if (withC) {
                    GridJob J{};
                    J.in = tmp + (((size_t)i * 3 + n) * 4 + l) * V;
                    double* o = dC + (((size_t)i * 3 + n) * 4 + l) * V;
                    (n == 0 ? J.dx : n == 1 ? J.dy : J.dz) = o;
                    for (int a = 0; a < 3; ++a)
                        J.slot[a] = (int8_t)lag_slot(a, -P, sp[n][0], sp[n][1], l + 1);
                    jobs.push_back(J);
                }
                if (withD) {
                    GridJob J{};
                    J.in = der + (((size_t)i * 3 + n) * 4 + l) * V;
                    J.dx = dd + ((((size_t)i * 3 + 0) * 3 + n) * 4 + l) * V;
                    J.dy = dd + ((((size_t)i * 3 + 1) * 3 + n) * 4 + l) * V;
                    J.dz = dd + ((((size_t)i * 3 + 2) * 3 + n) * 4 + l) * V;
                    for (int a = 0; a < 3; ++a)
                        J.slot[a] = (int8_t)lag_slot(a, -P, sp[n][0], sp[n][1], l + 1);
                    jobs.push_back(J);
                }
            }
    }
    // the job table changes only with the spinors, their quantum numbers
    // and the count: upload it when it differs from the last one
    const size_t bytes = jobs.size() * sizeof(GridJob);
    if (bytes != c->todd_jobs_host.size() ||
        std::memcmp(c->todd_jobs_host.data(), jobs.data(), bytes) != 0) {
        MG_CUDA(cudaStreamSynchronize(c->stream));
        MG_CUDA(cudaMemcpy(c->todd_act_jobs, jobs.data(), bytes, cudaMemcpyHostToDevice));
        c->todd_jobs_host.assign(reinterpret_cast<const unsigned char*>(jobs.data()),
                                 reinterpret_cast<const unsigned char*>(jobs.data()) + bytes);
    }
    dim3 grid(div_up(V, kThreads), count);
    if (withC) {
        k_c_temp<<<grid, kThreads, 0, c->stream>>>(der, d_qn, c->Cpot, V, tmp);
        MG_LAUNCHED(c);
    }
    MG_TRY(run_jobs(c, c->todd_act_jobs, (int)jobs.size()));
    k_cd_action<<<grid, kThreads, 0, c->stream>>>(der, d_qn, dC, dd, c->Dpot, c->dDpot, c->divD,
                                                  V, withC ? 1 : 0, withD ? 1 : 0, x);
    MG_LAUNCHED(c);
    return MG_OK;
}

// compSkyrme's terms 21, 22, 27-32 (unscaled by dv) into t.
int tensor_odd_energy(mg_ctx* c, double* t) {
    const long V = c->V;
    const mg_skyrme_b& B = c->B;
    const int nblk = std::max(1, std::min(2 * c->num_sms, div_up(V, kThreads)));
    if ((size_t)nblk * kTensorOddSums > c->red_len) return MG_ERR_STATE;
    k_tensor_odd_energy<<<nblk, kThreads, 0, c->stream>>>(c->odd + 6 * V, c->odd + 24 * V,
                                                          c->odd + 30 * V, c->odd + 36 * V, V,
                                                          c->red);
    MG_LAUNCHED(c);
    std::vector<double> h((size_t)nblk * kTensorOddSums);
    MG_CUDA(cudaMemcpyAsync(h.data(), c->red, h.size() * sizeof(double), cudaMemcpyDeviceToHost,
                            c->stream));
    MG_CUDA(cudaStreamSynchronize(c->stream));
    double S[kTensorOddSums] = {0};
    for (int b = 0; b < nblk; ++b)
        for (int q = 0; q < kTensorOddSums; ++q) S[q] += h[(size_t)b * kTensorOddSums + q];
    t[20] = B.B14 != 0.0 ? -B.B14 * S[0] : 0.0;
    t[21] = B.B15 != 0.0 ? -B.B15 * S[3] : 0.0;
    t[26] = B.B16 != 0.0 ? -2.0 * B.B16 * S[1] : 0.0;
    t[27] = B.B17 != 0.0 ? (0.0 - 2.0 * B.B17 * S[4]) - 2.0 * B.B17 * S[5] : 0.0;
    t[28] = B.B18 != 0.0 ? B.B18 * S[2] : 0.0;
    t[29] = B.B19 != 0.0 ? (0.0 + B.B19 * S[6]) + B.B19 * S[7] : 0.0;
    t[30] = 0.0;
    t[31] = 0.0;
    return MG_OK;
}

}  // namespace mg

extern "C" int mg_get_time_odd_tensor(mg_ctx* c, double* vect, double* vecf, double* laps,
                                      double* graddivs, double* cpot, double* dpot,
                                      double* divd) {
    if (!c || c->p.trc || !c->todd) return MG_ERR_ARG;
    const long V = c->V;
    const double* src[7] = {c->odd + 24 * V, c->odd + 30 * V, c->odd + 36 * V, c->odd + 42 * V,
                            c->Cpot, c->Dpot, c->divD};
    double* dst[7] = {vect, vecf, laps, graddivs, cpot, dpot, divd};
    for (int q = 0; q < 7; ++q)
        if (dst[q])
            MG_CUDA(cudaMemcpyAsync(dst[q], src[q], (q == 6 ? 2 : 6) * V * sizeof(double),
                                    cudaMemcpyDeviceToHost, c->stream));
    MG_CUDA(cudaStreamSynchronize(c->stream));
    return MG_OK;
}
