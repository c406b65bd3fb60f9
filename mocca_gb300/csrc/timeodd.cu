// timeodd.cu -- time-odd densities and fields without time-reversal
// invariance (cranked, signature and time simplex conserved), FP64.
//
// Replaces, for the functional without N2LO terms (the time-odd tensor
// terms are in tensor_odd.cu):
//   ComputeDensity's time-odd part (src/Densities.f90:431-550, :1004-1106):
//     vecj_q += v^2 Im(psi^+ d_m psi)   GetVecj src/Spwf.f90:2034-2046
//     vecs_q += v^2 Re(psi^+ sigma_m psi)  GetVecs :2066-2079
//     and their curls, with the symmetry arguments of Table V of Hellemans
//     et al., Phys. Rev. C 85 (2012) 014326 (the reference's table);
//   CalcAPot (src/MeanFields.f90:411-492) and CalcSPot (:618-712):
//     A_q = -2 ((B3+B4) j_q + B3 j_q') + (B9+B9q) rot s_q + B9 rot s_q'
//           - f_cut omega x r                       CrankAPot src/Cranking.f90:234-258
//     S_q = (B9+B9q) rot j_q + B9 rot j_q' + 2 ((B10+B11) s_q + B10 s_q')
//           + 2 ((B12+B13) rho^a s_q + B12 rho^a s_q') - f_cut omega / 2
//                                                   CrankSPot :309-324
//     div A from the Lagrange derivatives of the components;
//   compSkyrme's time-odd terms 5, 6, 13-18, 35, 36 (src/Energy.f90:623-860).
// The actions S.sigma psi and -i (A.grad psi + div A psi / 2) are in
// hpsi.cu's FP64 kernel; the mixing of the time-odd densities in mixing.cu.
// The cutoff f_cut is the Rutz cutoff of the constraints (constraints.cu),
// computed in every moments pass while cranking (CompCutoff runs in every
// CalculateAllMoments, src/Moments.f90:2267).
#include <cmath>
#include <vector>

#include "mg_internal.cuh"

namespace mg {

namespace {

constexpr int kThreads = 256;
constexpr int kOddTerms = 10;

__device__ __forceinline__ void pauli(const double* p, int dir, double* o) {
    if (dir == 1) { o[0] = p[2]; o[1] = p[3]; o[2] = p[0]; o[3] = p[1]; }
    else if (dir == 2) { o[0] = p[3]; o[1] = -p[2]; o[2] = -p[1]; o[3] = p[0]; }
    else { o[0] = p[0]; o[1] = p[1]; o[2] = -p[2]; o[3] = -p[3]; }
}
// Im(a^+ b) = a0 b1 - a1 b0 + a2 b3 - a3 b2, unfused, left to right
__device__ __forceinline__ double imag_mult(const double* a, const double* b) {
    return __dsub_rn(__dadd_rn(__dsub_rn(__dmul_rn(a[0], b[1]), __dmul_rn(a[1], b[0])),
                               __dmul_rn(a[2], b[3])),
                     __dmul_rn(a[3], b[2]));
}

// vecj and vecs at one point, summed over the density basis in index order
__global__ void __launch_bounds__(kThreads)
k_odd_dens(const double* __restrict__ psi, const double* __restrict__ der,
           const double* __restrict__ occ, const int* __restrict__ qn, int nwt, long V,
           double* __restrict__ vecj, double* __restrict__ vecs) {
    const long v = (long)blockIdx.x * kThreads + threadIdx.x;
    if (v >= V) return;
    double j[2][3] = {{0, 0, 0}, {0, 0, 0}}, s[2][3] = {{0, 0, 0}, {0, 0, 0}};
    for (int i = 0; i < nwt; ++i) {
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
        // unfused products and sums in the reference's order: the partners
        // of a time-reversal pair cancel in both densities, so the net
        // values are orders of magnitude below their terms and FMA
        // contraction alone would move them by ~eps times the terms
#pragma unroll
        for (int m = 0; m < 3; ++m) {
            double sg[4];
            pauli(p, m + 1, sg);
            const double sm = __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(p[0], sg[0]), __dmul_rn(p[1], sg[1])),
                                                  __dmul_rn(p[2], sg[2])),
                                        __dmul_rn(p[3], sg[3]));
            const double jm = imag_mult(p, d[m]);
            if (it == 0) {
                j[0][m] = __dadd_rn(j[0][m], __dmul_rn(o, jm));
                s[0][m] = __dadd_rn(s[0][m], __dmul_rn(o, sm));
            } else {
                j[1][m] = __dadd_rn(j[1][m], __dmul_rn(o, jm));
                s[1][m] = __dadd_rn(s[1][m], __dmul_rn(o, sm));
            }
        }
    }
#pragma unroll
    for (int it = 0; it < 2; ++it)
#pragma unroll
        for (int m = 0; m < 3; ++m) {
            vecj[(it * 3 + m) * V + v] = j[it][m];
            vecs[(it * 3 + m) * V + v] = s[it][m];
        }
}

// rot f from the derivatives d[(g * 3 + a) * 3 + m] (grid g = it*2 + pass,
// axis a, component m) of vecj (pass 0) and vecs (pass 1)
__global__ void k_odd_curls(const double* __restrict__ d, long V, double* __restrict__ rotj,
                            double* __restrict__ rots) {
    const long v = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const int g = blockIdx.y;   // it * 2 + pass
    if (v >= V) return;
    const int it = g / 2, pass = g % 2;
    auto D = [&](int a, int m) { return d[((long)(g * 3 + a) * 3 + m) * V + v]; };
    double* rot = (pass == 0 ? rotj : rots) + (long)it * 3 * V;
    rot[0 * V + v] = D(1, 2) - D(2, 1);
    rot[1 * V + v] = D(2, 0) - D(0, 2);
    rot[2 * V + v] = D(0, 1) - D(1, 0);
}

struct OddCoef {
    double B3, B4, B9, B9q, B10, B11, B12a, B13a, B12b, B13b, byt3a, byt3b;
    double B14, B15, B16, B17, B18, B19, B20, B21;
    double om[3];
    double dx;
    int nx, ny, crank;
};

// tz: T, F, lap s, grad div s ([it][m][V] each, tensor_odd.cu), or NULL
__global__ void k_odd_potentials(const double* __restrict__ rho, const double* __restrict__ vecj,
                                 const double* __restrict__ vecs, const double* __restrict__ rotj,
                                 const double* __restrict__ rots, const double* __restrict__ cut,
                                 const double* __restrict__ tz, OddCoef k, long V,
                                 double* __restrict__ A, double* __restrict__ S) {
    const long v = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= V) return;
    const double rt = rho[v] + rho[V + v];
    const double ra = pow(rt, k.byt3a);
    const double rb = (k.B12b != 0.0 || k.B13b != 0.0) ? pow(rt, k.byt3b) : 0.0;
    const int x = (int)(v % k.nx), y = (int)((v / k.nx) % k.ny), z = (int)(v / ((long)k.nx * k.ny));
    const double r[3] = {k.dx / 2.0 + k.dx * x, k.dx / 2.0 + k.dx * y, k.dx / 2.0 + k.dx * z};
    for (int it = 0; it < 2; ++it) {
        const int at = 1 - it;
        const double fc = k.crank ? cut[it * V + v] : 0.0;
        for (int m = 0; m < 3; ++m) {
            const long q = (it * 3 + m) * V + v, qa = (at * 3 + m) * V + v;
            double a = -2.0 * ((k.B3 + k.B4) * vecj[q] + k.B3 * vecj[qa]);
            a = a + ((k.B9 + k.B9q) * rots[q] + k.B9 * rots[qa]);
            double sv = (k.B9 + k.B9q) * rotj[q] + k.B9 * rotj[qa] +
                        2.0 * ((k.B10 + k.B11) * vecs[q] + k.B10 * vecs[qa]) +
                        2.0 * ((k.B12a + k.B13a) * (ra * vecs[q]) + k.B12a * (ra * vecs[qa]));
            if (tz) {
                // the time-odd tensor terms (src/MeanFields.f90:651-670)
                const double *T = tz, *F = tz + 6 * V, *L = tz + 12 * V, *G = tz + 18 * V;
                if (k.B14 != 0.0 || k.B15 != 0.0)
                    sv = sv - (k.B14 + k.B15) * T[q] - k.B14 * T[qa];
                if (k.B16 != 0.0 || k.B17 != 0.0)
                    sv = sv - 2.0 * (k.B16 + k.B17) * F[q] - 2.0 * k.B16 * F[qa];
                if (k.B18 != 0.0 || k.B19 != 0.0 || k.B20 != 0.0 || k.B21 != 0.0)
                    sv = sv + 2.0 * ((k.B18 + k.B19) * L[q] + k.B18 * L[qa]) -
                         2.0 * ((k.B20 + k.B21) * G[q] - k.B20 * G[qa]);
            }
            if (k.B12b != 0.0 || k.B13b != 0.0)
                sv = sv + 2.0 * ((k.B12b + k.B13b) * (rb * vecs[q]) + k.B12b * (rb * vecs[qa]));
            if (k.crank) {
                // - sum_jk eps_mjk omega_j r_k f_cut, in the reference's (k, j) order
                for (int kk = 0; kk < 3; ++kk)
                    for (int jj = 0; jj < 3; ++jj) {
                        int e = 0;
                        if (m != jj && jj != kk && kk != m)
                            e = ((m == 0 && jj == 1) || (m == 1 && jj == 2) || (m == 2 && jj == 0)) ? 1 : -1;
                        if (e != 0) a = a - e * k.om[jj] * r[kk] * fc;
                    }
                sv = sv - 1 / 2.0 * k.om[m] * fc;
            }
            A[q] = a;
            S[q] = sv;
        }
    }
}

__global__ void k_odd_sum3(const double* __restrict__ t, long V, double* __restrict__ out) {
    const long v = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const int it = blockIdx.y;
    if (v >= V) return;
    const double* b = t + (long)it * 3 * V;
    out[it * V + v] = b[v] + b[V + v] + b[2 * V + v];
}

// block partials of the ten time-odd energy sums
__global__ void __launch_bounds__(kThreads)
k_odd_energy(const double* __restrict__ rho, const double* __restrict__ vecj,
             const double* __restrict__ vecs, const double* __restrict__ rots, double byt3a,
             double byt3b, long V, double* __restrict__ part) {
    __shared__ double red[kThreads / 32][kOddTerms];
    double acc[kOddTerms];
#pragma unroll
    for (int q = 0; q < kOddTerms; ++q) acc[q] = 0.0;
    for (long v = (long)blockIdx.x * kThreads + threadIdx.x; v < V;
         v += (long)gridDim.x * kThreads) {
        const double rt = rho[v] + rho[V + v];
        const double ra = pow(rt, byt3a), rb = pow(rt, byt3b);
        for (int m = 0; m < 3; ++m) {
            const double j0 = vecj[m * V + v], j1 = vecj[(3 + m) * V + v];
            const double s0 = vecs[m * V + v], s1 = vecs[(3 + m) * V + v];
            const double r0 = rots[m * V + v], r1 = rots[(3 + m) * V + v];
            const double jt = j0 + j1, st = s0 + s1, rs = r0 + r1;
            acc[0] = fma(jt, jt, acc[0]);                    // sum j_t^2
            acc[1] = fma(jt, rs, acc[1]);                    // sum j_t . rot s_t
            acc[2] = fma(st, st, acc[2]);                    // sum s_t^2
            acc[3] = fma(ra, st * st, acc[3]);               // sum rho^a s_t^2
            acc[4] = fma(rb, st * st, acc[4]);               // sum rho^b s_t^2
            acc[5] = fma(j0, j0, fma(j1, j1, acc[5]));       // sum_q j_q^2
            acc[6] = fma(j0, r0, fma(j1, r1, acc[6]));       // sum_q j_q . rot s_q
            acc[7] = fma(s0, s0, fma(s1, s1, acc[7]));       // sum_q s_q^2
            acc[8] = fma(ra, s0 * s0 + s1 * s1, acc[8]);     // sum_q rho^a s_q^2
            acc[9] = fma(rb, s0 * s0 + s1 * s1, acc[9]);     // sum_q rho^b s_q^2
        }
    }
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
#pragma unroll
    for (int q = 0; q < kOddTerms; ++q) {
        double x = acc[q];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
        if (lane == 0) red[warp][q] = x;
    }
    __syncthreads();
    if (threadIdx.x < kOddTerms) {
        double t = 0.0;
        for (int w = 0; w < kThreads / 32; ++w) t += red[w][threadIdx.x];
        part[(long)blockIdx.x * kOddTerms + threadIdx.x] = t;
    }
}

}  // namespace

// Buffers and derivative jobs (mg_create, time reversal broken).
int time_odd_setup(mg_ctx* c) {
    const long V = c->V;
    auto A = [&](double** p, long n) {
        return cudaMalloc(p, n * sizeof(double)) == cudaSuccess &&
               cudaMemset(*p, 0, n * sizeof(double)) == cudaSuccess;
    };
    if (!(A(&c->odd, c->odd_len * V) && A(&c->odd_hist, c->odd_len * V) && A(&c->Apot, 6 * V) &&
          A(&c->Spot, 6 * V) && A(&c->divA, 2 * V) && A(&c->odd_der, 36 * V) &&
          A(&c->odd_tmp, 6 * V)))
        return MG_ERR_CUDA;
    // curls: grid (it, pass, component m), derivatives along the other axes
    std::vector<GridJob> jobs(18);
    for (int it = 0; it < 2; ++it)
        for (int pass = 0; pass < 2; ++pass)
            for (int m = 0; m < 3; ++m) {
                const int g = it * 2 + pass;
                GridJob& J = jobs[g * 3 + m];
                J = GridJob{};
                J.in = (pass == 0 ? c->odd : c->odd + 6 * V) + (it * 3 + m) * V;
                const int pp = pass == 0 ? -1 : 1, ss = m == 2 ? 1 : -1;
                const int comp = pass == 0 ? (m == 1 ? 1 : 2) : (m == 1 ? 2 : 1);
                double* outs[3];
                for (int a = 0; a < 3; ++a) {
                    outs[a] = a == m ? nullptr : c->odd_der + ((long)(g * 3 + a) * 3 + m) * V;
                    J.slot[a] = (int8_t)lag_slot(a, pp, ss, 1, comp);
                }
                J.dx = outs[0];
                J.dy = outs[1];
                J.dz = outs[2];
                J.lap = nullptr;
            }
    // div A: d_x A_x (-P, -S, TS, 2), d_y A_y (-P, -S, TS, 1), d_z A_z (-P, S, TS, 2)
    for (int it = 0; it < 2; ++it)
        for (int m = 0; m < 3; ++m) {
            GridJob& J = jobs[12 + it * 3 + m];
            J = GridJob{};
            J.in = c->Apot + (it * 3 + m) * V;
            const int ss = m == 2 ? 1 : -1, comp = m == 1 ? 1 : 2;
            for (int a = 0; a < 3; ++a) J.slot[a] = (int8_t)lag_slot(a, -1, ss, 1, comp);
            double* o = c->odd_tmp + (it * 3 + m) * V;
            J.dx = m == 0 ? o : nullptr;
            J.dy = m == 1 ? o : nullptr;
            J.dz = m == 2 ? o : nullptr;
            J.lap = nullptr;
        }
    MG_CUDA(cudaMalloc(&c->odd_jobs, jobs.size() * sizeof(GridJob)));
    MG_CUDA(cudaMemcpy(c->odd_jobs, jobs.data(), jobs.size() * sizeof(GridJob),
                       cudaMemcpyHostToDevice));
    if (c->todd) MG_TRY(tensor_odd_setup(c));
    return MG_OK;
}

// vecj, vecs of the density basis and their curls.
int time_odd_densities(mg_ctx* c, const Basis& D) {
    const long V = c->V;
    k_odd_dens<<<div_up(V, kThreads), kThreads, 0, c->stream>>>(D.psi, D.der, D.occ, D.qn, c->p.nwt,
                                                                V, c->odd, c->odd + 6 * V);
    MG_LAUNCHED(c);
    MG_TRY(run_jobs(c, c->odd_jobs, 12));
    k_odd_curls<<<dim3(div_up(V, kThreads), 4), kThreads, 0, c->stream>>>(
        c->odd_der, V, c->odd + 12 * V, c->odd + 18 * V);
    MG_LAUNCHED(c);
    if (c->todd) MG_TRY(tensor_odd_densities(c, D));
    return MG_OK;
}

// A, S (with the cranking fields) and div A.
int time_odd_potentials(mg_ctx* c) {
    const long V = c->V;
    const mg_skyrme_b& B = c->B;
    OddCoef k{B.B3, B.B4, B.B9, B.B9q, B.B10, B.B11, B.B12a, B.B13a, B.B12b, B.B13b, B.byt3a,
              B.byt3b, B.B14, B.B15, B.B16, B.B17, B.B18, B.B19, B.B20, B.B21,
              {c->p.omega[0], c->p.omega[1], c->p.omega[2]}, c->p.dx, c->nx, c->ny,
              cranking(c) ? 1 : 0};
    if (k.crank && !c->cons.cut) return MG_ERR_STATE;   // the moments pass computes it
    k_odd_potentials<<<div_up(V, kThreads), kThreads, 0, c->stream>>>(
        c->rho, c->odd, c->odd + 6 * V, c->odd + 12 * V, c->odd + 18 * V, c->cons.cut,
        c->todd ? c->odd + 24 * V : nullptr, k, V, c->Apot, c->Spot);
    MG_LAUNCHED(c);
    MG_TRY(run_jobs(c, c->odd_jobs + 12, 6));
    k_odd_sum3<<<dim3(div_up(V, kThreads), 2), kThreads, 0, c->stream>>>(c->odd_tmp, V, c->divA);
    MG_LAUNCHED(c);
    if (c->todd) MG_TRY(tensor_odd_fields(c));
    return MG_OK;
}

// compSkyrme's time-odd terms (unscaled by dv) into t.
int time_odd_energy(mg_ctx* c, double* t) {
    const long V = c->V;
    const mg_skyrme_b& B = c->B;
    const int nblk = std::max(1, std::min(2 * c->num_sms, div_up(V, kThreads)));
    if ((size_t)nblk * kOddTerms > c->red_len) return MG_ERR_STATE;
    k_odd_energy<<<nblk, kThreads, 0, c->stream>>>(c->rho, c->odd, c->odd + 6 * V,
                                                    c->odd + 18 * V, B.byt3a, B.byt3b, V, c->red);
    MG_LAUNCHED(c);
    std::vector<double> h((size_t)nblk * kOddTerms);
    MG_CUDA(cudaMemcpyAsync(h.data(), c->red, h.size() * sizeof(double), cudaMemcpyDeviceToHost,
                            c->stream));
    MG_CUDA(cudaStreamSynchronize(c->stream));
    double S[kOddTerms] = {0};
    for (int b = 0; b < nblk; ++b)
        for (int q = 0; q < kOddTerms; ++q) S[q] += h[(size_t)b * kOddTerms + q];
    t[4] = -B.B3 * S[0];
    t[5] = -B.B4 * S[5];
    t[12] = B.B9 * S[1];
    t[13] = B.B9q * S[6];
    t[14] = B.B10 * S[2];
    t[15] = B.B11 * S[7];
    t[16] = B.B12a * S[3];
    t[17] = B.B13a * S[8];
    t[34] = B.B12b != 0.0 ? B.B12b * S[4] : 0.0;
    t[35] = B.B13b != 0.0 ? B.B13b * S[9] : 0.0;
    if (c->todd) MG_TRY(tensor_odd_energy(c, t));
    return MG_OK;
}

}  // namespace mg

extern "C" int mg_get_time_odd(mg_ctx* c, double* vecj, double* vecs, double* rotj, double* rots,
                               double* apot, double* spot, double* diva) {
    if (!c || c->p.trc || !c->odd) return MG_ERR_ARG;
    const long V = c->V;
    const double* src[7] = {c->odd, c->odd + 6 * V, c->odd + 12 * V, c->odd + 18 * V, c->Apot,
                            c->Spot, c->divA};
    double* dst[7] = {vecj, vecs, rotj, rots, apot, spot, diva};
    for (int q = 0; q < 7; ++q)
        if (dst[q])
            MG_CUDA(cudaMemcpyAsync(dst[q], src[q], (q == 6 ? 2 : 6) * V * sizeof(double),
                                    cudaMemcpyDeviceToHost, c->stream));
    MG_CUDA(cudaStreamSynchronize(c->stream));
    return MG_OK;
}
