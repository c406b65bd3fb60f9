// mixing.cu -- the reference's mixing between iterations, FP64.
//
//   scheme 0 (default): MixDensities, src/DensityMixing.f90:38-47: every
//     density is mixed with the previous iteration's,
//     Density = (1 - DampingParam) Density + DampingParam DensityHistory(1);
//     UpdateDensities(0) (src/Densities.f90:406-429) keeps the replaced
//     densities as that history.
//   scheme 2: the U update is preconditioned instead,
//     Upot = UpotOld + PreconditionPotential(Upot - UpotOld)
//     and, without time reversal, each component of the S update with the
//     symmetries of s, and with PreConW > 0 each W component's
//     (src/PotentialMixing.f90:143-210,
//     src/Damping.f90:158-228): per isospin
//     a CG on (beta + alpha Lap) x = dU with alpha = -preconu, beta = 1 and
//     the Lagrange Laplacian, at most 300 steps, stopping when
//     sum(residual^2) dv < 1e-8.  Both isospins step together with their own
//     scalars; an isospin that has converged stops changing.  The sums are
//     block partials added on the host in block order (deterministic).
#include <cmath>
#include <vector>

#include "mg_internal.cuh"

namespace mg {

namespace {

constexpr int kThreads = 256;

__global__ void k_mix(double* __restrict__ x, const double* __restrict__ h, long n, double d) {
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) x[t] = (1.0 - d) * x[t] + d * h[t];
}

__device__ double block_sum(double s, double* red) {
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (threadIdx.x % 32 == 0) red[threadIdx.x / 32] = s;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x == 0)
        for (int q = 0; q < kThreads / 32; ++q) t += red[q];
    return t;
}

// upd = beta dir + alpha lap (isospin blockIdx.y) and block partials of dir.upd
__global__ void __launch_bounds__(kThreads)
k_pc_update(const double* __restrict__ dir, const double* __restrict__ lap,
            double* __restrict__ upd, long V, double alpha, double beta,
            double* __restrict__ part) {
    __shared__ double red[kThreads / 32];
    const int it = blockIdx.y;
    const long v = (long)blockIdx.x * kThreads + threadIdx.x;
    double s = 0.0;
    if (v < V) {
        const long o = it * V + v;
        const double u = beta * dir[o] + alpha * lap[o];
        upd[o] = u;
        s = dir[o] * u;
    }
    const double t = block_sum(s, red);
    if (threadIdx.x == 0) part[(long)it * gridDim.x + blockIdx.x] = t;
}

// inv += a dir, res -= a upd (per isospin), block partials of res.res
__global__ void __launch_bounds__(kThreads)
k_pc_step(double* __restrict__ inv, double* __restrict__ res, const double* __restrict__ dir,
          const double* __restrict__ upd, long V, double a0, double a1,
          double* __restrict__ part) {
    __shared__ double red[kThreads / 32];
    const int it = blockIdx.y;
    const double a = it == 0 ? a0 : a1;
    const long v = (long)blockIdx.x * kThreads + threadIdx.x;
    double s = 0.0;
    if (v < V) {
        const long o = it * V + v;
        inv[o] = inv[o] + a * dir[o];
        const double r = res[o] - a * upd[o];
        res[o] = r;
        s = r * r;
    }
    const double t = block_sum(s, red);
    if (threadIdx.x == 0) part[(long)it * gridDim.x + blockIdx.x] = t;
}

// dir = res + b dir (isospins with b < 0 are left alone: converged)
__global__ void k_pc_direction(double* __restrict__ dir, const double* __restrict__ res, long V,
                               double b0, double b1) {
    const int it = blockIdx.y;
    const double b = it == 0 ? b0 : b1;
    const long v = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= V || b < 0.0) return;
    dir[it * V + v] = res[it * V + v] + b * dir[it * V + v];
}

// dir = res = dU, inv = 0, block partials of dU.dU (the potential's
// isospins stride apart)
__global__ void __launch_bounds__(kThreads)
k_pc_start(const double* __restrict__ U, const double* __restrict__ Uold, long stride,
           double* __restrict__ res, double* __restrict__ dir, double* __restrict__ inv, long V,
           double* __restrict__ part) {
    __shared__ double red[kThreads / 32];
    const int it = blockIdx.y;
    const long v = (long)blockIdx.x * kThreads + threadIdx.x;
    double s = 0.0;
    if (v < V) {
        const long o = it * V + v;
        const double d = U[it * stride + v] - Uold[it * stride + v];
        res[o] = d;
        dir[o] = d;
        inv[o] = 0.0;
        s = d * d;
    }
    const double t = block_sum(s, red);
    if (threadIdx.x == 0) part[(long)it * gridDim.x + blockIdx.x] = t;
}

__global__ void k_pc_finish(double* __restrict__ U, const double* __restrict__ Uold, long stride,
                            const double* __restrict__ inv, long V) {
    const long v = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const int it = blockIdx.y;
    if (v < V) U[it * stride + v] = Uold[it * stride + v] + inv[it * V + v];
}

}  // namespace

// Device buffers and the two Laplacian jobs of the preconditioner.
int mixing_setup(mg_ctx* c) {
    const long V = c->V;
    auto A = [&](double** p, long n) {
        return cudaMalloc(p, n * sizeof(double)) == cudaSuccess &&
               cudaMemset(*p, 0, n * sizeof(double)) == cudaSuccess;
    };
    if (!(A(&c->dhist, 14 * V) && A(&c->Uold, 2 * V) && A(&c->pc_buf, 10 * V)))
        return MG_ERR_CUDA;
    if (!c->p.trc && !A(&c->Sold, 6 * V)) return MG_ERR_CUDA;
    if (c->p.precon_w > 0.0 && !A(&c->Wold, 18 * V)) return MG_ERR_CUDA;
    // the Laplacian of the direction: U (P, S, TS, 1); the S components
    // (P, -S, TS, 1), (P, -S, TS, 2), (P, S, TS, 1); the W classes
    // (-P, S, TS, 2) of W_11, W_22, W_33, (-P, S, TS, 1) of W_12, W_21,
    // (-P, -S, TS, 2) of W_13, W_31, (-P, -S, TS, 1) of W_23, W_32
    std::vector<GridJob> jobs(16);
    const int P = c->p.pc, S = c->p.sc, TS = c->p.tsc;
    const int sym[8][3] = {{P, S, 1},   {P, -S, 1},  {P, -S, 2},  {P, S, 1},
                           {-P, S, 2},  {-P, S, 1},  {-P, -S, 2}, {-P, -S, 1}};
    for (int k = 0; k < 8; ++k)
        for (int it = 0; it < 2; ++it) {
            GridJob J{};
            J.in = c->pc_buf + (2 + it) * V;        // direction
            J.lap = c->pc_buf + (6 + it) * V;       // Laplacian of the direction
            for (int d = 0; d < 3; ++d)
                J.slot[d] = (int8_t)lag_slot(d, sym[k][0], sym[k][1], TS, sym[k][2]);
            jobs[2 * k + it] = J;
        }
    MG_CUDA(cudaMalloc(&c->pc_jobs, jobs.size() * sizeof(GridJob)));
    MG_CUDA(cudaMemcpy(c->pc_jobs, jobs.data(), jobs.size() * sizeof(GridJob),
                       cudaMemcpyHostToDevice));
    return MG_OK;
}

// UpdateDensities(0): the current densities become the history.
int save_density_history(mg_ctx* c) {
    const long V = c->V;
    const double* src[5] = {c->rho, c->tau, c->nablaj, c->derrho, c->laprho};
    const long len[5] = {2 * V, 2 * V, 2 * V, 6 * V, 2 * V};
    long off = 0;
    for (int q = 0; q < 5; ++q) {
        MG_CUDA(cudaMemcpyAsync(c->dhist + off, src[q], len[q] * sizeof(double),
                                cudaMemcpyDeviceToDevice, c->stream));
        off += len[q];
    }
    if (c->odd)
        MG_CUDA(cudaMemcpyAsync(c->odd_hist, c->odd, c->odd_len * V * sizeof(double),
                                cudaMemcpyDeviceToDevice, c->stream));
    if (c->tensor)
        MG_CUDA(cudaMemcpyAsync(c->jmunu_hist, c->jmunu, 18 * V * sizeof(double),
                                cudaMemcpyDeviceToDevice, c->stream));
    c->have_dhist = true;
    return MG_OK;
}

int mix_densities(mg_ctx* c) {
    if (c->p.mixing_scheme != 0 || !c->have_dhist) return MG_OK;
    const long V = c->V;
    double* dst[5] = {c->rho, c->tau, c->nablaj, c->derrho, c->laprho};
    const long len[5] = {2 * V, 2 * V, 2 * V, 6 * V, 2 * V};
    long off = 0;
    for (int q = 0; q < 5; ++q) {
        k_mix<<<div_up(len[q], kThreads), kThreads, 0, c->stream>>>(dst[q], c->dhist + off, len[q],
                                                                    c->p.damping);
        MG_LAUNCHED(c);
        off += len[q];
    }
    if (c->odd) {   // the time-odd densities mix with the rest
        k_mix<<<div_up(c->odd_len * V, kThreads), kThreads, 0, c->stream>>>(c->odd, c->odd_hist, c->odd_len * V,
                                                                    c->p.damping);
        MG_LAUNCHED(c);
    }
    if (c->tensor) {   // and J_{mu nu}
        k_mix<<<div_up(18 * V, kThreads), kThreads, 0, c->stream>>>(c->jmunu, c->jmunu_hist,
                                                                    18 * V, c->p.damping);
        MG_LAUNCHED(c);
    }
    return MG_OK;
}

static int read_pair(mg_ctx* c, int nblk, std::vector<double>& h, double out[2]) {
    MG_CUDA(cudaMemcpyAsync(h.data(), c->red, 2 * nblk * sizeof(double), cudaMemcpyDeviceToHost,
                            c->stream));
    MG_CUDA(cudaStreamSynchronize(c->stream));
    for (int it = 0; it < 2; ++it) {
        double s = 0.0;
        for (int q = 0; q < nblk; ++q) s += h[(size_t)it * nblk + q];
        out[it] = s * c->dv;
    }
    return MG_OK;
}

// F = Fold + PreconditionPotential(F - Fold) for a potential whose two
// isospins lie stride apart, with the Laplacian jobs of its symmetry
static int precondition_pot(mg_ctx* c, double* F, const double* Fold, long stride,
                            const GridJob* jobs) {
    const long V = c->V;
    const int nblk = div_up(V, kThreads);
    const dim3 g2(nblk, 2);
    double* res = c->pc_buf;
    double* dir = c->pc_buf + 2 * V;
    double* upd = c->pc_buf + 4 * V;
    double* lap = c->pc_buf + 6 * V;
    double* inv = c->pc_buf + 8 * V;
    const double alpha = -c->p.precon_u, beta = 1.0;
    std::vector<double> h((size_t)2 * nblk);
    double nn[2], dd[2], nn_new[2];
    k_pc_start<<<g2, kThreads, 0, c->stream>>>(F, Fold, stride, res, dir, inv, V, c->red);
    MG_LAUNCHED(c);
    MG_TRY(read_pair(c, nblk, h, nn));
    // an isospin whose update is identically zero keeps it (its first CG
    // step would divide 0 by 0), e.g. W_11 of a functional without J^2 terms
    bool conv[2] = {nn[0] == 0.0, nn[1] == 0.0};
    for (int iter = 1; iter <= 300 && !(conv[0] && conv[1]); ++iter) {
        MG_TRY(run_jobs(c, jobs, 2));
        k_pc_update<<<g2, kThreads, 0, c->stream>>>(dir, lap, upd, V, alpha, beta, c->red);
        MG_LAUNCHED(c);
        MG_TRY(read_pair(c, nblk, h, dd));
        double a[2];
        for (int it = 0; it < 2; ++it) a[it] = conv[it] ? 0.0 : nn[it] / dd[it];
        k_pc_step<<<g2, kThreads, 0, c->stream>>>(inv, res, dir, upd, V, a[0], a[1], c->red);
        MG_LAUNCHED(c);
        MG_TRY(read_pair(c, nblk, h, nn_new));
        double b[2] = {-1.0, -1.0};
        for (int it = 0; it < 2; ++it) {
            if (conv[it]) continue;
            b[it] = nn_new[it] / nn[it];
            nn[it] = nn_new[it];
        }
        k_pc_direction<<<g2, kThreads, 0, c->stream>>>(dir, res, V, b[0], b[1]);
        MG_LAUNCHED(c);
        for (int it = 0; it < 2; ++it)
            if (!conv[it] && nn[it] < 1e-8) conv[it] = true;
    }
    k_pc_finish<<<g2, kThreads, 0, c->stream>>>(F, Fold, stride, inv, V);
    MG_LAUNCHED(c);
    return MG_OK;
}

// Upot = UpotOld + PreconditionPotential(Upot - UpotOld); without time
// reversal each S component the same way
int precondition_u(mg_ctx* c) {
    const long V = c->V;
    MG_TRY(precondition_pot(c, c->U, c->Uold, V, c->pc_jobs));
    if (!c->p.trc)
        for (int m = 0; m < 3; ++m)
            MG_TRY(precondition_pot(c, c->Spot + m * V, c->Sold + m * V, 3 * V,
                                    c->pc_jobs + 2 * (m + 1)));
    if (c->Wold) {
        // W (mu, nu) at [it][nu][mu]; its symmetry class by (mu, nu)
        const int cls[3][3] = {{4, 5, 6}, {5, 4, 7}, {6, 7, 4}};
        for (int mu = 0; mu < 3; ++mu)
            for (int nu = 0; nu < 3; ++nu) {
                const long off = (nu * 3 + mu) * V;
                MG_TRY(precondition_pot(c, c->W + off, c->Wold + off, 9 * V,
                                        c->pc_jobs + 2 * cls[mu][nu]));
            }
    }
    return MG_OK;
}

}  // namespace mg
