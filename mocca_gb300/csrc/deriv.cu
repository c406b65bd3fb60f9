// deriv.cu -- Lagrange-mesh first derivatives and Laplacians, FP64.
//
// Replaces Opt_LAG{X,Y,Z}_EV8 / Lapla_LAG_EV8
// (src/OptimizedDerivatives.f90:115-148, :306-338, :432-464, :551-615) and,
// for the symmetry-free box, DerLag{X,Y,Z} / Laplacian_Lag
// (src/Derivatives.f90:1080-1312 with zero line extension).  Every
// derivative is a small dense matrix applied along one axis of a real grid:
// out(i) = sum_q M(i,q) in(q), q ascending, so the FP64 result follows the
// reference's matmul order (with fused multiply-adds).
//
// A batch of grids is described by a GridJob table (one job per real grid:
// a spinor component, a density or a field).  Two kernels cover a job:
//   k_deriv_xy : per z-plane, d/dx, d/dy and Lxx+Lyy (plane staged in smem)
//   k_deriv_z  : per tile of (x,y) columns, d/dz and lap += Lzz
// so the Laplacian is summed (X + Y) + Z as in Lapla_LAG_EV8.
// Matrices are stored transposed, MT[q*n + i], so the threads of a warp
// (consecutive output points i) read consecutive shared-memory words.
#include "mg_internal.cuh"

namespace mg {

namespace {

constexpr int kThreads = 256;
constexpr int kColTile = 32;  // (x,y) columns per k_deriv_z block

struct MatPtrs {
    const double* m[3][2][2];  // [axis][kind][slot]
};

__global__ void __launch_bounds__(kThreads)
k_deriv_xy(const GridJob* __restrict__ jobs, MatPtrs mp, int nx, int ny, int nz,
           int planes_per_block) {
    extern __shared__ double sm[];
    const GridJob J = jobs[blockIdx.x];
    const bool want_x = J.dx != nullptr || J.lap != nullptr;
    const bool want_y = J.dy != nullptr || J.lap != nullptr;
    if (!want_x && !want_y) return;
    double* sDx = sm;
    double* sLx = sDx + nx * nx;
    double* sDy = sLx + nx * nx;
    double* sLy = sDy + ny * ny;
    double* sP = sLy + ny * ny;
    const double* gDx = J.slot[0] ? mp.m[0][0][1] : mp.m[0][0][0];
    const double* gLx = J.slot[0] ? mp.m[0][1][1] : mp.m[0][1][0];
    const double* gDy = J.slot[1] ? mp.m[1][0][1] : mp.m[1][0][0];
    const double* gLy = J.slot[1] ? mp.m[1][1][1] : mp.m[1][1][0];
    for (int t = threadIdx.x; t < nx * nx; t += kThreads) {
        sDx[t] = gDx[t];
        sLx[t] = gLx[t];
    }
    for (int t = threadIdx.x; t < ny * ny; t += kThreads) {
        sDy[t] = gDy[t];
        sLy[t] = gLy[t];
    }
    const int plane = nx * ny;
    const int k0 = blockIdx.y * planes_per_block;
    const int k1 = min(nz, k0 + planes_per_block);
    for (int k = k0; k < k1; ++k) {
        const double* in = J.in + (long)k * plane;
        __syncthreads();
        for (int t = threadIdx.x; t < plane; t += kThreads) sP[t] = in[t];
        __syncthreads();
        for (int t = threadIdx.x; t < plane; t += kThreads) {
            const int x = t % nx, y = t / nx;
            const long o = (long)k * plane + t;
            double ax = 0.0, axx = 0.0, ay = 0.0, ayy = 0.0;
            if (want_x) {
                const double* row = sP + y * nx;
#pragma unroll 4
                for (int q = 0; q < nx; ++q) {
                    const double v = row[q];
                    ax = fma(sDx[q * nx + x], v, ax);
                    axx = fma(sLx[q * nx + x], v, axx);
                }
            }
            if (want_y) {
#pragma unroll 4
                for (int q = 0; q < ny; ++q) {
                    const double v = sP[q * nx + x];
                    ay = fma(sDy[q * ny + y], v, ay);
                    ayy = fma(sLy[q * ny + y], v, ayy);
                }
            }
            if (J.dx) J.dx[o] = ax;
            if (J.dy) J.dy[o] = ay;
            if (J.lap) J.lap[o] = axx + ayy;
        }
    }
}

__global__ void __launch_bounds__(kThreads)
k_deriv_z(const GridJob* __restrict__ jobs, MatPtrs mp, int nx, int ny, int nz) {
    extern __shared__ double sm[];
    const GridJob J = jobs[blockIdx.x];
    if (J.dz == nullptr && J.lap == nullptr) return;
    double* sDz = sm;
    double* sLz = sDz + nz * nz;
    double* sG = sLz + nz * nz;  // [q][col]
    const double* gDz = J.slot[2] ? mp.m[2][0][1] : mp.m[2][0][0];
    const double* gLz = J.slot[2] ? mp.m[2][1][1] : mp.m[2][1][0];
    for (int t = threadIdx.x; t < nz * nz; t += kThreads) {
        sDz[t] = gDz[t];
        sLz[t] = gLz[t];
    }
    const int plane = nx * ny;
    const int c0 = blockIdx.y * kColTile;
    const int col = threadIdx.x % kColTile;
    const int rg = threadIdx.x / kColTile;
    constexpr int kRowGroups = kThreads / kColTile;
    for (int t = threadIdx.x; t < nz * kColTile; t += kThreads) {
        const int q = t / kColTile, cc = t % kColTile;
        sG[t] = (c0 + cc < plane) ? J.in[(long)q * plane + c0 + cc] : 0.0;
    }
    __syncthreads();
    if (c0 + col >= plane) return;
    for (int i = rg; i < nz; i += kRowGroups) {
        double az = 0.0, azz = 0.0;
#pragma unroll 4
        for (int q = 0; q < nz; ++q) {
            const double v = sG[q * kColTile + col];
            az = fma(sDz[q * nz + i], v, az);
            azz = fma(sLz[q * nz + i], v, azz);
        }
        const long o = (long)i * plane + c0 + col;
        if (J.dz) J.dz[o] = az;
        if (J.lap) J.lap[o] = J.lap[o] + azz;
    }
}

MatPtrs mat_ptrs(const mg_ctx* c) {
    MatPtrs mp;
    for (int a = 0; a < 3; ++a)
        for (int k = 0; k < 2; ++k)
            for (int s = 0; s < 2; ++s) mp.m[a][k][s] = c->mats + c->mat_off[a][k][s];
    return mp;
}

}  // namespace

int upload_matrices(mg_ctx* c) {
    const int ns[3] = {c->nx, c->ny, c->nz};
    long total = 0;
    for (int a = 0; a < 3; ++a)
        for (int k = 0; k < 2; ++k)
            for (int s = 0; s < 2; ++s) {
                c->mat_off[a][k][s] = total;
                total += (long)ns[a] * ns[a];
            }
    std::vector<double> h(total);
    for (int a = 0; a < 3; ++a) {
        const int n = ns[a];
        const long nn = (long)n * n;
        std::vector<double> d1(2 * nn), d2(2 * nn);
        int st = mg_lagrange_matrices(n, c->p.dx, c->folded ? 1 : 0, d1.data(), d2.data());
        if (st != MG_OK) return st;
        for (int s = 0; s < 2; ++s)
            for (int i = 0; i < n; ++i)
                for (int q = 0; q < n; ++q) {
                    h[c->mat_off[a][0][s] + (long)q * n + i] = d1[s * nn + (long)i * n + q];
                    h[c->mat_off[a][1][s] + (long)q * n + i] = d2[s * nn + (long)i * n + q];
                }
    }
    MG_CUDA(cudaMalloc(&c->mats, total * sizeof(double)));
    MG_CUDA(cudaMemcpy(c->mats, h.data(), total * sizeof(double), cudaMemcpyHostToDevice));
    return MG_OK;
}

int build_basis_jobs(mg_ctx* c, int b) {
    Basis& B = c->bas[b];
    const int nwt = c->p.nwt;
    const long V = c->V;
    std::vector<GridJob> jobs(4 * nwt);
    for (int i = 0; i < nwt; ++i) {
        const int P = B.h_qn[4 * i + 1], S = B.h_qn[4 * i + 2], TS = B.h_qn[4 * i + 3];
        for (int l = 0; l < 4; ++l) {
            GridJob& J = jobs[4 * i + l];
            J.in = B.psi + ((long)i * 4 + l) * V;
            J.dx = B.der + ((long)i * 12 + 0 * 4 + l) * V;
            J.dy = B.der + ((long)i * 12 + 1 * 4 + l) * V;
            J.dz = B.der + ((long)i * 12 + 2 * 4 + l) * V;
            J.lap = B.lap + ((long)i * 4 + l) * V;
            for (int d = 0; d < 3; ++d) J.slot[d] = (int8_t)lag_slot(d, P, S, TS, l + 1);
        }
    }
    MG_CUDA(cudaMemcpyAsync(B.jobs, jobs.data(), jobs.size() * sizeof(GridJob),
                            cudaMemcpyHostToDevice, c->stream));
    MG_CUDA(cudaStreamSynchronize(c->stream));
    return MG_OK;
}

int run_jobs(mg_ctx* c, const GridJob* jobs, int njobs) {
    if (njobs <= 0) return MG_OK;
    const int nx = c->nx, ny = c->ny, nz = c->nz;
    MatPtrs mp = mat_ptrs(c);
    const int ppb = 4;
    size_t sm_xy = (size_t)(2 * nx * nx + 2 * ny * ny + nx * ny) * sizeof(double);
    size_t sm_z = (size_t)(2 * nz * nz + nz * kColTile) * sizeof(double);
    static bool attr_done = false;
    if (!attr_done) {
        MG_CUDA(cudaFuncSetAttribute(k_deriv_xy, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     200 * 1024));
        MG_CUDA(cudaFuncSetAttribute(k_deriv_z, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     200 * 1024));
        attr_done = true;
    }
    dim3 gxy(njobs, div_up(nz, ppb));
    k_deriv_xy<<<gxy, kThreads, sm_xy, c->stream>>>(jobs, mp, nx, ny, nz, ppb);
    MG_LAUNCHED(c);
    dim3 gz(njobs, div_up((long)nx * ny, kColTile));
    k_deriv_z<<<gz, kThreads, sm_z, c->stream>>>(jobs, mp, nx, ny, nz);
    MG_LAUNCHED(c);
    return MG_OK;
}

int derive_basis(mg_ctx* c, int b) {
    if (!c->bas[b].have_qn) return MG_ERR_STATE;
    return run_jobs(c, c->bas[b].jobs, 4 * c->p.nwt);
}

}  // namespace mg
