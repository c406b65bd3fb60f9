// multigrid.cu -- Coulomb Poisson solve by FP32 multigrid V-cycles inside an
// FP64 iteration (CoulombSolver = 2).
//
// The reference's MGSolve / VCycle / Restrict / Prolong
// (src/MultiGrid.f90:14-348, with Gauss_Seidel_Update
// src/CoulombDerivatives.f90:20-141) are a multigrid for the same problem as
// ConjugGrad: the 4th-order difference Laplacian on the stored box, mirror
// planes at the low end of each axis, the multipole Dirichlet values on the
// two planes beyond the high end (src/Coulomb.f90:255-346, :583-674).  Here
// the multigrid is the preconditioner of a conjugate-gradient iteration
// carried in FP64:
//   - FP64: the residual with the 4th-order operator and the Dirichlet
//     planes, the search directions, the two dot products of an iteration
//     (deterministic block partials summed in a fixed order), the updates of
//     the solution and the residual, the stopping test |r| <= tol |b|;
//   - FP32: one V-cycle per iteration on the 7-point Laplacian of each level
//     (spacing dx 2^l), with red-black Gauss-Seidel smoothing (one sweep red
//     then black before the coarse correction, one black then red after, so
//     the cycle is a symmetric operator), cell-centred restriction
//     R = P^T / 8 (weights 1/8, 3/8, 3/8, 1/8 per axis) and trilinear
//     prolongation P (3/4, 1/4 per axis), the mirror planes and the
//     homogeneous Dirichlet planes of the correction on every level, and a
//     single-block Gauss-Seidel solve of the coarsest level in shared memory.
// Coarsening halves every axis while all of them are even and the halves
// stay >= 3 (64 -> 32 -> 16 -> 8 -> 4, 24 -> 12 -> 6 -> 3); the coarsest
// level must fit the shared-memory solve (4096 points), so an odd line
// length above 16 is refused (MG_ERR_ARG).  The 7-point operator is
// spectrally equivalent to the 4th-order one (ratio between 1 and 4/3), so
// the preconditioned iteration needs few steps whatever the mesh.  Every
// kernel of an iteration first reads the convergence flag and returns once
// it is set; the host reads the flag every kChunk iterations, which replay
// as one CUDA graph.
#include <algorithm>
#include <cmath>
#include <vector>

#include "mg_internal.cuh"

namespace mg {

namespace {

constexpr int kThreads = 256;
constexpr int kMaxLevels = 8;
constexpr int kChunk = 4;           // iterations between host checks of the flag
constexpr int kCoarseMax = 4096;    // points of the coarsest level (shared memory)
constexpr int kPartBlocks = 256;    // blocks of the FP64 dot products

struct Level {
    int n[3];
    long V;
    float inv_h2;
    float *u, *f, *r;
};

struct PcgScalars {
    int conv;       // 1 once |r| <= tol |b|; 2 when the cap is reached first
    int iters;      // iterations run
    double bb;      // |b|^2
    double rz_old;  // r.z of the previous iteration
    double rr;      // |r|^2 of the last iteration
};

__device__ __forceinline__ void cell(long v, const int* n, int& i, int& j, int& k) {
    i = (int)(v % n[0]);
    j = (int)((v / n[0]) % n[1]);
    k = (int)(v / ((long)n[0] * n[1]));
}

// one colour of a red-black Gauss-Seidel sweep of A u = f on one level
__global__ void k_mg_smooth(float* __restrict__ u, const float* __restrict__ f, int nx, int ny,
                            int nz, float inv_h2, int color, const int* __restrict__ conv) {
    if (*conv) return;
    const long V = (long)nx * ny * nz;
    const long v = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= V) return;
    const int n[3] = {nx, ny, nz};
    int i, j, k;
    cell(v, n, i, j, k);
    if (((i + j + k) & 1) != color) return;
    const long sx = 1, sy = nx, sz = (long)nx * ny;
    float nb = 0.0f, diag = -6.0f;
    // low end: mirror (the neighbour is the cell itself); high end: zero
    if (i > 0) nb += u[v - sx]; else diag += 1.0f;
    if (i < nx - 1) nb += u[v + sx];
    if (j > 0) nb += u[v - sy]; else diag += 1.0f;
    if (j < ny - 1) nb += u[v + sy];
    if (k > 0) nb += u[v - sz]; else diag += 1.0f;
    if (k < nz - 1) nb += u[v + sz];
    u[v] = (f[v] / inv_h2 - nb) / diag;
}

__global__ void k_mg_residual(const float* __restrict__ u, const float* __restrict__ f,
                              float* __restrict__ r, int nx, int ny, int nz, float inv_h2,
                              const int* __restrict__ conv) {
    if (*conv) return;
    const long V = (long)nx * ny * nz;
    const long v = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= V) return;
    const int n[3] = {nx, ny, nz};
    int i, j, k;
    cell(v, n, i, j, k);
    const long sx = 1, sy = nx, sz = (long)nx * ny;
    const float c = u[v];
    float a = -6.0f * c;
    a += i > 0 ? u[v - sx] : c;
    a += i < nx - 1 ? u[v + sx] : 0.0f;
    a += j > 0 ? u[v - sy] : c;
    a += j < ny - 1 ? u[v + sy] : 0.0f;
    a += k > 0 ? u[v - sz] : c;
    a += k < nz - 1 ? u[v + sz] : 0.0f;
    r[v] = f[v] - inv_h2 * a;
}

// per-axis restriction weights of coarse c: fine 2c-1 .. 2c+2 (P^T / 2)
__device__ __forceinline__ void rweights(int c, int nf, int* fi, float* w) {
    fi[0] = 2 * c - 1; w[0] = c > 0 ? 0.125f : 0.0f;
    fi[1] = 2 * c;     w[1] = c > 0 ? 0.375f : 0.5f;
    fi[2] = 2 * c + 1; w[2] = 0.375f;
    fi[3] = 2 * c + 2; w[3] = 2 * c + 2 < nf ? 0.125f : 0.0f;
}

__global__ void k_mg_restrict(const float* __restrict__ rf, float* __restrict__ fc, int fx,
                              int fy, int fz, int cx, int cy, int cz, const int* __restrict__ conv) {
    if (*conv) return;
    const long Vc = (long)cx * cy * cz;
    const long v = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= Vc) return;
    const int n[3] = {cx, cy, cz};
    int I, J, K;
    cell(v, n, I, J, K);
    int ix[4], iy[4], iz[4];
    float wx[4], wy[4], wz[4];
    rweights(I, fx, ix, wx);
    rweights(J, fy, iy, wy);
    rweights(K, fz, iz, wz);
    float s = 0.0f;
    for (int c = 0; c < 4; ++c) {
        if (wz[c] == 0.0f) continue;
        for (int b = 0; b < 4; ++b) {
            if (wy[b] == 0.0f) continue;
            const long row = (long)fx * (iy[b] + (long)fy * iz[c]);
            float sr = 0.0f;
            for (int a = 0; a < 4; ++a)
                if (wx[a] != 0.0f) sr = fmaf(wx[a], rf[row + ix[a]], sr);
            s = fmaf(wy[b] * wz[c], sr, s);
        }
    }
    fc[v] = s;
}

// per-axis prolongation of fine f: coarse f/2 (3/4) and its neighbour on the
// side of f (1/4); the low-end neighbour is the mirror image, the high-end
// one the zero Dirichlet value
__device__ __forceinline__ void pweights(int f, int nc, int* ci, float* w) {
    const int c = f >> 1;
    ci[0] = c;
    w[0] = 0.75f;
    if (f & 1) {
        ci[1] = c + 1 < nc ? c + 1 : c;
        w[1] = c + 1 < nc ? 0.25f : 0.0f;
    } else {
        ci[1] = c > 0 ? c - 1 : 0;
        w[1] = 0.25f;
    }
}

__global__ void k_mg_prolong(float* __restrict__ uf, const float* __restrict__ uc, int fx, int fy,
                             int fz, int cx, int cy, int cz, const int* __restrict__ conv) {
    if (*conv) return;
    const long Vf = (long)fx * fy * fz;
    const long v = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= Vf) return;
    const int n[3] = {fx, fy, fz};
    int i, j, k;
    cell(v, n, i, j, k);
    int ix[2], iy[2], iz[2];
    float wx[2], wy[2], wz[2];
    pweights(i, cx, ix, wx);
    pweights(j, cy, iy, wy);
    pweights(k, cz, iz, wz);
    float s = 0.0f;
    for (int c = 0; c < 2; ++c)
        for (int b = 0; b < 2; ++b)
            for (int a = 0; a < 2; ++a) {
                const float w = wx[a] * wy[b] * wz[c];
                if (w != 0.0f) s = fmaf(w, uc[ix[a] + (long)cx * (iy[b] + (long)cy * iz[c])], s);
            }
    uf[v] += s;
}

// the coarsest level: Gauss-Seidel sweeps in shared memory by one block
__global__ void __launch_bounds__(1024)
k_mg_coarsest(float* __restrict__ u, const float* __restrict__ f, int nx, int ny, int nz,
              float inv_h2, int sweeps, const int* __restrict__ conv) {
    if (*conv) return;
    __shared__ float su[kCoarseMax], sf[kCoarseMax];
    const int V = nx * ny * nz;
    for (int v = threadIdx.x; v < V; v += blockDim.x) {
        su[v] = 0.0f;
        sf[v] = f[v] / inv_h2;
    }
    __syncthreads();
    const int sy = nx, sz = nx * ny;
    for (int s = 0; s < sweeps; ++s)
        for (int color = 0; color < 2; ++color) {
            for (int v = threadIdx.x; v < V; v += blockDim.x) {
                const int i = v % nx, j = (v / nx) % ny, k = v / sz;
                if (((i + j + k) & 1) != color) continue;
                float nb = 0.0f, diag = -6.0f;
                if (i > 0) nb += su[v - 1]; else diag += 1.0f;
                if (i < nx - 1) nb += su[v + 1];
                if (j > 0) nb += su[v - sy]; else diag += 1.0f;
                if (j < ny - 1) nb += su[v + sy];
                if (k > 0) nb += su[v - sz]; else diag += 1.0f;
                if (k < nz - 1) nb += su[v + sz];
                su[v] = (sf[v] - nb) / diag;
            }
            __syncthreads();
        }
    for (int v = threadIdx.x; v < V; v += blockDim.x) u[v] = su[v];
}

__global__ void k_mg_in(const double* __restrict__ r, float* __restrict__ f, long V,
                        const int* __restrict__ conv) {
    if (*conv) return;
    const long v = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v < V) f[v] = (float)r[v];
}

__global__ void k_mg_out(const float* __restrict__ u, double* __restrict__ z, long V,
                         const int* __restrict__ conv) {
    if (*conv) return;
    const long v = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v < V) z[v] = (double)u[v];
}

// ---- FP64 preconditioned conjugate gradients --------------------------------

__device__ double block_reduce(double x, double* sh) {
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if (threadIdx.x % 32 == 0) sh[threadIdx.x / 32] = x;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int q = 0; q < kThreads / 32; ++q) s += sh[q];
    __syncthreads();
    return s;   // thread 0
}

// the sum of the block partials, in the same order in every block
__device__ double partial_total(const double* __restrict__ part, double* sh) {
    double x = 0.0;
    for (int q = threadIdx.x; q < kPartBlocks; q += kThreads) x += part[q];
    __syncthreads();
    const double s = block_reduce(x, sh);
    if (threadIdx.x == 0) sh[kThreads / 32] = s;
    __syncthreads();
    const double t = sh[kThreads / 32];
    __syncthreads();
    return t;
}

// 4th-order Laplacian of p on the stored box, zero on the Dirichlet planes
__device__ __forceinline__ double lap4(const double* g, int i, int j, int k, int nx, int ny,
                                       int nz, double inv_dx2) {
    const double cf[5] = {-1.0 / 12.0, 4.0 / 3.0, -5.0 / 2.0, 4.0 / 3.0, -1.0 / 12.0};
    double ax = 0.0, ay = 0.0, az = 0.0;
#pragma unroll
    for (int q = -2; q <= 2; ++q) {
        const int ii = i + q < 0 ? -(i + q) - 1 : i + q;
        const int jj = j + q < 0 ? -(j + q) - 1 : j + q;
        const int kk = k + q < 0 ? -(k + q) - 1 : k + q;
        if (ii < nx) ax = fma(cf[q + 2], g[ii + (long)nx * (j + (long)ny * k)], ax);
        if (jj < ny) ay = fma(cf[q + 2], g[i + (long)nx * (jj + (long)ny * k)], ay);
        if (kk < nz) az = fma(cf[q + 2], g[i + (long)nx * (j + (long)ny * kk)], az);
    }
    return ax * inv_dx2 + ay * inv_dx2 + az * inv_dx2;
}

// |b|^2 over the stored box (b: the source), and the state reset
__global__ void __launch_bounds__(kThreads)
k_pcg_start(const double* __restrict__ src, int nx, int ny, int nz, int mx, int my,
            double* __restrict__ e, double* __restrict__ p, double* __restrict__ part) {
    __shared__ double sh[kThreads / 32 + 1];
    const long V = (long)nx * ny * nz;
    double loc = 0.0;
    for (long v = (long)blockIdx.x * kThreads + threadIdx.x; v < V;
         v += (long)kPartBlocks * kThreads) {
        const int i = (int)(v % nx), j = (int)((v / nx) % ny), k = (int)(v / ((long)nx * ny));
        const double s = src[i + mx * (j + (long)my * k)];
        loc = fma(s, s, loc);
        e[v] = 0.0;
        p[v] = 0.0;
    }
    const double s = block_reduce(loc, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
}

__global__ void __launch_bounds__(kThreads)
k_pcg_init_scalars(const double* __restrict__ part, PcgScalars* __restrict__ S) {
    __shared__ double sh[kThreads / 32 + 1];
    const double bb = partial_total(part, sh);
    if (threadIdx.x == 0) {
        S->conv = bb == 0.0 ? 1 : 0;
        S->iters = 0;
        S->bb = bb;
        S->rz_old = 1.0;
        S->rr = 0.0;
    }
}

__global__ void __launch_bounds__(kThreads)
k_pcg_dot(const double* __restrict__ a, const double* __restrict__ b, long V,
          double* __restrict__ part, const int* __restrict__ conv) {
    if (*conv) return;
    __shared__ double sh[kThreads / 32 + 1];
    double loc = 0.0;
    for (long v = (long)blockIdx.x * kThreads + threadIdx.x; v < V;
         v += (long)kPartBlocks * kThreads)
        loc = fma(a[v], b[v], loc);
    const double s = block_reduce(loc, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// p = z + beta p, beta = rz / rz_old (0 on the first iteration)
__global__ void __launch_bounds__(kThreads)
k_pcg_dir(const double* __restrict__ z, double* __restrict__ p, long V,
          const double* __restrict__ part_rz, const PcgScalars* __restrict__ S) {
    if (S->conv) return;
    __shared__ double sh[kThreads / 32 + 1];
    const double rz = partial_total(part_rz, sh);
    const double beta = S->iters == 0 ? 0.0 : rz / S->rz_old;
    for (long v = (long)blockIdx.x * kThreads + threadIdx.x; v < V;
         v += (long)gridDim.x * kThreads)
        p[v] = fma(beta, p[v], z[v]);
}

// q = L p and the partials of p.q
__global__ void __launch_bounds__(kThreads)
k_pcg_matvec(const double* __restrict__ p, double* __restrict__ q, int nx, int ny, int nz,
             double inv_dx2, double* __restrict__ part, const int* __restrict__ conv) {
    if (*conv) return;
    __shared__ double sh[kThreads / 32 + 1];
    const long V = (long)nx * ny * nz;
    double loc = 0.0;
    for (long v = (long)blockIdx.x * kThreads + threadIdx.x; v < V;
         v += (long)kPartBlocks * kThreads) {
        const int i = (int)(v % nx), j = (int)((v / nx) % ny), k = (int)(v / ((long)nx * ny));
        const double x = lap4(p, i, j, k, nx, ny, nz, inv_dx2);
        q[v] = x;
        loc = fma(p[v], x, loc);
    }
    const double s = block_reduce(loc, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// alpha = rz / pq; e += alpha p; r -= alpha q; partials of r.r
__global__ void __launch_bounds__(kThreads)
k_pcg_update(double* __restrict__ e, double* __restrict__ r, const double* __restrict__ p,
             const double* __restrict__ q, long V, const double* __restrict__ part_rz,
             const double* __restrict__ part_pq, double* __restrict__ part_rr,
             const int* __restrict__ conv) {
    if (*conv) return;
    __shared__ double sh[kThreads / 32 + 1];
    const double rz = partial_total(part_rz, sh);
    const double pq = partial_total(part_pq, sh);
    const double alpha = rz / pq;
    double loc = 0.0;
    for (long v = (long)blockIdx.x * kThreads + threadIdx.x; v < V;
         v += (long)kPartBlocks * kThreads) {
        e[v] = fma(alpha, p[v], e[v]);
        const double x = fma(-alpha, q[v], r[v]);
        r[v] = x;
        loc = fma(x, x, loc);
    }
    const double s = block_reduce(loc, sh);
    if (threadIdx.x == 0) part_rr[blockIdx.x] = s;
}

__global__ void __launch_bounds__(kThreads)
k_pcg_check(const double* __restrict__ part_rz, const double* __restrict__ part_rr, double tol2,
            int maxit, PcgScalars* __restrict__ S) {
    if (S->conv) return;
    __shared__ double sh[kThreads / 32 + 1];
    const double rz = partial_total(part_rz, sh);
    const double rr = partial_total(part_rr, sh);
    if (threadIdx.x == 0) {
        S->rz_old = rz;
        S->rr = rr;
        S->iters += 1;
        if (rr <= tol2 * S->bb) S->conv = 1;
        else if (S->iters >= maxit) S->conv = 2;
    }
}

__global__ void k_pcg_finish(double* __restrict__ sol, const double* __restrict__ e, int nx,
                             int ny, int nz, int mx, int my) {
    const long V = (long)nx * ny * nz;
    const long v = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= V) return;
    const int i = (int)(v % nx), j = (int)((v / nx) % ny), k = (int)(v / ((long)nx * ny));
    sol[i + mx * (j + (long)my * k)] += e[v];
}

// r = src - L sol on the stored box, with sol's Dirichlet planes
__global__ void k_pcg_residual(const double* __restrict__ sol, const double* __restrict__ src,
                               double* __restrict__ r, int nx, int ny, int nz, int mx, int my,
                               double inv_dx2) {
    const long V = (long)nx * ny * nz;
    const long v = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= V) return;
    const int i = (int)(v % nx), j = (int)((v / nx) % ny), k = (int)(v / ((long)nx * ny));
    const double cf[5] = {-1.0 / 12.0, 4.0 / 3.0, -5.0 / 2.0, 4.0 / 3.0, -1.0 / 12.0};
    double ax = 0.0, ay = 0.0, az = 0.0;
#pragma unroll
    for (int q = -2; q <= 2; ++q) {
        const int ii = i + q < 0 ? -(i + q) - 1 : i + q;
        const int jj = j + q < 0 ? -(j + q) - 1 : j + q;
        const int kk = k + q < 0 ? -(k + q) - 1 : k + q;
        ax = fma(cf[q + 2], sol[ii + mx * (j + (long)my * k)], ax);
        ay = fma(cf[q + 2], sol[i + mx * (jj + (long)my * k)], ay);
        az = fma(cf[q + 2], sol[i + mx * (j + (long)my * kk)], az);
    }
    r[v] = src[i + mx * (j + (long)my * k)] - (ax * inv_dx2 + ay * inv_dx2 + az * inv_dx2);
}

}  // namespace

// Multigrid hierarchy and FP64 work vectors of one context.
struct Multigrid {
    int nlev = 0;
    Level lev[kMaxLevels];
    int coarse_sweeps = 0;
    float* f32 = nullptr;               // every level's u, f, r
    double *r = nullptr, *z = nullptr, *p = nullptr, *q = nullptr, *e = nullptr;
    double* part = nullptr;             // 4 x kPartBlocks partials
    PcgScalars* S = nullptr;
    PcgScalars* h_S = nullptr;          // pinned
    cudaGraphExec_t chunk = nullptr;    // kChunk iterations, captured on first use
    double tol2 = 0.0;                  // ... for this tolerance and cap
    int maxit = 0;
    long long chunk_launches = 0;
    bool no_graph = false;
};

void multigrid_free(Multigrid* M) {
    if (!M) return;
    for (void* p : {(void*)M->f32, (void*)M->r, (void*)M->z, (void*)M->p, (void*)M->q, (void*)M->e,
                    (void*)M->part, (void*)M->S})
        if (p) cudaFree(p);
    if (M->h_S) cudaFreeHost(M->h_S);
    if (M->chunk) cudaGraphExecDestroy(M->chunk);
    delete M;
}

static int multigrid_setup(mg_ctx* c) {
    Multigrid* M = new Multigrid();
    c->mgrid = M;
    int n[3] = {c->nx, c->ny, c->nz};
    double h = c->p.dx;
    long total = 0;
    while (M->nlev < kMaxLevels) {
        Level& L = M->lev[M->nlev++];
        for (int a = 0; a < 3; ++a) L.n[a] = n[a];
        L.V = (long)n[0] * n[1] * n[2];
        L.inv_h2 = (float)(1.0 / (h * h));
        total += 3 * L.V;
        const bool even = n[0] % 2 == 0 && n[1] % 2 == 0 && n[2] % 2 == 0;
        const bool room = n[0] / 2 >= 3 && n[1] / 2 >= 3 && n[2] / 2 >= 3;
        if (!(even && room)) break;
        for (int a = 0; a < 3; ++a) n[a] /= 2;
        h *= 2.0;
    }
    // the last level is solved in shared memory
    if (M->lev[M->nlev - 1].V > kCoarseMax) return MG_ERR_ARG;
    const Level& C = M->lev[M->nlev - 1];
    const int nm = std::max(C.n[0], std::max(C.n[1], C.n[2]));
    M->coarse_sweeps = std::min(200, 2 * nm * nm);
    MG_CUDA(cudaMalloc(&M->f32, total * sizeof(float)));
    float* q = M->f32;
    for (int l = 0; l < M->nlev; ++l) {
        Level& L = M->lev[l];
        L.u = q; q += L.V;
        L.f = q; q += L.V;
        L.r = q; q += L.V;
    }
    const long V = c->V;
    for (double** b : {&M->r, &M->z, &M->p, &M->q, &M->e})
        MG_CUDA(cudaMalloc(b, V * sizeof(double)));
    MG_CUDA(cudaMalloc(&M->part, 4 * kPartBlocks * sizeof(double)));
    MG_CUDA(cudaMalloc(&M->S, sizeof(PcgScalars)));
    MG_CUDA(cudaMallocHost(&M->h_S, sizeof(PcgScalars)));
    return MG_OK;
}

// One V-cycle: z = M^{-1} r (FP32 inside).
static int vcycle(mg_ctx* c, Multigrid* M, const int* conv) {
    const Level& L0 = M->lev[0];
    k_mg_in<<<div_up(L0.V, kThreads), kThreads, 0, c->stream>>>(M->r, L0.f, L0.V, conv);
    MG_LAUNCHED(c);
    for (int l = 0; l + 1 < M->nlev; ++l) {
        const Level& L = M->lev[l];
        const Level& Cl = M->lev[l + 1];
        const int g = div_up(L.V, kThreads);
        MG_CUDA(cudaMemsetAsync(L.u, 0, L.V * sizeof(float), c->stream));
        for (int color = 0; color < 2; ++color) {
            k_mg_smooth<<<g, kThreads, 0, c->stream>>>(L.u, L.f, L.n[0], L.n[1], L.n[2], L.inv_h2,
                                                       color, conv);
            MG_LAUNCHED(c);
        }
        k_mg_residual<<<g, kThreads, 0, c->stream>>>(L.u, L.f, L.r, L.n[0], L.n[1], L.n[2],
                                                     L.inv_h2, conv);
        MG_LAUNCHED(c);
        k_mg_restrict<<<div_up(Cl.V, kThreads), kThreads, 0, c->stream>>>(
            L.r, Cl.f, L.n[0], L.n[1], L.n[2], Cl.n[0], Cl.n[1], Cl.n[2], conv);
        MG_LAUNCHED(c);
    }
    const Level& C = M->lev[M->nlev - 1];
    k_mg_coarsest<<<1, 1024, 0, c->stream>>>(C.u, C.f, C.n[0], C.n[1], C.n[2], C.inv_h2,
                                             M->coarse_sweeps, conv);
    MG_LAUNCHED(c);
    for (int l = M->nlev - 2; l >= 0; --l) {
        const Level& L = M->lev[l];
        const Level& Cl = M->lev[l + 1];
        const int g = div_up(L.V, kThreads);
        k_mg_prolong<<<g, kThreads, 0, c->stream>>>(L.u, Cl.u, L.n[0], L.n[1], L.n[2], Cl.n[0],
                                                    Cl.n[1], Cl.n[2], conv);
        MG_LAUNCHED(c);
        for (int color = 1; color >= 0; --color) {
            k_mg_smooth<<<g, kThreads, 0, c->stream>>>(L.u, L.f, L.n[0], L.n[1], L.n[2], L.inv_h2,
                                                       color, conv);
            MG_LAUNCHED(c);
        }
    }
    k_mg_out<<<div_up(L0.V, kThreads), kThreads, 0, c->stream>>>(L0.u, M->z, L0.V, conv);
    MG_LAUNCHED(c);
    return MG_OK;
}

// Solve L phi = src on the stored box (cpot holds the start and the
// Dirichlet planes) to |r| <= tol |src|; *iters: PCG iterations.
// Returns MG_NOT_CONVERGED when maxit iterations did not reach tol.
int coulomb_multigrid(mg_ctx* c, double tol, int maxit, int* iters) {
    if (!c->mgrid) MG_TRY(multigrid_setup(c));
    Multigrid* M = c->mgrid;
    const int nx = c->nx, ny = c->ny, nz = c->nz;
    const long V = c->V;
    const double inv_dx2 = 1.0 / (c->p.dx * c->p.dx);
    double *p_rz = M->part, *p_pq = M->part + kPartBlocks, *p_rr = M->part + 2 * kPartBlocks;
    const int* conv = &M->S->conv;
    k_pcg_start<<<kPartBlocks, kThreads, 0, c->stream>>>(c->csource, nx, ny, nz, c->mx, c->my,
                                                          M->e, M->p, M->part);
    MG_LAUNCHED(c);
    k_pcg_init_scalars<<<1, kThreads, 0, c->stream>>>(M->part, M->S);
    MG_LAUNCHED(c);
    k_pcg_residual<<<div_up(V, kThreads), kThreads, 0, c->stream>>>(c->cpot, c->csource, M->r, nx,
                                                                     ny, nz, c->mx, c->my, inv_dx2);
    MG_LAUNCHED(c);
    const double tol2 = tol * tol;
    auto iterations = [&](int count) -> int {
        for (int s = 0; s < count; ++s) {
            MG_TRY(vcycle(c, M, conv));
            k_pcg_dot<<<kPartBlocks, kThreads, 0, c->stream>>>(M->r, M->z, V, p_rz, conv);
            MG_LAUNCHED(c);
            k_pcg_dir<<<div_up(V, kThreads), kThreads, 0, c->stream>>>(M->z, M->p, V, p_rz, M->S);
            MG_LAUNCHED(c);
            k_pcg_matvec<<<kPartBlocks, kThreads, 0, c->stream>>>(M->p, M->q, nx, ny, nz, inv_dx2,
                                                                  p_pq, conv);
            MG_LAUNCHED(c);
            k_pcg_update<<<kPartBlocks, kThreads, 0, c->stream>>>(M->e, M->r, M->p, M->q, V, p_rz,
                                                                  p_pq, p_rr, conv);
            MG_LAUNCHED(c);
            k_pcg_check<<<1, kThreads, 0, c->stream>>>(p_rz, p_rr, tol2, maxit, M->S);
            MG_LAUNCHED(c);
        }
        return MG_OK;
    };
    // the launches of kChunk iterations (about 40 per iteration, small ones on
    // the coarse levels) replay as one CUDA graph; tol and maxit are baked
    // into it, so it is rebuilt when they change
    if (M->chunk && (M->tol2 != tol2 || M->maxit != maxit)) {
        cudaGraphExecDestroy(M->chunk);
        M->chunk = nullptr;
    }
    if (!M->chunk && !M->no_graph) {
        if (cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
            cudaGetLastError();   // e.g. the legacy default stream: launch directly
            M->no_graph = true;
        } else {
            const long long l0 = c->launches;
            const int st = iterations(kChunk);
            cudaGraph_t graph = nullptr;
            const cudaError_t ce = cudaStreamEndCapture(c->stream, &graph);
            if (st != MG_OK || ce != cudaSuccess) {
                if (graph) cudaGraphDestroy(graph);
                return st != MG_OK ? st : MG_ERR_CUDA;
            }
            const cudaError_t ie = cudaGraphInstantiate(&M->chunk, graph, 0);
            cudaGraphDestroy(graph);
            if (ie != cudaSuccess) {
                M->chunk = nullptr;
                return MG_ERR_CUDA;
            }
            M->chunk_launches = c->launches - l0;
            c->launches = l0;
            M->tol2 = tol2;
            M->maxit = maxit;
        }
    }
    int done = 0;
    while (done < maxit) {
        const int chunk = std::min(kChunk, maxit - done);
        if (M->chunk && chunk == kChunk) {
            MG_CUDA(cudaGraphLaunch(M->chunk, c->stream));
            c->launches += M->chunk_launches;
        } else {
            MG_TRY(iterations(chunk));
        }
        done += chunk;
        MG_CUDA(cudaMemcpyAsync(M->h_S, M->S, sizeof(PcgScalars), cudaMemcpyDeviceToHost,
                                c->stream));
        MG_CUDA(cudaStreamSynchronize(c->stream));
        if (M->h_S->conv) break;
    }
    k_pcg_finish<<<div_up(V, kThreads), kThreads, 0, c->stream>>>(c->cpot, M->e, nx, ny, nz, c->mx,
                                                                  c->my);
    MG_LAUNCHED(c);
    if (iters) *iters = M->h_S->iters;
    return M->h_S->conv == 1 ? MG_OK : MG_NOT_CONVERGED;
}

int multigrid_levels(const mg_ctx* c) { return c->mgrid ? c->mgrid->nlev : 0; }

}  // namespace mg
