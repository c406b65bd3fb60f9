// coulomb.cu -- Coulomb Poisson solve on the symmetry-reduced box, FP64.
//
// Replaces SolveCoulomb with CoulombSolver = 1 (src/Coulomb.f90:255-346):
//   CoulombBound (:583-674): source -4 pi e2 rho_p on the stored box and
//     Dirichlet values sum_lm e2 4pi/(2l+1) Q_lm r^l Y_lm / r^(2l+1) on the
//     BCNumber = 2 extra planes of the extended box;
//   ConjugGrad (:755-900) with CoulombLaplacian (5-point FD, even mirror at
//     the low end of each axis, src/CoulombDerivatives.f90:144-281);
//   Slater exchange -(3/pi)^(1/3) e2 rho_p^(1/3) (:338-344).
// The CG runs as ONE cooperative kernel: every block owns a slice of the
// extended box, the two dot products per iteration are block partials summed
// by every block in the same order (so every block takes the same branch),
// and blocks meet at a sense-reversing grid barrier whose spin is bounded:
// a barrier that waits longer than its cap sets the timeout status and the
// kernel returns instead of hanging.
#include <cmath>

#include "mg_internal.cuh"

namespace mg {

namespace {

constexpr int kThreads = 256;
constexpr long long kSpinCap = 1ll << 22;  // ~0.2 s of 50 ns sleeps per barrier

struct CgArgs {
    double* sol;
    double* res;
    double* p;
    double* t;
    const double* src;
    double* red;          // 2 * gridDim.x
    unsigned* bar;        // [0] arrival count, [1] generation
    int* status;          // [0] state, [1] iterations
    int nx, ny, nz, mx, my, mz;
    double inv_dx2;
    double prec;
    double rel;           // > 0: stop at |r| <= rel |src| instead of |r|^2 <= prec
    int maxit;
};

__device__ bool grid_barrier(unsigned* bar, int* status) {
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned* gen = bar + 1;
        const unsigned g = *gen;
        __threadfence();
        const unsigned arrived = atomicAdd(bar, 1u) + 1u;
        if (arrived == gridDim.x) {
            atomicExch(bar, 0u);
            __threadfence();
            atomicAdd(bar + 1, 1u);
        } else {
            long long spins = 0;
            while (*gen == g) {
                if (++spins > kSpinCap) {
                    atomicExch(status, 2);
                    break;
                }
                __nanosleep(50);
            }
        }
        __threadfence();
    }
    __syncthreads();
    return *(volatile int*)status != 2;
}

__device__ __forceinline__ double lap_at(const double* g, int i, int j, int k, int mx, int my,
                                         double inv_dx2) {
    const double cf[5] = {-1.0 / 12.0, 4.0 / 3.0, -5.0 / 2.0, 4.0 / 3.0, -1.0 / 12.0};
    double ax = 0.0, ay = 0.0, az = 0.0;
#pragma unroll
    for (int q = -2; q <= 2; ++q) {
        const int ii = i + q < 0 ? -(i + q) - 1 : i + q;
        const int jj = j + q < 0 ? -(j + q) - 1 : j + q;
        const int kk = k + q < 0 ? -(k + q) - 1 : k + q;
        ax = fma(cf[q + 2], g[ii + mx * (j + (long)my * k)], ax);
        ay = fma(cf[q + 2], g[i + mx * (jj + (long)my * k)], ay);
        az = fma(cf[q + 2], g[i + mx * (j + (long)my * kk)], az);
    }
    return ax * inv_dx2 + ay * inv_dx2 + az * inv_dx2;
}

__device__ double block_sum(double x, double* sh) {
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if (threadIdx.x % 32 == 0) sh[threadIdx.x / 32] = x;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int q = 0; q < kThreads / 32; ++q) s += sh[q];
    __syncthreads();
    return s;  // valid in thread 0
}

__device__ double grid_total(const double* red, double* bc) {
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (unsigned q = 0; q < gridDim.x; ++q) s += ((volatile const double*)red)[q];
        *bc = s;
    }
    __syncthreads();
    const double v = *bc;
    __syncthreads();
    return v;
}

__global__ void __launch_bounds__(kThreads) k_cg(CgArgs a) {
    __shared__ double sh[kThreads / 32];
    __shared__ double bcast;
    const long M = (long)a.mx * a.my * a.mz;
    const long stride = (long)gridDim.x * kThreads;
    const long t0 = (long)blockIdx.x * kThreads + threadIdx.x;
    double* red1 = a.red;
    double* red2 = a.red + gridDim.x;

    // r0 = src - Lap(sol); p0 = r0; pnorm = r0.r0
    double loc = 0.0;
    for (long o = t0; o < M; o += stride) {
        const int i = (int)(o % a.mx), j = (int)((o / a.mx) % a.my), k = (int)(o / ((long)a.mx * a.my));
        double lap = 0.0;
        if (i < a.nx && j < a.ny && k < a.nz) lap = lap_at(a.sol, i, j, k, a.mx, a.my, a.inv_dx2);
        const double r = -lap + a.src[o];
        a.res[o] = r;
        a.p[o] = r;
        loc = fma(r, r, loc);
    }
    double s = block_sum(loc, sh);
    if (threadIdx.x == 0) red2[blockIdx.x] = s;
    double prec = a.prec;
    if (a.rel > 0.0) {
        // |src|^2 over the stored box for the relative test
        loc = 0.0;
        for (long o = t0; o < M; o += stride) {
            const int i = (int)(o % a.mx), j = (int)((o / a.mx) % a.my);
            const int k = (int)(o / ((long)a.mx * a.my));
            if (i < a.nx && j < a.ny && k < a.nz) loc = fma(a.src[o], a.src[o], loc);
        }
        s = block_sum(loc, sh);
        if (threadIdx.x == 0) red1[blockIdx.x] = s;
    }
    if (!grid_barrier(a.bar, a.status)) return;
    double pnorm = grid_total(red2, &bcast);
    if (a.rel > 0.0) {
        prec = a.rel * a.rel * grid_total(red1, &bcast);
        // every block has read red1 before the first iteration rewrites it
        if (!grid_barrier(a.bar, a.status)) return;
    }
    int it;
    for (it = 1; it <= a.maxit; ++it) {
        // t = Lap(p), integral = r.t
        loc = 0.0;
        for (long o = t0; o < M; o += stride) {
            const int i = (int)(o % a.mx), j = (int)((o / a.mx) % a.my), k = (int)(o / ((long)a.mx * a.my));
            double lap = 0.0;
            if (i < a.nx && j < a.ny && k < a.nz) lap = lap_at(a.p, i, j, k, a.mx, a.my, a.inv_dx2);
            a.t[o] = lap;
            loc = fma(a.res[o], lap, loc);
        }
        s = block_sum(loc, sh);
        if (threadIdx.x == 0) red1[blockIdx.x] = s;
        if (!grid_barrier(a.bar, a.status)) return;
        const double integral = grid_total(red1, &bcast);
        const double ak = pnorm / integral;
        loc = 0.0;
        for (long o = t0; o < M; o += stride) {
            a.sol[o] = fma(ak, a.p[o], a.sol[o]);
            const double r = fma(-ak, a.t[o], a.res[o]);
            a.res[o] = r;
            loc = fma(r, r, loc);
        }
        s = block_sum(loc, sh);
        if (threadIdx.x == 0) red2[blockIdx.x] = s;
        if (!grid_barrier(a.bar, a.status)) return;
        const double nn = grid_total(red2, &bcast);
        if (nn <= prec) break;
        const double ck = nn / pnorm;
        pnorm = nn;
        for (long o = t0; o < M; o += stride) a.p[o] = fma(ck, a.p[o], a.res[o]);
        if (!grid_barrier(a.bar, a.status)) return;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        a.status[1] = it > a.maxit ? a.maxit : it;
        if (it > a.maxit && a.status[0] == 0) a.status[0] = 1;
    }
}

// Source and multipole Dirichlet values on the extended box.
__global__ void k_coulomb_bound(const double* __restrict__ rho_p, const double* __restrict__ sh,
                                const double* __restrict__ rpow, const double* __restrict__ mval,
                                const double* __restrict__ mfac, int nmom, int nx, int ny, int nz,
                                int mx, int my, int mz, double e2, double* __restrict__ src,
                                double* __restrict__ sol) {
    const long M = (long)mx * my * mz;
    const long o = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= M) return;
    const int i = (int)(o % mx), j = (int)((o / mx) % my), k = (int)(o / ((long)mx * my));
    const double pi = 4.0 * atan2(1.0, 1.0);
    if (i < nx && j < ny && k < nz) {
        src[o] = -4 * pi * e2 * rho_p[i + nx * (j + (long)ny * k)];
        return;
    }
    src[o] = 0.0;
    double bc = 0.0;
    for (int m = 0; m < nmom; ++m) {
        const double value = mval[2 * m + 1] * mfac[m];
        bc = bc + value * sh[(long)m * M + o] * e2 / rpow[(long)m * M + o];
    }
    if (bc != 0.0) sol[o] = bc;
}

__global__ void k_coulomb_out(const double* __restrict__ sol, const double* __restrict__ rho_p,
                              int nx, int ny, int nz, int mx, int my, double fac,
                              double* __restrict__ coul, double* __restrict__ coulex) {
    const long V = (long)nx * ny * nz;
    const long v = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= V) return;
    const int i = (int)(v % nx), j = (int)((v / nx) % ny), k = (int)(v / ((long)nx * ny));
    coul[v] = sol[i + mx * (j + (long)my * k)];
    coulex[v] = fac * pow(rho_p[v], 1 / 3.0);
}

// ---- direct separable solve (mixed form) ---------------------------------------
//
// The CG operator is the 4th-order difference Laplacian on the stored box
// with a mirror at each symmetry plane and the two Dirichlet planes of the
// extended box moved to the right-hand side: a Kronecker sum
// L = (L_x + L_y + L_z) / dx^2 of three 1-D symmetric operators.  With the
// 1-D eigendecompositions L_a = C_a diag(mu_a) C_a^T (computed once on the
// host), L^{-1} r = (C_x C_y C_z) diag(dx^2 / (mu_x + mu_y + mu_z))
// (C_x C_y C_z)^T r: six small contractions along the axes and one scaling
// instead of ~140 CG iterations with four grid barriers each.  Two rounds of
// FP64 iterative refinement (residual with the full stencil, correction
// from the direct solve) leave a residual at FP64 rounding.

__global__ void k_cfast_residual(const double* __restrict__ sol, const double* __restrict__ src,
                                 double* __restrict__ r, int nx, int ny, int nz, int mx, int my,
                                 double inv_dx2) {
    const long V = (long)nx * ny * nz;
    const long v = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= V) return;
    const int i = (int)(v % nx), j = (int)((v / nx) % ny), k = (int)(v / ((long)nx * ny));
    const long o = i + mx * (j + (long)my * k);
    r[v] = src[o] - lap_at(sol, i, j, k, mx, my, inv_dx2);
}

// out = M^T in (fwd) or M in (back) along one axis of an nx x ny x nz grid;
// C is the axis' n x n eigenvector matrix, C[i * n + kk] = component i of
// eigenvector kk.
__global__ void k_cfast_axis(const double* __restrict__ in, double* __restrict__ out,
                             const double* __restrict__ C, int axis, int nx, int ny, int nz,
                             int fwd) {
    const long V = (long)nx * ny * nz;
    const long v = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= V) return;
    const int c3[3] = {(int)(v % nx), (int)((v / nx) % ny), (int)(v / ((long)nx * ny))};
    const int n = axis == 0 ? nx : axis == 1 ? ny : nz;
    const long step = axis == 0 ? 1 : axis == 1 ? nx : (long)nx * ny;
    const int a = c3[axis];
    const long base = v - a * step;
    double s = 0.0;
    for (int q = 0; q < n; ++q) {
        const double m = fwd ? C[q * n + a] : C[a * n + q];
        s = fma(m, in[base + q * step], s);
    }
    out[v] = s;
}

__global__ void k_cfast_scale(double* __restrict__ x, const double* __restrict__ mux,
                              const double* __restrict__ muy, const double* __restrict__ muz,
                              int nx, int ny, int nz, double dx2) {
    const long V = (long)nx * ny * nz;
    const long v = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= V) return;
    const int i = (int)(v % nx), j = (int)((v / nx) % ny), k = (int)(v / ((long)nx * ny));
    x[v] *= dx2 / (mux[i] + muy[j] + muz[k]);
}

__global__ void k_cfast_update(double* __restrict__ sol, const double* __restrict__ e, int nx,
                               int ny, int nz, int mx, int my) {
    const long V = (long)nx * ny * nz;
    const long v = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= V) return;
    const int i = (int)(v % nx), j = (int)((v / nx) % ny), k = (int)(v / ((long)nx * ny));
    sol[i + mx * (j + (long)my * k)] += e[v];
}

// 1-D operator of one axis (mirror at -1/2, Dirichlet planes beyond n-1
// dropped) and its eigendecomposition by cyclic Jacobi in FP64.
void axis_eigen(int n, std::vector<double>& C, std::vector<double>& mu) {
    const double cf[5] = {-1.0 / 12.0, 4.0 / 3.0, -5.0 / 2.0, 4.0 / 3.0, -1.0 / 12.0};
    std::vector<double> A((size_t)n * n, 0.0);
    for (int i = 0; i < n; ++i)
        for (int q = -2; q <= 2; ++q) {
            int m = i + q;
            if (m < 0) m = -m - 1;
            if (m >= n) continue;
            A[(size_t)i * n + m] += cf[q + 2];
        }
    C.assign((size_t)n * n, 0.0);
    for (int i = 0; i < n; ++i) C[(size_t)i * n + i] = 1.0;
    for (int sweep = 0; sweep < 60; ++sweep) {
        double off = 0.0, nrm = 0.0;
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) {
                nrm += A[(size_t)i * n + j] * A[(size_t)i * n + j];
                if (i != j) off += A[(size_t)i * n + j] * A[(size_t)i * n + j];
            }
        if (off <= 1e-30 * nrm) break;
        for (int p = 0; p < n - 1; ++p)
            for (int q = p + 1; q < n; ++q) {
                const double apq = A[(size_t)p * n + q];
                if (std::fabs(apq) < 1e-300) continue;
                const double th = (A[(size_t)q * n + q] - A[(size_t)p * n + p]) / (2.0 * apq);
                const double t = (th >= 0 ? 1.0 : -1.0) / (std::fabs(th) + std::sqrt(th * th + 1.0));
                const double cs = 1.0 / std::sqrt(t * t + 1.0), sn = t * cs;
                for (int k = 0; k < n; ++k) {
                    const double akp = A[(size_t)k * n + p], akq = A[(size_t)k * n + q];
                    A[(size_t)k * n + p] = cs * akp - sn * akq;
                    A[(size_t)k * n + q] = sn * akp + cs * akq;
                }
                for (int k = 0; k < n; ++k) {
                    const double apk = A[(size_t)p * n + k], aqk = A[(size_t)q * n + k];
                    A[(size_t)p * n + k] = cs * apk - sn * aqk;
                    A[(size_t)q * n + k] = sn * apk + cs * aqk;
                }
                for (int k = 0; k < n; ++k) {
                    const double vkp = C[(size_t)k * n + p], vkq = C[(size_t)k * n + q];
                    C[(size_t)k * n + p] = cs * vkp - sn * vkq;
                    C[(size_t)k * n + q] = sn * vkp + cs * vkq;
                }
            }
    }
    mu.resize(n);
    for (int i = 0; i < n; ++i) mu[i] = A[(size_t)i * n + i];
}

}  // namespace

// ---- host-side restatement of the spherical harmonics of the moments -----
// legendre_pnm src/Mesh.f90:96-262; SphericalHarmonics src/Moments.f90:584-691
static void legendre(int n, int m, double x, double* cx) {
    for (int i = 0; i < m; ++i) cx[i] = 0.0;
    cx[m] = 1.0;
    const double somx2 = std::sqrt(1.0 - x * x);
    double fact = 1.0;
    for (int i = 1; i <= m; ++i) { cx[m] = -cx[m] * fact * somx2; fact += 2.0; }
    if (m == n) return;
    cx[m + 1] = x * double(2 * m + 1) * cx[m];
    for (int i = m + 2; i <= n; ++i)
        cx[i] = (double(2 * i - 1) * x * cx[i - 1] - double(i + m - 1) * cx[i - 2]) / double(i - m);
}

static double ipow(double x, int n) {
    double r = 1.0;
    for (int i = 0; i < n; ++i) r *= x;
    return r;
}

double rlylm(int l, int m, int im, double X, double Y, double Z) {
    const double pi = 4.0 * std::atan2(1.0, 1.0);
    const int maxl = 10;
    const double r = std::sqrt(X * X + Y * Y + Z * Z);
    double leg[16];
    legendre(maxl, m, Z / r, leg);
    double fq = 1.0;
    for (int q = 1; q <= 2 * m; ++q) fq = fq / double(l + m - q + 1);
    double fac = ((m % 2) ? -1.0 : 1.0) * std::sqrt(fq) * ipow(r, l);
    fac = fac * std::sqrt(double(2 * l + 1) / (4 * pi));
    const double phi = std::atan2(Y, X);
    return fac * leg[l] * (im ? std::sin(m * phi) : std::cos(m * phi));
}

// Moment table (IniMoments, src/Moments.f90:372-582; EV8 selection of
// NewMoment_Electric), spherical harmonics on the stored and extended
// meshes, the extended-box geometry and the initial guess (SetupCoulomb
// :348-540, InitialGuess :542-581).
int coulomb_setup(mg_ctx* c) {
    const double pi = 4.0 * std::atan2(1.0, 1.0);
    const int maxl = c->p.max_l_coul > 0 ? std::min(c->p.max_l_coul, 10) : 10;
    std::vector<int> L, Mm, Im;
    L.push_back(0); Mm.push_back(0); Im.push_back(0);
    for (int l = 1; l <= 10; ++l)
        for (int m = 0; m <= l; ++m)
            for (int im = 0; im <= 1; ++im) {
                if (c->p.pc && (l % 2)) continue;
                if (c->p.tsc && im == 1) continue;
                if (c->p.sc && (m % 2)) continue;
                if (m == 0 && im == 1) continue;
                L.push_back(l); Mm.push_back(m); Im.push_back(im);
            }
    const int nmom_all = (int)L.size();
    int nmom_bc = 0;
    while (nmom_bc < nmom_all && L[nmom_bc] <= maxl) ++nmom_bc;
    c->n_moments = nmom_all;
    for (int q = 0; q < nmom_all && q < kNumMoments; ++q) c->h_moment_l[q] = L[q];
    const int nx = c->nx, ny = c->ny, nz = c->nz;
    const long V = c->V;
    std::vector<double> sh(nmom_all * V);
    for (int q = 0; q < nmom_all; ++q)
        for (int k = 0; k < nz; ++k)
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nx; ++i) {
                    const double X = c->p.dx / 2.0 + c->p.dx * i, Y = c->p.dx / 2.0 + c->p.dx * j,
                                 Z = c->p.dx / 2.0 + c->p.dx * k;
                    sh[q * V + i + nx * (j + (long)ny * k)] =
                        q == 0 ? 1.0 / std::sqrt(4.0 * pi) : rlylm(L[q], Mm[q], Im[q], X, Y, Z);
                }
    MG_CUDA(cudaMalloc(&c->sh_mesh, sh.size() * sizeof(double)));
    MG_CUDA(cudaMemcpy(c->sh_mesh, sh.data(), sh.size() * sizeof(double), cudaMemcpyHostToDevice));
    MG_CUDA(cudaMalloc(&c->moment_values, 2 * nmom_all * sizeof(double)));
    MG_CUDA(cudaMemset(c->moment_values, 0, 2 * nmom_all * sizeof(double)));

    // extended box: BCNumber = 2 planes beyond the stored box on each axis
    c->mx = nx + 2; c->my = ny + 2; c->mz = nz + 2;
    const long M = (long)c->mx * c->my * c->mz;
    c->M = M;
    std::vector<double> shx(nmom_bc * M), rp(nmom_bc * M), guess(M, 0.0), mfac(nmom_bc);
    for (int q = 0; q < nmom_bc; ++q) mfac[q] = 4 * pi / (2 * L[q] + 1);
    const double R = 1.25 * std::pow(c->p.neutrons + c->p.protons, 1.0 / 3.0);
    const double charge = c->p.protons * c->f.e2, fac = charge / (2 * R);
    for (int k = 0; k < c->mz; ++k)
        for (int j = 0; j < c->my; ++j)
            for (int i = 0; i < c->mx; ++i) {
                const long o = i + c->mx * (j + (long)c->my * k);
                const double X = (0.5 + i) * c->p.dx, Y = (0.5 + j) * c->p.dx, Z = (0.5 + k) * c->p.dx;
                const double r = std::sqrt(X * X + Y * Y + Z * Z);
                for (int q = 0; q < nmom_bc; ++q) {
                    shx[q * M + o] = rlylm(L[q], Mm[q], Im[q], X, Y, Z);
                    rp[q * M + o] = ipow(r, 2 * L[q] + 1);
                }
                if (i < nx && j < ny && k < nz) guess[o] = r <= R ? fac * (3 - r * r / (R * R)) : charge / r;
            }
    c->n_bc_moments = nmom_bc;
    MG_CUDA(cudaMalloc(&c->sh_ext, shx.size() * sizeof(double) + 8));
    MG_CUDA(cudaMalloc(&c->rpow_ext, rp.size() * sizeof(double) + 8));
    MG_CUDA(cudaMalloc(&c->mfac, mfac.size() * sizeof(double) + 8));
    MG_CUDA(cudaMemcpy(c->sh_ext, shx.data(), shx.size() * sizeof(double), cudaMemcpyHostToDevice));
    MG_CUDA(cudaMemcpy(c->rpow_ext, rp.data(), rp.size() * sizeof(double), cudaMemcpyHostToDevice));
    MG_CUDA(cudaMemcpy(c->mfac, mfac.data(), mfac.size() * sizeof(double), cudaMemcpyHostToDevice));
    for (double** b : {&c->cpot, &c->csource, &c->cres, &c->cp, &c->ct})
        MG_CUDA(cudaMalloc(b, M * sizeof(double)));
    MG_CUDA(cudaMemcpy(c->cpot, guess.data(), M * sizeof(double), cudaMemcpyHostToDevice));
    MG_CUDA(cudaMalloc(&c->cguess, M * sizeof(double)));
    MG_CUDA(cudaMemcpy(c->cguess, guess.data(), M * sizeof(double), cudaMemcpyHostToDevice));
    MG_CUDA(cudaMalloc(&c->cg_bar, 4 * sizeof(unsigned)));
    MG_CUDA(cudaMalloc(&c->cg_status, 4 * sizeof(int)));
    int per_sm = 0;
    MG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_cg, kThreads, 0));
    if (per_sm < 1) return MG_ERR_CUDA;
    // The CG runs 4 grid barriers per iteration on a small box (26^3 for a
    // 24^3 mesh): about two mesh points per thread and few blocks make the
    // barriers cheaper than spreading the points over every SM (measured on
    // GB300: 32 blocks beat 152 by ~1.3 ms per solve at 26^3).
    c->cg_blocks = std::max(1, std::min(c->num_sms, std::max(8, div_up(M, 2 * kThreads))));
    // eigendecompositions of the three 1-D operators for the direct solve
    {
        const int ns[3] = {nx, ny, nz};
        std::vector<double> all;
        for (int a = 0; a < 3; ++a) {
            std::vector<double> Ca, mua;
            axis_eigen(ns[a], Ca, mua);
            c->cfast_off[a][0] = (long)all.size();
            all.insert(all.end(), Ca.begin(), Ca.end());
            c->cfast_off[a][1] = (long)all.size();
            all.insert(all.end(), mua.begin(), mua.end());
        }
        MG_CUDA(cudaMalloc(&c->cfast, all.size() * sizeof(double)));
        MG_CUDA(cudaMemcpy(c->cfast, all.data(), all.size() * sizeof(double),
                           cudaMemcpyHostToDevice));
    }
    c->coulomb_init = true;
    return MG_OK;
}

// Sums of r^2 and of the source's square over the stored box (a diagnostic:
// atomics, so the last bits vary between runs).
__global__ void k_residual_norms(const double* __restrict__ r, const double* __restrict__ src,
                                 int nx, int ny, int nz, int mx, int my,
                                 double* __restrict__ out) {
    const long V = (long)nx * ny * nz;
    double a = 0.0, b = 0.0;
    for (long v = (long)blockIdx.x * blockDim.x + threadIdx.x; v < V;
         v += (long)gridDim.x * blockDim.x) {
        const int i = (int)(v % nx), j = (int)((v / nx) % ny), k = (int)(v / ((long)nx * ny));
        const double s = src[i + mx * (j + (long)my * k)];
        a = fma(r[v], r[v], a);
        b = fma(s, s, b);
    }
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, o);
        b += __shfl_xor_sync(0xffffffffu, b, o);
    }
    if (threadIdx.x % 32 == 0) {
        atomicAdd(out, a);
        atomicAdd(out + 1, b);
    }
}

// Mixed form: two rounds of (FP64 residual, direct separable correction).
static int coulomb_direct_launches(mg_ctx* c) {
    const int nx = c->nx, ny = c->ny, nz = c->nz;
    const long V = c->V;
    const int g = div_up(V, kThreads);
    const double dx2 = c->p.dx * c->p.dx;
    double *r = c->cres, *t1 = c->cp, *t2 = c->ct;   // CG buffers, unused here
    const double* C[3] = {c->cfast + c->cfast_off[0][0], c->cfast + c->cfast_off[1][0],
                          c->cfast + c->cfast_off[2][0]};
    const double* mu[3] = {c->cfast + c->cfast_off[0][1], c->cfast + c->cfast_off[1][1],
                           c->cfast + c->cfast_off[2][1]};
    for (int round = 0; round < 2; ++round) {
        k_cfast_residual<<<g, kThreads, 0, c->stream>>>(c->cpot, c->csource, r, nx, ny, nz, c->mx,
                                                        c->my, 1.0 / dx2);
        MG_LAUNCHED(c);
        k_cfast_axis<<<g, kThreads, 0, c->stream>>>(r, t1, C[0], 0, nx, ny, nz, 1);
        MG_LAUNCHED(c);
        k_cfast_axis<<<g, kThreads, 0, c->stream>>>(t1, t2, C[1], 1, nx, ny, nz, 1);
        MG_LAUNCHED(c);
        k_cfast_axis<<<g, kThreads, 0, c->stream>>>(t2, t1, C[2], 2, nx, ny, nz, 1);
        MG_LAUNCHED(c);
        k_cfast_scale<<<g, kThreads, 0, c->stream>>>(t1, mu[0], mu[1], mu[2], nx, ny, nz, dx2);
        MG_LAUNCHED(c);
        k_cfast_axis<<<g, kThreads, 0, c->stream>>>(t1, t2, C[2], 2, nx, ny, nz, 0);
        MG_LAUNCHED(c);
        k_cfast_axis<<<g, kThreads, 0, c->stream>>>(t2, t1, C[1], 1, nx, ny, nz, 0);
        MG_LAUNCHED(c);
        k_cfast_axis<<<g, kThreads, 0, c->stream>>>(t1, t2, C[0], 0, nx, ny, nz, 0);
        MG_LAUNCHED(c);
        k_cfast_update<<<g, kThreads, 0, c->stream>>>(c->cpot, t2, nx, ny, nz, c->mx, c->my);
        MG_LAUNCHED(c);
    }
    return MG_OK;
}

// The eighteen launches of the two rounds replay as one CUDA graph (fixed
// buffers per context): a few microseconds each, they would otherwise run at
// the host's enqueue rate.
static int coulomb_direct(mg_ctx* c) {
    if (c->cfast_no_graph) return coulomb_direct_launches(c);
    if (!c->cfast_graph) {
        if (cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
            cudaGetLastError();
            c->cfast_no_graph = true;
            return coulomb_direct_launches(c);
        }
        const long long l0 = c->launches;
        const int st = coulomb_direct_launches(c);
        cudaGraph_t graph = nullptr;
        const cudaError_t ce = cudaStreamEndCapture(c->stream, &graph);
        if (st != MG_OK || ce != cudaSuccess) {
            if (graph) cudaGraphDestroy(graph);
            return st != MG_OK ? st : MG_ERR_CUDA;
        }
        const cudaError_t ie = cudaGraphInstantiate(&c->cfast_graph, graph, 0);
        cudaGraphDestroy(graph);
        if (ie != cudaSuccess) {
            c->cfast_graph = nullptr;
            return MG_ERR_CUDA;
        }
        c->cfast_graph_launches = c->launches - l0;
        c->launches = l0;
    }
    MG_CUDA(cudaGraphLaunch(c->cfast_graph, c->stream));
    c->launches += c->cfast_graph_launches;
    return MG_OK;
}

// |b - L phi| / |b| of the current Coulomb potential on the stored box, with
// the solver's own Laplacian (CoulombLaplacian with the boundary planes).
int coulomb_residual(mg_ctx* c, double* rel) {
    if (!c->coulomb_init) return MG_ERR_STATE;
    const long V = c->V;
    const double dx2 = c->p.dx * c->p.dx;
    k_cfast_residual<<<div_up(V, kThreads), kThreads, 0, c->stream>>>(
        c->cpot, c->csource, c->cres, c->nx, c->ny, c->nz, c->mx, c->my, 1.0 / dx2);
    MG_LAUNCHED(c);
    MG_CUDA(cudaMemsetAsync(c->red, 0, 2 * sizeof(double), c->stream));
    k_residual_norms<<<std::min(div_up(V, kThreads), 4 * c->num_sms), kThreads, 0, c->stream>>>(
        c->cres, c->csource, c->nx, c->ny, c->nz, c->mx, c->my, c->red);
    MG_LAUNCHED(c);
    double h[2];
    MG_CUDA(cudaMemcpyAsync(h, c->red, 2 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    MG_CUDA(cudaStreamSynchronize(c->stream));
    *rel = h[1] > 0.0 ? std::sqrt(h[0] / h[1]) : std::sqrt(h[0]);
    return MG_OK;
}

// The potential back to InitialGuess (the start of a cold solve).
int coulomb_reset(mg_ctx* c) {
    if (!c->coulomb_init) MG_TRY(coulomb_setup(c));
    MG_CUDA(cudaMemcpyAsync(c->cpot, c->cguess, c->M * sizeof(double), cudaMemcpyDeviceToDevice,
                            c->stream));
    return MG_OK;
}

int coulomb_solve(mg_ctx* c, int* iters) {
    if (!c->coulomb_init) MG_TRY(coulomb_setup(c));
    const long M = c->M;
    k_coulomb_bound<<<div_up(M, kThreads), kThreads, 0, c->stream>>>(
        c->rho + c->V, c->sh_ext, c->rpow_ext, c->moment_values, c->mfac, c->n_bc_moments, c->nx,
        c->ny, c->nz, c->mx, c->my, c->mz, c->f.e2, c->csource, c->cpot);
    MG_LAUNCHED(c);
    if (c->p.coulomb_solver == 2) {
        const double pi_ = 4.0 * std::atan2(1.0, 1.0);
        const int maxit = c->p.coulomb_max > 0 ? c->p.coulomb_max : 500;
        const int st = coulomb_multigrid(c, c->p.coulomb_prec > 0 ? c->p.coulomb_prec : 1e-10,
                                         maxit, iters);
        if (st < 0) return st;
        k_coulomb_out<<<div_up(c->V, kThreads), kThreads, 0, c->stream>>>(
            c->cpot, c->rho + c->V, c->nx, c->ny, c->nz, c->mx, c->my,
            -std::pow(3 / pi_, 1 / 3.0) * c->f.e2, c->coulomb, c->coulex);
        MG_LAUNCHED(c);
        return st;
    }
    if (c->cur_precision == MG_MIXED) {
        MG_TRY(coulomb_direct(c));
        const double pi = 4.0 * std::atan2(1.0, 1.0);
        const double fac = -std::pow(3 / pi, 1 / 3.0) * c->f.e2;
        k_coulomb_out<<<div_up(c->V, kThreads), kThreads, 0, c->stream>>>(
            c->cpot, c->rho + c->V, c->nx, c->ny, c->nz, c->mx, c->my, fac, c->coulomb,
            c->coulex);
        MG_LAUNCHED(c);
        if (iters) *iters = 2;
        return MG_OK;
    }
    MG_CUDA(cudaMemsetAsync(c->cg_bar, 0, 4 * sizeof(unsigned), c->stream));
    MG_CUDA(cudaMemsetAsync(c->cg_status, 0, 4 * sizeof(int), c->stream));
    CgArgs a;
    a.sol = c->cpot; a.res = c->cres; a.p = c->cp; a.t = c->ct; a.src = c->csource;
    a.red = c->red; a.bar = c->cg_bar; a.status = c->cg_status;
    a.nx = c->nx; a.ny = c->ny; a.nz = c->nz; a.mx = c->mx; a.my = c->my; a.mz = c->mz;
    a.inv_dx2 = 1.0 / (c->p.dx * c->p.dx);
    a.prec = 1.0e-9 / (c->p.dx * c->p.dx * c->p.dx * c->nx * c->ny * c->nz);
    a.rel = c->p.coulomb_prec > 0 ? c->p.coulomb_prec : 0.0;
    a.maxit = c->p.coulomb_max > 0 ? c->p.coulomb_max : 500;
    void* args[] = {&a};
    MG_CUDA(cudaLaunchCooperativeKernel((const void*)k_cg, dim3(c->cg_blocks), dim3(kThreads), args,
                                        0, c->stream));
    ++c->launches;
    const double pi = 4.0 * std::atan2(1.0, 1.0);
    const double fac = -std::pow(3 / pi, 1 / 3.0) * c->f.e2;
    k_coulomb_out<<<div_up(c->V, kThreads), kThreads, 0, c->stream>>>(
        c->cpot, c->rho + c->V, c->nx, c->ny, c->nz, c->mx, c->my, fac, c->coulomb, c->coulex);
    MG_LAUNCHED(c);
    MG_CUDA(cudaMemcpyAsync(c->h_cg_status, c->cg_status, 4 * sizeof(int), cudaMemcpyDeviceToHost,
                            c->stream));
    if (iters) {
        MG_CUDA(cudaStreamSynchronize(c->stream));
        *iters = c->h_cg_status[1];
        if (c->h_cg_status[0] == 2) return MG_ERR_TIMEOUT;
        if (c->h_cg_status[0] == 1) return MG_NOT_CONVERGED;
    }
    return MG_OK;
}

}  // namespace mg
