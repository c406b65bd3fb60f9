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
#include <algorithm>
#include <mutex>

#include "df.cuh"

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

// ---- mixed precision: double-float arithmetic, FP64 grids in and out -------------
//
// The mixed form evaluates the contractions in double-float (df.cuh): every
// FP64 value is split into hi + lo floats, products are exact FMA residuals
// and the running sum is a (hi, lo) pair (df_acc), ~1e-14 relative at ~12
// FP32 operations per term.  Each thread owns four consecutive outputs along the contracted axis
// (or four rows for d/dx), so every shared-memory pair it loads feeds four or
// eight terms.  Matrices are stored transposed as (hi, lo) float planes with
// a row stride rounded up to a multiple of 4 (zero padding).

struct MatPtrs32 {
    const float* m[3][2][2];  // [axis][kind][slot]: hi plane [q][ld4], lo plane after it
    int ld4[3];
};


__global__ void __launch_bounds__(256)
k_deriv_xy_df(const GridJob* __restrict__ jobs, MatPtrs32 mp, int nx, int ny, int nz,
              int planes_per_block, int out_df) {
    extern __shared__ float smf[];
    const GridJob J = jobs[blockIdx.x];
    const bool want_x = J.dx != nullptr || J.lap != nullptr;
    const bool want_y = J.dy != nullptr || J.lap != nullptr;
    if (!want_x && !want_y) return;
    const int lx = mp.ld4[0], ly = mp.ld4[1];
    const int ny4 = (ny + 3) / 4;
    const int mx = nx * lx, my = ny * ly;
    float* sDx = smf;              // hi [mx], lo [mx]
    float* sLx = sDx + 2 * mx;
    float* sDy = sLx + 2 * mx;
    float* sLy = sDy + 2 * my;
    float* sPh = sLy + 2 * my;     // (4 * ny4) rows x nx, rows >= ny zero
    float* sPl = sPh + 4 * ny4 * nx;
    const float* gDx = J.slot[0] ? mp.m[0][0][1] : mp.m[0][0][0];
    const float* gLx = J.slot[0] ? mp.m[0][1][1] : mp.m[0][1][0];
    const float* gDy = J.slot[1] ? mp.m[1][0][1] : mp.m[1][0][0];
    const float* gLy = J.slot[1] ? mp.m[1][1][1] : mp.m[1][1][0];
    for (int t = threadIdx.x; t < 2 * mx; t += blockDim.x) {
        sDx[t] = gDx[t];
        sLx[t] = gLx[t];
    }
    for (int t = threadIdx.x; t < 2 * my; t += blockDim.x) {
        sDy[t] = gDy[t];
        sLy[t] = gLy[t];
    }
    for (int t = ny * nx + threadIdx.x; t < 4 * ny4 * nx; t += blockDim.x) {
        sPh[t] = 0.0f;
        sPl[t] = 0.0f;
    }
    const int plane = nx * ny;
    const int items = nx * ny4;
    const int k0 = blockIdx.y * planes_per_block;
    const int k1 = min(nz, k0 + planes_per_block);
    for (int k = k0; k < k1; ++k) {
        const double* in = J.in + (long)k * plane;
        __syncthreads();
        for (int t = threadIdx.x; t < plane; t += blockDim.x) {
            const dfl v = df_split(in[t]);
            sPh[t] = v.h;
            sPl[t] = v.l;
        }
        __syncthreads();
        for (int it = threadIdx.x; it < items; it += blockDim.x) {
            const int x = it % nx, y0 = 4 * (it / nx);
            float axh[4] = {0.f, 0.f, 0.f, 0.f}, axl[4] = {0.f, 0.f, 0.f, 0.f};
            float bxh[4] = {0.f, 0.f, 0.f, 0.f}, bxl[4] = {0.f, 0.f, 0.f, 0.f};
            float ayh[4] = {0.f, 0.f, 0.f, 0.f}, ayl[4] = {0.f, 0.f, 0.f, 0.f};
            float byh[4] = {0.f, 0.f, 0.f, 0.f}, byl[4] = {0.f, 0.f, 0.f, 0.f};
            if (want_x) {
                for (int q = 0; q < nx; ++q) {
                    const float dh = sDx[q * lx + x], dl = sDx[mx + q * lx + x];
                    const float lh = sLx[q * lx + x], ll = sLx[mx + q * lx + x];
#pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        const float vh = sPh[(y0 + j) * nx + q], vl = sPl[(y0 + j) * nx + q];
                        df_acc(axh[j], axl[j], dfl{dh, dl}, dfl{vh, vl});
                        df_acc(bxh[j], bxl[j], dfl{lh, ll}, dfl{vh, vl});
                    }
                }
            }
            if (want_y) {
                for (int q = 0; q < ny; ++q) {
                    const float vh = sPh[q * nx + x], vl = sPl[q * nx + x];
                    const float4 dh = *reinterpret_cast<const float4*>(sDy + q * ly + y0);
                    const float4 dl = *reinterpret_cast<const float4*>(sDy + my + q * ly + y0);
                    const float4 lh = *reinterpret_cast<const float4*>(sLy + q * ly + y0);
                    const float4 ll = *reinterpret_cast<const float4*>(sLy + my + q * ly + y0);
                    df_acc(ayh[0], ayl[0], dfl{dh.x, dl.x}, dfl{vh, vl});
                    df_acc(ayh[1], ayl[1], dfl{dh.y, dl.y}, dfl{vh, vl});
                    df_acc(ayh[2], ayl[2], dfl{dh.z, dl.z}, dfl{vh, vl});
                    df_acc(ayh[3], ayl[3], dfl{dh.w, dl.w}, dfl{vh, vl});
                    df_acc(byh[0], byl[0], dfl{lh.x, ll.x}, dfl{vh, vl});
                    df_acc(byh[1], byl[1], dfl{lh.y, ll.y}, dfl{vh, vl});
                    df_acc(byh[2], byl[2], dfl{lh.z, ll.z}, dfl{vh, vl});
                    df_acc(byh[3], byl[3], dfl{lh.w, ll.w}, dfl{vh, vl});
                }
            }
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                if (y0 + j >= ny) break;
                const long o = (long)k * plane + (long)(y0 + j) * nx + x;
                const dfl ox = df_norm(dfl{axh[j], axl[j]}), oy = df_norm(dfl{ayh[j], ayl[j]});
                const dfl ol = df_add(df_norm(dfl{bxh[j], bxl[j]}), df_norm(dfl{byh[j], byl[j]}));
                if (out_df) {
                    if (J.dx) df_st(reinterpret_cast<float2*>(J.dx) + o, ox);
                    if (J.dy) df_st(reinterpret_cast<float2*>(J.dy) + o, oy);
                    if (J.lap) df_st(reinterpret_cast<float2*>(J.lap) + o, ol);
                } else {
                    if (J.dx) J.dx[o] = df_to(ox);
                    if (J.dy) J.dy[o] = df_to(oy);
                    if (J.lap) J.lap[o] = df_to(ol);
                }
            }
        }
    }
}

__global__ void __launch_bounds__(512)
k_deriv_z_df(const GridJob* __restrict__ jobs, MatPtrs32 mp, int nx, int ny, int nz,
             int out_df) {
    extern __shared__ float smf[];
    const GridJob J = jobs[blockIdx.x];
    if (J.dz == nullptr && J.lap == nullptr) return;
    const int lz = mp.ld4[2];
    const int mz = nz * lz;
    float* sDz = smf;
    float* sLz = sDz + 2 * mz;
    float* sGh = sLz + 2 * mz;  // [q][col]
    float* sGl = sGh + nz * kColTile;
    const float* gDz = J.slot[2] ? mp.m[2][0][1] : mp.m[2][0][0];
    const float* gLz = J.slot[2] ? mp.m[2][1][1] : mp.m[2][1][0];
    for (int t = threadIdx.x; t < 2 * mz; t += blockDim.x) {
        sDz[t] = gDz[t];
        sLz[t] = gLz[t];
    }
    const int plane = nx * ny;
    const int c0 = blockIdx.y * kColTile;
    for (int t = threadIdx.x; t < nz * kColTile; t += blockDim.x) {
        const int q = t / kColTile, cc = t % kColTile;
        const dfl v = df_split((c0 + cc < plane) ? J.in[(long)q * plane + c0 + cc] : 0.0);
        sGh[t] = v.h;
        sGl[t] = v.l;
    }
    __syncthreads();
    const int nz4 = (nz + 3) / 4;
    for (int it = threadIdx.x; it < kColTile * nz4; it += blockDim.x) {
        const int col = it % kColTile, i0 = 4 * (it / kColTile);
        if (c0 + col >= plane) continue;
        float azh[4] = {0.f, 0.f, 0.f, 0.f}, azl[4] = {0.f, 0.f, 0.f, 0.f};
        float bzh[4] = {0.f, 0.f, 0.f, 0.f}, bzl[4] = {0.f, 0.f, 0.f, 0.f};
        for (int q = 0; q < nz; ++q) {
            const float vh = sGh[q * kColTile + col], vl = sGl[q * kColTile + col];
            const float4 dh = *reinterpret_cast<const float4*>(sDz + q * lz + i0);
            const float4 dl = *reinterpret_cast<const float4*>(sDz + mz + q * lz + i0);
            const float4 lh = *reinterpret_cast<const float4*>(sLz + q * lz + i0);
            const float4 ll = *reinterpret_cast<const float4*>(sLz + mz + q * lz + i0);
            df_acc(azh[0], azl[0], dfl{dh.x, dl.x}, dfl{vh, vl});
            df_acc(azh[1], azl[1], dfl{dh.y, dl.y}, dfl{vh, vl});
            df_acc(azh[2], azl[2], dfl{dh.z, dl.z}, dfl{vh, vl});
            df_acc(azh[3], azl[3], dfl{dh.w, dl.w}, dfl{vh, vl});
            df_acc(bzh[0], bzl[0], dfl{lh.x, ll.x}, dfl{vh, vl});
            df_acc(bzh[1], bzl[1], dfl{lh.y, ll.y}, dfl{vh, vl});
            df_acc(bzh[2], bzl[2], dfl{lh.z, ll.z}, dfl{vh, vl});
            df_acc(bzh[3], bzl[3], dfl{lh.w, ll.w}, dfl{vh, vl});
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            if (i0 + j >= nz) break;
            const long o = (long)(i0 + j) * plane + c0 + col;
            const dfl oz = df_norm(dfl{azh[j], azl[j]}), olz = df_norm(dfl{bzh[j], bzl[j]});
            if (out_df) {
                if (J.dz) df_st(reinterpret_cast<float2*>(J.dz) + o, oz);
                if (J.lap) {
                    float2* pl = reinterpret_cast<float2*>(J.lap) + o;
                    df_st(pl, df_add(df_ld(pl), olz));
                }
            } else {
                if (J.dz) J.dz[o] = df_to(oz);
                if (J.lap) J.lap[o] = J.lap[o] + df_to(olz);
            }
        }
    }
}

MatPtrs32 mat_ptrs32(const mg_ctx* c) {
    MatPtrs32 mp;
    const int ns[3] = {c->nx, c->ny, c->nz};
    for (int a = 0; a < 3; ++a) {
        mp.ld4[a] = (ns[a] + 3) / 4 * 4;
        for (int k = 0; k < 2; ++k)
            for (int s = 0; s < 2; ++s) mp.m[a][k][s] = c->mats32 + c->mat32_off[a][k][s];
    }
    return mp;
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
    // double-float copy for the mixed-precision kernels: hi plane [q][ld4]
    // then lo plane, zero padding
    long total32 = 0;
    for (int a = 0; a < 3; ++a) {
        const int ld4 = (ns[a] + 3) / 4 * 4;
        for (int k = 0; k < 2; ++k)
            for (int s = 0; s < 2; ++s) {
                c->mat32_off[a][k][s] = total32;
                total32 += 2L * ns[a] * ld4;
            }
    }
    std::vector<float> h32(total32, 0.0f);
    for (int a = 0; a < 3; ++a) {
        const int n = ns[a], ld4 = (n + 3) / 4 * 4;
        for (int k = 0; k < 2; ++k)
            for (int s = 0; s < 2; ++s)
                for (int q = 0; q < n; ++q)
                    for (int i = 0; i < n; ++i) {
                        const double x = h[c->mat_off[a][k][s] + (long)q * n + i];
                        const float hi = (float)x;
                        const long o = c->mat32_off[a][k][s] + (long)q * ld4 + i;
                        h32[o] = hi;
                        h32[o + (long)n * ld4] = (float)(x - (double)hi);
                    }
    }
    MG_CUDA(cudaMalloc(&c->mats32, total32 * sizeof(float)));
    MG_CUDA(cudaMemcpy(c->mats32, h32.data(), total32 * sizeof(float), cudaMemcpyHostToDevice));
    return tc_setup(c);
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

// Tile autotuner of the x/y kernels: z planes per block trade the per-block
// staging of the axis matrices against parallelism, and the best count
// depends on the mesh and on how many grids a call derives.  On the first
// call of each (form, grid-count class) every candidate (1, 2, 4, 8 planes,
// at most nz) runs twice on the real jobs, timed with events on the
// context's stream, and the fastest is kept.  The x/y kernel writes the
// same values whatever the count (every line is computed the same way), so
// the repeated runs leave the outputs as one run does; the z kernel, which
// adds to the Laplacian, runs once afterwards.
template <class Launch>
static int tuned_planes(mg_ctx* c, int& slot, Launch launch_xy) {
    if (slot > 0) return MG_OK;
    const int cand[4] = {1, 2, 4, 8};
    cudaEvent_t ev[2];
    MG_CUDA(cudaEventCreate(&ev[0]));
    MG_CUDA(cudaEventCreate(&ev[1]));
    float best = 1e30f;
    int best_p = 1;
    int st = MG_OK;
    for (int p : cand) {
        if (p > c->nz && p > 1) break;
        if ((st = launch_xy(p)) != MG_OK) break;            // warm-up
        if (cudaEventRecord(ev[0], c->stream) != cudaSuccess) { st = MG_ERR_CUDA; break; }
        for (int r = 0; r < 2 && st == MG_OK; ++r) st = launch_xy(p);
        if (st != MG_OK) break;
        float ms = 0.0f;
        if (cudaEventRecord(ev[1], c->stream) != cudaSuccess ||
            cudaEventSynchronize(ev[1]) != cudaSuccess ||
            cudaEventElapsedTime(&ms, ev[0], ev[1]) != cudaSuccess) { st = MG_ERR_CUDA; break; }
        if (ms < best) { best = ms; best_p = p; }
    }
    cudaEventDestroy(ev[0]);
    cudaEventDestroy(ev[1]);
    if (st == MG_OK) slot = best_p;
    return st;
}

int run_jobs(mg_ctx* c, const GridJob* jobs, int njobs, bool out_df) {
    if (njobs <= 0) return MG_OK;
    const int nx = c->nx, ny = c->ny, nz = c->nz;
    // z planes per k_deriv_xy block, tuned per (form, grid-count class):
    // few grids (densities, fields) and whole bases
    int& ppb = c->deriv_planes[c->cur_precision == MG_MIXED ? 1 : 0][njobs < 64 ? 0 : 1];
    // the shared-memory opt-in is a per-device attribute: set it once per
    // device (contexts of a batch call this from several host threads)
    {
        static std::mutex attr_mu;
        static bool attr_done[64] = {};
        int dev = 0;
        MG_CUDA(cudaGetDevice(&dev));
        if (dev < 0 || dev >= 64) return MG_ERR_ARG;
        std::lock_guard<std::mutex> lock(attr_mu);
        if (!attr_done[dev]) {
            const void* fns[4] = {(const void*)k_deriv_xy, (const void*)k_deriv_z,
                                  (const void*)k_deriv_xy_df, (const void*)k_deriv_z_df};
            for (const void* f : fns)
                MG_CUDA(cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             200 * 1024));
            attr_done[dev] = true;
        }
    }
    if (c->cur_precision == MG_MIXED) {
        // out_df: the outputs stay double-float ({hi, lo} float pairs)
        MatPtrs32 mp = mat_ptrs32(c);
        const int ny4 = (ny + 3) / 4, nz4 = (nz + 3) / 4;
        const size_t sm_xy =
            (size_t)(4 * nx * mp.ld4[0] + 4 * ny * mp.ld4[1] + 8 * ny4 * nx) * sizeof(float);
        const size_t sm_z = (size_t)(4 * nz * mp.ld4[2] + 2 * nz * kColTile) * sizeof(float);
        const int txy = std::min(256, div_up((long)nx * ny4, 32) * 32);
        const int tz = std::min(512, kColTile * nz4);
        auto xy = [&](int p) {
            k_deriv_xy_df<<<dim3(njobs, div_up(nz, p)), txy, sm_xy, c->stream>>>(jobs, mp, nx, ny,
                                                                               nz, p, out_df);
            MG_LAUNCHED(c);
            return MG_OK;
        };
        if (ppb == 0) MG_TRY(tuned_planes(c, ppb, xy));
        MG_TRY(xy(ppb));
        k_deriv_z_df<<<dim3(njobs, div_up((long)nx * ny, kColTile)), tz, sm_z, c->stream>>>(
            jobs, mp, nx, ny, nz, out_df ? 1 : 0);
        MG_LAUNCHED(c);
        return MG_OK;
    }
    if (out_df) return MG_ERR_STATE;   // double-float outputs only from the mixed kernels
    MatPtrs mp = mat_ptrs(c);
    size_t sm_xy = (size_t)(2 * nx * nx + 2 * ny * ny + nx * ny) * sizeof(double);
    size_t sm_z = (size_t)(2 * nz * nz + nz * kColTile) * sizeof(double);
    auto xy = [&](int p) {
        k_deriv_xy<<<dim3(njobs, div_up(nz, p)), kThreads, sm_xy, c->stream>>>(jobs, mp, nx, ny,
                                                                              nz, p);
        MG_LAUNCHED(c);
        return MG_OK;
    };
    if (ppb == 0) MG_TRY(tuned_planes(c, ppb, xy));
    MG_TRY(xy(ppb));
    dim3 gz(njobs, div_up((long)nx * ny, kColTile));
    k_deriv_z<<<gz, kThreads, sm_z, c->stream>>>(jobs, mp, nx, ny, nz);
    MG_LAUNCHED(c);
    return MG_OK;
}

// In the mixed form the basis derivatives stay double-float in HBM (the same
// 8 bytes per value), so that h.psi and the densities read them without FP64
// conversions; Basis::der_df records the format.  They come from the tensor
// cores (deriv_tc.cu) when every line length is at most 32, else from the
// double-float kernels above.
int derive_basis(mg_ctx* c, int b) {
    if (!c->bas[b].have_qn) return MG_ERR_STATE;
    const bool df = c->cur_precision == MG_MIXED;
    if (df && c->tc_ok)
        MG_TRY(run_jobs_tc(c, c->bas[b].jobs, 4 * c->p.nwt));
    else
        MG_TRY(run_jobs(c, c->bas[b].jobs, 4 * c->p.nwt, df));
    c->bas[b].der_df = df;
    return MG_OK;
}

}  // namespace mg
