// symops.cu -- SymmetryOperators (src/Spwf.f90:2289-2347) and CalcRMSRadius
// (:2339-2347) for every spwf of a basis, FP64.
//
// A conserved symmetry's expectation value is its quantum number; on the
// symmetry-free box the kernel forms, per spwf,
//   parity       Re <psi| P psi>,  P psi(r) = psi(-r)          ActionOfParity
//   signature    Im <psi| R psi>,  R psi = i sigma_z psi(-x,-y,z)  ActionOfSignature
//   time simplex Re <psi| T psi>,  T psi = conj psi(x,-y,z)    ActionOfTimeSimplex
//   x-simplex    Im <psi| X psi>,  X psi = -i sigma_x psi(-x,y,z) ActionOfXSimplex
// (src/Spinor.f90:391-490, grids mirrored about the box centre) and, on
// either box, <r^2> with the reference's mesh coordinates (IniMesh,
// src/Mesh.f90:40-85).  One CTA column per spwf writes block partials in a
// fixed order; the host adds them.
#include <cmath>
#include <vector>

#include "mg_internal.cuh"

namespace mg {

namespace {

constexpr int kThreads = 256;
constexpr int kQ = 5;   // r^2 |psi|^2, parity, signature, time simplex, x-simplex

__global__ void __launch_bounds__(kThreads)
k_symops(const double* __restrict__ psi, int nx, int ny, int nz, double dx, int full, long V,
         double* __restrict__ part) {
    __shared__ double red[kThreads / 32][kQ];
    const int i = blockIdx.y;
    const double* p = psi + (long)i * 4 * V;
    double acc[kQ] = {0, 0, 0, 0, 0};
    const double ox = full ? nx / 2.0 * dx : 0.0, oy = full ? ny / 2.0 * dx : 0.0,
                 oz = full ? nz / 2.0 * dx : 0.0;
    for (long v = (long)blockIdx.x * kThreads + threadIdx.x; v < V;
         v += (long)gridDim.x * kThreads) {
        const int x = (int)(v % nx), y = (int)((v / nx) % ny), z = (int)(v / ((long)nx * ny));
        double a[4];
#pragma unroll
        for (int l = 0; l < 4; ++l) a[l] = p[l * V + v];
        const double X = dx / 2.0 + dx * x - ox, Y = dx / 2.0 + dx * y - oy,
                     Z = dx / 2.0 + dx * z - oz;
        const double den = a[0] * a[0] + a[1] * a[1] + a[2] * a[2] + a[3] * a[3];
        acc[0] = fma(X * X + Y * Y + Z * Z, den, acc[0]);
        if (!full) continue;
        const int mx = nx - 1 - x, my = ny - 1 - y, mz = nz - 1 - z;
        double b[4];
        // parity: psi(-r)
        const long vp = mx + (long)nx * (my + (long)ny * mz);
#pragma unroll
        for (int l = 0; l < 4; ++l) b[l] = p[l * V + vp];
        acc[1] += a[0] * b[0] + a[1] * b[1] + a[2] * b[2] + a[3] * b[3];
        // signature: i sigma_z psi(-x,-y,z) = (-c2, c1, c4, -c3)
        const long vs = mx + (long)nx * (my + (long)ny * z);
        {
            const double c1 = p[vs], c2 = p[V + vs], c3 = p[2 * V + vs], c4 = p[3 * V + vs];
            const double t[4] = {-c2, c1, c4, -c3};
            acc[2] += t[1] * a[0] - t[0] * a[1] + t[3] * a[2] - t[2] * a[3];
        }
        // time simplex: conj psi(x,-y,z) = (c1, -c2, c3, -c4)
        const long vt = x + (long)nx * (my + (long)ny * z);
        {
            const double t[4] = {p[vt], -p[V + vt], p[2 * V + vt], -p[3 * V + vt]};
            acc[3] += a[0] * t[0] + a[1] * t[1] + a[2] * t[2] + a[3] * t[3];
        }
        // x-simplex: -i sigma_x psi(-x,y,z) = (c4, -c3, c2, -c1)
        const long vx = mx + (long)nx * (y + (long)ny * z);
        {
            const double c1 = p[vx], c2 = p[V + vx], c3 = p[2 * V + vx], c4 = p[3 * V + vx];
            const double t[4] = {c4, -c3, c2, -c1};
            acc[4] += t[1] * a[0] - t[0] * a[1] + t[3] * a[2] - t[2] * a[3];
        }
    }
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
#pragma unroll
    for (int q = 0; q < kQ; ++q) {
        double s = acc[q];
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) red[warp][q] = s;
    }
    __syncthreads();
    if (threadIdx.x < kQ) {
        double s = 0.0;
        for (int w = 0; w < kThreads / 32; ++w) s += red[w][threadIdx.x];
        part[((long)i * gridDim.x + blockIdx.x) * kQ + threadIdx.x] = s;
    }
}

// DiagAng's <J> (src/Spwf.f90:976-1085): spin part sigma/2 plus the
// orbital part -i r x nabla, real parts, per spwf.  der holds Der(1:3) as
// [d][l][V] per spwf, FP64 or double-float {hi, lo} pairs.  jx / jy are
// skipped where signature (and, for jy, time simplex) makes them zero.
constexpr int kJ = 3;

__device__ __forceinline__ double der_at(const double* p, long k, int df) {
    if (!df) return p[k];
    const float2 hl = reinterpret_cast<const float2*>(p)[k];
    return (double)hl.x + (double)hl.y;
}

__global__ void __launch_bounds__(kThreads)
k_angmom(const double* __restrict__ psi, const double* __restrict__ der, int df, int nx, int ny,
         int nz, double dx, int full, int want_x, int want_y, long V, double* __restrict__ part) {
    __shared__ double red[kThreads / 32][kJ];
    const int i = blockIdx.y;
    const double* p = psi + (long)i * 4 * V;
    const double* d = der + (long)i * 12 * V;
    double acc[kJ] = {0, 0, 0};
    const double ox = full ? nx / 2.0 * dx : 0.0, oy = full ? ny / 2.0 * dx : 0.0,
                 oz = full ? nz / 2.0 * dx : 0.0;
    for (long v = (long)blockIdx.x * kThreads + threadIdx.x; v < V;
         v += (long)gridDim.x * kThreads) {
        const int x = (int)(v % nx), y = (int)((v / nx) % ny), z = (int)(v / ((long)nx * ny));
        const double X = dx / 2.0 + dx * x - ox, Y = dx / 2.0 + dx * y - oy,
                     Z = dx / 2.0 + dx * z - oz;
        double a[4], gx[4], gy[4], gz[4];
#pragma unroll
        for (int l = 0; l < 4; ++l) {
            a[l] = p[l * V + v];
            gx[l] = der_at(d, (0 * 4 + l) * V + v, df);
            gy[l] = der_at(d, (1 * 4 + l) * V + v, df);
        }
        // Jz: spin 1/2 (|1|^2 + |2|^2 - |3|^2 - |4|^2); orbital with the
        // (re, im) pairs (1, 2) and (3, 4) of the two spin components
        double jz = 0.5 * (a[0] * a[0] + a[1] * a[1] - a[2] * a[2] - a[3] * a[3]);
        jz += a[1] * (Y * gx[0] - X * gy[0]) - a[0] * (Y * gx[1] - X * gy[1]) +
              a[3] * (Y * gx[2] - X * gy[2]) - a[2] * (Y * gx[3] - X * gy[3]);
        acc[2] += jz;
        if (want_x | want_y) {
#pragma unroll
            for (int l = 0; l < 4; ++l) gz[l] = der_at(d, (2 * 4 + l) * V + v, df);
            if (want_x) {
                double jx = a[0] * a[2] + a[1] * a[3];
                jx += a[1] * (Z * gy[0] - Y * gz[0]) - a[0] * (Z * gy[1] - Y * gz[1]) +
                      a[3] * (Z * gy[2] - Y * gz[2]) - a[2] * (Z * gy[3] - Y * gz[3]);
                acc[0] += jx;
            }
            if (want_y) {
                double jy = a[0] * a[3] - a[1] * a[2];
                jy += a[1] * (X * gz[0] - Z * gx[0]) - a[0] * (X * gz[1] - Z * gx[1]) +
                      a[3] * (X * gz[2] - Z * gx[2]) - a[2] * (X * gz[3] - Z * gx[3]);
                acc[1] += jy;
            }
        }
    }
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
#pragma unroll
    for (int q = 0; q < kJ; ++q) {
        double s = acc[q];
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) red[warp][q] = s;
    }
    __syncthreads();
    if (threadIdx.x < kJ) {
        double s = 0.0;
        for (int w = 0; w < kThreads / 32; ++w) s += red[w][threadIdx.x];
        part[((long)i * gridDim.x + blockIdx.x) * kJ + threadIdx.x] = s;
    }
}

}  // namespace

}  // namespace mg

extern "C" int mg_symmetry_operators(mg_ctx* c, int b, double* out) {
    using namespace mg;
    if (!c || !out || b < 0 || b > 1) return MG_ERR_ARG;
    if (b == MG_CAN_BASIS && c->p.pairing != MG_PAIRING_HFB) return MG_ERR_ARG;
    Basis& B = c->bas[b];
    if (!B.have_qn) return MG_ERR_STATE;
    const long V = c->V;
    const int nwt = c->p.nwt;
    const int nch = std::max(1, std::min(16, div_up(V, kThreads * 4)));
    if ((size_t)nwt * nch * kQ > c->red_len) return MG_ERR_STATE;
    const int full = c->folded ? 0 : 1;
    k_symops<<<dim3(nch, nwt), kThreads, 0, c->stream>>>(B.psi, c->nx, c->ny, c->nz, c->p.dx, full,
                                                         V, c->red);
    MG_LAUNCHED(c);
    std::vector<double> h((size_t)nwt * nch * kQ);
    MG_CUDA(cudaMemcpyAsync(h.data(), c->red, h.size() * sizeof(double), cudaMemcpyDeviceToHost,
                            c->stream));
    MG_CUDA(cudaStreamSynchronize(c->stream));
    for (int i = 0; i < nwt; ++i) {
        double s[kQ] = {0, 0, 0, 0, 0};
        for (int q = 0; q < nch; ++q)
            for (int k = 0; k < kQ; ++k) s[k] += h[((size_t)i * nch + q) * kQ + k];
        const int* qn = &B.h_qn[4 * i];
        double* o = out + 6 * i;
        // a nonzero quantum number is its own expectation value (the
        // symmetry-free box stores 0 for the ones it breaks)
        o[0] = qn[0];
        o[1] = qn[2] != 0 ? qn[2] : s[2] * c->dv;
        o[2] = qn[1] != 0 ? qn[1] : s[1] * c->dv;
        o[3] = qn[3] != 0 ? qn[3] : s[3] * c->dv;
        o[4] = qn[2] != 0 ? 0.0 : s[4] * c->dv;
        o[5] = std::sqrt(s[0] * c->dv);
    }
    return MG_OK;
}

extern "C" int mg_angular_momentum(mg_ctx* c, int b, double* out) {
    using namespace mg;
    if (!c || !out || b < 0 || b > 1) return MG_ERR_ARG;
    if (b == MG_CAN_BASIS && c->p.pairing != MG_PAIRING_HFB) return MG_ERR_ARG;
    Basis& B = c->bas[b];
    if (!B.have_qn) return MG_ERR_STATE;
    MG_TRY(derive_basis(c, b));
    const long V = c->V;
    const int nwt = c->p.nwt;
    const int nch = std::max(1, std::min(16, div_up(V, kThreads * 4)));
    if ((size_t)nwt * nch * kJ > c->red_len) return MG_ERR_STATE;
    const int full = c->folded ? 0 : 1;
    const int want_x = c->p.sc ? 0 : 1, want_y = (c->p.sc || c->p.tsc) ? 0 : 1;
    k_angmom<<<dim3(nch, nwt), kThreads, 0, c->stream>>>(B.psi, B.der, B.der_df ? 1 : 0, c->nx,
                                                         c->ny, c->nz, c->p.dx, full, want_x,
                                                         want_y, V, c->red);
    MG_LAUNCHED(c);
    std::vector<double> h((size_t)nwt * nch * kJ);
    MG_CUDA(cudaMemcpyAsync(h.data(), c->red, h.size() * sizeof(double), cudaMemcpyDeviceToHost,
                            c->stream));
    MG_CUDA(cudaStreamSynchronize(c->stream));
    for (int i = 0; i < nwt; ++i) {
        double s[kJ] = {0, 0, 0};
        for (int q = 0; q < nch; ++q)
            for (int k = 0; k < kJ; ++k) s[k] += h[((size_t)i * nch + q) * kJ + k];
        for (int k = 0; k < kJ; ++k) out[3 * i + k] = s[k] * c->dv;
    }
    return MG_OK;
}
