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
