// transform.cu -- BreakParity, BreakSignature and BreakTimeSimplex
// (src/Transform.f90:187-366) of every HF spwf of an EV8 context, in the
// order TransformInput applies them (src/Transform.f90:83-99), into a
// symmetry-free context with twice the points per axis.
//
// Each break doubles one axis: the stored half keeps its values on the
// positive side and the mirrored line, times the sign CompSignExtension
// gives the component (src/Derivatives.f90:348-439), fills the negative
// side.  With the symmetries still conserved at each step (parity with
// signature and time simplex, then signature with time simplex, then time
// simplex alone) the mirrored lines are the stored ones, so a point of the
// full box reads the stored point |x|, |y|, |z| times the product of the
// signs of the mirrored axes:
//   z: signature * parity      (spin up),  -signature * parity      (spin down)
//   x: signature * time simplex (Re up, Im down), the opposite for Im up, Re down
//   y: time simplex (real parts), -time simplex (imaginary parts)
#include <algorithm>
#include <vector>

#include "mg_internal.cuh"

namespace mg {

namespace {

constexpr int kThreads = 256;

// qn of every spwf: (isospin, parity, signature, time simplex)
__global__ void __launch_bounds__(kThreads)
k_unfold(const double* __restrict__ src, const int* __restrict__ qn, int nx, int ny, int nz,
         double* __restrict__ dst) {
    const int i = blockIdx.y, l = blockIdx.z;
    const long V = (long)nx * ny * nz;
    const int X2 = 2 * nx, Y2 = 2 * ny;
    const long V8 = 8 * V;
    const int par = qn[4 * i + 1], sig = qn[4 * i + 2], ts = qn[4 * i + 3];
    const int sz = (l < 2 ? 1 : -1) * sig * par;
    const int sx = (l == 0 || l == 3 ? 1 : -1) * sig * ts;
    const int sy = (l == 0 || l == 2 ? 1 : -1) * ts;
    const double* s = src + ((long)i * 4 + l) * V;
    double* d = dst + ((long)i * 4 + l) * V8;
    for (long k = (long)blockIdx.x * kThreads + threadIdx.x; k < V8;
         k += (long)gridDim.x * kThreads) {
        const int X = (int)(k % X2), Y = (int)((k / X2) % Y2), Z = (int)(k / ((long)X2 * Y2));
        const int x = X >= nx ? X - nx : nx - 1 - X;
        const int y = Y >= ny ? Y - ny : ny - 1 - Y;
        const int z = Z >= nz ? Z - nz : nz - 1 - Z;
        int sg = 1;
        if (X < nx) sg *= sx;
        if (Y < ny) sg *= sy;
        if (Z < nz) sg *= sz;
        const double v = s[x + (long)nx * (y + (long)ny * z)];
        d[k] = sg > 0 ? v : -v;
    }
}

}  // namespace

}  // namespace mg

extern "C" int mg_break_symmetries(mg_ctx* ev8, mg_ctx* full) {
    using namespace mg;
    if (!ev8 || !full || ev8 == full) return MG_ERR_ARG;
    const mg_params &a = ev8->p, &b = full->p;
    if (!(a.pc && a.sc && a.tsc) || !ev8->folded) return MG_ERR_ARG;
    if (b.pc || b.sc || b.tsc || full->folded) return MG_ERR_ARG;
    if (b.nx != 2 * a.nx || b.ny != 2 * a.ny || b.nz != 2 * a.nz || b.nwt != a.nwt ||
        !b.trc != !a.trc || !(b.dx == a.dx))
        return MG_ERR_ARG;
    Basis& S = ev8->bas[MG_HF_BASIS];
    if (!S.have_qn) return MG_ERR_STATE;
    const int nwt = a.nwt;
    // the EV8 context's work is done before the other stream reads it
    MG_CUDA(cudaStreamSynchronize(ev8->stream));
    if (nwt > 0) {
        const long V8 = 8 * ev8->V;
        k_unfold<<<dim3(std::max(1, std::min(1024, div_up(V8, kThreads * 4))), nwt, 4), kThreads,
                   0, full->stream>>>(S.psi, S.qn, a.nx, a.ny, a.nz,
                                      full->bas[MG_HF_BASIS].psi);
        MG_LAUNCHED(full);
    }
    MG_CUDA(cudaStreamSynchronize(full->stream));
    // quantum numbers: isospin kept, the broken ones 0 (NewWaveFunction
    // calls of src/Transform.f90:239, :298, :357)
    std::vector<int> qn(4 * (size_t)nwt, 0);
    for (int i = 0; i < nwt; ++i) qn[4 * i] = S.h_qn[4 * i];
    MG_TRY(mg_upload_spinors(full, MG_HF_BASIS, nullptr, qn.data(), 0, nwt));
    std::vector<double> occ(nwt), e(nwt), disp(nwt);
    MG_TRY(mg_get_occupations(ev8, MG_HF_BASIS, occ.data()));
    MG_TRY(mg_get_energies(ev8, MG_HF_BASIS, e.data(), disp.data()));
    MG_TRY(mg_set_occupations(full, MG_HF_BASIS, occ.data()));
    MG_TRY(mg_set_energies(full, MG_HF_BASIS, e.data()));
    return MG_OK;
}
