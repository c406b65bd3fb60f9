// hfb.cu -- small dense HFB algebra on the device, FP64, and the host driver
// of the HFB pairing step.
//
// Replaces, for the EV8 + time-reversal case (signature and time simplex
// conserved, no Lipkin-Nogami, no blocking):
//   ConstructHFBHamiltonian              src/HFB.f90:2554-2631
//   DiagonaliseHFBHamiltonian_Signature  :2695-2786 (diagoncr8 :5880-6087)
//   HFBNumberofParticles_ordinary        :810-1072  (PfSolver off: CR8 columns)
//   constructRhoHFB / ConstructKappaHFB  :3128-3154, :3335-3359
//   DiagonaliseRhoHFB / HFBOccupations   :3156-3284, :3361-3560
//   HFBEnergy                            :296-348
//   GuessHFBMatrices (case 2, TRC)       :3645-3835
// The signature-reduced HFB matrix of a block is
//   T = [[e - lambda, D], [D^T, -(e - lambda)]],  D(i,j) = Delta(i, j+h),
// with eigenvectors X (ascending).  With the CR8 column choice the positive
// quasiparticle half gives, for the stored (+) and reversed (-) halves,
//   rho_++ = rho_-- = Y Y^T,  kappa_-+ = Y W^T,  Y = X(h:N, h:N), W = X(0:h, h:N)
// and zero elsewhere.  The eigen-decompositions (of T per particle-number
// evaluation and of rho_++ for the canonical basis) use the batched solver of
// eig.cu: FP32 Jacobi seed + FP64 Ogita-Aishima refinement to FP64 accuracy.
//
// FindFermiEnergy: the reference's damped Broyden (src/HFB.f90:1849-2161)
// is replaced by a safeguarded Newton iteration on the same equation
// N(lambda) = N0 with the same tolerance FermiPrec per isospin; both reach the
// same root.  dN/dlambda comes analytically from the eigen-decomposition, and
// every particle-number evaluation is one short stream of launches ending in
// a 12-double read-back.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "mg_internal.cuh"

namespace mg {

namespace {

constexpr int kThreads = 256;
// Rotation angle |S_mn| / |E_m - E_n| between states of opposite
// quasiparticle-energy sign below which the refinement step that measured it
// leaves the positive/negative split exact to FP64 rounding (the angle left
// is ~ tol^2).
constexpr double kRefineTol = 1e-8;
// Largest Newton step of the Fermi energy finished by the first-order
// expansion instead of an evaluation (the second-order remainder in N is
// below 1e-13 for the curvatures seen, far inside FermiPrec = 1e-12).  With
// a recent estimate of the curvature |N''| (kCurvatureAge iterations at
// most) the step may grow to sqrt(kCurvatureBudget FermiPrec / |N''|), which
// keeps the remainder |N''| dl^2 / 2 below FermiPrec / 40, up to kTaylorMax.
// Measured at 24^3, nwt=160: |N''| between 0.003 and 1.1 MeV^-2.
constexpr double kTaylorStep = 2e-7;
constexpr double kTaylorMax = 1e-5;
constexpr double kCurvatureBudget = 0.05;
constexpr int kCurvatureAge = 20;
// ... and only while the step is small against the quasiparticle gap around
// zero energy (2 min E): the expansion coefficients go as 1 / (E_m - E_n), so
// the neglected second order is ~(dl / gap)^2.  A level at the Fermi energy
// with vanishing pairing (unbound neutrons, say) closes the gap and takes
// every step back to a full evaluation.
constexpr double kTaylorGap = 1e-6;
// Fermi-energy step (MeV) above which an evaluation re-seeds its
// eigen-decomposition instead of refining the previous vectors.
constexpr double kFarStep = 0.5;

__device__ double cta_sum(double x, double* red) {
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    __syncthreads();
    if (threadIdx.x % 32 == 0) red[threadIdx.x / 32] = x;
    __syncthreads();
    double s = 0.0;
    for (int w = 0; w < (int)(blockDim.x / 32); ++w) s += red[w];
    __syncthreads();
    return s;
}

// T_b(lambda) for the four blocks (ConstructHFBHamiltonian restricted to the
// real signature-reduced matrix of DiagonaliseHFBHamiltonian_Signature).
__global__ void k_build_T(const double* __restrict__ delta, const double* __restrict__ e_hf,
                          const int* __restrict__ members, const int* __restrict__ hsz, int hmax,
                          int nmax, const double* __restrict__ fermi, double* __restrict__ T) {
    const int b = blockIdx.y;
    const int h = hsz[b], N = 2 * h;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= N * N) return;
    const int i = t / N, j = t % N;
    const double lam = fermi[b / 2];
    const double* D = delta + (long)b * nmax * nmax;
    double v = 0.0;
    if (i < h && j < h) {
        if (i == j) v = e_hf[members[b * hmax + i]] - lam;
    } else if (i >= h && j >= h) {
        if (i == j) v = -(e_hf[members[b * hmax + i - h]] - lam);
    } else if (i < h) {
        v = D[(long)i * N + j];
    } else {
        v = D[(long)j * N + i];
    }
    T[(long)b * nmax * nmax + (long)i * nmax + j] = v;
}

// rho and kappa from the positive quasiparticle half of the eigenvectors
__global__ void k_rho_kappa(const double* __restrict__ X, const int* __restrict__ hsz, int nmax,
                            double* __restrict__ rho, double* __restrict__ kappa) {
    const int b = blockIdx.y;
    const int h = hsz[b], N = 2 * h;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= h * h) return;
    const int r = t / h, s = t % h;
    const double* Xb = X + (long)b * nmax * nmax;
    double rr = 0.0, kk = 0.0;
    for (int m = N - 1; m >= h; --m) {
        const double y = Xb[(long)(h + r) * nmax + m];
        rr = fma(y, Xb[(long)(h + s) * nmax + m], rr);
        kk = fma(y, Xb[(long)s * nmax + m], kk);
    }
    double* R = rho + (long)b * nmax * nmax;
    double* K = kappa + (long)b * nmax * nmax;
    R[(long)r * N + s] = rr;
    R[(long)(h + r) * N + h + s] = rr;
    R[(long)r * N + h + s] = 0.0;
    R[(long)(h + r) * N + s] = 0.0;
    K[(long)(h + r) * N + s] = kk;
    K[(long)s * N + h + r] = -kk;
    K[(long)r * N + s] = 0.0;
    K[(long)(h + r) * N + h + s] = 0.0;
}

// dN/dlambda of a block from its eigen-decomposition.  T(lambda) = T0 -
// lambda Sigma, Sigma = diag(I, -I); first-order perturbation of the vectors
// gives, with P the projector on the lower (time-reversed) half and the
// quasiparticle energies E,
//   dN/dlambda = 8 sum_{m > 0 > n} (x_m^T P x_n)^2 / (E_m - E_n)  (> 0).
// One CTA per positive state m; dpart[b][m - h] receives its row of the sum.
__global__ void __launch_bounds__(128)
k_dn_dlambda(const double* __restrict__ X, const double* __restrict__ E,
             const int* __restrict__ hsz, int nmax, double* __restrict__ dpart) {
    __shared__ double xm[kEigMax / 2];
    __shared__ double red[32];
    const int b = blockIdx.y, h = hsz[b], N = 2 * h;
    const int mm = blockIdx.x;
    if (mm >= h) return;
    const int m = h + mm;
    const double* Xb = X + (long)b * nmax * nmax;
    for (int r = threadIdx.x; r < h; r += blockDim.x) xm[r] = Xb[(long)(h + r) * nmax + m];
    __syncthreads();
    const double Em = E[(long)b * nmax + m];
    double part = 0.0;
    for (int n = threadIdx.x; n < h; n += blockDim.x) {
        double p = 0.0;
        for (int r = 0; r < h; ++r) p = fma(xm[r], Xb[(long)(h + r) * nmax + n], p);
        part += p * p / (Em - E[(long)b * nmax + n]);
    }
    const double s = cta_sum(part, red);
    if (threadIdx.x == 0) dpart[(long)b * (nmax / 2) + mm] = 8.0 * s;
    (void)N;
}

// Per block: Tr rho (the particle number of HFBNumberofParticles) into
// out[b], dN/dlambda into out[4 + b], and the largest opposite-sign rotation
// angle seen by the last refinement step into out[8 + b].
__global__ void k_trace(const double* __restrict__ rho, const int* __restrict__ hsz, int nmax,
                        const double* __restrict__ dpart, const double* __restrict__ emax,
                        const double* __restrict__ w, long wstride, double* __restrict__ out) {
    __shared__ double red[32];
    const int b = blockIdx.x;
    const int h = hsz[b], N = 2 * h;
    double p = 0.0, d = 0.0, e = 0.0;
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
        p += rho[(long)b * nmax * nmax + (long)i * N + i];
        e = fmax(e, emax[(long)b * nmax + i]);
    }
    for (int i = threadIdx.x; i < h; i += blockDim.x) d += dpart[(long)b * (nmax / 2) + i];
    const double s = cta_sum(p, red);
    const double ds = cta_sum(d, red);
    for (int o = 16; o > 0; o >>= 1) e = fmax(e, __shfl_xor_sync(0xffffffffu, e, o));
    if (threadIdx.x % 32 == 0) red[threadIdx.x / 32] = e;
    __syncthreads();
    if (threadIdx.x == 0) {
        double em = 0.0;
        for (int k = 0; k < (int)(blockDim.x / 32); ++k) em = fmax(em, red[k]);
        out[b] = s;
        out[4 + b] = ds;
        out[8 + b] = em;
        // quasiparticle gap around zero energy: the spectrum of a block is
        // +-E pairs in ascending order, so it is w[h] - w[h-1] = 2 min E
        out[12 + b] = h > 0 ? w[(long)b * wstride + h] - w[(long)b * wstride + h - 1] : 1e300;
    }
}

// First-order finish of the Fermi search.  With T(lambda) = T0 - lambda
// Sigma and the eigenpairs (E, x) of the last evaluation, the vectors move as
// dx_m = sum_{n != m} x_n 2 p_nm / (E_m - E_n), p_nm = y_n . y_m (y, w: lower
// and upper halves).  Pairs of positive states cancel, so with the
// positive (p) and negative (n) halves Y_p, Y_n, W_p, W_n and
//   C[n][m] = 2 p_nm / (E_m - E_n)      (m > 0 > n)
//   d rho_++ / d lambda = Z + Z^T,  Z = Y_n C Y_p^T
//   d kappa_-+ / d lambda = Y_n C W_p^T + Y_p C^T W_n^T,
// whose trace gives back dN/dlambda = 8 sum p_nm^2 / (E_m - E_n).
__global__ void k_taylor_coef(const double* __restrict__ P, const double* __restrict__ w,
                              long wstride, const int* __restrict__ hsz, int hmax,
                              double* __restrict__ C) {
    const int b = blockIdx.y, h = hsz[b];
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= h * h) return;
    const int n = t / h, m = t % h;
    const long o = (long)b * hmax * hmax + (long)n * hmax + m;
    C[o] = 2.0 * P[o] / (w[b * wstride + h + m] - w[b * wstride + n]);
}

// rho += dl (Z + Z^T) in both diagonal blocks, kappa_-+ += dl K and
// kappa_+- -= dl K^T, dl = the isospin's step (0: converged already)
__global__ void k_taylor_update(const double* __restrict__ Z, const double* __restrict__ K,
                                const int* __restrict__ hsz, int hmax, int nmax,
                                const double* __restrict__ dls, double* __restrict__ rho,
                                double* __restrict__ kappa) {
    const int b = blockIdx.y, h = hsz[b], N = 2 * h;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const double dl = dls[b / 2];
    if (t >= h * h || dl == 0.0) return;
    const int r = t / h, s = t % h;
    const double* Zb = Z + (long)b * hmax * hmax;
    const double dr = Zb[r * hmax + s] + Zb[s * hmax + r];
    const double dk = K[(long)b * hmax * hmax + r * hmax + s];
    double* R = rho + (long)b * nmax * nmax;
    double* Kp = kappa + (long)b * nmax * nmax;
    R[(long)r * N + s] += dl * dr;
    R[(long)(h + r) * N + h + s] += dl * dr;
    Kp[(long)(h + r) * N + s] += dl * dk;
    Kp[(long)s * N + h + r] -= dl * dk;
}

// Quasiparticle energies moved with the same step: dE_m / d lambda =
// -x_m^T Sigma x_m = 2 |y_m|^2 - 1 (y: lower half of the vector), so that the
// spectrum left behind belongs to the final lambda, as an evaluation there
// would report it (to O(dl^2)).
__global__ void k_taylor_energies(const double* __restrict__ X, const int* __restrict__ hsz,
                                  int nmax, long wstride, const double* __restrict__ dls,
                                  double* __restrict__ w) {
    const int b = blockIdx.y, h = hsz[b], N = 2 * h;
    const int col = blockIdx.x * blockDim.x + threadIdx.x;
    const double dl = dls[b / 2];
    if (col >= N || dl == 0.0) return;
    const double* Xb = X + (long)b * nmax * nmax;
    double s = 0.0;
    for (int r = h; r < N; ++r) {
        const double y = Xb[(long)r * nmax + col];
        s = fma(y, y, s);
    }
    w[(long)b * wstride + col] += dl * (2.0 * s - 1.0);
}

// rho_++ blocks into the eigensolver batch (leading dimension hmax); HF
// occupations 2 rho_ii (HFBOccupations, src/HFB.f90:3519-3527)
__global__ void k_copy_rpp(const double* __restrict__ rho, const int* __restrict__ hsz,
                           const int* __restrict__ members, int hmax, int nmax,
                           double* __restrict__ Rpp, double* __restrict__ hf_occ) {
    const int b = blockIdx.y;
    const int h = hsz[b], N = 2 * h;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= h * h) return;
    const int r = t / h, s = t % h;
    const double x = rho[(long)b * nmax * nmax + (long)r * N + s];
    Rpp[(long)b * hmax * hmax + (long)r * hmax + s] = x;
    if (r == s) hf_occ[members[b * hmax + r]] = 2.0 * x;
}

// canonical transformation (|x| < 1e-11 -> 0, DiagonaliseRhoHFB) and the
// canonical occupations 2 v^2 (clamped as HFBOccupations does), with the
// dispersion partials sum v2 (2 - v2) per block.
__global__ void __launch_bounds__(kThreads)
k_occupations(const double* __restrict__ X, const double* __restrict__ w,
              const int* __restrict__ hsz, const int* __restrict__ cstart, int hmax,
              double* __restrict__ cantr, double* __restrict__ can_occ, double* __restrict__ scal,
              int* __restrict__ flags) {
    __shared__ double red[32];
    const int b = blockIdx.x;
    const int h = hsz[b];
    for (int t = threadIdx.x; t < h * h; t += kThreads) {
        const int r = t / h, C = t % h;
        const double x = X[(long)b * hmax * hmax + (long)r * hmax + C];
        cantr[(long)b * hmax * hmax + t] = fabs(x) < 1e-11 ? 0.0 : x;
    }
    double part = 0.0, omax = 0.0;
    for (int C = threadIdx.x; C < h; C += kThreads) {
        double o = w[(long)b * hmax + C];
        omax = fmax(omax, o);
        if (o > 1.0 + 1e-5) atomicExch(flags + 3, 1);
        if (o < -0.1) o += 2.0;
        if (o < 0.0) o = 0.0;
        if (o > 1.0) o = 1.0;
        o = 2.0 * o;
        can_occ[cstart[b] + C] = o;
        part += o * (2.0 - o);
    }
    const double s = cta_sum(part, red);
    for (int o = 16; o > 0; o >>= 1) omax = fmax(omax, __shfl_xor_sync(0xffffffffu, omax, o));
    __syncthreads();
    if (threadIdx.x % 32 == 0) red[threadIdx.x / 32] = omax;
    __syncthreads();
    if (threadIdx.x == 0) {
        double m = 0.0;
        for (int k = 0; k < kThreads / 32; ++k) m = fmax(m, red[k]);
        scal[4 + b] = s;
        scal[8 + b] = m;   // largest canonical occupation v^2 of the block
    }
}

// rho/kappa mixing with the previous iteration's matrices (HFBMix) and the
// block pairing energy -sum Delta_ij kappa_ij (HFBEnergy) with mixed kappa.
__global__ void __launch_bounds__(kThreads)
k_hfb_mix(double* rho, double* kappa, double* oldrho, double* oldkappa, const double* delta,
          const int* hsz, int nmax, double mix, int mix_rho, int mix_kappa, double* scal,
          double* __restrict__ bak_rho, double* __restrict__ bak_kappa) {
    __shared__ double red[32];
    const int b = blockIdx.x;
    const int N = 2 * hsz[b];
    const long o0 = (long)b * nmax * nmax;
    double part = 0.0;
    for (int t = threadIdx.x; t < N * N; t += kThreads) {
        const long o = o0 + t;
        double r = rho[o], k = kappa[o];
        const double ro = oldrho[o], ko = oldkappa[o];
        bak_rho[o] = ro;     // the history as it was, for a redo of the step
        bak_kappa[o] = ko;
        if (mix_rho) r = mix * r + (1.0 - mix) * ro;
        if (mix_kappa) k = mix * k + (1.0 - mix) * ko;
        rho[o] = r;
        kappa[o] = k;
        oldrho[o] = r;
        oldkappa[o] = k;
        part = part - delta[o] * k;
    }
    const double s = cta_sum(part, red);
    if (threadIdx.x == 0) scal[b] = s;
}

}  // namespace

// Block structure, device buffers, canonical quantum numbers, kappa guess.
int hfb_prepare(mg_ctx* c) {
    Hfb& H = c->hfb;
    Basis& B = c->bas[MG_HF_BASIS];
    const int nwt = c->p.nwt;
    std::vector<int> lists[4];
    for (int i = 0; i < nwt; ++i) {
        if (B.h_qn[4 * i + 2] != 1 || B.h_qn[4 * i + 3] != 1) return MG_ERR_ARG;
        const int it = (B.h_qn[4 * i] + 3) / 2 - 1, P = (B.h_qn[4 * i + 1] + 1) / 2;
        lists[it * 2 + P].push_back(i);
    }
    int hmax = 1;
    for (int b = 0; b < 4; ++b) {
        H.hsz_h[b] = (int)lists[b].size();
        H.parity_h[b] = (b % 2) ? 1 : -1;
        hmax = std::max(hmax, H.hsz_h[b]);
    }
    if (2 * hmax > kEigMax) return MG_ERR_ARG;  // block matrices of the batched eigensolver
    H.hmax = hmax;
    H.nmax = 2 * hmax;
    H.members_h.assign(4 * hmax, 0);
    std::vector<int> cst(4), nT(4);
    int acc = 0;
    for (int b = 0; b < 4; ++b) {
        for (int j = 0; j < H.hsz_h[b]; ++j) H.members_h[b * hmax + j] = lists[b][j];
        cst[b] = acc;
        acc += H.hsz_h[b];
        nT[b] = 2 * H.hsz_h[b];
    }
    const long nm2 = 4L * H.nmax * H.nmax, V = c->V;
    auto A = [&](double** p, long n) {
        return cudaMalloc(p, std::max(1L, n) * sizeof(double)) == cudaSuccess &&
               cudaMemset(*p, 0, std::max(1L, n) * sizeof(double)) == cudaSuccess;
    };
    H.gchunk = std::max(1, (2 * c->num_sms) / 4);
    bool ok = A(&H.rho, nm2) && A(&H.kappa, nm2) && A(&H.oldrho, nm2) && A(&H.oldkappa, nm2) &&
              A(&H.oldrho_bak, nm2) && A(&H.oldkappa_bak, nm2) &&
              A(&H.delta, nm2) && A(&H.T, nm2) && A(&H.Rpp, 4L * hmax * hmax) &&
              A(&H.dfac, 2 * V) && A(&H.pcut, nwt) && A(&H.ktil, 4L * hmax * hmax) &&
              A(&H.fpart, 8 * V) && A(&H.fre, 2 * V) && A(&H.fim, 2 * V) &&
              A(&H.gpart, 4L * H.gchunk * hmax * hmax) && A(&H.cantr, 4L * hmax * hmax) &&
              A(&H.occ, 4L * hmax) && A(&H.fermi_d, 2) && A(&H.dl_d, 2) && A(&H.trace_d, 16) && A(&H.dpart, 4L * hmax) && A(&H.scal_d, 16) &&
              cudaMalloc(&H.members, 4 * hmax * sizeof(int)) == cudaSuccess &&
              cudaMalloc(&H.hsz, 4 * sizeof(int)) == cudaSuccess &&
              cudaMalloc(&H.nsz_T, 4 * sizeof(int)) == cudaSuccess &&
              cudaMalloc(&H.cstart, 4 * sizeof(int)) == cudaSuccess &&
              cudaMallocHost(&H.h_pinned, 32 * sizeof(double)) == cudaSuccess;
    if (!ok) return MG_ERR_CUDA;
    MG_CUDA(cudaMemcpy(H.members, H.members_h.data(), 4 * hmax * sizeof(int), cudaMemcpyHostToDevice));
    MG_CUDA(cudaMemcpy(H.hsz, H.hsz_h, 4 * sizeof(int), cudaMemcpyHostToDevice));
    MG_CUDA(cudaMemcpy(H.nsz_T, nT.data(), 4 * sizeof(int), cudaMemcpyHostToDevice));
    MG_CUDA(cudaMemcpy(H.cstart, cst.data(), 4 * sizeof(int), cudaMemcpyHostToDevice));
    MG_TRY(pairing_set_smem(c));
    MG_TRY(eig_setup(c, H.eT, 4, H.nmax, H.nsz_T, H.T, (long)H.nmax * H.nmax, H.nmax));
    H.eT.skip_tol = 1e-10;
    MG_TRY(eig_setup(c, H.eR, 4, hmax, H.hsz, H.Rpp, (long)hmax * hmax, hmax));
    H.nref = 3;
    {
        const long hh = 4L * hmax * hmax;
        if (!(A(&H.tP, hh) && A(&H.tC, hh) && A(&H.tT1, hh) && A(&H.tT2, hh) && A(&H.tZ, hh) &&
              A(&H.tK, hh)))
            return MG_ERR_CUDA;
        std::vector<GemmDesc> d(24);
        const int nm = H.nmax;
        for (int b = 0; b < 4; ++b) {
            const int h = H.hsz_h[b];
            const double* X = H.eT.X + (long)b * nm * nm;
            const double *Yn = X + (long)h * nm, *Yp = X + (long)h * nm + h, *Wn = X, *Wp = X + h;
            const long o = (long)b * hmax * hmax;
            // P = Y_n^T Y_p
            d[b] = GemmDesc{Yn, Yp, H.tP + o, h, h, h, nm, nm, hmax, 1, 0, 1.0, 0.0, b, 0};
            // T1 = Y_n C, T2 = Y_p C^T
            d[4 + 2 * b] = GemmDesc{Yn, H.tC + o, H.tT1 + o, h, h, h, nm, hmax, hmax, 0, 0, 1.0, 0.0, b, 0};
            d[5 + 2 * b] = GemmDesc{Yp, H.tC + o, H.tT2 + o, h, h, h, nm, hmax, hmax, 0, 1, 1.0, 0.0, b, 0};
            // Z = T1 Y_p^T, K = T1 W_p^T
            d[12 + 2 * b] = GemmDesc{H.tT1 + o, Yp, H.tZ + o, h, h, h, hmax, nm, hmax, 0, 1, 1.0, 0.0, b, 0};
            d[13 + 2 * b] = GemmDesc{H.tT1 + o, Wp, H.tK + o, h, h, h, hmax, nm, hmax, 0, 1, 1.0, 0.0, b, 0};
            // K += T2 W_n^T
            d[20 + b] = GemmDesc{H.tT2 + o, Wn, H.tK + o, h, h, h, hmax, nm, hmax, 0, 1, 1.0, 1.0, b, 0};
        }
        MG_CUDA(cudaMalloc(&H.d_taylor, d.size() * sizeof(GemmDesc)));
        MG_CUDA(cudaMemcpy(H.d_taylor, d.data(), d.size() * sizeof(GemmDesc), cudaMemcpyHostToDevice));
    }
    // canonical basis quantum numbers: block order (it, parity -1 then +1)
    std::vector<int> cqn(4 * nwt);
    for (int b = 0; b < 4; ++b)
        for (int j = 0; j < H.hsz_h[b]; ++j) {
            int* q = &cqn[4 * (cst[b] + j)];
            q[0] = 2 * (b / 2) - 1;
            q[1] = H.parity_h[b];
            q[2] = 1;
            q[3] = 1;
        }
    MG_TRY(mg_upload_spinors(c, MG_CAN_BASIS, nullptr, cqn.data(), 0, nwt));
    if (H.restart_pending) {
        // RhoHFB / KappaHFB read from a wavefunction file (TransformHFBMatrices
        // with matching symmetries copies them, src/Transform.f90:1056-1064);
        // GuessKappa still overrides kappa afterwards, as the pairing
        // initialisation guesses after the read (src/Pairing.f90:800-803)
        for (int b = 0; b < 4; ++b)
            if (H.restart_n[b] != 2 * H.hsz_h[b]) return MG_ERR_STATE;
        std::vector<double> r(nm2, 0.0), k(nm2, 0.0);
        for (int b = 0; b < 4; ++b) {
            const size_t N2 = (size_t)H.restart_n[b] * H.restart_n[b];
            std::copy(H.restart_rho[b].begin(), H.restart_rho[b].begin() + N2,
                      r.begin() + (long)b * H.nmax * H.nmax);
            std::copy(H.restart_kappa[b].begin(), H.restart_kappa[b].begin() + N2,
                      k.begin() + (long)b * H.nmax * H.nmax);
            H.restart_rho[b].clear();
            H.restart_kappa[b].clear();
        }
        MG_CUDA(cudaMemcpy(H.rho, r.data(), nm2 * sizeof(double), cudaMemcpyHostToDevice));
        MG_CUDA(cudaMemcpy(H.kappa, k.data(), nm2 * sizeof(double), cudaMemcpyHostToDevice));
        H.restart_pending = false;
    }
    // GuessHFBMatrices case(2) with time reversal: kappa(i, i+h) = -1/4,
    // kappa(i+h, i) = +1/4
    if (H.pp.guess_kappa) {
        std::vector<double> k(nm2, 0.0);
        for (int b = 0; b < 4; ++b) {
            const int h = H.hsz_h[b], N = 2 * h;
            for (int i = 0; i < h; ++i) {
                k[(long)b * H.nmax * H.nmax + (long)i * N + i + h] = -0.25;
                k[(long)b * H.nmax * H.nmax + (long)(i + h) * N + i] = 0.25;
            }
        }
        MG_CUDA(cudaMemcpy(H.kappa, k.data(), nm2 * sizeof(double), cudaMemcpyHostToDevice));
        H.pp.guess_kappa = 0;
    }
    H.ready = true;
    return MG_OK;
}

void hfb_free(mg_ctx* c) {
    Hfb& H = c->hfb;
    if (H.dl_d) cudaFree(H.dl_d);
    if (H.oldrho_bak) cudaFree(H.oldrho_bak);
    if (H.oldkappa_bak) cudaFree(H.oldkappa_bak);
    for (double* p : {H.rho, H.kappa, H.oldrho, H.oldkappa, H.delta, H.qe, H.dfac, H.pcut, H.ktil,
                      H.fpart, H.fre, H.fim, H.gpart, H.cantr, H.occ, H.fermi_d, H.trace_d, H.dpart,
                      H.scal_d, H.T, H.Rpp, H.tP, H.tC, H.tT1, H.tT2, H.tZ, H.tK})
        if (p) cudaFree(p);
    if (H.d_taylor) cudaFree(H.d_taylor);
    for (int* p : {H.members, H.hsz, H.cstart, H.nsz_T})
        if (p) cudaFree(p);
    if (H.h_pinned) cudaFreeHost(H.h_pinned);
    for (cudaGraphExec_t& g : H.eval_graph)
        if (g) cudaGraphExecDestroy(g);
    for (cudaGraphExec_t& g : H.can_graph) {
        if (g) cudaGraphExecDestroy(g);
        g = nullptr;
    }
    if (H.taylor_graph) cudaGraphExecDestroy(H.taylor_graph);
    H.taylor_graph = nullptr;
    eig_free(H.eT);
    eig_free(H.eR);
    gradient_hfb_free(H.grad);
    H.grad = nullptr;
}

// One particle-number evaluation at lambda (both isospins): T(lambda),
// eigen-decomposition, rho, kappa, block traces and dN/dlambda.  The first
// evaluation of a pairing step (T changed with the mean fields) starts from
// an FP32 Jacobi seed warm-started from the previous vectors; the later ones
// (only lambda moved) refine the previous vectors directly, up to four steps,
// a matrix whose off-diagonal part fell below 1e-10 of its norm skipping the
// rest.  An FP64 Jacobi polish of X^T T X then rotates the pairs the
// refinement leaves coupled inside its clusters (a quasiparticle pair close
// to zero energy decides the particle number).  If before the last step
// states of opposite sign were still mixed by an angle above kRefineTol, the
// evaluation is redone from the Jacobi seed.
// The launches of one evaluation after lambda is on the device: T(lambda),
// eigen-decomposition, rho, kappa, dN/dlambda, block traces.
static int eval_launches(mg_ctx* c, int seed) {
    Hfb& H = c->hfb;
    k_build_T<<<dim3(div_up(H.nmax * H.nmax, kThreads), 4), kThreads, 0, c->stream>>>(
        H.delta, c->bas[MG_HF_BASIS].e, H.members, H.hsz, H.hmax, H.nmax, H.fermi_d, H.T);
    MG_LAUNCHED(c);
    MG_TRY(eig_batched(c, H.eT, seed, seed == kSeedRefine ? 4 : H.nref, true));
    k_rho_kappa<<<dim3(div_up(H.hmax * H.hmax, kThreads), 4), kThreads, 0, c->stream>>>(
        H.eT.X, H.hsz, H.nmax, H.rho, H.kappa);
    MG_LAUNCHED(c);
    k_dn_dlambda<<<dim3(H.hmax, 4), 128, 0, c->stream>>>(H.eT.X, H.eT.w, H.hsz, H.nmax, H.dpart);
    MG_LAUNCHED(c);
    k_trace<<<4, 128, 0, c->stream>>>(H.rho, H.hsz, H.nmax, H.dpart, H.eT.emax, H.eT.w,
                                      H.eT.wstride, H.trace_d);
    MG_LAUNCHED(c);
    return MG_OK;
}

// One evaluation's launches.  The warm seeds (every evaluation after the
// first pairing step) replay a CUDA graph captured on first use: ~40 small
// launches become one, the early exits inside stay device-side decisions.
static int eval_run(mg_ctx* c, int seed) {
    Hfb& H = c->hfb;
    if (seed == kSeedCold || H.no_graph) return eval_launches(c, seed);
    // the mixed and FP64 forms launch different polish kernels: recapture on
    // a switch of form
    if (H.eval_graph[seed] && H.eval_graph_prec[seed] != c->cur_precision) {
        cudaGraphExecDestroy(H.eval_graph[seed]);
        H.eval_graph[seed] = nullptr;
    }
    if (!H.eval_graph[seed]) {
        if (cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
            cudaGetLastError();    // e.g. the legacy default stream: launch directly
            H.no_graph = true;
            return eval_launches(c, seed);
        }
        const long long l0 = c->launches;
        const int st = eval_launches(c, seed);
        cudaGraph_t graph = nullptr;
        const cudaError_t ce = cudaStreamEndCapture(c->stream, &graph);
        if (st != MG_OK || ce != cudaSuccess) {
            if (graph) cudaGraphDestroy(graph);
            return st != MG_OK ? st : MG_ERR_CUDA;
        }
        const cudaError_t ie = cudaGraphInstantiate(&H.eval_graph[seed], graph, 0);
        cudaGraphDestroy(graph);
        if (ie != cudaSuccess) {
            H.eval_graph[seed] = nullptr;
            return MG_ERR_CUDA;
        }
        H.eval_graph_launches[seed] = c->launches - l0;
        H.eval_graph_prec[seed] = c->cur_precision;
        c->launches = l0;
    }
    MG_CUDA(cudaGraphLaunch(H.eval_graph[seed], c->stream));
    c->launches += H.eval_graph_launches[seed];
    return MG_OK;
}

// seed < 0: the Jacobi warm seed for a first evaluation (or a far jump of
// lambda), refinement of the previous vectors otherwise.
static int hfb_evaluate(mg_ctx* c, const double* lam, double* N_out, double* dN_out,
                        bool first, int seed = -1) {
    Hfb& H = c->hfb;
    double* hp = H.h_pinned;
    hp[24] = lam[0];
    hp[25] = lam[1];
    MG_CUDA(cudaMemcpyAsync(H.fermi_d, hp + 24, 2 * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    if (seed < 0) seed = !H.eT.have_vectors ? kSeedCold : first ? kSeedJacobiWarm : kSeedRefine;
    for (int attempt = 0; attempt < 2; ++attempt) {
        MG_TRY(eval_run(c, seed));
        H.eT.have_vectors = true;
        MG_CUDA(cudaMemcpyAsync(hp, H.trace_d, 16 * sizeof(double), cudaMemcpyDeviceToHost,
                                c->stream));
        MG_CUDA(cudaStreamSynchronize(c->stream));
        const double em = std::max(std::max(hp[8], hp[9]), std::max(hp[10], hp[11]));
        if (seed != kSeedRefine || em <= kRefineTol) break;
        seed = kSeedJacobiWarm;   // T is rebuilt identically (same lambda)
        ++H.reseeds;
    }
    N_out[0] = hp[0] + hp[1] - c->p.neutrons;
    N_out[1] = hp[2] + hp[3] - c->p.protons;
    dN_out[0] = hp[4] + hp[5];
    dN_out[1] = hp[6] + hp[7];
    H.qp_gap[0] = std::min(hp[12], hp[13]);
    H.qp_gap[1] = std::min(hp[14], hp[15]);
    if (std::isnan(N_out[0]) || std::isnan(N_out[1])) return MG_ERR_NAN;
    return MG_OK;
}

// One evaluation at lambda from the Jacobi seed (the gradient solver's first
// U and V).
int hfb_evaluate_at(mg_ctx* c, const double* lam, double* N_out, double* dN_out) {
    return hfb_evaluate(c, lam, N_out, dN_out, true);
}

// rho, kappa and the quasiparticle energies moved to lambda + dl from the
// eigen-decomposition of the last evaluation (first order in dl).
static int taylor_launches(mg_ctx* c) {
    Hfb& H = c->hfb;
    const int hmax = H.hmax;
    const dim3 g(div_up(hmax * hmax, kThreads), 4);
    const bool df = c->cur_precision == MG_MIXED;   // the mixed form's eigen GEMMs
    MG_TRY(gemm_batched(c, H.d_taylor, 4, hmax, df));
    k_taylor_coef<<<g, kThreads, 0, c->stream>>>(H.tP, H.eT.w, H.eT.wstride, H.hsz, hmax, H.tC);
    MG_LAUNCHED(c);
    MG_TRY(gemm_batched(c, H.d_taylor + 4, 8, hmax, df));
    MG_TRY(gemm_batched(c, H.d_taylor + 12, 8, hmax, df));
    MG_TRY(gemm_batched(c, H.d_taylor + 20, 4, hmax, df));
    k_taylor_update<<<g, kThreads, 0, c->stream>>>(H.tZ, H.tK, H.hsz, hmax, H.nmax, H.dl_d,
                                                  H.rho, H.kappa);
    MG_LAUNCHED(c);
    k_taylor_energies<<<dim3(div_up(H.nmax, 128), 4), 128, 0, c->stream>>>(
        H.eT.X, H.hsz, H.nmax, H.eT.wstride, H.dl_d, H.eT.w);
    MG_LAUNCHED(c);
    return MG_OK;
}

// The steps dl go to the device (from the pinned block; the host writes it
// once per pairing step, several synchronisations before it is reused) and
// the seven launches replay as one CUDA graph.
static int taylor_finish(mg_ctx* c, const double dl[2]) {
    Hfb& H = c->hfb;
    double* hp = H.h_pinned;
    hp[26] = dl[0];
    hp[27] = dl[1];
    MG_CUDA(cudaMemcpyAsync(H.dl_d, hp + 26, 2 * sizeof(double), cudaMemcpyHostToDevice,
                            c->stream));
    if (H.no_graph) return taylor_launches(c);
    if (H.taylor_graph && H.taylor_graph_prec != c->cur_precision) {
        cudaGraphExecDestroy(H.taylor_graph);   // the two forms launch different GEMMs
        H.taylor_graph = nullptr;
    }
    if (!H.taylor_graph) {
        if (cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
            cudaGetLastError();
            H.no_graph = true;
            return taylor_launches(c);
        }
        const long long l0 = c->launches;
        const int st = taylor_launches(c);
        cudaGraph_t graph = nullptr;
        const cudaError_t ce = cudaStreamEndCapture(c->stream, &graph);
        if (st != MG_OK || ce != cudaSuccess) {
            if (graph) cudaGraphDestroy(graph);
            return st != MG_OK ? st : MG_ERR_CUDA;
        }
        const cudaError_t ie = cudaGraphInstantiate(&H.taylor_graph, graph, 0);
        cudaGraphDestroy(graph);
        if (ie != cudaSuccess) {
            H.taylor_graph = nullptr;
            return MG_ERR_CUDA;
        }
        H.taylor_graph_launches = c->launches - l0;
        H.taylor_graph_prec = c->cur_precision;
        c->launches = l0;
    }
    MG_CUDA(cudaGraphLaunch(H.taylor_graph, c->stream));
    c->launches += H.taylor_graph_launches;
    return MG_OK;
}

// Start of a Fermi search: the last Fermi energies, extrapolated along the
// iterations by the polynomial through the last k converged ones (degree
// k - 1, up to 5), as long as the sequence moves by less than kFarStep per
// iteration.  The root does not depend on it; a closer start lets one
// evaluation and the first-order finish complete the search.  On the roots
// of a 280-iteration run at 24^3, nwt=160, the median miss over iterations
// 50-100 was 6.9e-7 MeV for the cubic and 6.7e-9 for the quintic (degrees
// above five amplify the iterations' rounding-level wobble).
static void start_guess(const Hfb& H, double lam[2]) {
    // binomial coefficients: the degree k - 1 extrapolation is
    // sum_j (-1)^j C(k, j + 1) l_j
    static const double kC[7][6] = {{0, 0, 0, 0, 0, 0},        {1, 0, 0, 0, 0, 0},
                                    {2, -1, 0, 0, 0, 0},       {3, -3, 1, 0, 0, 0},
                                    {4, -6, 4, -1, 0, 0},      {5, -10, 10, -5, 1, 0},
                                    {6, -15, 20, -15, 6, -1}};
    for (int it = 0; it < 2; ++it) {
        const double l[6] = {H.fermi[it],       H.fermi_prev[it],  H.fermi_old[0][it],
                             H.fermi_old[1][it], H.fermi_old[2][it], H.fermi_old[3][it]};
        int k = std::min(H.n_solved, 6);
        for (int j = 1; j < k; ++j)
            if (std::fabs(l[j - 1] - l[j]) >= kFarStep) k = j;
        k = std::max(k, 1);
        double p = 0.0;
        for (int j = 0; j < k; ++j) p += kC[k][j] * l[j];
        lam[it] = p;
    }
}

// ---- particle-number root finder: Newton with the analytic dN/dlambda,
// safeguarded by the bracket the evaluations build (bisection when a step
// leaves it, steps clamped to 5 MeV).  On return lam holds the Fermi
// energies, f the particle-number deviations, conv which isospins met
// FermiPrec; *first_order tells whether rho and kappa took the last step to
// first order.
static int fermi_newton(mg_ctx* c, double lam[2], double f[2], bool conv[2], int* evals_out,
                        bool* first_order_out) {
    Hfb& H = c->hfb;
    const double prec = H.pp.fermi_prec;
    int evals = 0;
    // start from the last Fermi energies extrapolated along the iterations
    // (the root is the same; the first evaluation only lands closer to it)
    double fp[2];
    start_guess(H, lam);
    // The first evaluation starts from the FP32 Jacobi seed, except in the
    // mixed form once the search has settled (the last step took one
    // evaluation and the first-order finish): the previous vectors then
    // refine in place in double-float, cheaper than the seed there (a
    // refinement that falls short re-seeds itself).  In FP64 the refinement
    // steps run on the slow FP64 pipe and the seed stays the cheaper start.
    const bool refine = c->cur_precision == MG_MIXED && H.settled;
    MG_TRY(hfb_evaluate(c, lam, f, fp, !refine));
    ++evals;
    conv[0] = std::fabs(f[0]) < prec;
    conv[1] = std::fabs(f[1]) < prec;
    double lo[2] = {0, 0}, hi[2] = {0, 0};
    bool has_lo[2] = {false, false}, has_hi[2] = {false, false};
    auto bracket = [&](int it) {
        if (f[it] < 0) { lo[it] = lam[it]; has_lo[it] = true; }
        else { hi[it] = lam[it]; has_hi[it] = true; }
    };
    bracket(0);
    bracket(1);
    const int maxit = H.pp.max_iter > 0 ? H.pp.max_iter : 50;
    bool first_order = false;
    for (int k = 0; k < maxit && !(conv[0] && conv[1]); ++k) {
        double dl[2] = {0.0, 0.0};
        bool newton[2] = {true, true};
        for (int it = 0; it < 2; ++it) {
            if (conv[it]) continue;
            double step = fp[it] > 1e-12 ? -f[it] / fp[it] : (f[it] < 0 ? 0.5 : -0.5);
            newton[it] = fp[it] > 1e-12 && std::fabs(step) <= 5.0;
            step = std::max(-5.0, std::min(5.0, step));
            double next = lam[it] + step;
            if (has_lo[it] && has_hi[it] && !(next > lo[it] && next < hi[it])) {
                next = 0.5 * (lo[it] + hi[it]);
                newton[it] = false;
            }
            dl[it] = next - lam[it];
            lam[it] = next;
        }
        // Last Newton step: when every remaining step is a plain Newton step
        // below kTaylorStep, rho and kappa move to the new lambda to first
        // order from the evaluation just made.  N(lambda) then misses N0 by
        // ~N'' dl^2 / 2 (~1e-14 at this step), the same as an evaluation at
        // the new lambda would report; no eigen-decomposition is redone.
        bool taylor = true;
        first_order = false;
        const bool recent = c->iteration - H.npp_iter <= kCurvatureAge;
        for (int it = 0; it < 2; ++it) {
            double dl_max = kTaylorStep;
            if (recent)
                dl_max = std::min(kTaylorMax, std::max(kTaylorStep,
                                  std::sqrt(kCurvatureBudget * prec / std::max(H.npp[it], 1e-6))));
            taylor = taylor && (conv[it] || (newton[it] && std::fabs(dl[it]) <= dl_max &&
                                             std::fabs(dl[it]) <= kTaylorGap * H.qp_gap[it]));
        }
        if (taylor) {
            MG_TRY(taylor_finish(c, dl));
            ++H.taylor_steps;
            first_order = true;
            for (int it = 0; it < 2; ++it) {
                if (conv[it]) continue;
                f[it] += fp[it] * dl[it];
                conv[it] = true;
            }
            break;
        }
        // a far move of lambda (a search that has not settled) starts from
        // the Jacobi warm seed: refinement alone is for nearby vectors
        const bool far = std::fabs(dl[0]) > kFarStep || std::fabs(dl[1]) > kFarStep;
        const double fp_prev[2] = {fp[0], fp[1]};
        MG_TRY(hfb_evaluate(c, lam, f, fp, far));
        ++evals;
        // curvature of N(lambda) from the two evaluations' slopes, over local
        // steps only (a bisection step's secant is not the curvature there)
        bool est = false;
        for (int it = 0; it < 2; ++it)
            if (std::fabs(dl[it]) > 1e-9 && std::fabs(dl[it]) <= 1e-3) {
                H.npp[it] = std::fabs((fp[it] - fp_prev[it]) / dl[it]);
                est = true;
            }
        if (est) H.npp_iter = c->iteration;
        for (int it = 0; it < 2; ++it) {
            if (conv[it]) continue;
            if (std::fabs(f[it]) < prec) { conv[it] = true; continue; }
            bracket(it);
        }
    }
    *evals_out = evals;
    *first_order_out = first_order;
    H.settled = evals == 1 && first_order;
    return MG_OK;
}

// ---- the reference's particle-number search (HFBFindFermiEnergyBroyden,
// src/HFB.f90:1849-2161, FermiSolver 'BROYDEN'): a second evaluation 0.01 MeV
// above the start gives the secant slope, then damped (x 0.5) quasi-Newton
// steps with Broyden's update of the slope, up to HFBIter of them; the slope
// is replaced by +-1/0.99 when |J| < 0.001.  The same particle-number
// equation and tolerance as fermi_newton, every step a full evaluation; it
// follows the reference's iterates, including where they stop short of the
// tolerance.
static int fermi_broyden(mg_ctx* c, double lam[2], double f[2], bool conv[2], int* evals_out) {
    Hfb& H = c->hfb;
    const double prec = H.pp.fermi_prec;
    int evals = 0;
    double fp[2], hist[2] = {H.fermi[0] + 0.01, H.fermi[1] + 0.01}, NX[2], J[2];
    double upd[2] = {0.0, 0.0}, norm[2] = {1.0, 1.0};
    lam[0] = H.fermi[0];
    lam[1] = H.fermi[1];
    MG_TRY(hfb_evaluate(c, lam, f, fp, true));
    ++evals;
    for (int it = 0; it < 2; ++it) conv[it] = std::fabs(f[it]) < prec;
    MG_TRY(hfb_evaluate(c, hist, NX, fp, false));
    ++evals;
    for (int it = 0; it < 2; ++it) J[it] = (f[it] - NX[it]) / (lam[it] - hist[it]);
    const double step = 0.5;
    const int maxit = H.pp.max_iter > 0 ? H.pp.max_iter : 50;
    for (int iter = 1; iter <= maxit; ++iter) {
        double invJ[2];
        for (int it = 0; it < 2; ++it)
            invJ[it] = std::fabs(J[it]) < 0.001 ? (J[it] >= 0 ? 0.99 : -0.99) : 1.0 / J[it];
        for (int it = 0; it < 2; ++it) {
            if (conv[it]) continue;
            upd[it] = -invJ[it] * f[it];
            norm[it] = upd[it] * upd[it];
        }
        for (int it = 0; it < 2; ++it) upd[it] = step * upd[it];
        bool far = false;
        for (int it = 0; it < 2; ++it) {
            if (conv[it]) continue;
            hist[it] = lam[it];
            lam[it] = lam[it] + upd[it];
            far = far || std::fabs(upd[it]) > kFarStep;
        }
        MG_TRY(hfb_evaluate(c, lam, f, fp, far));
        ++evals;
        for (int it = 0; it < 2; ++it)
            if (std::fabs(f[it]) < prec) conv[it] = true;
        if (conv[0] && conv[1]) break;
        if (iter > 1)
            for (int it = 0; it < 2; ++it) {
                if (conv[it]) continue;
                J[it] = J[it] + f[it] * upd[it] / norm[it];
            }
    }
    *evals_out = evals;
    return MG_OK;
}

// FermiBrent (src/HFB.f90:2273-2487): Brent's root search on N(lambda) - N0
// per isospin from the bracket [a, b] (a == b: nothing to search), both
// isospins evaluated together at b; the tolerance is prec on lambda.
static int fermi_brent(mg_ctx* c, double a[2], double b[2], double fa[2], double fb[2],
                       double prec, bool found[2], int* evals) {
    double cc[2], fc[2], d[2] = {0.0, 0.0}, e[2] = {0.0, 0.0}, dN[2];
    for (int it = 0; it < 2; ++it) {
        found[it] = a[it] == b[it];
        if (!found[it] && fa[it] * fb[it] > 0.0) return MG_ERR_STATE;   // not bracketed
        cc[it] = b[it];
        fc[it] = fb[it];
    }
    // each step shrinks the bracket by prec at least; the cap only guards
    // a non-finite bracket
    for (int iter = 0; iter < 100000 && !(found[0] && found[1]); ++iter) {
        for (int it = 0; it < 2; ++it) {
            if (found[it]) continue;
            if ((fb[it] > 0.0 && fc[it] > 0.0) || (fb[it] < 0.0 && fc[it] < 0.0)) {
                cc[it] = a[it];
                fc[it] = fa[it];
                d[it] = b[it] - a[it];
                e[it] = d[it];
            }
            if (std::fabs(fc[it]) < std::fabs(fb[it])) {
                a[it] = b[it];
                fa[it] = fb[it];
                b[it] = cc[it];
                fb[it] = fc[it];
                cc[it] = a[it];
                fc[it] = fa[it];
            }
            const double tol = prec, xm = 0.5 * (cc[it] - b[it]);
            if (std::fabs(xm) <= tol) {
                found[it] = true;
                continue;
            }
            if (std::fabs(e[it]) >= tol && std::fabs(fa[it]) > std::fabs(fb[it])) {
                const double sv = fb[it] / fa[it];
                double p, q;
                if (a[it] == cc[it]) {
                    p = 2.0 * xm * sv;
                    q = 1.0 - sv;
                } else {
                    const double qa = fa[it] / fc[it], r = fb[it] / fc[it];
                    p = sv * (2.0 * xm * qa * (qa - r) - (b[it] - a[it]) * (r - 1.0));
                    q = (qa - 1.0) * (r - 1.0) * (sv - 1.0);
                }
                if (p > 0.0) q = -q;
                p = std::fabs(p);
                if (2.0 * p < std::min(3.0 * xm * q - std::fabs(tol * q), std::fabs(e[it] * q))) {
                    e[it] = d[it];
                    d[it] = p / q;
                } else {
                    d[it] = xm;
                    e[it] = d[it];
                }
            } else {
                d[it] = xm;
                e[it] = d[it];
            }
            a[it] = b[it];
            fa[it] = fb[it];
            b[it] = b[it] + (std::fabs(d[it]) > tol ? d[it] : std::copysign(tol, xm));
        }
        MG_TRY(hfb_evaluate(c, b, fb, dN, false));
        ++*evals;
    }
    return MG_OK;
}

// HFBFindFermiEnergyBisection (src/HFB.f90:1074-1342, FermiSolver
// 'BISECTION', without LN and the emergency handling the reference keeps
// off): from the stored Fermi energies, step the boundary on the side of
// the root out by 0.01 MeV times the attempt (0.01, 0.03, 0.06, ...) until
// N - N0 changes sign, then Brent's method to prec on lambda.
static int fermi_bisection(mg_ctx* c, double lam[2], double f[2], bool conv[2], int* evals_out) {
    Hfb& H = c->hfb;
    const double prec = H.pp.fermi_prec;
    const double part[2] = {c->p.neutrons, c->p.protons};
    int evals = 0;
    double dN[2];
    for (int it = 0; it < 2; ++it) lam[it] = part[it] < 0.1 ? -100.0 : H.fermi[it];
    MG_TRY(hfb_evaluate(c, lam, f, dN, true));
    ++evals;
    conv[0] = conv[1] = false;
    if (std::fabs(f[0]) < prec && std::fabs(f[1]) < prec) {
        conv[0] = conv[1] = true;
        *evals_out = evals;
        return MG_OK;
    }
    double br[2][2], fa[2], fb[2];
    int idir[2], sig[2];
    bool notfound[2] = {true, true};
    for (int it = 0; it < 2; ++it) {
        br[0][it] = br[1][it] = lam[it];
        idir[it] = f[it] < 0.0 ? 1 : 0;
        sig[it] = f[it] < 0.0 ? 1 : -1;
    }
    for (int fail = 0;; ++fail) {
        for (int it = 0; it < 2; ++it)
            if (std::fabs(f[it]) < prec) notfound[it] = false;
        for (int it = 0; it < 2; ++it)
            if (notfound[it]) br[idir[it]][it] = br[idir[it]][it] + sig[it] * 0.01 * (fail + 1);
        MG_TRY(hfb_evaluate(c, br[0], fa, dN, false));
        MG_TRY(hfb_evaluate(c, br[1], fb, dN, false));
        evals += 2;
        for (int it = 0; it < 2; ++it)
            if (notfound[it] && fa[it] * fb[it] <= 0.0) notfound[it] = false;
        if (!notfound[0] && !notfound[1]) break;
        if (fail + 1 > 130) {   // the reference stops: no bracket within ~85 MeV
            *evals_out = evals;
            return MG_ERR_STATE;
        }
        for (int it = 0; it < 2; ++it)
            if (notfound[it]) br[1 - idir[it]][it] = br[idir[it]][it];
    }
    bool found[2];
    MG_TRY(fermi_brent(c, br[0], br[1], fa, fb, prec, found, &evals));
    for (int it = 0; it < 2; ++it) {
        lam[it] = br[1][it];
        f[it] = fb[it];
        conv[it] = found[it];
    }
    *evals_out = evals;
    return MG_OK;
}

// SolvePairing for HFB (src/Pairing.f90:743-890, PairingIter 1).
// The canonical-basis decomposition of the four rho_++ blocks.  From the
// second pairing step on it starts from last step's vectors (the Jacobi warm
// seed) and replays as one CUDA graph, like the evaluations of the Fermi
// search (recaptured when the precision form changes: the two forms launch
// different polish kernels).
static int canonical_eig(mg_ctx* c) {
    Hfb& H = c->hfb;
    if (!H.eR.have_vectors || H.no_graph) {
        return eig_batched(c, H.eR, H.eR.have_vectors ? kSeedJacobiWarm : kSeedCold, H.nref, true);
    }
    // as the Fermi search's first evaluation: the mixed form refines the
    // last vectors in place once the search has settled
    const int k = c->cur_precision == MG_MIXED && H.settled ? 1 : 0;
    const int seed = k ? kSeedRefine : kSeedJacobiWarm;
    cudaGraphExec_t& gr = H.can_graph[k];
    if (gr && H.can_graph_prec[k] != c->cur_precision) {
        cudaGraphExecDestroy(gr);
        gr = nullptr;
    }
    if (!gr) {
        if (cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
            cudaGetLastError();
            H.no_graph = true;
            return eig_batched(c, H.eR, seed, H.nref, true);
        }
        const long long l0 = c->launches;
        const int st = eig_batched(c, H.eR, seed, H.nref, true);
        cudaGraph_t graph = nullptr;
        const cudaError_t ce = cudaStreamEndCapture(c->stream, &graph);
        if (st != MG_OK || ce != cudaSuccess) {
            if (graph) cudaGraphDestroy(graph);
            return st != MG_OK ? st : MG_ERR_CUDA;
        }
        const cudaError_t ie = cudaGraphInstantiate(&gr, graph, 0);
        cudaGraphDestroy(graph);
        if (ie != cudaSuccess) {
            gr = nullptr;
            return MG_ERR_CUDA;
        }
        H.can_graph_launches[k] = c->launches - l0;
        H.can_graph_prec[k] = c->cur_precision;
        c->launches = l0;
    }
    MG_CUDA(cudaGraphLaunch(gr, c->stream));
    c->launches += H.can_graph_launches[k];
    return MG_OK;
}

int hfb_solve(mg_ctx* c, mg_pairing_info* info) {
    Hfb& H = c->hfb;
    if (!H.ready) MG_TRY(hfb_prepare(c));
    const long nm2 = 4L * H.nmax * H.nmax;
    if (H.oldrho_zero) {
        MG_CUDA(cudaMemcpyAsync(H.oldrho, H.rho, nm2 * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
        MG_CUDA(cudaMemcpyAsync(H.oldkappa, H.kappa, nm2 * sizeof(double), cudaMemcpyDeviceToDevice,
                                c->stream));
    }
    H.pc.cut[0] = H.pp.cut[0];
    H.pc.cut[1] = H.pp.cut[1];
    H.pc.mu[0] = H.pp.mu[0];
    H.pc.mu[1] = H.pp.mu[1];
    MG_CUDA(cudaMemcpyAsync(H.fermi_d, H.fermi, 2 * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    MG_CUDA(cudaMemsetAsync(c->flags, 0, 16 * sizeof(int), c->stream));
    MG_TRY(pairing_mesh(c));
    phase_mark(c, MG_PH_PAIRING_MESH);
    // the HF-basis DeriveAll of the iteration (mg_iterate) overlaps the
    // latency-bound rest of the step
    if (c->side_derive_pending) MG_TRY(side_derive_hf(c));

    double lam[2], f[2];
    bool conv[2];
    int evals = 0;
    bool first_order = false;
    if (H.pp.fermi_solver == 2) {
        MG_TRY(fermi_gradient(c, lam, f, conv, &evals));
    } else if (H.pp.fermi_solver == 1) {
        MG_TRY(fermi_broyden(c, lam, f, conv, &evals));
    } else if (H.pp.fermi_solver == 3) {
        MG_TRY(fermi_bisection(c, lam, f, conv, &evals));
    } else {
        MG_TRY(fermi_newton(c, lam, f, conv, &evals, &first_order));
    }
    phase_mark(c, MG_PH_FERMI);
    if (conv[0] && conv[1]) {
        for (int it = 0; it < 2; ++it) {
            for (int j = 3; j > 0; --j) H.fermi_old[j][it] = H.fermi_old[j - 1][it];
            H.fermi_old[0][it] = H.fermi_prev[it];
            H.fermi_prev[it] = H.fermi[it];
        }
        ++H.n_solved;
    } else {
        H.n_solved = 0;
    }
    H.fermi[0] = lam[0];
    H.fermi[1] = lam[1];
    for (int i = 0; i < 6; ++i) H.fermi_hist[i] = H.fermi_hist[i + 1];
    H.fermi_hist[6] = std::fabs(f[0]) > 0.9 || std::fabs(f[1]) > 0.9;
    bool lost = true;
    for (int i = 0; i < 7; ++i) lost = lost && H.fermi_hist[i];
    double tr0 = f[0] + c->p.neutrons, tr1 = f[1] + c->p.protons;

    // ---- canonical basis, occupations, mixing, pairing energy ------------------
    double* hp = H.h_pinned;
    const bool was_zero = H.oldrho_zero;
    int hflags[8];
    // redo: the canonical basis by plain FP64 Jacobi instead of the warm-seeded
    // decomposition.  One synchronisation at the end reads the pairing
    // energies and the flags, the occupation check among them.
    auto canonical_part = [&](bool redo) -> int {
        k_copy_rpp<<<dim3(div_up(H.hmax * H.hmax, kThreads), 4), kThreads, 0, c->stream>>>(
            H.rho, H.hsz, H.members, H.hmax, H.nmax, H.Rpp, c->bas[MG_HF_BASIS].occ);
        MG_LAUNCHED(c);
        if (redo) {
            MG_TRY(eig_jacobi_fp64(c, H.eR));
        } else {
            // the occupations cluster near 0 and 1 and the individual vectors
            // matter, so the FP32 Jacobi seed (warm-started from last
            // iteration's vectors) resolves the clusters before the refinement
            // and the polish
            MG_TRY(canonical_eig(c));
            H.eR.have_vectors = true;
        }
        k_occupations<<<4, kThreads, 0, c->stream>>>(H.eR.X, H.eR.w, H.hsz, H.cstart, H.hmax,
                                                     H.cantr, c->bas[MG_CAN_BASIS].occ, H.scal_d,
                                                     c->flags);
        MG_LAUNCHED(c);
        MG_TRY(canonical_transform(c));
        k_hfb_mix<<<4, kThreads, 0, c->stream>>>(H.rho, H.kappa, H.oldrho, H.oldkappa, H.delta,
                                                 H.hsz, H.nmax, H.pp.mix, was_zero ? 0 : 1, 1,
                                                 H.scal_d, H.oldrho_bak, H.oldkappa_bak);
        MG_LAUNCHED(c);
        MG_CUDA(cudaMemcpyAsync(hp + 16, H.scal_d, 8 * sizeof(double), cudaMemcpyDeviceToHost,
                                c->stream));
        MG_CUDA(cudaMemcpyAsync(hflags, c->flags, 8 * sizeof(int), cudaMemcpyDeviceToHost,
                                c->stream));
        MG_CUDA(cudaStreamSynchronize(c->stream));
        return MG_OK;
    };
    MG_TRY(canonical_part(false));
    if (hflags[3]) {
        // An occupation above one: a decomposition that lost orthonormality
        // (the refinement can, on spectra clustered at 0 and 1).  Put the
        // mixing history back, redo the evaluation at the final lambda from
        // scratch and the canonical basis by plain FP64 Jacobi, then mix
        // again, before reporting the state as the reference does.
        const long nbytes = nm2 * (long)sizeof(double);
        MG_CUDA(cudaMemcpyAsync(H.oldrho, H.oldrho_bak, nbytes, cudaMemcpyDeviceToDevice,
                                c->stream));
        MG_CUDA(cudaMemcpyAsync(H.oldkappa, H.oldkappa_bak, nbytes, cudaMemcpyDeviceToDevice,
                                c->stream));
        double f2[2], fp2[2];
        MG_TRY(hfb_evaluate(c, lam, f2, fp2, true, kSeedCold));
        ++evals;
        tr0 = f2[0] + c->p.neutrons;
        tr1 = f2[1] + c->p.protons;
        first_order = false;
        MG_CUDA(cudaMemsetAsync(c->flags + 3, 0, sizeof(int), c->stream));
        MG_TRY(canonical_part(true));
        ++H.reseeds;
    }
    H.oldrho_zero = false;
    H.epair[0] = -0.5 * (hp[16] + hp[17]);
    H.epair[1] = -0.5 * (hp[18] + hp[19]);
    H.disp[0] = hp[20] + hp[21];
    H.disp[1] = hp[22] + hp[23];
    c->pairing_energy[0] = H.epair[0];
    c->pairing_energy[1] = H.epair[1];
    phase_mark(c, MG_PH_CANONICAL);
    if (info) {
        std::memset(info, 0, sizeof(*info));
        info->fermi[0] = H.fermi[0];
        info->fermi[1] = H.fermi[1];
        info->particles[0] = tr0;
        info->particles[1] = tr1;
        info->evaluations = evals;
        info->converged = conv[0] && conv[1];
        info->pairing_energy[0] = H.epair[0];
        info->pairing_energy[1] = H.epair[1];
        info->dispersion[0] = H.disp[0];
        info->dispersion[1] = H.disp[1];
        info->first_order = first_order ? 1 : 0;
    }
    if (hflags[3]) {   // src/HFB.f90:3392-3395
        double om[4];
        MG_CUDA(cudaMemcpyAsync(om, H.scal_d + 8, 4 * sizeof(double), cudaMemcpyDeviceToHost,
                                c->stream));
        MG_CUDA(cudaStreamSynchronize(c->stream));
        fprintf(stderr, "mocca_gpu: some occupations are bigger than one in the canonical basis "
                "(largest v^2 per block: %.9f %.9f %.9f %.9f)\n", om[0], om[1], om[2], om[3]);
        return MG_ERR_STATE;
    }
    if (lost) {        // src/HFB.f90:2154-2158
        fprintf(stderr, "mocca_gpu: particle number lost in 7 consecutive Fermi searches "
                "(last deviations %.3e %.3e)\n", f[0], f[1]);
        return MG_ERR_STATE;
    }
    return (conv[0] && conv[1]) ? MG_OK : MG_NOT_CONVERGED;
}

}  // namespace mg
