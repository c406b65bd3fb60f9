// gradient_hfb.cu -- the gradient HFB solver (FermiSolver 'GRADIENT') on the
// device, FP64.
//
// Replaces HFBFermiGradient (src/GradientHFB.f90:473-733) for signature and
// time simplex conserved, without HFBReduce, blocking, Lipkin-Nogami or
// FermiMomentum (the defaults): H20_sig (:1014-1068), N20 (:1070-1108),
// GradUpdate_sig (:884-920), ortho_sig (:1148-1222), and OutHFBModule's
// rho = V V^T, kappa = V U^T (:188-269).
//
// In a block of h stored spwfs the reference's N = 2h by N matrices U and V
// hold four nonzero h x h blocks: the S = h positive-signature columns have
// Ua = U(0:h, 0:S) and Va = V(h:N, 0:S), the others Ub = U(h:N, S:N) and
// Vb = V(0:h, S:N).  The solver works on those blocks, with hb = diag(e) (the
// HF energies, Fermi energy zero) and Delta's two off-diagonal blocks
// Dpm = Delta(0:h, h:N), Dmp = Delta(h:N, 0:h):
//   H20_BA = Ub^T (E Va + Dmp Ua) - Vb^T (Dpm Va + E Ua)
//   N20_AB = Ua^T Vb - Va^T Ub
//   G_BA   = H20_BA + lambda N20_AB^T            (Gradient = H20 - lambda N20)
//   lambda += (N0 - |V|^2) / |N20|^2  per isospin (|N20|^2 = 2 sum of both blocks')
//   Ua -= s Vb G,  Va -= s Ub G,  Ub += s Va G^T,  Vb += s Ua G^T   (s = 0.020)
// then modified Gram-Schmidt of the columns of [Ua; Va] and of [Vb; Ub]; an
// isospin stops when |Gradient|, sqrt|sum G_ij G_ji|, and |N - N0| are below
// FermiPrec in both its blocks.  The matrix products are batched FP64 GEMMs
// (eig.cu's k_gemm64, a converged isospin's blocks skipped), the Fermi
// update and the convergence test one small kernel, the orthonormalisation
// one CTA per block and column set.  Iterations replay in chunks of kChunk
// as one CUDA graph; the host reads the state after each chunk.
//
// GradU and GradV persist between pairing steps as in the reference.  The
// reference takes the first ones from the HFB module's U and V (an earlier
// diagonalisation or a restart file); here the first call seeds them from
// one diagonalisation at the Fermi energies the step starts from: the
// positive half of T's eigenvectors (w; y) gives Ua = w, Va = y, Ub = -w,
// Vb = y, as DiagonaliseHFBHamiltonian_Signature and GetUandV place them
// (src/HFB.f90:2695-2786, src/GradientHFB.f90:108-186).
#include <algorithm>
#include <climits>
#include <cmath>
#include <vector>

#include "mg_internal.cuh"

namespace mg {

namespace {

constexpr int kThreads = 256;
constexpr int kChunk = 10;          // iterations per graph launch / host check
constexpr double kStep = 0.020;     // src/GradientHFB.f90:511

struct GhState {
    double fermi[2];
    double n20[2];
    double par[2];
    double gnorm[4];
    int conv[2];
    int iters;
    int stop;        // both isospins converged, or the iteration cap reached
    int done[4];     // per block: 0 = skip (its isospin converged or stopped)
};

// row i of a block: e of the stored spwf i (its partner has the same energy)
__global__ void k_gh_seed(const double* __restrict__ X, const int* __restrict__ hsz, int hmax,
                          int nmax, double* __restrict__ U4) {
    const int b = blockIdx.y, h = hsz[b];
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= h * h) return;
    const int r = t / h, k = t % h;
    const double* Xb = X + (long)b * nmax * nmax;
    const double w = Xb[(long)r * nmax + h + k], y = Xb[(long)(h + r) * nmax + h + k];
    const long hh = (long)hmax * hmax, o = (long)b * 4 * hh + (long)r * hmax + k;
    U4[o] = w;            // Ua
    U4[o + hh] = y;       // Va
    U4[o + 2 * hh] = -w;  // Ub
    U4[o + 3 * hh] = y;   // Vb
}

__global__ void k_gh_pre(const double* __restrict__ U4, const double* __restrict__ e_hf,
                         const int* __restrict__ members, const int* __restrict__ hsz, int hmax,
                         double* __restrict__ A1, double* __restrict__ A2,
                         GhState* __restrict__ S) {
    const int b = blockIdx.y, h = hsz[b];
    // after the last iteration every later launch of the chunk is skipped
    if (S->stop) {
        if (blockIdx.x == 0 && threadIdx.x == 0) S->done[b] = 0;
        return;
    }
    if (S->done[b] == 0) return;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= h * h) return;
    const int r = t / h, k = t % h;
    const long hh = (long)hmax * hmax, o = (long)r * hmax + k;
    const double e = e_hf[members[b * hmax + r]];
    A1[b * hh + o] = e * U4[b * 4 * hh + hh + o];   // E Va
    A2[b * hh + o] = e * U4[b * 4 * hh + o];        // E Ua
}

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

// Fermi energies, total gradient, convergence (one CTA, every block).
__global__ void __launch_bounds__(1024)
k_gh_ctrl(const double* __restrict__ U4, const double* __restrict__ Hm,
          const double* __restrict__ Nm, double* __restrict__ G, const int* __restrict__ hsz,
          int hmax, double n0, double p0, double prec, int maxit, GhState* __restrict__ S) {
    __shared__ double red[32];
    if (S->stop) return;
    const long hh = (long)hmax * hmax;
    const double parts[2] = {n0, p0};
    for (int it = 0; it < 2; ++it) {
        double n20 = 0.0, par = 0.0;
        for (int b = 2 * it; b < 2 * it + 2; ++b) {
            const int h = hsz[b];
            double pn = 0.0, pv = 0.0;
            for (int t = threadIdx.x; t < h * h; t += blockDim.x) {
                const long o = (long)(t / h) * hmax + t % h;
                const double x = Nm[b * hh + o];
                const double va = U4[b * 4 * hh + hh + o], vb = U4[b * 4 * hh + 3 * hh + o];
                pn = fma(x, x, pn);
                pv = fma(va, va, fma(vb, vb, pv));
            }
            n20 += 2.0 * cta_sum(pn, red);
            par += cta_sum(pv, red);
        }
        // the reference recomputes |N20|^2 only for isospins still running
        // but moves every isospin's Fermi energy
        if (threadIdx.x == 0) {
            if (!S->conv[it]) S->n20[it] = n20;
            S->par[it] = par;
            const double n = S->n20[it];
            if (fabs(n) > 1e-10) S->fermi[it] = S->fermi[it] + (parts[it] - par) / n;
            else S->fermi[it] = S->fermi[it] + 0.1 * (parts[it] - par);
        }
    }
    __syncthreads();
    for (int it = 0; it < 2; ++it) {
        if (S->conv[it]) continue;
        const double lam = S->fermi[it];
        bool ok = fabs(S->par[it] - parts[it]) < prec;
        for (int b = 2 * it; b < 2 * it + 2; ++b) {
            const int h = hsz[b];
            double pg = 0.0;
            for (int t = threadIdx.x; t < h * h; t += blockDim.x) {
                const int r = t / h, k = t % h;
                const double g = Hm[b * hh + (long)r * hmax + k] + lam * Nm[b * hh + (long)k * hmax + r];
                G[b * hh + (long)r * hmax + k] = g;
                pg = fma(g, g, pg);
            }
            const double gn = -2.0 * cta_sum(pg, red);   // sum G_ij G_ji, G antisymmetric
            if (threadIdx.x == 0) S->gnorm[b] = gn;
            ok = ok && sqrt(fabs(gn)) < prec;
        }
        if (threadIdx.x == 0 && ok) S->conv[it] = 1;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        S->iters += 1;
        const bool all = S->conv[0] && S->conv[1];
        S->stop = all || S->iters >= maxit;
        // this iteration's step still runs for the isospins not converged
        // (as the reference's last iteration does); the next k_gh_pre turns
        // everything off once stop is set
        for (int b = 0; b < 4; ++b) S->done[b] = S->conv[b / 2] ? 0 : INT_MAX;
    }
}

// ortho_sig: modified Gram-Schmidt of the columns of [Ua; Va] (set 0) or of
// [Vb; Ub] (set 1) of one block, in column order.
__global__ void __launch_bounds__(kThreads)
k_gh_ortho(double* __restrict__ U4, const int* __restrict__ hsz, int hmax,
           const GhState* __restrict__ S) {
    __shared__ double red[32];
    __shared__ double bc;
    const int b = blockIdx.x / 2, set = blockIdx.x % 2, h = hsz[b];
    if (S->done[b] == 0) return;
    const long hh = (long)hmax * hmax;
    double* top = U4 + b * 4 * hh + (set == 0 ? 0 : 3 * hh);     // Ua or Vb
    double* bot = U4 + b * 4 * hh + (set == 0 ? hh : 2 * hh);    // Va or Ub
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32, nw = kThreads / 32;
    for (int j = 0; j < h; ++j) {
        double p = 0.0;
        for (int r = threadIdx.x; r < 2 * h; r += kThreads) {
            const double x = r < h ? top[(long)r * hmax + j] : bot[(long)(r - h) * hmax + j];
            p = fma(x, x, p);
        }
        const double nrm = cta_sum(p, red);
        if (threadIdx.x == 0) bc = 1.0 / sqrt(nrm);
        __syncthreads();
        const double sc = bc;
        for (int r = threadIdx.x; r < 2 * h; r += kThreads) {
            if (r < h) top[(long)r * hmax + j] *= sc;
            else bot[(long)(r - h) * hmax + j] *= sc;
        }
        __syncthreads();
        // later columns: one warp per column
        for (int i = j + 1 + warp; i < h; i += nw) {
            double o = 0.0;
            for (int r = lane; r < 2 * h; r += 32) {
                o = r < h ? fma(top[(long)r * hmax + j], top[(long)r * hmax + i], o)
                          : fma(bot[(long)(r - h) * hmax + j], bot[(long)(r - h) * hmax + i], o);
            }
            for (int q = 16; q > 0; q >>= 1) o += __shfl_xor_sync(0xffffffffu, o, q);
            for (int r = lane; r < 2 * h; r += 32) {
                if (r < h) top[(long)r * hmax + i] -= o * top[(long)r * hmax + j];
                else bot[(long)(r - h) * hmax + i] -= o * bot[(long)(r - h) * hmax + j];
            }
        }
        __syncthreads();
    }
}

__global__ void k_gh_init(GhState* __restrict__ S, double l0, double l1) {
    if (threadIdx.x != 0) return;
    S->fermi[0] = l0;
    S->fermi[1] = l1;
    S->n20[0] = S->n20[1] = 0.0;
    S->par[0] = S->par[1] = 0.0;
    S->conv[0] = S->conv[1] = 0;
    S->iters = 0;
    S->stop = 0;
    for (int b = 0; b < 4; ++b) {
        S->done[b] = INT_MAX;
        S->gnorm[b] = 0.0;
    }
}

}  // namespace

struct GradHfb {
    double* U4 = nullptr;     // [4][Ua, Va, Ub, Vb][hmax^2]
    double* U4n = nullptr;    // the updated copy
    double *A1 = nullptr, *A2 = nullptr, *Hm = nullptr, *Nm = nullptr, *G = nullptr;  // [4][hmax^2]
    GemmDesc* d = nullptr;    // 8 + 8 + 8 + 16 + 16 descriptors
    GhState* S = nullptr;
    GhState* h_S = nullptr;   // pinned
    bool seeded = false;
    cudaGraphExec_t chunk = nullptr;
    long long chunk_launches = 0;
    int maxit = 0;
    double prec = 0.0;
    bool no_graph = false;
};

void gradient_hfb_free(GradHfb* g) {
    if (!g) return;
    for (void* p : {(void*)g->U4, (void*)g->U4n, (void*)g->A1, (void*)g->A2, (void*)g->Hm,
                    (void*)g->Nm, (void*)g->G, (void*)g->d, (void*)g->S})
        if (p) cudaFree(p);
    if (g->h_S) cudaFreeHost(g->h_S);
    if (g->chunk) cudaGraphExecDestroy(g->chunk);
    delete g;
}

static int gradient_setup(mg_ctx* c) {
    Hfb& H = c->hfb;
    GradHfb* g = new GradHfb();
    H.grad = g;
    const int hm = H.hmax, nm = H.nmax;
    const long hh = (long)hm * hm;
    MG_CUDA(cudaMalloc(&g->U4, 16 * hh * sizeof(double)));
    MG_CUDA(cudaMalloc(&g->U4n, 16 * hh * sizeof(double)));
    MG_CUDA(cudaMemset(g->U4, 0, 16 * hh * sizeof(double)));
    for (double** p : {&g->A1, &g->A2, &g->Hm, &g->Nm, &g->G}) {
        MG_CUDA(cudaMalloc(p, 4 * hh * sizeof(double)));
        MG_CUDA(cudaMemset(*p, 0, 4 * hh * sizeof(double)));
    }
    MG_CUDA(cudaMalloc(&g->S, sizeof(GhState)));
    MG_CUDA(cudaMallocHost(&g->h_S, sizeof(GhState)));
    std::vector<GemmDesc> d(56);
    for (int b = 0; b < 4; ++b) {
        const int h = H.hsz_h[b], N = 2 * h;
        const double* Db = H.delta + (long)b * nm * nm;   // N x N, row stride N
        const double* Dpm = Db + h;
        const double* Dmp = Db + (long)h * N;
        double* U = g->U4 + (long)b * 4 * hh;
        double *Ua = U, *Va = U + hh, *Ub = U + 2 * hh, *Vb = U + 3 * hh;
        double* Un = g->U4n + (long)b * 4 * hh;
        double *Ua2 = Un, *Va2 = Un + hh, *Ub2 = Un + 2 * hh, *Vb2 = Un + 3 * hh;
        const long o = (long)b * hh;
        double *A1 = g->A1 + o, *A2 = g->A2 + o, *Hm = g->Hm + o, *Nm = g->Nm + o, *G = g->G + o;
        // A1 += Dmp Ua, A2 += Dpm Va
        d[2 * b] = GemmDesc{Dmp, Ua, A1, h, h, h, N, hm, hm, 0, 0, 1.0, 1.0, b, 0};
        d[2 * b + 1] = GemmDesc{Dpm, Va, A2, h, h, h, N, hm, hm, 0, 0, 1.0, 1.0, b, 0};
        // Hm = Ub^T A1, Nm = Ua^T Vb
        d[8 + 2 * b] = GemmDesc{Ub, A1, Hm, h, h, h, hm, hm, hm, 1, 0, 1.0, 0.0, b, 0};
        d[8 + 2 * b + 1] = GemmDesc{Ua, Vb, Nm, h, h, h, hm, hm, hm, 1, 0, 1.0, 0.0, b, 0};
        // Hm -= Vb^T A2, Nm -= Va^T Ub
        d[16 + 2 * b] = GemmDesc{Vb, A2, Hm, h, h, h, hm, hm, hm, 1, 0, -1.0, 1.0, b, 0};
        d[16 + 2 * b + 1] = GemmDesc{Va, Ub, Nm, h, h, h, hm, hm, hm, 1, 0, -1.0, 1.0, b, 0};
        // the step: Ua -= s Vb G, Va -= s Ub G, Ub += s Va G^T, Vb += s Ua G^T
        d[24 + 4 * b] = GemmDesc{Vb, G, Ua2, h, h, h, hm, hm, hm, 0, 0, -kStep, 1.0, b, 0};
        d[24 + 4 * b + 1] = GemmDesc{Ub, G, Va2, h, h, h, hm, hm, hm, 0, 0, -kStep, 1.0, b, 0};
        d[24 + 4 * b + 2] = GemmDesc{Va, G, Ub2, h, h, h, hm, hm, hm, 0, 1, kStep, 1.0, b, 0};
        d[24 + 4 * b + 3] = GemmDesc{Ua, G, Vb2, h, h, h, hm, hm, hm, 0, 1, kStep, 1.0, b, 0};
        // OutHFBModule: rho_++ = Vb Vb^T, rho_-- = Va Va^T, kappa_-+ = Va Ua^T,
        // kappa_+- = -Ua Va^T (rows of the N x N blocks have stride N)
        double* R = H.rho + (long)b * nm * nm;
        double* K = H.kappa + (long)b * nm * nm;
        d[40 + 4 * b] = GemmDesc{Vb, Vb, R, h, h, h, hm, hm, N, 0, 1, 1.0, 0.0, b, 0};
        d[40 + 4 * b + 1] = GemmDesc{Va, Va, R + (long)h * N + h, h, h, h, hm, hm, N, 0, 1, 1.0, 0.0, b, 0};
        d[40 + 4 * b + 2] = GemmDesc{Va, Ua, K + (long)h * N, h, h, h, hm, hm, N, 0, 1, 1.0, 0.0, b, 0};
        d[40 + 4 * b + 3] = GemmDesc{Ua, Va, K + h, h, h, h, hm, hm, N, 0, 1, -1.0, 0.0, b, 0};
    }
    MG_CUDA(cudaMalloc(&g->d, d.size() * sizeof(GemmDesc)));
    MG_CUDA(cudaMemcpy(g->d, d.data(), d.size() * sizeof(GemmDesc), cudaMemcpyHostToDevice));
    return MG_OK;
}

// HFBFermiGradient for the pairing step: lam in/out (the Fermi energies),
// f the particle-number deviations, conv per isospin, iters the gradient
// iterations run.  Leaves rho and kappa in H.rho, H.kappa.
int fermi_gradient(mg_ctx* c, double lam[2], double f[2], bool conv[2], int* iters) {
    Hfb& H = c->hfb;
    if (!H.grad) MG_TRY(gradient_setup(c));
    GradHfb* g = H.grad;
    const int hm = H.hmax;
    const long hh = (long)hm * hm;
    const dim3 gb(div_up(hm * hm, kThreads), 4);
    if (!g->seeded) {
        double Nt[2], dN[2];
        MG_TRY(hfb_evaluate_at(c, H.fermi, Nt, dN));
        k_gh_seed<<<gb, kThreads, 0, c->stream>>>(H.eT.X, H.hsz, hm, H.nmax, g->U4);
        MG_LAUNCHED(c);
        g->seeded = true;
    }
    const int maxit = H.pp.max_iter > 0 ? H.pp.max_iter : 500;
    const double prec = H.pp.fermi_prec;
    k_gh_init<<<1, 32, 0, c->stream>>>(g->S, H.fermi[0], H.fermi[1]);
    MG_LAUNCHED(c);
    const int* done = g->S->done;
    auto iterations = [&](int count) -> int {
        for (int s = 0; s < count; ++s) {
            k_gh_pre<<<gb, kThreads, 0, c->stream>>>(g->U4, c->bas[MG_HF_BASIS].e, H.members, H.hsz,
                                                     hm, g->A1, g->A2, g->S);
            MG_LAUNCHED(c);
            MG_TRY(gemm_batched_skip(c, g->d, 8, hm, const_cast<int*>(done)));
            MG_TRY(gemm_batched_skip(c, g->d + 8, 8, hm, const_cast<int*>(done)));
            MG_TRY(gemm_batched_skip(c, g->d + 16, 8, hm, const_cast<int*>(done)));
            k_gh_ctrl<<<1, 1024, 0, c->stream>>>(g->U4, g->Hm, g->Nm, g->G, H.hsz, hm,
                                                 c->p.neutrons, c->p.protons, prec, maxit, g->S);
            MG_LAUNCHED(c);
            MG_CUDA(cudaMemcpyAsync(g->U4n, g->U4, 16 * hh * sizeof(double),
                                    cudaMemcpyDeviceToDevice, c->stream));
            MG_TRY(gemm_batched_skip(c, g->d + 24, 16, hm, const_cast<int*>(done)));
            k_gh_ortho<<<8, kThreads, 0, c->stream>>>(g->U4n, H.hsz, hm, g->S);
            MG_LAUNCHED(c);
            MG_CUDA(cudaMemcpyAsync(g->U4, g->U4n, 16 * hh * sizeof(double),
                                    cudaMemcpyDeviceToDevice, c->stream));
        }
        return MG_OK;
    };
    if (g->chunk && (g->maxit != maxit || g->prec != prec)) {
        cudaGraphExecDestroy(g->chunk);
        g->chunk = nullptr;
    }
    if (!g->chunk && !g->no_graph) {
        if (cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
            cudaGetLastError();
            g->no_graph = true;
        } else {
            const long long l0 = c->launches;
            const int st = iterations(kChunk);
            cudaGraph_t graph = nullptr;
            const cudaError_t ce = cudaStreamEndCapture(c->stream, &graph);
            if (st != MG_OK || ce != cudaSuccess) {
                if (graph) cudaGraphDestroy(graph);
                return st != MG_OK ? st : MG_ERR_CUDA;
            }
            const cudaError_t ie = cudaGraphInstantiate(&g->chunk, graph, 0);
            cudaGraphDestroy(graph);
            if (ie != cudaSuccess) {
                g->chunk = nullptr;
                return MG_ERR_CUDA;
            }
            g->chunk_launches = c->launches - l0;
            c->launches = l0;
            g->maxit = maxit;
            g->prec = prec;
        }
    }
    for (int done_it = 0; done_it < maxit; done_it += kChunk) {
        if (g->chunk) {
            MG_CUDA(cudaGraphLaunch(g->chunk, c->stream));
            c->launches += g->chunk_launches;
        } else {
            MG_TRY(iterations(kChunk));
        }
        MG_CUDA(cudaMemcpyAsync(g->h_S, g->S, sizeof(GhState), cudaMemcpyDeviceToHost, c->stream));
        MG_CUDA(cudaStreamSynchronize(c->stream));
        if (g->h_S->stop) break;
    }
    // rho and kappa from the final U and V
    const long nm2 = (long)H.nmax * H.nmax;
    MG_CUDA(cudaMemsetAsync(H.rho, 0, 4 * nm2 * sizeof(double), c->stream));
    MG_CUDA(cudaMemsetAsync(H.kappa, 0, 4 * nm2 * sizeof(double), c->stream));
    MG_TRY(gemm_batched(c, g->d + 40, 16, hm));
    const GhState& S = *g->h_S;
    lam[0] = S.fermi[0];
    lam[1] = S.fermi[1];
    f[0] = S.par[0] - c->p.neutrons;
    f[1] = S.par[1] - c->p.protons;
    conv[0] = S.conv[0] != 0;
    conv[1] = S.conv[1] != 0;
    *iters = S.iters;
    if (std::isnan(lam[0]) || std::isnan(lam[1])) return MG_ERR_NAN;
    return MG_OK;
}

}  // namespace mg
