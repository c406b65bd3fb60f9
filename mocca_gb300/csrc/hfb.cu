// hfb.cu -- small dense HFB algebra on the device, FP64, and the host driver
// of the HFB pairing step.
//
// Replaces, for the EV8 + time-reversal case (signature and time simplex
// conserved, no Lipkin-Nogami, no blocking):
//   ConstructHFBHamiltonian          src/HFB.f90:2554-2631
//   DiagonaliseHFBHamiltonian_Signature  :2695-2786 (diagoncr8 :5880-6087)
//   HFBNumberofParticles_ordinary    :810-1072  (PfSolver off: CR8 columns)
//   constructRhoHFB / ConstructKappaHFB  :3128-3154, :3335-3359
//   DiagonaliseRhoHFB / HFBOccupations   :3156-3284, :3361-3560
//   HFBEnergy                        :296-348
//   GuessHFBMatrices (case 2, TRC)   :3645-3835
// The signature-reduced HFB matrix of a block is
//   T = [[e - lambda, D], [D^T, -(e - lambda)]],  D(i,j) = Delta(i, j+h),
// with eigenvectors X (ascending).  With the CR8 column choice the positive
// quasiparticle half gives, for the stored (+) and reversed (-) halves,
//   rho_++ = rho_-- = Y Y^T,  kappa_-+ = Y W^T,  Y = X(h:N, h:N), W = X(0:h, h:N)
// and zero elsewhere.  Each (isospin, parity) block is one CTA with its
// matrix in shared memory; the symmetric eigensolver is the Householder
// tridiagonalisation + implicit QL method (the algorithm diagoncr8 also
// implements) with the O(n^2) inner loops spread over the CTA's threads and
// each QL sweep's rotations applied row-parallel after the scalar chain.
//
// FindFermiEnergy: the reference's damped Broyden (src/HFB.f90:1849-2161)
// is replaced by a safeguarded secant iteration on the same equation
// N(lambda) = N0 with the same tolerance FermiPrec per isospin; both reach the
// same root.  Every particle-number evaluation is one launch of k_hfb_eval.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "mg_internal.cuh"

namespace mg {

namespace {

constexpr int kThreads = 256;
constexpr int kMaxQL = 60;

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

// Symmetric eigen-decomposition of A (n x n, row-major, leading dim lda, in
// shared memory).  On return A holds the eigenvectors (column k <-> d[k]),
// d the eigenvalues in ascending order.  Scratch: e, g (n), rc, rs (n),
// perm (n ints), red (32), ctl (8 ints).  Returns 0, or 1 when a QL sweep
// exceeded its cap (the reference's diagoncr8 ifail).
__device__ int eigh_cta(double* A, int lda, int n, double* d, double* e, double* g, double* rc,
                        double* rs, int* perm, double* red, int* ctl) {
    const int tid = threadIdx.x, nt = blockDim.x;
    auto a = [&](int i, int j) -> double& { return A[i * lda + j]; };
    // ---- Householder reduction to tridiagonal form ----------------------------
    for (int i = n - 1; i > 0; --i) {
        const int l = i - 1;
        double part = 0.0;
        for (int k = tid; k <= l; k += nt) part += fabs(a(i, k));
        const double scale = cta_sum(part, red);
        double h = 0.0;
        if (l > 0 && scale != 0.0) {
            part = 0.0;
            for (int k = tid; k <= l; k += nt) {
                const double x = a(i, k) / scale;
                a(i, k) = x;
                part += x * x;
            }
            h = cta_sum(part, red);
            const double f = a(i, l);
            const double gg = f >= 0.0 ? -sqrt(h) : sqrt(h);
            h -= f * gg;
            __syncthreads();
            if (tid == 0) {
                e[i] = scale * gg;
                a(i, l) = f - gg;
            }
            __syncthreads();
            part = 0.0;
            for (int j = tid; j <= l; j += nt) {
                a(j, i) = a(i, j) / h;
                double s = 0.0;
                for (int k = 0; k <= j; ++k) s += a(j, k) * a(i, k);
                for (int k = j + 1; k <= l; ++k) s += a(k, j) * a(i, k);
                e[j] = s / h;
                part += e[j] * a(i, j);
            }
            const double ff = cta_sum(part, red);
            const double hh = ff / (h + h);
            for (int j = tid; j <= l; j += nt) e[j] = e[j] - hh * a(i, j);
            __syncthreads();
            for (int t = tid; t < (l + 1) * (l + 1); t += nt) {
                const int j = t / (l + 1), k = t % (l + 1);
                if (k <= j) a(j, k) -= (a(i, j) * e[k] + e[j] * a(i, k));
            }
            __syncthreads();
        } else {
            if (tid == 0) e[i] = a(i, l);
            __syncthreads();
        }
        if (tid == 0) d[i] = h;
        __syncthreads();
    }
    if (tid == 0) {
        d[0] = 0.0;
        e[0] = 0.0;
    }
    __syncthreads();
    // ---- accumulate the transformations -----------------------------------------
    for (int i = 0; i < n; ++i) {
        const int l = i - 1;
        if (d[i] != 0.0) {
            for (int j = tid; j <= l; j += nt) {
                double s = 0.0;
                for (int k = 0; k <= l; ++k) s += a(i, k) * a(k, j);
                g[j] = s;
            }
            __syncthreads();
            for (int t = tid; t < (l + 1) * (l + 1); t += nt) {
                const int k = t / (l + 1), j = t % (l + 1);
                a(k, j) -= g[j] * a(k, i);
            }
            __syncthreads();
        }
        if (tid == 0) {
            d[i] = a(i, i);
            a(i, i) = 1.0;
        }
        for (int j = tid; j <= l; j += nt) {
            a(j, i) = 0.0;
            a(i, j) = 0.0;
        }
        __syncthreads();
    }
    // ---- implicit QL on the tridiagonal matrix --------------------------------
    if (tid == 0) {
        for (int i = 1; i < n; ++i) e[i - 1] = e[i];
        e[n - 1] = 0.0;
        ctl[0] = 0;  // failure flag
    }
    __syncthreads();
    for (int l = 0; l < n; ++l) {
        int iter = 0;
        while (true) {
            if (tid == 0) {
                int m;
                for (m = l; m < n - 1; ++m) {
                    const double dd = fabs(d[m]) + fabs(d[m + 1]);
                    if (fabs(e[m]) <= 2.2e-16 * dd) break;
                }
                ctl[1] = m;      // m == l: converged
                ctl[2] = l;      // lowest rotation applied
                ctl[3] = m - 1;  // highest rotation applied
                if (m != l) {
                    if (iter >= kMaxQL) {
                        ctl[0] = 1;
                        ctl[1] = l;
                    } else {
                        double gq = (d[l + 1] - d[l]) / (2.0 * e[l]);
                        double r = hypot(gq, 1.0);
                        gq = d[m] - d[l] + e[l] / (gq + (gq >= 0.0 ? fabs(r) : -fabs(r)));
                        double s = 1.0, c = 1.0, p = 0.0;
                        int i;
                        bool early = false;
                        for (i = m - 1; i >= l; --i) {
                            const double f = s * e[i], b = c * e[i];
                            e[i + 1] = (r = hypot(f, gq));
                            if (r == 0.0) {
                                d[i + 1] -= p;
                                e[m] = 0.0;
                                early = true;
                                break;
                            }
                            s = f / r;
                            c = gq / r;
                            gq = d[i + 1] - p;
                            r = (d[i] - gq) * s + 2.0 * c * b;
                            d[i + 1] = gq + (p = s * r);
                            gq = c * r - b;
                            rc[i] = c;
                            rs[i] = s;
                        }
                        ctl[2] = early ? i + 1 : l;
                        if (!early) {
                            d[l] -= p;
                            e[l] = gq;
                            e[m] = 0.0;
                        }
                    }
                }
            }
            __syncthreads();
            const int m = ctl[1], lo = ctl[2], hi = ctl[3];
            if (m == l) break;
            for (int k = tid; k < n; k += nt)
                for (int i = hi; i >= lo; --i) {
                    const double f = a(k, i + 1);
                    a(k, i + 1) = rs[i] * a(k, i) + rc[i] * f;
                    a(k, i) = rc[i] * a(k, i) - rs[i] * f;
                }
            __syncthreads();
            ++iter;
        }
        if (ctl[0]) break;
    }
    // ---- sort ascending (selection sort as diagoncr8), swap columns ------------
    // perm[i] records the column exchanged with column i at step i; every
    // thread replays the same exchanges on the rows it owns.
    if (tid == 0) {
        for (int i = 0; i < n - 1; ++i) {
            int k = i;
            double p = d[i];
            for (int j = i + 1; j < n; ++j)
                if (d[j] < p) { k = j; p = d[j]; }
            perm[i] = k;
            if (k != i) {
                d[k] = d[i];
                d[i] = p;
            }
        }
    }
    __syncthreads();
    for (int k = tid; k < n; k += nt)
        for (int i = 0; i < n - 1; ++i) {
            const int j = perm[i];
            if (j != i) {
                const double t = a(k, i);
                a(k, i) = a(k, j);
                a(k, j) = t;
            }
        }
    __syncthreads();
    return ctl[0];
}

struct EvalArgs {
    const double* delta;
    const double* e_hf;
    const int* members;
    const int* hsz;
    int hmax, nmax;
    const double* fermi;
    double* rho;
    double* kappa;
    double* qe;
    double* trace;
    int* flags;
};

// One particle-number evaluation: per block, build T(lambda), diagonalise,
// form rho and kappa, write the block trace of rho.
__global__ void __launch_bounds__(kThreads) k_hfb_eval(EvalArgs a) {
    extern __shared__ double sm[];
    __shared__ double red[32];
    __shared__ int ctl[8];
    const int b = blockIdx.x, it = b / 2;
    const int h = a.hsz[b], N = 2 * h, lda = N + 1;
    const double lam = a.fermi[it];
    double* A = sm;
    double* d = A + N * lda;
    double* e = d + N;
    double* g = e + N;
    double* rc = g + N;
    double* rs = rc + N;
    int* perm = (int*)(rs + N);
    const double* D = a.delta + (long)b * a.nmax * a.nmax;
    for (int t = threadIdx.x; t < N * N; t += kThreads) {
        const int i = t / N, j = t % N;
        double v = 0.0;
        if (i < h && j < h) {
            if (i == j) v = a.e_hf[a.members[b * a.hmax + i]] - lam;
        } else if (i >= h && j >= h) {
            if (i == j) v = -(a.e_hf[a.members[b * a.hmax + i - h]] - lam);
        } else if (i < h) {
            v = D[(long)i * N + j];
        } else {
            v = D[(long)j * N + i];
        }
        A[i * lda + j] = v;
    }
    __syncthreads();
    if (N == 0) return;
    const int fail = eigh_cta(A, lda, N, d, e, g, rc, rs, perm, red, ctl);
    if (fail && threadIdx.x == 0) atomicExch(a.flags + 1, 1);
    double* R = a.rho + (long)b * a.nmax * a.nmax;
    double* K = a.kappa + (long)b * a.nmax * a.nmax;
    double part = 0.0;
    for (int t = threadIdx.x; t < h * h; t += kThreads) {
        const int r = t / h, s = t % h;
        double rr = 0.0, kk = 0.0;
        for (int m = N - 1; m >= h; --m) {
            const double y = A[(h + r) * lda + m];
            rr = fma(y, A[(h + s) * lda + m], rr);
            kk = fma(y, A[s * lda + m], kk);
        }
        R[(long)r * N + s] = rr;
        R[(long)(h + r) * N + h + s] = rr;
        R[(long)r * N + h + s] = 0.0;
        R[(long)(h + r) * N + s] = 0.0;
        K[(long)(h + r) * N + s] = kk;
        K[(long)s * N + h + r] = -kk;
        K[(long)r * N + s] = 0.0;
        K[(long)(h + r) * N + h + s] = 0.0;
        if (r == s) part += 2.0 * rr;
    }
    for (int t = threadIdx.x; t < N; t += kThreads) a.qe[(long)b * a.nmax + t] = d[t];
    const double tr = cta_sum(part, red);
    if (threadIdx.x == 0) a.trace[b] = tr;
}

struct OccArgs {
    const double* rho;
    const int* members;
    const int* hsz;
    const int* cstart;
    int hmax, nmax;
    double* cantr;
    double* can_occ;
    double* hf_occ;
    double* scal;   // [4 blocks] dispersion partials at scal[4 + b]
    int* flags;
};

// DiagonaliseRhoHFB + the occupation part of HFBOccupations.
__global__ void __launch_bounds__(kThreads) k_rho_diag(OccArgs a) {
    extern __shared__ double sm[];
    __shared__ double red[32];
    __shared__ int ctl[8];
    const int b = blockIdx.x;
    const int h = a.hsz[b], N = 2 * h, lda = h + 1;
    if (h == 0) return;
    double* A = sm;
    double* d = A + h * lda;
    double* e = d + h;
    double* g = e + h;
    double* rc = g + h;
    double* rs = rc + h;
    int* perm = (int*)(rs + h);
    const double* R = a.rho + (long)b * a.nmax * a.nmax;
    for (int t = threadIdx.x; t < h * h; t += kThreads) A[(t / h) * lda + t % h] = R[(long)(t / h) * N + t % h];
    for (int j = threadIdx.x; j < N; j += kThreads)
        a.hf_occ[a.members[b * a.hmax + (j % h)]] = 2.0 * R[(long)j * N + j];
    __syncthreads();
    const int fail = eigh_cta(A, lda, h, d, e, g, rc, rs, perm, red, ctl);
    if (fail && threadIdx.x == 0) atomicExch(a.flags + 2, 1);
    double* T = a.cantr + (long)b * a.hmax * a.hmax;
    for (int t = threadIdx.x; t < h * h; t += kThreads) {
        const double x = A[(t / h) * lda + t % h];
        T[t] = fabs(x) < 1e-11 ? 0.0 : x;
    }
    double part = 0.0;
    for (int C = threadIdx.x; C < h; C += kThreads) {
        double o = d[C];
        if (o > 1.0 + 1e-5) atomicExch(a.flags + 3, 1);
        if (o < -0.1) o += 2.0;
        if (o < 0.0) o = 0.0;
        if (o > 1.0) o = 1.0;
        o = 2.0 * o;
        a.can_occ[a.cstart[b] + C] = o;
        part += o * (2.0 - o);
    }
    const double s = cta_sum(part, red);
    if (threadIdx.x == 0) a.scal[4 + b] = s;
}

// rho/kappa mixing with the previous iteration's matrices (HFBMix) and the
// block pairing energy -sum Delta_ij kappa_ij (HFBEnergy) with mixed kappa.
__global__ void __launch_bounds__(kThreads)
k_hfb_mix(double* rho, double* kappa, double* oldrho, double* oldkappa, const double* delta,
          const int* hsz, int nmax, double mix, int mix_rho, int mix_kappa, double* scal) {
    __shared__ double red[32];
    const int b = blockIdx.x;
    const int N = 2 * hsz[b];
    const long o0 = (long)b * nmax * nmax;
    double part = 0.0;
    for (int t = threadIdx.x; t < N * N; t += kThreads) {
        const long o = o0 + (t / N) * N + t % N;
        double r = rho[o], k = kappa[o];
        if (mix_rho) r = mix * r + (1.0 - mix) * oldrho[o];
        if (mix_kappa) k = mix * k + (1.0 - mix) * oldkappa[o];
        rho[o] = r;
        kappa[o] = k;
        oldrho[o] = r;
        oldkappa[o] = k;
        part = part - delta[o] * k;
    }
    const double s = cta_sum(part, red);
    if (threadIdx.x == 0) scal[b] = s;
}

size_t eval_smem(int N) {
    return (size_t)(N * (N + 1) + 5 * N) * sizeof(double) + (size_t)N * sizeof(int) + 64;
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
    if (2 * hmax > 128) return MG_ERR_ARG;  // one block matrix per CTA in shared memory
    H.hmax = hmax;
    H.nmax = 2 * hmax;
    H.members_h.assign(4 * hmax, 0);
    std::vector<int> cst(4);
    int acc = 0;
    for (int b = 0; b < 4; ++b) {
        for (int j = 0; j < H.hsz_h[b]; ++j) H.members_h[b * hmax + j] = lists[b][j];
        cst[b] = acc;
        acc += H.hsz_h[b];
    }
    const long nm2 = 4L * H.nmax * H.nmax, V = c->V;
    auto A = [&](double** p, long n) {
        return cudaMalloc(p, std::max(1L, n) * sizeof(double)) == cudaSuccess &&
               cudaMemset(*p, 0, std::max(1L, n) * sizeof(double)) == cudaSuccess;
    };
    H.gchunk = std::max(1, (2 * c->num_sms) / 4);
    bool ok = A(&H.rho, nm2) && A(&H.kappa, nm2) && A(&H.oldrho, nm2) && A(&H.oldkappa, nm2) &&
              A(&H.delta, nm2) && A(&H.qe, 4L * H.nmax) && A(&H.dfac, 2 * V) &&
              A(&H.pcut, nwt) && A(&H.ktil, 4L * hmax * hmax) && A(&H.fpart, 8 * V) &&
              A(&H.fre, 2 * V) && A(&H.fim, 2 * V) &&
              A(&H.gpart, 4L * H.gchunk * hmax * hmax) && A(&H.cantr, 4L * hmax * hmax) &&
              A(&H.occ, 4L * hmax) && A(&H.fermi_d, 2) && A(&H.trace_d, 4) && A(&H.scal_d, 16) &&
              cudaMalloc(&H.members, 4 * hmax * sizeof(int)) == cudaSuccess &&
              cudaMalloc(&H.hsz, 4 * sizeof(int)) == cudaSuccess &&
              cudaMalloc(&H.cstart, 4 * sizeof(int)) == cudaSuccess &&
              cudaMallocHost(&H.h_pinned, 32 * sizeof(double)) == cudaSuccess;
    if (!ok) return MG_ERR_CUDA;
    MG_CUDA(cudaMemcpy(H.members, H.members_h.data(), 4 * hmax * sizeof(int), cudaMemcpyHostToDevice));
    MG_CUDA(cudaMemcpy(H.hsz, H.hsz_h, 4 * sizeof(int), cudaMemcpyHostToDevice));
    MG_CUDA(cudaMemcpy(H.cstart, cst.data(), 4 * sizeof(int), cudaMemcpyHostToDevice));
    MG_TRY(pairing_set_smem(c));
    MG_CUDA(cudaFuncSetAttribute(k_hfb_eval, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    MG_CUDA(cudaFuncSetAttribute(k_rho_diag, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
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
    for (double* p : {H.rho, H.kappa, H.oldrho, H.oldkappa, H.delta, H.qe, H.dfac, H.pcut, H.ktil,
                      H.fpart, H.fre, H.fim, H.gpart, H.cantr, H.occ, H.fermi_d, H.trace_d, H.scal_d})
        if (p) cudaFree(p);
    for (int* p : {H.members, H.hsz, H.cstart})
        if (p) cudaFree(p);
    if (H.h_pinned) cudaFreeHost(H.h_pinned);
}

// SolvePairing for HFB (src/Pairing.f90:743-890, PairingIter 1).
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

    // ---- particle-number root finder -------------------------------------------
    EvalArgs ea{H.delta, c->bas[MG_HF_BASIS].e, H.members, H.hsz, H.hmax, H.nmax, H.fermi_d,
                H.rho, H.kappa, H.qe, H.trace_d, c->flags};
    const size_t sm = eval_smem(H.nmax);
    const double part0[2] = {c->p.neutrons, c->p.protons};
    double* hp = H.h_pinned;
    int evals = 0;
    auto evaluate = [&](const double* lam, double* f) -> int {
        hp[8] = lam[0];
        hp[9] = lam[1];
        MG_CUDA(cudaMemcpyAsync(H.fermi_d, hp + 8, 2 * sizeof(double), cudaMemcpyHostToDevice, c->stream));
        k_hfb_eval<<<4, kThreads, sm, c->stream>>>(ea);
        MG_LAUNCHED(c);
        MG_CUDA(cudaMemcpyAsync(hp, H.trace_d, 4 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
        MG_CUDA(cudaStreamSynchronize(c->stream));
        ++evals;
        f[0] = hp[0] + hp[1] - part0[0];
        f[1] = hp[2] + hp[3] - part0[1];
        if (std::isnan(f[0]) || std::isnan(f[1])) return MG_ERR_NAN;
        return MG_OK;
    };
    const double prec = H.pp.fermi_prec;
    double lam[2] = {H.fermi[0], H.fermi[1]}, f[2];
    MG_TRY(evaluate(lam, f));
    bool conv[2] = {std::fabs(f[0]) < prec, std::fabs(f[1]) < prec};
    double lo[2], hi[2], flo[2], fhi[2];
    bool has_lo[2] = {false, false}, has_hi[2] = {false, false};
    double plam[2], pf[2], slope[2];
    for (int it = 0; it < 2; ++it) {
        if (f[it] < 0) { lo[it] = lam[it]; flo[it] = f[it]; has_lo[it] = true; }
        else { hi[it] = lam[it]; fhi[it] = f[it]; has_hi[it] = true; }
        plam[it] = lam[it];
        pf[it] = f[it];
        slope[it] = H.slope[it] > 0.0 ? H.slope[it] : 0.0;
    }
    const int maxit = H.pp.max_iter > 0 ? H.pp.max_iter : 50;
    for (int k = 0; k < maxit && !(conv[0] && conv[1]); ++k) {
        for (int it = 0; it < 2; ++it) {
            if (conv[it]) continue;
            double next;
            if (slope[it] <= 0.0) {
                next = lam[it] + (f[it] < 0 ? 0.01 : -0.01);  // first probe, as the reference
            } else {
                double step = -f[it] / slope[it];
                step = std::max(-5.0, std::min(5.0, step));
                next = lam[it] + step;
            }
            if (has_lo[it] && has_hi[it] && !(next > lo[it] && next < hi[it]))
                next = 0.5 * (lo[it] + hi[it]);
            plam[it] = lam[it];
            pf[it] = f[it];
            lam[it] = next;
        }
        MG_TRY(evaluate(lam, f));
        for (int it = 0; it < 2; ++it) {
            if (conv[it]) continue;
            if (std::fabs(f[it]) < prec) { conv[it] = true; continue; }
            if (lam[it] != plam[it]) {
                const double s = (f[it] - pf[it]) / (lam[it] - plam[it]);
                if (s > 0.0) slope[it] = s;
            }
            if (f[it] < 0) { lo[it] = lam[it]; flo[it] = f[it]; has_lo[it] = true; }
            else { hi[it] = lam[it]; fhi[it] = f[it]; has_hi[it] = true; }
        }
    }
    (void)flo;
    (void)fhi;
    H.fermi[0] = lam[0];
    H.fermi[1] = lam[1];
    for (int it = 0; it < 2; ++it)
        if (slope[it] > 0.0) H.slope[it] = slope[it];
    for (int i = 0; i < 6; ++i) H.fermi_hist[i] = H.fermi_hist[i + 1];
    H.fermi_hist[6] = std::fabs(f[0]) > 0.9 || std::fabs(f[1]) > 0.9;
    bool lost = true;
    for (int i = 0; i < 7; ++i) lost = lost && H.fermi_hist[i];
    const double tr0 = hp[0] + hp[1], tr1 = hp[2] + hp[3];

    // ---- canonical basis, occupations, mixing, pairing energy ------------------
    OccArgs oa{H.rho, H.members, H.hsz, H.cstart, H.hmax, H.nmax, H.cantr,
               c->bas[MG_CAN_BASIS].occ, c->bas[MG_HF_BASIS].occ, H.scal_d, c->flags};
    k_rho_diag<<<4, kThreads, eval_smem(H.hmax), c->stream>>>(oa);
    MG_LAUNCHED(c);
    MG_TRY(canonical_transform(c));
    k_hfb_mix<<<4, kThreads, 0, c->stream>>>(H.rho, H.kappa, H.oldrho, H.oldkappa, H.delta, H.hsz,
                                           H.nmax, H.pp.mix, H.oldrho_zero ? 0 : 1, 1, H.scal_d);
    MG_LAUNCHED(c);
    H.oldrho_zero = false;
    MG_CUDA(cudaMemcpyAsync(hp + 16, H.scal_d, 8 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    int hflags[4];
    MG_CUDA(cudaMemcpyAsync(hflags, c->flags, 4 * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    MG_CUDA(cudaStreamSynchronize(c->stream));
    H.epair[0] = -0.5 * (hp[16] + hp[17]);
    H.epair[1] = -0.5 * (hp[18] + hp[19]);
    H.disp[0] = hp[20] + hp[21];
    H.disp[1] = hp[22] + hp[23];
    c->pairing_energy[0] = H.epair[0];
    c->pairing_energy[1] = H.epair[1];
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
    }
    if (hflags[1] || hflags[2]) return MG_NOT_CONVERGED;
    if (hflags[3]) return MG_ERR_STATE;  // occupation above one (src/HFB.f90:3392-3395)
    if (lost) return MG_ERR_STATE;       // particle number lost 7 times (src/HFB.f90:2154-2158)
    return MG_OK;
}

}  // namespace mg
