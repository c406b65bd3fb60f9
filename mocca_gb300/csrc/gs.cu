// gs.cu -- energy-ordered Gram-Schmidt of the HF basis, FP64.
//
// Replaces GramSchmidt (src/SpwfStorage.f90:372-480): per isospin, in
// ascending single-particle energy (OrderSpwfsISO, :795-848), normalise
// psi_k and remove its projection from every later spwf with the same
// parity and signature.  That modified Gram-Schmidt on an energy-ordered
// block equals, in exact arithmetic, Q = Psi R^{-1} with S = R^T R the
// Cholesky factorisation of the block's overlap matrix S = dv Psi^T Psi.
// The GPU form is therefore three passes per (isospin, parity, signature)
// block instead of nb^2 sequential dot/axpy sweeps:
//   k_gs_order    : stable insertion sort of each block by energy (device)
//   k_gs_overlap  : S partial sums over point chunks (block-owned, deterministic)
//   k_gs_sum      : chunk partials of S summed in order, one entry per thread
//   k_gs_factor   : S = R^T R, X = R^{-1} (one block per CTA, in smem)
//   k_gs_apply    : psi'_l = sum_{k<=l} X_kl psi_k in place (+ update history)
// For the near-orthonormal input of an imaginary-time step cond(S) ~ 1, so
// the Cholesky form keeps full FP64 accuracy.  In the mixed form the overlap
// and the apply run on the tensor cores instead (meshgemm_tc.cu); the sum, the
// factorisation and the order stay these FP64 kernels.
#include "mg_internal.cuh"

namespace mg {

namespace {

constexpr int kThreads = 256;
constexpr int kPts = 64;  // points per shared-memory tile

// gs_index layout: [0..nblk] block starts, then member lists (nwt ints) in
// index order (static), then the energy-ordered lists (nwt ints).  One CTA
// per block; member i goes to its rank in (energy, list position) order, a
// stable sort (NaN energies sort last, in list order).
__global__ void k_gs_order(const int* __restrict__ lists, int nblk, int nwt,
                           const double* __restrict__ e, int* __restrict__ ordered) {
    extern __shared__ double se[];
    const int b = blockIdx.x;
    const int s0 = lists[b], nb = lists[b + 1] - s0;
    const int* mem = lists + nblk + 1 + s0;
    for (int i = threadIdx.x; i < nb; i += blockDim.x) se[i] = e[mem[i]];
    __syncthreads();
    for (int i = threadIdx.x; i < nb; i += blockDim.x) {
        const double ei = se[i];
        const bool ni = isnan(ei);
        int rank = 0;
        for (int j = 0; j < nb; ++j) {
            const double ej = se[j];
            const bool nj = isnan(ej);
            const bool before = (!ni && !nj) ? (ej < ei || (ej == ei && j < i))
                                             : (nj == ni ? j < i : !nj);
            rank += before ? 1 : 0;
        }
        ordered[s0 + rank] = mem[i];
    }
}

// Upper-triangle overlap partial sums: part[(b*nchunk + chunk)*nbmax^2 + k*nbmax + l]
__global__ void __launch_bounds__(kThreads)
k_gs_overlap(const double* __restrict__ psi, const int* __restrict__ starts,
             const int* __restrict__ ordered, int nbmax, long V4, int nchunk,
             double* __restrict__ part) {
    extern __shared__ double sm[];
    const int b = blockIdx.y, chunk = blockIdx.x;
    const int s0 = starts[b], nb = starts[b + 1] - s0;
    if (nb == 0) return;
    const int npair = nb * (nb + 1) / 2;
    double* tile = sm;                 // nb * kPts
    double* acc = sm + nb * kPts;      // npair accumulators
    for (int t = threadIdx.x; t < npair; t += kThreads) acc[t] = 0.0;
    const long per = (V4 + nchunk - 1) / nchunk;
    const long p0 = (long)chunk * per, p1 = min(V4, p0 + per);
    for (long base = p0; base < p1; base += kPts) {
        __syncthreads();
        for (int t = threadIdx.x; t < nb * kPts; t += kThreads) {
            const int k = t / kPts, q = t % kPts;
            const long pt = base + q;
            tile[t] = pt < p1 ? psi[(long)ordered[s0 + k] * V4 + pt] : 0.0;
        }
        __syncthreads();
        for (int pr = threadIdx.x; pr < npair; pr += kThreads) {
            // pair index -> (k, l), k <= l, row-major over the upper triangle
            int k = 0, rem = pr;
            while (rem >= nb - k) { rem -= nb - k; ++k; }
            const int l = k + rem;
            const double* a = tile + k * kPts;
            const double* c = tile + l * kPts;
            double s = acc[pr];
#pragma unroll 8
            for (int q = 0; q < kPts; ++q) s = fma(a[q], c[q], s);
            acc[pr] = s;
        }
    }
    __syncthreads();
    double* out = part + ((long)b * nchunk + chunk) * nbmax * nbmax;
    for (int pr = threadIdx.x; pr < npair; pr += kThreads) {
        int k = 0, rem = pr;
        while (rem >= nb - k) { rem -= nb - k; ++k; }
        out[k * nbmax + k + rem] = acc[pr];
    }
}

// Sum the chunk partials of the upper triangle, one warp per entry: lane j
// adds chunks j, j + 32, ... in order, then a fixed xor tree combines the
// lanes (deterministic); the result goes to chunk slot 0.
__global__ void k_gs_sum(double* __restrict__ part, int nbmax, int nchunk) {
    const int b = blockIdx.y;
    const int t = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
    const int lane = threadIdx.x & 31;
    if (t >= nbmax * nbmax || t / nbmax > t % nbmax) return;
    double* pb = part + (long)b * nchunk * nbmax * nbmax;
    double s = 0.0;
    for (int q = lane; q < nchunk; q += 32) s += pb[(long)q * nbmax * nbmax + t];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    __syncwarp();
    if (lane == 0) pb[t] = s;
}

// Cholesky S = R^T R (R upper), X = R^{-1}; X to xout[b].
__global__ void __launch_bounds__(kThreads)
k_gs_factor(const double* __restrict__ part, const int* __restrict__ starts, int nbmax,
            int nchunk, double dv, double* __restrict__ xout, int* __restrict__ flag) {
    // S = L D L^T by symmetric elimination (L unit lower, D the pivots), so
    // that R = D^(1/2) L^T; the same row operations applied to the identity
    // leave W = L^(-1), and X = R^(-1) = W^T D^(-1/2) needs no back
    // substitution.  GB300 issues a warp's FP64 instruction over ~16 clocks
    // and a divide or square root is a sequence of them, so each pivot's
    // reciprocal and reciprocal square root are taken once, by one thread.
    extern __shared__ double sm[];
    const int b = blockIdx.x;
    const int nb = starts[b + 1] - starts[b];
    if (nb == 0) return;
    double* S = sm;              // nb x nb (upper used)
    double* W = sm + nb * nb;    // nb x nb (lower used), L^(-1)
    __shared__ double rsq[256];  // D^(-1/2)
    __shared__ double u[256];
    __shared__ double inv_d;
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    constexpr int kWarps = kThreads / 32;
    for (int t = threadIdx.x; t < nb * nb; t += kThreads) {
        const int k = t / nb, l = t % nb;
        S[t] = k <= l ? part[(long)b * nchunk * nbmax * nbmax + k * nbmax + l] * dv : 0.0;
        W[t] = k == l ? 1.0 : 0.0;
    }
    __syncthreads();
    for (int j = 0; j < nb; ++j) {
        if (threadIdx.x == 0) {
            const double d = S[j * nb + j];
            if (!(d > 0.0)) atomicExch(flag, 1);
            const double dd = fmax(d, 1e-300);
            inv_d = 1.0 / dd;
            rsq[j] = 1.0 / sqrt(dd);
        }
        __syncthreads();
        // pivot row scaled once (u_k = S_jk / S_jj), then one FMA per entry
        // of the trailing upper triangle and of W's rows below j, a warp per row
        const double id = inv_d;
        for (int k = j + 1 + threadIdx.x; k < nb; k += kThreads) u[k] = S[j * nb + k] * id;
        __syncthreads();
        for (int k = j + 1 + warp; k < nb; k += kWarps) {
            const double uk = u[k];
            for (int l = k + lane; l < nb; l += 32) S[k * nb + l] = fma(-uk, S[j * nb + l], S[k * nb + l]);
            for (int l = lane; l <= j; l += 32) W[k * nb + l] = fma(-uk, W[j * nb + l], W[k * nb + l]);
        }
        __syncthreads();
    }
    // X[i][j] = W[j][i] d_j^(-1/2) (i <= j), zero below the diagonal
    double* xo = xout + (long)b * nbmax * nbmax;
    for (int t = threadIdx.x; t < nb * nb; t += kThreads) {
        const int i = t / nb, j = t % nb;
        xo[i * nbmax + j] = i <= j ? W[j * nb + i] * rsq[j] : 0.0;
    }
}

// psi'_l = sum_{k<=l} X[k][l] psi_k over a chunk of points, in place; when
// upd != NULL also upd_l = psi'_l - upd_l (GradDesc history,
// src/ImaginaryTime.f90:496-499).
__global__ void __launch_bounds__(kThreads)
k_gs_apply(double* __restrict__ psi, double* __restrict__ upd, const int* __restrict__ starts,
           const int* __restrict__ ordered, const double* __restrict__ xin, int nbmax, long V4) {
    extern __shared__ double sm[];
    const int b = blockIdx.y;
    const int s0 = starts[b], nb = starts[b + 1] - s0;
    if (nb == 0) return;
    double* X = sm;               // nb x nb
    double* tile = sm + nb * nb;  // nb x kPts
    const double* xg = xin + (long)b * nbmax * nbmax;
    for (int t = threadIdx.x; t < nb * nb; t += kThreads) X[t] = xg[(t / nb) * nbmax + t % nb];
    const long base = (long)blockIdx.x * kPts;
    for (int t = threadIdx.x; t < nb * kPts; t += kThreads) {
        const int k = t / kPts, q = t % kPts;
        const long pt = base + q;
        tile[t] = pt < V4 ? psi[(long)ordered[s0 + k] * V4 + pt] : 0.0;
    }
    __syncthreads();
    for (int t = threadIdx.x; t < nb * kPts; t += kThreads) {
        const int l = t / kPts, q = t % kPts;
        const long pt = base + q;
        if (pt >= V4) continue;
        double s = 0.0;
        for (int k = 0; k <= l; ++k) s = fma(X[k * nb + l], tile[k * kPts + q], s);
        const long o = (long)ordered[s0 + l] * V4 + pt;
        psi[o] = s;
        if (upd) upd[o] = s - upd[o];
    }
}

}  // namespace

// Block lists (isospin, parity, signature) from the quantum numbers; they
// are static for a run, so they are built once and kept on the device.
static int gs_prepare(mg_ctx* c) {
    Basis& B = c->bas[MG_HF_BASIS];
    std::vector<int> keys;
    std::vector<std::vector<int>> members;
    for (int i = 0; i < c->p.nwt; ++i) {
        const int key = (B.h_qn[4 * i] + 2) * 100 + (B.h_qn[4 * i + 1] + 2) * 10 +
                        (B.h_qn[4 * i + 2] + 2);
        size_t k = 0;
        while (k < keys.size() && keys[k] != key) ++k;
        if (k == keys.size()) { keys.push_back(key); members.emplace_back(); }
        members[k].push_back(i);
    }
    const int nblk = (int)keys.size();
    std::vector<int> lists(nblk + 1 + c->p.nwt);
    int nbmax = 0, pos = 0;
    for (int b = 0; b < nblk; ++b) {
        lists[b] = pos;
        for (int i : members[b]) lists[nblk + 1 + pos++] = i;
        nbmax = std::max(nbmax, (int)members[b].size());
    }
    lists[nblk] = pos;
    if (2L * nbmax * nbmax * (long)sizeof(double) > 220L * 1024) return MG_ERR_ARG;
    c->gs_nblk = nblk;
    c->gs_nbmax = nbmax;
    c->gs_nchunk = std::max(1, 2 * c->num_sms / nblk);
    c->gs_lists_len = (int)lists.size();
    if (c->gs_index) cudaFree(c->gs_index);
    if (c->gs_S) cudaFree(c->gs_S);
    if (c->gs_R) cudaFree(c->gs_R);
    MG_CUDA(cudaMalloc(&c->gs_index, (lists.size() + c->p.nwt) * sizeof(int)));
    MG_CUDA(cudaMalloc(&c->gs_S, (size_t)nblk * c->gs_nchunk * nbmax * nbmax * sizeof(double)));
    MG_CUDA(cudaMalloc(&c->gs_R, (size_t)nblk * nbmax * nbmax * sizeof(double)));
    MG_CUDA(cudaMemcpy(c->gs_index, lists.data(), lists.size() * sizeof(int),
                       cudaMemcpyHostToDevice));
    MG_CUDA(cudaFuncSetAttribute(k_gs_overlap, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024));
    MG_CUDA(cudaFuncSetAttribute(k_gs_factor, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024));
    MG_CUDA(cudaFuncSetAttribute(k_gs_apply, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024));
    return MG_OK;
}

int gram_schmidt_impl(mg_ctx* c, double* upd) {
    Basis& B = c->bas[MG_HF_BASIS];
    if (!B.have_qn) return MG_ERR_STATE;
    if (c->gs_nblk == 0) MG_TRY(gs_prepare(c));
    const int nblk = c->gs_nblk, nbmax = c->gs_nbmax, nchunk = c->gs_nchunk;
    const long V4 = 4 * c->V;
    const int* d_lists = c->gs_index;
    int* d_ordered = c->gs_index + c->gs_lists_len;
    k_gs_order<<<nblk, 128, nbmax * sizeof(double), c->stream>>>(d_lists, nblk, c->p.nwt, B.e,
                                                                 d_ordered);
    MG_LAUNCHED(c);
    const size_t sm_f = (size_t)(2 * nbmax * nbmax) * sizeof(double);
    if (c->cur_precision == MG_MIXED && gs_tc_prepare(c)) {
        // mixed form: the overlap and the apply on the tensor cores (meshgemm_tc.cu)
        const int nct = c->gs_nchunk_tc;
        MG_TRY(gs_overlap_tc(c, B.psi, d_lists, d_ordered));
        k_gs_sum<<<dim3(div_up((long)nbmax * nbmax, kThreads / 32), nblk), kThreads, 0,
                   c->stream>>>(c->gs_Stc, nbmax, nct);
        MG_LAUNCHED(c);
        k_gs_factor<<<nblk, kThreads, sm_f, c->stream>>>(c->gs_Stc, d_lists, nbmax, nct, c->dv,
                                                         c->gs_R, c->flags);
        MG_LAUNCHED(c);
        return gs_apply_tc(c, B.psi, upd, d_lists, d_ordered);
    }
    const int npair_max = nbmax * (nbmax + 1) / 2;
    const size_t sm_ov = (size_t)(nbmax * kPts + npair_max) * sizeof(double);
    const size_t sm_ap = (size_t)(nbmax * nbmax + nbmax * kPts) * sizeof(double);
    k_gs_overlap<<<dim3(nchunk, nblk), kThreads, sm_ov, c->stream>>>(B.psi, d_lists, d_ordered,
                                                                      nbmax, V4, nchunk, c->gs_S);
    MG_LAUNCHED(c);
    k_gs_sum<<<dim3(div_up((long)nbmax * nbmax, kThreads / 32), nblk), kThreads, 0,
               c->stream>>>(c->gs_S, nbmax, nchunk);
    MG_LAUNCHED(c);
    k_gs_factor<<<nblk, kThreads, sm_f, c->stream>>>(c->gs_S, d_lists, nbmax, nchunk, c->dv,
                                                     c->gs_R, c->flags);
    MG_LAUNCHED(c);
    k_gs_apply<<<dim3(div_up(V4, kPts), nblk), kThreads, sm_ap, c->stream>>>(
        B.psi, upd, d_lists, d_ordered, c->gs_R, nbmax, V4);
    MG_LAUNCHED(c);
    return MG_OK;
}

int gram_schmidt(mg_ctx* c) { return gram_schmidt_impl(c, nullptr); }

}  // namespace mg
