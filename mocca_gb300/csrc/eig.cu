// eig.cu -- batched symmetric eigensolver for the small dense HFB matrices.
//
// GB300 runs FP64 at ~1.75 FMA/clk/SM and long dependent FP64 chains (the
// tridiagonal QL sweeps of a Householder/QL solver such as diagoncr8,
// src/HFB.f90:5880-6087) at a small fraction of that, so the FP64 work is
// arranged as batched GEMMs and the sequential part runs in FP32:
//
//   1. k_jacobi32: cyclic two-sided Jacobi in FP32, one CTA per matrix, the
//      n/2 rotations of a round-robin round applied in parallel (rows, then
//      columns and vectors), optionally warm-started from earlier vectors
//      (B = X^T A X).  Eigenpairs sorted ascending.
//   2. FP64 iterative refinement (Ogita & Aishima, "Iterative refinement for
//      symmetric eigenvalue decomposition", Japan J. Indust. Appl. Math. 35
//      (2018) 1007-1035):  R = I - X^T X, S = X^T A X, lambda_i = s_ii/(1-r_ii),
//      E_ij = (s_ij + lambda_j r_ij)/(lambda_j - lambda_i) for separated
//      pairs, r_ij/2 inside clusters (|lambda_i - lambda_j| <= delta),
//      X <- X (I + E).  Each step is three batched FP64 GEMM launches plus one
//      correction launch, quadratically convergent from the FP32 seed.
//
// The result has FP64 accuracy: eigenvalues to ~1e-15 relative, and the
// invariant subspaces to the same level; inside an exactly degenerate
// cluster any orthonormal basis of the cluster is returned (the HFB density
// matrices are projector blocks and do not depend on that choice).
#include <cmath>
#include <mutex>

#include "df.cuh"
#include "mg_internal.cuh"

namespace mg {

namespace {

constexpr int kThreads = 256;
constexpr int kTile = 16;
// Jacobi kernels: one CTA per matrix, so the whole SM's warps work on its
// rounds (128 lanes for the columns / rows x 8 groups of rotation pairs)
constexpr int kJThreads = 1024;
constexpr int kJGroups = kJThreads / 128;
// largest matrix whose FP32 Jacobi keeps its warm-start scratch in shared
// memory (3 planes of n x (n+1) floats)
constexpr int kJSmemMax = 128;
// dynamic shared memory the Jacobi kernels opt in to: their largest need,
// two float planes (FP32 seed) or one double plane (FP64 polish) of
// kEigMax x (kEigMax + 1) -- 206 KB, which leaves room for their static arrays
constexpr int kSmemOptIn = kEigMax * (kEigMax + 1) * 8;
// FP32 Jacobi seed: couplings at or below kJacobiSkip |A|_F do not rotate
// (at 1e-8, a cold seed of clusters split by 1e-10 left the FP64 polish
// churning past its sweep cap; 1e-9 keeps most of the skipped rounds)
constexpr float kJacobiSkip = 1e-9f;

__device__ float cta_sumf(float x, float* red) {
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    __syncthreads();
    if (threadIdx.x % 32 == 0) red[threadIdx.x / 32] = x;
    __syncthreads();
    float s = 0.0f;
    for (int w = 0; w < (int)(blockDim.x / 32); ++w) s += red[w];
    __syncthreads();
    return s;
}

__device__ double cta_sumd(double x, double* red) {
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    __syncthreads();
    if (threadIdx.x % 32 == 0) red[threadIdx.x / 32] = x;
    __syncthreads();
    double s = 0.0;
    for (int w = 0; w < (int)(blockDim.x / 32); ++w) s += red[w];
    __syncthreads();
    return s;
}

// round-robin tournament: in round r, slot j of n (n even) holds player f(j);
// pairs (f(i), f(n-1-i)), i < n/2, cover every pair once in n-1 rounds.
__device__ __forceinline__ int rr_player(int j, int r, int n) {
    return j == 0 ? 0 : 1 + (j - 1 + r) % (n - 1);
}

// The round in which players p < q meet: q mod m for p = 0, else
// (p + q) (m + 1) / 2 mod m (m = n - 1 is odd, so 2 is invertible mod m).
__device__ __forceinline__ int rr_round(int p, int q, int n) {
    const int m = n - 1;
    return p == 0 ? q % m : ((p + q) * ((m + 1) / 2)) % m;
}

}  // namespace

// C = op(A) B for n x n FP32 matrices in shared memory (leading dimension
// ld), op(A) = A or A^T.  Each thread holds a 4 x 4 register tile: rows
// 4 it .. 4 it + 3 and columns jt + m nq (m = 0..3), so that a warp's loads
// of B's row k are consecutive words and its loads of A are broadcasts.  The
// sums run over k in order with fused multiply-adds.
__device__ void smem_mm32(const float* A, const float* B, float* C, int n, int ld, bool transA) {
    const int nq = (n + 3) / 4;
    for (int t = threadIdx.x; t < nq * nq; t += blockDim.x) {
        const int it = t / nq, jt = t % nq;
        float acc[4][4];
#pragma unroll
        for (int r = 0; r < 4; ++r)
#pragma unroll
            for (int m = 0; m < 4; ++m) acc[r][m] = 0.0f;
        for (int k = 0; k < n; ++k) {
            float x[4], y[4];
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                const int i = 4 * it + r;
                x[r] = i < n ? (transA ? A[k * ld + i] : A[i * ld + k]) : 0.0f;
            }
#pragma unroll
            for (int m = 0; m < 4; ++m) {
                const int j = jt + m * nq;
                y[m] = j < n ? B[k * ld + j] : 0.0f;
            }
#pragma unroll
            for (int r = 0; r < 4; ++r)
#pragma unroll
                for (int m = 0; m < 4; ++m) acc[r][m] = fmaf(x[r], y[m], acc[r][m]);
        }
#pragma unroll
        for (int r = 0; r < 4; ++r)
#pragma unroll
            for (int m = 0; m < 4; ++m) {
                const int i = 4 * it + r, j = jt + m * nq;
                if (i < n && j < n) C[i * ld + j] = acc[r][m];
            }
    }
}

// One matrix per CTA.  A: FP64 n x n (lda) input; Xw: optional FP64 warm
// start (n x n, ldx); X: FP64 output vectors (n x n, ldx, column k <-> w[k]);
// w: eigenvalues ascending.  n <= kEigMax.  Above kJSmemMax the warm start's
// product A V goes through X (FP64) instead of a third shared-memory plane;
// Xw may alias X, whose contents are in v by then.
//
// A round-robin round's n/2 rotations J act on disjoint index pairs, so
// A <- J^T A J splits into (n/2)^2 independent 2 x 2 blocks (rows of pair i,
// columns of pair j): each thread rotates its blocks' rows, then their
// columns, in registers, one pass over the matrix per round; V <- V J is the
// same pass over V's rows.  A pair rotates when its coupling is above
// kJacobiSkip |A| (FP32 rounding of the matrix entries is ~6e-8 |A|); a
// round without such a pair is skipped, which makes the later sweeps of a
// warm start cheap.
__global__ void __launch_bounds__(kJThreads)
k_jacobi32(const double* __restrict__ A, long astride, int lda, const int* __restrict__ nsz,
           const double* Xw, double* X, long xstride, int ldx,
           double* __restrict__ w, long wstride, int max_sweeps, int* __restrict__ flag) {
    extern __shared__ float smf[];
    __shared__ float red[32];
    __shared__ float4 prm[kEigMax / 2];   // c, s, p, q (index bits) of the round's pairs
    __shared__ int perm[kEigMax];
    const int b = blockIdx.x;
    const int n0 = nsz[b];
    if (n0 == 0) return;
    const int n = n0 + (n0 & 1);  // pad odd sizes with an isolated zero row
    const int ld = n + 1;
    float* a = smf;             // n x ld
    float* v = a + n * ld;      // n x ld
    float* t = n <= kJSmemMax ? v + n * ld : nullptr;   // n x ld scratch
    const double* Ab = A + b * astride;
    const int tid = threadIdx.x;
    for (int q = tid; q < n * n; q += kJThreads) {
        const int i = q / n, j = q % n;
        a[i * ld + j] = (i < n0 && j < n0) ? (float)Ab[(long)i * lda + j] : 0.0f;
        float vv = i == j ? 1.0f : 0.0f;
        if (Xw && i < n0 && j < n0) vv = (float)Xw[b * xstride + (long)i * ldx + j];
        v[i * ld + j] = vv;
    }
    __syncthreads();
    if (Xw && t) {
        // a <- V^T A V
        smem_mm32(a, v, t, n, ld, false);
        __syncthreads();
        smem_mm32(v, t, a, n, ld, true);
        __syncthreads();
    } else if (Xw) {
        // the same through X: the padding row and column of A V and of
        // V^T A V are zero (A's padding is zero, V's is the identity)
        double* tg = X + b * xstride;
        for (int q = tid; q < n0 * n0; q += kJThreads) {
            const int i = q / n0, j = q % n0;
            float s = 0.0f;
            for (int k = 0; k < n0; ++k) s = fmaf(a[i * ld + k], v[k * ld + j], s);
            tg[(long)i * ldx + j] = (double)s;
        }
        __syncthreads();
        for (int q = tid; q < n0 * n0; q += kJThreads) {
            const int i = q / n0, j = q % n0;
            float s = 0.0f;
            for (int k = 0; k < n0; ++k) s = fmaf(v[k * ld + i], (float)tg[(long)k * ldx + j], s);
            a[i * ld + j] = s;
        }
        __syncthreads();
    }
    if (Xw) {
        // symmetrise
        for (int q = tid; q < n * n; q += kJThreads) {
            const int i = q / n, j = q % n;
            if (i < j) {
                const float m = 0.5f * (a[i * ld + j] + a[j * ld + i]);
                a[i * ld + j] = m;
                a[j * ld + i] = m;
            }
        }
        __syncthreads();
    }
    const int half = n / 2;
    float part = 0.0f;
    for (int q = tid; q < n * n; q += kJThreads) {
        const float x = a[(q / n) * ld + q % n];
        part += x * x;
    }
    const float norm2 = cta_sumf(part, red);
    const float tol2 = 1e-11f * norm2;  // off-diagonal <= 3e-6 |A|: an FP32-level seed
    const float thr = kJacobiSkip * sqrtf(norm2);
    int sweep = 0;
    for (; sweep < max_sweeps; ++sweep) {
        part = 0.0f;
        for (int q = tid; q < n * n; q += kJThreads) {
            const int i = q / n, j = q % n;
            if (i != j) part += a[i * ld + j] * a[i * ld + j];
        }
        const float off = cta_sumf(part, red);
        if (off <= tol2) break;
        for (int r = 0; r < n - 1; ++r) {
            int on = 0;
            if (tid < half) {
                const int p = rr_player(tid, r, n), q = rr_player(n - 1 - tid, r, n);
                const float apq = a[p * ld + q];
                float c = 1.0f, s = 0.0f;
                if (fabsf(apq) > thr) {
                    const float th = (a[q * ld + q] - a[p * ld + p]) / (2.0f * apq);
                    const float tt = (th >= 0.0f ? 1.0f : -1.0f) / (fabsf(th) + sqrtf(th * th + 1.0f));
                    c = rsqrtf(tt * tt + 1.0f);
                    s = tt * c;
                    on = 1;
                }
                prm[tid] = make_float4(c, s, __int_as_float(p), __int_as_float(q));
            }
            if (!__syncthreads_or(on)) continue;
            for (int u = tid; u < half * half; u += kJThreads) {
                const float4 R = prm[u / half], Cc = prm[u % half];
                float* ap = a + __float_as_int(R.z) * ld;
                float* aq = a + __float_as_int(R.w) * ld;
                const int jp = __float_as_int(Cc.z), jq = __float_as_int(Cc.w);
                const float x00 = ap[jp], x01 = ap[jq], x10 = aq[jp], x11 = aq[jq];
                // rows of pair i, then columns of pair j
                const float r00 = R.x * x00 - R.y * x10, r10 = R.y * x00 + R.x * x10;
                const float r01 = R.x * x01 - R.y * x11, r11 = R.y * x01 + R.x * x11;
                ap[jp] = Cc.x * r00 - Cc.y * r01;
                ap[jq] = Cc.y * r00 + Cc.x * r01;
                aq[jp] = Cc.x * r10 - Cc.y * r11;
                aq[jq] = Cc.y * r10 + Cc.x * r11;
            }
            for (int u = tid; u < n * half; u += kJThreads) {
                const float4 Cc = prm[u / n];
                float* vr = v + (u % n) * ld;
                const int jp = __float_as_int(Cc.z), jq = __float_as_int(Cc.w);
                const float vp = vr[jp], vq = vr[jq];
                vr[jp] = Cc.x * vp - Cc.y * vq;
                vr[jq] = Cc.y * vp + Cc.x * vq;
            }
            __syncthreads();
        }
    }
    if (sweep == max_sweeps && tid == 0 && flag) atomicExch(flag, 1);
    // sort the n0 real eigenpairs ascending, ties by index (the padding row
    // stays last): rank of each diagonal entry; perm starts as the identity
    // so that it stays a valid index table whatever the values
    for (int i = tid; i < n0; i += kJThreads) perm[i] = i;
    __syncthreads();
    for (int i = tid; i < n0; i += kJThreads) {
        const float di = a[i * ld + i];
        int rank = 0;
        for (int j = 0; j < n0; ++j) {
            const float dj = a[j * ld + j];
            rank += (dj < di || (dj == di && j < i)) ? 1 : 0;
        }
        if (rank < n0) perm[rank] = i;
    }
    __syncthreads();
    for (int q = tid; q < n0 * n0; q += kJThreads) {
        const int i = q / n0, col = q % n0;
        X[b * xstride + (long)i * ldx + col] = (double)v[i * ld + perm[col]];
    }
    for (int k = tid; k < n0; k += kJThreads) w[b * wstride + k] = (double)a[perm[k] * ld + perm[k]];
}

// Early exit of the refinement steps (EigBatch::skip_tol).  Step s of
// matrix b is skipped when done[b] <= s.  The first launch of step s (decide)
// sets done[b] = s when step s - 1 saw |S - diag S|_F <= tol |A|_F: its
// correction already left every off-diagonal element at ~tol^2 |A|^2 / gap,
// clusters included.  Every CTA of the deciding launch reads the same value
// and so takes the same branch; the later launches of the step read done[b].
struct SkipCtl {
    int* done;              // nullptr: no early exit
    const double* offrel;   // nb: |S - diag S|_F / |A|_F of the last step run
    int step, decide;
    double tol;
};

__device__ __forceinline__ bool skip_step(const SkipCtl& k, int b) {
    if (k.done == nullptr) return false;
    if (k.done[b] <= k.step) return true;
    if (!k.decide || k.step == 0) return false;
    if (!(k.offrel[b] <= k.tol)) return false;
    if (blockIdx.x == 0 && threadIdx.x == 0) k.done[b] = k.step;
    return true;
}

// Batched FP64 GEMM, C = alpha op(A) op(B) + beta C, k <= kEigMax, row-major.
// With g.sym (C symmetric, and C itself when beta != 0) only the upper
// triangle is computed and written to both halves, which also makes C
// exactly symmetric.
__global__ void __launch_bounds__(kThreads) k_gemm64(const GemmDesc* __restrict__ descs,
                                                     SkipCtl sk) {
    __shared__ double sA[kTile][kEigMax + 1];
    __shared__ double sB[kEigMax + 1][kTile + 1];
    const GemmDesc g = descs[blockIdx.y];
    if (skip_step(sk, g.mat)) return;
    const int tiles_n = (g.n + kTile - 1) / kTile;
    const int ti = blockIdx.x / tiles_n, tj = blockIdx.x % tiles_n;
    if (ti * kTile >= g.m || (g.sym && ti > tj)) return;
    const int r = threadIdx.x / kTile, cidx = threadIdx.x % kTile;
    // tile loads with the fastest thread index along the operand's contiguous
    // dimension (transposed operands included), so that a warp reads
    // consecutive words
    for (int q = threadIdx.x; q < kTile * g.k; q += kThreads) {
        int i, kk;
        if (g.ta) { i = q % kTile; kk = q / kTile; }
        else { i = q / g.k; kk = q % g.k; }
        const int gi = ti * kTile + i;
        double x = 0.0;
        if (gi < g.m) x = g.ta ? g.A[(long)kk * g.lda + gi] : g.A[(long)gi * g.lda + kk];
        sA[i][kk] = x;
    }
    for (int q = threadIdx.x; q < kTile * g.k; q += kThreads) {
        int kk, j;
        if (g.tb) { kk = q % g.k; j = q / g.k; }
        else { kk = q / kTile; j = q % kTile; }
        const int gj = tj * kTile + j;
        double x = 0.0;
        if (gj < g.n) x = g.tb ? g.B[(long)gj * g.ldb + kk] : g.B[(long)kk * g.ldb + gj];
        sB[kk][j] = x;
    }
    __syncthreads();
    const int gi = ti * kTile + r, gj = tj * kTile + cidx;
    if (gi >= g.m || gj >= g.n) return;
    if (g.sym && gi > gj) return;   // the mirror of an entry another thread writes
    double s = 0.0;
    for (int kk = 0; kk < g.k; ++kk) s = fma(sA[r][kk], sB[kk][cidx], s);
    double* c = g.C + (long)gi * g.ldc + gj;
    const double v = g.beta == 0.0 ? g.alpha * s : fma(g.alpha, s, g.beta * *c);
    *c = v;
    if (g.sym && gi < gj) g.C[(long)gj * g.ldc + gi] = v;
}

// The same GEMMs in double-float arithmetic for the mixed form: operands
// split into FP32 pairs at the tile load (integer instructions, df_split),
// products and sums with the exact FP32 error terms (df_acc, ~11 FP32
// instructions per term), one FP64 add per output.  ~1e-14 relative like
// the mixed form's Jacobi polish, at several times the rate of the FP64
// pipe, which bounds k_gemm64 on GB300.
__global__ void __launch_bounds__(kThreads) k_gemm_df(const GemmDesc* __restrict__ descs,
                                                      SkipCtl sk) {
    __shared__ float2 sA[kTile][kEigMax + 1];
    __shared__ float2 sB[kEigMax + 1][kTile + 1];
    const GemmDesc g = descs[blockIdx.y];
    if (skip_step(sk, g.mat)) return;
    const int tiles_n = (g.n + kTile - 1) / kTile;
    const int ti = blockIdx.x / tiles_n, tj = blockIdx.x % tiles_n;
    if (ti * kTile >= g.m || (g.sym && ti > tj)) return;
    const int r = threadIdx.x / kTile, cidx = threadIdx.x % kTile;
    for (int q = threadIdx.x; q < kTile * g.k; q += kThreads) {
        int i, kk;
        if (g.ta) { i = q % kTile; kk = q / kTile; }
        else { i = q / g.k; kk = q % g.k; }
        const int gi = ti * kTile + i;
        double x = 0.0;
        if (gi < g.m) x = g.ta ? g.A[(long)kk * g.lda + gi] : g.A[(long)gi * g.lda + kk];
        const dfl d = df_split(x);
        sA[i][kk] = make_float2(d.h, d.l);
    }
    for (int q = threadIdx.x; q < kTile * g.k; q += kThreads) {
        int kk, j;
        if (g.tb) { kk = q % g.k; j = q / g.k; }
        else { kk = q / kTile; j = q % kTile; }
        const int gj = tj * kTile + j;
        double x = 0.0;
        if (gj < g.n) x = g.tb ? g.B[(long)gj * g.ldb + kk] : g.B[(long)kk * g.ldb + gj];
        const dfl d = df_split(x);
        sB[kk][j] = make_float2(d.h, d.l);
    }
    __syncthreads();
    const int gi = ti * kTile + r, gj = tj * kTile + cidx;
    if (gi >= g.m || gj >= g.n) return;
    if (g.sym && gi > gj) return;
    float sh = 0.0f, sl = 0.0f;
    for (int kk = 0; kk < g.k; ++kk) {
        const float2 a = sA[r][kk], b = sB[kk][cidx];
        df_acc(sh, sl, dfl{a.x, a.y}, dfl{b.x, b.y});
    }
    const double s = df_to_fast(dfl{sh, sl});
    double* c = g.C + (long)gi * g.ldc + gj;
    const double v = g.beta == 0.0 ? g.alpha * s : fma(g.alpha, s, g.beta * *c);
    *c = v;
    if (g.sym && gi < gj) g.C[(long)gj * g.ldc + gi] = v;
}

// Ogita-Aishima correction, spread over one CTA per matrix row so that the
// FP64 work (divisions included) runs on many SMs.  k_oa_rows: lambda_i =
// s_ii / g_ii (into w) and the row sums of (S - diag lambda)^2 and
// (I - G)^2; k_oa_apply: delta from those sums (every CTA of a matrix adds
// them in the same order; row 0 records |S - diag S|_F / |A|_F in offrel),
// then row i of F = I + E written over row i of G,
// and emax(i) = max |S_ij| / |lambda_i - lambda_j| over the pairs whose
// eigenvalue estimates have opposite signs: the rotation angle by which the
// vectors still miss the split of the space into its positive and negative
// parts (the refinement leaves pairs inside a cluster |lambda_i - lambda_j|
// <= delta unrotated, so a start too far away shows here and not in E).
__global__ void __launch_bounds__(128)
k_oa_rows(const double* __restrict__ S, const double* __restrict__ G, long stride, int ld,
          const int* __restrict__ nsz, double* __restrict__ w, long wstride,
          double* __restrict__ part, SkipCtl sk) {
    __shared__ double red[32];
    const int b = blockIdx.y, i = blockIdx.x, n = nsz[b];
    if (i >= n || skip_step(sk, b)) return;
    const double* Sr = S + b * stride + (long)i * ld;
    const double* Gr = G + b * stride + (long)i * ld;
    const double lam = Sr[i] / Gr[i];
    double ps = 0.0, pr = 0.0;
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
        const double sd = Sr[j] - (j == i ? lam : 0.0);
        const double rd = (j == i ? 1.0 : 0.0) - Gr[j];
        ps += sd * sd;
        pr += rd * rd;
    }
    ps = cta_sumd(ps, red);
    pr = cta_sumd(pr, red);
    if (threadIdx.x == 0) {
        part[2 * ((long)b * ld + i)] = ps;
        part[2 * ((long)b * ld + i) + 1] = pr;
        w[b * wstride + i] = lam;
    }
}

__global__ void __launch_bounds__(128)
k_oa_apply(const double* __restrict__ S, double* __restrict__ G, long stride, int ld,
           const int* __restrict__ nsz, const double* __restrict__ anorm,
           const double* __restrict__ w, long wstride, const double* __restrict__ part,
           double* __restrict__ emax, double* __restrict__ offrel, SkipCtl sk) {
    __shared__ double red[32];
    const int b = blockIdx.y, i = blockIdx.x, n = nsz[b];
    if (i >= n || skip_step(sk, b)) return;
    double ps = 0.0, pr = 0.0;
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
        ps += part[2 * ((long)b * ld + j)];
        pr += part[2 * ((long)b * ld + j) + 1];
    }
    ps = cta_sumd(ps, red);
    pr = cta_sumd(pr, red);
    const double delta = 2.0 * (sqrt(ps) + anorm[b] * sqrt(pr));
    if (i == 0 && threadIdx.x == 0) offrel[b] = sqrt(ps) / anorm[b];
    const double* lam = w + b * wstride;
    const double li = lam[i];
    const double* Sr = S + b * stride + (long)i * ld;
    double* Gr = G + b * stride + (long)i * ld;
    double em = 0.0;
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
        const double r = (j == i ? 1.0 : 0.0) - Gr[j];
        double e;
        if (j != i && fabs(lam[j] - li) > delta) {
            e = (Sr[j] + lam[j] * r) / (lam[j] - li);
        } else {
            e = 0.5 * r;
        }
        if (lam[j] * li < 0.0) em = fmax(em, fabs(Sr[j]) / fabs(lam[j] - li));
        Gr[j] = (j == i ? 1.0 : 0.0) + e;
    }
    for (int o = 16; o > 0; o >>= 1) em = fmax(em, __shfl_xor_sync(0xffffffffu, em, o));
    __syncthreads();
    if (threadIdx.x % 32 == 0) red[threadIdx.x / 32] = em;
    __syncthreads();
    if (threadIdx.x == 0) {
        double m = 0.0;
        for (int k = 0; k < (int)(blockDim.x / 32); ++k) m = fmax(m, red[k]);
        emax[(long)b * ld + i] = m;
    }
}

// FP64 Jacobi polish of S = X^T A X after refinement: S is diagonal up to
// rounding outside clusters of (near-)degenerate eigenvalues, so only the
// pairs with |s_pq| above the rounding level rotate.  Q accumulates the
// rotations (X <- X Q afterwards) and w receives diag(S).  Needed where the
// individual vectors inside a cluster matter (the canonical basis: the
// occupation-weighted density sum is not invariant under rotations between
// states of slightly different occupation).
__global__ void __launch_bounds__(kJThreads)
k_jacobi64_polish(const double* __restrict__ S, long stride, int ld, const int* __restrict__ nsz,
                  const double* __restrict__ anorm, double* __restrict__ Q,
                  double* __restrict__ w, long wstride, int* __restrict__ pfail,
                  int max_sweeps) {
    extern __shared__ double smd[];
    __shared__ double red[32];
    __shared__ double cs[2][kEigMax / 2];
    __shared__ int act[kEigMax / 2];
    __shared__ int pqi[2][kEigMax / 2];
    __shared__ unsigned rmask[(kEigMax + 31) / 32];
    const int b = blockIdx.x;
    const int n0 = nsz[b];
    if (n0 == 0) {
        if (threadIdx.x == 0 && pfail) pfail[b] = 0;
        return;
    }
    const int n = n0 + (n0 & 1);
    const int l2 = n + 1;
    double* a = smd;
    // Q accumulates in the output buffer (global, L1/L2 resident): row r, col c
    double* q = Q + b * stride;
    auto Qa = [&](int r, int c) -> double& { return q[(long)r * ld + c]; };
    const int tid = threadIdx.x;
    for (int t = tid; t < n * n; t += kJThreads) {
        const int i = t / n, j = t % n;
        const double x = (i < n0 && j < n0) ? S[b * stride + (long)i * ld + j] : 0.0;
        const double y = (i < n0 && j < n0) ? S[b * stride + (long)j * ld + i] : 0.0;
        a[i * l2 + j] = i == j ? x : 0.5 * (x + y);
    }
    for (int t = tid; t < n0 * n0; t += kJThreads) Qa(t / n0, t % n0) = (t / n0 == t % n0) ? 1.0 : 0.0;
    __syncthreads();
    const double thr = 1e-14 * anorm[b];
    const int lane = tid & 127, kg = tid >> 7;
    const int half = n / 2;
    int sweep = 0;
    for (; sweep < max_sweeps; ++sweep) {
        // a pair rotates when its coupling is above the FP64 noise of X^T A X
        // (~ sqrt(n) eps |A|): rotating noise would only churn, at FP64 cost.
        // Only the rounds holding such a pair at the start of the sweep run
        // (after a refinement these are the few near-degenerate clusters); a
        // pair that a rotation lifts above the threshold waits for the next
        // sweep.
        if (tid < (kEigMax + 31) / 32) rmask[tid] = 0u;
        __syncthreads();
        int any = 0;
        for (int col = lane; col < n; col += 128)
            for (int i = kg; i < col; i += kJGroups)
                if (fabs(a[i * l2 + col]) > thr) {
                    const int r = rr_round(i, col, n);
                    atomicOr(&rmask[r >> 5], 1u << (r & 31));
                    any = 1;
                }
        if (!__syncthreads_or(any)) break;
        for (int r = 0; r < n - 1; ++r) {
            if (!((rmask[r >> 5] >> (r & 31)) & 1u)) continue;
            int on = 0;
            if (tid < half) {
                const int p = rr_player(tid, r, n), qq = rr_player(n - 1 - tid, r, n);
                const double apq = a[p * l2 + qq];
                const double d = a[qq * l2 + qq] - a[p * l2 + p];
                double c = 1.0, s = 0.0;
                if (fabs(apq) > thr) {
                    if (fabs(d) > 1e8 * fabs(apq)) {
                        // small angle: tan = a_pq / d to 1/(4 tau^2) < 1e-16 relative
                        // (FP64 divides and square roots are slow on this part)
                        const double tt = apq / d;
                        c = 1.0 - 0.5 * tt * tt;
                        s = tt * c;
                    } else {
                        const double th = d / (2.0 * apq);
                        const double tt =
                            (th >= 0.0 ? 1.0 : -1.0) / (fabs(th) + sqrt(th * th + 1.0));
                        c = 1.0 / sqrt(tt * tt + 1.0);
                        s = tt * c;
                    }
                    on = 1;
                }
                cs[0][tid] = c;
                cs[1][tid] = s;
                act[tid] = on;
                pqi[0][tid] = p;
                pqi[1][tid] = qq;
            }
            // rounds without a pair above the threshold rotate nothing
            if (!__syncthreads_or(on)) continue;
            for (int col = lane; col < n; col += 128)
                for (int k = kg; k < half; k += kJGroups) {
                    if (!act[k]) continue;
                    const int p = pqi[0][k], qq = pqi[1][k];
                    const double c = cs[0][k], s = cs[1][k];
                    const double ap = a[p * l2 + col], aq = a[qq * l2 + col];
                    a[p * l2 + col] = c * ap - s * aq;
                    a[qq * l2 + col] = s * ap + c * aq;
                }
            __syncthreads();
            for (int row = lane; row < n; row += 128)
                for (int k = kg; k < half; k += kJGroups) {
                    if (!act[k]) continue;
                    const int p = pqi[0][k], qq = pqi[1][k];
                    const double c = cs[0][k], s = cs[1][k];
                    const double ap = a[row * l2 + p], aq = a[row * l2 + qq];
                    a[row * l2 + p] = c * ap - s * aq;
                    a[row * l2 + qq] = s * ap + c * aq;
                    if (row < n0 && p < n0 && qq < n0) {
                        const double vp = Qa(row, p), vq = Qa(row, qq);
                        Qa(row, p) = c * vp - s * vq;
                        Qa(row, qq) = s * vp + c * vq;
                    }
                }
            __syncthreads();
        }
    }
    if (tid == 0 && pfail) pfail[b] = sweep == max_sweeps ? 1 : 0;
    for (int i = tid; i < n0; i += kJThreads) w[b * wstride + i] = a[i * l2 + i];
}

// The polish of the mixed form: k_jacobi64_polish in double-float
// arithmetic (df.cuh) on the FP32 pipes, which GB300 issues at ~60x its FP64
// rate.  S and the rotations Q are held in shared memory as {hi, lo} pairs
// (48 significant bits; S split from FP64 with integer instructions), so
// the threshold is 4e-14 |A| against the FP64 polish's 1e-14.  tan(theta)
// is taken in FP32 -- an inexact angle only leaves a smaller coupling for
// the next sweep -- and c = (1 + t^2)^(-1/2), s = t c are completed to
// double-float precision by one Newton step on the FP32 reciprocal square
// root, so that every rotation stays orthogonal to ~1e-14.  A round rotates
// the 2 x 2 blocks (rows of pair i, columns of pair j) whose row or column
// pair is active, and the columns of Q of its active pairs.  Q is written
// back in FP64.  n <= kDfPolishMax.
constexpr int kDfPolishMax = 112;

size_t df_polish_smem(int n) {
    const int np = n + (n & 1);
    return (size_t)2 * np * (np + 1) * sizeof(float2);
}

__device__ __forceinline__ dfl df_rot_a(dfl c, dfl s, dfl x, dfl y) {   // c x - s y
    return df_fma(c, x, df_neg(df_mul(s, y)));
}

__device__ __forceinline__ dfl df_rot_b(dfl c, dfl s, dfl x, dfl y) {   // s x + c y
    return df_fma(s, x, df_mul(c, y));
}

__global__ void __launch_bounds__(kJThreads)
k_jacobi_df_polish(const double* __restrict__ S, long stride, int ld, const int* __restrict__ nsz,
                   const double* __restrict__ anorm, double* __restrict__ Q,
                   double* __restrict__ w, long wstride, int* __restrict__ pfail,
                   int max_sweeps) {
    extern __shared__ float2 smq[];
    __shared__ float4 cs[kDfPolishMax / 2];   // c.h, c.l, s.h, s.l
    __shared__ int act[kDfPolishMax / 2];
    __shared__ int pqi[2][kDfPolishMax / 2];
    __shared__ unsigned rmask[(kDfPolishMax + 31) / 32];
    const int b = blockIdx.x;
    const int n0 = nsz[b];
    if (n0 == 0) {
        if (threadIdx.x == 0 && pfail) pfail[b] = 0;
        return;
    }
    const int n = n0 + (n0 & 1);
    const int l2 = n + 1;
    float2* a = smq;            // n x l2
    float2* qs = a + n * l2;    // n x l2 (rows and columns < n0 used)
    const int tid = threadIdx.x;
    for (int t = tid; t < n * n; t += kJThreads) {
        const int i = t / n, j = t % n;
        dfl x{0.0f, 0.0f};
        if (i < n0 && j < n0) {
            x = df_split(S[b * stride + (long)i * ld + j]);
            if (i != j) {
                // symmetrise: (x + y) / 2 (the halving is exact)
                const dfl y = df_split(S[b * stride + (long)j * ld + i]);
                x = df_add(x, y);
                x.h *= 0.5f;
                x.l *= 0.5f;
            }
        }
        a[i * l2 + j] = make_float2(x.h, x.l);
        qs[i * l2 + j] = make_float2(i == j ? 1.0f : 0.0f, 0.0f);
    }
    __syncthreads();
    const float thr = (float)(4e-14 * anorm[b]);
    const int half = n / 2;
    int sweep = 0;
    for (; sweep < max_sweeps; ++sweep) {
        // as in k_jacobi64_polish: only the rounds that hold a coupling above
        // the threshold at the start of the sweep run
        if (tid < (kDfPolishMax + 31) / 32) rmask[tid] = 0u;
        __syncthreads();
        int any = 0;
        for (int t = tid; t < n * n; t += kJThreads) {
            const int i = t / n, col = t % n;
            if (i < col && fabsf(a[i * l2 + col].x) > thr) {
                const int r = rr_round(i, col, n);
                atomicOr(&rmask[r >> 5], 1u << (r & 31));
                any = 1;
            }
        }
        if (!__syncthreads_or(any)) break;
        for (int r = 0; r < n - 1; ++r) {
            if (!((rmask[r >> 5] >> (r & 31)) & 1u)) continue;
            int on = 0;
            if (tid < half) {
                const int p = rr_player(tid, r, n), q = rr_player(n - 1 - tid, r, n);
                const dfl apq = df_ld(a + p * l2 + q);
                dfl c{1.0f, 0.0f}, sn{0.0f, 0.0f};
                if (fabsf(apq.h) > thr) {
                    const dfl d = df_sub(df_ld(a + q * l2 + q), df_ld(a + p * l2 + p));
                    float tt;
                    if (fabsf(d.h) > 1e6f * fabsf(apq.h)) {
                        tt = apq.h / d.h;   // small angle: tan = a_pq / d to ~1e-12
                    } else {
                        const float th = d.h / (2.0f * apq.h);
                        tt = (th >= 0.0f ? 1.0f : -1.0f) / (fabsf(th) + sqrtf(th * th + 1.0f));
                    }
                    // c = (1 + t^2)^(-1/2): FP32 estimate r, then r (3 - x r^2) / 2
                    const dfl x = df_add(dfl{1.0f, 0.0f}, df_mul(dfl{tt, 0.0f}, dfl{tt, 0.0f}));
                    const float r0 = rsqrtf(x.h);
                    const dfl xr2 = df_mul(x, df_mul(dfl{r0, 0.0f}, dfl{r0, 0.0f}));
                    dfl corr = df_sub(dfl{3.0f, 0.0f}, xr2);
                    corr.h *= 0.5f;
                    corr.l *= 0.5f;
                    c = df_mul(dfl{r0, 0.0f}, corr);
                    sn = df_mul(dfl{tt, 0.0f}, c);
                    on = 1;
                }
                cs[tid] = make_float4(c.h, c.l, sn.h, sn.l);
                act[tid] = on;
                pqi[0][tid] = p;
                pqi[1][tid] = q;
            }
            if (!__syncthreads_or(on)) continue;
            for (int u = tid; u < half * half; u += kJThreads) {
                const int i = u / half, j = u % half;
                const int ai = act[i], aj = act[j];
                if (!ai && !aj) continue;
                float2* ap = a + pqi[0][i] * l2;
                float2* aq = a + pqi[1][i] * l2;
                const int jp = pqi[0][j], jq = pqi[1][j];
                dfl x00 = df_ld(ap + jp), x01 = df_ld(ap + jq), x10 = df_ld(aq + jp),
                    x11 = df_ld(aq + jq);
                if (ai) {   // rows of pair i
                    const float4 C = cs[i];
                    const dfl c{C.x, C.y}, sn{C.z, C.w};
                    const dfl r00 = df_rot_a(c, sn, x00, x10), r10 = df_rot_b(c, sn, x00, x10);
                    const dfl r01 = df_rot_a(c, sn, x01, x11), r11 = df_rot_b(c, sn, x01, x11);
                    x00 = r00;
                    x10 = r10;
                    x01 = r01;
                    x11 = r11;
                }
                if (aj) {   // columns of pair j
                    const float4 C = cs[j];
                    const dfl c{C.x, C.y}, sn{C.z, C.w};
                    const dfl r00 = df_rot_a(c, sn, x00, x01), r01 = df_rot_b(c, sn, x00, x01);
                    const dfl r10 = df_rot_a(c, sn, x10, x11), r11 = df_rot_b(c, sn, x10, x11);
                    x00 = r00;
                    x01 = r01;
                    x10 = r10;
                    x11 = r11;
                }
                df_st(ap + jp, x00);
                df_st(ap + jq, x01);
                df_st(aq + jp, x10);
                df_st(aq + jq, x11);
            }
            for (int u = tid; u < n0 * half; u += kJThreads) {
                const int k = u / n0, row = u % n0;
                if (!act[k]) continue;
                const float4 C = cs[k];
                const dfl c{C.x, C.y}, sn{C.z, C.w};
                float2* qr = qs + row * l2;
                const int p = pqi[0][k], q = pqi[1][k];
                const dfl vp = df_ld(qr + p), vq = df_ld(qr + q);
                df_st(qr + p, df_rot_a(c, sn, vp, vq));
                df_st(qr + q, df_rot_b(c, sn, vp, vq));
            }
            __syncthreads();
        }
    }
    if (tid == 0 && pfail) pfail[b] = sweep == max_sweeps ? 1 : 0;
    for (int t = tid; t < n0 * n0; t += kJThreads) {
        const int r = t / n0, c = t % n0;
        const float2 v = qs[r * l2 + c];
        Q[b * stride + (long)r * ld + c] = df_to_fast(dfl{v.x, v.y});
    }
    for (int i = tid; i < n0; i += kJThreads) {
        const float2 v = a[i * l2 + i];
        w[b * wstride + i] = df_to_fast(dfl{v.x, v.y});
    }
}

// Re-orthonormalisation X <- X (I + R/2 + 3/8 R^2), R = I - X^T X (third-order
// accurate): from G = X^T X write R into Rm and I + R/2 into F.
__global__ void k_orth_prep(const double* __restrict__ G, double* __restrict__ Rm,
                            double* __restrict__ F, long stride, int ld,
                            const int* __restrict__ nsz) {
    const int b = blockIdx.y, n = nsz[b];
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n * n) return;
    const int i = t / n, j = t % n;
    const long o = b * stride + (long)i * ld + j;
    const double r = (i == j ? 1.0 : 0.0) - G[o];
    Rm[o] = r;
    F[o] = (i == j ? 1.0 : 0.0) + 0.5 * r;
}

// Ascending order after a refinement that started from earlier vectors (the
// eigenvalue estimates keep the column order of the start, which need not be
// sorted any more): rank each eigenvalue (ties by index), move column j of X
// to column rank(j) of X2 and reorder w.  Grid (row chunks, matrices): every
// CTA ranks the eigenvalues itself (integer compares of order-preserving
// keys of the FP64 bit patterns) and moves kSortRows rows.
constexpr int kSortRows = 8;

__device__ __forceinline__ unsigned long long order_key(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

__global__ void __launch_bounds__(128)
k_sort_cols(const double* __restrict__ X, double* __restrict__ X2, const double* __restrict__ w,
            double* __restrict__ w2, long stride, int ld, long wstride,
            const int* __restrict__ nsz) {
    __shared__ unsigned long long key[kEigMax];
    __shared__ double sw[kEigMax];
    __shared__ int rank[kEigMax];
    const int b = blockIdx.y, n = nsz[b];
    const int r0 = blockIdx.x * kSortRows;
    if (r0 >= n) return;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        sw[i] = w[b * wstride + i];
        key[i] = order_key(sw[i]);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const unsigned long long ki = key[i];
        int r = 0;
        for (int j = 0; j < n; ++j) r += (key[j] < ki || (key[j] == ki && j < i)) ? 1 : 0;
        rank[i] = r < n ? r : n - 1;
    }
    __syncthreads();
    const int r1 = min(n, r0 + kSortRows);
    for (int t = threadIdx.x; t < (r1 - r0) * n; t += blockDim.x) {
        const int r = r0 + t / n, j = t % n;
        X2[b * stride + (long)r * ld + rank[j]] = X[b * stride + (long)r * ld + j];
    }
    // every CTA holds the same values; the first writes the sorted w (to a
    // second buffer: the other CTAs may still be reading w)
    if (blockIdx.x == 0)
        for (int i = threadIdx.x; i < n; i += blockDim.x) w2[b * wstride + rank[i]] = sw[i];
}

// Frobenius norms of the batch matrices (delta of the refinement uses ||A||).
__global__ void k_frob(const double* __restrict__ A, long stride, int ld, const int* __restrict__ nsz,
                       double* __restrict__ out) {
    __shared__ double red[32];
    const int b = blockIdx.x, n = nsz[b];
    double p = 0.0;
    for (int q = threadIdx.x; q < n * n; q += blockDim.x) {
        const double x = A[b * stride + (long)(q / n) * ld + q % n];
        p += x * x;
    }
    const double s = cta_sumd(p, red);
    if (threadIdx.x == 0) out[b] = sqrt(s);
}

size_t jacobi_smem(int n) {
    const int np = n + (n & 1);
    return (size_t)(np <= kJSmemMax ? 3 : 2) * np * (np + 1) * sizeof(float);
}

// One launch of a GEMM table: double-float in the mixed form, FP64 otherwise.
static void launch_gemm(mg_ctx* c, bool df, dim3 grid, const GemmDesc* descs, SkipCtl sk) {
    if (df)
        k_gemm_df<<<grid, kThreads, 0, c->stream>>>(descs, sk);
    else
        k_gemm64<<<grid, kThreads, 0, c->stream>>>(descs, sk);
}

// Eigen-decomposition of a batch (nb <= 64: the GEMM grids hold 2 nb
// matrices in y) of symmetric matrices of sizes nsz (device) <= nmax, stored
// with leading dimension ld and stride `stride`.  E.X: in/out (the warm start
// of kSeedJacobiWarm / kSeedRefine), E.w: eigenvalues; the work matrices,
// norms and GEMM tables are E's (eig_setup).  E.pfail[b] is set to 1 when the
// FP64 Jacobi polish of matrix b reached its sweep cap.
int eig_batched(mg_ctx* c, EigBatch& E, int seed, int nref, bool polish) {
    if (!E.attr_done) {
        MG_CUDA(cudaFuncSetAttribute(k_jacobi32, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     kSmemOptIn));
        MG_CUDA(cudaFuncSetAttribute(k_jacobi64_polish, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     kSmemOptIn));
        MG_CUDA(cudaFuncSetAttribute(k_jacobi_df_polish,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)df_polish_smem(kDfPolishMax)));
        E.attr_done = true;
    }
    if (seed != kSeedRefine) {
        const bool warm = seed == kSeedJacobiWarm;
        const size_t sm = jacobi_smem(E.nmax);
        k_jacobi32<<<E.nb, kJThreads, sm, c->stream>>>(E.A, E.stride, E.ld, E.nsz,
                                                      warm ? E.X : nullptr, E.X, E.stride, E.ld,
                                                      E.w, E.wstride, warm ? 12 : 30, c->flags + 4);
        MG_LAUNCHED(c);
    }
    k_frob<<<E.nb, 1024, 0, c->stream>>>(E.A, E.stride, E.ld, E.nsz, E.anorm);
    MG_LAUNCHED(c);
    const int tiles = div_up(E.nmax, kTile) * div_up(E.nmax, kTile);
    const bool dfg = c->cur_precision == MG_MIXED;
    const SkipCtl none{nullptr, nullptr, 0, 0, 0.0};
    if (E.skip_tol >= 0.0)
        MG_CUDA(cudaMemsetAsync(E.done, 0x7f, (size_t)E.nb * sizeof(int), c->stream));
    for (int s = 0; s < nref; ++s) {
        // AX = A X ; S = X^T AX ; G = X^T X ; F = I + E ; X2 = X F ; X <- X2
        SkipCtl sk{E.skip_tol >= 0.0 ? E.done : nullptr, E.offrel, s, 1, E.skip_tol};
        launch_gemm(c, dfg, dim3(tiles, E.nb), E.d_ax, sk);
        MG_LAUNCHED(c);
        sk.decide = 0;
        launch_gemm(c, dfg, dim3(tiles, 2 * E.nb), E.d_sg, sk);
        MG_LAUNCHED(c);
        k_oa_rows<<<dim3(E.nmax, E.nb), 128, 0, c->stream>>>(E.S, E.G, E.stride, E.ld, E.nsz,
                                                             E.w, E.wstride, E.part, sk);
        MG_LAUNCHED(c);
        k_oa_apply<<<dim3(E.nmax, E.nb), 128, 0, c->stream>>>(E.S, E.G, E.stride, E.ld, E.nsz,
                                                              E.anorm, E.w, E.wstride, E.part,
                                                              E.emax, E.offrel, sk);
        MG_LAUNCHED(c);
        launch_gemm(c, dfg, dim3(tiles, E.nb), E.d_xf, sk);
        MG_LAUNCHED(c);
        MG_CUDA(cudaMemcpyAsync(E.X, E.X2, (size_t)E.nb * E.stride * sizeof(double),
                                cudaMemcpyDeviceToDevice, c->stream));
    }
    // re-orthonormalise: G = X^T X, F = I + R/2 + 3/8 R^2, X <- X F, leaving
    // ~(5/16) R^3.  With the polish a second pass follows: the polish
    // diagonalises X^T A X, whose diagonal misses the eigenvalues by the
    // non-orthogonality of X, and a refinement that stops inside a cluster
    // of near-degenerate eigenvalues (density-matrix occupations ~1e-8 apart
    // near 0 or 1) can leave R ~ 1e-2, which one pass only brings to 1e-7.
    for (int pass = 0; pass < (polish ? 2 : 1); ++pass) {
        launch_gemm(c, dfg, dim3(tiles, 2 * E.nb), E.d_sg, none);
        MG_LAUNCHED(c);
        k_orth_prep<<<dim3(div_up((long)E.nmax * E.nmax, kThreads), E.nb), kThreads, 0,
                      c->stream>>>(E.G, E.AX, E.G, E.stride, E.ld, E.nsz);
        MG_LAUNCHED(c);
        launch_gemm(c, dfg, dim3(tiles, E.nb), E.d_rr, none);
        MG_LAUNCHED(c);
        launch_gemm(c, dfg, dim3(tiles, E.nb), E.d_xf, none);
        MG_LAUNCHED(c);
        MG_CUDA(cudaMemcpyAsync(E.X, E.X2, (size_t)E.nb * E.stride * sizeof(double),
                                cudaMemcpyDeviceToDevice, c->stream));
    }
    if (polish) {
        const int np = E.nmax + (E.nmax & 1);
        const size_t psm = (size_t)np * (np + 1) * sizeof(double);
        if (psm > (size_t)kSmemOptIn) return MG_ERR_ARG;
        // Rayleigh-Ritz matrix and the FP64 Jacobi polish
        launch_gemm(c, dfg, dim3(tiles, E.nb), E.d_ax, none);
        MG_LAUNCHED(c);
        launch_gemm(c, dfg, dim3(tiles, 2 * E.nb), E.d_sg, none);
        MG_LAUNCHED(c);
        if (c->cur_precision == MG_MIXED && E.nmax <= kDfPolishMax)
            k_jacobi_df_polish<<<E.nb, kJThreads, df_polish_smem(E.nmax), c->stream>>>(
                E.S, E.stride, E.ld, E.nsz, E.anorm, E.G, E.w, E.wstride, E.pfail, 12);
        else
            k_jacobi64_polish<<<E.nb, kJThreads, psm, c->stream>>>(
                E.S, E.stride, E.ld, E.nsz, E.anorm, E.G, E.w, E.wstride, E.pfail, 12);
        MG_LAUNCHED(c);
        launch_gemm(c, dfg, dim3(tiles, E.nb), E.d_xf, none);
        MG_LAUNCHED(c);
        MG_CUDA(cudaMemcpyAsync(E.X, E.X2, (size_t)E.nb * E.stride * sizeof(double),
                                cudaMemcpyDeviceToDevice, c->stream));
    }
    // ascending order: the refinement keeps the column order of its start and
    // the polish leaves diag(S) in place
    if (seed == kSeedRefine || polish) {
        // E.part (2 * nb * ld doubles, free after the refinement) takes the sorted w
        k_sort_cols<<<dim3(div_up(E.nmax, kSortRows), E.nb), 128, 0, c->stream>>>(
            E.X, E.X2, E.w, E.part, E.stride, E.ld, E.wstride, E.nsz);
        MG_LAUNCHED(c);
        MG_CUDA(cudaMemcpyAsync(E.w, E.part, (size_t)E.nb * E.wstride * sizeof(double),
                                cudaMemcpyDeviceToDevice, c->stream));
        MG_CUDA(cudaMemcpyAsync(E.X, E.X2, (size_t)E.nb * E.stride * sizeof(double),
                                cudaMemcpyDeviceToDevice, c->stream));
    }
    return MG_OK;
}

// The whole batch by cyclic FP64 Jacobi on A itself (the polish kernel
// started from the identity, up to 40 sweeps), eigenvalues ascending: the
// fallback when a refined decomposition is found wanting.  Slow (every
// rotation in FP64) but it converges for any symmetric matrix.
int eig_jacobi_fp64(mg_ctx* c, EigBatch& E) {
    const int np = E.nmax + (E.nmax & 1);
    const size_t psm = (size_t)np * (np + 1) * sizeof(double);
    if (psm > (size_t)kSmemOptIn) return MG_ERR_ARG;
    if (!E.attr_done) {
        MG_CUDA(cudaFuncSetAttribute(k_jacobi32, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     kSmemOptIn));
        MG_CUDA(cudaFuncSetAttribute(k_jacobi64_polish, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     kSmemOptIn));
        MG_CUDA(cudaFuncSetAttribute(k_jacobi_df_polish,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)df_polish_smem(kDfPolishMax)));
        E.attr_done = true;
    }
    k_frob<<<E.nb, 1024, 0, c->stream>>>(E.A, E.stride, E.ld, E.nsz, E.anorm);
    MG_LAUNCHED(c);
    k_jacobi64_polish<<<E.nb, kJThreads, psm, c->stream>>>(E.A, E.stride, E.ld, E.nsz, E.anorm,
                                                           E.X, E.w, E.wstride, E.pfail, 40);
    MG_LAUNCHED(c);
    k_sort_cols<<<dim3(div_up(E.nmax, kSortRows), E.nb), 128, 0, c->stream>>>(
        E.X, E.X2, E.w, E.part, E.stride, E.ld, E.wstride, E.nsz);
    MG_LAUNCHED(c);
    MG_CUDA(cudaMemcpyAsync(E.w, E.part, (size_t)E.nb * E.wstride * sizeof(double),
                            cudaMemcpyDeviceToDevice, c->stream));
    MG_CUDA(cudaMemcpyAsync(E.X, E.X2, (size_t)E.nb * E.stride * sizeof(double),
                            cudaMemcpyDeviceToDevice, c->stream));
    E.have_vectors = true;
    return MG_OK;
}

// The same, skipping the GEMMs whose matrix index m has done[m] <= 0.
int gemm_batched_skip(mg_ctx* c, const GemmDesc* descs, int ndesc, int maxdim, int* done) {
    const SkipCtl sk{done, nullptr, 0, 0, 0.0};
    const int tiles = div_up(maxdim, kTile) * div_up(maxdim, kTile);
    k_gemm64<<<dim3(tiles, ndesc), kThreads, 0, c->stream>>>(descs, sk);
    MG_LAUNCHED(c);
    return MG_OK;
}

// ndesc FP64 GEMMs of at most maxdim x maxdim from a device descriptor
// table (double-float when df is set).
int gemm_batched(mg_ctx* c, const GemmDesc* descs, int ndesc, int maxdim, bool df) {
    const SkipCtl none{nullptr, nullptr, 0, 0, 0.0};
    const int tiles = div_up(maxdim, kTile) * div_up(maxdim, kTile);
    launch_gemm(c, df, dim3(tiles, ndesc), descs, none);
    MG_LAUNCHED(c);
    return MG_OK;
}

// Workspace and GEMM descriptor tables for a batch.
int eig_setup(mg_ctx* c, EigBatch& E, int nb, int nmax, const int* nsz_dev, double* A, long stride,
              int ld) {
    E.nb = nb;
    E.nmax = nmax;
    E.nsz = nsz_dev;
    E.A = A;
    E.stride = stride;
    E.ld = ld;
    E.wstride = nmax;
    const size_t bytes = (size_t)nb * stride * sizeof(double);
    MG_CUDA(cudaMalloc(&E.X, bytes));
    MG_CUDA(cudaMemset(E.X, 0, bytes));
    MG_CUDA(cudaMalloc(&E.X2, bytes));
    MG_CUDA(cudaMalloc(&E.AX, bytes));
    MG_CUDA(cudaMalloc(&E.S, bytes));
    MG_CUDA(cudaMalloc(&E.G, bytes));
    MG_CUDA(cudaMalloc(&E.w, (size_t)nb * nmax * sizeof(double)));
    MG_CUDA(cudaMalloc(&E.anorm, (size_t)nb * sizeof(double)));
    MG_CUDA(cudaMalloc(&E.part, (size_t)nb * ld * 2 * sizeof(double)));
    MG_CUDA(cudaMalloc(&E.emax, (size_t)nb * ld * sizeof(double)));
    MG_CUDA(cudaMemset(E.emax, 0, (size_t)nb * ld * sizeof(double)));
    MG_CUDA(cudaMalloc(&E.done, (size_t)nb * sizeof(int)));
    MG_CUDA(cudaMalloc(&E.offrel, (size_t)nb * sizeof(double)));
    MG_CUDA(cudaMalloc(&E.pfail, (size_t)nb * sizeof(int)));
    MG_CUDA(cudaMemset(E.pfail, 0, (size_t)nb * sizeof(int)));
    std::vector<int> hn(nb);
    MG_CUDA(cudaMemcpy(hn.data(), nsz_dev, nb * sizeof(int), cudaMemcpyDeviceToHost));
    std::vector<GemmDesc> ax(nb), sg(2 * nb), xf(nb), rr(nb);
    for (int b = 0; b < nb; ++b) {
        const int n = hn[b];
        const long o = (long)b * stride;
        ax[b] = GemmDesc{A + o, E.X + o, E.AX + o, n, n, n, ld, ld, ld, 0, 0, 1.0, 0.0, b};
        sg[2 * b] = GemmDesc{E.X + o, E.AX + o, E.S + o, n, n, n, ld, ld, ld, 1, 0, 1.0, 0.0, b, 1};
        sg[2 * b + 1] = GemmDesc{E.X + o, E.X + o, E.G + o, n, n, n, ld, ld, ld, 1, 0, 1.0, 0.0, b, 1};
        xf[b] = GemmDesc{E.X + o, E.G + o, E.X2 + o, n, n, n, ld, ld, ld, 0, 0, 1.0, 0.0, b};
        rr[b] = GemmDesc{E.AX + o, E.AX + o, E.G + o, n, n, n, ld, ld, ld, 0, 0, 0.375, 1.0, b, 1};
    }
    MG_CUDA(cudaMalloc(&E.d_ax, nb * sizeof(GemmDesc)));
    MG_CUDA(cudaMalloc(&E.d_sg, 2 * nb * sizeof(GemmDesc)));
    MG_CUDA(cudaMalloc(&E.d_xf, nb * sizeof(GemmDesc)));
    MG_CUDA(cudaMalloc(&E.d_rr, nb * sizeof(GemmDesc)));
    MG_CUDA(cudaMemcpy(E.d_ax, ax.data(), nb * sizeof(GemmDesc), cudaMemcpyHostToDevice));
    MG_CUDA(cudaMemcpy(E.d_sg, sg.data(), 2 * nb * sizeof(GemmDesc), cudaMemcpyHostToDevice));
    MG_CUDA(cudaMemcpy(E.d_xf, xf.data(), nb * sizeof(GemmDesc), cudaMemcpyHostToDevice));
    MG_CUDA(cudaMemcpy(E.d_rr, rr.data(), nb * sizeof(GemmDesc), cudaMemcpyHostToDevice));
    return MG_OK;
}

}  // namespace mg

extern "C" int mg_eigh_batched(int nb, const int* n, int ld, const double* a, double* w,
                               double* z) {
    using namespace mg;
    if (nb <= 0 || nb > 64 || !n || !a || !w || !z || ld <= 0 || ld > kEigMax) return MG_ERR_ARG;
    for (int b = 0; b < nb; ++b)
        if (n[b] < 0 || n[b] > ld) return MG_ERR_ARG;
    mg_ctx tmp;  // a throw-away context carrying only the stream, flags and counters
    MG_CUDA(cudaStreamCreateWithFlags(&tmp.stream, cudaStreamNonBlocking));
    MG_CUDA(cudaMalloc(&tmp.flags, 16 * sizeof(int)));
    MG_CUDA(cudaMemset(tmp.flags, 0, 16 * sizeof(int)));
    const long stride = (long)ld * ld;
    double* dA = nullptr;
    int* dn = nullptr;
    MG_CUDA(cudaMalloc(&dA, nb * stride * sizeof(double)));
    MG_CUDA(cudaMalloc(&dn, nb * sizeof(int)));
    MG_CUDA(cudaMemcpy(dA, a, nb * stride * sizeof(double), cudaMemcpyHostToDevice));
    MG_CUDA(cudaMemcpy(dn, n, nb * sizeof(int), cudaMemcpyHostToDevice));
    EigBatch E;
    int st = eig_setup(&tmp, E, nb, ld, dn, dA, stride, ld);
    if (st == MG_OK) st = eig_batched(&tmp, E, kSeedCold, 3, true);
    if (st == MG_OK) {
        MG_CUDA(cudaStreamSynchronize(tmp.stream));
        MG_CUDA(cudaMemcpy(w, E.w, nb * (size_t)ld * sizeof(double), cudaMemcpyDeviceToHost));
        MG_CUDA(cudaMemcpy(z, E.X, nb * stride * sizeof(double), cudaMemcpyDeviceToHost));
        // the polish of a matrix that ran out of sweeps: results written, status > 0
        std::vector<int> pf(nb, 0);
        MG_CUDA(cudaMemcpy(pf.data(), E.pfail, nb * sizeof(int), cudaMemcpyDeviceToHost));
        for (int b = 0; b < nb; ++b)
            if (pf[b]) st = MG_NOT_CONVERGED;
    }
    eig_free(E);
    cudaFree(dA);
    cudaFree(dn);
    cudaFree(tmp.flags);
    tmp.flags = nullptr;
    cudaStreamDestroy(tmp.stream);
    tmp.stream = nullptr;
    return st;
}

// ---- allocation-free variant ---------------------------------------------------------
//
// Hosts that own all device memory through their own pool, and code that runs
// while a stream is being captured (where cudaMalloc is not allowed), cannot
// let the solver allocate.  mg_eigh_batched_noalloc takes device buffers from
// the caller and keeps its workspace in one file-scope device array, so a call
// only launches kernels and stream-ordered memsets/copies.

namespace mg {
namespace {

constexpr long kNoAllocElems = 65536;   // nb * ld * ld capacity (512 KB per work matrix)
constexpr int kNoAllocNb = 64;
constexpr int kNoAllocLd = 128;
constexpr int kNoAllocMaxDevices = 64;

constexpr size_t round256(size_t b) { return (b + 255) / 256 * 256; }
constexpr size_t kMatBytes = (size_t)kNoAllocElems * sizeof(double);
constexpr size_t kOffX2 = 0, kOffAX = kMatBytes, kOffS = 2 * kMatBytes, kOffG = 3 * kMatBytes;
constexpr size_t kOffNorm = 4 * kMatBytes;
constexpr size_t kOffDesc = kOffNorm + round256(kNoAllocNb * sizeof(double));
constexpr size_t kDescBytes = round256(5 * kNoAllocNb * sizeof(GemmDesc));
constexpr size_t kOffNsz = kOffDesc + kDescBytes;
constexpr size_t kOffFlags = kOffNsz + round256(kNoAllocNb * sizeof(int));
constexpr size_t kOffPart = kOffFlags + 256;
constexpr size_t kOffEmax = kOffPart + (size_t)2 * kNoAllocNb * kNoAllocLd * sizeof(double);
constexpr size_t kOffOffrel = kOffEmax + (size_t)kNoAllocNb * kNoAllocLd * sizeof(double);
constexpr size_t kOffPfail = kOffOffrel + kNoAllocNb * sizeof(double);
constexpr size_t kNoAllocBytes = kOffPfail + kNoAllocNb * sizeof(int);
// ~2.2 MiB

// The whole workspace: four nb x ld x ld work matrices, norms, GEMM tables,
// sizes, flags, refinement row sums.
static __device__ __align__(256) unsigned char g_eig_scratch[kNoAllocBytes];

struct NoAllocDevice {
    bool ready = false;
    unsigned char* base = nullptr;
};
NoAllocDevice g_noalloc_dev[kNoAllocMaxDevices];
std::mutex g_noalloc_mu;

struct NoAllocArgs {
    int n[kNoAllocNb];
    int nb, ld;
    const double* A;
    double *X, *X2, *AX, *S, *G;
};

// Same tables as eig_setup builds on the host, written by the device so that
// a call uploads nothing from host memory.
__global__ void k_eig_noalloc_tables(NoAllocArgs a, int* nsz, GemmDesc* ax, GemmDesc* sg,
                                     GemmDesc* xf, GemmDesc* rr) {
    const int b = threadIdx.x;
    if (b >= a.nb) return;
    const int n = a.n[b], ld = a.ld;
    const long o = (long)b * ld * ld;
    nsz[b] = n;
    ax[b] = GemmDesc{a.A + o, a.X + o, a.AX + o, n, n, n, ld, ld, ld, 0, 0, 1.0, 0.0, b};
    sg[2 * b] = GemmDesc{a.X + o, a.AX + o, a.S + o, n, n, n, ld, ld, ld, 1, 0, 1.0, 0.0, b, 1};
    sg[2 * b + 1] = GemmDesc{a.X + o, a.X + o, a.G + o, n, n, n, ld, ld, ld, 1, 0, 1.0, 0.0, b, 1};
    xf[b] = GemmDesc{a.X + o, a.G + o, a.X2 + o, n, n, n, ld, ld, ld, 0, 0, 1.0, 0.0, b};
    rr[b] = GemmDesc{a.AX + o, a.AX + o, a.G + o, n, n, n, ld, ld, ld, 0, 0, 0.375, 1.0, b, 1};
}

// Once per device, with that device current: the scratch address, the
// shared-memory opt-ins, and a query of every kernel the call launches so
// that they are loaded before the first real call.
int noalloc_setup(int dev, unsigned char** base) {
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    NoAllocDevice& d = g_noalloc_dev[dev];
    if (!d.ready) {
        void* p = nullptr;
        MG_CUDA(cudaGetSymbolAddress(&p, g_eig_scratch));
        MG_CUDA(cudaFuncSetAttribute(k_jacobi32, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     kSmemOptIn));
        MG_CUDA(cudaFuncSetAttribute(k_jacobi64_polish, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     kSmemOptIn));
        cudaFuncAttributes fa;
        MG_CUDA(cudaFuncGetAttributes(&fa, k_jacobi32));
        MG_CUDA(cudaFuncGetAttributes(&fa, k_jacobi64_polish));
        MG_CUDA(cudaFuncGetAttributes(&fa, k_sort_cols));
        MG_CUDA(cudaFuncGetAttributes(&fa, k_gemm64));
        MG_CUDA(cudaFuncGetAttributes(&fa, k_oa_rows));
        MG_CUDA(cudaFuncGetAttributes(&fa, k_oa_apply));
        MG_CUDA(cudaFuncGetAttributes(&fa, k_orth_prep));
        MG_CUDA(cudaFuncGetAttributes(&fa, k_frob));
        MG_CUDA(cudaFuncGetAttributes(&fa, k_eig_noalloc_tables));
        d.base = static_cast<unsigned char*>(p);
        d.ready = true;
    }
    *base = d.base;
    return MG_OK;
}

}  // namespace
}  // namespace mg

extern "C" int mg_eigh_batched_noalloc(int nb, const int* n, int ld, const double* a, double* w,
                                       double* z, int* info, void* stream) {
    using namespace mg;
    if (nb <= 0 || !n || !a || !w || !z || ld <= 0) return MG_ERR_ARG;
    if (nb > kNoAllocNb || ld > kNoAllocLd || (long)nb * ld * ld > kNoAllocElems) {
        fprintf(stderr,
                "mocca_gpu: mg_eigh_batched_noalloc: nb=%d ld=%d exceeds the static workspace "
                "(nb <= %d, ld <= %d, nb*ld*ld <= %ld)\n",
                nb, ld, kNoAllocNb, kNoAllocLd, kNoAllocElems);
        return MG_ERR_ARG;
    }
    for (int b = 0; b < nb; ++b)
        if (n[b] < 0 || n[b] > ld) return MG_ERR_ARG;
    int dev = 0;
    MG_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kNoAllocMaxDevices) return MG_ERR_ARG;
    unsigned char* base = nullptr;
    MG_TRY(noalloc_setup(dev, &base));

    mg_ctx tmp;   // carries the caller's stream, the scratch flags and the launch counter
    tmp.stream = static_cast<cudaStream_t>(stream);
    tmp.flags = reinterpret_cast<int*>(base + kOffFlags);
    EigBatch E;
    E.nb = nb;
    E.nmax = ld;
    E.ld = ld;
    E.stride = (long)ld * ld;
    E.wstride = ld;
    E.nsz = reinterpret_cast<int*>(base + kOffNsz);
    E.A = const_cast<double*>(a);   // read only
    E.X = z;
    E.w = w;
    E.X2 = reinterpret_cast<double*>(base + kOffX2);
    E.AX = reinterpret_cast<double*>(base + kOffAX);
    E.S = reinterpret_cast<double*>(base + kOffS);
    E.G = reinterpret_cast<double*>(base + kOffG);
    E.anorm = reinterpret_cast<double*>(base + kOffNorm);
    E.part = reinterpret_cast<double*>(base + kOffPart);
    E.emax = reinterpret_cast<double*>(base + kOffEmax);
    E.offrel = reinterpret_cast<double*>(base + kOffOffrel);
    E.pfail = reinterpret_cast<int*>(base + kOffPfail);
    GemmDesc* desc = reinterpret_cast<GemmDesc*>(base + kOffDesc);
    E.d_ax = desc;
    E.d_sg = desc + nb;
    E.d_xf = desc + 3 * nb;
    E.d_rr = desc + 4 * nb;
    E.attr_done = true;

    // Must start at zero on every call: the flags, and X2, whose padding
    // (outside each leading n x n block) is copied into z.
    MG_CUDA(cudaMemsetAsync(tmp.flags, 0, 256, tmp.stream));
    MG_CUDA(cudaMemsetAsync(E.X2, 0, (size_t)nb * E.stride * sizeof(double), tmp.stream));
    NoAllocArgs args{};
    for (int b = 0; b < nb; ++b) args.n[b] = n[b];
    args.nb = nb;
    args.ld = ld;
    args.A = a;
    args.X = E.X;
    args.X2 = E.X2;
    args.AX = E.AX;
    args.S = E.S;
    args.G = E.G;
    k_eig_noalloc_tables<<<1, kNoAllocNb, 0, tmp.stream>>>(args, const_cast<int*>(E.nsz), E.d_ax,
                                                          E.d_sg, E.d_xf, E.d_rr);
    MG_CUDA(cudaGetLastError());
    int st = eig_batched(&tmp, E, kSeedCold, 3, true);
    // per-matrix polish status for the caller (read after its synchronisation)
    if (st == MG_OK && info) {
        const cudaError_t ce = cudaMemcpyAsync(info, E.pfail, (size_t)nb * sizeof(int),
                                               cudaMemcpyDeviceToDevice, tmp.stream);
        if (ce != cudaSuccess) {
            fprintf(stderr, "mocca_gpu: mg_eigh_batched_noalloc: info copy failed: %s\n",
                    cudaGetErrorString(ce));
            st = MG_ERR_CUDA;
        }
    }
    tmp.flags = nullptr;
    tmp.stream = nullptr;
    return st;
}

namespace mg {

void eig_free(EigBatch& E) {
    for (void* p : {(void*)E.X, (void*)E.X2, (void*)E.AX, (void*)E.S, (void*)E.G, (void*)E.w,
                    (void*)E.anorm, (void*)E.part, (void*)E.emax, (void*)E.done,
                    (void*)E.offrel, (void*)E.pfail, (void*)E.d_ax, (void*)E.d_sg, (void*)E.d_xf,
                    (void*)E.d_rr})
        if (p) cudaFree(p);
}

}  // namespace mg
