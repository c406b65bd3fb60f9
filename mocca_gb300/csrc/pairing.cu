// pairing.cu -- mesh side of the HFB pairing step, FP64 (double-float in the
// mixed-precision form).
//
// With time reversal and signature conserved, the pairs that enter the
// pairing field and the gaps are (stored spwf j, time-reversed partner of
// stored spwf i) inside one (isospin, parity) block, and GetPairDensity with
// the time-reversal option is (src/PairingInteraction.f90:101-180)
//   P_ji(r) = -sum_c psi_jc psi_ic + i (psi_j1 psi_i2 - psi_j2 psi_i1
//                                       + psi_j3 psi_i4 - psi_j4 psi_i3).
// Both pair loops of the reference therefore become small GEMMs:
//   HFBPairingField (src/HFB.f90:350-518):
//     Y_c = Psi_c K,  K[j][i] = f_j f_i kappa(i+h, j)   (h = stored spwfs)
//     F_re += sum_c sum_i Y_c(r,i) psi_ic(r)
//     F_im -= sum_i [Y_1 psi_2 - Y_2 psi_1 + Y_3 psi_4 - Y_4 psi_3](r,i)
//     F *= DensityFactor (CompDensityFactor, ULB form,
//          src/PairingInteraction.f90:265-354)
//   HFBGaps (src/HFB.f90:520-632):
//     Delta(i, j+h) = dv f_i f_j sum_r sum_c psi_ic(r) Z_jc(r),
//     Z_j = M(r) psi_j with M built from (F_re, F_im),  Delta(j+h, i) = -Delta(i, j+h)
// and the canonical transformation of HFBOccupations (src/HFB.f90:3448-3487)
//   CanBasis_C = sum_j CanTransfo(j, C) HFBasis_j
// is a (4V x h) x (h x h) GEMM per block.  The reference's numerical cutoffs
// (HFBNumCut = 1e-12 on f_j, f_i f_j |kappa| and f_i f_j) zero the same
// entries here.
#include <cmath>

#include "df.cuh"
#include "mg_internal.cuh"

namespace mg {

namespace {

constexpr int kThreads = 256;
constexpr int kPts = 64;
constexpr int kGPts = 32;   // points per gap tile (rows padded by one word)
constexpr double kNumCut = 1e-12;

// DensityFactor = -G (1 - alpha/rhosat rho0) and the symmetric-Fermi cutoffs
__global__ void k_density_factor(const double* __restrict__ rho, long V, double g0, double g1,
                                 double a0, double a1, double rhosat, double* __restrict__ df) {
    const long v = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= V) return;
    const double r0 = rho[v] + rho[V + v];
    df[v] = -g0 * (1.0 - a0 / rhosat * r0);
    df[V + v] = -g1 * (1.0 - a1 / rhosat * r0);
}

__global__ void k_cutoffs(const double* __restrict__ e, const int* __restrict__ qn, int nwt,
                          const double* __restrict__ fermi, PairCoef pc, double* __restrict__ f) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nwt) return;
    const int it = (qn[4 * i] + 3) / 2 - 1;
    const double lam = fermi[it];
    const double up = (e[i] - lam - pc.cut[it]) / pc.mu[it];
    const double down = -(e[i] - lam + pc.cut[it]) / pc.mu[it];
    double c = sqrt(sqrt(1.0 / (1.0 + exp(up))));
    c = c * sqrt(sqrt(1.0 / (1.0 + exp(down))));
    f[i] = c;
}

// K[b][j][i] = f_j f_i kappa_b(i+h, j) with the reference's cutoffs
__global__ void k_ktilde(const double* __restrict__ kappa, const int* __restrict__ members,
                         const int* __restrict__ hsz, int hmax, int nmax,
                         const double* __restrict__ f, double* __restrict__ K) {
    const int b = blockIdx.y;
    const int h = hsz[b];
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= h * h) return;
    const int j = t / h, i = t % h;
    const int N = 2 * h;
    const double fj = f[members[b * hmax + j]], fi = f[members[b * hmax + i]];
    const double kij = kappa[(long)b * nmax * nmax + (long)(i + h) * N + j];
    double val = fj * fi * kij;
    if (fj < kNumCut || fj * fi * fabs(kij) < kNumCut) val = 0.0;
    K[(long)b * hmax * hmax + (long)j * h + i] = val;
}

// Per-block pairing-field partials: part[b][0|1][V]
__global__ void __launch_bounds__(kThreads)
k_pair_field(const double* __restrict__ psi, const int* __restrict__ members,
             const int* __restrict__ hsz, int hmax, const double* __restrict__ K, long V,
             double* __restrict__ part) {
    extern __shared__ double sm[];
    const int b = blockIdx.y;
    const int h = hsz[b];
    const long p0 = (long)blockIdx.x * kPts;
    double* sK = sm;                    // h*h
    double* sP = sm + h * h;            // [j][c][kPts]
    double* red = sP + h * 4 * kPts;    // [2][kThreads]
    for (int t = threadIdx.x; t < h * h; t += kThreads) sK[t] = K[(long)b * hmax * hmax + t];
    for (int t = threadIdx.x; t < h * 4 * kPts; t += kThreads) {
        const int j = t / (4 * kPts), c = (t / kPts) % 4, q = t % kPts;
        const long v = p0 + q;
        sP[t] = v < V ? psi[((long)members[b * hmax + j] * 4 + c) * V + v] : 0.0;
    }
    __syncthreads();
    const int q = threadIdx.x % kPts;
    const int grp = threadIdx.x / kPts;
    constexpr int kGroups = kThreads / kPts;
    double fr = 0.0, fi = 0.0;
    for (int i = grp; i < h; i += kGroups) {
        double y[4] = {0.0, 0.0, 0.0, 0.0};
        for (int j = 0; j < h; ++j) {
            const double k = sK[j * h + i];
            const double* pj = sP + j * 4 * kPts + q;
#pragma unroll
            for (int c = 0; c < 4; ++c) y[c] = fma(pj[c * kPts], k, y[c]);
        }
        const double* pi = sP + i * 4 * kPts + q;
        const double a0 = pi[0], a1 = pi[kPts], a2 = pi[2 * kPts], a3 = pi[3 * kPts];
        fr = fma(y[0], a0, fr);
        fr = fma(y[1], a1, fr);
        fr = fma(y[2], a2, fr);
        fr = fma(y[3], a3, fr);
        fi = fi - (y[0] * a1 - y[1] * a0 + y[2] * a3 - y[3] * a2);
    }
    red[threadIdx.x] = fr;
    red[kThreads + threadIdx.x] = fi;
    __syncthreads();
    if (grp == 0 && p0 + q < V) {
        double sr = 0.0, si = 0.0;
        for (int g = 0; g < kGroups; ++g) {
            sr += red[g * kPts + q];
            si += red[kThreads + g * kPts + q];
        }
        part[((long)b * 2 + 0) * V + p0 + q] = sr;
        part[((long)b * 2 + 1) * V + p0 + q] = si;
    }
}

// F_it = (part[2it] + part[2it+1]) * DensityFactor_it
__global__ void k_pair_field_finish(const double* __restrict__ part, const double* __restrict__ df,
                                    long V, double* __restrict__ fre, double* __restrict__ fim) {
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 2 * V) return;
    const int it = (int)(t / V);
    const long v = t % V;
    const double r = part[((long)(2 * it) * 2 + 0) * V + v] + part[((long)(2 * it + 1) * 2 + 0) * V + v];
    const double m = part[((long)(2 * it) * 2 + 1) * V + v] + part[((long)(2 * it + 1) * 2 + 1) * V + v];
    fre[t] = r * df[t];
    fim[t] = m * df[t];
}

// Gap partials over point chunks: gpart[b][chunk][i*h + j]
__global__ void __launch_bounds__(kThreads)
k_pair_gaps(const double* __restrict__ psi, const int* __restrict__ members,
            const int* __restrict__ hsz, int hmax, const double* __restrict__ fre,
            const double* __restrict__ fim, long V, int nchunk, double* __restrict__ gpart) {
    extern __shared__ double sm[];
    const int b = blockIdx.y, it = b / 2;
    const int h = hsz[b];
    constexpr int kRow = 4 * kGPts + 1;   // padded row: spreads j over banks
    double* sA = sm;                   // [i][c][kGPts] psi
    double* sZ = sm + h * kRow;        // [j][c][kGPts] M psi
    double* acc = sZ + h * kRow;       // h*h accumulators
    for (int t = threadIdx.x; t < h * h; t += kThreads) acc[t] = 0.0;
    const long per = (V + nchunk - 1) / nchunk;
    const long v0 = (long)blockIdx.x * per, v1 = min(V, v0 + per);
    for (long base = v0; base < v1; base += kGPts) {
        __syncthreads();
        for (int t = threadIdx.x; t < h * kGPts; t += kThreads) {
            const int j = t / kGPts, q = t % kGPts;
            const long v = base + q;
            double a[4] = {0, 0, 0, 0}, r = 0.0, m = 0.0;
            if (v < v1) {
                const long o = (long)members[b * hmax + j] * 4 * V + v;
#pragma unroll
                for (int c = 0; c < 4; ++c) a[c] = psi[o + c * V];
                r = fre[it * V + v];
                m = fim[it * V + v];
            }
            double* pa = sA + j * kRow + q;
            double* pz = sZ + j * kRow + q;
#pragma unroll
            for (int c = 0; c < 4; ++c) pa[c * kGPts] = a[c];
            pz[0] = fma(m, a[1], -r * a[0]);
            pz[kGPts] = fma(-m, a[0], -r * a[1]);
            pz[2 * kGPts] = fma(m, a[3], -r * a[2]);
            pz[3 * kGPts] = fma(-m, a[2], -r * a[3]);
        }
        __syncthreads();
        for (int pr = threadIdx.x; pr < h * h; pr += kThreads) {
            const int i = pr / h, j = pr % h;
            const double* pa = sA + i * kRow;
            const double* pz = sZ + j * kRow;
            double s = acc[pr];
#pragma unroll 4
            for (int q = 0; q < 4 * kGPts; ++q) s = fma(pa[q], pz[q], s);
            acc[pr] = s;
        }
    }
    __syncthreads();
    for (int t = threadIdx.x; t < h * h; t += kThreads)
        gpart[((long)b * nchunk + blockIdx.x) * hmax * hmax + t] = acc[t];
}

// Delta(i, j+h) = dv f_i f_j sum_chunks, Delta(j+h, i) = -Delta(i, j+h); rest 0
__global__ void k_gaps_finish(const double* __restrict__ gpart, const int* __restrict__ members,
                              const int* __restrict__ hsz, int hmax, int nmax, int nchunk,
                              const double* __restrict__ f, double dv, double* __restrict__ delta) {
    const int b = blockIdx.y;
    const int h = hsz[b], N = 2 * h;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= N * N) return;
    const int r = t / N, c = t % N;
    double val = 0.0;
    if (r < h && c >= h) {
        const int i = r, j = c - h;
        const double fi = f[members[b * hmax + i]], fj = f[members[b * hmax + j]];
        if (fi * fj >= kNumCut) {
            double s = 0.0;
            for (int q = 0; q < nchunk; ++q) s += gpart[((long)b * nchunk + q) * hmax * hmax + i * h + j];
            val = dv * fi * fj * s;
        }
    } else if (r >= h && c < h) {
        const int i = c, j = r - h;
        const double fi = f[members[b * hmax + i]], fj = f[members[b * hmax + j]];
        if (fi * fj >= kNumCut) {
            double s = 0.0;
            for (int q = 0; q < nchunk; ++q) s += gpart[((long)b * nchunk + q) * hmax * hmax + i * h + j];
            val = -(dv * fi * fj * s);
        }
    }
    delta[(long)b * nmax * nmax + t] = val;
}

// CanBasis_{start_b + C} = sum_j T[b][j][C] HFBasis_{members[j]} over a tile of points
__global__ void __launch_bounds__(kThreads)
k_can_transform(const double* __restrict__ psi, const int* __restrict__ members,
                const int* __restrict__ hsz, const int* __restrict__ cstart, int hmax,
                const double* __restrict__ T, long V4, double* __restrict__ can) {
    extern __shared__ double sm[];
    const int b = blockIdx.y;
    const int h = hsz[b];
    double* sT = sm;            // h*h
    double* sP = sm + h * h;    // [j][kPts]
    for (int t = threadIdx.x; t < h * h; t += kThreads) sT[t] = T[(long)b * hmax * hmax + t];
    const long p0 = (long)blockIdx.x * kPts;
    for (int t = threadIdx.x; t < h * kPts; t += kThreads) {
        const int j = t / kPts, q = t % kPts;
        const long p = p0 + q;
        sP[t] = p < V4 ? psi[(long)members[b * hmax + j] * V4 + p] : 0.0;
    }
    __syncthreads();
    for (int t = threadIdx.x; t < h * kPts; t += kThreads) {
        const int C = t / kPts, q = t % kPts;
        const long p = p0 + q;
        if (p >= V4) continue;
        double s = 0.0;
        for (int j = 0; j < h; ++j) s = fma(sT[j * h + C], sP[j * kPts + q], s);
        can[(long)(cstart[b] + C) * V4 + p] = s;
    }
}

// ---- mixed precision: the three mesh contractions in double-float -----------------
// (df.cuh; same tiling, a dfl takes the 8 bytes of a double in shared memory;
// partial sums leave the kernels as FP64)

__global__ void __launch_bounds__(kThreads)
k_pair_field_df(const double* __restrict__ psi, const int* __restrict__ members,
                const int* __restrict__ hsz, int hmax, const double* __restrict__ K, long V,
                double* __restrict__ part) {
    extern __shared__ double sm[];
    const int b = blockIdx.y;
    const int h = hsz[b];
    const long p0 = (long)blockIdx.x * kPts;
    dfl* sK = reinterpret_cast<dfl*>(sm);   // h*h
    dfl* sP = sK + h * h;                   // [j][c][kPts]
    double* red = sm + h * h + h * 4 * kPts;  // [2][kThreads]
    for (int t = threadIdx.x; t < h * h; t += kThreads) sK[t] = df_from(K[(long)b * hmax * hmax + t]);
    for (int t = threadIdx.x; t < h * 4 * kPts; t += kThreads) {
        const int j = t / (4 * kPts), c = (t / kPts) % 4, q = t % kPts;
        const long v = p0 + q;
        sP[t] = df_from(v < V ? psi[((long)members[b * hmax + j] * 4 + c) * V + v] : 0.0);
    }
    __syncthreads();
    const int q = threadIdx.x % kPts;
    const int grp = threadIdx.x / kPts;
    constexpr int kGroups = kThreads / kPts;
    float frh = 0.f, frl = 0.f, fih = 0.f, fil = 0.f;
    for (int i = grp; i < h; i += kGroups) {
        float yh[4] = {0.f, 0.f, 0.f, 0.f}, yl[4] = {0.f, 0.f, 0.f, 0.f};
        for (int j = 0; j < h; ++j) {
            const dfl k = sK[j * h + i];
            const dfl* pj = sP + j * 4 * kPts + q;
#pragma unroll
            for (int c = 0; c < 4; ++c) df_acc(yh[c], yl[c], pj[c * kPts], k);
        }
        dfl y[4];
#pragma unroll
        for (int c = 0; c < 4; ++c) y[c] = df_norm(dfl{yh[c], yl[c]});
        const dfl* pi = sP + i * 4 * kPts + q;
        const dfl a0 = pi[0], a1 = pi[kPts], a2 = pi[2 * kPts], a3 = pi[3 * kPts];
        df_acc(frh, frl, y[0], a0);
        df_acc(frh, frl, y[1], a1);
        df_acc(frh, frl, y[2], a2);
        df_acc(frh, frl, y[3], a3);
        df_acc(fih, fil, y[0], df_neg(a1));
        df_acc(fih, fil, y[1], a0);
        df_acc(fih, fil, y[2], df_neg(a3));
        df_acc(fih, fil, y[3], a2);
    }
    red[threadIdx.x] = df_to(dfl{frh, frl});
    red[kThreads + threadIdx.x] = df_to(dfl{fih, fil});
    __syncthreads();
    if (grp == 0 && p0 + q < V) {
        double sr = 0.0, si = 0.0;
        for (int g = 0; g < kGroups; ++g) {
            sr += red[g * kPts + q];
            si += red[kThreads + g * kPts + q];
        }
        part[((long)b * 2 + 0) * V + p0 + q] = sr;
        part[((long)b * 2 + 1) * V + p0 + q] = si;
    }
}

__global__ void __launch_bounds__(kThreads)
k_pair_gaps_df(const double* __restrict__ psi, const int* __restrict__ members,
               const int* __restrict__ hsz, int hmax, const double* __restrict__ fre,
               const double* __restrict__ fim, long V, int nchunk, double* __restrict__ gpart) {
    extern __shared__ double sm[];
    const int b = blockIdx.y, it = b / 2;
    const int h = hsz[b];
    constexpr int kRow = 4 * kGPts + 1;
    dfl* sA = reinterpret_cast<dfl*>(sm);   // [i][c][kGPts] psi
    dfl* sZ = sA + h * kRow;                // [j][c][kGPts] M psi
    double* acc = sm + 2 * h * kRow;        // h*h accumulators (FP64)
    for (int t = threadIdx.x; t < h * h; t += kThreads) acc[t] = 0.0;
    const long per = (V + nchunk - 1) / nchunk;
    const long v0 = (long)blockIdx.x * per, v1 = min(V, v0 + per);
    for (long base = v0; base < v1; base += kGPts) {
        __syncthreads();
        for (int t = threadIdx.x; t < h * kGPts; t += kThreads) {
            const int j = t / kGPts, q = t % kGPts;
            const long v = base + q;
            dfl a[4] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
            dfl r = {0.f, 0.f}, m = {0.f, 0.f};
            if (v < v1) {
                const long o = (long)members[b * hmax + j] * 4 * V + v;
#pragma unroll
                for (int c = 0; c < 4; ++c) a[c] = df_from(psi[o + c * V]);
                r = df_from(fre[it * V + v]);
                m = df_from(fim[it * V + v]);
            }
            dfl* pa = sA + j * kRow + q;
            dfl* pz = sZ + j * kRow + q;
#pragma unroll
            for (int c = 0; c < 4; ++c) pa[c * kGPts] = a[c];
            const dfl nr = df_neg(r), nm = df_neg(m);
            pz[0] = df_fma(m, a[1], df_mul(nr, a[0]));
            pz[kGPts] = df_fma(nm, a[0], df_mul(nr, a[1]));
            pz[2 * kGPts] = df_fma(m, a[3], df_mul(nr, a[2]));
            pz[3 * kGPts] = df_fma(nm, a[2], df_mul(nr, a[3]));
        }
        __syncthreads();
        for (int pr = threadIdx.x; pr < h * h; pr += kThreads) {
            const int i = pr / h, j = pr % h;
            const dfl* pa = sA + i * kRow;
            const dfl* pz = sZ + j * kRow;
            float sh = 0.f, sl = 0.f;
#pragma unroll 4
            for (int q = 0; q < 4 * kGPts; ++q) df_acc(sh, sl, pa[q], pz[q]);
            acc[pr] += df_to(dfl{sh, sl});
        }
    }
    __syncthreads();
    for (int t = threadIdx.x; t < h * h; t += kThreads)
        gpart[((long)b * nchunk + blockIdx.x) * hmax * hmax + t] = acc[t];
}

__global__ void __launch_bounds__(kThreads)
k_can_transform_df(const double* __restrict__ psi, const int* __restrict__ members,
                   const int* __restrict__ hsz, const int* __restrict__ cstart, int hmax,
                   const double* __restrict__ T, long V4, double* __restrict__ can) {
    extern __shared__ double sm[];
    const int b = blockIdx.y;
    const int h = hsz[b];
    dfl* sT = reinterpret_cast<dfl*>(sm);   // h*h
    dfl* sP = sT + h * h;                   // [j][kPts]
    for (int t = threadIdx.x; t < h * h; t += kThreads) sT[t] = df_from(T[(long)b * hmax * hmax + t]);
    const long p0 = (long)blockIdx.x * kPts;
    for (int t = threadIdx.x; t < h * kPts; t += kThreads) {
        const int j = t / kPts, q = t % kPts;
        const long p = p0 + q;
        sP[t] = df_from(p < V4 ? psi[(long)members[b * hmax + j] * V4 + p] : 0.0);
    }
    __syncthreads();
    for (int t = threadIdx.x; t < h * kPts; t += kThreads) {
        const int C = t / kPts, q = t % kPts;
        const long p = p0 + q;
        if (p >= V4) continue;
        float sh = 0.f, sl = 0.f;
        for (int j = 0; j < h; ++j) df_acc(sh, sl, sT[j * h + C], sP[j * kPts + q]);
        can[(long)(cstart[b] + C) * V4 + p] = df_to(dfl{sh, sl});
    }
}

}  // namespace

int pairing_mesh(mg_ctx* c) {
    Hfb& H = c->hfb;
    const long V = c->V;
    const int hmax = H.hmax, nmax = H.nmax;
    const Basis& B = c->bas[MG_HF_BASIS];
    k_density_factor<<<div_up(V, kThreads), kThreads, 0, c->stream>>>(
        c->rho, V, H.pp.strength[0], H.pp.strength[1], H.pp.alpha[0], H.pp.alpha[1], H.pp.rhosat,
        H.dfac);
    MG_LAUNCHED(c);
    k_cutoffs<<<div_up(c->p.nwt, 128), 128, 0, c->stream>>>(B.e, B.qn, c->p.nwt, H.fermi_d, H.pc,
                                                            H.pcut);
    MG_LAUNCHED(c);
    k_ktilde<<<dim3(div_up(hmax * hmax, 128), 4), 128, 0, c->stream>>>(H.kappa, H.members, H.hsz,
                                                                       hmax, nmax, H.pcut, H.ktil);
    MG_LAUNCHED(c);
    const size_t sm_f = (size_t)(hmax * hmax + hmax * 4 * kPts + 2 * kThreads) * sizeof(double);
    const bool mixed = c->cur_precision == MG_MIXED;
    if (mixed && c->tc_mesh_ok && hmax <= kMeshTcMax)
        MG_TRY(pair_field_tc(c));   // tensor cores (meshgemm_tc.cu)
    else if (mixed)
        k_pair_field_df<<<dim3(div_up(V, kPts), 4), kThreads, sm_f, c->stream>>>(
            B.psi, H.members, H.hsz, hmax, H.ktil, V, H.fpart);
    else
        k_pair_field<<<dim3(div_up(V, kPts), 4), kThreads, sm_f, c->stream>>>(
            B.psi, H.members, H.hsz, hmax, H.ktil, V, H.fpart);
    if (!(mixed && c->tc_mesh_ok && hmax <= kMeshTcMax)) MG_LAUNCHED(c);
    k_pair_field_finish<<<div_up(2 * V, kThreads), kThreads, 0, c->stream>>>(H.fpart, H.dfac, V,
                                                                           H.fre, H.fim);
    MG_LAUNCHED(c);
    const size_t sm_g = (size_t)(2 * hmax * (4 * kGPts + 1) + hmax * hmax) * sizeof(double);
    if (mixed && c->tc_mesh_ok && hmax <= kMeshTcMax) {
        // tensor cores (meshgemm_tc.cu): the summed partials go to chunk slot 0
        MG_TRY(gaps_tc(c, H.gpart));
        k_gaps_finish<<<dim3(div_up(nmax * nmax, 128), 4), 128, 0, c->stream>>>(
            H.gpart, H.members, H.hsz, hmax, nmax, 1, H.pcut, c->dv, H.delta);
        MG_LAUNCHED(c);
        return MG_OK;
    }
    if (mixed)
        k_pair_gaps_df<<<dim3(H.gchunk, 4), kThreads, sm_g, c->stream>>>(
            B.psi, H.members, H.hsz, hmax, H.fre, H.fim, V, H.gchunk, H.gpart);
    else
        k_pair_gaps<<<dim3(H.gchunk, 4), kThreads, sm_g, c->stream>>>(
            B.psi, H.members, H.hsz, hmax, H.fre, H.fim, V, H.gchunk, H.gpart);
    MG_LAUNCHED(c);
    k_gaps_finish<<<dim3(div_up(nmax * nmax, 128), 4), 128, 0, c->stream>>>(
        H.gpart, H.members, H.hsz, hmax, nmax, H.gchunk, H.pcut, c->dv, H.delta);
    MG_LAUNCHED(c);
    return MG_OK;
}

int canonical_transform(mg_ctx* c) {
    Hfb& H = c->hfb;
    const long V4 = 4 * c->V;
    const size_t sm = (size_t)(H.hmax * H.hmax + H.hmax * kPts) * sizeof(double);
    if (c->cur_precision == MG_MIXED && c->tc_mesh_ok && H.hmax <= kMeshTcMax)
        return can_transform_tc(c);   // tensor cores (meshgemm_tc.cu)
    if (c->cur_precision == MG_MIXED)
        k_can_transform_df<<<dim3(div_up(V4, kPts), 4), kThreads, sm, c->stream>>>(
            c->bas[MG_HF_BASIS].psi, H.members, H.hsz, H.cstart, H.hmax, H.cantr, V4,
            c->bas[MG_CAN_BASIS].psi);
    else
        k_can_transform<<<dim3(div_up(V4, kPts), 4), kThreads, sm, c->stream>>>(
            c->bas[MG_HF_BASIS].psi, H.members, H.hsz, H.cstart, H.hmax, H.cantr, V4,
            c->bas[MG_CAN_BASIS].psi);
    MG_LAUNCHED(c);
    return MG_OK;
}

int pairing_set_smem(mg_ctx* c) {
    const int hmax = c->hfb.hmax;
    const size_t sm_f = (size_t)(hmax * hmax + hmax * 4 * kPts + 2 * kThreads) * sizeof(double);
    const size_t sm_g = (size_t)(2 * hmax * (4 * kGPts + 1) + hmax * hmax) * sizeof(double);
    if (sm_f > 220 * 1024 || sm_g > 220 * 1024) return MG_ERR_ARG;
    MG_CUDA(cudaFuncSetAttribute(k_pair_field, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024));
    MG_CUDA(cudaFuncSetAttribute(k_pair_gaps, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024));
    MG_CUDA(cudaFuncSetAttribute(k_can_transform, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024));
    MG_CUDA(cudaFuncSetAttribute(k_pair_field_df, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024));
    MG_CUDA(cudaFuncSetAttribute(k_pair_gaps_df, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024));
    MG_CUDA(cudaFuncSetAttribute(k_can_transform_df, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024));
    return MG_OK;
}

}  // namespace mg
