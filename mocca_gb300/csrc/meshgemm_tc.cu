// meshgemm_tc.cu -- the mesh-sized contractions of the mixed form on the
// tcgen05 tensor cores (exact BF16 digit products, ozaki.cuh): the
// Gram-Schmidt overlap and apply, and the canonical-basis transform.
//
// Blocks of up to kMeshTcMax (80) spinors; above 64, four accumulators take
// 512 TMEM columns and the kernels run one CTA per SM.
//
// Gram-Schmidt (gs.cu; GramSchmidt, src/SpwfStorage.f90:372-480, as
// Q = Psi R^{-1} with S = R^T R per (isospin, parity, signature) block in
// energy order):
//   k_gs_overlap_tc : S partial sums over 256-point chunks.  Rows of the
//                     MMA are the block's spinors (zero beyond nb), K the
//                     chunk's points; A and B are the same digit planes.  Each
//                     (spinor, chunk) row gets its own power of two.  The
//                     partials go to the same table as the FP64 kernel, so
//                     k_gs_sum / k_gs_factor (gs.cu) finish the job.
// Block apply, out_l(p) = sum_k C[k][l] in_k(p) per block of spinors:
//   k_coef_digits   : digit planes of C (rows: output l, K: input k), one
//                     power of two per row;
//   k_apply_tc      : 128 points per CTA (MMA M), K = the block's spinors, FP64
//                     output.  Gram-Schmidt: C = R^{-1}, in place, plus the
//                     GradDesc history upd_l = out_l - upd_l.  Canonical basis
//                     (HFBOccupations, src/HFB.f90:3448-3487): C = CanTransfo,
//                     HF basis in, canonical basis out.
// A 256-point chunk keeps every digit-weight group of the overlap below 2^24
// (at most 3 pairs x 256 points x 2^14), so its FP32 sums are exact.
#include <algorithm>
#include <vector>

#include "df.cuh"
#include "mg_internal.cuh"
#include "ozaki.cuh"
#include "tc.cuh"

namespace mg {

namespace {

using oz::kDigits;
constexpr int kRows = 128;            // MMA M
constexpr int kChunk = 256;           // overlap points per CTA
constexpr int kStage = 32;            // overlap points per MMA stage (K)
constexpr int kStagePlane = kRows * kStage * 2;   // bytes of one digit plane of a stage
// TMEM columns for four accumulators of N columns: 256 up to N = 64, 512 above
// (one CTA per SM then; the launches keep the shared memory above half of the
// SM's so that a second CTA never waits in tcgen05.alloc)
__host__ __device__ constexpr uint32_t tmem_cols(int N) { return 4 * N <= 256 ? 256u : 512u; }
constexpr long kXdStride = (long)kMeshTcMax * kMeshTcMax;   // per block in the coefficient planes
constexpr size_t kOneCtaSmem = 116 * 1024;
constexpr long long kWaitCycles = 4000000000LL;

// Block sizes and list offsets: Gram-Schmidt blocks come from a start table,
// pairing blocks have hsz[b] members listed at b * hmax.
struct BlockIdx {
    const int* starts;
    const int* hsz;
    int hmax;
    __device__ int nb(int b) const { return starts ? starts[b + 1] - starts[b] : hsz[b]; }
    __device__ int off(int b) const { return starts ? starts[b] : b * hmax; }
};

__device__ __forceinline__ double pow2d(int x) {
    return x < -1022 ? 0.0 : __longlong_as_double((long long)(min(x, 1023) + 1023) << 52);
}

__global__ void __launch_bounds__(256, 2)
k_gs_overlap_tc(const double* __restrict__ psi, const int* __restrict__ starts,
                const int* __restrict__ ordered, int nbmax, long V4, int nchunk,
                double* __restrict__ part, int* __restrict__ status) {
    extern __shared__ uint8_t smraw[];
    __shared__ __align__(8) uint64_t mbar[2];
    __shared__ uint32_t tmem_slot;
    __shared__ int sE[kRows];
    const int b = blockIdx.y, chunk = blockIdx.x;
    const int s0 = starts[b], nb = starts[b + 1] - s0;
    if (nb == 0) return;
    const int N = max(16, (nb + 15) / 16 * 16);
    const uint32_t tcols = tmem_cols(N);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    // rows row0 and row0 + 64 (blocks above 64 spinors); a row's 4 K groups
    // sit on 4 neighbouring lanes
    const int row0 = tid >> 2, g = tid & 3;

    const uint32_t s0a = tc::smem_u32(smraw);
    uint8_t* base = smraw + ((128u - (s0a & 127u)) & 127u);
    // two stage buffers of kDigits planes; rows >= nb stay zero
    for (int t = tid; t < 2 * kDigits * kStagePlane / 16; t += 256)
        reinterpret_cast<uint4*>(base)[t] = make_uint4(0u, 0u, 0u, 0u);
    if (warp == 0) tc::alloc(&tmem_slot, tcols);
    if (tid == 0) {
        tc::mbar_init(&mbar[0], 1);
        tc::mbar_init(&mbar[1], 1);
    }
    const long p0 = (long)chunk * kChunk;
    const int npts = (int)min((long)kChunk, V4 - p0);
    const int nst = (npts + kStage - 1) / kStage;
    bool live[2];
    const double* src[2];
    int emax[2] = {0, 0};
#pragma unroll
    for (int r = 0; r < 2; ++r) {
        const int row = row0 + 64 * r;
        live[r] = row < nb;
        src[r] = live[r] ? psi + (long)ordered[s0 + row] * V4 + p0 : psi;
        // largest exponent of the row over the chunk
        if (live[r]) {
            for (int s = 0; s < nst; ++s) {
#pragma unroll
                for (int h = 0; h < 8; ++h) {
                    const int q = s * kStage + 8 * g + h;
                    if (q < npts) emax[r] = max(emax[r], oz::bexp(src[r][q]));
                }
            }
        }
        emax[r] = max(emax[r], __shfl_xor_sync(0xffffffffu, emax[r], 1));
        emax[r] = max(emax[r], __shfl_xor_sync(0xffffffffu, emax[r], 2));
        if (live[r] && g == 0) sE[row] = emax[r];
    }

    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tmem = tmem_slot;
    const uint32_t idesc = tc::idesc_bf16(kRows, N);
    bool ok = true;
    for (int s = 0; s < nst; ++s) {
        const int buf = s & 1;
        uint8_t* planes = base + buf * kDigits * kStagePlane;
        if (s >= 2) ok &= tc::mbar_wait(&mbar[buf], ((s - 2) >> 1) & 1, kWaitCycles);
#pragma unroll
        for (int r = 0; r < 2; ++r) {
            if (!live[r]) continue;
            double v[8];
#pragma unroll
            for (int h = 0; h < 8; ++h) {
                const int q = s * kStage + 8 * g + h;
                v[h] = q < npts ? src[r][q] : 0.0;
            }
            uint4 w[kDigits];
            oz::digits8(v, emax[r], w);
#pragma unroll
            for (int a = 0; a < kDigits; ++a)
                *reinterpret_cast<uint4*>(planes + a * kStagePlane +
                                          tc::kmajor_off(row0 + 64 * r, 8 * g)) = w[a];
        }
        tc::fence_proxy_async();
        tc::fence_before();
        __syncthreads();
        tc::fence_after();
        if (tid == 0) {
            const uint32_t pa = tc::smem_u32(planes);
            oz::issue_pairs<2>(tmem, N, idesc, pa, kStagePlane, tc::kSbo, pa, kStagePlane,
                               tc::kSbo, s > 0);
            tc::commit(&mbar[buf]);
        }
    }
    const int last = nst - 1;
    ok &= tc::mbar_wait(&mbar[last & 1], (last >> 1) & 1, kWaitCycles);
    ok = __syncthreads_and(ok) != 0;
    tc::fence_after();
    if (ok) {
        // D[k][l], k = TMEM lane (row), l = column; warps w and w + 4 share lane quarter w % 4
        const int quarter = warp & 3, colh = warp >> 2;
        const int k = quarter * 32 + lane;
        const uint32_t trow = tmem + ((uint32_t)(quarter * 32) << 16);
        double* out = part + ((long)b * nchunk + chunk) * nbmax * nbmax;
        const int ek = k < nb ? sE[k] - 1023 : 0;
        for (int q = 0; q < N / 16; ++q) {
            const int c0 = 16 * q + 8 * colh;
            uint32_t r0[8], r1[8], r2[8], r3[8];
            __syncwarp();
            tc::ld8(trow + (uint32_t)(0 * N + c0), r0);
            tc::ld8(trow + (uint32_t)(1 * N + c0), r1);
            tc::ld8(trow + (uint32_t)(2 * N + c0), r2);
            tc::ld8(trow + (uint32_t)(3 * N + c0), r3);
            tc::wait_ld(r0);
            tc::wait_ld(r1);
            tc::wait_ld(r2);
            tc::wait_ld(r3);
            if (k >= nb) continue;
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const int l = c0 + u;
                if (l >= nb || l < k) continue;
                const dfl o = oz::combine4(__uint_as_float(r0[u]), __uint_as_float(r1[u]),
                                           __uint_as_float(r2[u]), __uint_as_float(r3[u]));
                const double val = (f2d_bits(o.h) + f2d_bits(o.l)) * pow2d(ek + sE[l] - 1023 - 12);
                out[k * nbmax + l] = val;
            }
        }
    } else if (tid == 0) {
        atomicExch(status, 1);
    }
    if (!ok) {
        tc::mbar_wait(&mbar[0], 0, kWaitCycles);   // let the MMAs drain before the columns go
        tc::mbar_wait(&mbar[1], 0, kWaitCycles);
    }
    tc::fence_before();
    __syncthreads();
    if (warp == 0) tc::dealloc(tmem, tcols);
}

// Digit planes of C (per block: kDigits planes of Np rows x Np, row l = output
// l, K = input k; C[k][l] = coef[b * bstride + k * ld + l], ld = nb when 0) and
// the row exponents (biased).
__global__ void k_coef_digits(const double* __restrict__ coef, long bstride, int ld, BlockIdx bi,
                              uint16_t* __restrict__ xd, int* __restrict__ xe) {
    const int b = blockIdx.x;
    const int nb = bi.nb(b);
    const int Np = max(16, (nb + 15) / 16 * 16);
    const int l = threadIdx.x;
    if (nb == 0 || l >= Np) return;
    const int ldc = ld > 0 ? ld : nb;
    const double* X = coef + (long)b * bstride;
    uint16_t* out = xd + (long)b * kDigits * kXdStride;
    int emax = 0;
    if (l < nb)
        for (int k = 0; k < nb; ++k) emax = max(emax, oz::bexp(X[k * ldc + l]));
    xe[b * kMeshTcMax + l] = emax;
    for (int k = 0; k < Np; ++k) {
        const double v = (l < nb && k < nb) ? X[k * ldc + l] : 0.0;
        uint32_t d[kDigits];
        oz::digits(v, emax, d);
        const uint32_t o = tc::kmajor_off_g(l, k, Np / 8) / 2;
#pragma unroll
        for (int a = 0; a < kDigits; ++a) out[(long)a * Np * Np + o] = (uint16_t)(d[a] >> 16);
    }
}

// out_l = sum_k C[k][l] in_k over 128 points (in_k = in[in_list[off + k]],
// out_l = out[out_list[off + l]] or out[out_base[b] + l]); when upd is given,
// upd_l = out_l - upd_l.  in and out may be the same array (in place).
// Thread t: point row = t % 128, K groups h, h + 2, h + 4, ... (h = t / 128);
// up to 48 spinors the point's values stay in registers between the
// exponent and the digits, above they are read twice.
__global__ void __launch_bounds__(256, 2)
k_apply_tc(const double* in, double* out, double* __restrict__ upd, BlockIdx bi,
           const int* __restrict__ in_list, const int* __restrict__ out_list,
           const int* __restrict__ out_base, const uint16_t* __restrict__ xd,
           const int* __restrict__ xe, long V4, int* __restrict__ status) {
    extern __shared__ uint8_t smraw[];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_slot;
    __shared__ int sEmax[256];
    __shared__ int sXe[kMeshTcMax];
    __shared__ int sIdx[kMeshTcMax];
    __shared__ int sOut[kMeshTcMax];
    const int b = blockIdx.y;
    const int s0 = bi.off(b), nb = bi.nb(b);
    if (nb == 0) return;
    const int Np = max(16, (nb + 15) / 16 * 16);
    const int kg = Np / 8;
    const uint32_t tcols = tmem_cols(Np);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int row = tid & (kRows - 1), half = tid >> 7;
    const long p = (long)blockIdx.x * kRows + row;
    const bool live = p < V4;

    const uint32_t s0a = tc::smem_u32(smraw);
    uint8_t* base = smraw + ((128u - (s0a & 127u)) & 127u);
    const int aPlane = kRows * Np * 2, bPlane = Np * Np * 2;
    uint8_t* sA = base;
    uint8_t* sB = sA + kDigits * aPlane;
    if (warp == 0) tc::alloc(&tmem_slot, tcols);
    if (tid == 0) tc::mbar_init(&mbar, 1);
    {
        const uint4* src = reinterpret_cast<const uint4*>(xd + (long)b * kDigits * kXdStride);
        uint4* dst = reinterpret_cast<uint4*>(sB);
        for (int t = tid; t < kDigits * bPlane / 16; t += 256) dst[t] = src[t];
        if (tid < kMeshTcMax) {
            sXe[tid] = tid < Np ? xe[b * kMeshTcMax + tid] : 0;
            sIdx[tid] = tid < nb ? in_list[s0 + tid] : 0;
            sOut[tid] = tid < nb ? (out_list ? out_list[s0 + tid] : out_base[b] + tid) : 0;
        }
    }
    __syncthreads();
    if (kg <= 6) {
        // the point's values psi_k(p) for this thread's K groups
        double v[24];
#pragma unroll
        for (int u = 0; u < 24; ++u) {
            const int k = 8 * (half + 2 * (u >> 3)) + (u & 7);
            v[u] = (live && k < nb) ? in[(long)sIdx[k] * V4 + p] : 0.0;
        }
        int emax = 0;
#pragma unroll
        for (int u = 0; u < 24; ++u) emax = max(emax, oz::bexp(v[u]));
        sEmax[tid] = emax;
        __syncthreads();
        emax = max(sEmax[row], sEmax[row + kRows]);
#pragma unroll
        for (int gg = 0; gg < 3; ++gg) {
            const int g = half + 2 * gg;
            if (g >= kg) continue;
            uint4 w[kDigits];
            if (8 * g < nb) {
                double v8[8];
#pragma unroll
                for (int h = 0; h < 8; ++h) v8[h] = v[8 * gg + h];
                oz::digits8(v8, emax, w);
            } else {
#pragma unroll
                for (int a = 0; a < kDigits; ++a) w[a] = make_uint4(0u, 0u, 0u, 0u);
            }
#pragma unroll
            for (int a = 0; a < kDigits; ++a)
                *reinterpret_cast<uint4*>(sA + a * aPlane + tc::kmajor_off_g(row, 8 * g, kg)) = w[a];
        }
    } else {
        // blocks of 49 to kMeshTcMax spinors: the exponent pass, then the
        // digits pass over the same values
        int emax = 0;
        for (int g = half; g < kg; g += 2)
#pragma unroll
            for (int h = 0; h < 8; ++h) {
                const int k = 8 * g + h;
                if (live && k < nb) emax = max(emax, oz::bexp(in[(long)sIdx[k] * V4 + p]));
            }
        sEmax[tid] = emax;
        __syncthreads();
        emax = max(sEmax[row], sEmax[row + kRows]);
        for (int g = half; g < kg; g += 2) {
            uint4 w[kDigits];
            if (8 * g < nb) {
                double v8[8];
#pragma unroll
                for (int h = 0; h < 8; ++h) {
                    const int k = 8 * g + h;
                    v8[h] = (live && k < nb) ? in[(long)sIdx[k] * V4 + p] : 0.0;
                }
                oz::digits8(v8, emax, w);
            } else {
#pragma unroll
                for (int a = 0; a < kDigits; ++a) w[a] = make_uint4(0u, 0u, 0u, 0u);
            }
#pragma unroll
            for (int a = 0; a < kDigits; ++a)
                *reinterpret_cast<uint4*>(sA + a * aPlane + tc::kmajor_off_g(row, 8 * g, kg)) = w[a];
        }
    }
    tc::fence_proxy_async();
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tmem = tmem_slot;
    if (tid == 0) {
        const uint32_t idesc = tc::idesc_bf16(kRows, Np);
        const uint32_t sbo = (uint32_t)kg * 128u;
        const uint32_t aB = tc::smem_u32(sA), bB = tc::smem_u32(sB);
        if (kg == 2)
            oz::issue_pairs<1>(tmem, Np, idesc, aB, aPlane, sbo, bB, bPlane, sbo, false);
        else if (kg == 4)
            oz::issue_pairs<2>(tmem, Np, idesc, aB, aPlane, sbo, bB, bPlane, sbo, false);
        else if (kg == 6)
            oz::issue_pairs<3>(tmem, Np, idesc, aB, aPlane, sbo, bB, bPlane, sbo, false);
        else if (kg == 8)
            oz::issue_pairs<4>(tmem, Np, idesc, aB, aPlane, sbo, bB, bPlane, sbo, false);
        else
            oz::issue_pairs<5>(tmem, Np, idesc, aB, aPlane, sbo, bB, bPlane, sbo, false);
        tc::commit(&mbar);
    }
    bool ok = tc::mbar_wait(&mbar, 0, kWaitCycles);
    ok = __syncthreads_and(ok) != 0;
    tc::fence_after();
    if (ok) {
        const int quarter = warp & 3, colh = warp >> 2;
        const uint32_t trow = tmem + ((uint32_t)(quarter * 32) << 16);
        // the epilogue's lane is point (quarter * 32 + lane) of the tile
        const int erow = quarter * 32 + lane;
        const long pe = (long)blockIdx.x * kRows + erow;
        const int ep = max(sEmax[erow], sEmax[erow + kRows]) - 1023;
        const bool elive = pe < V4 && max(sEmax[erow], sEmax[erow + kRows]) > 0;
        for (int q = 0; q < Np / 16; ++q) {
            const int c0 = 16 * q + 8 * colh;
            uint32_t r0[8], r1[8], r2[8], r3[8];
            __syncwarp();
            tc::ld8(trow + (uint32_t)(0 * Np + c0), r0);
            tc::ld8(trow + (uint32_t)(1 * Np + c0), r1);
            tc::ld8(trow + (uint32_t)(2 * Np + c0), r2);
            tc::ld8(trow + (uint32_t)(3 * Np + c0), r3);
            tc::wait_ld(r0);
            tc::wait_ld(r1);
            tc::wait_ld(r2);
            tc::wait_ld(r3);
            if (pe >= V4) continue;
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const int l = c0 + u;
                if (l >= nb) break;
                double val = 0.0;
                if (elive) {
                    dfl o = oz::combine4(__uint_as_float(r0[u]), __uint_as_float(r1[u]),
                                         __uint_as_float(r2[u]), __uint_as_float(r3[u]));
                    const float sc = oz::pow2f(ep + sXe[l] - 1023 - 12);
                    o.h = __fmul_rn(o.h, sc);
                    o.l = __fmul_rn(o.l, sc);
                    val = f2d_bits(o.h) + f2d_bits(o.l);
                }
                const long o = (long)sOut[l] * V4 + pe;
                out[o] = val;
                if (upd) upd[o] = val - upd[o];
            }
        }
    } else {
        if (tid == 0) atomicExch(status, 1);
        tc::mbar_wait(&mbar, 0, kWaitCycles);
    }
    tc::fence_before();
    __syncthreads();
    if (warp == 0) tc::dealloc(tmem, tcols);
}

// Pairing gaps, HFBGaps (src/HFB.f90:520-632), per block b (isospin b / 2):
//   G_ij = sum_p sum_c psi_ic(p) Z_jc(p)  over a 64-point chunk,
//   Z_j0 = -Fr psi_j0 + Fi psi_j1, Z_j1 = -Fi psi_j0 - Fr psi_j1 (same for 2, 3),
// the form of k_pair_gaps (pairing.cu).  K runs over (component, point):
// stage s covers 8 points, K group c = component c.  A rows are the spinors
// (one power of two per spinor and chunk), B rows their Z, formed in
// double-float and cut into digits through the fixed-point form with the
// exponent bound 2 max|F| max|psi_j| of the chunk.  One plane buffer per
// stage, two CTAs per SM.
constexpr int kGapPts = 64;

__global__ void __launch_bounds__(256, 2)
k_gaps_tc(const double* __restrict__ psi, const int* __restrict__ members,
          const int* __restrict__ hsz, int hmax, const double* __restrict__ fre,
          const double* __restrict__ fim, long V, int nchunk, double* __restrict__ gpart,
          int* __restrict__ status) {
    extern __shared__ uint8_t smraw[];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_slot;
    __shared__ int sE[kRows], sEz[kRows], sFe[kGapPts];
    __shared__ float4 sF[kGapPts];   // (Fr hi, Fr lo, Fi hi, Fi lo)
    const int b = blockIdx.y, it = b >> 1, chunk = blockIdx.x;
    const int h = hsz[b];
    if (h == 0) return;
    const int N = max(16, (h + 15) / 16 * 16);
    const uint32_t tcols = tmem_cols(N);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    // rows row0 and row0 + 64 (blocks above 64 spinors), component c
    const int row0 = tid >> 2, c = tid & 3;
    const int bPlane = N * tc::kRowBytes;

    const uint32_t s0a = tc::smem_u32(smraw);
    uint8_t* base = smraw + ((128u - (s0a & 127u)) & 127u);
    uint8_t* sA = base;                          // kDigits planes of 128 x 32
    uint8_t* sB = sA + kDigits * kStagePlane;    // kDigits planes of N x 32
    for (int t = tid; t < (kDigits * kStagePlane + kDigits * bPlane) / 16; t += 256)
        reinterpret_cast<uint4*>(base)[t] = make_uint4(0u, 0u, 0u, 0u);
    if (warp == 0) tc::alloc(&tmem_slot, tcols);
    if (tid == 0) tc::mbar_init(&mbar, 1);
    const long p0 = (long)chunk * kGapPts;
    const int npts = (int)min((long)kGapPts, V - p0);
    // the pairing field of the chunk, double-float, and its largest exponent
    if (tid < kGapPts) {
        double fr = 0.0, fi = 0.0;
        if (tid < npts) {
            fr = fre[(long)it * V + p0 + tid];
            fi = fim[(long)it * V + p0 + tid];
        }
        const dfl a = df_split(fr), d = df_split(fi);
        sF[tid] = make_float4(a.h, a.l, d.h, d.l);
        sFe[tid] = max(oz::bexp(fr), oz::bexp(fi));
    }
    const int pc = c ^ 1;   // the partner component of Z
    bool live[2];
    const double *src[2], *srp[2];
    int emax[2] = {0, 0}, ez[2];
#pragma unroll
    for (int r = 0; r < 2; ++r) {
        const int row = row0 + 64 * r;
        live[r] = row < h;
        src[r] = live[r] ? psi + ((long)members[b * hmax + row] * 4 + c) * V + p0 : psi;
        srp[r] = live[r] ? psi + ((long)members[b * hmax + row] * 4 + pc) * V + p0 : psi;
        if (live[r])
            for (int q = 0; q < npts; ++q) emax[r] = max(emax[r], oz::bexp(src[r][q]));
        emax[r] = max(emax[r], __shfl_xor_sync(0xffffffffu, emax[r], 1));
        emax[r] = max(emax[r], __shfl_xor_sync(0xffffffffu, emax[r], 2));
    }
    __syncthreads();
    int efmax = 0;
    for (int q = 0; q < kGapPts; ++q) efmax = max(efmax, sFe[q]);
#pragma unroll
    for (int r = 0; r < 2; ++r) {
        // |Z| <= |F| (|psi_c| + |psi_c'|) < 2^(E_F + E_psi + 3)
        ez[r] = (emax[r] == 0 || efmax == 0) ? 0 : emax[r] + efmax - 1023 + 2;
        if (live[r] && c == 0) {
            sE[row0 + 64 * r] = emax[r];
            sEz[row0 + 64 * r] = ez[r];
        }
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tmem = tmem_slot;
    const uint32_t idesc = tc::idesc_bf16(kRows, N);
    bool ok = true;
    const int nst = kGapPts / 8;
    for (int s = 0; s < nst; ++s) {
        if (s > 0) ok &= tc::mbar_wait(&mbar, (s - 1) & 1, kWaitCycles);
#pragma unroll
        for (int r = 0; r < 2; ++r) {
            if (!live[r]) continue;
            const int row = row0 + 64 * r;
            double a[8];
            long long zx[8];
#pragma unroll
            for (int hh = 0; hh < 8; ++hh) {
                const int q = 8 * s + hh;
                const bool in = q < npts;
                a[hh] = in ? src[r][q] : 0.0;
                const double ap = in ? srp[r][q] : 0.0;
                const float4 f = sF[q];
                const dfl fr = {f.x, f.y}, fi = {f.z, f.w};
                const dfl ac = df_split(a[hh]), ao = df_split(ap);
                // c even: Z = -Fr a_c + Fi a_c' ; c odd: Z = -Fi a_c' - Fr a_c
                const dfl t1 = df_mul(fr, ac), t2 = df_mul(fi, ao);
                const dfl z = (c & 1) ? df_neg(df_add(t1, t2)) : df_sub(t2, t1);
                zx[hh] = ez[r] ? oz::fixed_f(z.h, ez[r]) + oz::fixed_f(z.l, ez[r]) : 0ll;
            }
            uint4 w[kDigits];
            oz::digits8(a, emax[r], w);
#pragma unroll
            for (int d = 0; d < kDigits; ++d)
                *reinterpret_cast<uint4*>(sA + d * kStagePlane + tc::kmajor_off(row, 8 * c)) = w[d];
            oz::digits8_fixed(zx, w);
#pragma unroll
            for (int d = 0; d < kDigits; ++d)
                *reinterpret_cast<uint4*>(sB + d * bPlane + tc::kmajor_off(row, 8 * c)) = w[d];
        }
        tc::fence_proxy_async();
        tc::fence_before();
        __syncthreads();
        tc::fence_after();
        if (tid == 0) {
            oz::issue_pairs<2>(tmem, N, idesc, tc::smem_u32(sA), kStagePlane, tc::kSbo,
                               tc::smem_u32(sB), bPlane, tc::kSbo, s > 0);
            tc::commit(&mbar);
        }
    }
    ok &= tc::mbar_wait(&mbar, (nst - 1) & 1, kWaitCycles);
    ok = __syncthreads_and(ok) != 0;
    tc::fence_after();
    if (ok) {
        const int quarter = warp & 3, colh = warp >> 2;
        const int i = quarter * 32 + lane;
        const uint32_t trow = tmem + ((uint32_t)(quarter * 32) << 16);
        double* out = gpart + ((long)b * nchunk + chunk) * hmax * hmax;
        const int ei = i < h ? sE[i] - 1023 : 0;
        for (int q = 0; q < N / 16; ++q) {
            const int c0 = 16 * q + 8 * colh;
            uint32_t r0[8], r1[8], r2[8], r3[8];
            __syncwarp();
            tc::ld8(trow + (uint32_t)(0 * N + c0), r0);
            tc::ld8(trow + (uint32_t)(1 * N + c0), r1);
            tc::ld8(trow + (uint32_t)(2 * N + c0), r2);
            tc::ld8(trow + (uint32_t)(3 * N + c0), r3);
            tc::wait_ld(r0);
            tc::wait_ld(r1);
            tc::wait_ld(r2);
            tc::wait_ld(r3);
            if (i >= h) continue;
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const int j = c0 + u;
                if (j >= h) break;
                double val = 0.0;
                if (sE[i] != 0 && sEz[j] != 0) {
                    const dfl o = oz::combine4(__uint_as_float(r0[u]), __uint_as_float(r1[u]),
                                               __uint_as_float(r2[u]), __uint_as_float(r3[u]));
                    val = (f2d_bits(o.h) + f2d_bits(o.l)) * pow2d(ei + sEz[j] - 1023 - 12);
                }
                out[i * h + j] = val;
            }
        }
    } else {
        if (tid == 0) atomicExch(status, 1);
        tc::mbar_wait(&mbar, 0, kWaitCycles);
    }
    tc::fence_before();
    __syncthreads();
    if (warp == 0) tc::dealloc(tmem, tcols);
}

// Chunk partials of the gaps summed per entry, one warp each (fixed order):
// gsum[b][i * h + j].
__global__ void k_gaps_sum(const double* __restrict__ gpart, const int* __restrict__ hsz,
                           int hmax, int nchunk, double* __restrict__ gsum) {
    const int b = blockIdx.y;
    const int h = hsz[b];
    const int t = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
    const int lane = threadIdx.x & 31;
    if (t >= h * h) return;
    const double* pb = gpart + (long)b * nchunk * hmax * hmax;
    double s = 0.0;
    for (int q = lane; q < nchunk; q += 32) s += pb[(long)q * hmax * hmax + t];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    __syncwarp();
    if (lane == 0) gsum[(long)b * hmax * hmax + t] = s;
}

// Pairing field (HFBPairingField, src/HFB.f90:350-518) after the block apply
// Y_i = sum_j Ktilde[j][i] psi_j (tensor cores): per point and block,
//   Fr = sum_i sum_c Y_ic psi_ic,  Fi = sum_i (-Y_i0 psi_i1 + Y_i1 psi_i0
//                                               - Y_i2 psi_i3 + Y_i3 psi_i2)
// in double-float, as k_pair_field (pairing.cu) forms it; part[b][0|1][V].
// Four lanes per point (spinors i = sub, sub + 4, ...), combined by a fixed
// shuffle order.
__global__ void __launch_bounds__(256)
k_field_contract(const double* __restrict__ Y, const double* __restrict__ psi,
                 const int* __restrict__ members, const int* __restrict__ hsz, int hmax, long V,
                 double* __restrict__ part) {
    const int b = blockIdx.y, h = hsz[b];
    const long v = (long)blockIdx.x * (blockDim.x / 4) + threadIdx.x / 4;
    const int sub = threadIdx.x & 3;
    float rh = 0.f, rl = 0.f, ih = 0.f, il = 0.f;
    for (int i = sub; i < h && v < V; i += 4) {
        const double* y = Y + (long)(b * hmax + i) * 4 * V + v;
        const double* p = psi + (long)members[b * hmax + i] * 4 * V + v;
        dfl yy[4], pp[4];
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            yy[c] = df_split(y[c * V]);
            pp[c] = df_split(p[c * V]);
        }
#pragma unroll
        for (int c = 0; c < 4; ++c) df_acc(rh, rl, yy[c], pp[c]);
        df_acc(ih, il, yy[0], df_neg(pp[1]));
        df_acc(ih, il, yy[1], pp[0]);
        df_acc(ih, il, yy[2], df_neg(pp[3]));
        df_acc(ih, il, yy[3], pp[2]);
    }
    dfl re = df_norm(dfl{rh, rl}), im = df_norm(dfl{ih, il});
#pragma unroll
    for (int o = 1; o < 4; o <<= 1) {
        re = df_add(re, dfl{__shfl_xor_sync(0xffffffffu, re.h, o),
                            __shfl_xor_sync(0xffffffffu, re.l, o)});
        im = df_add(im, dfl{__shfl_xor_sync(0xffffffffu, im.h, o),
                            __shfl_xor_sync(0xffffffffu, im.l, o)});
    }
    if (sub == 0 && v < V) {
        part[((long)b * 2 + 0) * V + v] = df_to_fast(re);
        part[((long)b * 2 + 1) * V + v] = df_to_fast(im);
    }
}

}  // namespace

// Buffers and attributes of the tensor-core Gram-Schmidt (blocks of at most
// kMeshTcMax spinors).  Returns false when the blocks are larger.
bool gs_tc_prepare(mg_ctx* c) {
    if (!c->tc_mesh_ok || c->gs_nbmax > kMeshTcMax) return false;
    if (c->gs_xd == nullptr) {
        const int nblk = c->gs_nblk;
        c->gs_nchunk_tc = div_up(4 * c->V, kChunk);
        if (cudaMalloc(&c->gs_Stc, (size_t)nblk * c->gs_nchunk_tc * c->gs_nbmax * c->gs_nbmax *
                                       sizeof(double)) != cudaSuccess ||
            cudaMalloc(&c->gs_xd, (size_t)nblk * kDigits * kXdStride * sizeof(uint16_t)) !=
                cudaSuccess ||
            cudaMalloc(&c->gs_xe, (size_t)nblk * kMeshTcMax * sizeof(int)) != cudaSuccess ||
            cudaMemset(c->gs_xd, 0, (size_t)nblk * kDigits * kXdStride * sizeof(uint16_t)) !=
                cudaSuccess)
            return false;
        cudaFuncSetAttribute(k_gs_overlap_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             200 * 1024);
        cudaFuncSetAttribute(k_apply_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             200 * 1024);
    }
    return true;
}

int gs_overlap_tc(mg_ctx* c, const double* psi, const int* d_lists, const int* d_ordered) {
    size_t sm = 128 + 2 * (size_t)kDigits * kStagePlane;
    const int N = std::max(16, (c->gs_nbmax + 15) / 16 * 16);
    if (tmem_cols(N) > 256) sm = std::max(sm, kOneCtaSmem);
    k_gs_overlap_tc<<<dim3(c->gs_nchunk_tc, c->gs_nblk), 256, sm, c->stream>>>(
        psi, d_lists, d_ordered, c->gs_nbmax, 4 * c->V, c->gs_nchunk_tc, c->gs_Stc,
        c->tc_status);
    MG_LAUNCHED(c);
    return MG_OK;
}

static int apply_tc(mg_ctx* c, int nblk, int nbmax, const double* coef, long bstride, int ld,
                    BlockIdx bi, const double* in, double* out, double* upd, const int* in_list,
                    const int* out_list, const int* out_base, uint16_t* xd, int* xe) {
    k_coef_digits<<<nblk, 96, 0, c->stream>>>(coef, bstride, ld, bi, xd, xe);
    MG_LAUNCHED(c);
    const int Np = std::max(16, (nbmax + 15) / 16 * 16);
    size_t sm = 128 + (size_t)kDigits * (kRows * Np * 2 + Np * Np * 2);
    // at most two CTAs per SM (2 x 256 TMEM columns), one above N = 64
    sm = std::max(sm, tmem_cols(Np) > 256 ? kOneCtaSmem : (size_t)80 * 1024);
    const long V4 = 4 * c->V;
    k_apply_tc<<<dim3(div_up(V4, kRows), nblk), 256, sm, c->stream>>>(
        in, out, upd, bi, in_list, out_list, out_base, xd, xe, V4, c->tc_status);
    MG_LAUNCHED(c);
    return MG_OK;
}

int gs_apply_tc(mg_ctx* c, double* psi, double* upd, const int* d_lists, const int* d_ordered) {
    const BlockIdx bi{d_lists, nullptr, 0};
    return apply_tc(c, c->gs_nblk, c->gs_nbmax, c->gs_R, (long)c->gs_nbmax * c->gs_nbmax,
                    c->gs_nbmax, bi, psi, psi, upd, d_ordered, d_ordered, nullptr, c->gs_xd,
                    c->gs_xe);
}

// Canonical basis of the four pairing blocks (hsz[b] <= kMeshTcMax):
// CanTransfo is stored densely per block (ld = h) at b * hmax^2.
int can_transform_tc(mg_ctx* c) {
    Hfb& H = c->hfb;
    if (!c->tc_mesh_ok || H.hmax > kMeshTcMax) return MG_ERR_STATE;
    if (c->can_xd == nullptr) {
        MG_CUDA(cudaMalloc(&c->can_xd, (size_t)4 * kDigits * kXdStride * sizeof(uint16_t)));
        MG_CUDA(cudaMemset(c->can_xd, 0, (size_t)4 * kDigits * kXdStride * sizeof(uint16_t)));
        MG_CUDA(cudaMalloc(&c->can_xe, (size_t)4 * kMeshTcMax * sizeof(int)));
        MG_CUDA(cudaFuncSetAttribute(k_apply_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     200 * 1024));
    }
    const BlockIdx bi{nullptr, H.hsz, H.hmax};
    return apply_tc(c, 4, H.hmax, H.cantr, (long)H.hmax * H.hmax, 0, bi,
                    c->bas[MG_HF_BASIS].psi, c->bas[MG_CAN_BASIS].psi, nullptr, H.members,
                    nullptr, H.cstart, c->can_xd, c->can_xe);
}

// Gaps partial sums of the four pairing blocks on the tensor cores into
// gsum[b][i * h + j] (to be finished by k_gaps_finish with one chunk).
int gaps_tc(mg_ctx* c, double* gsum) {
    Hfb& H = c->hfb;
    if (!c->tc_mesh_ok || H.hmax > kMeshTcMax) return MG_ERR_STATE;
    const long V = c->V;
    const int nchunk = div_up(V, kGapPts);
    if (c->gap_part == nullptr) {
        MG_CUDA(cudaMalloc(&c->gap_part, (size_t)4 * nchunk * H.hmax * H.hmax * sizeof(double)));
        MG_CUDA(cudaFuncSetAttribute(k_gaps_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     200 * 1024));
    }
    const int Np = std::max(16, (H.hmax + 15) / 16 * 16);
    size_t sm = 128 + (size_t)kDigits * kStagePlane + (size_t)kDigits * Np * tc::kRowBytes;
    // two CTAs per SM (2 x 256 TMEM columns), one above N = 64
    sm = std::max(sm, tmem_cols(Np) > 256 ? kOneCtaSmem : (size_t)80 * 1024);
    k_gaps_tc<<<dim3(nchunk, 4), 256, sm, c->stream>>>(c->bas[MG_HF_BASIS].psi, H.members, H.hsz,
                                                      H.hmax, H.fre, H.fim, V, nchunk, c->gap_part,
                                                      c->tc_status);
    MG_LAUNCHED(c);
    k_gaps_sum<<<dim3(div_up((long)H.hmax * H.hmax, 8), 4), 256, 0, c->stream>>>(
        c->gap_part, H.hsz, H.hmax, nchunk, gsum);
    MG_LAUNCHED(c);
    return MG_OK;
}

// Pairing-field partials of the four blocks: Y = block apply of Ktilde
// (tensor cores) into the scratch basis, then the pointwise contraction.
int pair_field_tc(mg_ctx* c) {
    Hfb& H = c->hfb;
    if (!c->tc_mesh_ok || H.hmax > kMeshTcMax) return MG_ERR_STATE;
    const long V = c->V;
    if (c->field_y == nullptr) {
        MG_CUDA(cudaMalloc(&c->field_y, (size_t)4 * H.hmax * 4 * V * sizeof(double)));
        MG_CUDA(cudaMalloc(&c->field_xd, (size_t)4 * kDigits * kXdStride * sizeof(uint16_t)));
        MG_CUDA(cudaMemset(c->field_xd, 0, (size_t)4 * kDigits * kXdStride * sizeof(uint16_t)));
        MG_CUDA(cudaMalloc(&c->field_xe, (size_t)4 * kMeshTcMax * sizeof(int)));
        MG_CUDA(cudaMalloc(&c->field_ybase, 4 * sizeof(int)));
        const int yb[4] = {0, H.hmax, 2 * H.hmax, 3 * H.hmax};
        MG_CUDA(cudaMemcpy(c->field_ybase, yb, sizeof(yb), cudaMemcpyHostToDevice));
        MG_CUDA(cudaFuncSetAttribute(k_apply_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     200 * 1024));
    }
    const BlockIdx bi{nullptr, H.hsz, H.hmax};
    MG_TRY(apply_tc(c, 4, H.hmax, H.ktil, (long)H.hmax * H.hmax, 0, bi,
                    c->bas[MG_HF_BASIS].psi, c->field_y, nullptr, H.members, nullptr,
                    c->field_ybase, c->field_xd, c->field_xe));
    k_field_contract<<<dim3(div_up(V, 64), 4), 256, 0, c->stream>>>(
        c->field_y, c->bas[MG_HF_BASIS].psi, H.members, H.hsz, H.hmax, V, H.fpart);
    MG_LAUNCHED(c);
    return MG_OK;
}

}  // namespace mg
