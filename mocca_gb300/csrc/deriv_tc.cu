// deriv_tc.cu -- the mixed form of DeriveAll on the tcgen05 tensor cores.
//
// Same operation as the double-float kernels of deriv.cu (Opt_LAG{X,Y,Z}_EV8
// and Lapla_LAG_EV8, src/OptimizedDerivatives.f90:115-148, :306-338,
// :432-464, :551-615): per line of a real grid, out(i) = sum_q M(i,q) in(q)
// for the first- and second-derivative matrices of the axis, as exact BF16
// digit products (ozaki.cuh).  A line is one MMA row; the Lagrange block of
// the axis is N = 2n rows rounded up to 16 (first-derivative rows, then
// second-derivative rows); K = n padded to 32.  The result carries the
// rounding of the inputs to 47 bits (about 2e-12 of the line's largest
// |M|*|psi| sum) and is stored as {hi, lo} float pairs, the format the
// double-float consumers read.
//
// One persistent CTA per SM walks the pass's 128-line tiles (static
// round-robin) with warp-specialised roles:
//   warps 0-3  slicers: thread r owns line r of a tile; it prefetches the
//              next tile's line with cp.async into a staging row while it
//              turns the current one into digit planes (two plane buffers);
//   warp 4     MMA issue (one thread): 21 digit pairs x 2 K steps into one of
//              two TMEM accumulator sets (4 accumulators of N columns each);
//   warps 5-20 epilogue: four warps per TMEM lane quarter (a 4-column
//              quarter of every 16 columns), combine the accumulators to
//              double-float, scale, store; the Laplacian values they add to
//              are loaded before the MMA wait.
// Hand-offs are mbarriers: fullA (128 slicer arrivals), emptyA and fullT
// (tcgen05.commit), emptyT (256 epilogue arrivals); every wait is bounded
// and a timeout sets the context's status word.  The slicers wait only for
// the MMAs to release their plane buffer; the line exponents the epilogue
// reads sit in a four-tile ring.
// Three launches, one per axis: x writes d/dx and Lxx, y writes d/dy and
// adds Lyy, z writes d/dz and adds Lzz, so the Laplacian is summed
// (X + Y) + Z as in Lapla_LAG_EV8.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "df.cuh"
#include "mg_internal.cuh"
#include "ozaki.cuh"
#include "tc.cuh"

namespace mg {

namespace {

using oz::kDigits;
constexpr int kTile = 128;                      // lines per tile (MMA M)
// Two forms: KP = 32 (lines up to 32) with two plane buffers, two staging
// buffers and two TMEM accumulator sets; KP = 48 (lines of 33 to kLongMax)
// with one of each (N up to 80: four accumulators take 320 TMEM columns and
// the planes of both parity slots ~92 KB of shared memory).  With one buffer
// the slicers still work on tile k + 1 while the epilogue reads tile k; the
// MMAs of tile k + 1 wait for that epilogue, and the next tile's lines are
// fetched once the current ones are sliced.
constexpr int kShortK = 32;
constexpr int kLongK = 48;
constexpr int kLongMax = 40;
constexpr int kSlicers = 128;                   // warps 0-3
constexpr int kMmaWarp = 4;
constexpr int kEpi = 512;                       // warps 5-20
constexpr int kThreads = kSlicers + 32 + kEpi;  // 672
constexpr uint32_t kTmemCols = 512;             // 2 sets x 4 x N (N <= 64) or 1 set x 4 x N (N <= 80)
constexpr long long kWaitCycles = 4000000000LL; // ~2 s at the top SM clock

struct TcPass {
    const GridJob* jobs;
    const uint16_t* bmat[2];   // per slot: kDigits planes, N rows x KP, K-major core matrices
    const int* erow[2];        // per slot: N row exponents
    int axis, n, N, nlines, tpj, ntiles, nx, ny;
    int lap_stage;             // y/z passes: Laplacian values staged in shared memory
    int* status;
};

struct TcShared {
    uint64_t fullA[2], emptyA[2], fullT[2], emptyT[2];
    uint64_t emaxReady[4];   // tile k's line exponents written (128 slicer arrivals)
    uint64_t staged;         // x pass: every slicer's copies of the tile landed (128 arrivals)
    uint32_t tmem;
    // line exponents of the last four tiles: the slicers write tile k's while
    // the epilogue may still read tile k-2's (slicer k waits for MMA k-2,
    // which waited for epilogue k-4)
    int emax[4][kTile];
    float srow[2][96];
};

// global offset of element k of line l of a grid (axis order: x, y, z)
__device__ __forceinline__ void line_geom(const TcPass& P, int l, long& off, long& stride) {
    if (P.axis == 0) {
        off = (long)l * P.n;
        stride = 1;
    } else if (P.axis == 1) {
        off = (long)(l / P.nx) * P.nx * P.ny + l % P.nx;
        stride = P.nx;
    } else {
        off = l;
        stride = (long)P.nx * P.ny;
    }
}

__device__ __forceinline__ int slot_of(const GridJob& J, int axis) {
    return axis == 0 ? J.slot[0] : (axis == 1 ? J.slot[1] : J.slot[2]);
}

__device__ __forceinline__ double* out_of(const GridJob& J, int axis) {
    return axis == 0 ? J.dx : (axis == 1 ? J.dy : J.dz);
}

template <int KP, int NBUF>
__global__ void __launch_bounds__(kThreads, 1)
k_deriv_tc(TcPass P) {
    constexpr int kPlane = kTile * KP * 2;     // bytes of one digit plane of a tile
    constexpr int kKg = KP / 8;                // K groups of 8
    constexpr uint32_t kSboK = 128u * kKg;     // stride byte offset of the planes
    extern __shared__ uint8_t smraw[];
    __shared__ TcShared S;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int n = P.n, N = P.N;

    const uint32_t s0 = tc::smem_u32(smraw);
    uint8_t* base = smraw + ((128u - (s0 & 127u)) & 127u);
    uint8_t* sA = base;                                         // NBUF x kDigits planes
    uint8_t* sB = sA + NBUF * kDigits * kPlane;                 // 2 slots x kDigits x N x KP
    const int bBytes = kDigits * N * KP * 2;
    double* sIn = reinterpret_cast<double*>(sB + 2 * bBytes);   // NBUF x 128 x (n + 1)
    float2* sLap = reinterpret_cast<float2*>(sIn + NBUF * kTile * (n + 1));   // 128 x (n + 1)

    if (warp == 0) tc::alloc(&S.tmem, kTmemCols);
    if (tid == 0) {
        for (int b = 0; b < 2; ++b) {
            tc::mbar_init(&S.fullA[b], kSlicers);
            tc::mbar_init(&S.emptyA[b], 1);
            tc::mbar_init(&S.fullT[b], 1);
            tc::mbar_init(&S.emptyT[b], kEpi);
        }
        for (int b = 0; b < 4; ++b) tc::mbar_init(&S.emaxReady[b], kSlicers);
        tc::mbar_init(&S.staged, kSlicers);
    }
    for (int s = 0; s < 2; ++s) {
        const uint4* src = reinterpret_cast<const uint4*>(P.bmat[s]);
        uint4* dst = reinterpret_cast<uint4*>(sB + s * bBytes);
        for (int t = tid; t < bBytes / 16; t += kThreads) dst[t] = src[t];
        if (tid < N) S.srow[s][tid] = oz::pow2f(P.erow[s][tid]);
    }
    tc::fence_proxy_async();
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tmem = S.tmem;
    bool ok = true;

    if (warp < 4) {
        // ---------------- slicers ----------------
        const int r = tid;
        // x pass: a tile's lines are one contiguous block, staged by all
        // slicers with consecutive elements on consecutive lanes (element e
        // is point e mod n of line e / n; (e * ceil(2^18 / n)) >> 18 = e / n
        // exactly for n <= 32, e < 128 n); y and z passes: one line per
        // thread, consecutive lines on consecutive lanes
        const uint32_t magic = ((1u << 18) + (uint32_t)n - 1u) / (uint32_t)n;
        auto prefetch = [&](int T, int sbuf) {
            const int job = T / P.tpj, l0 = (T % P.tpj) * kTile;
            const double* in = P.jobs[job].in;
            // (with one staging buffer the next tile's lines are fetched while
            // other slicers may still read the current ones: own line only)
            if (NBUF == 2 && P.axis == 0) {
                const int tot = min(kTile, P.nlines - l0) * n;
                const double* blk = in + (long)l0 * n;
                double* dst = sIn + (long)sbuf * kTile * (n + 1);
                for (int e = r; e < tot; e += kSlicers) {
                    const int line = (int)(((uint32_t)e * magic) >> 18);
                    tc::cp_async8(dst + line * (n + 1) + (e - line * n), blk + e);
                }
                return;
            }
            const int l = l0 + r;
            if (l >= P.nlines) return;
            long off, stride;
            line_geom(P, l, off, stride);
            double* dst = sIn + ((long)sbuf * kTile + r) * (n + 1);
            for (int k = 0; k < n; ++k) tc::cp_async8(dst + k, in + off + k * stride);
        };
        int T = blockIdx.x;
        if (T < P.ntiles) prefetch(T, 0);
        tc::cp_async_commit();
        for (int k = 0; T < P.ntiles; T += gridDim.x, ++k) {
            const int buf = k % NBUF;
            tc::cp_async_wait_all();
            if (NBUF == 2 && P.axis == 0) {
                // the tile's lines come from every slicer's copies; passing this
                // also means every slicer has finished the tile before, whose
                // staging buffer the prefetch below reuses
                tc::mbar_arrive(&S.staged);
                ok &= tc::mbar_wait(&S.staged, k & 1, kWaitCycles);
                if (!ok) break;
            }
            const int Tn = T + gridDim.x;
            const bool live = (T % P.tpj) * kTile + r < P.nlines;
            const double* src = sIn + ((long)buf * kTile + r) * (n + 1);
            int emax = 0;
            if (live)
                for (int q = 0; q < n; ++q) emax = max(emax, oz::bexp(src[q]));
            // the staging row of the other buffer was read in the iteration before
            if (NBUF == 2 && Tn < P.ntiles) prefetch(Tn, buf ^ 1);
            tc::cp_async_commit();
            if (k >= NBUF) {
                ok &= tc::mbar_wait(&S.emptyA[buf], ((k - NBUF) / NBUF) & 1, kWaitCycles);
                if (!ok) break;
            }
            S.emax[k & 3][r] = emax;
            tc::mbar_arrive(&S.emaxReady[k & 3]);
            uint8_t* planes = sA + buf * kDigits * kPlane;
#pragma unroll 1
            for (int g = 0; g < kKg; ++g) {
                uint4 w[kDigits];
                if (8 * g < n) {
                    double v8[8];
#pragma unroll
                    for (int h = 0; h < 8; ++h)
                        v8[h] = (live && 8 * g + h < n) ? src[8 * g + h] : 0.0;
                    oz::digits8(v8, emax, w);
                } else {
#pragma unroll
                    for (int a = 0; a < kDigits; ++a) w[a] = make_uint4(0u, 0u, 0u, 0u);
                }
#pragma unroll
                for (int a = 0; a < kDigits; ++a)
                    *reinterpret_cast<uint4*>(planes + a * kPlane + tc::kmajor_off_g(r, 8 * g, kKg)) =
                        w[a];
            }
            tc::fence_proxy_async();
            tc::mbar_arrive(&S.fullA[buf]);
            // one staging buffer: this thread's line of the next tile, once its
            // line of this tile has been sliced
            if (NBUF == 1 && Tn < P.ntiles) {
                prefetch(Tn, 0);
                tc::cp_async_commit();
            }
        }
        tc::cp_async_wait_all();
    } else if (warp == kMmaWarp) {
        // ---------------- MMA issue ----------------
        int k = 0, T = blockIdx.x;
        if (lane == 0) {
            const uint32_t idesc = tc::idesc_bf16(kTile, N);
            for (; T < P.ntiles; T += gridDim.x, ++k) {
                const int buf = k % NBUF;
                const int slot = slot_of(P.jobs[T / P.tpj], P.axis);
                ok &= tc::mbar_wait(&S.fullA[buf], (k / NBUF) & 1, kWaitCycles);
                if (k >= NBUF)
                    ok &= tc::mbar_wait(&S.emptyT[buf], ((k - NBUF) / NBUF) & 1, kWaitCycles);
                if (!ok) break;
                tc::fence_after();
                oz::issue_pairs<KP / 16>(tmem + (uint32_t)(buf * 4 * N), N, idesc,
                                         tc::smem_u32(sA + buf * kDigits * kPlane), kPlane, kSboK,
                                         tc::smem_u32(sB + slot * bBytes), N * KP * 2, kSboK,
                                         false);
                tc::commit(&S.emptyA[buf]);
                tc::commit(&S.fullT[buf]);
            }
            // the last commit covers every MMA of this CTA
            if (k > 0)
                ok &= tc::mbar_wait(&S.fullT[(k - 1) % NBUF], ((k - 1) / NBUF) & 1, kWaitCycles);
        }
        __syncwarp();
    } else {
        // ---------------- epilogue ----------------
        const int e = tid - (kSlicers + 32);
        const int quarter = warp & 3, colg = e >> 7;
        const int erow = quarter * 32 + lane;   // TMEM lane = tile row
        const uint32_t tq = (uint32_t)(quarter * 32) << 16;
        const int nq = N / 16;
        for (int k = 0, T = blockIdx.x; T < P.ntiles; T += gridDim.x, ++k) {
            const int buf = k % NBUF;
            const GridJob& J = P.jobs[T / P.tpj];
            float2* gD = reinterpret_cast<float2*>(out_of(J, P.axis));
            float2* gL = reinterpret_cast<float2*>(J.lap);
            const int l = (T % P.tpj) * kTile + erow;
            const bool live = l < P.nlines;
            long off = 0, stride = 0;
            if (live) line_geom(P, l, off, stride);
            // Laplacian values this thread adds to (y and z passes): staged in
            // its own slots of sLap while the MMAs run
            const bool stage = P.axis != 0 && gL != nullptr && live && P.lap_stage;
            if (stage) {
                for (int q = 0; q < nq; ++q)
                    for (int u = 0; u < 4; ++u) {
                        const int j = 16 * q + 4 * colg + u;
                        if (j >= n && j < 2 * n)
                            tc::cp_async8(sLap + erow * (n + 1) + (j - n),
                                          gL + off + (long)(j - n) * stride);
                    }
            }
            tc::cp_async_commit();
            // ring of four: slicer k + 4 waits for MMA k + 4 - NBUF, which waited
            // for epilogue k + 4 - 2 NBUF >= k, so it cannot arrive before this
            // epilogue is done
            ok &= tc::mbar_wait(&S.emaxReady[k & 3], (k >> 2) & 1, kWaitCycles);
            ok &= tc::mbar_wait(&S.fullT[buf], (k / NBUF) & 1, kWaitCycles);
            if (!ok) break;
            tc::fence_after();
            const int emax = S.emax[k & 3][erow];
            const float sline = emax == 0 ? 0.0f : oz::pow2f(emax - 1023 - 12);
            const float* srow = S.srow[slot_of(J, P.axis)];
            const uint32_t tb = tmem + tq + (uint32_t)(buf * 4 * N);
            bool landed = !stage;
#pragma unroll 1
            for (int q = 0; q < nq; ++q) {
                const int c0 = 16 * q + 4 * colg;
                // the staged Laplacian values are needed from the first
                // chunk that holds second-derivative columns
                if (!landed && c0 + 4 > n) {
                    tc::cp_async_wait_all();
                    landed = true;
                }
                uint32_t r0[4], r1[4], r2[4], r3[4];
                __syncwarp();
                tc::ld4(tb + (uint32_t)(0 * N + c0), r0);
                tc::ld4(tb + (uint32_t)(1 * N + c0), r1);
                tc::ld4(tb + (uint32_t)(2 * N + c0), r2);
                tc::ld4(tb + (uint32_t)(3 * N + c0), r3);
                tc::wait_ld(r0);
                tc::wait_ld(r1);
                tc::wait_ld(r2);
                tc::wait_ld(r3);
                if (!live) continue;
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int j = c0 + u;
                    if (j >= 2 * n) break;
                    dfl o = oz::combine4(__uint_as_float(r0[u]), __uint_as_float(r1[u]),
                                         __uint_as_float(r2[u]), __uint_as_float(r3[u]));
                    const float sc = __fmul_rn(sline, srow[j]);
                    o.h = __fmul_rn(o.h, sc);
                    o.l = __fmul_rn(o.l, sc);
                    if (j < n) {
                        if (gD) df_st(gD + off + (long)j * stride, o);
                    } else if (gL) {
                        const long pp = off + (long)(j - n) * stride;
                        if (P.axis == 0) {
                            df_st(gL + pp, o);
                        } else {
                            const float2 a = stage ? sLap[erow * (n + 1) + (j - n)] : gL[pp];
                            df_st(gL + pp, df_add(dfl{a.x, a.y}, o));
                        }
                    }
                }
            }
            tc::fence_before();
            tc::mbar_arrive(&S.emptyT[buf]);
        }
        tc::cp_async_wait_all();
    }
    if (!ok) atomicExch(P.status, 1);
    tc::fence_before();
    __syncthreads();
    if (warp == 0) tc::dealloc(tmem, kTmemCols);
}

}  // namespace

constexpr size_t kSmemCap = 224 * 1024;   // plus ~2.7 KB of static TcShared

size_t tc_smem_bytes(int n, int N, bool lap_stage, int kp, int nbuf) {
    size_t b = 128 + (size_t)nbuf * kDigits * kTile * kp * 2 + 2 * (size_t)kDigits * N * kp * 2 +
               (size_t)nbuf * kTile * (n + 1) * sizeof(double);
    if (lap_stage) b += (size_t)kTile * (n + 1) * sizeof(float2);
    return b;
}

// Digit planes of the Lagrange blocks, built once per context.  The tensor
// path serves line lengths up to 32 (K padded to 32, two buffers) and up to
// kLongMax (K padded to 48, one buffer); N = 2n rounded to 16.  Row exponents
// sit at a stride of 96 per (axis, slot).
int tc_setup(mg_ctx* c) {
    const int ns[3] = {c->nx, c->ny, c->nz};
    c->tc_ok = false;
    // the mesh-sized GEMMs of meshgemm_tc.cu need no Lagrange planes: they
    // run on any mesh
    if (!c->tc_status) {
        MG_CUDA(cudaMalloc(&c->tc_status, sizeof(int)));
        MG_CUDA(cudaMemset(c->tc_status, 0, sizeof(int)));
        MG_CUDA(cudaMallocHost(&c->h_tc_status, sizeof(int)));
        *c->h_tc_status = 0;
    }
    c->tc_mesh_ok = true;
    const int nmax = std::max(ns[0], std::max(ns[1], ns[2]));
    if (nmax > kLongMax) return MG_OK;
    const int kp = nmax <= kShortK ? kShortK : kLongK;
    c->tc_kp = kp;
    long total = 0;
    for (int a = 0; a < 3; ++a) {
        c->tc_N[a] = (2 * ns[a] + 15) / 16 * 16;
        for (int s = 0; s < 2; ++s) {
            c->tc_off[a][s] = total;
            total += (long)kDigits * c->tc_N[a] * kp;
        }
    }
    std::vector<uint16_t> h(total, 0);
    std::vector<int> he(3 * 2 * 96, 0);
    for (int a = 0; a < 3; ++a) {
        const int n = ns[a], N = c->tc_N[a];
        const long nn = (long)n * n;
        std::vector<double> d1(2 * nn), d2(2 * nn);
        MG_TRY(mg_lagrange_matrices(n, c->p.dx, c->folded ? 1 : 0, d1.data(), d2.data()));
        for (int s = 0; s < 2; ++s) {
            for (int j = 0; j < 2 * n; ++j) {
                const double* row = (j < n ? d1.data() + s * nn + (long)j * n
                                           : d2.data() + s * nn + (long)(j - n) * n);
                double mx = 0.0;
                for (int k = 0; k < n; ++k) mx = std::max(mx, std::fabs(row[k]));
                const int E = oz::host_row_exponent(mx);
                he[(a * 2 + s) * 96 + j] = E;
                const int g = 8 * kDigits - 2 - E;
                for (int k = 0; k < n; ++k) {
                    uint16_t dg[kDigits];
                    oz::host_digits(row[k], g, dg);
                    for (int b = 0; b < kDigits; ++b)
                        h[c->tc_off[a][s] + (long)b * N * kp + tc::kmajor_off_g(j, k, kp / 8) / 2] =
                            dg[b];
                }
            }
        }
    }
    MG_CUDA(cudaMalloc(&c->tcmats, total * sizeof(uint16_t)));
    MG_CUDA(cudaMemcpy(c->tcmats, h.data(), total * sizeof(uint16_t), cudaMemcpyHostToDevice));
    MG_CUDA(cudaMalloc(&c->tc_erow, he.size() * sizeof(int)));
    MG_CUDA(cudaMemcpy(c->tc_erow, he.data(), he.size() * sizeof(int), cudaMemcpyHostToDevice));
    MG_CUDA(cudaFuncSetAttribute(k_deriv_tc<kShortK, 2>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemCap));
    MG_CUDA(cudaFuncSetAttribute(k_deriv_tc<kLongK, 1>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemCap));
    c->tc_ok = true;
    return MG_OK;
}

// DeriveAll of the jobs on the tensor cores (mixed form, double-float output).
int run_jobs_tc(mg_ctx* c, const GridJob* jobs, int njobs) {
    if (njobs <= 0) return MG_OK;
    const int ns[3] = {c->nx, c->ny, c->nz};
    for (int axis = 0; axis < 3; ++axis) {
        TcPass P{};
        P.jobs = jobs;
        for (int s = 0; s < 2; ++s) {
            P.bmat[s] = c->tcmats + c->tc_off[axis][s];
            P.erow[s] = c->tc_erow + (axis * 2 + s) * 96;
        }
        P.axis = axis;
        P.n = ns[axis];
        P.N = c->tc_N[axis];
        P.nlines = (int)(c->V / ns[axis]);
        P.tpj = div_up(P.nlines, kTile);
        P.ntiles = P.tpj * njobs;
        P.nx = c->nx;
        P.ny = c->ny;
        P.status = c->tc_status;
        const int kp = c->tc_kp, nbuf = kp == kShortK ? 2 : 1;
        P.lap_stage = tc_smem_bytes(P.n, P.N, true, kp, nbuf) <= kSmemCap ? 1 : 0;
        const size_t sm = tc_smem_bytes(P.n, P.N, P.lap_stage != 0, kp, nbuf);
        if (sm > kSmemCap) return MG_ERR_ARG;
        const int sms = c->tc_grid_cap > 0 ? std::min(c->tc_grid_cap, c->num_sms) : c->num_sms;
        const int grid = std::min(sms, P.ntiles);
        if (kp == kShortK)
            k_deriv_tc<kShortK, 2><<<grid, kThreads, sm, c->stream>>>(P);
        else
            k_deriv_tc<kLongK, 1><<<grid, kThreads, sm, c->stream>>>(P);
        MG_LAUNCHED(c);
    }
    return MG_OK;
}

// Status of the tensor-core waits since the last call (MG_ERR_TIMEOUT when an
// MMA completion wait ran out of its cap, in the derivatives or the mesh
// GEMMs); synchronises the stream.
int tc_status_async(mg_ctx* c) {
    if (!c->tc_ok && !c->tc_mesh_ok) return MG_OK;
    MG_CUDA(cudaMemcpyAsync(c->h_tc_status, c->tc_status, sizeof(int), cudaMemcpyDeviceToHost,
                            c->stream));
    return MG_OK;
}

int tc_status_result(mg_ctx* c) {
    if (!c->tc_ok && !c->tc_mesh_ok) return MG_OK;
    return *c->h_tc_status ? MG_ERR_TIMEOUT : MG_OK;
}

int tc_check(mg_ctx* c) {
    if (!c->tc_ok && !c->tc_mesh_ok) return MG_OK;
    int h = 0;
    MG_CUDA(cudaMemcpyAsync(&h, c->tc_status, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    MG_CUDA(cudaStreamSynchronize(c->stream));
    return h ? MG_ERR_TIMEOUT : MG_OK;
}

}  // namespace mg
