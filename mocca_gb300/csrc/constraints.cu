// constraints.cu -- multipole-moment constraints of the alternating kind, FP64.
//
// The kind the &MomentConstraint namelist defaults to (ConstraintType 2,
// Isoswitch 1, Total false) with the density-dependent cutoff (CutoffType 0)
// and Damping 0:
//   RutzCutOff            src/Moments.f90:2703-2871  -> k_cut_stats, k_cut_surface, k_cut_apply
//   Calculate_Multipole   src/Moments.f90:1907-1966  -> k_cons_moments (value and square)
//   CalcConstraintEnergy  src/Moments.f90:2368-2486  -> k_cons_field
//   AlternateStep         src/ImaginaryTime.f90:306-437 -> k_alt_apply + Gram-Schmidt
//   Readjust / ReadjustAllMoments / TurnOffConstraints
//                         src/Moments.f90:2336-2366, :2994-3058, :3516-3550 (host)
//
// The cutoff needs, for each mesh point, the distance to the nearest point of
// the equidensity surface rho = max(rho)/10 (linearly interpolated between
// neighbours of the stored box).  One kernel lists the surface points (an
// atomic counter per isospin: the list order varies, the minimum does not),
// the next gives every mesh point its minimum over the list, staged through
// shared memory in tiles.  The pointwise products keep the reference's
// operation order with explicitly rounded FP64 operations, so they are not
// contracted into FMAs.
#include <cmath>

#include "mg_internal.cuh"

namespace mg {

namespace {

constexpr int kThreads = 256;
constexpr double kRadd = 4.0, kAcut = 0.4;   // src/Moments.f90:258
// d0 = 0.1 is a default-kind (single precision) literal assigned to a
// real(dp) variable (src/Moments.f90:258): its value is 0.1f widened.
constexpr double kD0 = (double)0.1f;

struct ConsCoef {
    double a[kMaxConstraints];   // per constraint: the coefficient of Q_lm * Cutoff
    int n;
};

// Per isospin (blockIdx.x): max(rho) / 10 and dv * sum(rho); resets the
// surface counter.
__global__ void __launch_bounds__(1024)
k_cut_stats(const double* __restrict__ rho, long V, double dv, double* __restrict__ stat,
            int* __restrict__ count) {
    const int it = blockIdx.x;
    const double* r = rho + it * V;
    double mx = -INFINITY, s = 0.0;
    for (long v = threadIdx.x; v < V; v += blockDim.x) {
        mx = fmax(mx, r[v]);
        s += r[v];
    }
    __shared__ double smx[32], ssum[32];
    for (int o = 16; o > 0; o >>= 1) {
        mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        s += __shfl_xor_sync(0xffffffffu, s, o);
    }
    if (threadIdx.x % 32 == 0) { smx[threadIdx.x / 32] = mx; ssum[threadIdx.x / 32] = s; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double m = smx[0], t = ssum[0];
        for (int w = 1; w < (int)(blockDim.x / 32); ++w) { m = fmax(m, smx[w]); t += ssum[w]; }
        stat[2 * it] = m / 10.0;
        stat[2 * it + 1] = dv * t;
        count[it] = 0;
    }
}

__device__ __forceinline__ bool crosses(double a, double b, double tr) {
    return (a >= tr && b <= tr) || (a <= tr && b >= tr);
}

// Surface points between each stored point and its +x, +y, +z neighbours.
__global__ void __launch_bounds__(kThreads)
k_cut_surface(const double* __restrict__ rho, int nx, int ny, int nz, double dx,
              const double* __restrict__ stat, int* __restrict__ count,
              double* __restrict__ surf, long cap) {
    const int it = blockIdx.y;
    const long nin = (long)(nx - 1) * (ny - 1) * (nz - 1);
    const long t = (long)blockIdx.x * kThreads + threadIdx.x;
    if (t >= nin) return;
    const int i = (int)(t % (nx - 1));
    const int j = (int)((t / (nx - 1)) % (ny - 1));
    const int k = (int)(t / ((long)(nx - 1) * (ny - 1)));
    const long V = (long)nx * ny * nz;
    const double* r = rho + it * V;
    const long v = i + (long)nx * (j + (long)ny * k);
    const double tr = stat[2 * it];
    const double r0 = r[v];
    const double X = __dadd_rn(dx / 2.0, __dmul_rn(dx, (double)i));   // src/Mesh.f90:50
    const double Y = __dadd_rn(dx / 2.0, __dmul_rn(dx, (double)j));
    const double Z = __dadd_rn(dx / 2.0, __dmul_rn(dx, (double)k));
    const double nb[3] = {r[v + 1], r[v + nx], r[v + (long)nx * ny]};
    double* sx = surf + (long)it * 3 * cap;
    for (int d = 0; d < 3; ++d) {
        if (!crosses(r0, nb[d], tr)) continue;
        // X + dx (tr - r0) / (r1 - r0) along the crossing direction
        const double off = __ddiv_rn(__dmul_rn(dx, __dsub_rn(tr, r0)), __dsub_rn(nb[d], r0));
        const int slot = atomicAdd(&count[it], 1);
        if (slot >= cap) continue;
        sx[slot] = d == 0 ? __dadd_rn(X, off) : X;
        sx[cap + slot] = d == 1 ? __dadd_rn(Y, off) : Y;
        sx[2 * cap + slot] = d == 2 ? __dadd_rn(Z, off) : Z;
    }
}

// Cutoff = 1 / (1 + exp((DeltaR - radd) / acut)), DeltaR = -/+ the distance to
// the nearest surface point (inside / outside the surface).
__global__ void __launch_bounds__(kThreads)
k_cut_apply(const double* __restrict__ rho, int nx, int ny, int nz, double dx,
            const double* __restrict__ stat, const int* __restrict__ count,
            const double* __restrict__ surf, long cap, double* __restrict__ cut) {
    const int it = blockIdx.y;
    const long V = (long)nx * ny * nz;
    const long v = (long)blockIdx.x * kThreads + threadIdx.x;
    __shared__ double sp[3][kThreads];
    const bool live = v < V;
    const int i = live ? (int)(v % nx) : 0;
    const int j = live ? (int)((v / nx) % ny) : 0;
    const int k = live ? (int)(v / ((long)nx * ny)) : 0;
    const double X = __dadd_rn(dx / 2.0, __dmul_rn(dx, (double)i));
    const double Y = __dadd_rn(dx / 2.0, __dmul_rn(dx, (double)j));
    const double Z = __dadd_rn(dx / 2.0, __dmul_rn(dx, (double)k));
    const long T = min((long)count[it], cap);
    const double* sx = surf + (long)it * 3 * cap;
    double d = 1.0e12;
    for (long t0 = 0; t0 < T; t0 += kThreads) {
        const long t = t0 + threadIdx.x;
        __syncthreads();
        if (t < T) {
            sp[0][threadIdx.x] = sx[t];
            sp[1][threadIdx.x] = sx[cap + t];
            sp[2][threadIdx.x] = sx[2 * cap + t];
        }
        __syncthreads();
        const int nt = (int)min((long)kThreads, T - t0);
        for (int q = 0; q < nt; ++q) {
            const double a = __dsub_rn(X, sp[0][q]), b = __dsub_rn(Y, sp[1][q]),
                         e = __dsub_rn(Z, sp[2][q]);
            d = fmin(d, __dadd_rn(__dadd_rn(__dmul_rn(a, a), __dmul_rn(b, b)), __dmul_rn(e, e)));
        }
    }
    if (!live) return;
    double out = 0.0;
    if (stat[2 * it + 1] >= 0.0000000001) {   // no particles: Cutoff = 0
        const double sig = rho[it * V + v] > stat[2 * it] ? -1.0 : 1.0;
        const double delta = sig * sqrt(d);
        out = 1.0 / (1.0 + exp((delta - kRadd) / kAcut));
    }
    cut[it * V + v] = out;
}

// Per constraint (blockIdx.x): dv sum Q rho_it and dv sum Q^2 rho_it.
__global__ void __launch_bounds__(kThreads)
k_cons_moments(const double* __restrict__ sh, const double* __restrict__ rho, long V, double dv,
               double* __restrict__ red) {
    const int q = blockIdx.x;
    const double* s = sh + (long)q * V;
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    for (long v = threadIdx.x; v < V; v += kThreads) {
        const double y = s[v], yy = y * y;
        const double r0 = rho[v], r1 = rho[V + v];
        acc[0] = fma(y, r0, acc[0]);
        acc[1] = fma(y, r1, acc[1]);
        acc[2] = fma(yy, r0, acc[2]);
        acc[3] = fma(yy, r1, acc[3]);
    }
    __shared__ double part[4][kThreads / 32];
    for (int c = 0; c < 4; ++c) {
        double x = acc[c];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
        if (threadIdx.x % 32 == 0) part[c][threadIdx.x / 32] = x;
    }
    __syncthreads();
    if (threadIdx.x < 4) {
        double x = 0.0;
        for (int w = 0; w < kThreads / 32; ++w) x += part[threadIdx.x][w];
        red[4 * q + threadIdx.x] = x * dv;
    }
}

// field(it) = sum_q (a_q Q_q) Cutoff(it)  (the products in the order of
// CalcConstraintEnergy: Factor (Value - Desired) * SpherHarm * Cutoff)
__global__ void __launch_bounds__(kThreads)
k_cons_field(const double* __restrict__ sh, const double* __restrict__ cut, long V, ConsCoef cf,
             double* __restrict__ field) {
    const long t = (long)blockIdx.x * kThreads + threadIdx.x;
    if (t >= 2 * V) return;
    const long v = t % V;
    double f = 0.0;
    for (int q = 0; q < cf.n; ++q)
        f = __dadd_rn(f, __dmul_rn(__dmul_rn(cf.a[q], sh[(long)q * V + v]), cut[t]));
    field[t] = f;
}

// psi <- psi - multipole(it) psi, multipole(it) = sum_q (f_q Cutoff(it)) Q_q
// (Update of AlternateStep, src/ImaginaryTime.f90:357-359, :426)
__global__ void __launch_bounds__(kThreads)
k_alt_apply(double* __restrict__ psi, const int* __restrict__ qn, const double* __restrict__ sh,
            const double* __restrict__ cut, long V, ConsCoef cf) {
    const int i = blockIdx.y;
    const long t = (long)blockIdx.x * kThreads + threadIdx.x;
    if (t >= 4 * V) return;
    const long v = t % V;
    const int it = (qn[4 * i] + 3) / 2 - 1;
    const double cu = cut[it * V + v];
    double m = 0.0;
    for (int q = 0; q < cf.n; ++q)
        m = __dadd_rn(m, __dmul_rn(__dmul_rn(cf.a[q], cu), sh[(long)q * V + v]));
    double* p = psi + (long)i * 4 * V + t;
    *p = __dsub_rn(*p, __dmul_rn(m, *p));
}

int rutz_cutoff(mg_ctx* c) {
    Constraints& K = c->cons;
    const long V = c->V;
    k_cut_stats<<<2, 1024, 0, c->stream>>>(c->rho, V, c->dv, K.stat, K.count);
    MG_LAUNCHED(c);
    const long nin = (long)(c->nx - 1) * (c->ny - 1) * (c->nz - 1);
    if (nin > 0) {
        k_cut_surface<<<dim3(div_up(nin, kThreads), 2), kThreads, 0, c->stream>>>(
            c->rho, c->nx, c->ny, c->nz, c->p.dx, K.stat, K.count, K.surf, K.cap);
        MG_LAUNCHED(c);
    }
    k_cut_apply<<<dim3(div_up(V, kThreads), 2), kThreads, 0, c->stream>>>(
        c->rho, c->nx, c->ny, c->nz, c->p.dx, K.stat, K.count, K.surf, K.cap, K.cut);
    MG_LAUNCHED(c);
    return MG_OK;
}

}  // namespace

// The cutoff's buffers (first constraint, or the cranking fields).
static int cutoff_alloc(mg_ctx* c) {
    Constraints& K = c->cons;
    const long V = c->V;
    if (!K.cut) {
        K.cap = 3L * std::max(1, c->nx - 1) * std::max(1, c->ny - 1) * std::max(1, c->nz - 1);
        auto A = [&](double** ptr, long n) {
            return cudaMalloc(ptr, n * sizeof(double)) == cudaSuccess &&
                   cudaMemset(*ptr, 0, n * sizeof(double)) == cudaSuccess;
        };
        if (!A(&K.sh, (long)kMaxConstraints * V) || !A(&K.cut, 2 * V) || !A(&K.field, 2 * V) ||
            !A(&K.surf, 2 * 3 * K.cap) || !A(&K.stat, 4) || !A(&K.red, 4 * kMaxConstraints) ||
            cudaMalloc(&K.count, 2 * sizeof(int)) != cudaSuccess ||
            cudaMallocHost(&K.h_red, 4 * kMaxConstraints * sizeof(double)) != cudaSuccess) {
            constraints_free(c);
            return MG_ERR_CUDA;
        }
    }
    return MG_OK;
}

int cranking_cutoff(mg_ctx* c) {
    if (!c->folded) return MG_ERR_ARG;
    MG_TRY(cutoff_alloc(c));
    return rutz_cutoff(c);
}

int add_constraint(mg_ctx* c, const mg_moment_constraint* mc) {
    Constraints& K = c->cons;
    if (!c->folded || mc->l < 1 || mc->l > 10 || mc->m < 0 || mc->m > mc->l ||
        (int)K.list.size() >= kMaxConstraints)
        return MG_ERR_ARG;
    // moments kept by the conserved symmetries (NewMoment_Electric,
    // src/Moments.f90:787-884, quantisation axis z): EV8 keeps even l, even m
    if ((c->p.pc && mc->l % 2) || (c->p.sc && mc->m % 2)) return MG_ERR_ARG;
    const long V = c->V;
    MG_TRY(cutoff_alloc(c));
    const int q = (int)K.list.size();
    std::vector<double> sh(V);
    for (int k = 0; k < c->nz; ++k)
        for (int j = 0; j < c->ny; ++j)
            for (int i = 0; i < c->nx; ++i) {
                const double X = c->p.dx / 2.0 + c->p.dx * i, Y = c->p.dx / 2.0 + c->p.dx * j,
                             Z = c->p.dx / 2.0 + c->p.dx * k;
                sh[i + c->nx * (j + (long)c->ny * k)] = rlylm(mc->l, mc->m, 0, X, Y, Z);
            }
    MG_CUDA(cudaMemcpy(K.sh + (long)q * V, sh.data(), V * sizeof(double), cudaMemcpyHostToDevice));
    MomentConstraint k;
    k.l = mc->l;
    k.m = mc->m;
    k.iteration = mc->iteration;
    k.constraint = k.true_constraint = mc->constraint;   // src/Moments.f90:3719-3726
    k.intensity = mc->intensity;
    K.list.push_back(k);
    K.alternate_check = true;   // CheckForAlternateConstraints, src/Main.f90:247
    return q;
}

bool any_alternating(const mg_ctx* c) {
    for (const MomentConstraint& k : c->cons.list)
        if (k.type == 2) return true;
    return false;
}

// The constrained part of CalculateAllMoments: cutoff, values and squares
// (read back: the readjustment is host logic), the running targets on the
// first call, and the constraint field.
int constraint_moments(mg_ctx* c) {
    Constraints& K = c->cons;
    if (K.list.empty()) return MG_OK;
    const long V = c->V;
    const int nc = (int)K.list.size();
    MG_TRY(rutz_cutoff(c));
    k_cons_moments<<<nc, kThreads, 0, c->stream>>>(K.sh, c->rho, V, c->dv, K.red);
    MG_LAUNCHED(c);
    MG_CUDA(cudaMemcpyAsync(K.h_red, K.red, 4 * nc * sizeof(double), cudaMemcpyDeviceToHost,
                            c->stream));
    MG_CUDA(cudaStreamSynchronize(c->stream));
    ConsCoef cf{};
    for (int q = 0; q < nc; ++q) {
        MomentConstraint& k = K.list[q];
        // OldValue shifts and takes the previous Value (SaveOld = 1,
        // src/Moments.f90:1921-1931)
        for (int i = 6; i > 0; --i) {
            k.old_value[i] = k.old_value[i - 1];
            k.old_iso[i][0] = k.old_iso[i - 1][0];
            k.old_iso[i][1] = k.old_iso[i - 1][1];
        }
        k.old_value[0] = k.value[0] + k.value[1];
        k.old_iso[0][0] = k.value[0];
        k.old_iso[0][1] = k.value[1];
        for (int it = 0; it < 2; ++it) {
            k.value[it] = K.h_red[4 * q + it];
            k.squared[it] = K.h_red[4 * q + 2 + it];
        }
        // first call: the running target starts at the current value
        if (!k.started && k.type != 0) k.constraint = k.value[0] + k.value[1];
        k.started = true;
        // CalcConstraintEnergy: Factor = 2 Intensity, (Value - Desired)
        cf.a[q] = k.type == 2 ? (2.0 * k.intensity) * ((k.value[0] + k.value[1]) - k.constraint)
                              : 0.0;
    }
    cf.n = nc;
    k_cons_field<<<div_up(2 * V, kThreads), kThreads, 0, c->stream>>>(K.sh, K.cut, V, cf,
                                                                        K.field);
    MG_LAUNCHED(c);
    return MG_OK;
}

void readjust_moments(mg_ctx* c, int iteration) {
    const double momentum = c->step_mom;   // the GradDesc momentum in use
    for (MomentConstraint& k : c->cons.list) {
        if (k.type != 2) continue;
        if (k.intensity == 0.0) {
            k.intensity = 2.0 / (k.squared[0] + k.squared[1]);
            if (momentum != 0.0) k.intensity = 0.5 * k.intensity;
        }
        k.constraint = k.constraint - ((k.value[0] + k.value[1]) - k.true_constraint);
    }
    for (MomentConstraint& k : c->cons.list)
        if (k.type != 0 && k.iteration > 0 && iteration > k.iteration) k.type = 0;
}

int alternate_step(mg_ctx* c) {
    Constraints& K = c->cons;
    Basis& B = c->bas[MG_HF_BASIS];
    if (!B.have_qn) return MG_ERR_STATE;
    if (!K.list.empty()) MG_TRY(rutz_cutoff(c));
    ConsCoef cf{};
    bool any = false;
    for (size_t q = 0; q < K.list.size(); ++q) {
        const MomentConstraint& k = K.list[q];
        if (k.type == 2) {
            any = true;
            const double o2 = k.squared[0] + k.squared[1];
            const double value = k.value[0] + k.value[1];
            cf.a[q] = 0.5 * (value - k.true_constraint) / (o2 + kD0);
        } else {
            cf.a[q] = 0.0;
        }
    }
    cf.n = (int)K.list.size();
    if (any) {
        const long V = c->V;
        k_alt_apply<<<dim3(div_up(4 * V, kThreads), c->p.nwt), kThreads, 0, c->stream>>>(
            B.psi, B.qn, K.sh, K.cut, V, cf);
        MG_LAUNCHED(c);
    }
    return gram_schmidt(c);
}

// ConverMultipoleAll (src/Moments.f90:2628-2701) over the constrained moments.
bool moments_converged(const mg_ctx* c, double prec) {
    for (const MomentConstraint& k : c->cons.list) {
        if (k.type == 0) continue;
        const double C = k.constraint;
        double d[8];
        const double v = k.value[0] + k.value[1];
        if (k.true_constraint != 0.0) {
            d[0] = std::fabs((C - v) / C);
            for (int i = 1; i < 8; ++i) d[i] = std::fabs((C - k.old_value[i - 1]) / C);
        } else {
            d[0] = std::fabs(C - v);
            for (int i = 1; i < 8; ++i) d[i] = std::fabs(C - k.old_value[i - 1]);
        }
        for (int i = 0; i < 8; ++i)
            if (d[i] >= prec) return false;
    }
    return true;
}

void constraints_free(mg_ctx* c) {
    Constraints& K = c->cons;
    auto F = [](void* p) { if (p) cudaFree(p); };
    F(K.sh); F(K.cut); F(K.field); F(K.surf); F(K.stat); F(K.red); F(K.count);
    if (K.h_red) cudaFreeHost(K.h_red);
    K.sh = K.cut = K.field = K.surf = K.stat = K.red = K.h_red = nullptr;
    K.count = nullptr;
}

}  // namespace mg

// ---------------------------------------------------------------------------
// Entry points
// ---------------------------------------------------------------------------
extern "C" int mg_add_constraint(mg_ctx* c, const mg_moment_constraint* mc) {
    if (!c || !mc) return MG_ERR_ARG;
    return mg::add_constraint(c, mc);
}

extern "C" int mg_get_constraint(mg_ctx* c, int q, mg_constraint_state* out) {
    if (!c || !out || q < 0 || q >= (int)c->cons.list.size()) return MG_ERR_ARG;
    const mg::MomentConstraint& k = c->cons.list[q];
    for (int it = 0; it < 2; ++it) {
        out->value[it] = k.value[it];
        out->squared[it] = k.squared[it];
    }
    out->constraint = k.constraint;
    out->intensity = k.intensity;
    out->active = k.type != 0;
    return MG_OK;
}

extern "C" int mg_get_constraint_fields(mg_ctx* c, double* cutoff, double* field) {
    if (!c) return MG_ERR_ARG;
    const long V = c->V;
    const mg::Constraints& K = c->cons;
    for (int w = 0; w < 2; ++w) {
        double* dst = w == 0 ? cutoff : field;
        if (!dst) continue;
        const double* src = w == 0 ? K.cut : K.field;
        if (src) {
            MG_CUDA(cudaMemcpyAsync(dst, src, 2 * V * sizeof(double), cudaMemcpyDeviceToHost,
                                    c->stream));
        } else {
            for (long v = 0; v < 2 * V; ++v) dst[v] = 0.0;
        }
    }
    MG_CUDA(cudaStreamSynchronize(c->stream));
    return MG_OK;
}

extern "C" int mg_alternate_step(mg_ctx* c) {
    if (!c) return MG_ERR_ARG;
    return mg::alternate_step(c);
}

extern "C" int mg_readjust_moments(mg_ctx* c, int iteration) {
    if (!c) return MG_ERR_ARG;
    mg::readjust_moments(c, iteration);
    return MG_OK;
}
