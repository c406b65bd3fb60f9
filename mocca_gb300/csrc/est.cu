// est.cu -- IterativeEstimation (src/ImaginaryTime.f90:28-211), FP64: the
// imaginary-time step dt and the momentum, re-estimated at every GradDesc
// when ParameterEstimation = 1.
//   1. maxspwf (a spinor with the quantum numbers of the last HF spwf, or of
//      the last neutron spwf without protons) climbs towards the largest
//      eigenvalue of h: up to 500 steps of
//        maxE = <psi|h psi>, update = dt/hbar (h psi - maxE psi) + mu update,
//        psi <- (psi + update) / norm,
//      stopping when maxE moves by less than 1e-2 MeV.  It starts (first call)
//      from uniform random grid values and keeps its state between calls.
//   2. relE: the smallest positive quasiparticle energy (HFB), or the
//      smallest positive HF gap between an occupied and an empty spwf of the
//      same isospin, at least 0.1 (HF).
//   3. maxE -= min spwf energy; kappa = relE / maxE;
//      mu = ((sqrt(kappa) - 1) / (sqrt(kappa) + 1))^2,
//      dt = 0.9 hbar 4 / (maxE + relE + 2 sqrt(maxE relE)).
// The reference fills the start with Fortran's random_number (unseeded); this
// uses a fixed-seed splitmix64 stream instead, so that runs repeat.
#include <cmath>
#include <vector>

#include "mg_internal.cuh"

namespace mg {

namespace {

constexpr int kThreads = 256;

// uniform [0, 1) value k of the fixed start stream: splitmix64 (Steele, Lea,
// Flood, OOPSLA 2014) at state seed + (k + 1) * golden gamma, top 53 bits
inline double start_value(unsigned long long k) {
    unsigned long long z = 0x2545F4914F6CDD1Dull + (k + 1) * 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}

// update = fac (h psi - maxE psi) + mu update ; psi += update ; block partials of psi^2
__global__ void __launch_bounds__(kThreads)
k_est_step(double* __restrict__ psi, const double* __restrict__ hp, double* __restrict__ up,
           const double* __restrict__ e_dev, double fac, double mom, long n,
           double* __restrict__ part) {
    __shared__ double red[kThreads / 32];
    const long t = (long)blockIdx.x * kThreads + threadIdx.x;
    double s = 0.0;
    if (t < n) {
        const double maxE = e_dev[0];
        const double u = fac * (hp[t] - maxE * psi[t]) + mom * up[t];
        up[t] = u;
        const double x = psi[t] + u;
        psi[t] = x;
        s = x * x;
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (threadIdx.x % 32 == 0) red[threadIdx.x / 32] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0;
        for (int q = 0; q < kThreads / 32; ++q) a += red[q];
        part[blockIdx.x] = a;
    }
}

// psi /= sqrt(norm), norm = dv * (partials added in block order)
__global__ void k_est_normalise(double* __restrict__ psi, const double* __restrict__ part,
                                int nblk, double dv, long n) {
    __shared__ double scale;
    if (threadIdx.x == 0) {
        double a = 0.0;
        for (int q = 0; q < nblk; ++q) a += part[q];
        scale = 1.0 / std::sqrt(a * dv);
    }
    __syncthreads();
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x)
        psi[t] *= scale;
}

}  // namespace

int estimate_parameters(mg_ctx* c) {
    Basis& B = c->bas[MG_HF_BASIS];
    if (!B.have_qn) return MG_ERR_STATE;
    const long V = c->V, V4 = 4 * V;
    const int nwt = c->p.nwt;
    double* psi = nullptr;
    if (!c->est) {
        MG_CUDA(cudaMalloc(&c->est, (28 * V + 2) * sizeof(double)));
        MG_CUDA(cudaMalloc(&c->est_jobs, 4 * sizeof(GridJob)));
        MG_CUDA(cudaMalloc(&c->est_qn, 4 * sizeof(int)));
    }
    psi = c->est;
    double* der = psi + V4;
    double* lap = der + 12 * V;
    double* hp = lap + V4;
    double* up = hp + V4;
    double* e_dev = up + V4;
    ++c->est_iter;
    if (c->est_iter == 1) {
        // maxspwf: quantum numbers of HFBasis(nwt), or of the last neutron
        // spwf when there are no protons
        int iw = nwt - 1;
        if (c->p.protons < 1e-9)
            for (int i = 0; i < nwt; ++i)
                if (B.h_qn[4 * i] == -1) iw = i;
        const int* q = &B.h_qn[4 * iw];
        MG_CUDA(cudaMemcpy(c->est_qn, q, 4 * sizeof(int), cudaMemcpyHostToDevice));
        for (int k = 0; k < 4; ++k) c->est_h_qn[k] = q[k];
        std::vector<GridJob> jobs(4);
        for (int l = 0; l < 4; ++l) {
            GridJob J{};
            J.in = psi + l * V;
            J.dx = der + (0 * 4 + l) * V;
            J.dy = der + (1 * 4 + l) * V;
            J.dz = der + (2 * 4 + l) * V;
            J.lap = lap + l * V;
            for (int d = 0; d < 3; ++d) J.slot[d] = (int8_t)lag_slot(d, q[1], q[2], q[3], l + 1);
            jobs[l] = J;
        }
        MG_CUDA(cudaMemcpy(c->est_jobs, jobs.data(), 4 * sizeof(GridJob), cudaMemcpyHostToDevice));
        std::vector<double> h(V4);
        double norm = 0.0;
        for (long k = 0; k < V4; ++k) {
            h[k] = start_value((unsigned long long)k);
            norm += h[k] * h[k];
        }
        const double sc = 1.0 / std::sqrt(norm * c->dv);
        for (long k = 0; k < V4; ++k) h[k] *= sc;
        MG_CUDA(cudaMemcpyAsync(psi, h.data(), V4 * sizeof(double), cudaMemcpyHostToDevice,
                                c->stream));
        MG_CUDA(cudaStreamSynchronize(c->stream));
        // FP64 derivatives of the probe (the double-float kernels write FP64
        // when asked to in the mixed form)
        MG_TRY(run_jobs(c, c->est_jobs, 4, false));
    }
    MG_CUDA(cudaMemsetAsync(up, 0, V4 * sizeof(double), c->stream));
    const double fac = c->step_dt / c->f.hbar, mom = c->step_mom;
    const int nblk = div_up(V4, kThreads);
    double maxE = 0.0, prev = NAN, con = NAN;
    for (int it = 0; it < 500; ++it) {
        MG_TRY(hpsi_single(c, psi, der, lap, c->est_qn, hp, e_dev));
        MG_CUDA(cudaMemcpyAsync(&maxE, e_dev, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
        k_est_step<<<nblk, kThreads, 0, c->stream>>>(psi, hp, up, e_dev, fac, mom, V4, c->red);
        MG_LAUNCHED(c);
        k_est_normalise<<<std::min(nblk, 4 * c->num_sms), kThreads, 0, c->stream>>>(psi, c->red,
                                                                                  nblk, c->dv, V4);
        MG_LAUNCHED(c);
        MG_TRY(run_jobs(c, c->est_jobs, 4, false));
        MG_CUDA(cudaStreamSynchronize(c->stream));
        con = prev - maxE;
        prev = maxE;
        if (std::fabs(con) < 1e-2) break;
    }
    if (std::isnan(maxE)) return MG_ERR_NAN;   // src/ImaginaryTime.f90:190-192
    // the smallest excitation
    double relE = 10000.0;
    std::vector<double> e(nwt), occ(nwt);
    MG_CUDA(cudaMemcpy(e.data(), B.e, nwt * sizeof(double), cudaMemcpyDeviceToHost));
    if (c->p.pairing == MG_PAIRING_HFB && c->hfb.ready && c->hfb.eT.have_vectors) {
        const Hfb& H = c->hfb;
        std::vector<double> w(4L * H.nmax);
        MG_CUDA(cudaMemcpy(w.data(), H.eT.w, w.size() * sizeof(double), cudaMemcpyDeviceToHost));
        for (int b = 0; b < 4; ++b)
            for (int m = H.hsz_h[b]; m < 2 * H.hsz_h[b]; ++m) {
                const double x = w[(size_t)b * H.eT.wstride + m];
                if (x > 0.0) relE = std::min(relE, std::fabs(x));
            }
    } else {
        MG_CUDA(cudaMemcpy(occ.data(), B.occ, nwt * sizeof(double), cudaMemcpyDeviceToHost));
        for (int i = 0; i < nwt; ++i) {
            if (std::fabs(occ[i]) < 0.5) continue;
            for (int k = 0; k < nwt; ++k) {
                if (std::fabs(occ[k]) > 0.5 || B.h_qn[4 * k] != B.h_qn[4 * i]) continue;
                const double d = e[k] - e[i];
                if (d > 0.0) relE = std::min(relE, d);
            }
        }
        if (relE < 0.1) relE = 0.1;
    }
    double minh = 10000.0;
    for (int i = 0; i < nwt; ++i) minh = std::min(minh, e[i]);
    maxE -= minh;
    const double kappa = relE / maxE;
    c->step_mom = std::pow((std::sqrt(kappa) - 1.0) / (std::sqrt(kappa) + 1.0), 2.0);
    c->step_dt = 4.0 / (maxE + relE + 2.0 * std::sqrt(maxE * relE)) * c->f.hbar * 0.90;
    return MG_OK;
}

}  // namespace mg
