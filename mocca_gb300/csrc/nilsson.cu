// nilsson.cu -- the Nilsson start of an EV8 run on the device: INITWF
// (src/InOut.f90:1418-1473) calling nil8's nilsson (src/nil8.f90:16-546),
// then a seeded uniform perturbation of every grid value and the
// normalisation of each spwf.
//
// The small algebra stays on the host: the Cartesian oscillator states of
// the major shells (src/nil8.f90:162-268), the 1-D oscillator functions on
// the half line (:283-339, a few hundred values), the Nilsson Hamiltonian
// of each shell (:383-433) and its diagonalisation (cyclic Jacobi here, in
// place of diagoncr8), the exchange sort of the levels (:437-449) and the
// selection of the lowest nw states, positive parity first (:455-470).
// The device evaluates the mesh: every spwf is a sum of products
// he_z(z) he_y(y) he_x(x) over the states of its shell (:471-536), one
// thread per mesh point of one spwf, then adds the perturbation from a
// counter-based generator keyed on (seed, spwf, component, point) and
// divides by the norm (block partial sums in a fixed order).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "mg_internal.cuh"

namespace mg {

namespace {

constexpr int kThreads = 256;
constexpr int kMaxTerms = 512;   // states of one shell (11 shells: at most 66)

// Cartesian HO states (nx, ny, nz) of the first meven even and modd odd
// shells in nil8's order: per shell the four (x, y)-parity sub-blocks.
void shell_states(int meven, int modd, std::vector<int>& st, std::vector<int>& starts,
                  std::vector<int>& subs) {
    std::vector<int> shells;
    for (int ni = 1; ni <= meven; ++ni) shells.push_back(2 * (ni - 1));
    for (int ni = 1; ni <= modd; ++ni) shells.push_back(2 * ni - 1);
    starts.assign(1, 0);
    subs.clear();
    st.clear();
    for (int n : shells) {
        const int ni = n % 2 == 0 ? n / 2 + 1 : (n + 1) / 2;
        std::vector<std::pair<int, int>> blocks[4];
        if (n % 2 == 0) {
            for (int i = 1; i <= ni; ++i)
                for (int j = 1; j <= ni - i + 1; ++j) blocks[0].push_back({2 * (i - 1), 2 * (j - 1)});
            for (int i = 1; i < ni; ++i)
                for (int j = 1; j <= ni - i; ++j) {
                    blocks[1].push_back({2 * (i - 1) + 1, 2 * (j - 1) + 1});
                }
            for (int i = 1; i < ni; ++i)
                for (int j = 1; j <= ni - i; ++j) blocks[2].push_back({2 * (i - 1) + 1, 2 * (j - 1)});
            for (int i = 1; i < ni; ++i)
                for (int j = 1; j <= ni - i; ++j) blocks[3].push_back({2 * (i - 1), 2 * (j - 1) + 1});
        } else {
            for (int i = 1; i <= ni; ++i)
                for (int j = 1; j <= ni - i + 1; ++j) blocks[0].push_back({2 * (i - 1), 2 * (j - 1)});
            for (int i = 1; i < ni; ++i)
                for (int j = 1; j <= ni - i; ++j) blocks[1].push_back({2 * i - 1, 2 * j - 1});
            for (int i = 1; i <= ni; ++i)
                for (int j = 1; j <= ni - i + 1; ++j) blocks[2].push_back({2 * i - 1, 2 * (j - 1)});
            for (int i = 1; i <= ni; ++i)
                for (int j = 1; j <= ni - i + 1; ++j) blocks[3].push_back({2 * (i - 1), 2 * j - 1});
        }
        for (int k = 0; k < 4; ++k) {
            subs.push_back((int)blocks[k].size());
            for (auto& ac : blocks[k]) {
                st.push_back(ac.first);
                st.push_back(ac.second);
                st.push_back(n - ac.first - ac.second);
            }
        }
        starts.push_back((int)st.size() / 3);
    }
}

// Nilsson Hamiltonian of one shell in units of hbar omega0 (stretched l.s
// with kappa = x, l^2 with x mu = x y), src/nil8.f90:383-433.
void shell_matrix(const int* s, int n, double x, double y, double ax, double ay, double az,
                  std::vector<double>& h) {
    h.assign((size_t)n * n, 0.0);
    for (int i = 0; i < n; ++i) {
        const int nx1 = s[3 * i], ny1 = s[3 * i + 1], nz1 = s[3 * i + 2];
        const int nb = nx1 + ny1 + nz1;
        const double x1 = 1 - 2 * ((nb - nz1) % 2), x2 = 1 - 2 * (ny1 % 2);
        for (int j = i; j < n; ++j) {
            const int nx2 = s[3 * j], ny2 = s[3 * j + 1], nz2 = s[3 * j + 2];
            double v = 0.0;
            if (j == i) {
                v = ax * (nx1 + 0.5) + ay * (ny1 + 0.5) + az * (nz1 + 0.5) -
                    x * y * ((nb * (nb + 1)) / 2.0 - nx1 * nx1 - ny1 * ny1 - nz1 * nz1);
            } else if (nx1 == nx2) {
                const double an = ny2, am = ny1;
                if (ny2 == ny1 + 1) v = x * std::sqrt(an * nz1);
                if (ny2 == ny1 - 1) v = x * std::sqrt(am * nz2);
                if (ny2 == ny1 + 2) v = -x * y * std::sqrt(an * (ny2 - 1) * nz1 * (nz1 - 1));
                if (ny2 == ny1 - 2) v = -x * y * std::sqrt(am * (ny1 - 1) * nz2 * (nz2 - 1));
            } else if (nz1 == nz2) {
                const double am = nx1, an = nx2;
                if (nx2 == nx1 + 1) v = -x * x1 * std::sqrt(an * ny1);
                if (nx2 == nx1 - 1) v = -x * x1 * std::sqrt(am * ny2);
                if (nx2 == nx1 + 2) v = -x * y * std::sqrt(an * (nx2 - 1) * ny1 * (ny1 - 1));
                if (nx2 == nx1 - 2) v = -x * y * std::sqrt(am * (nx1 - 1) * ny2 * (ny2 - 1));
            } else if (ny1 == ny2) {
                const double x3 = 1.0 - 2.0 * (nx1 % 2), x4 = 1.0 - 2.0 * (nx2 % 2);
                const double an = nx2, am = nx1;
                if (nz2 == nz1 + 1) v = -x * x2 * x3 * std::sqrt(am * nz2);
                if (nz2 == nz1 - 1) v = -x * x2 * x4 * std::sqrt(an * nz1);
                if (nz2 == nz1 + 2) v = x * y * std::sqrt(nz2 * (nz2 - 1) * am * (nx1 - 1));
                if (nz2 == nz1 - 2) v = x * y * std::sqrt(nz1 * (nz1 - 1) * an * (nx2 - 1));
            }
            h[(size_t)i * n + j] = h[(size_t)j * n + i] = v;
        }
    }
}

// Cyclic Jacobi eigen-decomposition of a small symmetric matrix (row-major,
// overwritten); vectors in the columns of z, ascending values, each vector
// with its largest component positive.
void jacobi_eigh(std::vector<double>& a, int n, std::vector<double>& w, std::vector<double>& z) {
    z.assign((size_t)n * n, 0.0);
    for (int i = 0; i < n; ++i) z[(size_t)i * n + i] = 1.0;
    for (int sweep = 0; sweep < 100; ++sweep) {
        double off = 0.0, tot = 0.0;
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) {
                const double v = a[(size_t)i * n + j] * a[(size_t)i * n + j];
                tot += v;
                if (i != j) off += v;
            }
        if (off <= 1e-30 * tot || off == 0.0) break;
        for (int p = 0; p < n - 1; ++p)
            for (int q = p + 1; q < n; ++q) {
                const double apq = a[(size_t)p * n + q];
                if (apq == 0.0) continue;
                const double app = a[(size_t)p * n + p], aqq = a[(size_t)q * n + q];
                const double th = (aqq - app) / (2.0 * apq);
                const double t = (th >= 0 ? 1.0 : -1.0) / (std::fabs(th) + std::sqrt(th * th + 1.0));
                const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < n; ++k) {
                    const double akp = a[(size_t)k * n + p], akq = a[(size_t)k * n + q];
                    a[(size_t)k * n + p] = c * akp - s * akq;
                    a[(size_t)k * n + q] = s * akp + c * akq;
                }
                for (int k = 0; k < n; ++k) {
                    const double apk = a[(size_t)p * n + k], aqk = a[(size_t)q * n + k];
                    a[(size_t)p * n + k] = c * apk - s * aqk;
                    a[(size_t)q * n + k] = s * apk + c * aqk;
                }
                for (int k = 0; k < n; ++k) {
                    const double zkp = z[(size_t)k * n + p], zkq = z[(size_t)k * n + q];
                    z[(size_t)k * n + p] = c * zkp - s * zkq;
                    z[(size_t)k * n + q] = s * zkp + c * zkq;
                }
            }
    }
    std::vector<int> ord(n);
    for (int i = 0; i < n; ++i) ord[i] = i;
    std::stable_sort(ord.begin(), ord.end(), [&](int i, int j) {
        return a[(size_t)i * n + i] < a[(size_t)j * n + j];
    });
    std::vector<double> zs((size_t)n * n);
    w.resize(n);
    for (int c = 0; c < n; ++c) {
        const int o = ord[c];
        w[c] = a[(size_t)o * n + o];
        int big = 0;
        for (int k = 1; k < n; ++k)
            if (std::fabs(z[(size_t)k * n + o]) > std::fabs(z[(size_t)big * n + o])) big = k;
        const double sg = z[(size_t)big * n + o] < 0 ? -1.0 : 1.0;
        for (int k = 0; k < n; ++k) zs[(size_t)k * n + c] = sg * z[(size_t)k * n + o];
    }
    z.swap(zs);
}

// nil8's 1-D oscillator functions on the stored half line
// (src/nil8.f90:283-339): x^k exp(-x^2/2) by repeated multiplication,
// orthogonalised against the lower functions of the same parity and
// normalised on the mirrored line.  he[f * npts + i].
void half_line_functions(int nfun, int npts, double xho, double dx, std::vector<double>& he) {
    he.assign((size_t)nfun * npts, 0.0);
    auto row = [&](int f) { return he.data() + (size_t)f * npts; };
    for (int j = 1; j <= nfun / 2; ++j) {
        const int a = 2 * j - 2, b = 2 * j - 1;
        if (j == 1) {
            for (int i = 0; i < npts; ++i) {
                const double xs = xho * (i + 0.5);
                row(0)[i] = std::exp(-xs * xs / 2.0);
                row(1)[i] = xs * row(0)[i];
            }
        } else {
            for (int i = 0; i < npts; ++i) {
                const double xs = xho * (i + 0.5), x2 = xs * xs;
                row(a)[i] = row(a - 2)[i] * x2;
                row(b)[i] = row(b - 2)[i] * x2;
            }
            for (int k = 1; k < j; ++k) {
                const int c = 2 * k - 2, d = 2 * k - 1;
                double s1 = 0.0, s2 = 0.0;
                for (int i = 0; i < npts; ++i) {
                    s1 += row(a)[i] * row(c)[i];
                    s2 += row(b)[i] * row(d)[i];
                }
                s1 *= dx * 2.0;
                s2 *= dx * 2.0;
                for (int i = 0; i < npts; ++i) {
                    row(a)[i] -= s1 * row(c)[i];
                    row(b)[i] -= s2 * row(d)[i];
                }
            }
        }
        for (int f : {a, b}) {
            double s = 0.0;
            for (int i = 0; i < npts; ++i) s += row(f)[i] * row(f)[i];
            const double sc = std::sqrt(0.5 / (dx * s));
            for (int i = 0; i < npts; ++i) row(f)[i] *= sc;
        }
    }
}

// splitmix64 of a 64-bit counter: a uniform value in [-1, 1)
__device__ __forceinline__ double uniform_pm1(unsigned long long seed, unsigned long long ctr) {
    unsigned long long z = seed + 0x9E3779B97F4A7C15ULL * (ctr + 1);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    z ^= z >> 31;
    return (double)(z >> 11) * (2.0 / 9007199254740992.0) - 1.0;
}

// One thread per mesh point of one spwf (blockIdx.y): the sum over the
// spwf's terms of c he_z(z) he_y(y) he_x(x) into its component, plus the
// perturbation; block partial sums of psi^2 into part[spwf][chunk].
__global__ void __launch_bounds__(kThreads)
k_nilsson_eval(const int4* __restrict__ terms, const double* __restrict__ coef,
               const int* __restrict__ toff, const int* __restrict__ tiso,
               const double* __restrict__ he, int nfun, int npts, int nx, int ny, int nz, long V,
               double amplitude, unsigned long long seed, double* __restrict__ psi,
               double* __restrict__ part) {
    __shared__ double red[kThreads / 32];
    const int i = blockIdx.y;
    const int t0 = toff[i], t1 = toff[i + 1];
    const double* hx = he + (size_t)(tiso[i] * 3 + 0) * nfun * npts;
    const double* hy = he + (size_t)(tiso[i] * 3 + 1) * nfun * npts;
    const double* hz = he + (size_t)(tiso[i] * 3 + 2) * nfun * npts;
    double sq = 0.0;
    for (long v = (long)blockIdx.x * kThreads + threadIdx.x; v < V;
         v += (long)gridDim.x * kThreads) {
        const int x = (int)(v % nx), y = (int)((v / nx) % ny), z = (int)(v / ((long)nx * ny));
        double g0 = 0.0, g1 = 0.0, g2 = 0.0, g3 = 0.0;
        for (int t = t0; t < t1; ++t) {
            const int4 q = terms[t];
            const double val =
                coef[t] * hx[(size_t)q.x * npts + x] * hy[(size_t)q.y * npts + y] *
                hz[(size_t)q.z * npts + z];
            g0 += q.w == 0 ? val : 0.0;
            g1 += q.w == 1 ? val : 0.0;
            g2 += q.w == 2 ? val : 0.0;
            g3 += q.w == 3 ? val : 0.0;
        }
        const double g[4] = {g0, g1, g2, g3};
#pragma unroll
        for (int l = 0; l < 4; ++l) {
            double u = g[l];
            if (amplitude != 0.0)
                u += amplitude *
                     uniform_pm1(seed, ((unsigned long long)i * 4 + l) * (unsigned long long)V + v);
            psi[(size_t)i * 4 * V + (size_t)l * V + v] = u;
            sq = fma(u, u, sq);
        }
    }
    for (int o = 16; o > 0; o >>= 1) sq += __shfl_xor_sync(0xffffffffu, sq, o);
    if (threadIdx.x % 32 == 0) red[threadIdx.x / 32] = sq;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int w = 0; w < kThreads / 32; ++w) s += red[w];
        part[(size_t)i * gridDim.x + blockIdx.x] = s;
    }
}

// psi /= sqrt(dv sum psi^2): every block sums its spwf's partials in the
// same order, then scales its points
__global__ void __launch_bounds__(kThreads)
k_nilsson_norm(const double* __restrict__ part, int nch, double dv, long V4,
               double* __restrict__ psi) {
    const int i = blockIdx.y;
    double s = 0.0;
    for (int c = 0; c < nch; ++c) s += part[(size_t)i * nch + c];
    const double sc = 1.0 / sqrt(s * dv);
    for (long k = (long)blockIdx.x * kThreads + threadIdx.x; k < V4;
         k += (long)gridDim.x * kThreads)
        psi[(size_t)i * V4 + k] *= sc;
}

}  // namespace

}  // namespace mg

extern "C" int mg_nilsson_start(mg_ctx* c, const mg_nilsson_params* np) {
    using namespace mg;
    if (!c || !np) return MG_ERR_ARG;
    const mg_params& p = c->p;
    const int nwt = p.nwt, n_neutron = np->n_neutron;
    if (!(p.pc && p.sc && p.tsc) || !c->folded) return MG_ERR_ARG;   // EV8 states
    if (std::max(p.nx, p.ny) > p.nz) return MG_ERR_ARG;             // nil8 needs nz >= nx, ny
    if (n_neutron < 0 || n_neutron > nwt || np->meven < 1 || np->modd < 1 ||
        np->meven > 12 || np->modd > 12 || !(np->ho[0] > 0 && np->ho[1] > 0 && np->ho[2] > 0) ||
        !(np->amplitude >= 0.0) || !(std::floor(p.neutrons) + std::floor(p.protons) > 0))
        return MG_ERR_ARG;
    std::vector<int> st, starts, subs;
    shell_states(np->meven, np->modd, st, starts, subs);
    const int nvec = starts.back(), nblk = (int)starts.size() - 1;
    if (std::max(n_neutron, nwt - n_neutron) > nvec) return MG_ERR_ARG;
    for (int b = 0; b < nblk; ++b)
        if (starts[b + 1] - starts[b] > kMaxTerms) return MG_ERR_ARG;
    const int nmax = std::max(np->meven, np->modd), nfun = 2 * nmax;
    const int npts = std::max(p.nx, std::max(p.ny, p.nz));
    // nilsson's arguments as INITWF passes them (src/InOut.f90:1454-1455):
    // floor(neutrons) as npp, floor(protons) as npn
    const double npp = std::floor(p.neutrons), npn = std::floor(p.protons);
    const double xk[4] = {0.08, 0.08, 0.0637, 0.0637}, xmu[4] = {0.0, 0.0, 0.42, 0.60};
    const double hbm = 6.58218 * 6.58218 / 1.044673;
    const double xis = (npn - npp) / (npn + npp);
    const double cf[2] = {1.0 + 0.14 * xis, 0.986 - 0.14 * xis};
    const double hox = np->ho[0], hoy = np->ho[1], hoz = np->ho[2];
    std::vector<double> he_all((size_t)2 * 3 * nfun * npts);
    std::vector<int4> terms;
    std::vector<double> coef;
    std::vector<int> toff(1, 0), tiso;
    std::vector<int> qn(4 * (size_t)nwt);
    std::vector<double> en(nwt);
    int w = 0;
    for (int it = 0; it < 2; ++it) {
        const int iso = it == 0 ? -1 : 1, nw = it == 0 ? n_neutron : nwt - n_neutron;
        const double hos[3] = {hox, hoy, hoz};
        for (int a = 0; a < 3; ++a) {
            std::vector<double> he;
            half_line_functions(nfun, npts, std::sqrt(hos[a]) * p.dx * std::sqrt(cf[it]), p.dx,
                                he);
            std::copy(he.begin(), he.end(), he_all.begin() + (size_t)(it * 3 + a) * nfun * npts);
        }
        double ho0 = std::cbrt(hox * hoy * hoz);
        const double ax = hox / ho0, ay = hoy / ho0, az = hoz / ho0;
        ho0 = ho0 * hbm * cf[it];
        const double npart = it == 0 ? npn : npp;
        const double x = npart <= 50 ? xk[it] : xk[it + 2], y = npart <= 50 ? xmu[it] : xmu[it + 2];
        std::vector<double> e(nvec);
        std::vector<std::vector<double>> vecs(nblk);
        for (int b = 0; b < nblk; ++b) {
            const int n = starts[b + 1] - starts[b];
            std::vector<double> h, d;
            shell_matrix(&st[3 * (size_t)starts[b]], n, x, y, ax, ay, az, h);
            jacobi_eigh(h, n, d, vecs[b]);
            for (int k = 0; k < n; ++k) e[starts[b] + k] = d[k] * ho0 - 50.0;
        }
        // exchange sort (src/nil8.f90:437-449): ties keep their order
        std::vector<int> nor(nvec);
        for (int i = 0; i < nvec; ++i) nor[i] = i;
        std::vector<double> ev = e;
        for (int i = 0; i < nvec - 1; ++i)
            for (int j = i + 1; j < nvec; ++j)
                if (ev[j] < ev[i]) {
                    std::swap(ev[i], ev[j]);
                    std::swap(nor[i], nor[j]);
                }
        std::vector<int> npa(nvec), order;
        for (int i = 0; i < nvec; ++i) {
            const int j = nor[i];
            npa[i] = 1 - 2 * ((st[3 * j] + st[3 * j + 1] + st[3 * j + 2]) % 2);
        }
        for (int i = 0; i < nw; ++i)
            if (npa[i] != -1) order.push_back(i);
        for (int i = 0; i < nw; ++i)
            if (npa[i] != 1) order.push_back(i);
        for (int i : order) {
            const int j = nor[i];
            int b = 0;
            while (j >= starts[b + 1]) ++b;
            const int n = starts[b + 1] - starts[b];
            const std::vector<double>& s = vecs[b];
            const int col = j - starts[b];
            int off = 0;
            for (int k = 0; k < 4; ++k) {
                const int flip = (k == 0 || k == 2) ? 3 : 0;
                for (int q = off; q < off + subs[4 * b + k]; ++q) {
                    const int* a = &st[3 * (size_t)(starts[b] + q)];
                    double xph = s[(size_t)q * n + col];
                    if ((a[1] + 1) % 4 == flip) xph = -xph;
                    terms.push_back(make_int4(a[0], a[1], a[2], k));
                    coef.push_back(xph);
                }
                off += subs[4 * b + k];
            }
            toff.push_back((int)terms.size());
            tiso.push_back(it);
            qn[4 * w + 0] = iso;
            qn[4 * w + 1] = npa[i];
            qn[4 * w + 2] = 1;
            qn[4 * w + 3] = 1;
            en[w] = ev[i];
            ++w;
        }
    }
    // the mesh on the device
    const long V = c->V;
    const int nch = std::max(1, std::min(64, div_up(V, kThreads * 4)));
    int4* d_terms = nullptr;
    double *d_coef = nullptr, *d_he = nullptr, *d_part = nullptr;
    int *d_toff = nullptr, *d_tiso = nullptr;
    auto release = [&]() {
        cudaFree(d_terms);
        cudaFree(d_coef);
        cudaFree(d_he);
        cudaFree(d_part);
        cudaFree(d_toff);
        cudaFree(d_tiso);
    };
    bool ok = cudaMalloc(&d_terms, std::max<size_t>(1, terms.size()) * sizeof(int4)) == cudaSuccess &&
              cudaMalloc(&d_coef, std::max<size_t>(1, coef.size()) * sizeof(double)) == cudaSuccess &&
              cudaMalloc(&d_he, he_all.size() * sizeof(double)) == cudaSuccess &&
              cudaMalloc(&d_part, (size_t)nwt * nch * sizeof(double)) == cudaSuccess &&
              cudaMalloc(&d_toff, toff.size() * sizeof(int)) == cudaSuccess &&
              cudaMalloc(&d_tiso, std::max<size_t>(1, tiso.size()) * sizeof(int)) == cudaSuccess;
    if (ok)
        ok = cudaMemcpyAsync(d_terms, terms.data(), terms.size() * sizeof(int4),
                             cudaMemcpyHostToDevice, c->stream) == cudaSuccess &&
             cudaMemcpyAsync(d_coef, coef.data(), coef.size() * sizeof(double),
                             cudaMemcpyHostToDevice, c->stream) == cudaSuccess &&
             cudaMemcpyAsync(d_he, he_all.data(), he_all.size() * sizeof(double),
                             cudaMemcpyHostToDevice, c->stream) == cudaSuccess &&
             cudaMemcpyAsync(d_toff, toff.data(), toff.size() * sizeof(int),
                             cudaMemcpyHostToDevice, c->stream) == cudaSuccess &&
             cudaMemcpyAsync(d_tiso, tiso.data(), tiso.size() * sizeof(int),
                             cudaMemcpyHostToDevice, c->stream) == cudaSuccess;
    if (!ok) {
        release();
        return MG_ERR_CUDA;
    }
    Basis& B = c->bas[MG_HF_BASIS];
    if (nwt > 0) {
        k_nilsson_eval<<<dim3(nch, nwt), kThreads, 0, c->stream>>>(
            d_terms, d_coef, d_toff, d_tiso, d_he, nfun, npts, p.nx, p.ny, p.nz, V, np->amplitude,
            (unsigned long long)(unsigned)np->seed, B.psi, d_part);
        MG_LAUNCHED(c);
        k_nilsson_norm<<<dim3(div_up(4 * V, kThreads * 8), nwt), kThreads, 0, c->stream>>>(
            d_part, nch, c->dv, 4 * V, B.psi);
        MG_LAUNCHED(c);
    }
    const cudaError_t er = cudaStreamSynchronize(c->stream);
    release();
    if (er != cudaSuccess) return MG_ERR_CUDA;
    MG_TRY(mg_upload_spinors(c, MG_HF_BASIS, nullptr, qn.data(), 0, nwt));
    MG_TRY(mg_set_energies(c, MG_HF_BASIS, en.data()));
    return MG_OK;
}
