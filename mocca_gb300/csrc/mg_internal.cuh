// mg_internal.cuh -- device context and shared helpers of libmocca_gpu.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include <vector>

#include "../../include/mocca_gpu.h"

#define MG_CUDA(call)                                                              \
    do {                                                                           \
        cudaError_t e_ = (call);                                                   \
        if (e_ != cudaSuccess) {                                                   \
            fprintf(stderr, "mocca_gpu: %s failed at %s:%d: %s\n", #call, __FILE__, \
                    __LINE__, cudaGetErrorString(e_));                             \
            return MG_ERR_CUDA;                                                    \
        }                                                                          \
    } while (0)

// After a kernel launch: check the launch and count it (mg_launch_count).
#define MG_LAUNCHED(ctx)                    \
    do {                                    \
        MG_CUDA(cudaGetLastError());        \
        ++(ctx)->launches;                  \
    } while (0)

#define MG_TRY(call)            \
    do {                        \
        int s_ = (call);        \
        if (s_ < 0) return s_;  \
    } while (0)

namespace mg {

constexpr int kMaxN = 64;       // largest supported stored line length
constexpr int kNumMoments = 64; // capacity of the multipole table
constexpr int kMeshTcMax = 80;  // largest spwf block of the tensor-core mesh GEMMs (meshgemm_tc.cu)
constexpr int kEigMax = 160;    // largest matrix of the batched eigensolver (HFB block N = 2h)

// One derivative job: a real grid and where its derivatives go.  slot[d] is
// the Lagrange matrix slot (0 odd, 1 even) along axis d; a NULL output is
// skipped.  lap receives (Lxx + Lyy) + Lzz.
struct GridJob {
    const double* in;
    double* dx;
    double* dy;
    double* dz;
    double* lap;
    int8_t slot[3];
    int8_t pad[5];
};

// Per-basis device state.
struct Basis {
    double* psi = nullptr;   // nwt*4V
    double* der = nullptr;   // nwt*12V : [i][d][l][V]
    double* lap = nullptr;   // nwt*4V
    int* qn = nullptr;       // nwt*4 (device)
    double* occ = nullptr;   // nwt
    double* e = nullptr;     // nwt
    double* disp = nullptr;  // nwt
    GridJob* jobs = nullptr; // 4*nwt derivative jobs
    bool der_df = false;     // der / lap hold double-float {hi, lo} pairs (mixed form)
    std::vector<int> h_qn;
    std::vector<double> h_occ, h_e, h_disp;
    bool have_qn = false;
};

// One FP64 GEMM of a batch: C = alpha op(A) op(B) + beta C (row-major).
struct GemmDesc {
    const double* A;
    const double* B;
    double* C;
    int m, n, k;
    int lda, ldb, ldc;
    int ta, tb;
    double alpha, beta;
    int mat;   // matrix of the batch (for the refinement's early exit)
    int sym;   // C is symmetric: tiles below the diagonal are skipped and mirrored
};
static_assert(sizeof(GemmDesc) == 80, "GemmDesc keeps its 80-byte workspace layout");

// A batch of small symmetric eigenproblems (eig.cu).
struct EigBatch {
    int nb = 0, nmax = 0, ld = 0;
    long stride = 0, wstride = 0;
    const int* nsz = nullptr;
    double* A = nullptr;
    double *X = nullptr, *X2 = nullptr, *AX = nullptr, *S = nullptr, *G = nullptr, *w = nullptr,
           *anorm = nullptr;
    double* part = nullptr;   // nb * ld * 2 row sums of a refinement step
    double* emax = nullptr;   // nb * ld largest opposite-sign angle |S_ij|/|l_i - l_j| per row
    int* done = nullptr;      // nb: first refinement step skipped (INT_MAX: none)
    double* offrel = nullptr; // nb: |S - diag S|_F / |A|_F seen by the last refinement step
    int* pfail = nullptr;     // nb: 1 when the FP64 Jacobi polish hit its sweep cap
    double skip_tol = -1.0;   // skip the remaining steps once offrel <= skip_tol (< 0: never)
    GemmDesc *d_ax = nullptr, *d_sg = nullptr, *d_xf = nullptr, *d_rr = nullptr;
    bool attr_done = false;
    bool have_vectors = false;
};

struct Multigrid;   // multigrid.cu: levels and work vectors of the Coulomb multigrid
struct GradHfb;     // gradient_hfb.cu: U, V and work matrices of the gradient solver

struct PairCoef {
    double cut[2];
    double mu[2];
};

// HFB pairing state.  Blocks b = it*2 + (parity+1)/2 hold h stored spwfs
// (members, in index order) and N = 2h HFB indices (stored, then their
// time-reversed partners).  rho / kappa / delta are N x N per block,
// row-major, padded to nmax.
struct Hfb {
    mg_pairing_params pp{};
    PairCoef pc{};
    bool ready = false;
    bool oldrho_zero = true;
    int hmax = 0, nmax = 0;
    int hsz_h[4] = {0, 0, 0, 0};
    int parity_h[4] = {0, 0, 0, 0};
    std::vector<int> members_h;        // 4*hmax
    int *members = nullptr, *hsz = nullptr, *cstart = nullptr;
    double *rho = nullptr, *kappa = nullptr, *oldrho = nullptr, *oldkappa = nullptr,
           *delta = nullptr, *qe = nullptr;
    double *dfac = nullptr, *pcut = nullptr, *ktil = nullptr, *fpart = nullptr, *fre = nullptr,
           *fim = nullptr, *gpart = nullptr;
    int gchunk = 0;
    double *cantr = nullptr, *occ = nullptr;   // 4*hmax*hmax, 4*hmax
    double* fermi_d = nullptr;                 // 2
    double* trace_d = nullptr;                 // traces, dN/dlambda, refinement size
    double* dpart = nullptr;                   // 4*hmax dN/dlambda row sums
    double* scal_d = nullptr;                  // [energy(2), disp(2)]
    double* h_pinned = nullptr;                // 32 pinned doubles
    double qp_gap[2] = {0.0, 0.0};             // per isospin: smallest 2 min E of its blocks
    double fermi[2] = {-10.0, -10.0};
    double fermi_prev[2] = {-10.0, -10.0};     // Fermi energies of the solve before
    double fermi_old[4][2] = {};               // the four before that ([0] newer)
    double npp[2] = {0.0, 0.0};                // |d2N/dlambda2| from the last two-evaluation search
    int npp_iter = -1000;                      // its iteration
    int n_solved = 0;                          // consecutive converged solves
    long long reseeds = 0;                     // evaluations redone from a Jacobi seed
    bool settled = false;                      // last search: one evaluation + first-order finish
    cudaGraphExec_t eval_graph[3] = {nullptr, nullptr, nullptr};  // per EigSeed
    long long eval_graph_launches[3] = {0, 0, 0};
    int eval_graph_prec[3] = {-1, -1, -1};   // precision form the graph was captured in
    cudaGraphExec_t taylor_graph = nullptr;   // first-order finish of the Fermi search
    long long taylor_graph_launches = 0;
    int taylor_graph_prec = -1;
    double* dl_d = nullptr;                   // its steps per isospin
    double *oldrho_bak = nullptr, *oldkappa_bak = nullptr;   // mixing history before the last mix
    cudaGraphExec_t can_graph[2] = {nullptr, nullptr};   // canonical-basis decomposition:
    long long can_graph_launches[2] = {0, 0};            // [0] Jacobi warm seed,
    int can_graph_prec[2] = {-1, -1};                    // [1] in-place refinement
    bool no_graph = false;
    bool fermi_hist[7] = {false, false, false, false, false, false, false};
    double epair[2] = {0.0, 0.0}, disp[2] = {0.0, 0.0};
    double* T = nullptr;      // 4 block HFB matrices (signature-reduced), nmax x nmax
    double* Rpp = nullptr;    // 4 blocks of rho_++, hmax x hmax
    int* nsz_T = nullptr;     // N per block
    EigBatch eT, eR;          // eigensolver batches for T and rho_++
    // first-order finish of the Fermi search (hfb.cu): h x h workspaces per
    // block (ld hmax) and the GEMM tables of d rho / d lambda, d kappa / d lambda
    double *tP = nullptr, *tC = nullptr, *tT1 = nullptr, *tT2 = nullptr, *tZ = nullptr,
           *tK = nullptr;
    GemmDesc* d_taylor = nullptr;    // 4 + 8 + 8 + 4 descriptors
    long long taylor_steps = 0;      // pairing steps finished by the expansion
    int nref = 2;             // FP64 refinement steps per eigen-decomposition
    GradHfb* grad = nullptr;  // fermi_solver 2 (gradient_hfb.cu)
    // RhoHFB / KappaHFB of a wavefunction file (wf_ctx.cu), N x N per block,
    // taken by hfb_prepare in place of the kappa guess
    bool restart_pending = false;
    int restart_n[4] = {0, 0, 0, 0};
    std::vector<double> restart_rho[4], restart_kappa[4];
};

// One multipole constraint of the alternating kind (constraints.cu): the
// fields of the reference's Moment type that it uses.
struct MomentConstraint {
    int l = 0, m = 0;
    int type = 2;               // 2 alternating, 0 switched off
    int iteration = -1;         // last Evolve iteration with the constraint (<= 0: all)
    double constraint = 0.0;    // running target of the constraint field
    double true_constraint = 0.0;
    double intensity = 0.0;     // 0: estimated on the first readjustment
    double value[2] = {0.0, 0.0}, squared[2] = {0.0, 0.0};
    double old_value[7] = {0, 0, 0, 0, 0, 0, 0};   // sums of OldValue(:, 1..7)
    double old_iso[7][2] = {};  // OldValue(it, 1..7) per isospin (the wavefunction file's)
    bool started = false;       // moments computed once (running target set)
};

constexpr int kMaxConstraints = 8;

struct Constraints {
    std::vector<MomentConstraint> list;
    double* sh = nullptr;       // [kMaxConstraints][V] r^l Y_lm on the stored mesh
    double* cut = nullptr;      // [2][V] density cutoff
    double* field = nullptr;    // [2][V] constraint field added to U
    double* surf = nullptr;     // [2][3][cap] surface points of the cutoff
    long cap = 0;
    double* stat = nullptr;     // [2][2]: threshold, dv * sum rho
    int* count = nullptr;       // [2] surface points found
    double* red = nullptr;      // [kMaxConstraints][4]: value[2], squared[2]
    double* h_red = nullptr;    // pinned host copy of red
    bool alternate_check = false;
};

}  // namespace mg

struct mg_ctx {
    mg_params p;
    mg_force f;
    mg_skyrme_b B;
    int nx, ny, nz;
    long V;
    double dv;
    bool folded;
    int device = 0;                     // CUDA device current at mg_create
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    cudaStream_t side = nullptr;        // low-priority stream for overlapped work
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    int num_sms = 0;

    // Lagrange matrices: [axis][kind: 0 first, 1 second][slot][q*n+i]
    // (stored transposed so consecutive output points read consecutive words)
    double* mats = nullptr;
    long mat_off[3][2][2];
    float* mats32 = nullptr;      // double-float copy: hi, lo planes [q][round4(n)] per matrix
    long mat32_off[3][2][2];
    int cur_precision = MG_FP64;  // precision of the next kernels (MG_FP64 / MG_MIXED)
    // digit planes of the Lagrange blocks for the tensor-core derivatives
    // (deriv_tc.cu): [axis][slot] blocks of 6 planes x N rows x 32, bf16
    uint16_t* tcmats = nullptr;
    int* tc_erow = nullptr;       // [axis][slot][64] row exponents
    int* tc_status = nullptr;     // set when an MMA completion wait ran out
    long tc_off[3][2];
    int tc_N[3] = {0, 0, 0};
    bool tc_ok = false;           // every line length <= 32
    bool tc_mesh_ok = false;      // mesh-sized GEMMs on the tensor cores (blocks <= kMeshTcMax)
    int tc_kp = 32;               // padded K of the tensor-core derivative planes (32 or 48)
    int* h_tc_status = nullptr;   // pinned copy of tc_status, read with the energy's sync
    // largest grid of the persistent tensor-core derivative kernel (0: one CTA
    // per SM); set while it runs beside other work on the side stream
    int tc_grid_cap = 0;

    // z planes per block of the Lagrange x/y kernels, [0 FP64, 1 double-float]
    // x [0 few grids, 1 whole bases]; 0 until deriv.cu's autotuner picks one
    int deriv_planes[2][2] = {{0, 0}, {0, 0}};

    mg::Basis bas[2];
    double* updates = nullptr;   // nwt*4V heavy-ball history
    double* hbuf = nullptr;      // nwt*4V h.psi scratch

    // densities [it][...][V]
    double *rho = nullptr, *tau = nullptr, *nablaj = nullptr, *derrho = nullptr,
           *laprho = nullptr;
    // potentials
    double *U = nullptr, *Bp = nullptr, *nablaB = nullptr, *W = nullptr, *divW = nullptr;
    double* divw_tmp = nullptr;   // 3 * 6V
    float2* fields_df = nullptr;  // mixed h.psi: the isospins' fields as double-float (2 x 17V)
    mg::GridJob* field_jobs = nullptr;  // rho derivs (2), B derivs (2), divW (18)
    int n_field_jobs = 0;

    // Gram-Schmidt scratch
    double* gs_S = nullptr;       // overlap blocks
    double* gs_R = nullptr;       // inverse Cholesky factors
    int* gs_index = nullptr;      // block lists + energy-ordered members
    int gs_nblk = 0, gs_nbmax = 0, gs_nchunk = 0, gs_lists_len = 0;
    // tensor-core form (meshgemm_tc.cu): overlap partials per 256-point chunk, digit
    // planes and row exponents of X = R^{-1}
    double* gs_Stc = nullptr;
    uint16_t* gs_xd = nullptr;
    int* gs_xe = nullptr;
    int gs_nchunk_tc = 0;
    uint16_t* can_xd = nullptr;   // digit planes of CanTransfo (tensor-core canonical basis)
    int* can_xe = nullptr;
    double* gap_part = nullptr;   // tensor-core gaps: partials per 64-point chunk
    double* field_y = nullptr;    // tensor-core pairing field: Y = Psi Ktilde per block (4 hmax x 4V)
    uint16_t* field_xd = nullptr;
    int* field_xe = nullptr;
    int* field_ybase = nullptr;   // first row of each block in field_y

    // Coulomb
    int mx, my, mz;
    long M = 0;
    double *cpot = nullptr, *csource = nullptr, *cres = nullptr, *cp = nullptr,
           *ct = nullptr, *rext = nullptr, *sh_ext = nullptr, *sh_mesh = nullptr,
           *coulomb = nullptr, *coulex = nullptr;
    int n_moments = 0, n_bc_moments = 0;
    int h_moment_l[mg::kNumMoments];
    double* moment_values = nullptr;   // [n_moments][2]
    double* rpow_ext = nullptr;        // r^(2l+1) on the extended box per moment
    double* mfac = nullptr;            // 4 pi / (2l+1) per moment
    unsigned* cg_bar = nullptr;        // grid barrier state of the CG kernel
    int* cg_status = nullptr;          // [state, iterations]
    int* h_cg_status = nullptr;        // pinned host copy
    int cg_blocks = 0;
    double* red = nullptr;             // reduction scratch
    size_t red_len = 0;
    int* flags = nullptr;              // device status flags
    bool coulomb_init = false;
    mg::Multigrid* mgrid = nullptr;    // CoulombSolver = 2 (multigrid.cu)
    double* cguess = nullptr;          // InitialGuess on the extended box (M)
    double* cfast = nullptr;           // 1-D eigenvectors and eigenvalues of the direct solve
    long cfast_off[3][2];              // [axis][0: C (n x n), 1: mu (n)]

    // mixing between iterations (mixing.cu)
    double* dhist = nullptr;           // previous densities: rho, tau, nablaj, derrho, laprho (14V)
    // the tensor density J_{mu nu} [it][nu][mu][V] and its history, when any
    // of B14..B17 is not zero (time reversal conserved)
    bool tensor = false;
    double *jmunu = nullptr, *jmunu_hist = nullptr;
    bool have_dhist = false;
    double* Uold = nullptr;            // UpotOld (2V)
    double* Sold = nullptr;            // SpotOld without time reversal (6V)
    double* Wold = nullptr;            // WpotOld with PreConW > 0 (18V)
    // time-odd densities and fields without time reversal (timeodd.cu):
    // odd = [vecj 6V, vecs 6V, rot j 6V, rot s 6V] ([it][m][V] each), its
    // history for the mixing, A and S ([it][m][V]), div A ([it][V]), the
    // derivative scratch of the curls (36V) and of div A (6V), 18 jobs
    double *odd = nullptr, *odd_hist = nullptr, *Apot = nullptr, *Spot = nullptr,
           *divA = nullptr, *odd_der = nullptr, *odd_tmp = nullptr;
    mg::GridJob* odd_jobs = nullptr;
    // the time-odd tensor terms (tensor_odd.cu), when B14..B21 are not all
    // zero: odd grows to 48V with [T, F, lap s, grad div s] behind the
    // curls (odd_len = 48, else 24, in units of V); the C and D fields
    // ([it][m][V]), d_n D_m ([it][m][n][V]), div D ([it][V]), the d_z s_z
    // scratch (2V), 16 fixed jobs; the h.psi scratch (60V per spwf), its
    // job table (device, and the last upload's bytes on the host) and the
    // C and D actions of the basis ([i][2][l][V])
    bool todd = false;
    int odd_len = 24;
    double *Cpot = nullptr, *Dpot = nullptr, *dDpot = nullptr, *divD = nullptr,
           *todd_tmp = nullptr, *todd_work = nullptr, *todd_x = nullptr;
    mg::GridJob* todd_jobs = nullptr;
    mg::GridJob* todd_act_jobs = nullptr;
    std::vector<unsigned char> todd_jobs_host;
    bool have_uold = false;            // UpotOld not all zero
    double* pc_buf = nullptr;          // preconditioner CG: res, dir, upd, lap, inv (10V)
    mg::GridJob* pc_jobs = nullptr;    // Laplacians of the two directions

    double pairing_energy[2] = {0.0, 0.0};
    long long launches = 0;
    bool side_derive_pending = false;  // mg_iterate: the pairing step forks the HF DeriveAll
    cudaGraphExec_t cfast_graph = nullptr;   // the direct Coulomb solve's two rounds
    long long cfast_graph_launches = 0;
    bool cfast_no_graph = false;

    // phase timer (mg_set_phase_timing): events between the phases of the
    // pass in progress, their phase ids, and the totals
    struct PhaseTimer {
        static constexpr int kMarks = 24;
        bool on = false;
        int n = 0;                          // marks of the pass in progress, 0: none
        cudaEvent_t ev[kMarks] = {};
        int id[kMarks] = {};
        cudaEvent_t side[2] = {};           // side-stream DeriveAll start, end
        bool side_used = false;
        double ms[MG_PH_COUNT] = {};
        long long passes = 0;
    } ph;

    // IterativeEstimation (est.cu): the probe spinor maxspwf with its
    // derivatives and update, its derivative jobs and quantum numbers, and the
    // dt / momentum in use
    double* est = nullptr;              // psi 4V, der 12V, lap 4V, hpsi 4V, update 4V, (e, disp)
    mg::GridJob* est_jobs = nullptr;
    int* est_qn = nullptr;
    int est_h_qn[4] = {0, 0, 0, 0};   // the probe's quantum numbers on the host
    int est_iter = 0;
    bool step_set = false;
    double step_dt = 0.0, step_mom = 0.0;

    mg::Hfb hfb;

    // multipole constraints (constraints.cu) and the Evolve iteration count
    mg::Constraints cons;
    int iteration = 0;

    // ConvergenceCheck histories: OldEnergy(7) and the last TotalEnergy
    // (src/Energy.f90:34, :93-98)
    double old_energy[7] = {0, 0, 0, 0, 0, 0, 0};
    double total_energy = 0.0;
};

namespace mg {

int upload_matrices(mg_ctx* c);
int build_basis_jobs(mg_ctx* c, int b);
int build_field_jobs(mg_ctx* c);
int run_jobs(mg_ctx* c, const GridJob* jobs, int njobs, bool out_df = false);
int derive_basis(mg_ctx* c, int b);
int tc_setup(mg_ctx* c);
int run_jobs_tc(mg_ctx* c, const GridJob* jobs, int njobs);
int tc_check(mg_ctx* c);
// tc_check in two halves: enqueue the status copy, read it after a later sync
int tc_status_async(mg_ctx* c);
int tc_status_result(mg_ctx* c);

int hpsi_basis(mg_ctx* c, int b, double* out, bool grad_step, double fac, double mom);
int hpsi_single(mg_ctx* c, double* psi, const double* der, const double* lap, const int* qn_dev,
                double* out, double* e_dev);
int estimate_parameters(mg_ctx* c);
int gram_schmidt(mg_ctx* c);
int gram_schmidt_impl(mg_ctx* c, double* upd);
bool gs_tc_prepare(mg_ctx* c);
int gs_overlap_tc(mg_ctx* c, const double* psi, const int* d_lists, const int* d_ordered);
int gs_apply_tc(mg_ctx* c, double* psi, double* upd, const int* d_lists, const int* d_ordered);
int can_transform_tc(mg_ctx* c);
int gaps_tc(mg_ctx* c, double* gsum);
int pair_field_tc(mg_ctx* c);
int densities(mg_ctx* c);
int moments(mg_ctx* c);
int coulomb_setup(mg_ctx* c);
int coulomb_solve(mg_ctx* c, int* iters);
int coulomb_residual(mg_ctx* c, double* rel);
int coulomb_reset(mg_ctx* c);
int coulomb_multigrid(mg_ctx* c, double tol, int maxit, int* iters);
void multigrid_free(Multigrid* M);
int multigrid_levels(const mg_ctx* c);
int potentials(mg_ctx* c);
int energy(mg_ctx* c, mg_energy_terms* out);
int basis_dots(mg_ctx* c, const double* a, const double* b, double* out, bool b_df = false);
int pairing_mesh(mg_ctx* c);
int canonical_transform(mg_ctx* c);
int pairing_set_smem(mg_ctx* c);
int eig_setup(mg_ctx* c, EigBatch& E, int nb, int nmax, const int* nsz_dev, double* A,
              long stride, int ld);
// Seeds of eig_batched: FP32 Jacobi from scratch, FP32 Jacobi on X^T A X of
// the vectors in E.X, or refinement started directly from E.X.
enum EigSeed { kSeedCold = 0, kSeedJacobiWarm = 1, kSeedRefine = 2 };
int eig_batched(mg_ctx* c, EigBatch& E, int seed, int nref, bool polish);
int gemm_batched(mg_ctx* c, const GemmDesc* descs, int ndesc, int maxdim, bool df = false);
int gemm_batched_skip(mg_ctx* c, const GemmDesc* descs, int ndesc, int maxdim, int* done);
int hfb_evaluate_at(mg_ctx* c, const double* lam, double* N_out, double* dN_out);
int fermi_gradient(mg_ctx* c, double lam[2], double f[2], bool conv[2], int* iters);
void gradient_hfb_free(GradHfb* g);
int eig_jacobi_fp64(mg_ctx* c, EigBatch& E);
void eig_free(EigBatch& E);
int hfb_prepare(mg_ctx* c);
int hfb_solve(mg_ctx* c, mg_pairing_info* info);
// phase timer: open a pass, mark the end of phase id on the stream, close
// the pass (waits for its last event and adds up the intervals)
int phase_begin(mg_ctx* c);
int side_derive_hf(mg_ctx* c);
void phase_mark(mg_ctx* c, int id);
int phase_end(mg_ctx* c);
void hfb_free(mg_ctx* c);
int density_groups(const mg_ctx* c);
int time_odd_setup(mg_ctx* c);
int time_odd_densities(mg_ctx* c, const Basis& D);
int time_odd_potentials(mg_ctx* c);
int time_odd_energy(mg_ctx* c, double* t);
int tensor_odd_setup(mg_ctx* c);
int tensor_odd_densities(mg_ctx* c, const Basis& D);
int tensor_odd_fields(mg_ctx* c);
int tensor_odd_action(mg_ctx* c, const double* der, const int* h_qn, const int* d_qn, int count,
                      double* x);
int tensor_odd_energy(mg_ctx* c, double* t);
int cranking_cutoff(mg_ctx* c);
inline bool cranking(const mg_ctx* c) {
    return c->p.omega[0] != 0.0 || c->p.omega[1] != 0.0 || c->p.omega[2] != 0.0;
}
int mixing_setup(mg_ctx* c);
int save_density_history(mg_ctx* c);
int mix_densities(mg_ctx* c);
int precondition_u(mg_ctx* c);
double rlylm(int l, int m, int im, double X, double Y, double Z);
int add_constraint(mg_ctx* c, const mg_moment_constraint* mc);
int constraint_moments(mg_ctx* c);
int alternate_step(mg_ctx* c);
void readjust_moments(mg_ctx* c, int iteration);
bool any_alternating(const mg_ctx* c);
bool moments_converged(const mg_ctx* c, double prec);
void constraints_free(mg_ctx* c);

// Lagrange matrix slot selection of Opt_LAG{X,Y,Z}_EV8 / Lapla_LAG_EV8.
__host__ __device__ inline int lag_slot(int dir, int P, int S, int TS, int comp) {
    int s;
    if (dir == 0) s = (comp == 1 || comp == 4) ? S * TS : -S * TS;
    else if (dir == 1) s = (comp == 1 || comp == 3) ? TS : -TS;
    else s = (comp == 1 || comp == 2) ? S * P : -S * P;
    return s > 0 ? 1 : 0;
}

inline int div_up(long a, long b) { return (int)((a + b - 1) / b); }

}  // namespace mg
