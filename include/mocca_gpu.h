/*
 * mocca_gpu.h -- C ABI of the GB300 (sm_103a) implementation of the MOCCa
 * per-iteration mesh hot path.
 *
 * Every entry point is `extern "C"`, takes plain pointers, sizes and opaque
 * handles, and returns an int status (MG_OK = 0, > 0 non-convergence, < 0
 * error).  A Fortran host binds them with `interface ... bind(C)` blocks; the
 * status replaces the reference's `stp()` call, which the shim raises on a
 * non-zero status.
 *
 * Data conventions (identical to the reference's Fortran memory order):
 *   - one real grid is (nx,ny,nz) with x fastest: g[x + nx*(y + ny*z)];
 *   - one spinor is Grid(nx,ny,nz,4): component c (0..3 = Re up, Im up,
 *     Re down, Im down) at offset c*V, V = nx*ny*nz
 *     (src/Spinor.f90:6-19, src/Spinor.f90:69);
 *   - isospin index it = 0 for neutrons (isospin -1), 1 for protons (+1)
 *     (the reference's it = (isospin+3)/2 minus one);
 *   - vector fields F(nx,ny,nz,3,2) are [it][k][V]; tensor fields
 *     W(nx,ny,nz,3,3,2) are [it][n][m][V] (m fastest), matching
 *     src/MeanFields.f90:79-85.
 *
 * Threading: one context per host thread; calls on a context are
 * stream-ordered on the context's stream and not re-entrant.
 */
#ifndef MOCCA_GPU_H
#define MOCCA_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------- */
#define MG_OK               0
#define MG_NOT_CONVERGED    1   /* iterative solver hit its cap           */
#define MG_ERR_ARG         -1   /* invalid argument / unsupported mode    */
#define MG_ERR_CUDA        -2   /* CUDA runtime error                     */
#define MG_ERR_STATE       -3   /* call out of order (e.g. no spinors)    */
#define MG_ERR_TIMEOUT     -4   /* a device-side wait ran out of its cap  */
#define MG_ERR_NAN         -5   /* NaN detected (reference: x .eq. x+1)   */

/* ---- precision modes ----------------------------------------------------- */
#define MG_FP64   0   /* plain path: every kernel in FP64                 */
#define MG_MIXED  1   /* tensor-core digit GEMMs, double-float mesh work  */

/* ---- bases --------------------------------------------------------------- */
#define MG_HF_BASIS   0   /* HFBasis(:), src/SpwfStorage.f90:27            */
#define MG_CAN_BASIS  1   /* CanBasis(:), src/SpwfStorage.f90:31           */

/* ---- pairing types (src/Pairing.f90:33-37) ------------------------------- */
#define MG_PAIRING_HF   0
#define MG_PAIRING_HFB  2

typedef struct mg_ctx mg_ctx;   /* opaque device context */

/*
 * Run parameters: the &GenInfo / &SpwfStorage / &Coulomb namelist values the
 * hot path needs (src/GenInfo.f90:302-378, src/Coulomb.f90:120-150).
 * nx,ny,nz are the STORED point counts.  Supported symmetry modes:
 *   pc=sc=tsc=1 (EV8, folded Lagrange matrices, src/OptimizedDerivatives.f90)
 *   pc=sc=tsc=0 (full box, unfolded Lagrange matrices,
 *                src/Derivatives.f90:1080-1217 with zero line extension).
 */
typedef struct mg_params {
    int    nx, ny, nz;
    double dx;                 /* fm */
    int    pc, sc, tsc, trc;   /* parity, signature, time simplex, time reversal conserved */
    int    nwt;                /* number of stored spwfs per basis */
    double neutrons, protons;
    int    precision;          /* MG_FP64 or MG_MIXED */
    int    pairing;            /* MG_PAIRING_HF or MG_PAIRING_HFB */
    int    coulomb_max;        /* CoulombMax, default 500 (src/Coulomb.f90:24) */
    int    max_l_coul;         /* MaxLCoul, default MaxMoment = 10 */
    int    coulomb_solver;     /* CoulombSolver: 0 none, 1 CG (reference default; the mixed
                                  form solves directly instead), 2 multigrid: FP32 V-cycles
                                  preconditioning an FP64 conjugate-gradient iteration
                                  (src/MultiGrid.f90:14-348) */
    int    mixing_scheme;      /* MixingScheme (src/DensityMixing.f90:22-86): 0 linear
                                  density mixing (reference default), 2 preconditioned
                                  U update (src/PotentialMixing.f90:143-154) */
    double damping;            /* DampingParam, 0.75 (src/Densities.f90:17) */
    double precon_u;           /* preconu, 1.0 (src/Densities.f90:34) */
    int    parameter_estimation; /* ParameterEstimation (src/GenInfo.f90:72): 1 re-estimates
                                    dt and the momentum at every GradDesc
                                    (IterativeEstimation, src/ImaginaryTime.f90:28-211) */
    double coulomb_prec;       /* > 0: the CG and multigrid solves stop at |b - L phi| <=
                                  coulomb_prec |b| on the stored box; 0: the reference's CG
                                  test |r|^2 <= 1e-9 / (dx^3 V) (src/Coulomb.f90:755-900), and
                                  1e-10 relative for the multigrid */
    double omega[3];           /* cranking frequencies OmegaX, OmegaY, OmegaZ (CrankType 0,
                                  fixed; src/Cranking.f90:24-60); nonzero only with trc = 0,
                                  and with EV8 symmetry only OmegaZ (the reference stops on
                                  OmegaX with signature and OmegaY with time simplex) */
    double precon_w;           /* PreConW, 0 (src/Densities.f90:37): > 0 also preconditions
                                  the update of each W component under MixingScheme 2
                                  (src/PotentialMixing.f90:169-210), with alpha = -preconu
                                  like U (the reference's own PreConW alpha is commented out) */
} mg_params;

/*
 * Skyrme parameters as read from a forces.param &skf group
 * (src/Force.f90:188-255).  hbm is hbar^2/m, i.e. already doubled as in
 * src/Force.f90:246 (41.4710382 for the default 20.73551910).
 * nucleonmass is used as given (pass the averaged mass when averagemass).
 */
typedef struct mg_force {
    double t0, x0, t1, x1, t2, x2, t3a, x3a, yt3a, t3b, x3b, yt3b, te, to;
    double wso, wsoq;
    double hbm, e2, hbar;
    double nucleonmass[2];
    int    com1body, com2body, cexchange;
    int    j2terms;      /* J2Terms: the central J^2 terms of t1, t2 and the tensor
                            te, to in B14, B15 (B16, B17 follow te, to always) */
    int    coupling;     /* CalcEDFCoef's overrides of B14..B17 by force name
                            (src/Force.f90:552-597): 0 none, MG_COUPLING_* */
} mg_force;

#define MG_COUPLING_SLY4T    1   /* "SLy4T":    B14 = 15, B15 = -120, B16 = B17 = 0 */
#define MG_COUPLING_SLY4TMIN 2   /* "SLy4Tmin": the same values                     */
#define MG_COUPLING_UNEDF2   3   /* "UNEDF2":   B14 = -54.43... + 65.90..., B15 = -2 x 65.90... */

/* The B-coefficients of the energy density (src/Force.f90:467-560).
 * B18, B19 (J2Terms) and B20, B21 (te, to) are time-odd: zero with time
 * reversal. */
typedef struct mg_skyrme_b {
    double B1, B2, B3, B4, B5, B6, B7a, B7b, B8a, B8b, byt3a, byt3b, B9, B9q;
    double B10, B11, B12a, B12b, B13a, B13b, B14, B15, B16, B17;
    double B18, B19, B20, B21;
} mg_skyrme_b;

/* Energy decomposition of CompEnergy (src/Energy.f90:62-179). */
typedef struct mg_energy_terms {
    double total;            /* TotalEnergy                                  */
    double kinetic[2];       /* Kinetic(it), src/Energy.f90:1426-1456        */
    double skyrme[36];       /* SkyrmeTerms, term by term, already times dv  */
    double coulomb;          /* CompCoulombEnergy, src/Coulomb.f90:215-231   */
    double coulomb_exchange; /* Slater exchange energy                       */
    double com[2][2];        /* COMCorrection(body, it)                      */
    double pairing[2];       /* PairingEnergy(it)                            */
    double sp_energy;        /* SpwfEnergy, src/Energy.f90:1483-1554         */
} mg_energy_terms;

/* HFB pairing parameters: the &Pairing namelist values of the HFB path
 * (src/Pairing.f90:164-305, src/PairingInteraction.f90:19-94,
 * src/HFB.f90:86).  Density-dependent delta pairing ("ULB",
 * DensityFactor = -G (1 - alpha rho0/rhosat)), symmetric-Fermi cutoffs. */
typedef struct mg_pairing_params {
    double strength[2];   /* PairingNeutron / PairingProton (MeV fm^3)     */
    double alpha[2];      /* AlphaNeutron / AlphaProton                     */
    double rhosat;        /* RhoSat, 0.16 fm^-3                             */
    double cut[2];        /* PairingCut, 5 MeV                              */
    double mu[2];         /* PairingMu, 0.5 MeV                             */
    double mix;           /* HFBMix, 0.1                                    */
    double fermi_prec;    /* FermiPrec, 1e-12                               */
    int    max_iter;      /* HFBIter, 50                                    */
    int    guess_kappa;   /* GuessKappa                                     */
    double fermi_start[2];/* initial Fermi energies (module default -10)    */
    int    fermi_solver;  /* 0: Newton with the analytic dN/dlambda (this    */
                          /* library's default); 1: the reference's damped   */
                          /* Broyden search (HFBFindFermiEnergyBroyden,      */
                          /* src/HFB.f90:1849-2161), iterate for iterate;    */
                          /* 2: the gradient solver (FermiSolver 'GRADIENT', */
                          /* HFBFermiGradient src/GradientHFB.f90:473-733),  */
                          /* max_iter gradient steps at most (the reference  */
                          /* defaults HFBIter to 500 for it); its first U, V */
                          /* come from one diagonalisation at fermi_start;   */
                          /* 3: FermiSolver 'BISECTION' (bracketing and      */
                          /* Brent's method, HFBFindFermiEnergyBisection and */
                          /* FermiBrent, src/HFB.f90:1074-1342, 2273-2487),  */
                          /* fermi_prec the tolerance on lambda              */
} mg_pairing_params;

/* Per-call diagnostics of the HFB pairing step. */
typedef struct mg_pairing_info {
    double fermi[2];          /* converged Fermi energies                   */
    double particles[2];      /* Tr rho per isospin at the converged Fermi  */
    int    evaluations;       /* particle-number evaluations used           */
    int    converged;         /* 1 when |N - N0| < FermiPrec for both       */
    double pairing_energy[2]; /* HFBEnergy with the new kappa               */
    double dispersion[2];     /* PairingDisp                                */
    int    first_order;       /* 1 when rho and kappa took the last Newton  */
                              /* step to first order (no new evaluation)    */
} mg_pairing_info;

/* ---- host-side helpers (no device work) ---------------------------------- */

/* B-coefficients from Skyrme parameters; replaces CalcEDFCoef
 * (src/Force.f90:467-560) up to B17 (the name-based overrides of SLy4T,
 * SLy4Tmin and UNEDF2 aside). */
int mg_skyrme_coefficients(const mg_force* f, int trc, mg_skyrme_b* out);

/* Lagrange derivative matrices for one axis; replaces IniLag + reduceLag
 * (src/Derivatives.f90:899-1078).  folded=1: the EV8 matrices LagXMat /
 * LagXXMat for a stored half-line of n points (full line 2n); out arrays are
 * [s][i][j] row-major, s=0 the odd extension (Fortran index 1), s=1 the even
 * one (index 2).  folded=0: the full-line matrices of DerLag_1D /
 * SecondDerLag with zero extension (src/Derivatives.f90:1177-1312), written
 * to both s slots. */
int mg_lagrange_matrices(int n, double dx, int folded, double* d1, double* d2);

/* Batched symmetric eigensolver used by the HFB step (replaces diagoncr8,
 * src/HFB.f90:5880-6087): nb <= 64 matrices of sizes n[b] <= ld <= 160, row-major with
 * leading dimension ld and stride ld*ld in a (host arrays); w receives the
 * eigenvalues ascending (stride ld), z the eigenvectors (column k <-> w[k]).
 * Runs on the current CUDA device; FP64-accurate (FP32 Jacobi seed, FP64
 * refinement, FP64 Jacobi polish inside clusters).  Returns MG_NOT_CONVERGED
 * (results written) when the polish of some matrix reached its sweep cap. */
int mg_eigh_batched(int nb, const int* n, int ld, const double* a, double* w, double* z);

/* mg_eigh_batched for callers that must not allocate device memory: a host
 * that owns every byte of the device through its own pool allocator (a
 * solver framework, an embedding application with a fixed budget) cannot
 * let a library call cudaMalloc behind its back.  No reference counterpart:
 * the Fortran code has no device.
 * n: host array; a, w, z: DEVICE buffers laid out as for mg_eigh_batched;
 * info: DEVICE array of nb ints or NULL, receiving 1 for a matrix whose FP64
 * Jacobi polish reached its sweep cap (results still written) and 0
 * otherwise; stream: a cudaStream_t (NULL: the legacy default stream).  Work
 * is only enqueued on `stream`; the caller synchronises before reading w, z
 * and info.  The workspace is one static device array of ~2.2 MiB per
 * device, so the limits are nb <= 64, ld <= 128 and nb*ld*ld <= 65536
 * (MG_ERR_ARG with a message on stderr beyond that).  z outside each leading
 * n x n block is set to zero, w beyond n[b] is not written.  The first call
 * on a device (that device current) looks up the workspace address and loads
 * the kernels; make it before any stream capture.  Calls share the
 * workspace: two calls that can overlap on one device (different streams,
 * host threads) race. */
int mg_eigh_batched_noalloc(int nb, const int* n, int ld, const double* a, double* w,
                            double* z, int* info, void* stream);

/* ---- context --------------------------------------------------------------- */

/* Allocates every device buffer of the hot path (spinors of both bases and
 * their derivatives, densities, fields, Coulomb box, HFB matrices) and builds
 * the Lagrange matrices; replaces the setup done by ReadDerivativesInfo,
 * SetupCoulomb and IniMoments.  stream: a cudaStream_t or NULL (a private
 * stream is created). */
int mg_create(const mg_params* p, const mg_force* f, void* stream, mg_ctx** out);
int mg_destroy(mg_ctx* ctx);
int mg_synchronize(mg_ctx* ctx);
/* Precision of the following calls (MG_FP64 or MG_MIXED), e.g. an FP64
 * polish after mixed-precision iterations.  MG_MIXED runs the Lagrange
 * derivative contractions, the Gram-Schmidt overlap and apply, the pairing
 * gaps and the canonical-basis transform as exact BF16 digit products on the
 * tensor cores (47-bit operands), and h.psi, the densities and the pairing
 * field in double-float (FP32 pairs), with FP64 storage, and the small
 * GEMMs and Jacobi polish of the HFB diagonalisation in double-float; the
 * Cholesky factor, energies and the HFB matrices stay FP64.
 * No reference counterpart (the reference is FP64 throughout). */
int mg_set_precision(mg_ctx* ctx, int precision);

/* ---- spinor transfer ------------------------------------------------------- */

/* grids[i] points at one Fortran Grid(nx,ny,nz,4) (4V doubles) for spwf
 * first+i; qn[4*i..] = (isospin, parity, signature, time simplex) as in
 * src/Spwf.f90:63-85.  qn may be NULL on later uploads to keep the numbers. */
int mg_upload_spinors(mg_ctx* ctx, int basis, const double* const* grids,
                      const int* qn, int first, int count);
int mg_download_spinors(mg_ctx* ctx, int basis, double* const* grids,
                        int first, int count);
/* der[i] receives Der(1:3) of spwf first+i as 3 consecutive spinors (12V
 * doubles), lap[i] the Laplacian (4V); either may be NULL. */
int mg_download_derivatives(mg_ctx* ctx, int basis, double* const* der,
                            double* const* lap, int first, int count);

/* Occupations / single-particle energies of a basis (Spwf%Occupation,
 * Spwf%Energy).  Arrays of nwt doubles. */
int mg_set_occupations(mg_ctx* ctx, int basis, const double* occ);
int mg_get_occupations(mg_ctx* ctx, int basis, double* occ);
int mg_set_energies(mg_ctx* ctx, int basis, const double* e);
int mg_get_energies(mg_ctx* ctx, int basis, double* e, double* disp);

/* ---- compute entry points --------------------------------------------------- */

/* Der(1:3) and Lap of every spwf of one basis; replaces CompDer over the
 * basis (src/Spwf.f90:778-792 via DeriveSpinor / LapSpinor with the Lagrange
 * kernels of src/OptimizedDerivatives.f90:115-615). */
int mg_derive_basis(mg_ctx* ctx, int basis);
/* DeriveAll (src/SpwfStorage.f90:586-604): HFBasis, and CanBasis under HFB. */
int mg_derive_all(mg_ctx* ctx);

/* h.psi for every spwf of a basis from the current fields; replaces hPsi
 * (src/ImaginaryTime.f90:213-304).  hpsi (nwt*4V, may be NULL) receives the
 * spinors, e[i] = <psi|h psi> and disp[i] = <h psi|h psi> - e^2 (may be NULL). */
int mg_hpsi(mg_ctx* ctx, int basis, double* hpsi, double* e, double* disp);

/* One GradDesc step on the HF basis (src/ImaginaryTime.f90:439-500), with
 * its Gram-Schmidt; dt in 1e-22 s as in &GenInfo. */
int mg_grad_desc(mg_ctx* ctx, double dt, double momentum);
/* dt and momentum in use: the GradDesc arguments, or with
 * parameter_estimation = 1 the values of the last IterativeEstimation (the
 * first GradDesc's arguments seed it). */
int mg_get_step_parameters(mg_ctx* ctx, double* dt, double* momentum);

/* Energy-ordered Gram-Schmidt of the HF basis (src/SpwfStorage.f90:372-480). */
int mg_gram_schmidt(mg_ctx* ctx);

/* Naive HF filling by energy (src/HartreeFock.f90:177-260). */
int mg_hf_fill(mg_ctx* ctx);

/* ComputeDensity over the density basis (src/Densities.f90:431-550):
 * rho, tau, div J, grad rho, lap rho. */
int mg_update_densities(mg_ctx* ctx);
/* MixDensities (src/DensityMixing.f90:22-86) after mg_update_densities:
 * scheme 0 mixes every density with the previous iteration's,
 * rho <- (1 - damping) rho + damping rho_previous; scheme 2 does nothing here
 * (mg_construct_potentials preconditions the U update instead).
 * mg_update_densities keeps the densities it replaces as that history. */
int mg_mix_densities(mg_ctx* ctx);
/* Arrays of 2V (rho,tau,nablaj,laprho) and 6V (derrho); any may be NULL. */
int mg_get_densities(mg_ctx* ctx, double* rho, double* tau, double* nablaj,
                     double* derrho, double* laprho);
int mg_set_densities(mg_ctx* ctx, const double* rho, const double* tau,
                     const double* nablaj, const double* derrho,
                     const double* laprho);
/* The tensor density J_{mu nu} (src/Densities.f90:148, GetJMuNu
 * src/Spwf.f90:2186-2204), 18V as [it][nu][mu][V]; only with J^2 terms
 * (B14..B17 not all zero), MG_ERR_ARG otherwise. */
int mg_get_jmunu(mg_ctx* ctx, double* jmunu);
int mg_set_jmunu(mg_ctx* ctx, const double* jmunu);

/* HFB pairing parameters (before the first mg_solve_pairing). */
int mg_set_pairing(mg_ctx* ctx, const mg_pairing_params* pp);

/* SolvePairing for HFB (src/Pairing.f90:743-890): density factor, cutoffs,
 * pairing field (HFBPairingField, src/HFB.f90:350-518), gaps (HFBGaps,
 * :520-632), Fermi energies (FindFermiEnergy, same particle-number equation
 * and tolerance as HFBFindFermiEnergyBroyden :1849-2161), the canonical
 * basis (HFBOccupations :3361-3560) and rho/kappa mixing.  The canonical
 * spinors land in MG_CAN_BASIS.  info may be NULL. */
int mg_solve_pairing(mg_ctx* ctx, mg_pairing_info* info);

/* Block b = it*2 + (parity+1)/2 of rho, kappa and Delta (N*N each, N the
 * block size including time-reversed partners); returns N, any pointer may
 * be NULL (then only N is returned). */
int mg_get_hfb_block(mg_ctx* ctx, int b, double* rho, double* kappa, double* delta);

/* Pairing field (real, imaginary) and DensityFactor, 2V each, may be NULL. */
int mg_get_pairing_field(mg_ctx* ctx, double* re, double* im, double* dfac);

/* Electric multipole moments of the densities (Calculate_Multipole,
 * src/Moments.f90:1907-2004) for the Coulomb boundary.  With constraints
 * this is CalculateAllMoments (src/Moments.f90:2250-2334): the density
 * cutoff, the constrained moments' values and squares (the first call also
 * sets each constraint's running target to the current value, :2277-2297)
 * and the constraint field (CalcConstraintEnergy :2368-2486) that
 * mg_construct_potentials adds to U (src/MeanFields.f90:403). */
int mg_calculate_moments(mg_ctx* ctx);

/* One constraint of &MomentConstraint (src/Moments.f90:3575-3790) of the
 * kind the namelist defaults to: alternating-direction (ConstraintType = 2)
 * on the neutron + proton value (Isoswitch = 1, Total = .false.) of Re Q_lm,
 * with the density-dependent cutoff (CutoffType = 0, RutzCutOff
 * :2703-2871, radd = 4 fm, acut = 0.4 fm) and Damping = 0.  EV8 meshes only
 * (l and m even). */
typedef struct mg_moment_constraint {
    int    l, m;          /* the constrained moment Re Q_lm                      */
    double constraint;    /* Constraint: target <Q_lm> (fm^l)                     */
    double intensity;     /* Intensity; 0 = estimated on the first readjustment  */
    int    iteration;     /* iteration: switched off once the Evolve iteration    */
                          /* count exceeds it (<= 0: never), src/Moments.f90:3516 */
} mg_moment_constraint;

typedef struct mg_constraint_state {
    double value[2];      /* Value: <Q_lm> of neutrons, protons                  */
    double squared[2];    /* Squared: <Q_lm^2> (one-body part)                   */
    double constraint;    /* Constraint(1): the readjusted target of the field   */
    double intensity;     /* Intensity(1)                                        */
    int    active;        /* ConstraintType /= 0 (not switched off yet)          */
} mg_constraint_state;

/* Adds a constraint (before the start, like the namelist read in
 * CheckForRutzMoments); returns its index >= 0. */
int mg_add_constraint(mg_ctx* ctx, const mg_moment_constraint* mc);
int mg_get_constraint(mg_ctx* ctx, int k, mg_constraint_state* out);
/* Cutoff(:,:,:,it) and ConstraintEnergy, 2V each, either may be NULL. */
int mg_get_constraint_fields(mg_ctx* ctx, double* cutoff, double* field);
/* AlternateStep (src/ImaginaryTime.f90:306-437, no cranking): the HF
 * spinors take psi - multipole(it) psi, multipole(it) = sum over the
 * alternating constraints of 0.5 (<Q> - target) / (<Q^2> + d0) Cutoff(it)
 * Q_lm, then the energy-ordered Gram-Schmidt. */
int mg_alternate_step(mg_ctx* ctx);
/* ReadjustAllMoments (src/Moments.f90:2336-2366, alternating branch of
 * Readjust :2994-3058) then TurnOffConstraints(iteration) (:3516-3550). */
int mg_readjust_moments(mg_ctx* ctx, int iteration);

/* Coulomb solve (src/Coulomb.f90:255-346): multipole boundary, CG, Slater
 * exchange.  iters may be NULL.  Returns MG_NOT_CONVERGED when the CG hits
 * CoulombMax (the reference prints and continues; so does this library). */
int mg_solve_coulomb(mg_ctx* ctx, int* iters);

/* Relative residual |b - L phi| / |b| of the last Coulomb solve on the stored
 * box, with the solver's Laplacian and boundary (a diagnostic; the
 * reference's CG stops on sum(Residual**2), src/Coulomb.f90:883-889). */
int mg_coulomb_residual(mg_ctx* ctx, double* rel);
/* Sets the Coulomb potential back to InitialGuess (the uniform-sphere
 * potential, src/Coulomb.f90:542-581), the start of a cold solve. */
int mg_coulomb_reset(mg_ctx* ctx);

/* ConstructPotentials (src/PotentialMixing.f90:17-201, MixingScheme 0):
 * Coulomb, U, W (+div W), B (+grad B).  iters may be NULL. */
int mg_construct_potentials(mg_ctx* ctx, int* coulomb_iters);
/* U,B,coul,coulex: 2V/2V/V/V; nablab,divw: 6V; w: 18V; any may be NULL. */
int mg_get_potentials(mg_ctx* ctx, double* u, double* b, double* nablab,
                      double* w, double* divw, double* coul, double* coulex);

/* Time-odd densities and fields of a run without time reversal (trc = 0):
 * vecj, vecs and their curls (ComputeDensity's time-odd part,
 * src/Densities.f90:1004-1106), A and S with the cranking fields (CalcAPot,
 * CalcSPot, src/MeanFields.f90:411-492, :618-712; CrankAPot, CrankSPot,
 * src/Cranking.f90:234-324) as [it][m][V] (6V each), div A as [it][V] (2V);
 * any may be NULL.  MG_ERR_ARG with time reversal. */
int mg_get_time_odd(mg_ctx* ctx, double* vecj, double* vecs, double* rotj, double* rots,
                    double* a, double* s, double* diva);

/* The time-odd tensor densities and fields without time reversal, when
 * B14..B21 are not all zero: T (GetVecT, src/Spwf.f90:2087-2129), F
 * (GetVecF :2162-2180), lap s and grad div s (src/Densities.f90:1055-1185),
 * the C and D fields (CalcCPot, CalcDPot, src/MeanFields.f90:714-790), each
 * [it][m][V] (6V), and div D [it][V] (2V); any may be NULL.  The densities
 * a coefficient does not use stay zero, as the reference leaves them
 * unallocated.  MG_ERR_ARG with time reversal or without these terms. */
int mg_get_time_odd_tensor(mg_ctx* ctx, double* vt, double* vf, double* ls, double* gds,
                           double* c, double* d, double* divd);

/* INITWF (src/InOut.f90:1418-1473) with nil8's Nilsson states
 * (src/nil8.f90:16-546) for an EV8 context (nz >= nx, ny): the lowest
 * n_neutron neutron and nwt - n_neutron proton levels of the deformed
 * oscillator with l.s and l^2 terms in meven even and modd odd major shells
 * (INITWF: 6 and 5, ho = 0.2 fm^-2 on every axis), positive parity first
 * within each isospin, evaluated on the mesh on the device; then every
 * grid value plus amplitude * u, u uniform in [-1, 1) from a generator
 * keyed on (seed, spwf, component, point), and each spwf normalised.
 * Sets the HF spinors, their quantum numbers and the Nilsson energies. */
typedef struct mg_nilsson_params {
    int    n_neutron;     /* stored neutron spwfs; the other nwt - n_neutron are protons */
    int    meven, modd;   /* even / odd major shells of the basis                        */
    double ho[3];         /* m omega / hbar per axis (fm^-2)                             */
    double amplitude;     /* perturbation of every grid value (0: none)                  */
    int    seed;
} mg_nilsson_params;
int mg_nilsson_start(mg_ctx* ctx, const mg_nilsson_params* np);

/* BreakParity, BreakSignature, BreakTimeSimplex (src/Transform.f90:187-366),
 * in TransformInput's order (:83-99), of every HF spwf of an EV8 context
 * into a symmetry-free context (pc = sc = tsc = 0) with twice the points
 * per axis, the same dx, nwt and time reversal: the full-box spinors, the
 * isospins (the broken quantum numbers 0), occupations and energies. */
int mg_break_symmetries(mg_ctx* ev8, mg_ctx* full);

/* SymmetryOperators + CalcRMSRadius (src/Spwf.f90:2289-2347) for every spwf
 * of a basis: out[6*i + 0..5] = isospin, signature, parity, time simplex,
 * x-simplex expectation values and the RMS radius sqrt(<r^2>).  A conserved
 * symmetry gives the spwf's quantum number; on the symmetry-free box the
 * expectation values of the mirror actions (src/Spinor.f90:391-490). */
int mg_symmetry_operators(mg_ctx* ctx, int basis, double* out);
int mg_set_potentials(mg_ctx* ctx, const double* u, const double* b,
                      const double* nablab, const double* w, const double* divw);

/* CompEnergy (src/Energy.f90:62-179). */
int mg_energy(mg_ctx* ctx, mg_energy_terms* out);

/* n_iter passes of the Evolve loop body (src/Main.f90:255-328) with fixed
 * dt and momentum, each ending with CompEnergy as the reference's does; out
 * (may be NULL) receives the last iteration's energy.
 * With constraints each pass also takes the AlternateStep first (while an
 * alternating constraint was active at the previous pass's check, :261-274)
 * and readjusts the constraints after the moments (:298-304); the context
 * numbers the passes from 1 across calls for TurnOffConstraints. */
int mg_iterate(mg_ctx* ctx, int n_iter, double dt, double momentum,
               mg_energy_terms* out);

/* ---- batches of independent instances ------------------------------------- */

/* A batch of independent HFB instances (uneven meshes, spwf counts,
 * particle numbers, constraints) run concurrently: the reference runs one
 * nucleus per process (src/Main.f90), so this has no single reference
 * counterpart; each instance follows Evolve exactly as mg_iterate does.
 * The contexts come from mg_create (each on its own stream: pass NULL) and
 * stay owned by the caller, who prepares them (spinors, pairing,
 * constraints, start) before batching.  Host worker threads drive the
 * instances, each instance on its own streams, so the latency-bound steps of
 * one overlap with the mesh kernels of others.  Until the batch is tuned
 * the workers are min(n, host threads), instances assigned longest first by
 * nwt * V.  MG_ERR_ARG when a context appears twice or was created on
 * another device than the current one. */
typedef struct mg_batch mg_batch;
int mg_batch_create(int n, mg_ctx* const* ctxs, mg_batch** out);
int mg_batch_destroy(mg_batch* b);
/* Schedule autotuner: `probe` passes of each instance alone give its pass
 * time; then `probe` rounds for each candidate worker count (powers of two
 * up to min(n, 4 x host threads), and n) with a longest-first assignment of
 * those times; the fastest is kept (workers_out, may be NULL).  The tuning
 * passes are ordinary Evolve passes: they advance every instance by
 * probe * (1 + candidates) iterations.  dt, momentum: n values. */
int mg_batch_tune(mg_batch* b, int probe, const double* dt, const double* momentum,
                  int* workers_out);
/* Fixes the worker count (longest-first assignment); returns it. */
int mg_batch_set_workers(mg_batch* b, int workers);
/* n_iter Evolve passes of every instance (mg_iterate with dt[i],
 * momentum[i]); out (n entries, may be NULL) receives each instance's last
 * energy.  An instance whose pass fails is marked failed and skipped from
 * then on (the reference would stop that nucleus's run); the others carry
 * on.  Returns when all instances' work is complete: a negative status if
 * any instance failed in this call, else MG_NOT_CONVERGED if any Coulomb
 * solve hit its cap, else MG_OK.  mg_batch_tune treats failures the same
 * way. */
int mg_batch_iterate(mg_batch* b, int n_iter, const double* dt, const double* momentum,
                     mg_energy_terms* out);
/* Per-instance status after the last call (n ints): MG_OK, MG_NOT_CONVERGED,
 * or the negative status with which the instance failed. */
int mg_batch_status(mg_batch* b, int* status);

/* Convergence thresholds of ConvergenceCheck (src/Main.f90:358-397), the
 * &GenInfo values: EnergyPrec (default 0.01E-08, a single-precision
 * literal), MomentPrec and PairingPrec (1e-4). */
typedef struct mg_convergence {
    double energy_prec;   /* relative change of E_total against each of the last 7 */
    double moment_prec;   /* constrained moments against their running targets     */
    double pairing_prec;  /* Fermi energies (HFB)                                   */
} mg_convergence;

/* ConvergenceCheck (src/Main.f90:358-397): ConverMultipoleAll
 * (src/Moments.f90:2628-2701, constrained moments, value and the 7 previous
 * ones against the running target), ConverEnergy (src/Energy.f90:1458-1481,
 * E_total against the 7 previous CompEnergy results; mg_energy and every
 * mg_iterate pass that computes the energy shift that history) and
 * ConverFermi (src/Pairing.f90:1048-1070).  ConverFermi compares the Fermi
 * energies with a history that the reference never writes (zeros), so an
 * HFB run only passes when both |Fermi| <= PairingPrec: in practice HFB runs
 * go to MaxIter, as in the reference.  prec may be NULL (defaults).  A total
 * energy >= 0 returns MG_ERR_STATE (the reference stops: 'Positive total
 * energy!'). */
int mg_convergence_check(mg_ctx* ctx, const mg_convergence* prec, int* converged);
/* The Evolve loop (src/Main.f90:255-328): up to max_iter passes of
 * mg_iterate, each followed by mg_convergence_check, leaving the loop when
 * it passes.  iterations (may be NULL): passes run; converged (may be NULL);
 * out (may be NULL): the last energy. */
int mg_evolve(mg_ctx* ctx, int max_iter, double dt, double momentum, const mg_convergence* prec,
              int* iterations, int* converged, mg_energy_terms* out);

/* Number of kernels this context has launched so far (instrumentation; the
 * reference's only counterpart is the CoulombTime accumulator,
 * src/Coulomb.f90:288, :333-334). */
int mg_launch_count(mg_ctx* ctx, long long* count);

/* Phases of one mg_iterate pass, for the timer below (the reference's
 * counterpart is its per-routine timing printout, e.g. CoulombTime,
 * src/Coulomb.f90:288, :333-334).  Each phase is timed on the context's
 * stream from the end of the phase before it; MG_PH_SIDE_DERIVE is the
 * HF-basis DeriveAll on the side stream, overlapping the pairing phases. */
#define MG_PH_GRAD_DESC     0   /* AlternateStep, GradDesc with Gram-Schmidt    */
#define MG_PH_PAIRING_MESH  1   /* pairing field, gaps, cutoffs                 */
#define MG_PH_FERMI         2   /* Fermi search (HFB evaluations)               */
#define MG_PH_CANONICAL     3   /* canonical basis, occupations, HFB mixing     */
#define MG_PH_DERIVE        4   /* DeriveAll (canonical basis after the join)   */
#define MG_PH_HPSI_CAN      5   /* canonical single-particle energies           */
#define MG_PH_DENSITIES     6   /* densities and MixDensities                   */
#define MG_PH_MOMENTS       7   /* moments, readjustment                        */
#define MG_PH_POTENTIALS    8   /* ConstructPotentials with the Coulomb solve   */
#define MG_PH_ENERGY        9   /* CompEnergy                                   */
#define MG_PH_SIDE_DERIVE  10   /* HF-basis DeriveAll on the side stream        */
#define MG_PH_COUNT        11
/* Switch the phase timer on (on != 0; clears the totals) or off.  While on,
 * every mg_iterate pass records CUDA events between its phases and waits
 * for the pass's last event to read them: a diagnostic mode, not for timed
 * production runs. */
int mg_set_phase_timing(mg_ctx* ctx, int on);
/* Totals since the timer was switched on: ms[k] (n >= MG_PH_COUNT doubles)
 * is the device time of phase k summed over the timed passes, whose count
 * goes to *passes (may be NULL). */
int mg_get_phase_times(mg_ctx* ctx, double* ms, int n, long long* passes);

#ifdef __cplusplus
}
#endif

#endif /* MOCCA_GPU_H */
