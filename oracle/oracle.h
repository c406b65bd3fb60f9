/*
 * oracle.h -- CPU FP64 restatement of MOCCa's per-iteration mesh hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the parity checker for the
 * CUDA library (mocca_gb300/csrc): only tests/, __graft_entry__.smoke() and
 * bench.py's cpu_baseline leg load it.  Nothing in the product links it.
 *
 * Parity status: the reference is Fortran and no Fortran compiler exists in
 * the build container, and the reference ships no golden outputs, so this
 * restatement is pinned against self-derived known-answer tests (Lagrange
 * derivatives exact on the Fourier basis of the full line, folded = unfolded
 * on mirror-extended lines, Gram-Schmidt orthonormality, analytic Coulomb of
 * a uniform sphere) rather than reference-produced numbers: parity unpinned
 * by reference artefacts.
 *
 * Every function follows the reference routine cited beside it, in the same
 * operation order where that order fixes the rounding.
 */
#ifndef MOCCA_ORACLE_H
#define MOCCA_ORACLE_H

#include "../include/mocca_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_ctx orc_ctx;

int  orc_skyrme_coefficients(const mg_force* f, int trc, mg_skyrme_b* out);
int  orc_lagrange_matrices(int n, double dx, int folded, double* d1, double* d2);

orc_ctx* orc_create(const mg_params* p, const mg_force* f);
void orc_destroy(orc_ctx* c);

/* psi: count*4V doubles (spwf-major), qn: count*4 ints (may be NULL). */
int orc_set_spinors(orc_ctx* c, int basis, const double* psi, const int* qn);
int orc_get_spinors(orc_ctx* c, int basis, double* psi);
int orc_get_qn(orc_ctx* c, int basis, int* qn);
int orc_get_derivatives(orc_ctx* c, int basis, double* der, double* lap);
int orc_set_occupations(orc_ctx* c, int basis, const double* occ);
int orc_get_occupations(orc_ctx* c, int basis, double* occ);
int orc_set_energies(orc_ctx* c, int basis, const double* e);
int orc_get_energies(orc_ctx* c, int basis, double* e, double* disp);

/* one real grid, derivative along dir (0,1,2) or Laplacian (dir=3), with the
 * symmetry arguments of DeriveX/Y/Z(Grid, P, S, TS, Component). */
int orc_derive_grid(orc_ctx* c, const double* grid, int dir, int P, int S,
                    int TS, int comp, double* out);

int orc_derive_basis(orc_ctx* c, int basis);
int orc_derive_all(orc_ctx* c);
int orc_hpsi(orc_ctx* c, int basis, double* hpsi, double* e, double* disp);
int orc_grad_desc(orc_ctx* c, double dt, double momentum);
int orc_get_step_parameters(orc_ctx* c, double* dt, double* momentum);
int orc_gram_schmidt(orc_ctx* c);
int orc_hf_fill(orc_ctx* c);
int orc_update_densities(orc_ctx* c);
int orc_mix_densities(orc_ctx* c);
int orc_get_densities(orc_ctx* c, double* rho, double* tau, double* nablaj,
                      double* derrho, double* laprho);
int orc_get_jmunu(orc_ctx* c, double* jmunu);   /* 18V: [it][nu][mu][V] */
/* time-odd tensor densities and fields without time reversal: T, F, lap s,
 * grad div s, C, D as [it][m][V], div D as [it][V] (any may be NULL) */
int orc_get_time_odd_tensor(orc_ctx* c, double* vect, double* vecf, double* laps,
                            double* graddivs, double* cpot, double* dpot, double* divd);
/* ActionOfC and ActionOfD of spwf i of basis b (4V each) */
int orc_tensor_odd_action(orc_ctx* c, int b, int i, double* xc, double* xd);
int orc_set_densities(orc_ctx* c, const double* rho, const double* tau,
                      const double* nablaj, const double* derrho,
                      const double* laprho);
int orc_calculate_moments(orc_ctx* c);
int orc_get_moments(orc_ctx* c, double* values, int* lm, int max_count);
/* multipole constraints (alternating kind), as mg_add_constraint & co. */
int orc_add_constraint(orc_ctx* c, const mg_moment_constraint* mc);
int orc_get_constraint(orc_ctx* c, int k, mg_constraint_state* out);
int orc_get_constraint_fields(orc_ctx* c, double* cutoff, double* field);
int orc_alternate_step(orc_ctx* c);
int orc_readjust_moments(orc_ctx* c, int iteration);
/* ConvergenceCheck, as mg_convergence_check */
int orc_convergence_check(orc_ctx* c, const mg_convergence* prec, int* converged);
int orc_solve_coulomb(orc_ctx* c, int* iters);
int orc_construct_potentials(orc_ctx* c, int* iters);
int orc_get_potentials(orc_ctx* c, double* u, double* b, double* nablab,
                       double* w, double* divw, double* coul, double* coulex);
int orc_set_potentials(orc_ctx* c, const double* u, const double* b,
                       const double* nablab, const double* w, const double* divw);
int orc_energy(orc_ctx* c, mg_energy_terms* out);
int orc_iterate(orc_ctx* c, int n_iter, double dt, double momentum,
                mg_energy_terms* out);

/* HFB pairing (src/Pairing.f90:743-890 with the HFB procedures). */
int orc_set_pairing(orc_ctx* c, const mg_pairing_params* pp);
int orc_solve_pairing(orc_ctx* c, mg_pairing_info* info);
/* block b = it*2 + (parity+1)/2: size N, rho/kappa/delta (N*N each), may be NULL */
int orc_get_hfb_block(orc_ctx* c, int b, double* rho, double* kappa, double* delta);
int orc_get_pairing_field(orc_ctx* c, double* re, double* im, double* dfac);
/* symmetric eigensolver of the oracle (tred2 + tql2, ascending) */
int orc_eigh(int n, const double* a, double* w, double* z);

#ifdef __cplusplus
}
#endif
#endif
