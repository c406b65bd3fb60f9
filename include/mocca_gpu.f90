! mocca_gpu.f90 -- iso_c_binding interface of libmocca_gpu (include/mocca_gpu.h)
! for the Fortran host: one bind(C) derived type per struct of the C header
! and one interface per entry point.  Every argument crosses as a value or a
! c_ptr: pass c_loc() of a scalar, array or derived-type variable, and an
! array of c_ptr for the lists of grids (one c_loc(HFBasis(i)%Value%Grid)
! per spwf).  Every function returns the status of the C header (0 ok,
! > 0 not converged, < 0 error); gpu_check turns an error into the
! reference's stp().  Written by include/make_fortran_module.py.
module mocca_gpu
  use iso_c_binding
  use GenInfo, only : stp
  implicit none

  type, bind(C) :: mg_params
    integer(c_int) :: nx
    integer(c_int) :: ny
    integer(c_int) :: nz
    real(c_double) :: dx
    integer(c_int) :: pc
    integer(c_int) :: sc
    integer(c_int) :: tsc
    integer(c_int) :: trc
    integer(c_int) :: nwt
    real(c_double) :: neutrons
    real(c_double) :: protons
    integer(c_int) :: precision
    integer(c_int) :: pairing
    integer(c_int) :: coulomb_max
    integer(c_int) :: max_l_coul
    integer(c_int) :: coulomb_solver
    integer(c_int) :: mixing_scheme
    real(c_double) :: damping
    real(c_double) :: precon_u
    integer(c_int) :: parameter_estimation
    real(c_double) :: coulomb_prec
    real(c_double) :: omega(3)
    real(c_double) :: precon_w
  end type mg_params
  type, bind(C) :: mg_force
    real(c_double) :: t0
    real(c_double) :: x0
    real(c_double) :: t1
    real(c_double) :: x1
    real(c_double) :: t2
    real(c_double) :: x2
    real(c_double) :: t3a
    real(c_double) :: x3a
    real(c_double) :: yt3a
    real(c_double) :: t3b
    real(c_double) :: x3b
    real(c_double) :: yt3b
    real(c_double) :: te
    real(c_double) :: to
    real(c_double) :: wso
    real(c_double) :: wsoq
    real(c_double) :: hbm
    real(c_double) :: e2
    real(c_double) :: hbar
    real(c_double) :: nucleonmass(2)
    integer(c_int) :: com1body
    integer(c_int) :: com2body
    integer(c_int) :: cexchange
    integer(c_int) :: j2terms
    integer(c_int) :: coupling
  end type mg_force
  type, bind(C) :: mg_skyrme_b
    real(c_double) :: B1
    real(c_double) :: B2
    real(c_double) :: B3
    real(c_double) :: B4
    real(c_double) :: B5
    real(c_double) :: B6
    real(c_double) :: B7a
    real(c_double) :: B7b
    real(c_double) :: B8a
    real(c_double) :: B8b
    real(c_double) :: byt3a
    real(c_double) :: byt3b
    real(c_double) :: B9
    real(c_double) :: B9q
    real(c_double) :: B10
    real(c_double) :: B11
    real(c_double) :: B12a
    real(c_double) :: B12b
    real(c_double) :: B13a
    real(c_double) :: B13b
    real(c_double) :: B14
    real(c_double) :: B15
    real(c_double) :: B16
    real(c_double) :: B17
    real(c_double) :: B18
    real(c_double) :: B19
    real(c_double) :: B20
    real(c_double) :: B21
  end type mg_skyrme_b
  type, bind(C) :: mg_energy_terms
    real(c_double) :: total
    real(c_double) :: kinetic(2)
    real(c_double) :: skyrme(36)
    real(c_double) :: coulomb
    real(c_double) :: coulomb_exchange
    real(c_double) :: com(2,2)
    real(c_double) :: pairing(2)
    real(c_double) :: sp_energy
  end type mg_energy_terms
  type, bind(C) :: mg_pairing_params
    real(c_double) :: strength(2)
    real(c_double) :: alpha(2)
    real(c_double) :: rhosat
    real(c_double) :: cut(2)
    real(c_double) :: mu(2)
    real(c_double) :: mix
    real(c_double) :: fermi_prec
    integer(c_int) :: max_iter
    integer(c_int) :: guess_kappa
    real(c_double) :: fermi_start(2)
    integer(c_int) :: fermi_solver
  end type mg_pairing_params
  type, bind(C) :: mg_pairing_info
    real(c_double) :: fermi(2)
    real(c_double) :: particles(2)
    integer(c_int) :: evaluations
    integer(c_int) :: converged
    real(c_double) :: pairing_energy(2)
    real(c_double) :: dispersion(2)
    integer(c_int) :: first_order
  end type mg_pairing_info
  type, bind(C) :: mg_moment_constraint
    integer(c_int) :: l
    integer(c_int) :: m
    real(c_double) :: constraint
    real(c_double) :: intensity
    integer(c_int) :: iteration
  end type mg_moment_constraint
  type, bind(C) :: mg_constraint_state
    real(c_double) :: value(2)
    real(c_double) :: squared(2)
    real(c_double) :: constraint
    real(c_double) :: intensity
    integer(c_int) :: active
  end type mg_constraint_state
  type, bind(C) :: mg_nilsson_params
    integer(c_int) :: n_neutron
    integer(c_int) :: meven
    integer(c_int) :: modd
    real(c_double) :: ho(3)
    real(c_double) :: amplitude
    integer(c_int) :: seed
  end type mg_nilsson_params
  type, bind(C) :: mg_convergence
    real(c_double) :: energy_prec
    real(c_double) :: moment_prec
    real(c_double) :: pairing_prec
  end type mg_convergence

  interface
    integer(c_int) function mg_skyrme_coefficients(f, trc, out) bind(C, name="mg_skyrme_coefficients")
      import
      type(c_ptr), value :: f
      integer(c_int), value :: trc
      type(c_ptr), value :: out
    end function
    integer(c_int) function mg_lagrange_matrices(n, dx, folded, d1, d2) bind(C, name="mg_lagrange_matrices")
      import
      integer(c_int), value :: n
      real(c_double), value :: dx
      integer(c_int), value :: folded
      type(c_ptr), value :: d1
      type(c_ptr), value :: d2
    end function
    integer(c_int) function mg_eigh_batched(nb, n, ld, a, w, z) bind(C, name="mg_eigh_batched")
      import
      integer(c_int), value :: nb
      type(c_ptr), value :: n
      integer(c_int), value :: ld
      type(c_ptr), value :: a
      type(c_ptr), value :: w
      type(c_ptr), value :: z
    end function
    integer(c_int) function mg_eigh_batched_noalloc(nb, n, ld, a, w, z, info, stream) bind(C, name="mg_eigh_batched_noalloc")
      import
      integer(c_int), value :: nb
      type(c_ptr), value :: n
      integer(c_int), value :: ld
      type(c_ptr), value :: a
      type(c_ptr), value :: w
      type(c_ptr), value :: z
      type(c_ptr), value :: info
      type(c_ptr), value :: stream
    end function
    integer(c_int) function mg_create(p, f, stream, out) bind(C, name="mg_create")
      import
      type(c_ptr), value :: p
      type(c_ptr), value :: f
      type(c_ptr), value :: stream
      type(c_ptr), intent(out) :: out
    end function
    integer(c_int) function mg_destroy(ctx) bind(C, name="mg_destroy")
      import
      type(c_ptr), value :: ctx
    end function
    integer(c_int) function mg_synchronize(ctx) bind(C, name="mg_synchronize")
      import
      type(c_ptr), value :: ctx
    end function
    integer(c_int) function mg_set_precision(ctx, precision) bind(C, name="mg_set_precision")
      import
      type(c_ptr), value :: ctx
      integer(c_int), value :: precision
    end function
    integer(c_int) function mg_upload_spinors(ctx, basis, grids, qn, first, count) bind(C, name="mg_upload_spinors")
      import
      type(c_ptr), value :: ctx
      integer(c_int), value :: basis
      type(c_ptr), value :: grids
      type(c_ptr), value :: qn
      integer(c_int), value :: first
      integer(c_int), value :: count
    end function
    integer(c_int) function mg_download_spinors(ctx, basis, grids, first, count) bind(C, name="mg_download_spinors")
      import
      type(c_ptr), value :: ctx
      integer(c_int), value :: basis
      type(c_ptr), value :: grids
      integer(c_int), value :: first
      integer(c_int), value :: count
    end function
    integer(c_int) function mg_download_derivatives(ctx, basis, der, lap, first, count) bind(C, name="mg_download_derivatives")
      import
      type(c_ptr), value :: ctx
      integer(c_int), value :: basis
      type(c_ptr), value :: der
      type(c_ptr), value :: lap
      integer(c_int), value :: first
      integer(c_int), value :: count
    end function
    integer(c_int) function mg_set_occupations(ctx, basis, occ) bind(C, name="mg_set_occupations")
      import
      type(c_ptr), value :: ctx
      integer(c_int), value :: basis
      type(c_ptr), value :: occ
    end function
    integer(c_int) function mg_get_occupations(ctx, basis, occ) bind(C, name="mg_get_occupations")
      import
      type(c_ptr), value :: ctx
      integer(c_int), value :: basis
      type(c_ptr), value :: occ
    end function
    integer(c_int) function mg_set_energies(ctx, basis, e) bind(C, name="mg_set_energies")
      import
      type(c_ptr), value :: ctx
      integer(c_int), value :: basis
      type(c_ptr), value :: e
    end function
    integer(c_int) function mg_get_energies(ctx, basis, e, disp) bind(C, name="mg_get_energies")
      import
      type(c_ptr), value :: ctx
      integer(c_int), value :: basis
      type(c_ptr), value :: e
      type(c_ptr), value :: disp
    end function
    integer(c_int) function mg_derive_basis(ctx, basis) bind(C, name="mg_derive_basis")
      import
      type(c_ptr), value :: ctx
      integer(c_int), value :: basis
    end function
    integer(c_int) function mg_derive_all(ctx) bind(C, name="mg_derive_all")
      import
      type(c_ptr), value :: ctx
    end function
    integer(c_int) function mg_hpsi(ctx, basis, hpsi, e, disp) bind(C, name="mg_hpsi")
      import
      type(c_ptr), value :: ctx
      integer(c_int), value :: basis
      type(c_ptr), value :: hpsi
      type(c_ptr), value :: e
      type(c_ptr), value :: disp
    end function
    integer(c_int) function mg_grad_desc(ctx, dt, momentum) bind(C, name="mg_grad_desc")
      import
      type(c_ptr), value :: ctx
      real(c_double), value :: dt
      real(c_double), value :: momentum
    end function
    integer(c_int) function mg_get_step_parameters(ctx, dt, momentum) bind(C, name="mg_get_step_parameters")
      import
      type(c_ptr), value :: ctx
      type(c_ptr), value :: dt
      type(c_ptr), value :: momentum
    end function
    integer(c_int) function mg_gram_schmidt(ctx) bind(C, name="mg_gram_schmidt")
      import
      type(c_ptr), value :: ctx
    end function
    integer(c_int) function mg_hf_fill(ctx) bind(C, name="mg_hf_fill")
      import
      type(c_ptr), value :: ctx
    end function
    integer(c_int) function mg_update_densities(ctx) bind(C, name="mg_update_densities")
      import
      type(c_ptr), value :: ctx
    end function
    integer(c_int) function mg_mix_densities(ctx) bind(C, name="mg_mix_densities")
      import
      type(c_ptr), value :: ctx
    end function
    integer(c_int) function mg_get_densities(ctx, rho, tau, nablaj, derrho, laprho) bind(C, name="mg_get_densities")
      import
      type(c_ptr), value :: ctx
      type(c_ptr), value :: rho
      type(c_ptr), value :: tau
      type(c_ptr), value :: nablaj
      type(c_ptr), value :: derrho
      type(c_ptr), value :: laprho
    end function
    integer(c_int) function mg_set_densities(ctx, rho, tau, nablaj, derrho, laprho) bind(C, name="mg_set_densities")
      import
      type(c_ptr), value :: ctx
      type(c_ptr), value :: rho
      type(c_ptr), value :: tau
      type(c_ptr), value :: nablaj
      type(c_ptr), value :: derrho
      type(c_ptr), value :: laprho
    end function
    integer(c_int) function mg_get_jmunu(ctx, jmunu) bind(C, name="mg_get_jmunu")
      import
      type(c_ptr), value :: ctx
      type(c_ptr), value :: jmunu
    end function
    integer(c_int) function mg_set_jmunu(ctx, jmunu) bind(C, name="mg_set_jmunu")
      import
      type(c_ptr), value :: ctx
      type(c_ptr), value :: jmunu
    end function
    integer(c_int) function mg_set_pairing(ctx, pp) bind(C, name="mg_set_pairing")
      import
      type(c_ptr), value :: ctx
      type(c_ptr), value :: pp
    end function
    integer(c_int) function mg_solve_pairing(ctx, info) bind(C, name="mg_solve_pairing")
      import
      type(c_ptr), value :: ctx
      type(c_ptr), value :: info
    end function
    integer(c_int) function mg_get_hfb_block(ctx, b, rho, kappa, delta) bind(C, name="mg_get_hfb_block")
      import
      type(c_ptr), value :: ctx
      integer(c_int), value :: b
      type(c_ptr), value :: rho
      type(c_ptr), value :: kappa
      type(c_ptr), value :: delta
    end function
    integer(c_int) function mg_get_pairing_field(ctx, re, im, dfac) bind(C, name="mg_get_pairing_field")
      import
      type(c_ptr), value :: ctx
      type(c_ptr), value :: re
      type(c_ptr), value :: im
      type(c_ptr), value :: dfac
    end function
    integer(c_int) function mg_calculate_moments(ctx) bind(C, name="mg_calculate_moments")
      import
      type(c_ptr), value :: ctx
    end function
    integer(c_int) function mg_add_constraint(ctx, mc) bind(C, name="mg_add_constraint")
      import
      type(c_ptr), value :: ctx
      type(c_ptr), value :: mc
    end function
    integer(c_int) function mg_get_constraint(ctx, k, out) bind(C, name="mg_get_constraint")
      import
      type(c_ptr), value :: ctx
      integer(c_int), value :: k
      type(c_ptr), value :: out
    end function
    integer(c_int) function mg_get_constraint_fields(ctx, cutoff, field) bind(C, name="mg_get_constraint_fields")
      import
      type(c_ptr), value :: ctx
      type(c_ptr), value :: cutoff
      type(c_ptr), value :: field
    end function
    integer(c_int) function mg_alternate_step(ctx) bind(C, name="mg_alternate_step")
      import
      type(c_ptr), value :: ctx
    end function
    integer(c_int) function mg_readjust_moments(ctx, iteration) bind(C, name="mg_readjust_moments")
      import
      type(c_ptr), value :: ctx
      integer(c_int), value :: iteration
    end function
    integer(c_int) function mg_solve_coulomb(ctx, iters) bind(C, name="mg_solve_coulomb")
      import
      type(c_ptr), value :: ctx
      type(c_ptr), value :: iters
    end function
    integer(c_int) function mg_coulomb_residual(ctx, rel) bind(C, name="mg_coulomb_residual")
      import
      type(c_ptr), value :: ctx
      type(c_ptr), value :: rel
    end function
    integer(c_int) function mg_coulomb_reset(ctx) bind(C, name="mg_coulomb_reset")
      import
      type(c_ptr), value :: ctx
    end function
    integer(c_int) function mg_construct_potentials(ctx, coulomb_iters) bind(C, name="mg_construct_potentials")
      import
      type(c_ptr), value :: ctx
      type(c_ptr), value :: coulomb_iters
    end function
    integer(c_int) function mg_get_potentials(ctx, u, b, nablab, w, divw, coul, coulex) bind(C, name="mg_get_potentials")
      import
      type(c_ptr), value :: ctx
      type(c_ptr), value :: u
      type(c_ptr), value :: b
      type(c_ptr), value :: nablab
      type(c_ptr), value :: w
      type(c_ptr), value :: divw
      type(c_ptr), value :: coul
      type(c_ptr), value :: coulex
    end function
    integer(c_int) function mg_get_time_odd(ctx, vecj, vecs, rotj, rots, a, s, diva) bind(C, name="mg_get_time_odd")
      import
      type(c_ptr), value :: ctx
      type(c_ptr), value :: vecj
      type(c_ptr), value :: vecs
      type(c_ptr), value :: rotj
      type(c_ptr), value :: rots
      type(c_ptr), value :: a
      type(c_ptr), value :: s
      type(c_ptr), value :: diva
    end function
    integer(c_int) function mg_get_time_odd_tensor(ctx, vt, vf, ls, gds, c, d, divd) bind(C, name="mg_get_time_odd_tensor")
      import
      type(c_ptr), value :: ctx
      type(c_ptr), value :: vt
      type(c_ptr), value :: vf
      type(c_ptr), value :: ls
      type(c_ptr), value :: gds
      type(c_ptr), value :: c
      type(c_ptr), value :: d
      type(c_ptr), value :: divd
    end function
    integer(c_int) function mg_nilsson_start(ctx, np) bind(C, name="mg_nilsson_start")
      import
      type(c_ptr), value :: ctx
      type(c_ptr), value :: np
    end function
    integer(c_int) function mg_break_symmetries(ev8, full) bind(C, name="mg_break_symmetries")
      import
      type(c_ptr), value :: ev8
      type(c_ptr), value :: full
    end function
    integer(c_int) function mg_symmetry_operators(ctx, basis, out) bind(C, name="mg_symmetry_operators")
      import
      type(c_ptr), value :: ctx
      integer(c_int), value :: basis
      type(c_ptr), value :: out
    end function
    integer(c_int) function mg_set_potentials(ctx, u, b, nablab, w, divw) bind(C, name="mg_set_potentials")
      import
      type(c_ptr), value :: ctx
      type(c_ptr), value :: u
      type(c_ptr), value :: b
      type(c_ptr), value :: nablab
      type(c_ptr), value :: w
      type(c_ptr), value :: divw
    end function
    integer(c_int) function mg_energy(ctx, out) bind(C, name="mg_energy")
      import
      type(c_ptr), value :: ctx
      type(c_ptr), value :: out
    end function
    integer(c_int) function mg_iterate(ctx, n_iter, dt, momentum, out) bind(C, name="mg_iterate")
      import
      type(c_ptr), value :: ctx
      integer(c_int), value :: n_iter
      real(c_double), value :: dt
      real(c_double), value :: momentum
      type(c_ptr), value :: out
    end function
    integer(c_int) function mg_batch_create(n, ctxs, out) bind(C, name="mg_batch_create")
      import
      integer(c_int), value :: n
      type(c_ptr), intent(out) :: ctxs
      type(c_ptr), intent(out) :: out
    end function
    integer(c_int) function mg_batch_destroy(b) bind(C, name="mg_batch_destroy")
      import
      type(c_ptr), value :: b
    end function
    integer(c_int) function mg_batch_tune(b, probe, dt, momentum, workers_out) bind(C, name="mg_batch_tune")
      import
      type(c_ptr), value :: b
      integer(c_int), value :: probe
      type(c_ptr), value :: dt
      type(c_ptr), value :: momentum
      type(c_ptr), value :: workers_out
    end function
    integer(c_int) function mg_batch_set_workers(b, workers) bind(C, name="mg_batch_set_workers")
      import
      type(c_ptr), value :: b
      integer(c_int), value :: workers
    end function
    integer(c_int) function mg_batch_iterate(b, n_iter, dt, momentum, out) bind(C, name="mg_batch_iterate")
      import
      type(c_ptr), value :: b
      integer(c_int), value :: n_iter
      type(c_ptr), value :: dt
      type(c_ptr), value :: momentum
      type(c_ptr), value :: out
    end function
    integer(c_int) function mg_batch_status(b, status) bind(C, name="mg_batch_status")
      import
      type(c_ptr), value :: b
      type(c_ptr), value :: status
    end function
    integer(c_int) function mg_convergence_check(ctx, prec, converged) bind(C, name="mg_convergence_check")
      import
      type(c_ptr), value :: ctx
      type(c_ptr), value :: prec
      type(c_ptr), value :: converged
    end function
    integer(c_int) function mg_evolve(ctx, max_iter, dt, momentum, prec, iterations, converged, out) bind(C, name="mg_evolve")
      import
      type(c_ptr), value :: ctx
      integer(c_int), value :: max_iter
      real(c_double), value :: dt
      real(c_double), value :: momentum
      type(c_ptr), value :: prec
      type(c_ptr), value :: iterations
      type(c_ptr), value :: converged
      type(c_ptr), value :: out
    end function
    integer(c_int) function mg_launch_count(ctx, count) bind(C, name="mg_launch_count")
      import
      type(c_ptr), value :: ctx
      type(c_ptr), value :: count
    end function
    integer(c_int) function mg_set_phase_timing(ctx, on) bind(C, name="mg_set_phase_timing")
      import
      type(c_ptr), value :: ctx
      integer(c_int), value :: on
    end function
    integer(c_int) function mg_get_phase_times(ctx, ms, n, passes) bind(C, name="mg_get_phase_times")
      import
      type(c_ptr), value :: ctx
      type(c_ptr), value :: ms
      integer(c_int), value :: n
      type(c_ptr), value :: passes
    end function
  end interface
contains
  subroutine gpu_check(st, where)
    integer(c_int), intent(in) :: st
    character(len=*), intent(in) :: where
    if (st .lt. 0) call stp('mocca_gpu call failed: ' // where, 'status', int(st))
  end subroutine gpu_check
end module mocca_gpu
