! ISO_C_BINDING interface to libpfgpu.so (include/pfgpu.h) for a Fortran host
! such as var_diff.f90.  Link with -L<dir of libpfgpu.so> -lpfgpu (or the
! full path of the library).  The Fortran-signature shims f_trans, inv_trans
! and k_space need no interface: the reference calls them as implicit
! externals and the library exports f_trans_, inv_trans_ and k_space_.
module pfgpu
  use, intrinsic :: iso_c_binding
  implicit none

  integer(c_int), parameter :: PF_OK = 0, PF_EINVAL = -1, PF_ECUDA = -2, &
       PF_ENOMEM = -3, PF_ENONFINITE = -4, PF_EIO = -5
  integer(c_int), parameter :: PF_MOB_REFERENCE = 0, PF_MOB_C1MC = 1
  integer(c_int), parameter :: PF_FP32_FUSED = 32, PF_FP64_PLAIN = 64

  type, bind(C) :: pf_config
     integer(c_int) :: nx, ny, nz, var
     real(c_double) :: t_step, grad_coeff_phi, grad_coeff_c, D_S, D_L, D_gb, mob_phi
     real(c_double) :: sigma_1, sigma_2
     real(c_double) :: am, ap, con_0_mat, con_0_ppt
     integer(c_int) :: mobility, precision, device
     integer(c_int) :: reserved(5)
  end type pf_config

  type, bind(C) :: pf_diag
     integer(c_int) :: step, nonfinite
     real(c_double) :: f_int, f_eta, f_ch, e_tot
     real(c_double) :: c_max, c_min, phi_min, phi_P_max
     real(c_double) :: mass
  end type pf_diag

  interface
     integer(c_int) function pf_create(cfg, run) bind(C, name="pf_create")
       import :: c_int, c_ptr, pf_config
       type(pf_config), intent(in) :: cfg
       type(c_ptr), intent(out) :: run
     end function pf_create

     integer(c_int) function pf_set_fields(run, phi, con) bind(C, name="pf_set_fields")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: run
       real(c_double), intent(in) :: phi(*), con(*)
     end function pf_set_fields

     integer(c_int) function pf_step(run, nsteps, diag) bind(C, name="pf_step")
       import :: c_int, c_ptr, pf_diag
       type(c_ptr), value :: run
       integer(c_int), value :: nsteps
       type(pf_diag), intent(out) :: diag(*)
     end function pf_step

     integer(c_int) function pf_get_fields(run, phi, con) bind(C, name="pf_get_fields")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: run
       real(c_double), intent(out) :: phi(*), con(*)
     end function pf_get_fields

     integer(c_int) function pf_destroy(run) bind(C, name="pf_destroy")
       import :: c_int, c_ptr
       type(c_ptr), value :: run
     end function pf_destroy

     type(c_ptr) function pf_last_error() bind(C, name="pf_last_error")
       import :: c_ptr
     end function pf_last_error
  end interface
end module pfgpu
