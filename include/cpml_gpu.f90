! cpml_gpu.f90 -- iso_c_binding interface to libcpml (include/cpml.h) for the
! reference's Fortran host programs.
!
! A program such as seismic_CPML_2D_isotropic_second_order.f90 keeps its
! parameter block, fills a cpml_params from it, and replaces its time loop
! (2D:550-735, 3D:802-1245) with cpml_run; its seismogram arrays
! sisvx(NSTEP,NREC) are passed unchanged, because their memory order is the
! C layout [nrec][nstep]. Build:
!   gfortran -c include/cpml_gpu.f90
!   gfortran prog.f90 cpml_gpu.o -L seismic_cpml_gb300/_build -lcpml
! Grid indices are 1-based as in the Fortran; every function returns CPML_OK
! (0) or a negative status (cpml_strerror gives its text).
module cpml_gpu
  use iso_c_binding
  implicit none

  integer(c_int), parameter :: CPML_OK = 0, CPML_ERR_INVALID = -1, CPML_ERR_CFL = -2
  integer(c_int), parameter :: CPML_ERR_OOM = -3, CPML_ERR_UNSTABLE = -4, CPML_ERR_TIMEOUT = -5
  integer(c_int), parameter :: CPML_ERR_CUDA = -6, CPML_ERR_NOT_READY = -7, CPML_ERR_IO = -8
  integer(c_int), parameter :: CPML_ERR_RANGE = -9
  integer(c_int), parameter :: CPML_STF_DGAUSSIAN = 0, CPML_STF_GAUSSIAN = 1, CPML_STF_RICKER = 2
  integer(c_int), parameter :: CPML_FLAG_ENERGY = 1, CPML_FLAG_EP_PHYSICAL = 2, CPML_FLAG_NO_STABILITY = 4
  integer(c_int), parameter :: CPML_SCHEME_CPML = 0, CPML_SCHEME_SPLIT = 1
  integer(c_int), parameter :: CPML_KERNEL_AUTO = 0, CPML_KERNEL_TWO_SWEEP = 1, CPML_KERNEL_FUSED = 2
  integer(c_int), parameter :: CPML_KERNEL_PERSISTENT = 3, CPML_KERNEL_CLUSTER = 4
  integer(c_int), parameter :: CPML_FIELD_VX = 0, CPML_FIELD_VY = 1, CPML_FIELD_VZ = 2
  integer(c_int), parameter :: CPML_FIELD_SXX = 3, CPML_FIELD_SYY = 4, CPML_FIELD_SZZ = 5
  integer(c_int), parameter :: CPML_FIELD_SXY = 6, CPML_FIELD_SXZ = 7, CPML_FIELD_SYZ = 8

  ! mirrors struct cpml_params field by field
  type, bind(c) :: cpml_params
    integer(c_int32_t) :: ndim, nx, ny, nz, nstep, npoints_pml
    integer(c_int32_t) :: use_pml(6)
    integer(c_int32_t) :: isource, jsource, ksource, stf, it_display, flags
    integer(c_int32_t) :: order, scheme
    integer(c_int32_t) :: reserved_i(2)
    real(c_double) :: deltax, deltay, deltaz, deltat
    real(c_double) :: cp, cs, rho, f0, t0, factor, angle_force
    real(c_double) :: npower, k_max_pml, alpha_max_pml, rcoef
    real(c_double) :: reserved_d(4)
  end type

  interface
    ! ---- parameter blocks, set-up helpers --------------------------------
    integer(c_int) function cpml_params_default_2d(p) bind(c)
      import; type(cpml_params), intent(out) :: p
    end function
    integer(c_int) function cpml_params_default_2d_fourth(p) bind(c)
      import; type(cpml_params), intent(out) :: p
    end function
    integer(c_int) function cpml_params_default_2d_split(p) bind(c)
      import; type(cpml_params), intent(out) :: p
    end function
    integer(c_int) function cpml_params_default_3d(p) bind(c)
      import; type(cpml_params), intent(out) :: p
    end function
    real(c_double) function cpml_courant(p, cp_max) bind(c)
      import; type(cpml_params), intent(in) :: p; real(c_double), value :: cp_max
    end function
    integer(c_int) function cpml_nearest_gridpoint(nx, ny, dx, dy, x, y, i, j) bind(c)
      import; integer(c_int), value :: nx, ny; real(c_double), value :: dx, dy, x, y
      integer(c_int), intent(out) :: i, j
    end function
    ! ---- one simulation ------------------------------------------------------
    integer(c_int) function cpml_create(p, h) bind(c)
      import; type(cpml_params), intent(in) :: p; type(c_ptr), intent(out) :: h
    end function
    integer(c_int) function cpml_set_model(h, lam, mu, rho) bind(c)
      import; type(c_ptr), value :: h; real(c_float), intent(in) :: lam(*), mu(*), rho(*)
    end function
    integer(c_int) function cpml_set_receivers(h, nrec, ix, iy, iz) bind(c)
      import; type(c_ptr), value :: h; integer(c_int), value :: nrec
      integer(c_int), intent(in) :: ix(*), iy(*), iz(*)
    end function
    integer(c_int) function cpml_reset(h) bind(c)
      import; type(c_ptr), value :: h
    end function
    integer(c_int) function cpml_run(h, nsteps) bind(c)
      import; type(c_ptr), value :: h; integer(c_int), value :: nsteps
    end function
    integer(c_int) function cpml_status(h, it, vmax) bind(c)
      import; type(c_ptr), value :: h; integer(c_int), intent(out) :: it; real(c_double), intent(out) :: vmax
    end function
    ! vz: c_loc of a 3D trace array, or c_null_ptr in 2D
    integer(c_int) function cpml_get_seismograms(h, vx, vy, vz) bind(c)
      import; type(c_ptr), value :: h; real(c_double) :: vx(*), vy(*); type(c_ptr), value :: vz
    end function
    integer(c_int) function cpml_get_energy(h, ek, ep) bind(c)
      import; type(c_ptr), value :: h; real(c_double) :: ek(*), ep(*)
    end function
    integer(c_int) function cpml_get_field(h, field, out) bind(c)
      import; type(c_ptr), value :: h; integer(c_int), value :: field; real(c_float) :: out(*)
    end function
    integer(c_int) function cpml_set_field(h, field, in) bind(c)
      import; type(c_ptr), value :: h; integer(c_int), value :: field; real(c_float), intent(in) :: in(*)
    end function
    integer(c_int) function cpml_get_plane(h, field, axis, idx, out) bind(c)
      import; type(c_ptr), value :: h; integer(c_int), value :: field, axis, idx
      real(c_float) :: out(*)
    end function
    ! ---- checkpoint / restart (a snapshot is an opaque byte buffer) --------
    integer(c_int) function cpml_state_size(h, bytes) bind(c)
      import; type(c_ptr), value :: h; integer(c_size_t), intent(out) :: bytes
    end function
    integer(c_int) function cpml_save_state(h, buf, bytes) bind(c)
      import; type(c_ptr), value :: h; integer(c_int8_t) :: buf(*); integer(c_size_t), value :: bytes
    end function
    integer(c_int) function cpml_load_state(h, buf, bytes) bind(c)
      import; type(c_ptr), value :: h; integer(c_int8_t), intent(in) :: buf(*)
      integer(c_size_t), value :: bytes
    end function
    ! ---- tuning ----------------------------------------------------------------
    integer(c_int) function cpml_set_tuning(h, kernel, tile_y, zchunk, lookahead) bind(c)
      import; type(c_ptr), value :: h; integer(c_int), value :: kernel, tile_y, zchunk, lookahead
    end function
    integer(c_int) function cpml_autotune(h, trial_steps, cache_path, kernel, tile_y, zchunk, ms) bind(c)
      import; type(c_ptr), value :: h; integer(c_int), value :: trial_steps
      character(kind=c_char), intent(in) :: cache_path(*)
      integer(c_int), intent(out) :: kernel, tile_y, zchunk; real(c_double), intent(out) :: ms
    end function
    subroutine cpml_destroy(h) bind(c)
      import; type(c_ptr), value :: h
    end subroutine
    ! ---- many 2D shots -----------------------------------------------------
    integer(c_int) function cpml_batch_create(n, params, b) bind(c)
      import; integer(c_int), value :: n; type(cpml_params), intent(in) :: params(*)
      type(c_ptr), intent(out) :: b
    end function
    integer(c_int) function cpml_batch_set_model(b, shot, lam, mu, rho) bind(c)
      import; type(c_ptr), value :: b; integer(c_int), value :: shot
      real(c_float), intent(in) :: lam(*), mu(*), rho(*)
    end function
    integer(c_int) function cpml_batch_set_receivers(b, shot, nrec, ix, iy) bind(c)
      import; type(c_ptr), value :: b; integer(c_int), value :: shot, nrec
      integer(c_int), intent(in) :: ix(*), iy(*)
    end function
    integer(c_int) function cpml_batch_set_tuning(b, depth, tile_y) bind(c)
      import; type(c_ptr), value :: b; integer(c_int), value :: depth, tile_y
    end function
    integer(c_int) function cpml_batch_autotune(b, trial_steps, depth, tile_y, ms) bind(c)
      import; type(c_ptr), value :: b; integer(c_int), value :: trial_steps
      integer(c_int), intent(out) :: depth, tile_y; real(c_double), intent(out) :: ms
    end function
    integer(c_int) function cpml_batch_run(b) bind(c)
      import; type(c_ptr), value :: b
    end function
    integer(c_int) function cpml_batch_get_seismograms(b, shot, vx, vy) bind(c)
      import; type(c_ptr), value :: b; integer(c_int), value :: shot
      real(c_double) :: vx(*), vy(*)
    end function
    subroutine cpml_batch_destroy(b) bind(c)
      import; type(c_ptr), value :: b
    end subroutine
    ! ---- the reference's output files -------------------------------------
    integer(c_int) function cpml_write_seismograms(dir, vx, vy, vz, nt, nrec, deltat) bind(c)
      import; character(kind=c_char), intent(in) :: dir(*)
      real(c_double), intent(in) :: vx(*), vy(*); type(c_ptr), value :: vz
      integer(c_int), value :: nt, nrec
      real(c_double), value :: deltat
    end function
    integer(c_int) function cpml_write_seismograms_su(dir, vx, vy, vz, nt, nrec, deltat) bind(c)
      import; character(kind=c_char), intent(in) :: dir(*)
      real(c_double), intent(in) :: vx(*), vy(*); type(c_ptr), value :: vz
      integer(c_int), value :: nt, nrec
      real(c_double), value :: deltat
    end function
    integer(c_int) function cpml_write_energy(dir, ek, ep, nt, deltat, ncol) bind(c)
      import; character(kind=c_char), intent(in) :: dir(*)
      real(c_double), intent(in) :: ek(*), ep(*); integer(c_int), value :: nt, ncol
      real(c_double), value :: deltat
    end function
  end interface
end module cpml_gpu
