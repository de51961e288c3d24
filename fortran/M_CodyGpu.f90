!> ISO_C_BINDING interface to the GB300 engine (include/cody_gpu.h).
!>
!> Standalone: it depends only on the intrinsic iso_c_binding module, so it
!> compiles outside the CodyFortran tree (`make -C fortran` with gfortran).
!> The GPU S_ submodules of this directory use it to bind the reference's
!> procedure pointers to the C ABI.  Every entry point returns an integer
!> status; CodyGpu_Check turns a nonzero status into `error stop` with the
!> library's message, the reference's own failure convention.
module M_CodyGpu
  use, intrinsic :: iso_c_binding
  implicit none
  private :: c_string

  !> The context of the run (one system; created by the GPU Method setup).
  type(c_ptr), save :: CodyGpu_ctx = c_null_ptr

  integer(c_int), parameter :: CGPU_OK = 0
  integer(c_int), parameter :: CGPU_GRID_CONST = 0, CGPU_GRID_FEDVR = 1
  integer(c_int), parameter :: CGPU_INT_TOEPLITZ = 0, CGPU_INT_DENSE = 1
  integer(c_int), parameter :: CGPU_LASER_NONE = 0, CGPU_LASER_SIN2 = 1, CGPU_LASER_SAMPLED = 2
  integer(c_int), parameter :: CGPU_METHOD_MCTDHX = 0, CGPU_METHOD_TDCI = 1
  integer(c_int), parameter :: CGPU_PREC_FP64 = 0, CGPU_PREC_MIXED_FX = 3, CGPU_PREC_MIXED_FX6 = 4
  integer(c_int), parameter :: CGPU_TD_FULL = 0, CGPU_TD_ORBS_LIN = 1, CGPU_TD_NONLIN = 2, CGPU_TD_TDCI = 3
  integer(c_int), parameter :: CGPU_TUNE_CACHED = 0, CGPU_TUNE_FORCE = 1

  !> cgpu_desc: the configuration tree of one run, field for field.
  type, bind(C) :: T_CgpuDesc
    integer(c_int) :: grid_kind = 0
    real(c_double) :: xmin = 0, xmax = 0
    integer(c_int) :: n_points = 0, n_elements = 0, n_locals = 0, xmin_excluded = 0, xmax_excluded = 0
    integer(c_int) :: n_body_types = 0, n_bodies(4) = 0, n_orbs(4) = 0
    real(c_double) :: body_mass(4) = 1
    integer(c_int) :: restricted = 0
    real(c_double) :: regularization = 1e-10_c_double
    integer(c_int) :: n_nuclei = 0
    real(c_double) :: nuc_position(8) = 0, nuc_charge(8) = 0, nuc_softening1(8) = 0, nuc_softening2(8) = 0
    real(c_double) :: nuc_dampening(8) = 0
    integer(c_int) :: has_interaction = 0
    real(c_double) :: int_strength = 0, int_softening1 = 0, int_softening2 = 0, int_dampening = 0
    integer(c_int) :: int_kind = 0, laser_kind = 0
    real(c_double) :: laser_E0 = 0, laser_omega = 0, laser_n_cycles = 0, laser_cep = 0, laser_t_start = 0
    type(c_ptr) :: field_samples = c_null_ptr
    integer(c_int) :: n_field_samples = 0
    real(c_double) :: field_dt = 1, field_t0 = 0
    integer(c_int) :: method = 0, precision = 0, max_krylov = 32, krylov_window = 0
  end type

  interface
    integer(c_int) function cgpu_ctx_create(desc, ctx) bind(C, name="cgpu_ctx_create")
      import :: c_int, c_ptr, T_CgpuDesc
      type(T_CgpuDesc), intent(in) :: desc
      type(c_ptr), intent(out) :: ctx
    end function
    integer(c_int) function cgpu_ctx_destroy(ctx) bind(C, name="cgpu_ctx_destroy")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
    end function
    type(c_ptr) function cgpu_last_error(ctx) bind(C, name="cgpu_last_error")
      import :: c_ptr
      type(c_ptr), value :: ctx
    end function
    type(c_ptr) function cgpu_last_global_error() bind(C, name="cgpu_last_global_error")
      import :: c_ptr
    end function
    integer(c_int) function cgpu_sizes(ctx, sizes) bind(C, name="cgpu_sizes")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), intent(out) :: sizes(6)
    end function
    ! ---- Method pointers
    integer(c_int) function cgpu_time_derivative(ctx, which, dState, state, time) bind(C, name="cgpu_time_derivative")
      import :: c_int, c_ptr, c_double, c_double_complex
      type(c_ptr), value :: ctx
      integer(c_int), value :: which
      complex(c_double_complex), intent(out) :: dState(*)
      complex(c_double_complex), intent(in) :: state(*)
      real(c_double), value :: time
    end function
    integer(c_int) function cgpu_energy(ctx, state, time, energy) bind(C, name="cgpu_energy")
      import :: c_int, c_ptr, c_double, c_double_complex
      type(c_ptr), value :: ctx
      complex(c_double_complex), intent(in) :: state(*)
      real(c_double), value :: time
      real(c_double), intent(out) :: energy
    end function
    integer(c_int) function cgpu_fill_h1(ctx, h1, orbs, time) bind(C, name="cgpu_fill_h1")
      import :: c_int, c_ptr, c_double, c_double_complex
      type(c_ptr), value :: ctx
      complex(c_double_complex), intent(out) :: h1(*)
      complex(c_double_complex), intent(in) :: orbs(*)
      real(c_double), value :: time
    end function
    integer(c_int) function cgpu_fill_h2(ctx, h2, orbs, time) bind(C, name="cgpu_fill_h2")
      import :: c_int, c_ptr, c_double, c_double_complex
      type(c_ptr), value :: ctx
      complex(c_double_complex), intent(out) :: h2(*)
      complex(c_double_complex), intent(in) :: orbs(*)
      real(c_double), value :: time
    end function
    ! ---- Coeffs pointers: absent Fortran optionals are c_null_ptr
    integer(c_int) function cgpu_ci_apply_h1_fill_rdm1(ctx, coeffs, rdm1, dCoeffs, h1) &
      bind(C, name="cgpu_ci_apply_h1_fill_rdm1")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx, coeffs, rdm1, dCoeffs, h1
    end function
    integer(c_int) function cgpu_ci_apply_h2_fill_rdm2(ctx, coeffs, rdm2, dCoeffs, h2) &
      bind(C, name="cgpu_ci_apply_h2_fill_rdm2")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx, coeffs, rdm2, dCoeffs, h2
    end function
    integer(c_int) function cgpu_project_coeffs(ctx, dCoeffs, coeffs) bind(C, name="cgpu_project_coeffs")
      import :: c_int, c_ptr, c_double_complex
      type(c_ptr), value :: ctx
      complex(c_double_complex), intent(inout) :: dCoeffs(*)
      complex(c_double_complex), intent(in) :: coeffs(*)
    end function
    ! ---- Orbs pointers
    integer(c_int) function cgpu_project_orbs(ctx, dOrbs, orbs) bind(C, name="cgpu_project_orbs")
      import :: c_int, c_ptr, c_double_complex
      type(c_ptr), value :: ctx
      complex(c_double_complex), intent(inout) :: dOrbs(*)
      complex(c_double_complex), intent(in) :: orbs(*)
    end function
    integer(c_int) function cgpu_orthonormalize_orbs(ctx, orbs) bind(C, name="cgpu_orthonormalize_orbs")
      import :: c_int, c_ptr, c_double_complex
      type(c_ptr), value :: ctx
      complex(c_double_complex), intent(inout) :: orbs(*)
    end function
    ! ---- Sys* pointers (one orbital; bt 1-based, 0 for an absent bt_)
    integer(c_int) function cgpu_sys_kinetic_multiply(ctx, dOrb, orb, time, bt) bind(C, name="cgpu_sys_kinetic_multiply")
      import :: c_int, c_ptr, c_double, c_double_complex
      type(c_ptr), value :: ctx
      complex(c_double_complex), intent(out) :: dOrb(*)
      complex(c_double_complex), intent(in) :: orb(*)
      real(c_double), value :: time
      integer(c_int), value :: bt
    end function
    integer(c_int) function cgpu_sys_potential_fill(ctx, potential, time, bt) bind(C, name="cgpu_sys_potential_fill")
      import :: c_int, c_ptr, c_double, c_double_complex
      type(c_ptr), value :: ctx
      complex(c_double_complex), intent(out) :: potential(*)
      real(c_double), value :: time
      integer(c_int), value :: bt
    end function
    integer(c_int) function cgpu_sys_potential_multiply(ctx, dOrb, potential, orb) &
      bind(C, name="cgpu_sys_potential_multiply")
      import :: c_int, c_ptr, c_double_complex
      type(c_ptr), value :: ctx
      complex(c_double_complex), intent(out) :: dOrb(*)
      complex(c_double_complex), intent(in) :: potential(*), orb(*)
    end function
    integer(c_int) function cgpu_sys_interaction_src(ctx, src, orbConjg, orb) bind(C, name="cgpu_sys_interaction_src")
      import :: c_int, c_ptr, c_double_complex
      type(c_ptr), value :: ctx
      complex(c_double_complex), intent(out) :: src(*)
      complex(c_double_complex), intent(in) :: orbConjg(*), orb(*)
    end function
    integer(c_int) function cgpu_sys_interaction_potential(ctx, potential, src, time, bt1, bt2) &
      bind(C, name="cgpu_sys_interaction_potential")
      import :: c_int, c_ptr, c_double, c_double_complex
      type(c_ptr), value :: ctx
      complex(c_double_complex), intent(out) :: potential(*)
      complex(c_double_complex), intent(in) :: src(*)
      real(c_double), value :: time
      integer(c_int), value :: bt1, bt2
    end function
    integer(c_int) function cgpu_sys_interaction_multiply(ctx, res, potential, orb) &
      bind(C, name="cgpu_sys_interaction_multiply")
      import :: c_int, c_ptr, c_double_complex
      type(c_ptr), value :: ctx
      complex(c_double_complex), intent(out) :: res(*)
      complex(c_double_complex), intent(in) :: potential(*), orb(*)
    end function
    ! ---- IntegratorList / Propagator pointers
    integer(c_int) function cgpu_integrate_sil(ctx, which, state, t0, t1, krylovDim, tolerance, maxRestarts, metric, &
                                               warnings) bind(C, name="cgpu_integrate_sil")
      import :: c_int, c_ptr, c_double, c_double_complex
      type(c_ptr), value :: ctx, metric
      integer(c_int), value :: which, krylovDim, maxRestarts
      complex(c_double_complex), intent(inout) :: state(*)
      real(c_double), value :: t0, t1, tolerance
      integer(c_int), intent(out) :: warnings
    end function
    integer(c_int) function cgpu_integrate_rk4(ctx, which, state, t0, t1) bind(C, name="cgpu_integrate_rk4")
      import :: c_int, c_ptr, c_double, c_double_complex
      type(c_ptr), value :: ctx
      integer(c_int), value :: which
      complex(c_double_complex), intent(inout) :: state(*)
      real(c_double), value :: t0, t1
    end function
    integer(c_int) function cgpu_propagate_split2(ctx, state, t0, t1, krylovDim, tolerance, maxRestarts, useMetric) &
      bind(C, name="cgpu_propagate_split2")
      import :: c_int, c_ptr, c_double, c_double_complex
      type(c_ptr), value :: ctx
      complex(c_double_complex), intent(inout) :: state(*)
      real(c_double), value :: t0, t1, tolerance
      integer(c_int), value :: krylovDim, maxRestarts, useMetric
    end function
    ! ---- resident state (a driver loop that keeps the state on the GPU)
    integer(c_int) function cgpu_state_upload(ctx, state) bind(C, name="cgpu_state_upload")
      import :: c_int, c_ptr, c_double_complex
      type(c_ptr), value :: ctx
      complex(c_double_complex), intent(in) :: state(*)
    end function
    integer(c_int) function cgpu_state_download(ctx, state) bind(C, name="cgpu_state_download")
      import :: c_int, c_ptr, c_double_complex
      type(c_ptr), value :: ctx
      complex(c_double_complex), intent(out) :: state(*)
    end function
    integer(c_int) function cgpu_propagate_resident(ctx, t0, dt, nSteps, krylovDim, useMetric, useGraph) &
      bind(C, name="cgpu_propagate_resident")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), value :: t0, dt
      integer(c_int), value :: nSteps, krylovDim, useMetric, useGraph
    end function
    integer(c_int) function cgpu_energy_resident(ctx, time, energy) bind(C, name="cgpu_energy_resident")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), value :: time
      real(c_double), intent(out) :: energy
    end function
    integer(c_int) function cgpu_autotune(ctx, cachePath, mode, report, reportLen) bind(C, name="cgpu_autotune")
      import :: c_int, c_ptr, c_char
      type(c_ptr), value :: ctx
      character(kind=c_char), intent(in) :: cachePath(*)
      integer(c_int), value :: mode, reportLen
      type(c_ptr), value :: report
    end function
    integer(c_long) function c_strlen(s) bind(C, name="strlen")
      import :: c_long, c_ptr
      type(c_ptr), value :: s
    end function
  end interface

contains

  !> The NUL-terminated C string at p as a Fortran string.
  function c_string(p) result(s)
    type(c_ptr), intent(in) :: p
    character(len=:), allocatable :: s
    character(kind=c_char), pointer :: chars(:)
    integer :: n, i
    if (.not. c_associated(p)) then
      s = ""
      return
    end if
    n = int(c_strlen(p))
    call c_f_pointer(p, chars, [n])
    allocate (character(len=n) :: s)
    do i = 1, n
      s(i:i) = chars(i)
    end do
  end function

  !> error stop with the library's message when rc is not CGPU_OK.
  subroutine CodyGpu_Check(rc, what)
    integer(c_int), intent(in) :: rc
    character(len=*), intent(in) :: what
    if (rc == CGPU_OK) return
    if (c_associated(CodyGpu_ctx)) then
      write (*, *) "cody_gpu: ", what, ": ", c_string(cgpu_last_error(CodyGpu_ctx))
    else
      write (*, *) "cody_gpu: ", what, ": ", c_string(cgpu_last_global_error())
    end if
    error stop "cody_gpu call failed"
  end subroutine

end module
