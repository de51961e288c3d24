!> The MCTDHX method on the GB300 engine: the procedure pointers the CPU
!> submodule binds (src/Method/Mb/OrbBased/Mctdhx/S_Method_Mb_OrbBased_Mctdhx.f90:15-37)
!> bound to wrappers of the C ABI (M_CodyGpu).  Method_state keeps the
!> reference layout [C(nC) | orbs(nG, nOS)] and stays a Fortran array: the
!> wrappers pass it to the library, which copies it to and from the device.
!> Setup fills the library's configuration from the same JSON keys the CPU
!> modules read (grid.linear.*, sysKinetic.linear.laplacian.bodyMass,
!> sysPotential.linear.softYukawa.*, sysInteraction.linear.softYukawa.*,
!> method.mb.*, orbs.restrictedQ) and creates the context once.
submodule(M_Method_Mb_OrbBased_MctdhxGpu) S_Method_Mb_OrbBased_MctdhxGpu
  use, intrinsic :: iso_c_binding
  use M_CodyGpu

  implicit none

contains

!~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~
  module subroutine Method_Mb_OrbBased_MctdhxGpu_Fabricate
    use M_Utils_Say
    use M_Method
    use M_Method_Mb_OrbBased

    call Say_Fabricate("method.manbody.orbbased.mctdhxGpu")

    Method_Setup => Setup
    Method_Mb_OrbBased_FillRdm1 => FillRdm1
    Method_Mb_OrbBased_FillRdm2 => FillRdm2
    Method_TimeDerivative => TimeDerivative
    Method_Mb_OrbBased_TimeDerivativeOrbsLin => TimeDerivativeOrbsLin
    Method_Mb_OrbBased_TimeDerivativeCoeffsPlusOrbsNonLin => TimeDerivativeCoeffsPlusOrbsNonLin
    Method_GetEnergy => GetEnergy

  end subroutine

!~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~
  !> The library's configuration from the JSON keys of the run.
  subroutine FillDesc(desc)
    use M_Utils_Json
    use M_Method_Mb
    use M_Method_Mb_OrbBased

    type(T_CgpuDesc), intent(out) :: desc
    real(R64), allocatable :: position(:), charge(:), s1(:), s2(:), damp(:), mass(:)
    integer(I32) :: nBt, nNuc

    desc % xmin = Json_Get("grid.linear.xmin", -10.0_R64)
    desc % xmax = Json_Get("grid.linear.xmax", 10.0_R64)
    if (Json_GetExistence("grid.linear.const")) then
      desc % grid_kind = CGPU_GRID_CONST
      desc % n_points = Json_Get("grid.linear.const.nPoints", 100)
    else
      ! 1D FEDVR: order + 1 Gauss-Lobatto points per element, nElements * order + 1 points
      desc % grid_kind = CGPU_GRID_FEDVR
      desc % n_elements = Json_Get("grid.linear.fedvr.nElements", 10)
      desc % n_locals = Json_Get("grid.linear.fedvr.order", 8) + 1
    end if

    nBt = Method_Mb_nBodyTypes
    desc % n_body_types = nBt
    desc % n_bodies(1:nBt) = Method_Mb_nBodies(1:nBt)
    desc % n_orbs(1:nBt) = Method_Mb_OrbBased_nOrbs(1:nBt)
    mass = Json_Get("sysKinetic.linear.laplacian.bodyMass", [(1.0_R64, nNuc=1, nBt)])
    desc % body_mass(1:nBt) = mass(1:nBt)
    desc % restricted = merge(1, 0, Json_Get("orbs.restrictedQ", .false.))
    desc % regularization = Method_Mb_OrbBased_regularizationParameter

    position = Json_Get("sysPotential.linear.softYukawa.position", [0.0_R64])
    charge = Json_Get("sysPotential.linear.softYukawa.charge", [1.0_R64])
    s1 = Json_Get("sysPotential.linear.softYukawa.softening1", [1.0_R64])
    s2 = Json_Get("sysPotential.linear.softYukawa.softening2", [0.0_R64])
    damp = Json_Get("sysPotential.linear.softYukawa.dampening", [0.0_R64])
    nNuc = size(position)
    desc % n_nuclei = nNuc
    desc % nuc_position(1:nNuc) = position
    desc % nuc_charge(1:nNuc) = charge
    desc % nuc_softening1(1:nNuc) = s1
    desc % nuc_softening2(1:nNuc) = s2
    desc % nuc_dampening(1:nNuc) = damp

    if (Json_GetExistence("sysInteraction")) then
      desc % has_interaction = 1
      desc % int_strength = Json_Get("sysInteraction.linear.softYukawa.strength", 1.0_R64)
      desc % int_softening1 = Json_Get("sysInteraction.linear.softYukawa.softening1", 1.0_R64)
      desc % int_softening2 = Json_Get("sysInteraction.linear.softYukawa.softening2", 0.0_R64)
      desc % int_dampening = Json_Get("sysInteraction.linear.softYukawa.dampening", 0.0_R64)
      ! the reference's Toeplitz kernel K(|i-j| dx) holds on uniform grids only
      desc % int_kind = merge(CGPU_INT_TOEPLITZ, CGPU_INT_DENSE, desc % grid_kind == CGPU_GRID_CONST)
    end if

    if (Json_GetExistence("sysPotential.linear.laser")) then
      desc % laser_kind = CGPU_LASER_SIN2
      desc % laser_E0 = Json_Get("sysPotential.linear.laser.E0", 0.0_R64)
      desc % laser_omega = Json_Get("sysPotential.linear.laser.omega", 0.057_R64)
      desc % laser_n_cycles = Json_Get("sysPotential.linear.laser.nCycles", 4.0_R64)
      desc % laser_cep = Json_Get("sysPotential.linear.laser.cep", 0.0_R64)
      desc % laser_t_start = Json_Get("sysPotential.linear.laser.tStart", 0.0_R64)
    end if

    desc % method = CGPU_METHOD_MCTDHX
    desc % precision = Json_Get("method.mb.orbBased.mctdhxGpu.precision", 0)
    desc % max_krylov = Json_Get("method.mb.orbBased.mctdhxGpu.maxKrylov", 32)
  end subroutine

!~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~
  subroutine Setup
    use M_Utils_Say
    use M_Grid
    use M_Orbs
    use M_OrbsInit
    use M_Coeffs
    use M_CoeffsInit
    use M_Method

    type(T_CgpuDesc) :: desc
    integer(c_int) :: sizes(6)
    integer(I32) :: nG, nOS, nC

    call Say_Setup("method.manbody.orbbased.mctdhxGpu")

    call FillDesc(desc)
    call CodyGpu_Check(cgpu_ctx_create(desc, CodyGpu_ctx), "cgpu_ctx_create")
    call CodyGpu_Check(cgpu_sizes(CodyGpu_ctx, sizes), "cgpu_sizes")

    nG = Grid_nPoints
    nOS = Orbs_nOrbsInState
    nC = Coeffs_nCoeffs
    if (sizes(1) /= nG .or. sizes(3) /= nOS .or. sizes(4) /= nC) &
      error stop "mctdhxGpu: the GPU context disagrees with the Grid / Orbs / Coeffs sizes"

    allocate (Method_state(1:(nC + nG * nOS)))
    Coeffs_coeffs(1:nC) => Method_state(1:nC)
    Orbs_orbs(1:nG, 1:nOS) => Method_state(nC + 1:nC + nG * nOS)
    call CoeffsInit_Initialize(Coeffs_coeffs)
    call OrbsInit_Initialize(Orbs_orbs)
  end subroutine

!~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~
  subroutine FillRdm1(rdm1, state)
    use M_Method_Mb_OrbBased
    complex(R64), intent(out), allocatable :: rdm1(:, :)
    complex(R64), intent(in), contiguous, target :: state(:)
    integer(I32) :: nO
    nO = Method_Mb_OrbBased_nOrbsTotal
    allocate (rdm1(nO, nO))
    call CodyGpu_Check(cgpu_ci_apply_h1_fill_rdm1(CodyGpu_ctx, c_loc(state), c_loc(rdm1), c_null_ptr, c_null_ptr), &
                       "cgpu_ci_apply_h1_fill_rdm1")
  end subroutine

!~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~
  subroutine FillRdm2(rdm2, state)
    use M_Method_Mb_OrbBased
    complex(R64), intent(out), allocatable :: rdm2(:, :, :, :)
    complex(R64), intent(in), contiguous, target :: state(:)
    integer(I32) :: nO
    nO = Method_Mb_OrbBased_nOrbsTotal
    allocate (rdm2(nO, nO, nO, nO))
    call CodyGpu_Check(cgpu_ci_apply_h2_fill_rdm2(CodyGpu_ctx, c_loc(state), c_loc(rdm2), c_null_ptr, c_null_ptr), &
                       "cgpu_ci_apply_h2_fill_rdm2")
  end subroutine

!~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~
  !> Method_TimeDerivative (src/Method/M_Method.f90:82-90)
  subroutine TimeDerivative(dState, state, time)
    complex(R64), intent(out), contiguous :: dState(:)
    complex(R64), intent(in), contiguous :: state(:)
    real(R64), intent(in) :: time
    call CodyGpu_Check(cgpu_time_derivative(CodyGpu_ctx, CGPU_TD_FULL, dState, state, time), "cgpu_time_derivative")
  end subroutine

  !> Method_Mb_OrbBased_TimeDerivativeOrbsLin (src/Method/Mb/OrbBased/M_Method_Mb_OrbBased.f90:272-281)
  subroutine TimeDerivativeOrbsLin(dState, state, time)
    complex(R64), intent(out), contiguous :: dState(:)
    complex(R64), intent(in), contiguous :: state(:)
    real(R64), intent(in) :: time
    call CodyGpu_Check(cgpu_time_derivative(CodyGpu_ctx, CGPU_TD_ORBS_LIN, dState, state, time), &
                       "cgpu_time_derivative")
  end subroutine

  !> Method_Mb_OrbBased_TimeDerivativeCoeffsPlusOrbsNonLin (M_Method_Mb_OrbBased.f90:282-291)
  subroutine TimeDerivativeCoeffsPlusOrbsNonLin(dState, state, time)
    complex(R64), intent(out), contiguous :: dState(:)
    complex(R64), intent(in), contiguous :: state(:)
    real(R64), intent(in) :: time
    call CodyGpu_Check(cgpu_time_derivative(CodyGpu_ctx, CGPU_TD_NONLIN, dState, state, time), "cgpu_time_derivative")
  end subroutine

  !> Method_GetEnergy (src/Method/M_Method.f90:102-108) of Method_state
  function GetEnergy(time) result(res)
    use M_Method
    real(R64), intent(in) :: time
    real(R64) :: res
    real(c_double) :: e
    call CodyGpu_Check(cgpu_energy(CodyGpu_ctx, Method_state, time, e), "cgpu_energy")
    res = e
  end function

end submodule
