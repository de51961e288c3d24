!> Propagator_Propagate (src/Propagator/M_Propagator.f90:90-98) as one call of
!> the engine: SIL on OrbsLin for dt/2, RK4 on CoeffsPlusOrbsNonLin for dt,
!> SIL on OrbsLin for dt/2 (src/Propagator/SplitStep/Order2/S_Propagator_SplitStep_Order2.f90:52-77),
!> with the SIL parameters of the run's first integrator
!> (integratorList.sil1.{krylovDim, tolerance, maxRestarts},
!> src/IntegratorList/Sil/S_IntegratorList_Sil.f90:86-88) and, with
!> propagator.splitStepGpu.useMetric, the metric [1 on C | grid weights on
!> orbitals] that the FEDVR programs assign to metricWeights.
submodule(M_Propagator_SplitStepGpu) S_Propagator_SplitStepGpu
  use, intrinsic :: iso_c_binding
  use M_CodyGpu

  implicit none

contains

  module subroutine Propagator_SplitStepGpu_Fabricate
    use M_Utils_Say
    use M_Utils_Json
    use M_Propagator

    call Say_Fabricate("propagator.splitStepGpu")

    Propagator_SplitStepGpu_krylovDim = Json_Get("integratorList.sil1.krylovDim", 32)
    Propagator_SplitStepGpu_tolerance = Json_Get("integratorList.sil1.tolerance", 1.0e-10_R64)
    Propagator_SplitStepGpu_maxRestarts = Json_Get("integratorList.sil1.maxRestarts", 8)
    Propagator_SplitStepGpu_useMetric = merge(1, 0, Json_Get("propagator.splitStepGpu.useMetric", .false.))

    Propagator_Propagate => Propagate

  end subroutine

  subroutine Propagate(state, t0, t1)
    complex(R64), intent(inout), contiguous :: state(:)
    real(R64), intent(in) :: t0
    real(R64), intent(in) :: t1

    call CodyGpu_Check(cgpu_propagate_split2(CodyGpu_ctx, state, t0, t1, Propagator_SplitStepGpu_krylovDim, &
                                             Propagator_SplitStepGpu_tolerance, Propagator_SplitStepGpu_maxRestarts, &
                                             Propagator_SplitStepGpu_useMetric), "cgpu_propagate_split2")
  end subroutine

end submodule
