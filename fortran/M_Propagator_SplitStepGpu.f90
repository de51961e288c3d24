!> GB300 second-order split step (JSON branch `propagator.splitStepGpu`).
!> Registered next to `splitStep` in Propagator_Fabricate
!> (src/Propagator/S_Propagator.f90:46-57):
!>
!>     else if (Json_GetExistence("propagator.splitStepGpu")) then
!>       call Propagator_SplitStepGpu_Fabricate
!>
!> Part of the CodyFortran build; needs the mctdhxGpu method (its context).
module M_Propagator_SplitStepGpu
  use M_Utils_Types

  implicit none

  integer(I32) :: Propagator_SplitStepGpu_krylovDim = 32
  real(R64) :: Propagator_SplitStepGpu_tolerance = 1e-10_R64
  integer(I32) :: Propagator_SplitStepGpu_maxRestarts = 8
  integer(I32) :: Propagator_SplitStepGpu_useMetric = 0

  interface
    module subroutine Propagator_SplitStepGpu_Fabricate
    end subroutine
  end interface

end module
