!> GB300 implementation of the MCTDHX method (JSON branch
!> `method.mb.orbBased.mctdhxGpu`).  Registered next to `mctdhx` in
!> Method_Mb_OrbBased_Fabricate (src/Method/Mb/OrbBased/S_Method_Mb_OrbBased.f90:116-127):
!>
!>     else if (Json_GetExistence("method.mb.orbBased.mctdhxGpu")) then
!>       call Method_Mb_OrbBased_MctdhxGpu_Fabricate
!>
!> Part of the CodyFortran build (uses its modules); compiled where gfortran
!> and the CodyFortran sources are present.
module M_Method_Mb_OrbBased_MctdhxGpu
  use M_Utils_Types

  implicit none

  interface
    module subroutine Method_Mb_OrbBased_MctdhxGpu_Fabricate
    end subroutine
  end interface

end module
