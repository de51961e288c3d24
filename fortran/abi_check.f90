!> A Fortran host on the C ABI through M_CodyGpu: the He1d system of the
!> reference's golden tests (21-point grid, 4 + 4 orbitals), one context,
!> harmonic-like start orbitals orthonormalised by the library, the energy,
!> one split step and the energy again.  Prints "abi_check OK" when the
!> calls succeed and the norm of the state is conserved to 1e-10.
program abi_check
  use, intrinsic :: iso_c_binding
  use M_CodyGpu
  implicit none

  type(T_CgpuDesc) :: desc
  integer(c_int) :: sizes(6), nG, nOS, nC, i, o
  real(c_double), allocatable :: x(:)
  complex(c_double_complex), allocatable :: state(:), orbs(:)
  real(c_double) :: e0, e1, n0, n1

  desc % grid_kind = CGPU_GRID_CONST
  desc % xmin = -20.0_c_double
  desc % xmax = 20.0_c_double
  desc % n_points = 21
  desc % n_body_types = 2
  desc % n_bodies(1:2) = 1
  desc % n_orbs(1:2) = 4
  desc % n_nuclei = 1
  desc % nuc_charge(1) = 2.0_c_double
  desc % nuc_softening2(1) = 1.0_c_double
  desc % has_interaction = 1
  desc % int_strength = 1.0_c_double
  desc % int_softening2 = 1.0_c_double
  desc % int_kind = CGPU_INT_TOEPLITZ
  desc % max_krylov = 24

  call CodyGpu_Check(cgpu_ctx_create(desc, CodyGpu_ctx), "cgpu_ctx_create")
  call CodyGpu_Check(cgpu_sizes(CodyGpu_ctx, sizes), "cgpu_sizes")
  nG = sizes(1)
  nOS = sizes(3)
  nC = sizes(4)
  allocate (x(nG), orbs(nG * nOS), state(nC + nG * nOS))
  do i = 1, nG
    x(i) = -20.0_c_double + 2.0_c_double * (i - 1)
  end do
  do o = 0, nOS - 1
    do i = 1, nG
      orbs(o * nG + i) = cmplx(x(i)**mod(o, 4) * exp(-x(i)**2 / 4.0_c_double), 0.0_c_double, c_double_complex)
    end do
  end do
  call CodyGpu_Check(cgpu_orthonormalize_orbs(CodyGpu_ctx, orbs), "cgpu_orthonormalize_orbs")
  state = (0.0_c_double, 0.0_c_double)
  state(1) = (1.0_c_double, 0.0_c_double)
  state(nC + 1:) = orbs
  call CodyGpu_Check(cgpu_energy(CodyGpu_ctx, state, 0.0_c_double, e0), "cgpu_energy")
  n0 = sqrt(sum(abs(state)**2))
  call CodyGpu_Check(cgpu_propagate_split2(CodyGpu_ctx, state, 0.0_c_double, 1e-3_c_double, 24_c_int, &
                                           1e-12_c_double, 8_c_int, 0_c_int), "cgpu_propagate_split2")
  call CodyGpu_Check(cgpu_energy(CodyGpu_ctx, state, 1e-3_c_double, e1), "cgpu_energy")
  n1 = sqrt(sum(abs(state)**2))
  write (*, *) "energy", e0, e1, "norm", n0, n1
  call CodyGpu_Check(cgpu_ctx_destroy(CodyGpu_ctx), "cgpu_ctx_destroy")
  if (abs(n1 - n0) > 1e-10_c_double) error stop "abi_check: norm not conserved"
  write (*, *) "abi_check OK"
end program
