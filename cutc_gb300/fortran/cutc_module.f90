! Fortran binding of libcutcint.so (GB300 engine), drop-in for CuTC's
! src/cutc_module.f90.  The array layouts are the reference's
! (src/cutc_module.f90:24-35).  The argument list is the one the C entry point
! actually has (src/cutc_int.c:15-20): six launch integers, where the
! reference module declares only two (nBlocks, blockSize), which shifts every
! later argument.  The launch integers are validated like the reference and
! otherwise ignored.  The function returns the status (0 = success, -1 = bad
! launch dimensions, other negative values = errors; see include/cutc_int.h).

module cutc_module

  use, intrinsic :: iso_c_binding

  implicit none

  interface

    integer(c_int) function cutc_int(nxBlocks, nyBlocks, nzBlocks,            &
                                     blockxSize, blockySize, blockzSize,      &
                                     n_grid1, n_grid2, n_ao, n_nuc, size_bh,  &
                                     r1, wr1, r2, wr2, rn,                    &
                                     aos_data1, aos_data2,                    &
                                     c_bh, m_bh, n_bh, o_bh,                  &
                                     int2_grad1_u12_ao, int_2e_ao) bind(C, name = "cutc_int")
      import c_int, c_double
      integer(c_int), intent(in), value :: nxBlocks, nyBlocks, nzBlocks
      integer(c_int), intent(in), value :: blockxSize, blockySize, blockzSize
      integer(c_int), intent(in), value :: n_grid1, n_grid2
      integer(c_int), intent(in), value :: n_ao
      integer(c_int), intent(in), value :: n_nuc
      integer(c_int), intent(in), value :: size_bh
      real(c_double), intent(in)        :: r1(3,n_grid1)
      real(c_double), intent(in)        :: wr1(n_grid1)
      real(c_double), intent(in)        :: r2(3,n_grid2)
      real(c_double), intent(in)        :: wr2(n_grid2)
      real(c_double), intent(in)        :: rn(3,n_nuc)
      real(c_double), intent(in)        :: aos_data1(n_grid1,n_ao,4)
      real(c_double), intent(in)        :: aos_data2(n_grid2,n_ao,4)
      real(c_double), intent(in)        :: c_bh(size_bh,n_nuc)
      integer(c_int), intent(in)        :: m_bh(size_bh,n_nuc)
      integer(c_int), intent(in)        :: n_bh(size_bh,n_nuc)
      integer(c_int), intent(in)        :: o_bh(size_bh,n_nuc)
      real(c_double), intent(out)       :: int2_grad1_u12_ao(n_ao,n_ao,n_grid1,3)
      real(c_double), intent(out)       :: int_2e_ao(n_ao,n_ao,n_ao,n_ao)
    end function cutc_int

  end interface

end module cutc_module
