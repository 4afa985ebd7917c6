! Test infrastructure (read by f90c.py, never compiled into the product).
!
! 2d_rtm_restart/working_Src/born-mod.f90:521,529,537,545 call
! explosive_sourcex / explosive_sourcez with six arguments
! (adj, add, source, xsource, zsource, data), but the source module it uses,
! working_Src/source-mod.f90:77-100, defines both with four
! (source, xsource, zsource, data), so the program does not build as shipped.
! These are the four-argument bodies behind the six-argument interface: every
! call in born-mod.f90 passes adj = .false., add = .true., for which the body
! adds the source sample at (zsource, xsource).  f90c.py places them in
! source_mod, so nz and nx are that module's (set by source_init).
module source_shim

  implicit none
  integer, private :: nz, nx

  contains

  subroutine explosive_sourcex(adj, add, source, xsource, zsource, data)
    logical                  :: adj, add
    real                     :: source
    integer                  :: xsource, zsource
    real, dimension(nz,nx)   :: data

    data(zsource, xsource) = data(zsource, xsource) + source
  endsubroutine

  subroutine explosive_sourcez(adj, add, source, xsource, zsource, data)
    logical                  :: adj, add
    real                     :: source
    integer                  :: xsource, zsource
    real, dimension(nz,nx)   :: data

    data(zsource, xsource) = data(zsource, xsource) + source
  endsubroutine

endmodule
