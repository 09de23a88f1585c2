! sesp_common_mod.f90 - ISO_C_BINDING interface to the COMMON-block layer of
! the GB300 engine (include/sesp_common.h).  A driver that keeps its state in
! the COMMON blocks of src/mybox.cmns points one sesp_cmn_domain per domain at
! its arrays (c_loc of rxw1, ryw1, ...), attaches them once after read_config,
! and then calls init_accel, move_surfactant_a, move_w1_a, move_w2_a,
! evalforces, move_surfactant_b, move_w1_b and move_w2_b, which the layer
! exports under their gfortran names.
module sesp_common_mod
  use iso_c_binding
  use sesp_mod, only: sesp_params
  implicit none

  integer(c_int), parameter :: SESP_CMN_NW3 = 300, SESP_CMN_NS29 = 580, SESP_CMN_NH = 10
  integer(c_int), parameter :: SESP_CMN_W1 = 0, SESP_CMN_W2 = 1, SESP_CMN_SURF = 2

  type, bind(C) :: sesp_cmn_domain
    integer(c_int) :: nw3, ns29
    type(c_ptr) :: rw1(3), rw2(3), vw1(3), vw2(3), fw1(3), fw2(3), aw1(3), aw2(3)
    type(c_ptr) :: rs(3), vs(3), as(3), fs(3)
    type(c_ptr) :: ictw1, ictw2, icts
    type(c_ptr) :: nh
  end type sesp_cmn_domain

  interface
    integer(c_int) function sesp_cmn_domain_count(n_cells, ndom) bind(C, name="sesp_cmn_domain_count")
      import :: c_int
      integer(c_int), intent(in) :: n_cells(3)
      integer(c_int), intent(out) :: ndom
    end function
    integer(c_int) function sesp_cmn_attach(p, doms, n_carbon, carbons, kb0) bind(C, name="sesp_cmn_attach")
      import :: c_int, c_double, sesp_params, sesp_cmn_domain
      type(sesp_params), intent(in) :: p
      type(sesp_cmn_domain), intent(inout) :: doms(*)
      integer(c_int), value :: n_carbon, kb0
      real(c_double), intent(in) :: carbons(*)
    end function
    integer(c_int) function sesp_cmn_detach() bind(C, name="sesp_cmn_detach")
      import :: c_int
    end function
    type(c_ptr) function sesp_cmn_context() bind(C, name="sesp_cmn_context")
      import :: c_ptr
    end function
    integer(c_int) function sesp_cmn_reload() bind(C, name="sesp_cmn_reload")
      import :: c_int
    end function
    integer(c_int) function sesp_cmn_status() bind(C, name="sesp_cmn_status")
      import :: c_int
    end function
    integer(c_int) function sesp_cmn_last_error(buf, len) bind(C, name="sesp_cmn_last_error")
      import :: c_int, c_char, c_size_t
      character(kind=c_char), intent(out) :: buf(*)
      integer(c_size_t), value :: len
    end function
  end interface
end module sesp_common_mod
