! crm_gb300_bind.F90 -- iso_c_binding interface of libcrm_gb300 (include/crm_gb300.h)
! for the Fortran host.  The reference's caller, crm_physics_tend
! (components/cam/src/physics/cam/crm_physics.F90:1145-1156), keeps its
! call crm(lchnk, icol, ncrms, dt_gl, plev, crm_input, crm_state, crm_rad,
! crm_ecpp_output, crm_output) (crm_module.F90:45-56); a wrapper of that name
! fills these bind(C) types with c_loc() of the derived-type components and
! calls crm_run.  The types declare the same components, in the same order,
! as the C structs of crm_gb300.h.
module crm_gb300_bind
  use iso_c_binding
  implicit none

  type, bind(C) :: crm_config_c
    integer(c_int)  :: crm_nx, crm_ny, crm_nz, crm_nx_rad, crm_ny_rad, plev
    real(c_double)  :: crm_dx, crm_dy, crm_dt
    integer(c_int)  :: microphysics, precision, batch_mode, max_ncrms
    integer(c_int)  :: use_crm_accel      ! namelist use_crm_accel
    real(c_double)  :: crm_accel_factor   ! namelist crm_accel_factor
    integer(c_int)  :: crm_accel_uv       ! namelist crm_accel_uv
  end type

  type, bind(C) :: crm_call_desc_c
    integer(c_int)  :: lchnk, ncrms, ld
    real(c_double)  :: dt_gl
    integer(c_int)  :: igstep
    type(c_ptr)     :: gcol
    type(c_ptr)     :: col_map            ! c_null_ptr: columns 1..ncrms
  end type

  ! crm_input_c / crm_state_c / crm_rad_c / crm_output_c: one type(c_ptr)
  ! per component, in the order of include/crm_gb300.h
  type, bind(C) :: crm_input_c
    type(c_ptr) :: zmid, zint, tl, ql, qccl, qiil, ps, pmid, pint, pdel, phis, &
                   ul, vl, ocnfrac, tau00, wndls, bflxls, fluxu00, fluxv00, fluxt00, fluxq00
  end type
  type, bind(C) :: crm_state_c
    type(c_ptr) :: u_wind, v_wind, w_wind, temperature, qt, qp, qn
  end type
  type, bind(C) :: crm_rad_c
    type(c_ptr) :: qrad, temperature, qv, qc, qi, cld
  end type
  type, bind(C) :: crm_output_c
    type(c_ptr) :: field(62)        ! CRM_NOUT = 62, indexed by enum crm_output_field
  end type

  interface
    function crm_create(cfg, status) bind(C, name='crm_create') result(h)
      import :: c_ptr, c_int, crm_config_c
      type(crm_config_c), intent(in) :: cfg
      integer(c_int), intent(out)    :: status
      type(c_ptr) :: h
    end function
    integer(c_int) function crm_run(h, desc, inp, st, rad, out, col_status) bind(C, name='crm_run')
      import :: c_ptr, c_int, crm_call_desc_c, crm_input_c, crm_state_c, crm_rad_c, crm_output_c
      type(c_ptr), value                  :: h
      type(crm_call_desc_c), intent(in)   :: desc
      type(crm_input_c), intent(in)       :: inp
      type(crm_state_c), intent(in)       :: st
      type(crm_rad_c), intent(in)         :: rad
      type(crm_output_c), intent(in)      :: out
      integer(c_int), intent(out)         :: col_status(*)
    end function
    subroutine crm_destroy(h) bind(C, name='crm_destroy')
      import :: c_ptr
      type(c_ptr), value :: h
    end subroutine

    ! continuous batching (crm_server_create ... crm_poll in crm_gb300.h):
    ! the chunk's CRM state stays on the device between GCM steps in place
    ! of the physics-buffer round trip of crm_physics.F90:126-191
    function crm_server_create(cfg, capacity, nhandles, hbm_budget_bytes, status) &
        bind(C, name='crm_server_create') result(srv)
      import :: c_ptr, c_int, c_long_long, crm_config_c
      type(crm_config_c), intent(in)   :: cfg
      integer(c_int), value            :: capacity, nhandles
      integer(c_long_long), value      :: hbm_budget_bytes
      integer(c_int), intent(out)      :: status
      type(c_ptr) :: srv
    end function
    subroutine crm_server_destroy(srv) bind(C, name='crm_server_destroy')
      import :: c_ptr
      type(c_ptr), value :: srv
    end subroutine
    integer(c_int) function crm_chunk_open(srv, ncols, gcol, ld, st, rad, chunk) bind(C, name='crm_chunk_open')
      import :: c_ptr, c_int, crm_state_c, crm_rad_c
      type(c_ptr), value              :: srv
      integer(c_int), value           :: ncols, ld
      integer(c_int), intent(in)      :: gcol(*)
      type(crm_state_c), intent(in)   :: st
      type(crm_rad_c), intent(in)     :: rad
      integer(c_int), intent(out)     :: chunk
    end function
    integer(c_int) function crm_chunk_read_state(srv, chunk, ld, st, qrad) bind(C, name='crm_chunk_read_state')
      import :: c_ptr, c_int, crm_state_c
      type(c_ptr), value              :: srv
      integer(c_int), value           :: chunk, ld
      type(crm_state_c), intent(in)   :: st
      type(c_ptr), value              :: qrad
    end function
    integer(c_int) function crm_chunk_close(srv, chunk) bind(C, name='crm_chunk_close')
      import :: c_ptr, c_int
      type(c_ptr), value    :: srv
      integer(c_int), value :: chunk
    end function
    integer(c_int) function crm_submit(srv, chunk, inp, qrad, ld, dt_gl, out, rad_means, col_status, ticket) &
        bind(C, name='crm_submit')
      import :: c_ptr, c_int, c_double, c_long_long, crm_input_c, crm_output_c
      type(c_ptr), value               :: srv
      integer(c_int), value            :: chunk, ld
      type(crm_input_c), intent(in)    :: inp
      type(c_ptr), value               :: qrad         ! c_null_ptr: keep the resident heating
      real(c_double), value            :: dt_gl
      type(crm_output_c), intent(in)   :: out
      type(c_ptr), value               :: rad_means    ! c_loc(crm_rad_c) or c_null_ptr
      type(c_ptr), value               :: col_status   ! c_loc(status(1)) or c_null_ptr
      integer(c_long_long), intent(out) :: ticket
    end function
    integer(c_int) function crm_poll(srv, ticket, wait) bind(C, name='crm_poll')
      import :: c_ptr, c_int, c_long_long
      type(c_ptr), value          :: srv
      integer(c_long_long), value :: ticket
      integer(c_int), value       :: wait
    end function
  end interface
end module
