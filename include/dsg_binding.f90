! dsg_binding.f90 -- Fortran 2003 ISO_C_BINDING interface of libdsg.so
! (declarations in dsg.h) for the reference driver main.f of
! farzan-t/3D_Droplet_simulation_2007.
!
! dsg_config mirrors the C struct field for field: the 38 inputdata.in values
! in file order (main.f:188-234), then the additions.  Every function returns
! an integer status, 0 = DSG_OK; the wrappers in the driver map a nonzero
! status to STOP, as the reference stops on errors.
module dsg_binding
  use iso_c_binding
  implicit none
  type, bind(C) :: dsg_config
    integer(c_int) :: nx, ny, nz, tmax, nfilter, cycles
    real(c_double) :: omega
    integer(c_int) :: npre, ntop, npost, restart
    real(c_double) :: maxcfl
    integer(c_int) :: iturb, convectype, hswitch
    real(c_double) :: xvel1_si, yvel1_si, zvel1_si, xvel2_si, yvel2_si, zvel2_si
    real(c_double) :: rho2_si, rho1_si, sigma_si, visc2_si, visc1_si, grav_si, grav1_si
    integer(c_int) :: icase, ibc
    real(c_double) :: length_si, radius_si, y0_si, z0_si
    integer(c_int) :: tprint, ntecplot, tsave, surfacet
    integer(c_int) :: mode
    real(c_double) :: tol
    integer(c_int) :: max_vcycles
    real(c_double) :: noise_si
    integer(c_int64_t) :: noise_seed
    integer(c_int) :: inner_vcycles, use_graphs, tail_nodes, warm_start
    real(c_double) :: mg32_omega
    integer(c_int) :: mg32_npre, mg32_npost, mg32_prolong, mg32_fmg_cycles
    integer(c_int) :: mg32_fine_npre, mg32_fine_npost
    integer(c_int) :: mg32_mid_npre, mg32_mid_npost
    integer(c_int) :: mg32_small_npre, mg32_small_npost
    integer(c_int) :: fp64_exact
    integer(c_int) :: mg32_krylov
    integer(c_int) :: mg32_fmg_fine_cycles
  end type
  interface
    integer(c_int) function dsg_create(cfg, ctx) bind(C, name='dsg_create')
      import :: c_int, c_ptr, dsg_config
      type(dsg_config), intent(in) :: cfg
      type(c_ptr), intent(out) :: ctx
    end function
    subroutine dsg_destroy(ctx) bind(C, name='dsg_destroy')
      import :: c_ptr
      type(c_ptr), value :: ctx
    end subroutine
    integer(c_int) function dsg_init_drop(ctx) bind(C, name='dsg_init_drop')
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
    end function
    integer(c_int) function dsg_upload(ctx, field, host) bind(C, name='dsg_upload')
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      integer(c_int), value :: field
      real(c_double), intent(in) :: host(*)
    end function
    integer(c_int) function dsg_download(ctx, field, host) bind(C, name='dsg_download')
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      integer(c_int), value :: field
      real(c_double), intent(out) :: host(*)
    end function
    integer(c_int) function dsg_vofmethod(ctx) bind(C, name='dsg_vofmethod')
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
    end function
    integer(c_int) function dsg_kepsmodel(ctx) bind(C, name='dsg_kepsmodel')
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
    end function
    integer(c_int) function dsg_checktime(ctx) bind(C, name='dsg_checktime')
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
    end function
    integer(c_int) function dsg_csf(ctx) bind(C, name='dsg_csf')
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
    end function
    integer(c_int) function dsg_solvelpres(ctx, t, stats) bind(C, name='dsg_solvelpres')
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: t
      type(c_ptr), value :: stats
    end function
    integer(c_int) function dsg_mglin(ctx, stats) bind(C, name='dsg_mglin')
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx, stats
    end function
    integer(c_int) function dsg_step(ctx, t, stats) bind(C, name='dsg_step')
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: t
      type(c_ptr), value :: stats
    end function
    integer(c_int) function dsg_step_host(ctx, t, stats, n_in, in_fields, in_host, &
        n_out, out_fields, out_host) bind(C, name='dsg_step_host')
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx, stats
      integer(c_int), value :: t, n_in, n_out
      integer(c_int), intent(in) :: in_fields(*), out_fields(*)
      type(c_ptr), intent(in) :: in_host(*), out_host(*)
    end function
    integer(c_int) function dsg_liquid_volume(ctx, vol) bind(C, name='dsg_liquid_volume')
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(out) :: vol
    end function
    integer(c_int) function dsg_printout(ctx, t, dir) bind(C, name='dsg_printout')
      import :: c_int, c_ptr, c_char
      type(c_ptr), value :: ctx
      integer(c_int), value :: t
      character(kind=c_char), intent(in) :: dir(*)
    end function
    integer(c_int) function dsg_iniget(ctx, path, t0) bind(C, name='dsg_iniget')
      import :: c_int, c_ptr, c_char
      type(c_ptr), value :: ctx
      character(kind=c_char), intent(in) :: path(*)
      integer(c_int), intent(out) :: t0
    end function
  end interface
  type(c_ptr), save :: dsgctx
end module
