!
! mod_moloch_gb300 -- ISO_C_BINDING shim that lets RegCM call the GB300
! MOLOCH step (libmoloch_gb300.so) in place of Main/mod_moloch.F90.
!
! The module keeps the three public names of the reference module,
! allocate_moloch, init_moloch and moloch (Main/mod_moloch.F90:127), so the
! call sites in Main/mod_params.F90:1979-1980, Main/mod_init.F90:922-923 and
! Main/mod_regcm_interface.F90:274-275 do not change.  It reads the same
! module globals the reference reads (mo_atm, mddom, sfs, the boundary
! arrays and the run parameters) and hands their addresses to the C ABI of
! include/moloch_gb300.h; a negative status becomes fatal(), as the
! reference's own error paths do.
!
! Physics still runs on the host, inside the step as in the reference:
! moloch uploads the prognostic state, runs the dynamics half of the step on
! the GPU (through mkslice's edits of the state), downloads the state for
! mkslice and the physics on the host, hands their tendencies back and lets
! the GPU finish the step (status_update, mass check), then downloads the
! state.  physical_parametrizations is a private procedure of
! Main/mod_moloch.F90 (:1143-1401); the maintainer makes it public (or
! moves it to its own module) for this call.
! Builds with real(rkx) = real(rk8) (the FP64 build); MLC_PREC_MIXED keeps
! the same host arrays and converts on the device.
!
module mod_moloch_gb300

  use iso_c_binding
  use mod_intkinds
  use mod_realkinds
  use mod_dynparam
  use mod_runparams
  use mod_mpmessage
  use mod_atm_interface
  use mod_bdycod
  use mod_zita
  use mod_slice, only : mkslice

  implicit none

  private

  public :: allocate_moloch, init_moloch, moloch

  type, bind(c) :: mlc_dims
    integer(c_int32_t) :: jx, iy, kz, nqx, ntr
  end type mlc_dims

  type, bind(c) :: mlc_params
    real(c_double) :: dtsec, dx, mo_ztop, mo_h, mo_a0, dtbdys
    integer(c_int32_t) :: mo_nadv, mo_nsound, mo_divdamp, mo_divfilter
    integer(c_int32_t) :: mo_top_nudge, mo_spectral_nudge, do_apply_bdy
    integer(c_int32_t) :: lrotllr, ipptls, present_qc, present_qi
    integer(c_int32_t) :: nspgx, nspgd, nztop, debug_level, precision
    real(c_double) :: dtrad
    integer(c_int32_t) :: bdy_use_lehmann, ibltyp
    real(c_double) :: high_nudge, medium_nudge, low_nudge
  end type mlc_params

  type, bind(c) :: mlc_static_ptrs
    type(c_ptr) :: msfu, msfv, msfx, ulat, vlat, rlat, hx, hy
    type(c_ptr) :: fmz, fmzf, rfmzu, rfmzv, zeta, dz, zita, zitah
    type(c_ptr) :: ffilt, hefc, fcx, tnudge, ibnd_cr, ibnd_ud, ibnd_vd
    type(c_ptr) :: cnudge
  end type mlc_static_ptrs

  type, bind(c) :: mlc_state_ptrs
    type(c_ptr) :: u, v, w, pai, tetav, t, tvirt, ux, vx, p, rho, qsat
    type(c_ptr) :: qx, trac, ps, tke
  end type mlc_state_ptrs

  type, bind(c) :: mlc_bdy_ptrs
    type(c_ptr) :: xtb(2), xqb(2), xpaib(2), xlb(2), xib(2)
    type(c_ptr) :: dub(2), dvb(2), xpsb(2), chib(2)
  end type mlc_bdy_ptrs

  type, bind(c) :: mlc_tend_ptrs
    type(c_ptr) :: tten, uten, vten, qxten, chiten, tketen
  end type mlc_tend_ptrs

  type, bind(c) :: mlc_diag
    real(c_double) :: ps_max, ps_min
    integer(c_int32_t) :: nonfinite, steps_done
    real(c_double) :: drymass, dryadv, qmass, qadv, xbctime
  end type mlc_diag

  interface
    subroutine mlc_default_params(p) bind(c, name='mlc_default_params')
      import :: mlc_params
      type(mlc_params), intent(out) :: p
    end subroutine
    integer(c_int) function mlc_create(d, p, ctx) bind(c, name='mlc_create')
      import :: mlc_dims, mlc_params, c_int, c_ptr
      type(mlc_dims), intent(in) :: d
      type(mlc_params), intent(in) :: p
      type(c_ptr), intent(out) :: ctx
    end function
    integer(c_int) function mlc_bind_static(ctx, s) bind(c, name='mlc_bind_static')
      import :: mlc_static_ptrs, c_int, c_ptr
      type(c_ptr), value :: ctx
      type(mlc_static_ptrs), intent(in) :: s
    end function
    integer(c_int) function mlc_upload_state(ctx, s) bind(c, name='mlc_upload_state')
      import :: mlc_state_ptrs, c_int, c_ptr
      type(c_ptr), value :: ctx
      type(mlc_state_ptrs), intent(in) :: s
    end function
    integer(c_int) function mlc_download_state(ctx, s) bind(c, name='mlc_download_state')
      import :: mlc_state_ptrs, c_int, c_ptr
      type(c_ptr), value :: ctx
      type(mlc_state_ptrs), intent(in) :: s
    end function
    integer(c_int) function mlc_set_boundary(ctx, b, xbct, dtbd) &
        bind(c, name='mlc_set_boundary')
      import :: mlc_bdy_ptrs, c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      type(mlc_bdy_ptrs), intent(in) :: b
      real(c_double), value :: xbct, dtbd
    end function
    integer(c_int) function mlc_step(ctx, n, diag) bind(c, name='mlc_step')
      import :: mlc_diag, c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: n
      type(mlc_diag), intent(out) :: diag
    end function
    integer(c_int) function mlc_step_dynamics(ctx) bind(c, name='mlc_step_dynamics')
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
    end function
    integer(c_int) function mlc_member_set_tendencies(ctx, m, t) &
        bind(c, name='mlc_member_set_tendencies')
      import :: mlc_tend_ptrs, c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: m
      type(mlc_tend_ptrs), intent(in) :: t
    end function
    integer(c_int) function mlc_step_finish(ctx, diag) bind(c, name='mlc_step_finish')
      import :: mlc_diag, c_int, c_ptr
      type(c_ptr), value :: ctx
      type(mlc_diag), intent(out) :: diag
    end function
    type(c_ptr) function mlc_strerror(st) bind(c, name='mlc_strerror')
      import :: c_ptr, c_int
      integer(c_int), value :: st
    end function
    integer(c_int) function mlc_setup_relaxation(d, p, zeta, hefc, fcx, tnudge, &
        ffilt, gmeanz) bind(c, name='mlc_setup_relaxation')
      import :: mlc_dims, mlc_params, c_int, c_ptr
      type(mlc_dims), intent(in) :: d
      type(mlc_params), intent(inout) :: p
      type(c_ptr), value :: zeta, hefc, fcx, tnudge, ffilt, gmeanz
    end function
    integer(c_int) function mlc_setup_spectral(p, kz, gmeanz, cnudge) &
        bind(c, name='mlc_setup_spectral')
      import :: c_int, c_ptr, mlc_params
      type(mlc_params), intent(in) :: p
      integer(c_int), value :: kz
      type(c_ptr), value :: gmeanz, cnudge
    end function
  end interface

  type(c_ptr), save :: ctx = c_null_ptr
  type(mlc_dims), save :: dims
  type(mlc_params), save :: prm
  integer(ik4), allocatable, target, save :: ibcr(:,:), ibud(:,:), ibvd(:,:)
  ! relaxation weights, top-nudging profile and sponge: hefc and tnudge are
  ! private to mod_bdycod and ffilt is filled after init_moloch in init, so
  ! the library's restatement of setup_bdycon/init builds them here
  real(c_double), allocatable, target, save :: hefc_l(:,:), fcx_l(:)
  real(c_double), allocatable, target, save :: tnudge_l(:), ffilt_l(:), gmeanz_l(:)
  real(c_double), allocatable, target, save :: cnudge_l(:)

  contains

  subroutine check(st, where)
    integer(c_int), intent(in) :: st
    character(len=*), intent(in) :: where
    if ( st /= 0 ) then
      call fatal(__FILE__,__LINE__,'moloch_gb300 '//where//' failed')
    end if
  end subroutine check

  ! replaces Main/mod_moloch.F90:159-199
  subroutine allocate_moloch
    call mlc_default_params(prm)
    dims%jx = jx
    dims%iy = iy
    dims%kz = kz
    dims%nqx = nqx
    dims%ntr = 0
    if ( ichem == 1 ) dims%ntr = ntr
    prm%dtsec = dtsec
    prm%dx = dx
    prm%mo_ztop = mo_ztop
    prm%mo_h = mo_h
    prm%mo_a0 = mo_a0
    prm%dtbdys = dtbdys
    prm%mo_nadv = mo_nadv
    prm%mo_nsound = mo_nsound
    prm%mo_divdamp = merge(1, 0, mo_divdamp)
    prm%mo_divfilter = merge(1, 0, mo_divfilter)
    prm%mo_top_nudge = merge(1, 0, mo_top_nudge)
    prm%mo_spectral_nudge = merge(1, 0, mo_spectral_nudge)
    prm%dtrad = dtrad
    prm%do_apply_bdy = 1
    prm%lrotllr = merge(1, 0, iproj == 'ROTLLR')
    prm%ipptls = ipptls
    prm%present_qc = merge(1, 0, is_present_qc( ))
    prm%present_qi = merge(1, 0, is_present_qi( ))
    prm%nspgx = nspgx
    prm%nspgd = nspgd
    prm%debug_level = debug_level
    prm%bdy_use_lehmann = merge(1, 0, bdy_use_lehmann)
    prm%ibltyp = ibltyp
    prm%high_nudge = high_nudge
    prm%medium_nudge = medium_nudge
    prm%low_nudge = low_nudge
    ! the context is created in init_moloch, once zeta exists
  end subroutine allocate_moloch

  ! replaces Main/mod_moloch.F90:201-308
  subroutine init_moloch
    type(mlc_static_ptrs) :: s
    type(mlc_bdy_ptrs) :: b
    allocate(hefc_l(nspgx,kz), fcx_l(nspgx), tnudge_l(kz), ffilt_l(kz), gmeanz_l(kz))
    call check(mlc_setup_relaxation(dims, prm, c_loc(mo_atm%zeta), c_loc(hefc_l), &
               c_loc(fcx_l), c_loc(tnudge_l), c_loc(ffilt_l), c_loc(gmeanz_l)), &
               'init_moloch(relaxation)')
    allocate(cnudge_l(kz))
    cnudge_l = 0.0_c_double
    if ( mo_spectral_nudge ) then
      call check(mlc_setup_spectral(prm, int(kz, c_int), c_loc(gmeanz_l), c_loc(cnudge_l)), &
                 'init_moloch(spectral)')
    end if
    call check(mlc_create(dims, prm, ctx), 'init_moloch(create)')
    allocate(ibcr(jde1:jde2,ide1:ide2), ibud(jde1:jde2,ide1:ide2), &
             ibvd(jde1:jde2,ide1:ide2))
    ibcr = ba_cr%ibnd
    ibud = ba_ud%ibnd
    ibvd = ba_vd%ibnd
    s%msfu = c_loc(mddom%msfu)
    s%msfv = c_loc(mddom%msfv)
    s%msfx = c_loc(mddom%msfx)
    s%ulat = c_loc(mddom%ulat)
    s%vlat = c_loc(mddom%vlat)
    s%rlat = c_loc(mddom%rlat)
    s%hx = c_loc(mddom%hx)
    s%hy = c_loc(mddom%hy)
    s%fmz = c_loc(mo_atm%fmz)
    s%fmzf = c_loc(mo_atm%fmzf)
    s%rfmzu = c_loc(mo_atm%rfmzu)
    s%rfmzv = c_loc(mo_atm%rfmzv)
    s%zeta = c_loc(mo_atm%zeta)
    s%dz = c_loc(mo_atm%dz)
    s%zita = c_loc(zita)
    s%zitah = c_loc(zitah)
    s%ffilt = c_loc(ffilt_l)
    s%hefc = c_loc(hefc_l)
    s%fcx = c_loc(fcx_l)
    s%tnudge = c_loc(tnudge_l)
    s%ibnd_cr = c_loc(ibcr)
    s%ibnd_ud = c_loc(ibud)
    s%ibnd_vd = c_loc(ibvd)
    s%cnudge = c_loc(cnudge_l)
    call check(mlc_bind_static(ctx, s), 'init_moloch(static)')
    call upload( )
    b%xtb(1) = c_loc(xtb%b0)
    b%xtb(2) = c_loc(xtb%b1)
    b%xqb(1) = c_loc(xqb%b0)
    b%xqb(2) = c_loc(xqb%b1)
    b%xpaib(1) = c_loc(xpaib%b0)
    b%xpaib(2) = c_loc(xpaib%b1)
    b%xlb = c_null_ptr
    b%xib = c_null_ptr
    if ( is_present_qc( ) ) then
      b%xlb(1) = c_loc(xlb%b0)
      b%xlb(2) = c_loc(xlb%b1)
    end if
    if ( is_present_qi( ) ) then
      b%xib(1) = c_loc(xib%b0)
      b%xib(2) = c_loc(xib%b1)
    end if
    b%dub(1) = c_loc(dub%b0)
    b%dub(2) = c_loc(dub%b1)
    b%dvb(1) = c_loc(dvb%b0)
    b%dvb(2) = c_loc(dvb%b1)
    b%xpsb(1) = c_loc(xpsb%b0)
    b%xpsb(2) = c_loc(xpsb%b1)
    b%chib = c_null_ptr
    call check(mlc_set_boundary(ctx, b, real(xbctime,c_double), &
                                real(dtbdys,c_double)), 'init_moloch(bdy)')
  end subroutine init_moloch

  subroutine upload( )
    type(mlc_state_ptrs) :: st
    call state_ptrs(st)
    call check(mlc_upload_state(ctx, st), 'upload')
  end subroutine upload

  subroutine state_ptrs(st)
    type(mlc_state_ptrs), intent(out) :: st
    st%u = c_loc(mo_atm%u)
    st%v = c_loc(mo_atm%v)
    st%w = c_loc(mo_atm%w)
    st%pai = c_loc(mo_atm%pai)
    st%tetav = c_loc(mo_atm%tetav)
    st%t = c_loc(mo_atm%t)
    st%tvirt = c_loc(mo_atm%tvirt)
    st%ux = c_loc(mo_atm%ux)
    st%vx = c_loc(mo_atm%vx)
    st%p = c_loc(mo_atm%p)
    st%rho = c_loc(mo_atm%rho)
    st%qsat = c_loc(mo_atm%qs)
    st%qx = c_loc(mo_atm%qx)
    st%trac = c_null_ptr
    st%ps = c_loc(sfs%psa)
    if ( ibltyp == 2 ) then
      st%tke = c_loc(mo_atm%tke)
    else
      st%tke = c_null_ptr
    end if
  end subroutine state_ptrs

  ! replaces Main/mod_moloch.F90:312-446: the GPU runs the dynamics half
  ! (:312-357) and status_update onwards (:376-446); mkslice and the physics
  ! (:357-370) run on the host in between
  subroutine moloch
    type(mlc_state_ptrs) :: st
    type(mlc_tend_ptrs) :: tp
    type(mlc_diag) :: dg
    integer(c_int) :: ist
    call state_ptrs(st)
    call check(mlc_upload_state(ctx, st), 'moloch(upload)')
    call check(mlc_step_dynamics(ctx), 'moloch(dynamics)')
    call check(mlc_download_state(ctx, st), 'moloch(download)')
    ! reset_tendencies (:1044-1083) for the host's arrays
    mo_atm%tten = d_zero
    mo_atm%uten = d_zero
    mo_atm%vten = d_zero
    mo_atm%qxten = d_zero
    if ( ibltyp == 2 ) mo_atm%tketen = d_zero
    call mkslice
    if ( do_phys .and. moloch_realcase ) then
      call physical_parametrizations
    end if
    tp%tten = c_loc(mo_atm%tten)
    tp%uten = c_loc(mo_atm%uten)
    tp%vten = c_loc(mo_atm%vten)
    tp%qxten = c_loc(mo_atm%qxten)
    tp%chiten = c_null_ptr
    if ( ibltyp == 2 ) then
      tp%tketen = c_loc(mo_atm%tketen)
    else
      tp%tketen = c_null_ptr
    end if
    call check(mlc_member_set_tendencies(ctx, 0_c_int, tp), 'moloch(tendencies)')
    ist = mlc_step_finish(ctx, dg)
    if ( ist == -6 ) then
      call fatal(__FILE__,__LINE__,'CFL VIOLATION')
    end if
    call check(ist, 'moloch(status_update)')
    call check(mlc_download_state(ctx, st), 'moloch(download)')
    xbctime = real(dg%xbctime,rkx)
  end subroutine moloch

end module mod_moloch_gb300
