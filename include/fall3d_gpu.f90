! fall3d_gpu.f90 -- Fortran interface of the GPU library (include/fall3d_gpu.h).
!
! A drop-in for FALL3D's transport path: the Fortran driver (Fall3d.f90,
! sizloop.f90, meteo.f90) calls these bind(C) interfaces instead of the
! routines they replace.  Every fine-grained entry point has the argument
! list of the reference subroutine it replaces (arguments by reference, no
! VALUE), so a call site changes only its name, e.g.
!     call advctx(c,nx,ny,nz,nz_loc,iz_loc,vx,dX1,dt,work,lmeth)
! becomes
!     call f3d_check( f3d_advctx(c,nx,ny,nz,nz_loc,iz_loc,vx,dX1,dt,work,lmeth) )
! The coarse context API keeps the state resident on the device between
! calls (f3d_ctx_*, f3d_meteo, f3d_source, f3d_step, f3d_budget, f3d_run).
! Every function returns F3D_OK (0) or an error code; f3d_check maps a
! non-zero code to the reference's runend with the library's message.
! Strings passed to the library (file paths) must end with c_null_char.
! Real arguments are real(rp) = real(c_double) (KindType.f90:11), integers
! integer(ip) = integer(c_int) (KindType.f90:10).
module fall3d_gpu
  use, intrinsic :: iso_c_binding
  implicit none

  integer(c_int), parameter :: F3D_OK = 0
  integer(c_int), parameter :: F3D_ERR_ARG = 1
  integer(c_int), parameter :: F3D_ERR_CUDA = 2
  integer(c_int), parameter :: F3D_ERR_NOCONV = 3
  integer(c_int), parameter :: F3D_ERR_STATE = 4
  integer(c_int), parameter :: F3D_ERR_OOM = 5
  integer(c_int), parameter :: F3D_ERR_RANGE = 6
  integer(c_int), parameter :: F3D_ERR_INTERNAL = 7
  integer(c_int), parameter :: F3D_MODV_ARASTOOPOUR = 1
  integer(c_int), parameter :: F3D_MODV_GANSER = 2
  integer(c_int), parameter :: F3D_MODV_WILSON = 3
  integer(c_int), parameter :: F3D_MODV_DELLINO = 4
  integer(c_int), parameter :: F3D_MODKV_CONSTANT = 0
  integer(c_int), parameter :: F3D_MODKV_SIMILARITY = 1
  integer(c_int), parameter :: F3D_MODKV_SURFACE = 2
  integer(c_int), parameter :: F3D_MODKH_CONSTANT = 0
  integer(c_int), parameter :: F3D_MODKH_RAMS = 1
  integer(c_int), parameter :: F3D_MODKH_CMAQ = 2
  integer(c_int), parameter :: F3D_COORD_LONLAT = 0
  integer(c_int), parameter :: F3D_COORD_UTM = 1
  integer(c_int), parameter :: F3D_PREC_FP64 = 64
  integer(c_int), parameter :: F3D_PREC_FP32 = 32
  integer(c_int), parameter :: F3D_NOALLOC_SCRATCH_BYTES = 32768
  integer(c_int), parameter :: F3D_OUT_LOAD = 1
  integer(c_int), parameter :: F3D_OUT_WET = 2
  integer(c_int), parameter :: F3D_OUT_THICK = 3
  integer(c_int), parameter :: F3D_OUT_COL_MASS = 4
  integer(c_int), parameter :: F3D_OUT_PM_COL = 5
  integer(c_int), parameter :: F3D_OUT_C_GRND = 6
  integer(c_int), parameter :: F3D_OUT_PM_GRND = 7
  integer(c_int), parameter :: F3D_OUT_AOT05 = 8
  integer(c_int), parameter :: F3D_OUT_CON = 9
  integer(c_int), parameter :: F3D_OUT_WIND = 10
  integer(c_int), parameter :: F3D_OUT_MAGGR = 11
  integer(c_int), parameter :: F3D_OUT_BINARY64 = 0
  integer(c_int), parameter :: F3D_OUT_BINARY32 = 1
  integer(c_int), parameter :: F3D_OPT_FUSED = 1
  integer(c_int), parameter :: F3D_OPT_TILE = 2
  integer(c_int), parameter :: F3D_OPT_GRAPH = 3
  integer(c_int), parameter :: F3D_OPT_PREFETCH = 4

  ! f3d_grid: the static description of one scenario (reagrd.f90, reagrn.f90, readat.f90)
  type, bind(C) :: f3d_grid
    integer(c_int) :: nx, ny, nz, nc, np, coord_sys, modkv, modkh, modv, wetdep, aggregate, precision
    real(c_double) :: dX1, dX2, dx, dy, rkh0, rkv0, Csh, safety_factor, vset_factor
    type(c_ptr) :: dz, zlayer, Hm1, topg, diam, rhop, psi, sphe  ! c_loc of the Master arrays
  end type f3d_grid
  ! f3d_met_series: nt DBS snapshots on the model levels (get_dbs_value_plane.f90:107-114)
  type, bind(C) :: f3d_met_series
    integer(c_int) :: nt
    type(c_ptr) :: times
    real(c_double) :: time_lag
    type(c_ptr) :: u, v, w, t, tp, rho, ust, pblh, rmol, znt, prate, ldu, qv, p
  end type f3d_met_series
  ! f3d_src_series: the source intervals of the .src file (get_source_*.f90)
  type, bind(C) :: f3d_src_series
    integer(c_int) :: nint
    type(c_ptr) :: t1, t2, nsou, isrc, jsrc, ksrc, tmrat, nplume, pix, piy, piz, ptemp, pwater
  end type f3d_src_series
  ! f3d_log_record: one line of the mass-budget log (writim.f90:18-52)
  type, bind(C) :: f3d_log_record
    integer(c_int) :: iiter
    real(c_double) :: time, dt, dtc, massvol, massdep, massdry, masswet, outmass, erumass
  end type f3d_log_record
  ! f3d_gravity_current: the GRAVITY_CURRENT block (readat.f90:150-213)
  type, bind(C) :: f3d_gravity_current
    real(c_double) :: c_flow_rate, lambda_grav, k_entrain, brunt_vaisala, center_x, center_y, &
                      xorigr, yorigr, h_tot, beg_time
  end type f3d_gravity_current
  ! f3d_aggregation: AGGREGATION_IN_TRANSPORT (readat.f90:350-440)
  type, bind(C) :: f3d_aggregation
    real(c_double) :: Df
    integer(c_int) :: ndtagr
    type(c_ptr) :: fc
  end type f3d_aggregation

  interface
    function f3d_last_error(buf, buflen) bind(C, name="f3d_last_error")
      import
      integer(c_int) :: f3d_last_error
      character(kind=c_char), intent(inout) :: buf(*)
      integer(c_int), value :: buflen
    end function f3d_last_error
    function f3d_version() bind(C, name="f3d_version")
      import
      type(c_ptr) :: f3d_version
    end function f3d_version
    function f3d_setbcc(c, nx, ny, nz, nz_loc, iz_loc, vx, vy, vz, vset, vdep, rkver, dz) bind(C, name="f3d_setbcc")
      import
      integer(c_int) :: f3d_setbcc
      real(c_double), intent(inout) :: c(*)
      integer(c_int), intent(in) :: nx
      integer(c_int), intent(in) :: ny
      integer(c_int), intent(in) :: nz
      integer(c_int), intent(in) :: nz_loc
      integer(c_int), intent(in) :: iz_loc
      real(c_double), intent(in) :: vx(*)
      real(c_double), intent(in) :: vy(*)
      real(c_double), intent(in) :: vz(*)
      real(c_double), intent(in) :: vset(*)
      real(c_double), intent(in) :: vdep(*)
      real(c_double), intent(in) :: rkver(*)
      real(c_double), intent(in) :: dz(*)
    end function f3d_setbcc
    function f3d_advctzc(c, nx, ny, nz, nz_loc, iz_loc, vz, vset, dz, dt, lmeth) bind(C, name="f3d_advctzc")
      import
      integer(c_int) :: f3d_advctzc
      real(c_double), intent(inout) :: c(*)
      integer(c_int), intent(in) :: nx
      integer(c_int), intent(in) :: ny
      integer(c_int), intent(in) :: nz
      integer(c_int), intent(in) :: nz_loc
      integer(c_int), intent(in) :: iz_loc
      real(c_double), intent(in) :: vz(*)
      real(c_double), intent(in) :: vset(*)
      real(c_double), intent(in) :: dz(*)
      real(c_double), intent(in) :: dt
      integer(c_int), intent(in) :: lmeth
    end function f3d_advctzc
    function f3d_advctx(c, nx, ny, nz, nz_loc, iz_loc, vx, dx, dt, work, lmeth) bind(C, name="f3d_advctx")
      import
      integer(c_int) :: f3d_advctx
      real(c_double), intent(inout) :: c(*)
      integer(c_int), intent(in) :: nx
      integer(c_int), intent(in) :: ny
      integer(c_int), intent(in) :: nz
      integer(c_int), intent(in) :: nz_loc
      integer(c_int), intent(in) :: iz_loc
      real(c_double), intent(in) :: vx(*)
      real(c_double), intent(in) :: dx
      real(c_double), intent(in) :: dt
      real(c_double), intent(inout) :: work(*)
      integer(c_int), intent(in) :: lmeth
    end function f3d_advctx
    function f3d_advcty(c, nx, ny, nz, nz_loc, iz_loc, vy, dy, dt, work, lmeth) bind(C, name="f3d_advcty")
      import
      integer(c_int) :: f3d_advcty
      real(c_double), intent(inout) :: c(*)
      integer(c_int), intent(in) :: nx
      integer(c_int), intent(in) :: ny
      integer(c_int), intent(in) :: nz
      integer(c_int), intent(in) :: nz_loc
      integer(c_int), intent(in) :: iz_loc
      real(c_double), intent(in) :: vy(*)
      real(c_double), intent(in) :: dy
      real(c_double), intent(in) :: dt
      real(c_double), intent(inout) :: work(*)
      integer(c_int), intent(in) :: lmeth
    end function f3d_advcty
    function f3d_diffz(c, nx, ny, nz, nz_loc, iz_loc, dz, dt, rkver, rho, work) bind(C, name="f3d_diffz")
      import
      integer(c_int) :: f3d_diffz
      real(c_double), intent(inout) :: c(*)
      integer(c_int), intent(in) :: nx
      integer(c_int), intent(in) :: ny
      integer(c_int), intent(in) :: nz
      integer(c_int), intent(in) :: nz_loc
      integer(c_int), intent(in) :: iz_loc
      real(c_double), intent(in) :: dz(*)
      real(c_double), intent(in) :: dt
      real(c_double), intent(in) :: rkver(*)
      real(c_double), intent(in) :: rho(*)
      real(c_double), intent(inout) :: work(*)
    end function f3d_diffz
    function f3d_diffx(c, nx, ny, nz, nz_loc, iz_loc, dx, dt, rkhor, rho, work) bind(C, name="f3d_diffx")
      import
      integer(c_int) :: f3d_diffx
      real(c_double), intent(inout) :: c(*)
      integer(c_int), intent(in) :: nx
      integer(c_int), intent(in) :: ny
      integer(c_int), intent(in) :: nz
      integer(c_int), intent(in) :: nz_loc
      integer(c_int), intent(in) :: iz_loc
      real(c_double), intent(in) :: dx
      real(c_double), intent(in) :: dt
      real(c_double), intent(in) :: rkhor(*)
      real(c_double), intent(in) :: rho(*)
      real(c_double), intent(inout) :: work(*)
    end function f3d_diffx
    function f3d_diffy(c, nx, ny, nz, nz_loc, iz_loc, dy, dt, rkhor, rho, work) bind(C, name="f3d_diffy")
      import
      integer(c_int) :: f3d_diffy
      real(c_double), intent(inout) :: c(*)
      integer(c_int), intent(in) :: nx
      integer(c_int), intent(in) :: ny
      integer(c_int), intent(in) :: nz
      integer(c_int), intent(in) :: nz_loc
      integer(c_int), intent(in) :: iz_loc
      real(c_double), intent(in) :: dy
      real(c_double), intent(in) :: dt
      real(c_double), intent(in) :: rkhor(*)
      real(c_double), intent(in) :: rho(*)
      real(c_double), intent(inout) :: work(*)
    end function f3d_diffy
    function f3d_wetdep(c, cwet, ic, nx, ny, nz, nz_loc, iz_loc, dt, diam, zlayer, dz, zi, prate) bind(C, name="f3d_wetdep")
      import
      integer(c_int) :: f3d_wetdep
      real(c_double), intent(inout) :: c(*)
      real(c_double), intent(inout) :: cwet(*)
      integer(c_int), intent(in) :: ic
      integer(c_int), intent(in) :: nx
      integer(c_int), intent(in) :: ny
      integer(c_int), intent(in) :: nz
      integer(c_int), intent(in) :: nz_loc
      integer(c_int), intent(in) :: iz_loc
      real(c_double), intent(in) :: dt
      real(c_double), intent(in) :: diam(*)
      real(c_double), intent(in) :: zlayer(*)
      real(c_double), intent(in) :: dz(*)
      real(c_double), intent(in) :: zi(*)
      real(c_double), intent(in) :: prate(*)
    end function f3d_wetdep
    function f3d_accum(c, cdry, ic, nx, ny, nz, nz_loc, iz_loc, vz, dt, vset, vdep) bind(C, name="f3d_accum")
      import
      integer(c_int) :: f3d_accum
      real(c_double), intent(inout) :: c(*)
      real(c_double), intent(inout) :: cdry(*)
      integer(c_int), intent(in) :: ic
      integer(c_int), intent(in) :: nx
      integer(c_int), intent(in) :: ny
      integer(c_int), intent(in) :: nz
      integer(c_int), intent(in) :: nz_loc
      integer(c_int), intent(in) :: iz_loc
      real(c_double), intent(in) :: vz(*)
      real(c_double), intent(in) :: dt
      real(c_double), intent(in) :: vset(*)
      real(c_double), intent(in) :: vdep(*)
    end function f3d_accum
    function f3d_clip(c, nx, ny, nz, nc, ic_loc, nc_loc) bind(C, name="f3d_clip")
      import
      integer(c_int) :: f3d_clip
      real(c_double), intent(inout) :: c(*)
      integer(c_int), intent(in) :: nx
      integer(c_int), intent(in) :: ny
      integer(c_int), intent(in) :: nz
      integer(c_int), intent(in) :: nc
      integer(c_int), intent(in) :: ic_loc
      integer(c_int), intent(in) :: nc_loc
    end function f3d_clip
    function f3d_cmass2d(c, vx, vy, vz, vset, nx, ny, nz, nc, ic_loc, nc_loc, iz_loc, nz_loc, dx, &
        dy, dz, dt, outmass) bind(C, name="f3d_cmass2d")
      import
      integer(c_int) :: f3d_cmass2d
      real(c_double), intent(in) :: c(*)
      real(c_double), intent(in) :: vx(*)
      real(c_double), intent(in) :: vy(*)
      real(c_double), intent(in) :: vz(*)
      real(c_double), intent(in) :: vset(*)
      integer(c_int), intent(in) :: nx
      integer(c_int), intent(in) :: ny
      integer(c_int), intent(in) :: nz
      integer(c_int), intent(in) :: nc
      integer(c_int), intent(in) :: ic_loc
      integer(c_int), intent(in) :: nc_loc
      integer(c_int), intent(in) :: iz_loc
      integer(c_int), intent(in) :: nz_loc
      real(c_double), intent(in) :: dx
      real(c_double), intent(in) :: dy
      real(c_double), intent(in) :: dz(*)
      real(c_double), intent(in) :: dt
      real(c_double), intent(inout) :: outmass
    end function f3d_cmass2d
    function f3d_cmass2d_noalloc(c, vx, vy, vz, vset, nx, ny, nz, nc, ic_loc, nc_loc, iz_loc, &
        nz_loc, dx, dy, dz, dt, outmass) bind(C, name="f3d_cmass2d_noalloc")
      import
      integer(c_int) :: f3d_cmass2d_noalloc
      type(c_ptr), value :: c
      type(c_ptr), value :: vx
      type(c_ptr), value :: vy
      type(c_ptr), value :: vz
      type(c_ptr), value :: vset
      integer(c_int), intent(in) :: nx
      integer(c_int), intent(in) :: ny
      integer(c_int), intent(in) :: nz
      integer(c_int), intent(in) :: nc
      integer(c_int), intent(in) :: ic_loc
      integer(c_int), intent(in) :: nc_loc
      integer(c_int), intent(in) :: iz_loc
      integer(c_int), intent(in) :: nz_loc
      real(c_double), intent(in) :: dx
      real(c_double), intent(in) :: dy
      type(c_ptr), value :: dz
      real(c_double), intent(in) :: dt
      real(c_double), intent(inout) :: outmass
    end function f3d_cmass2d_noalloc
    function f3d_cmass3d(c, cload, cdry, cwet, nx, ny, nz, nc, dx, dy, dz, massvol, massdep, &
        massdry, masswet) bind(C, name="f3d_cmass3d")
      import
      integer(c_int) :: f3d_cmass3d
      real(c_double), intent(in) :: c(*)
      real(c_double), intent(in) :: cload(*)
      real(c_double), intent(in) :: cdry(*)
      real(c_double), intent(in) :: cwet(*)
      integer(c_int), intent(in) :: nx
      integer(c_int), intent(in) :: ny
      integer(c_int), intent(in) :: nz
      integer(c_int), intent(in) :: nc
      real(c_double), intent(in) :: dx
      real(c_double), intent(in) :: dy
      real(c_double), intent(in) :: dz(*)
      real(c_double), intent(inout) :: massvol
      real(c_double), intent(inout) :: massdep
      real(c_double), intent(inout) :: massdry
      real(c_double), intent(inout) :: masswet
    end function f3d_cmass3d
    function f3d_getc0(cdry, cwet, cload, nx, ny, nc, np) bind(C, name="f3d_getc0")
      import
      integer(c_int) :: f3d_getc0
      real(c_double), intent(inout) :: cdry(*)
      real(c_double), intent(inout) :: cwet(*)
      real(c_double), intent(inout) :: cload(*)
      integer(c_int), intent(in) :: nx
      integer(c_int), intent(in) :: ny
      integer(c_int), intent(in) :: nc
      integer(c_int), intent(in) :: np
    end function f3d_getc0
    function f3d_setsrc(c, nx, ny, nz, nc, nsou, isrc, jsrc, ksrc, tmrat, dz, zlayer, Hm1, dX1, &
        dX2, dt) bind(C, name="f3d_setsrc")
      import
      integer(c_int) :: f3d_setsrc
      real(c_double), intent(inout) :: c(*)
      integer(c_int), intent(in) :: nx
      integer(c_int), intent(in) :: ny
      integer(c_int), intent(in) :: nz
      integer(c_int), intent(in) :: nc
      integer(c_int), intent(in) :: nsou
      integer(c_int), intent(in) :: isrc(*)
      integer(c_int), intent(in) :: jsrc(*)
      integer(c_int), intent(in) :: ksrc(*)
      real(c_double), intent(in) :: tmrat(*)
      real(c_double), intent(in) :: dz(*)
      real(c_double), intent(in) :: zlayer(*)
      real(c_double), intent(in) :: Hm1(*)
      real(c_double), intent(in) :: dX1
      real(c_double), intent(in) :: dX2
      real(c_double), intent(in) :: dt
    end function f3d_setsrc
    function f3d_finddt(nx, ny, nz, nc, dX1, dX2, dz, vx, vy, vz, vset, rkh1, rkhor, rkver, &
        safety_factor, dt, dtc) bind(C, name="f3d_finddt")
      import
      integer(c_int) :: f3d_finddt
      integer(c_int), intent(in) :: nx
      integer(c_int), intent(in) :: ny
      integer(c_int), intent(in) :: nz
      integer(c_int), intent(in) :: nc
      real(c_double), intent(in) :: dX1
      real(c_double), intent(in) :: dX2
      real(c_double), intent(in) :: dz(*)
      real(c_double), intent(in) :: vx(*)
      real(c_double), intent(in) :: vy(*)
      real(c_double), intent(in) :: vz(*)
      real(c_double), intent(in) :: vset(*)
      real(c_double), intent(in) :: rkh1(*)
      real(c_double), intent(in) :: rkhor(*)
      real(c_double), intent(in) :: rkver(*)
      real(c_double), intent(in) :: safety_factor
      real(c_double), intent(inout) :: dt
      real(c_double), intent(inout) :: dtc
    end function f3d_finddt
    function f3d_kappa3(nx, ny, nz, modkv, modkh, coord_sys, rkv0, rkh0, Csh, dX1, dX2, dx, dy, dz, &
        zlayer, Hm1, vx, vy, vptemp, ustar, zi, rl, rkver, rkhor) bind(C, name="f3d_kappa3")
      import
      integer(c_int) :: f3d_kappa3
      integer(c_int), intent(in) :: nx
      integer(c_int), intent(in) :: ny
      integer(c_int), intent(in) :: nz
      integer(c_int), intent(in) :: modkv
      integer(c_int), intent(in) :: modkh
      integer(c_int), intent(in) :: coord_sys
      real(c_double), intent(in) :: rkv0
      real(c_double), intent(in) :: rkh0
      real(c_double), intent(in) :: Csh
      real(c_double), intent(in) :: dX1
      real(c_double), intent(in) :: dX2
      real(c_double), intent(in) :: dx
      real(c_double), intent(in) :: dy
      real(c_double), intent(in) :: dz(*)
      real(c_double), intent(in) :: zlayer(*)
      real(c_double), intent(in) :: Hm1(*)
      real(c_double), intent(in) :: vx(*)
      real(c_double), intent(in) :: vy(*)
      real(c_double), intent(in) :: vptemp(*)
      real(c_double), intent(in) :: ustar(*)
      real(c_double), intent(in) :: zi(*)
      real(c_double), intent(in) :: rl(*)
      real(c_double), intent(inout) :: rkver(*)
      real(c_double), intent(inout) :: rkhor(*)
    end function f3d_kappa3
    function f3d_setvset(nx, ny, nz, nc, np, modv, diam, rhop, psi, sphe, tempe, rho, aggregate, &
        vset_factor, vset, cd) bind(C, name="f3d_setvset")
      import
      integer(c_int) :: f3d_setvset
      integer(c_int), intent(in) :: nx
      integer(c_int), intent(in) :: ny
      integer(c_int), intent(in) :: nz
      integer(c_int), intent(in) :: nc
      integer(c_int), intent(in) :: np
      integer(c_int), intent(in) :: modv
      real(c_double), intent(in) :: diam(*)
      real(c_double), intent(in) :: rhop(*)
      real(c_double), intent(in) :: psi(*)
      real(c_double), intent(in) :: sphe(*)
      real(c_double), intent(in) :: tempe(*)
      real(c_double), intent(in) :: rho(*)
      integer(c_int), intent(in) :: aggregate
      real(c_double), intent(in) :: vset_factor
      real(c_double), intent(inout) :: vset(*)
      real(c_double), intent(inout) :: cd
    end function f3d_setvset
    function f3d_dmath_eval(op, n, x, y) bind(C, name="f3d_dmath_eval")
      import
      integer(c_int) :: f3d_dmath_eval
      integer(c_int), value :: op
      integer(c_long_long), value :: n
      real(c_double), intent(in) :: x(*)
      real(c_double), intent(inout) :: y(*)
    end function f3d_dmath_eval
    function f3d_setvdrydep(nx, ny, nc, diam, zlayer, ldu, rl, znt, ustar, tempe, rho, vdep) bind(C, name="f3d_setvdrydep")
      import
      integer(c_int) :: f3d_setvdrydep
      integer(c_int), intent(in) :: nx
      integer(c_int), intent(in) :: ny
      integer(c_int), intent(in) :: nc
      real(c_double), intent(in) :: diam(*)
      real(c_double), intent(in) :: zlayer(*)
      real(c_double), intent(in) :: ldu(*)
      real(c_double), intent(in) :: rl(*)
      real(c_double), intent(in) :: znt(*)
      real(c_double), intent(in) :: ustar(*)
      real(c_double), intent(in) :: tempe(*)
      real(c_double), intent(in) :: rho(*)
      real(c_double), intent(inout) :: vdep(*)
    end function f3d_setvdrydep
    function f3d_meteo_scale(nx, ny, nz, coord_sys, dX1, dX2, dz, Hm1, topg, vx, vy, vz, rho, &
        rkhor, rkh1, divu) bind(C, name="f3d_meteo_scale")
      import
      integer(c_int) :: f3d_meteo_scale
      integer(c_int), intent(in) :: nx
      integer(c_int), intent(in) :: ny
      integer(c_int), intent(in) :: nz
      integer(c_int), intent(in) :: coord_sys
      real(c_double), intent(in) :: dX1
      real(c_double), intent(in) :: dX2
      real(c_double), intent(in) :: dz(*)
      real(c_double), intent(in) :: Hm1(*)
      real(c_double), intent(in) :: topg(*)
      real(c_double), intent(inout) :: vx(*)
      real(c_double), intent(inout) :: vy(*)
      real(c_double), intent(inout) :: vz(*)
      real(c_double), intent(inout) :: rho(*)
      real(c_double), intent(in) :: rkhor(*)
      real(c_double), intent(inout) :: rkh1(*)
      real(c_double), intent(inout) :: divu(*)
    end function f3d_meteo_scale
    function f3d_ctx_create(grid, out) bind(C, name="f3d_ctx_create")
      import
      integer(c_int) :: f3d_ctx_create
      type(f3d_grid), intent(in) :: grid
      type(c_ptr), intent(out) :: out
    end function f3d_ctx_create
    function f3d_ctx_destroy(ctx) bind(C, name="f3d_ctx_destroy")
      import
      integer(c_int) :: f3d_ctx_destroy
      type(c_ptr), value :: ctx
    end function f3d_ctx_destroy
    function f3d_ctx_footprint(grid, bytes) bind(C, name="f3d_ctx_footprint")
      import
      integer(c_int) :: f3d_ctx_footprint
      type(f3d_grid), intent(in) :: grid
      integer(c_long_long), intent(inout) :: bytes
    end function f3d_ctx_footprint
    function f3d_meteo(ctx, u, v, w, t, tp, rho, ust, pblh, rmol, znt, prate, ldu) bind(C, name="f3d_meteo")
      import
      integer(c_int) :: f3d_meteo
      type(c_ptr), value :: ctx
      real(c_double), intent(in) :: u(*)
      real(c_double), intent(in) :: v(*)
      real(c_double), intent(in) :: w(*)
      real(c_double), intent(in) :: t(*)
      real(c_double), intent(in) :: tp(*)
      real(c_double), intent(in) :: rho(*)
      real(c_double), intent(in) :: ust(*)
      real(c_double), intent(in) :: pblh(*)
      real(c_double), intent(in) :: rmol(*)
      real(c_double), intent(in) :: znt(*)
      real(c_double), intent(in) :: prate(*)
      real(c_double), intent(in) :: ldu(*)
    end function f3d_meteo
    function f3d_source(ctx, nsou, isrc, jsrc, ksrc, tmrat) bind(C, name="f3d_source")
      import
      integer(c_int) :: f3d_source
      type(c_ptr), value :: ctx
      integer(c_int), value :: nsou
      integer(c_int), intent(in) :: isrc(*)
      integer(c_int), intent(in) :: jsrc(*)
      integer(c_int), intent(in) :: ksrc(*)
      real(c_double), intent(in) :: tmrat(*)
    end function f3d_source
    function f3d_step(ctx) bind(C, name="f3d_step")
      import
      integer(c_int) :: f3d_step
      type(c_ptr), value :: ctx
    end function f3d_step
    function f3d_budget(ctx, massvol, massdep, massdry, masswet) bind(C, name="f3d_budget")
      import
      integer(c_int) :: f3d_budget
      type(c_ptr), value :: ctx
      real(c_double), intent(inout) :: massvol
      real(c_double), intent(inout) :: massdep
      real(c_double), intent(inout) :: massdry
      real(c_double), intent(inout) :: masswet
    end function f3d_budget
    function f3d_count_nonfinite(ctx, in_c, in_deposits) bind(C, name="f3d_count_nonfinite")
      import
      integer(c_int) :: f3d_count_nonfinite
      type(c_ptr), value :: ctx
      integer(c_long_long), intent(inout) :: in_c
      integer(c_long_long), intent(inout) :: in_deposits
    end function f3d_count_nonfinite
    function f3d_get_state(ctx, iiter, time, dt, dtc, erumass, outmass, flowrate) bind(C, name="f3d_get_state")
      import
      integer(c_int) :: f3d_get_state
      type(c_ptr), value :: ctx
      integer(c_int), intent(inout) :: iiter
      real(c_double), intent(inout) :: time
      real(c_double), intent(inout) :: dt
      real(c_double), intent(inout) :: dtc
      real(c_double), intent(inout) :: erumass
      real(c_double), intent(inout) :: outmass
      real(c_double), intent(inout) :: flowrate
    end function f3d_get_state
    function f3d_set_time(ctx, time, iiter) bind(C, name="f3d_set_time")
      import
      integer(c_int) :: f3d_set_time
      type(c_ptr), value :: ctx
      real(c_double), value :: time
      integer(c_int), value :: iiter
    end function f3d_set_time
    function f3d_download(ctx, c, cdry, cwet, vset, vdep) bind(C, name="f3d_download")
      import
      integer(c_int) :: f3d_download
      type(c_ptr), value :: ctx
      real(c_double), intent(inout) :: c(*)
      real(c_double), intent(inout) :: cdry(*)
      real(c_double), intent(inout) :: cwet(*)
      real(c_double), intent(inout) :: vset(*)
      real(c_double), intent(inout) :: vdep(*)
    end function f3d_download
    function f3d_upload_state(ctx, c, cdry, cwet, erumass, outmass, cd) bind(C, name="f3d_upload_state")
      import
      integer(c_int) :: f3d_upload_state
      type(c_ptr), value :: ctx
      real(c_double), intent(in) :: c(*)
      real(c_double), intent(in) :: cdry(*)
      real(c_double), intent(in) :: cwet(*)
      real(c_double), value :: erumass
      real(c_double), value :: outmass
      real(c_double), value :: cd
    end function f3d_upload_state
    function f3d_download_coeffs(ctx, vx, vy, vz, rho, rkhor, rkh1, rkver) bind(C, name="f3d_download_coeffs")
      import
      integer(c_int) :: f3d_download_coeffs
      type(c_ptr), value :: ctx
      real(c_double), intent(inout) :: vx(*)
      real(c_double), intent(inout) :: vy(*)
      real(c_double), intent(inout) :: vz(*)
      real(c_double), intent(inout) :: rho(*)
      real(c_double), intent(inout) :: rkhor(*)
      real(c_double), intent(inout) :: rkh1(*)
      real(c_double), intent(inout) :: rkver(*)
    end function f3d_download_coeffs
    function f3d_download_iters(ctx, iters) bind(C, name="f3d_download_iters")
      import
      integer(c_int) :: f3d_download_iters
      type(c_ptr), value :: ctx
      integer(c_int), intent(inout) :: iters(*)
    end function f3d_download_iters
    function f3d_get_cd(ctx, cd) bind(C, name="f3d_get_cd")
      import
      integer(c_int) :: f3d_get_cd
      type(c_ptr), value :: ctx
      real(c_double), intent(inout) :: cd
    end function f3d_get_cd
    function f3d_outputs(ctx, load, col_mass, c_grnd) bind(C, name="f3d_outputs")
      import
      integer(c_int) :: f3d_outputs
      type(c_ptr), value :: ctx
      real(c_double), intent(inout) :: load(*)
      real(c_double), intent(inout) :: col_mass(*)
      real(c_double), intent(inout) :: c_grnd(*)
    end function f3d_outputs
    function f3d_output(ctx, var, index, asl, dst, dst_type) bind(C, name="f3d_output")
      import
      integer(c_int) :: f3d_output
      type(c_ptr), value :: ctx
      integer(c_int), value :: var
      integer(c_int), value :: index
      integer(c_int), value :: asl
      type(c_ptr), value :: dst
      integer(c_int), value :: dst_type
    end function f3d_output
    function f3d_track_points(ctx, npts, xpts, ypts, xo, yo, out) bind(C, name="f3d_track_points")
      import
      integer(c_int) :: f3d_track_points
      type(c_ptr), value :: ctx
      integer(c_int), value :: npts
      real(c_double), intent(in) :: xpts(*)
      real(c_double), intent(in) :: ypts(*)
      real(c_double), value :: xo
      real(c_double), value :: yo
      real(c_double), intent(inout) :: out(*)
    end function f3d_track_points
    function f3d_output_fl(ctx, flight_level, p, dst, dst_type) bind(C, name="f3d_output_fl")
      import
      integer(c_int) :: f3d_output_fl
      type(c_ptr), value :: ctx
      real(c_double), value :: flight_level
      real(c_double), intent(in) :: p(*)
      type(c_ptr), value :: dst
      integer(c_int), value :: dst_type
    end function f3d_output_fl
    function f3d_set_gravity_current(ctx, gc) bind(C, name="f3d_set_gravity_current")
      import
      integer(c_int) :: f3d_set_gravity_current
      type(c_ptr), value :: ctx
      type(f3d_gravity_current), intent(in) :: gc
    end function f3d_set_gravity_current
    function f3d_set_aggregation(ctx, ag) bind(C, name="f3d_set_aggregation")
      import
      integer(c_int) :: f3d_set_aggregation
      type(c_ptr), value :: ctx
      type(f3d_aggregation), intent(in) :: ag
    end function f3d_set_aggregation
    function f3d_aggregation_met(ctx, qv, p) bind(C, name="f3d_aggregation_met")
      import
      integer(c_int) :: f3d_aggregation_met
      type(c_ptr), value :: ctx
      real(c_double), intent(in) :: qv(*)
      real(c_double), intent(in) :: p(*)
    end function f3d_aggregation_met
    function f3d_aggregation_plume(ctx, n, ix, iy, iz, temp, water) bind(C, name="f3d_aggregation_plume")
      import
      integer(c_int) :: f3d_aggregation_plume
      type(c_ptr), value :: ctx
      integer(c_int), value :: n
      integer(c_int), intent(in) :: ix(*)
      integer(c_int), intent(in) :: iy(*)
      integer(c_int), intent(in) :: iz(*)
      real(c_double), intent(in) :: temp(*)
      real(c_double), intent(in) :: water(*)
    end function f3d_aggregation_plume
    function f3d_download_maggr(ctx, maggr) bind(C, name="f3d_download_maggr")
      import
      integer(c_int) :: f3d_download_maggr
      type(c_ptr), value :: ctx
      real(c_double), intent(inout) :: maggr(*)
    end function f3d_download_maggr
    function f3d_run(ctx, met, src, beg_time, end_time, max_steps, log, log_cap, nlog) bind(C, name="f3d_run")
      import
      integer(c_int) :: f3d_run
      type(c_ptr), value :: ctx
      type(f3d_met_series), intent(in) :: met
      type(f3d_src_series), intent(in) :: src
      real(c_double), value :: beg_time
      real(c_double), value :: end_time
      integer(c_int), value :: max_steps
      type(f3d_log_record), intent(inout) :: log(*)
      integer(c_int), value :: log_cap
      integer(c_int), intent(inout) :: nlog
    end function f3d_run
    function f3d_run_reset(ctx) bind(C, name="f3d_run_reset")
      import
      integer(c_int) :: f3d_run_reset
      type(c_ptr), value :: ctx
    end function f3d_run_reset
    function f3d_ctx_save(ctx, path) bind(C, name="f3d_ctx_save")
      import
      integer(c_int) :: f3d_ctx_save
      type(c_ptr), value :: ctx
      character(kind=c_char), intent(in) :: path(*)
    end function f3d_ctx_save
    function f3d_ctx_restore(ctx, path) bind(C, name="f3d_ctx_restore")
      import
      integer(c_int) :: f3d_ctx_restore
      type(c_ptr), value :: ctx
      character(kind=c_char), intent(in) :: path(*)
    end function f3d_ctx_restore
    function f3d_set_option(ctx, key, value) bind(C, name="f3d_set_option")
      import
      integer(c_int) :: f3d_set_option
      type(c_ptr), value :: ctx
      integer(c_int), value :: key
      integer(c_int), value :: value
    end function f3d_set_option
    function f3d_get_option(ctx, key, value) bind(C, name="f3d_get_option")
      import
      integer(c_int) :: f3d_get_option
      type(c_ptr), value :: ctx
      integer(c_int), value :: key
      integer(c_int), intent(inout) :: value
    end function f3d_get_option
    function f3d_ctx_stream(ctx, stream) bind(C, name="f3d_ctx_stream")
      import
      integer(c_int) :: f3d_ctx_stream
      type(c_ptr), value :: ctx
      type(c_ptr), intent(out) :: stream
    end function f3d_ctx_stream
    function f3d_profile_enable(ctx, enable) bind(C, name="f3d_profile_enable")
      import
      integer(c_int) :: f3d_profile_enable
      type(c_ptr), value :: ctx
      integer(c_int), value :: enable
    end function f3d_profile_enable
    function f3d_profile_read(ctx, cap, names, name_len, launches, total_ms, nkinds) bind(C, name="f3d_profile_read")
      import
      integer(c_int) :: f3d_profile_read
      type(c_ptr), value :: ctx
      integer(c_int), value :: cap
      character(kind=c_char), intent(inout) :: names(*)
      integer(c_int), value :: name_len
      integer(c_long_long), intent(inout) :: launches(*)
      real(c_double), intent(inout) :: total_ms(*)
      integer(c_int), intent(inout) :: nkinds
    end function f3d_profile_read
    function f3d_kernel_launches() bind(C, name="f3d_kernel_launches")
      import
      integer(c_long_long) :: f3d_kernel_launches
    end function f3d_kernel_launches
    function f3d_sync(ctx) bind(C, name="f3d_sync")
      import
      integer(c_int) :: f3d_sync
      type(c_ptr), value :: ctx
    end function f3d_sync
    function f3d_batch_create(max_scenarios, out) bind(C, name="f3d_batch_create")
      import
      integer(c_int) :: f3d_batch_create
      integer(c_int), value :: max_scenarios
      type(c_ptr), intent(out) :: out
    end function f3d_batch_create
    function f3d_batch_destroy(b) bind(C, name="f3d_batch_destroy")
      import
      integer(c_int) :: f3d_batch_destroy
      type(c_ptr), value :: b
    end function f3d_batch_destroy
    function f3d_batch_add(b, ctx, met, src, beg_time, end_time, max_steps, log, log_cap, slot) bind(C, name="f3d_batch_add")
      import
      integer(c_int) :: f3d_batch_add
      type(c_ptr), value :: b
      type(c_ptr), value :: ctx
      type(f3d_met_series), intent(in) :: met
      type(f3d_src_series), intent(in) :: src
      real(c_double), value :: beg_time
      real(c_double), value :: end_time
      integer(c_int), value :: max_steps
      type(f3d_log_record), intent(inout) :: log(*)
      integer(c_int), value :: log_cap
      integer(c_int), intent(inout) :: slot
    end function f3d_batch_add
    function f3d_batch_step(b, n_running) bind(C, name="f3d_batch_step")
      import
      integer(c_int) :: f3d_batch_step
      type(c_ptr), value :: b
      integer(c_int), intent(inout) :: n_running
    end function f3d_batch_step
    function f3d_batch_poll(b, slot, state, steps, nlog) bind(C, name="f3d_batch_poll")
      import
      integer(c_int) :: f3d_batch_poll
      type(c_ptr), value :: b
      integer(c_int), value :: slot
      integer(c_int), intent(inout) :: state
      integer(c_int), intent(inout) :: steps
      integer(c_int), intent(inout) :: nlog
    end function f3d_batch_poll
    function f3d_batch_release(b, slot) bind(C, name="f3d_batch_release")
      import
      integer(c_int) :: f3d_batch_release
      type(c_ptr), value :: b
      integer(c_int), value :: slot
    end function f3d_batch_release
    function f3d_batch_sync(b) bind(C, name="f3d_batch_sync")
      import
      integer(c_int) :: f3d_batch_sync
      type(c_ptr), value :: b
    end function f3d_batch_sync
    function f3d_batch_set_option(b, key, value) bind(C, name="f3d_batch_set_option")
      import
      integer(c_int) :: f3d_batch_set_option
      type(c_ptr), value :: b
      integer(c_int), value :: key
      integer(c_int), value :: value
    end function f3d_batch_set_option
    function f3d_batch_get_option(b, key, value) bind(C, name="f3d_batch_get_option")
      import
      integer(c_int) :: f3d_batch_get_option
      type(c_ptr), value :: b
      integer(c_int), value :: key
      integer(c_int), intent(inout) :: value
    end function f3d_batch_get_option
    function f3d_batch_autotune(b, reps, best, ms) bind(C, name="f3d_batch_autotune")
      import
      integer(c_int) :: f3d_batch_autotune
      type(c_ptr), value :: b
      integer(c_int), value :: reps
      integer(c_int), intent(inout) :: best
      real(c_float), intent(inout) :: ms(*)
    end function f3d_batch_autotune
    function f3d_batch_stats(b, batch_steps, cell_class_steps, n_running) bind(C, name="f3d_batch_stats")
      import
      integer(c_int) :: f3d_batch_stats
      type(c_ptr), value :: b
      integer(c_long_long), intent(inout) :: batch_steps
      real(c_double), intent(inout) :: cell_class_steps
      integer(c_int), intent(inout) :: n_running
    end function f3d_batch_stats
    function f3d_batch_stream(b, stream) bind(C, name="f3d_batch_stream")
      import
      integer(c_int) :: f3d_batch_stream
      type(c_ptr), value :: b
      type(c_ptr), intent(out) :: stream
    end function f3d_batch_stream
    function f3d_server_create(hbm_cap_bytes, max_running, out) bind(C, name="f3d_server_create")
      import
      integer(c_int) :: f3d_server_create
      integer(c_long_long), value :: hbm_cap_bytes
      integer(c_int), value :: max_running
      type(c_ptr), intent(out) :: out
    end function f3d_server_create
    function f3d_server_destroy(srv) bind(C, name="f3d_server_destroy")
      import
      integer(c_int) :: f3d_server_destroy
      type(c_ptr), value :: srv
    end function f3d_server_destroy
    function f3d_server_submit(srv, grid, met, src, beg_time, end_time, log_cap, request_id) bind(C, name="f3d_server_submit")
      import
      integer(c_int) :: f3d_server_submit
      type(c_ptr), value :: srv
      type(f3d_grid), intent(in) :: grid
      type(f3d_met_series), intent(in) :: met
      type(f3d_src_series), intent(in) :: src
      real(c_double), value :: beg_time
      real(c_double), value :: end_time
      integer(c_int), value :: log_cap
      integer(c_int), intent(inout) :: request_id
    end function f3d_server_submit
    function f3d_server_progress(srv, max_steps, n_running, n_queued) bind(C, name="f3d_server_progress")
      import
      integer(c_int) :: f3d_server_progress
      type(c_ptr), value :: srv
      integer(c_int), value :: max_steps
      integer(c_int), intent(inout) :: n_running
      integer(c_int), intent(inout) :: n_queued
    end function f3d_server_progress
    function f3d_server_poll(srv, request_id, state, t_submit, t_admit, t_done, steps) bind(C, name="f3d_server_poll")
      import
      integer(c_int) :: f3d_server_poll
      type(c_ptr), value :: srv
      integer(c_int), value :: request_id
      integer(c_int), intent(inout) :: state
      real(c_double), intent(inout) :: t_submit
      real(c_double), intent(inout) :: t_admit
      real(c_double), intent(inout) :: t_done
      integer(c_long_long), intent(inout) :: steps
    end function f3d_server_poll
    function f3d_server_result(srv, request_id, load, col_mass, c_grnd, log, log_cap, nlog) bind(C, name="f3d_server_result")
      import
      integer(c_int) :: f3d_server_result
      type(c_ptr), value :: srv
      integer(c_int), value :: request_id
      real(c_double), intent(inout) :: load(*)
      real(c_double), intent(inout) :: col_mass(*)
      real(c_double), intent(inout) :: c_grnd(*)
      type(f3d_log_record), intent(inout) :: log(*)
      integer(c_int), value :: log_cap
      integer(c_int), intent(inout) :: nlog
    end function f3d_server_result
    function f3d_server_forget(srv, request_id) bind(C, name="f3d_server_forget")
      import
      integer(c_int) :: f3d_server_forget
      type(c_ptr), value :: srv
      integer(c_int), value :: request_id
    end function f3d_server_forget
    function f3d_server_stats(srv, used_bytes, cell_class_steps, batch_steps, n_running, n_queued) bind(C, name="f3d_server_stats")
      import
      integer(c_int) :: f3d_server_stats
      type(c_ptr), value :: srv
      integer(c_long_long), intent(inout) :: used_bytes
      real(c_double), intent(inout) :: cell_class_steps
      integer(c_long_long), intent(inout) :: batch_steps
      integer(c_int), intent(inout) :: n_running
      integer(c_int), intent(inout) :: n_queued
    end function f3d_server_stats
    function f3d_server_batch(srv, batch) bind(C, name="f3d_server_batch")
      import
      integer(c_int) :: f3d_server_batch
      type(c_ptr), value :: srv
      type(c_ptr), intent(out) :: batch
    end function f3d_server_batch
  end interface

contains

  ! A non-zero status is the reference's runend (runend.f90:1-68) with the
  ! library's message.
  subroutine f3d_check(status)
    integer(c_int), intent(in) :: status
    character(kind=c_char) :: buf(512)
    character(len=512) :: message
    integer :: i, n
    if (status == F3D_OK) return
    n = f3d_last_error(buf, 512_c_int)
    message = ' '
    do i = 1, 512
      if (buf(i) == c_null_char) exit
      message(i:i) = buf(i)
    end do
    call runend(trim(message))
  end subroutine f3d_check

end module fall3d_gpu
