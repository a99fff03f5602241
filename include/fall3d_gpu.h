/*
 * fall3d_gpu.h -- C ABI of the GB300 transport library for FALL3D 7.0.
 *
 * The library replaces the per-time-step transport of particle-class
 * concentrations of FALL3D 7.0 (lmingari/Fall3D) and the coefficient
 * chain that feeds it.  Two layers are exported:
 *
 *  1. Fine-grained entry points, one per reference subroutine, with the
 *     reference argument lists passed by reference (what a Fortran
 *     `interface ... bind(C)` without VALUE produces).  Array arguments
 *     may all be host memory (copied to the GPU and back around the
 *     kernel: the "compat" mode used when the Fortran driver owns the
 *     Master arrays) or all device memory (used in place).  Mixing the
 *     two in one call is rejected with F3D_ERR_ARG.
 *
 *  2. A coarse context API that keeps the whole state resident in HBM:
 *     create a context for one scenario, feed it meteorology and sources,
 *     step it, and read budgets and fields back only when needed.
 *
 * Layout is the reference's (Sources/Master.f90:92-136): Fortran column
 * major, x fastest.  c is (0:nx+1, 0:ny+1, 0:nz+1, nc), met fields are
 * (nx, ny, nz), vset is (nx, ny, nz, nc), vdep is (nx, ny, nc),
 * cdry/cwet/cload are (nx, ny, 0:nc), dz is (0:nz).  Integers are 32-bit
 * (Sources/KindType.f90:10), reals are IEEE binary64 (KindType.f90:11).
 *
 * Every entry point returns an int status: 0 is success.  The message of
 * the last failure on the calling thread is available from
 * f3d_last_error().  Nothing throws across this boundary and nothing traps
 * on the device: device wait time-outs come back as status codes, and
 * non-finite values are counted on request (f3d_count_nonfinite).
 */
#ifndef FALL3D_GPU_H
#define FALL3D_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ */
/* Status codes                                                        */
/* ------------------------------------------------------------------ */
#define F3D_OK            0
#define F3D_ERR_ARG       1  /* invalid argument, size or pointer kind        */
#define F3D_ERR_CUDA      2  /* CUDA runtime error                             */
#define F3D_ERR_NOCONV    3  /* vsettl / get_gama did not converge             */
#define F3D_ERR_STATE     4  /* call out of order (e.g. step before meteo)     */
#define F3D_ERR_OOM       5  /* device allocation failed                       */
#define F3D_ERR_RANGE     6  /* source index outside the grid, time not in DBS */
#define F3D_ERR_INTERNAL  7  /* device-side consistency check failed           */

/* Model selectors, as decoded by Sources/readat.f90:227-314. */
#define F3D_MODV_ARASTOOPOUR 1
#define F3D_MODV_GANSER      2
#define F3D_MODV_WILSON      3
#define F3D_MODV_DELLINO     4
#define F3D_MODKV_CONSTANT   0
#define F3D_MODKV_SIMILARITY 1
#define F3D_MODKV_SURFACE    2
#define F3D_MODKH_CONSTANT   0
#define F3D_MODKH_RAMS       1
#define F3D_MODKH_CMAQ       2
#define F3D_COORD_LONLAT     0
#define F3D_COORD_UTM        1

/* Precision forms of the coarse API. */
#define F3D_PREC_FP64 64  /* plain form: every operation in binary64, in the
                             reference's operation order                    */
#define F3D_PREC_FP32 32  /* precision form: stencil arithmetic in binary32;
                             budgets, accum, finddt and the coefficient chain
                             stay binary64                                  */

/* Returns the message of the last failing call on this thread (always
 * NUL-terminated, truncated to len-1 bytes).  Returns the full length. */
int f3d_last_error(char* buf, int len);

/* Library version string and the device it runs on (cudaGetDevice). */
const char* f3d_version(void);

/* ------------------------------------------------------------------ */
/* 1. Fine-grained entry points (reference argument lists)             */
/* ------------------------------------------------------------------ */

/* Sources/setbcc.f90:1 setbcc(c,nx,ny,nz,nz_loc,iz_loc,vx,vy,vz,vset,vdep,rkver,dz) */
int f3d_setbcc(double* c, const int* nx, const int* ny, const int* nz,
               const int* nz_loc, const int* iz_loc,
               const double* vx, const double* vy, const double* vz,
               const double* vset, const double* vdep, const double* rkver,
               const double* dz);

/* Sources/advctzc.f90:1 advctzc(c,nx,ny,nz,nz_loc,iz_loc,vz,vset,dz,dt,lmeth) */
int f3d_advctzc(double* c, const int* nx, const int* ny, const int* nz,
                const int* nz_loc, const int* iz_loc,
                const double* vz, const double* vset, const double* dz,
                const double* dt, const int* lmeth);

/* Sources/advctx.f90:1 advctx(c,nx,ny,nz,nz_loc,iz_loc,vx,dx,dt,work,lmeth).
 * work is accepted for signature compatibility and never touched. */
int f3d_advctx(double* c, const int* nx, const int* ny, const int* nz,
               const int* nz_loc, const int* iz_loc, const double* vx,
               const double* dx, const double* dt, double* work,
               const int* lmeth);

/* Sources/advcty.f90:1 advcty(c,nx,ny,nz,nz_loc,iz_loc,vy,dy,dt,work,lmeth) */
int f3d_advcty(double* c, const int* nx, const int* ny, const int* nz,
               const int* nz_loc, const int* iz_loc, const double* vy,
               const double* dy, const double* dt, double* work,
               const int* lmeth);

/* Sources/diffz.f90:1 diffz(c,nx,ny,nz,nz_loc,iz_loc,dz,dt,rkver,rho,work) */
int f3d_diffz(double* c, const int* nx, const int* ny, const int* nz,
              const int* nz_loc, const int* iz_loc, const double* dz,
              const double* dt, const double* rkver, const double* rho,
              double* work);

/* Sources/diffx.f90:1 diffx(c,nx,ny,nz,nz_loc,iz_loc,dx,dt,rkhor,rho,work) */
int f3d_diffx(double* c, const int* nx, const int* ny, const int* nz,
              const int* nz_loc, const int* iz_loc, const double* dx,
              const double* dt, const double* rkhor, const double* rho,
              double* work);

/* Sources/diffy.f90:1 diffy(c,nx,ny,nz,nz_loc,iz_loc,dy,dt,rkhor,rho,work) */
int f3d_diffy(double* c, const int* nx, const int* ny, const int* nz,
              const int* nz_loc, const int* iz_loc, const double* dy,
              const double* dt, const double* rkhor, const double* rho,
              double* work);

/* Sources/wetdep.f90:1 wetdep(c,cwet,ic,nx,ny,nz,nz_loc,iz_loc,dt,diam,zlayer,dz,zi,prate).
 * cwet points at cwet(1,1,0); ic is 1-based; diam holds all classes. */
int f3d_wetdep(double* c, double* cwet, const int* ic, const int* nx,
               const int* ny, const int* nz, const int* nz_loc,
               const int* iz_loc, const double* dt, const double* diam,
               const double* zlayer, const double* dz, const double* zi,
               const double* prate);

/* Sources/accum.f90:1 accum(c,cdry,ic,nx,ny,nz,nz_loc,iz_loc,vz,dt,vset,vdep).
 * cdry points at cdry(1,1,0); vz is unused by the reference and here. */
int f3d_accum(double* c, double* cdry, const int* ic, const int* nx,
              const int* ny, const int* nz, const int* nz_loc,
              const int* iz_loc, const double* vz, const double* dt,
              const double* vset, const double* vdep);

/* The clip of Sources/sizloop.f90:77-78: c = MAX(0,c) over the whole
 * halo array of classes ic_loc..ic_loc+nc_loc-1 (c holds all nc). */
int f3d_clip(double* c, const int* nx, const int* ny, const int* nz,
             const int* nc, const int* ic_loc, const int* nc_loc);

/* Sources/cmass2d.f90:1 cmass2d(c,vx,vy,vz,vset,nx,ny,nz,nc,ic_loc,nc_loc,
 * iz_loc,nz_loc,dx,dy,dz,dt,outmass): outmass += outflow of this step.
 * The device sum is exact-then-rounded (see the parity note in the
 * library docs); the reference sums sequentially. */
int f3d_cmass2d(const double* c, const double* vx, const double* vy,
                const double* vz, const double* vset, const int* nx,
                const int* ny, const int* nz, const int* nc,
                const int* ic_loc, const int* nc_loc, const int* iz_loc,
                const int* nz_loc, const double* dx, const double* dy,
                const double* dz, const double* dt, double* outmass);

/* f3d_cmass2d without any allocation.  No counterpart in the reference.
 *
 * f3d_cmass2d takes a cudaMalloc'd scratch buffer for the partial sums of
 * its reduction on every call (and device copies of host arrays).  Some
 * callers cannot allocate there: a program whose device memory is fully
 * committed to resident scenarios (so a new cudaMalloc can fail), and one
 * that keeps other streams busy and cannot accept the device-wide
 * synchronisation that cudaFree implies.  This variant uses a fixed device
 * array of F3D_NOALLOC_SCRATCH_BYTES bytes compiled into the library.
 *
 *  - every array argument must be device (or managed) memory; host arrays
 *    are rejected with F3D_ERR_ARG.  outmass may be host or device memory
 *    and is accumulated as in f3d_cmass2d (outmass = outmass + outflow).
 *  - the scratch this call needs is at most 1024 block partials of 16
 *    bytes plus padding and an 8-byte accumulator (16.7 KB) for any grid; a
 *    call needing more than F3D_NOALLOC_SCRATCH_BYTES returns F3D_ERR_RANGE.
 *  - nothing in the scratch has to start at zero: each call writes every
 *    partial before reading it and copies outmass in first.
 *  - the first call on each device looks up the array's device address
 *    (cudaGetSymbolAddress with that device current) and caches it; make
 *    that first call before any stream capture begins.  The cached address
 *    does not survive cudaDeviceReset (the module is loaded again at a new
 *    address): a program that resets a device must not call this entry
 *    point on that device afterwards.
 *  - the array is shared by all calls in the process on one device: calls
 *    that overlap in time (from several host threads) race on it and give
 *    wrong sums.  Serialise them.
 *  - the call runs on the legacy default stream with synchronous copies and
 *    returns when the result is in outmass.  The legacy default stream
 *    waits for, and holds up, every blocking stream of the device; callers
 *    that keep other work in flight should create those streams with
 *    cudaStreamNonBlocking (or build with per-thread default streams) so
 *    that this call does not serialise with them. */
#define F3D_NOALLOC_SCRATCH_BYTES 32768
int f3d_cmass2d_noalloc(const double* c, const double* vx, const double* vy,
                        const double* vz, const double* vset, const int* nx,
                        const int* ny, const int* nz, const int* nc,
                        const int* ic_loc, const int* nc_loc, const int* iz_loc,
                        const int* nz_loc, const double* dx, const double* dy,
                        const double* dz, const double* dt, double* outmass);

/* Sources/cmass3d.f90:1 cmass3d(c,cload,cdry,cwet,nx,ny,nz,nc,dx,dy,dz,
 * massvol,massdep,massdry,masswet) */
int f3d_cmass3d(const double* c, const double* cload, const double* cdry,
                const double* cwet, const int* nx, const int* ny,
                const int* nz, const int* nc, const double* dx,
                const double* dy, const double* dz, double* massvol,
                double* massdep, double* massdry, double* masswet);

/* Sources/endstep.f90:80 getc0 followed by cload = cdry + cwet
 * (endstep.f90:35,60).  np = number of particle classes. */
int f3d_getc0(double* cdry, double* cwet, double* cload, const int* nx,
              const int* ny, const int* nc, const int* np);

/* Sources/setsrc.f90:1 setsrc (module state made explicit): c(i,j,k,:) +=
 * dt*tmrat(is,:)/vol0.  tmrat(nsou,nc) is already scaled by Hm1
 * (Sources/source.f90:75-77).  Sources with ksrc outside 1..nz are skipped
 * as in the reference; isrc/jsrc outside 1..nx/1..ny are F3D_ERR_RANGE. */
int f3d_setsrc(double* c, const int* nx, const int* ny, const int* nz,
               const int* nc, const int* nsou, const int* isrc,
               const int* jsrc, const int* ksrc, const double* tmrat,
               const double* dz, const double* zlayer, const double* Hm1,
               const double* dX1, const double* dX2, const double* dt);

/* Sources/finddt.f90:1 finddt (module state made explicit).  rkh1, vx and
 * rho are the scaled fields (Sources/meteo.f90:108-112). */
int f3d_finddt(const int* nx, const int* ny, const int* nz, const int* nc,
               const double* dX1, const double* dX2, const double* dz,
               const double* vx, const double* vy, const double* vz,
               const double* vset, const double* rkh1, const double* rkhor,
               const double* rkver, const double* safety_factor,
               double* dt, double* dtc);

/* Sources/kappa3.f90:1 kappa3 (module state made explicit).  vx, vy are
 * unscaled; rkver/rkhor are in/out (cells kappa3 does not assign keep
 * their input value, e.g. rkver(:,:,1) under SIMILARITY). */
int f3d_kappa3(const int* nx, const int* ny, const int* nz,
               const int* modkv, const int* modkh, const int* coord_sys,
               const double* rkv0, const double* rkh0, const double* Csh,
               const double* dX1, const double* dX2, const double* dx,
               const double* dy, const double* dz, const double* zlayer,
               const double* Hm1, const double* vx, const double* vy,
               const double* vptemp, const double* ustar, const double* zi,
               const double* rl, double* rkver, double* rkhor);

/* Sources/setvset.f90:1 setvset with vsettl's SAVEd drag coefficient made
 * explicit: *cd is read as the chain's entry value and written back with
 * its exit value (it starts at 1.0 at program start, setvset.f90:89).
 * tempe and rho are unscaled.  aggregate = (classname(np)=='aggregate'). */
int f3d_setvset(const int* nx, const int* ny, const int* nz, const int* nc,
                const int* np, const int* modv, const double* diam,
                const double* rhop, const double* psi, const double* sphe,
                const double* tempe, const double* rho, const int* aggregate,
                const double* vset_factor, double* vset, double* cd);

/* Diagnostic: the binary64 log (op 0) or exp (op 1) that setvset's Ganser
 * drag iteration uses in place of pow (a table-driven restatement, within a
 * few ulp), on n host or device values; op 2: the quotients a/b of n pairs
 * x = (a0, b0, a1, b1, ...) formed from the reciprocal of b the way the
 * plain form's sweeps divide (equal to the IEEE quotient).  No reference
 * counterpart. */
int f3d_dmath_eval(int op, long long n, const double* x, double* y);

/* Sources/setvdrydep.f90:1 setvdrydep (module state made explicit). */
int f3d_setvdrydep(const int* nx, const int* ny, const int* nc,
                   const double* diam, const double* zlayer,
                   const double* ldu, const double* rl, const double* znt,
                   const double* ustar, const double* tempe,
                   const double* rho, double* vdep);

/* Sources/meteo.f90:108-123 + Sources/corvver.f90:21-34 +
 * Sources/setdivu.f90:16-30: scale vx, rho, build rkh1, correct vz for
 * terrain (LON-LAT only) and compute divu.  All arrays in/out. */
int f3d_meteo_scale(const int* nx, const int* ny, const int* nz,
                    const int* coord_sys, const double* dX1,
                    const double* dX2, const double* dz, const double* Hm1,
                    const double* topg, double* vx, double* vy, double* vz,
                    double* rho, const double* rkhor, double* rkh1,
                    double* divu);

/* ------------------------------------------------------------------ */
/* 2. Coarse context API (state resident on the GPU)                   */
/* ------------------------------------------------------------------ */

/* Static description of one scenario: the grid of Sources/reagrd.f90, the
 * classes of Sources/reagrn.f90 and the model switches of readat.f90.
 * Pointers are host memory and are copied at creation. */
typedef struct f3d_grid {
  int nx, ny, nz;        /* interior cells (each >= 3)                    */
  int nc, np;            /* classes; particle classes are 1..np           */
  int coord_sys;         /* F3D_COORD_*                                   */
  int modkv, modkh, modv;/* F3D_MODKV_*, F3D_MODKH_*, F3D_MODV_*           */
  int wetdep;            /* WET_DEPOSITION = YES                          */
  int aggregate;         /* classname(np) == 'aggregate'                  */
  int precision;         /* F3D_PREC_FP64 or F3D_PREC_FP32                 */
  double dX1, dX2;       /* scaled cell sizes in m (reagrd.f90:157-158)    */
  double dx, dy;         /* native spacing (deg or m), used by CMAQ        */
  double rkh0, rkv0;     /* constant diffusivities (m2/s)                  */
  double Csh;            /* RAMS constant (Sources/Numeric.f90:26)         */
  double safety_factor;  /* CFL safety (Sources/inidat.f90:21)             */
  double vset_factor;    /* aggregate settling factor (readat.f90:386)     */
  const double* dz;      /* dz(0:nz)                                       */
  const double* zlayer;  /* zlayer(nz)                                     */
  const double* Hm1;     /* Hm1(nx,ny)                                     */
  const double* topg;    /* topg(nx,ny)                                    */
  const double* diam;    /* diam(nc) in m                                  */
  const double* rhop;    /* rhop(nc)                                       */
  const double* psi;     /* psi(nc) from setpsi                            */
  const double* sphe;    /* sphe(nc)                                       */
} f3d_grid;

/* Time-dependent meteorology of one scenario: nt snapshots of the DBS
 * variables, each valid on [times(it), times(it+1)) as selected by
 * libMaster/get_dbs_value_plane.f90:107-114 (piecewise constant, no
 * interpolation in time).  Fields are already on the model levels.
 * Arrays are snapshot-slowest; host or device memory. */
typedef struct f3d_met_series {
  int nt;
  const int* times;      /* nt snapshot times, seconds after DBS origin   */
  double time_lag;       /* DBS origin to run origin (reagrd.f90:277-308) */
  const double *u, *v, *w, *t, *tp, *rho;          /* nt*nx*ny*nz          */
  const double *ust, *pblh, *rmol, *znt, *prate;   /* nt*nx*ny (PRATE mm/s) */
  const double* ldu;     /* nx*ny land use, time independent              */
  const double *qv, *p;  /* nt*nx*ny*nz QV and P: read only by the
                            aggregation model (may be NULL otherwise)     */
} f3d_met_series;

/* Source intervals as in the .src file (libMaster/get_source_*.f90): the
 * interval [t1(i), t2(i)) holds nsou(i) sources; index arrays and rates are
 * concatenated over intervals, rates (nsou_i, nc) column major, unscaled. */
typedef struct f3d_src_series {
  int nint;
  const int *t1, *t2, *nsou;
  const int *isrc, *jsrc, *ksrc;
  const double* tmrat;
  /* plume temperature file of the aggregation model (settemplume,
   * source.f90:89-149): nplume(i) cells per interval, 1-based indices,
   * temperature (K) and water rate (kg/s), concatenated over intervals;
   * NULL nplume when aggregation is off */
  const int* nplume;
  const int *pix, *piy, *piz;
  const double *ptemp, *pwater;
} f3d_src_series;

/* One line of the mass-budget log (Sources/writim.f90:18-52). */
typedef struct f3d_log_record {
  int iiter;
  double time, dt, dtc;
  double massvol, massdep, massdry, masswet, outmass, erumass;
} f3d_log_record;

typedef struct f3d_ctx f3d_ctx;

int f3d_ctx_create(const f3d_grid* grid, f3d_ctx** out);
int f3d_ctx_destroy(f3d_ctx* ctx);
/* Device bytes held by a context of this grid (admission control): the
 * context as f3d_ctx_create makes it and the batched and serving forms use
 * it.  The second coefficient set of f3d_run's look-ahead meteo update
 * (F3D_OPT_PREFETCH) is not included. */
int f3d_ctx_footprint(const f3d_grid* grid, long long* bytes);

/* Sources/meteo.f90:19-149 on the device for one DBS snapshot: reamet's
 * vz(:,:,1)=0 and PRATE*3600, kappa3, setvset (continuing the cd chain),
 * setvdrydep, scaling, corvver, setdivu and finddt.  Fields are the raw
 * DBS variables of the snapshot (host or device pointers). */
int f3d_meteo(f3d_ctx* ctx, const double* u, const double* v,
              const double* w, const double* t, const double* tp,
              const double* rho, const double* ust, const double* pblh,
              const double* rmol, const double* znt, const double* prate,
              const double* ldu);

/* Sources/source.f90:24-77: install the sources of one interval (rates
 * unscaled, as read), compute flowrate and scale rates by Hm1. */
int f3d_source(f3d_ctx* ctx, int nsou, const int* isrc, const int* jsrc,
               const int* ksrc, const double* tmrat);

/* Sources/Fall3d.f90:112-117: time += dt, iiter += 1,
 * erumass += flowrate*dt, setsrc, sizloop (setbcc, advection, diffusion,
 * wetdep, accum for every class, clip, cmass2d). */
int f3d_step(f3d_ctx* ctx);

/* Sources/endstep.f90:59-60 + writim.f90:18: getc0, cload = cdry + cwet and
 * cmass3d on the device. */
int f3d_budget(f3d_ctx* ctx, double* massvol, double* massdep,
               double* massdry, double* masswet);

/* The number of NaN or infinite values in the concentrations (the whole
 * halo array of every class, in the context's storage precision) and in
 * cdry + cwet.  The reference lets a non-finite value propagate; this is the
 * check a driver makes at its log steps to stop with runend instead (one
 * read of c, about 0.1 ms for 400x300x50 cells and 16 classes). */
int f3d_count_nonfinite(f3d_ctx* ctx, long long* in_c, long long* in_deposits);

/* Scalar state of the time loop. */
int f3d_get_state(const f3d_ctx* ctx, int* iiter, double* time, double* dt,
                  double* dtc, double* erumass, double* outmass,
                  double* flowrate);
int f3d_set_time(f3d_ctx* ctx, double time, int iiter);

/* Copy state to host (any pointer may be NULL): c (binary64 even in the
 * FP32 form), cdry, cwet (nx,ny,0:nc), vset (nx,ny,nz,nc), vdep. */
int f3d_download(f3d_ctx* ctx, double* c, double* cdry, double* cwet,
                 double* vset, double* vdep);
/* Overwrite the concentration state (restart): c (binary64), cdry, cwet
 * (NULL leaves a field unchanged), plus erumass, outmass and the cd state. */
int f3d_upload_state(f3d_ctx* ctx, const double* c, const double* cdry,
                     const double* cwet, double erumass, double outmass,
                     double cd);
/* Coefficient fields after the last f3d_meteo, for inspection: the scaled
 * vx, vy, vz, rho, rkhor, rkh1, rkver (each nx*ny*nz; NULL skips). */
int f3d_download_coeffs(f3d_ctx* ctx, double* vx, double* vy, double* vz,
                        double* rho, double* rkhor, double* rkh1,
                        double* rkver);
/* vsettl iteration counts of the last f3d_meteo, nx*ny*nz*nc int32
 * (0 for the closed-form Dellino model; the reference does not keep them). */
int f3d_download_iters(f3d_ctx* ctx, int* iters);
/* vsettl drag-coefficient chain state (setvset.f90:89). */
int f3d_get_cd(const f3d_ctx* ctx, double* cd);

/* Output quantities of Sources/printres_nc.f90 on the device:
 * LOAD = cload(:,:,0)/Hm1 (:105-123), COL_MASS (:216-247),
 * C_GRND (:389-411).  Each (nx,ny) binary64; NULL skips. */
int f3d_outputs(f3d_ctx* ctx, double* load, double* col_mass,
                double* c_grnd);

/* One output variable of Sources/printres_nc.f90, computed on the device
 * in binary64 in the reference's order of operations and written to dst
 * (host or device memory) as binary64 or, like the reference's NF90_FLOAT
 * netCDF variables (printres_nc.f90:805-841), as binary32.  2-D variables
 * are (nx,ny), x fastest; F3D_OUT_CON, _WIND and _MAGGR are (nx,ny,nz).
 * `index` selects:
 *   F3D_OUT_LOAD      deposit load kg/m2, cload(:,:,index)/Hm1 with
 *                     index 0 = all particles, 1..np one class (:105-146)
 *   F3D_OUT_WET       wet deposit kg/m2, cwet(:,:,index)/Hm1 (:148-189)
 *   F3D_OUT_THICK     deposit thickness in cm (:191-214); index unused
 *   F3D_OUT_COL_MASS  column mass g/m2: index 0 = particles (:216-247),
 *                     g = 1..nc-np the g-th gas class (:249-279)
 *   F3D_OUT_PM_COL    column mass of the particles with diameter <= index
 *                     micrometres, index 5, 10 or 20 (:281-387)
 *   F3D_OUT_C_GRND    first-layer particle concentration g/m3 (:389-411)
 *   F3D_OUT_PM_GRND   first-layer PM concentration, index 5/10/20 (:413-493)
 *   F3D_OUT_AOT05     aerosol optical thickness (:495-540, get_AOT_prop
 *                     :2066-2123); index unused
 *   F3D_OUT_CON       concentration g/m3: index 0 = all particles
 *                     (:575-601), 1..nc one class (:646-671); asl != 0
 *                     moves it from terrain-following levels to heights
 *                     above sea level (Sources/ter2asl.f90:1-55, used when
 *                     terrain_following is false)
 *   F3D_OUT_WIND      (nx,ny,nz) wind written with the gravity current,
 *                     index 1 = vx*Hm1, 2 = vy*Hm1 (:603-644); asl as above
 *   F3D_OUT_MAGGR     (nx,ny,nz) accumulated aggregate mass, kg
 *                     (:673-690; aggregation on); asl as above
 * The deposit variables first form cload = cdry + cwet and the class sums
 * (endstep.f90:35,60). */
#define F3D_OUT_LOAD      1
#define F3D_OUT_WET       2
#define F3D_OUT_THICK     3
#define F3D_OUT_COL_MASS  4
#define F3D_OUT_PM_COL    5
#define F3D_OUT_C_GRND    6
#define F3D_OUT_PM_GRND   7
#define F3D_OUT_AOT05     8
#define F3D_OUT_CON       9
#define F3D_OUT_WIND     10
#define F3D_OUT_MAGGR    11
#define F3D_OUT_BINARY64  0
#define F3D_OUT_BINARY32  1
int f3d_output(f3d_ctx* ctx, int var, int index, int asl, void* dst,
               int dst_type);
/* Tracking points (Sources/writps.f90, writps_air.f90, the point location
 * of Sources/reaout.f90:180-224): for each of npts points (x, y in the
 * grid's coordinates, origin xo, yo), bilinear in the cell that holds it,
 * out receives 7 + 3*nz + 1 + np binary64 values per point: deposit load
 * (kg/m2), thickness (cm), ground concentration, PM05, PM10, PM20 (g/m3),
 * column mass (g/m2); nz concentrations (g/m3), nz aerosol extinctions
 * (1/Mm), nz number concentrations (1/cm3) and the AOD; np class loads
 * (the final deposit of writps_end).  Forms cload = cdry + cwet first. */
int f3d_track_points(f3d_ctx* ctx, int npts, const double* xpts,
                     const double* ypts, double xo, double yo, double* out);

/* Particle concentration g/m3 at a flight level (hundreds of feet) of the
 * ICAO standard atmosphere (printres_nc.f90:542-573, Sources/setcut.f90):
 * interpolated in the pressure p(nx,ny,nz) of the model levels (Pa, the
 * DBS variable P; host or device memory); (nx,ny). */
int f3d_output_fl(f3d_ctx* ctx, double flight_level, const double* p,
                  void* dst, int dst_type);

/* Gravity current of the umbrella cloud (Costa and Macedonio;
 * GRAVITY_CURRENT = YES, Sources/readat.f90:150-213).  While it is on, every
 * f3d_meteo adds the radial wind of Sources/addradialwind.f90 to the scaled
 * vx, vy after corvver and before setdivu and finddt (meteo.f90:140), and
 * every mass-budget log step of f3d_run applies Sources/divcorr.f90 after
 * the budget (endstep.f90:71).  NULL switches it off.  Not available in a
 * batch (f3d_batch_add rejects such a context). */
typedef struct f3d_gravity_current {
  double c_flow_rate, lambda_grav, k_entrain, brunt_vaisala; /* readat.f90:169-205 */
  double center_x, center_y; /* radial_wind_lon/lat (LON-LAT) or radial_wind_x/y
                                (UTM): the vent (readat.f90:209-212)          */
  double xorigr, yorigr;     /* grid origin (Sources/reagrd.f90:152-153)      */
  double h_tot;              /* maxval(zs): the highest source point, m       */
  double beg_time;           /* the run's start (time of the eruption onset)  */
} f3d_gravity_current;
int f3d_set_gravity_current(f3d_ctx* ctx, const f3d_gravity_current* gc);

/* Aggregation in transport (Costa et al. 2010; AGGREGATION_IN_TRANSPORT
 * = yes, Sources/readat.f90:350-440), for a grid whose class np is the
 * aggregate (grid.aggregate).  While it is on, the first f3d_step after
 * an f3d_meteo or f3d_source runs agrpar (Sources/agrsrc.f90:95-319;
 * Fall3d.f90:101-110) and every step adds the aggregation source of
 * agrsrc (:1-91) every ndtagr steps after the point sources
 * (setsrc.f90:37-76), accumulating Maggr.  The classes iaggr..np-1 that
 * aggregate are those finer than the aggregate (readat.f90:400-409).
 * QV and P of the snapshot (f3d_aggregation_met, before f3d_meteo) and
 * the plume temperatures of the source interval (f3d_aggregation_plume,
 * after f3d_source; the reference's settemplume) are inputs; f3d_run
 * takes them from the series (qv/p of f3d_met_series, the plume lists of
 * f3d_src_series).  NULL switches it off.  Not available in a batch. */
typedef struct f3d_aggregation {
  double Df;          /* FRACTAL_EXPONENT (readat.f90:411-421, default 3) */
  int ndtagr;         /* N_DT_AGGREGATION (readat.f90:423-433, default 1) */
  const double* fc;   /* fc(1:np): mass fractions of the grn file (host) */
} f3d_aggregation;
int f3d_set_aggregation(f3d_ctx* ctx, const f3d_aggregation* ag);
int f3d_aggregation_met(f3d_ctx* ctx, const double* qv, const double* p);
int f3d_aggregation_plume(f3d_ctx* ctx, int n, const int* ix, const int* iy,
                          const int* iz, const double* temp,
                          const double* water);
/* Maggr(nx,ny,nz): accumulated mass of aggregates, kg (setsrc.f90:62-76) */
int f3d_download_maggr(f3d_ctx* ctx, double* maggr);

/* Sources/Fall3d.f90:73-121: the time loop from beg_time to end_time
 * (at most max_steps steps if max_steps > 0), reading meteorology and
 * sources when their intervals end, logging the mass budget at the steps
 * endstep.f90:51 selects.  Up to log_cap records are written to log. */
int f3d_run(f3d_ctx* ctx, const f3d_met_series* met,
            const f3d_src_series* src, double beg_time, double end_time,
            int max_steps, f3d_log_record* log, int log_cap, int* nlog);

/* Time loop state of f3d_run kept in the context so that f3d_run can be
 * called repeatedly to continue (each call resumes where the last ended). */
int f3d_run_reset(f3d_ctx* ctx);

/* Lossless checkpoint of a run's state (c in the context's precision, cdry,
 * cwet, time, iiter, erumass, outmass and the settling-velocity chain state)
 * to a file, and its restore into a context created with the same grid and
 * precision.  Replaces the reference's restart (Sources/wrirst.f90:1,
 * Sources/rearst.f90:1: c and cload in binary32, no chain state).  After
 * f3d_ctx_restore, f3d_run with the run's met and source series continues
 * exactly as the uninterrupted run: it replays the current meteo and source
 * updates from the saved chain state, which rebuilds every coefficient. */
int f3d_ctx_save(f3d_ctx* ctx, const char* path);
int f3d_ctx_restore(f3d_ctx* ctx, const char* path);

/* Options of a context (f3d_set_option / f3d_get_option). */
#define F3D_OPT_FUSED 1  /* FP32 form: 1 = one fused kernel per step (default),
                            0 = one kernel per reference routine.  Grids
                            with a decreasing zlayer or >= 2^31 cells per
                            class always use the per-routine kernels.     */
#define F3D_OPT_TILE  2  /* fused kernel tile region x by y / threads:
                            0 = 32x32/256, 1 = 32x64/512, 2 = 32x32/512,
                            3 = 64x32/512 with two columns per lane
                            (default); results do not depend on it       */
#define F3D_OPT_GRAPH 3  /* batches: 1 = replay one CUDA graph per batch step
                            (default), 0 = launch the kernels one by one   */
#define F3D_OPT_PREFETCH 4 /* f3d_run: 1 = compute the next DBS snapshot's
                            meteo update (meteo.f90:27-149) on a second,
                            lowest-priority stream while the current
                            interval steps, into a second set of the
                            coefficient fields, and exchange the sets when
                            the update is due (default); 0 = compute it
                            when due.  Results do not depend on it.  Not
                            used with the gravity current, aggregation or
                            in a batch; the second set is allocated on the
                            first use (or when the option is set to 1) and
                            is not counted by f3d_ctx_footprint (without
                            room for it the updates are made when due).    */
int f3d_set_option(f3d_ctx* ctx, int key, int value);
int f3d_get_option(const f3d_ctx* ctx, int key, int* value);

/* The CUDA stream all work of this context is enqueued on (cudaStream_t),
 * for callers that time or order their own work against it. */
int f3d_ctx_stream(f3d_ctx* ctx, void** stream);

/* Per-kernel timing with CUDA events recorded on the context's stream
 * around every launch of f3d_step while enabled.  f3d_profile_read returns,
 * for up to cap kernel kinds, the name, launch count and total milliseconds
 * since the last reset (it synchronises the stream). */
int f3d_profile_enable(f3d_ctx* ctx, int enable);
int f3d_profile_read(f3d_ctx* ctx, int cap, char* names, int name_len,
                     long long* launches, double* total_ms, int* nkinds);

/* Number of CUDA kernels this library launched since load (diagnostic). */
long long f3d_kernel_launches(void);

/* Synchronise the context's stream.  Returns F3D_ERR_CUDA if a staging wait
 * of the step kernel gave up since the last check (a tensor copy that did not
 * arrive within its bounded wait; the kernel then continues without hanging
 * and its results are not to be used); f3d_run checks the same at its end. */
int f3d_sync(f3d_ctx* ctx);

/* ------------------------------------------------------------------------
 * Batched precision form (no counterpart in the reference, whose unit of
 * work is one scenario per run).  A batch advances the time loops of up to
 * max_scenarios precision-form contexts together: each scenario runs its
 * own Fall3d.f90:79-121 loop (source and meteo updates when due, its own dt,
 * its own x/y alternation), and one batch step performs the transport step
 * of every running scenario in a single persistent launch, replayed as one
 * CUDA graph.  A scenario's results are those of f3d_run on the same
 * context.  Contexts stay owned by the caller and must not be used
 * elsewhere while they are in a batch.
 */
typedef struct f3d_batch f3d_batch;
int f3d_batch_create(int max_scenarios, f3d_batch** out);
int f3d_batch_destroy(f3d_batch* b);
/* Joins a context (FP32 form) to the batch: its time loop starts at
 * beg_time and ends at end_time (or after max_steps > 0 steps), with the
 * met and source series of f3d_run; log (log_cap records) receives the
 * mass-budget records of endstep.f90:51.  *slot identifies it. */
int f3d_batch_add(f3d_batch* b, f3d_ctx* ctx, const f3d_met_series* met,
                  const f3d_src_series* src, double beg_time, double end_time,
                  int max_steps, f3d_log_record* log, int log_cap, int* slot);
/* One step of every running scenario; *n_running = scenarios still running. */
int f3d_batch_step(f3d_batch* b, int* n_running);
/* state: 0 free, 1 running, 2 done, 3 failed (the return code and
 * f3d_last_error give the failure). */
int f3d_batch_poll(f3d_batch* b, int slot, int* state, int* steps, int* nlog);
/* Frees a slot (stops the scenario if still running). */
int f3d_batch_release(f3d_batch* b, int slot);
int f3d_batch_sync(f3d_batch* b);
/* F3D_OPT_TILE (tile shape of the step kernel) and F3D_OPT_GRAPH. */
int f3d_batch_set_option(f3d_batch* b, int key, int value);
int f3d_batch_get_option(const f3d_batch* b, int key, int* value);
/* Times the step kernel of the running scenarios for each tile shape (reps
 * launches each, without changing any result), keeps the fastest and
 * returns it and the per-shape milliseconds (ms[4]; -1 for a shape that
 * does not apply).  Call it after the first batch step. */
int f3d_batch_autotune(f3d_batch* b, int reps, int* best, float* ms);
int f3d_batch_stats(const f3d_batch* b, long long* batch_steps,
                    double* cell_class_steps, int* n_running);
int f3d_batch_stream(const f3d_batch* b, void** stream);

/* ------------------------------------------------------------------------
 * Serving form (no counterpart in the reference): continuous batching of
 * forecast requests.  Requests are submitted as they arrive and wait in
 * arrival order; f3d_server_progress admits waiting requests while the
 * resident footprint (f3d_ctx_footprint of each precision-form context)
 * stays under hbm_cap_bytes and a slot is free, then advances every running
 * request by batch steps.  A finished request's outputs (LOAD, COL_MASS,
 * C_GRND and the mass-budget log) are kept in host memory and its device
 * memory is freed for the next admission.  The grid, met and source arrays
 * of a request must stay valid until it completes.
 */
typedef struct f3d_server f3d_server;
int f3d_server_create(long long hbm_cap_bytes, int max_running, f3d_server** out);
int f3d_server_destroy(f3d_server* srv);
int f3d_server_submit(f3d_server* srv, const f3d_grid* grid, const f3d_met_series* met,
                      const f3d_src_series* src, double beg_time, double end_time,
                      int log_cap, int* request_id);
/* Admits, runs up to max_steps batch steps (fewer if a request completes),
 * collects completed requests. */
int f3d_server_progress(f3d_server* srv, int max_steps, int* n_running, int* n_queued);
/* state: 0 queued, 1 running, 2 done, 3 failed, 4 forgotten; seconds of a
 * monotonic clock at submission, admission and completion. */
int f3d_server_poll(f3d_server* srv, int request_id, int* state, double* t_submit,
                    double* t_admit, double* t_done, long long* steps);
int f3d_server_result(f3d_server* srv, int request_id, double* load, double* col_mass,
                      double* c_grnd, f3d_log_record* log, int log_cap, int* nlog);
int f3d_server_forget(f3d_server* srv, int request_id);
int f3d_server_stats(const f3d_server* srv, long long* used_bytes, double* cell_class_steps,
                     long long* batch_steps, int* n_running, int* n_queued);
int f3d_server_batch(f3d_server* srv, f3d_batch** batch);

#ifdef __cplusplus
}
#endif
#endif /* FALL3D_GPU_H */
