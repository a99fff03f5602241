// f3d_ctx_impl.h -- the context object behind the coarse C ABI (shared by
// the single-scenario API in f3d_ctx.cu and the batched form in f3d_batch.cu).
#pragma once

#include <string>
#include <vector>

#include "../../include/fall3d_gpu.h"
#include "f3d_internal.h"
#include "f3d_fused.h"

// The fields a meteo update writes and the steps read (f3d_meteo): the
// binary64 met and coefficients, the plain form's diffusion factors, the
// binary32 copies and the halo-layout copies of the precision form.  A
// look-ahead update (F3D_OPT_PREFETCH) fills a second set of them for the
// next DBS snapshot and the two sets are exchanged at the update.
#define F3D_MET_SET_D(X) \
  X(double, vx) X(double, vy) X(double, vz) X(double, tempe) X(double, vptemp) X(double, rho) \
  X(double, rkhor) X(double, rkh1) X(double, rkver) X(double, divu) X(double, vset) X(double, vdep) \
  X(double, ustar) X(double, zi) X(double, rl) X(double, znt) X(double, prate) X(int, iters) \
  X(double, lrho64) X(double, pkx64) X(double, pky64) X(double, rksz64)
#define F3D_MET_SET_F(X) \
  X(float, vx32) X(float, vy32) X(float, vz32) X(float, rho32) X(float, rkhor32) X(float, rkh132) \
  X(float, rkver32) X(float, vset32) X(float, vdep32) X(float, lrho32) X(float, pkx32) X(float, pky32) \
  X(float, pkz32) X(float, vk32) X(float, vxh) X(float, vyh) X(float, lrhoh) X(float, pkxh) \
  X(float, pkyh) X(float, pkzh) X(float, vkh)

struct f3d_met_set {
#define F3D_X(T, n) T* n = nullptr;
  F3D_MET_SET_D(F3D_X)
  F3D_MET_SET_F(F3D_X)
#undef F3D_X
  f3d::F2Maps maps2{};
};

struct f3d_ctx {
  f3d_grid g{};
  Dims d{};
  int prec = 64;
  cudaStream_t stream = nullptr;
  std::vector<void*> allocs;
  // static
  double *dz = nullptr, *zlayer = nullptr, *Hm1 = nullptr, *topg = nullptr;
  double *diam = nullptr, *rhop = nullptr, *psi = nullptr, *sphe = nullptr;
  std::vector<double> h_diam, h_rhop;  // host copies (output class selections)
  std::vector<double> h_zlayer;        // host copy (gravity current levels)
  double hm11 = 1.0;                   // Hm1(1,1)
  // gravity current (f3d_set_gravity_current)
  f3d_gravity_current gc{};
  int gc_on = 0;
  double mfr_scaled = 0.0;  // sum of the Hm1-scaled source rates (addradialwind.f90:61)
  // aggregation in transport (f3d_set_aggregation)
  int agr_on = 0, agr_iaggr = 0, agr_ndtagr = 1, agr_ipass = 0, agr_due = 0;
  int agr_npar = 0;    // agrpar calls since the last meteo update
  int agr_replay = 0;  // agrpar calls owed by a restored run
  double agr_Df = 3.0, agr_sumNi = 0.0;
  std::vector<double> agr_fc;  // fc(1:np)
  double *agr_fc_dev = nullptr, *agr_cls = nullptr;
  double *agr_al = nullptr, *agr_ab = nullptr, *agr_as = nullptr, *agr_ad = nullptr;  // Alagr..Adagr
  double *agr_maggr = nullptr, *agr_tplume = nullptr, *agr_qv = nullptr, *agr_p = nullptr;
  // met and coefficients (binary64)
  double *vx = nullptr, *vy = nullptr, *vz = nullptr, *tempe = nullptr, *vptemp = nullptr;
  double *rho = nullptr, *rkhor = nullptr, *rkh1 = nullptr, *rkver = nullptr, *divu = nullptr;
  double *vset = nullptr, *vdep = nullptr;
  double *ustar = nullptr, *zi = nullptr, *rl = nullptr, *znt = nullptr, *prate = nullptr,
         *ldu = nullptr;
  int* iters = nullptr;
  // state
  double* c64 = nullptr;
  float* c32 = nullptr;
  double *cdry = nullptr, *cwet = nullptr, *cload = nullptr;
  // FP32 copies
  float *vx32 = nullptr, *vy32 = nullptr, *vz32 = nullptr, *rho32 = nullptr, *rkhor32 = nullptr,
        *rkh132 = nullptr, *rkver32 = nullptr, *vset32 = nullptr, *vdep32 = nullptr,
        *dz32 = nullptr;
  // fused FP32 step: second concentration buffer, 1/rho, K*rho products,
  // per-column wet rate, per-class wet-deposition switch
  float* c32b = nullptr;
  float *lrho32 = nullptr, *pkx32 = nullptr, *pky32 = nullptr, *pkz32 = nullptr;
  // plain form: 1/rho, rkh1*rho, rkhor*rho and the diffz face coefficients
  // of the current meteo update (the class-independent factors of the
  // diffusion sweeps)
  double *lrho64 = nullptr, *pkx64 = nullptr, *pky64 = nullptr, *rksz64 = nullptr;
  float* vk32 = nullptr;  // vz + vset per class
  // the fused met fields in the halo layout of c (two-columns-per-lane kernel)
  float *vxh = nullptr, *vyh = nullptr, *lrhoh = nullptr, *pkxh = nullptr, *pkyh = nullptr,
        *pkzh = nullptr, *vkh = nullptr;
  f3d::F2Maps maps2{};  // tensor maps of those fields (shape-3 step kernel)
  double* lambda2d = nullptr;
  unsigned char* wet_class = nullptr;
  int opt_fused = 1, opt_tile = 3;
  // the fused kernel applies: zlayer non-decreasing, 32-bit offsets in a class
  int fused_ok = 1;
  // sources
  int *isrc = nullptr, *jsrc = nullptr, *ksrc = nullptr;
  int* slink = nullptr;  // source_links of the current sources (2 * nsou)
  double* tmrat = nullptr;
  int src_cap = 0, nsou = 0;
  // scratch
  void* red_scratch = nullptr;
  void* vset_scratch = nullptr;
  double* small = nullptr;  // [0] outmass, [1..4] budget, [8] cd, [16] dtcn bits, [24] status, [40..41] non-finite counts
  // host scalars of the time loop
  double time = 0.0, dt = 1.0, dtc = 0.0, erumass = 0.0, flowrate = 0.0;
  int iiter = 0, have_met = 0;
  // f3d_run loop state (Fall3d.f90:73-78)
  int run_started = 0, meteotime = 1, sourcetime = 1;
  double meteo_time = 0.0, source_time = 0.0;
  // look-ahead meteo update (F3D_OPT_PREFETCH, f3d_run only): the next
  // snapshot's coefficients computed into `shadow` on the lower-priority
  // stream `side` while the current interval steps
  int opt_prefetch = 1;
  int pref_ready = 0;      // a look-ahead update was enqueued (for snapshot pref_itime)
  int pref_itime = -1, pref_alloc = 0, pref_failed = 0;
  f3d_met_set shadow{};
  cudaStream_t side = nullptr;
  cudaEvent_t ev_pref = nullptr, ev_free = nullptr, ev_staged = nullptr;
  unsigned long long* pref_host = nullptr;  // page-locked: dtcn bits, status
  double* pref_stage = nullptr;             // the next snapshot's raw fields
  // per-kernel event profiler (f3d_profile_*)
  int prof = 0;
  struct ProfRec {
    int kind;
    cudaEvent_t a, b;
  };
  std::vector<ProfRec> prof_pending;
  std::vector<cudaEvent_t> prof_pool;
  std::vector<std::string> prof_names;
  std::vector<long long> prof_count;
  std::vector<double> prof_ms;
};

namespace f3d {
int ctx_error(int code, const char* msg);
// Pieces of the time loop (Fall3d.f90:79-121) shared with the batched form.
// Source and meteo updates due at x->time (Fall3d.f90:83-101).
// lookahead: compute the next snapshot's meteo update on the second stream
// while this interval steps (f3d_run with F3D_OPT_PREFETCH).
int ctx_run_prepare(f3d_ctx* x, const f3d_met_series* met, const f3d_src_series* src, double end_time,
                    int lookahead = 0);
// time = time + dt, iiter = iiter + 1, erumass (Fall3d.f90:112-114)
void ctx_advance(f3d_ctx* x);
// the mass-budget log of endstep.f90:51 when due
int ctx_log(f3d_ctx* x, f3d_log_record* log, int log_cap, int* nlog);
// arguments of the fused precision-form step for the context's state
FusedArgs ctx_fused_args(f3d_ctx* x);
int ctx_check_step_status(f3d_ctx* x);
inline double* ctx_outmass(f3d_ctx* x) { return x->small; }
// gravity current (f3d_gravity.cu): addradialwind on the scaled winds of
// a meteo update, divcorr with the budget of a log step
int gc_addradialwind(f3d_ctx* x);
int gc_divcorr(f3d_ctx* x, double massvol, double massdep, double outmass);
// aggregation (f3d_aggregation.cu): agrpar after the updates of a step,
// agrsrc after its point sources
int agg_agrpar(f3d_ctx* x);
int agg_setsrc(f3d_ctx* x);
int agg_restore_vset(f3d_ctx* x, int times);
// a zero-filled device allocation owned by the context
int ctx_alloc(f3d_ctx* x, void** p, size_t bytes);
// the binary32 copies of class ic's settling velocity (vset32, vk32 and
// its halo-layout copy) after vset changed on the device
void refresh_fp32_class(f3d_ctx* x, int ic);
// waits for a look-ahead meteo update in flight and drops it (its chain
// state is not committed)
void ctx_prefetch_drop(f3d_ctx* x);
}  // namespace f3d
