// f3d_batch.cu -- the batched precision form: the time loops of many
// scenarios (contexts) advanced together, one step of all of them per
// persistent launch.
//
// Each scenario keeps its own context (state, coefficients, sources, time
// loop scalars) and its own time loop, exactly Fall3d.f90:79-121: source and
// meteo updates when due (on the host, through the context's own path),
// time = time + dt, iiter = iiter + 1, then the step.  Only the step is
// batched: one CUDA graph holds
//
//   setsrc of every scenario              (k_setsrc_batch, scenario = grid.y)
//   the fused step of every (scenario, tile, class)   (persistent kernel)
//   cmass2d of every scenario             (k_cmass2d_batch + finish)
//   the per-scenario batch-step counters  (k_batch_advance)
//
// and is replayed once per batch step.  What changes from step to step lives
// in device memory: the batch-step counter of a scenario selects which of its
// two buffers holds the state and the x/y order (sizloop.f90:42-48).  The
// argument tables are rewritten (after a stream synchronisation) only when a
// scenario's dt or sources change or the set of scenarios changes; the graph
// is captured again only when the set changes.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "f3d_ctx_impl.h"

using namespace f3d;

namespace {

#define BK(call)                                                                             \
  do {                                                                                       \
    cudaError_t e_ = (call);                                                                 \
    if (e_ != cudaSuccess) {                                                                 \
      std::string m_ = std::string(#call) + ": " + cudaGetErrorString(e_);                   \
      return f3d::ctx_error(F3D_ERR_CUDA, m_.c_str());                                       \
    }                                                                                        \
  } while (0)

struct Scen {
  f3d_ctx* x = nullptr;
  const f3d_met_series* met = nullptr;
  const f3d_src_series* src = nullptr;
  double end = 0.0;
  int max_steps = 0, steps = 0;
  f3d_log_record* log = nullptr;
  int log_cap = 0, nlog = 0;
  int bstep = 0, iiter0 = 0;
  float *c_a = nullptr, *c_b = nullptr;  // the context's buffers when it joined
  int state = 0;                         // 0 free, 1 running, 2 done, 3 failed
  int status = 0;
  std::string error;
};

}  // namespace

struct f3d_batch {
  cudaStream_t stream = nullptr;
  BatchFork fork;  // second stream of the odd-nx part of the step kernel
  int cap = 0;
  std::vector<Scen> slot;
  std::vector<int> active;  // running slots in batch order
  // device tables (batch order)
  BatchAux* d_aux = nullptr;
  int *d_item_off = nullptr, *d_bstep = nullptr, *d_iiter0 = nullptr, *d_counter = nullptr;
  void* d_red = nullptr;
  // pinned staging of the tables
  BatchAux* h_aux = nullptr;
  FusedArgs* h_args = nullptr;
  F2Maps* h_maps = nullptr;  // the scenarios' tensor maps (shape 3), batch order
  F2Maps* d_maps = nullptr;
  int *h_item_off = nullptr, *h_bstep = nullptr, *h_iiter0 = nullptr;
  // graph of one step
  cudaGraphExec_t exec = nullptr;
  cudaEvent_t ev = nullptr;  // hands a finished scenario's context back to its own stream
  bool tables_dirty = true, graph_dirty = true;
  int use_graph = 1;
  int shape = 0, grid = 0, max_nz = 0, max_nc = 0, max_nsou = 0;
  int split = 0, total = 0;  // items of the even-nx scenarios come first (shape 3)
  int graph_kernels = 0;     // kernels in one replay of the graph
  long long batch_steps = 0;
  double cell_class_steps = 0.0;
};

namespace {

int table_rebuild(f3d_batch* b) {
  const int n = (int)b->active.size();
  BK(cudaStreamSynchronize(b->stream));  // the previous step no longer reads the tables
  // batch order: scenarios with an even nx first (the shape-3 kernel runs
  // them and the others in two launches)
  std::stable_partition(b->active.begin(), b->active.end(),
                        [&](int id) { return (b->slot[id].x->g.nx & 1) == 0; });
  int off = 0;
  b->split = -1;
  b->max_nz = 0;
  b->max_nc = 0;
  const int nsou_blocks = (b->max_nsou + 127) / 128;
  b->max_nsou = 0;
  for (int q = 0; q < n; ++q) {
    Scen& s = b->slot[b->active[q]];
    f3d_ctx* x = s.x;
    FusedArgs a = ctx_fused_args(x);
    a.c_in = s.c_a;
    a.c_out = s.c_b;
    b->h_args[q] = a;
    b->h_maps[q] = x->maps2;
    BatchAux& u = b->h_aux[q];
    u = BatchAux{};
    u.c_a = s.c_a;
    u.c_b = s.c_b;
    u.cstride = x->d.halo();
    u.d = x->d;
    u.nc = x->g.nc;
    u.dt = x->dt;
    u.nsou = x->nsou;
    u.isrc = x->isrc;
    u.jsrc = x->jsrc;
    u.ksrc = x->ksrc;
    u.link = x->slink;
    u.tmrat = x->tmrat;
    u.dz = x->dz;
    u.zlayer = x->zlayer;
    u.Hm1 = x->Hm1;
    u.dX1 = x->g.dX1;
    u.dX2 = x->g.dX2;
    u.vx = x->vx;
    u.vy = x->vy;
    u.vz = x->vz;
    u.vset = x->vset;
    u.outmass = ctx_outmass(x);
    if (b->split < 0 && (x->g.nx & 1)) b->split = off;
    b->h_item_off[q] = off;
    off += fused_tiles(x->g.nx, x->g.ny, b->shape) * x->g.nc;
    b->h_bstep[q] = s.bstep;
    b->h_iiter0[q] = s.iiter0;
    b->max_nz = std::max(b->max_nz, x->g.nz);
    b->max_nc = std::max(b->max_nc, x->g.nc);
    b->max_nsou = std::max(b->max_nsou, x->nsou);
  }
  if ((b->max_nsou + 127) / 128 != nsou_blocks) b->graph_dirty = true;  // setsrc's grid changed
  b->h_item_off[n] = off;
  b->total = off;
  if (b->split < 0) b->split = off;
  if (n > 0) {
    if (upload_batch_args(b->h_args, n, b->stream)) return ctx_error(F3D_ERR_CUDA, "constant table upload failed");
    BK(cudaMemcpyAsync(b->d_aux, b->h_aux, sizeof(BatchAux) * n, cudaMemcpyHostToDevice, b->stream));
    BK(cudaMemcpyAsync(b->d_maps, b->h_maps, sizeof(F2Maps) * n, cudaMemcpyHostToDevice, b->stream));
    BK(cudaMemcpyAsync(b->d_bstep, b->h_bstep, sizeof(int) * n, cudaMemcpyHostToDevice, b->stream));
    BK(cudaMemcpyAsync(b->d_iiter0, b->h_iiter0, sizeof(int) * n, cudaMemcpyHostToDevice, b->stream));
  }
  BK(cudaMemcpyAsync(b->d_item_off, b->h_item_off, sizeof(int) * (n + 1), cudaMemcpyHostToDevice, b->stream));
  BK(cudaStreamSynchronize(b->stream));  // the pinned staging may be rewritten from here on
  b->tables_dirty = false;
  return F3D_OK;
}

// the kernels of one batch step, in stream order
int enqueue_step(f3d_batch* b, int commit_only_fused) {
  const int n = (int)b->active.size();
  BK(cudaMemsetAsync(b->d_counter, 0, 2 * sizeof(int), b->stream));
  if (!commit_only_fused) launch_setsrc_batch(b->d_aux, b->d_bstep, n, b->max_nc, b->max_nsou, b->stream);
  launch_step_fused_batch(b->shape, b->grid, b->d_item_off, n, b->split, b->total, b->d_counter, b->d_bstep,
                          b->d_iiter0, commit_only_fused ? 0 : 1, b->max_nz, b->d_maps, b->stream, &b->fork);
  if (!commit_only_fused) {
    launch_cmass2d_batch(b->d_aux, b->d_bstep, n, b->d_red, b->stream);
    launch_batch_advance(b->d_bstep, n, b->stream);
  }
  return F3D_OK;
}

int graph_rebuild(f3d_batch* b) {
  if (b->exec) {
    cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;
  }
  b->grid = fused_batch_grid(b->shape, std::max(b->max_nz, 3));
  if (b->grid < 1) return ctx_error(F3D_ERR_CUDA, "persistent kernel does not fit on the device");
  if (b->use_graph && !b->active.empty()) {
    cudaGraph_t g = nullptr;
    const long long n0 = f3d_kernel_launches();
    BK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    const int rc = enqueue_step(b, 0);
    const cudaError_t e = cudaStreamEndCapture(b->stream, &g);
    b->graph_kernels = (int)(f3d_kernel_launches() - n0);
    count_launch(-b->graph_kernels);  // counted per replay instead
    if (rc) return rc;
    BK(e);
    const cudaError_t e2 = cudaGraphInstantiate(&b->exec, g, 0);
    cudaGraphDestroy(g);
    BK(e2);
  }
  b->graph_dirty = false;
  return F3D_OK;
}

void finish_slot(f3d_batch* b, int id, int state) {
  Scen& s = b->slot[id];
  // work enqueued later on the context's own stream (downloads, outputs,
  // budgets, f3d_run) waits for the batch's last step of this scenario
  if (cudaEventRecord(b->ev, b->stream) == cudaSuccess) cudaStreamWaitEvent(s.x->stream, b->ev, 0);
  s.state = state;
  b->active.erase(std::find(b->active.begin(), b->active.end(), id));
  b->tables_dirty = b->graph_dirty = true;
}

}  // namespace

extern "C" {

int f3d_batch_create(int max_scenarios, f3d_batch** out) {
  if (!out) return ctx_error(F3D_ERR_ARG, "NULL argument");
  *out = nullptr;
  if (max_scenarios < 1 || max_scenarios > F3D_BATCH_MAX)
    return ctx_error(F3D_ERR_ARG, "max_scenarios outside 1..F3D_BATCH_MAX");
  f3d_batch* b = new f3d_batch();
  b->cap = max_scenarios;
  b->slot.resize(max_scenarios);
  const int n = max_scenarios;
  bool ok = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) == cudaSuccess;
  ok = ok && cudaEventCreateWithFlags(&b->ev, cudaEventDisableTiming) == cudaSuccess;
  ok = ok && cudaStreamCreateWithFlags(&b->fork.s2, cudaStreamNonBlocking) == cudaSuccess;
  ok = ok && cudaEventCreateWithFlags(&b->fork.a, cudaEventDisableTiming) == cudaSuccess;
  ok = ok && cudaEventCreateWithFlags(&b->fork.b, cudaEventDisableTiming) == cudaSuccess;
  ok = ok && cudaMalloc(&b->d_aux, sizeof(BatchAux) * n) == cudaSuccess;
  ok = ok && cudaMalloc(&b->d_item_off, sizeof(int) * (n + 1)) == cudaSuccess;
  ok = ok && cudaMalloc(&b->d_bstep, sizeof(int) * n) == cudaSuccess;
  ok = ok && cudaMalloc(&b->d_iiter0, sizeof(int) * n) == cudaSuccess;
  ok = ok && cudaMalloc(&b->d_counter, 2 * sizeof(int)) == cudaSuccess;
  ok = ok && cudaMalloc(&b->d_red, cmass2d_batch_scratch_bytes(n)) == cudaSuccess;
  ok = ok && cudaMallocHost(&b->h_aux, sizeof(BatchAux) * n) == cudaSuccess;
  ok = ok && cudaMallocHost(&b->h_args, sizeof(FusedArgs) * n) == cudaSuccess;
  ok = ok && cudaMallocHost(&b->h_maps, sizeof(F2Maps) * n) == cudaSuccess;
  ok = ok && cudaMalloc(&b->d_maps, sizeof(F2Maps) * n) == cudaSuccess;
  ok = ok && cudaMallocHost(&b->h_item_off, sizeof(int) * (n + 1)) == cudaSuccess;
  ok = ok && cudaMallocHost(&b->h_bstep, sizeof(int) * n) == cudaSuccess;
  ok = ok && cudaMallocHost(&b->h_iiter0, sizeof(int) * n) == cudaSuccess;
  if (!ok) {
    cudaGetLastError();
    f3d_batch_destroy(b);
    return ctx_error(F3D_ERR_OOM, "batch allocation failed");
  }
  *out = b;
  return F3D_OK;
}

int f3d_batch_destroy(f3d_batch* b) {
  if (!b) return F3D_OK;
  if (b->stream) cudaStreamSynchronize(b->stream);
  if (b->exec) cudaGraphExecDestroy(b->exec);
  cudaFree(b->d_aux);
  cudaFree(b->d_item_off);
  cudaFree(b->d_bstep);
  cudaFree(b->d_iiter0);
  cudaFree(b->d_counter);
  cudaFree(b->d_red);
  cudaFreeHost(b->h_aux);
  cudaFreeHost(b->h_args);
  cudaFreeHost(b->h_maps);
  cudaFree(b->d_maps);
  cudaFreeHost(b->h_item_off);
  cudaFreeHost(b->h_bstep);
  cudaFreeHost(b->h_iiter0);
  if (b->fork.s2) cudaStreamSynchronize(b->fork.s2);
  if (b->ev) cudaEventDestroy(b->ev);
  if (b->fork.a) cudaEventDestroy(b->fork.a);
  if (b->fork.b) cudaEventDestroy(b->fork.b);
  if (b->fork.s2) cudaStreamDestroy(b->fork.s2);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return F3D_OK;
}

int f3d_batch_add(f3d_batch* b, f3d_ctx* x, const f3d_met_series* met, const f3d_src_series* src,
                  double beg_time, double end_time, int max_steps, f3d_log_record* log, int log_cap,
                  int* slot) {
  if (!b || !x || !met || !src || !slot) return ctx_error(F3D_ERR_ARG, "NULL argument");
  if (x->prec != F3D_PREC_FP32 || !x->fused_ok)
    return ctx_error(F3D_ERR_ARG, "batched contexts must be precision-form (FP32) contexts of the fused step");
  if (x->gc_on) return ctx_error(F3D_ERR_ARG, "the gravity current is not supported in a batch");
  if (x->agr_on) return ctx_error(F3D_ERR_ARG, "aggregation is not supported in a batch");
  ctx_prefetch_drop(x);  // the batch makes each update when it is due
  if (met->nt < 1) return ctx_error(F3D_ERR_ARG, "no meteorological snapshot");
  int id = -1;
  for (int q = 0; q < b->cap; ++q) {
    if (b->slot[q].x == x && b->slot[q].state == 1) return ctx_error(F3D_ERR_STATE, "context already in the batch");
    if (id < 0 && b->slot[q].state == 0) id = q;
  }
  if (id < 0) return ctx_error(F3D_ERR_RANGE, "batch is full");
  BK(cudaStreamSynchronize(x->stream));
  Scen& s = b->slot[id];
  s = Scen{};
  s.x = x;
  s.met = met;
  s.src = src;
  s.end = end_time;
  s.max_steps = max_steps;
  s.log = log;
  s.log_cap = log_cap;
  // Fall3d.f90:73-78
  x->time = beg_time;
  x->meteo_time = beg_time;
  x->source_time = beg_time;
  x->iiter = 0;
  x->meteotime = 1;
  x->sourcetime = 1;
  x->run_started = 1;
  s.iiter0 = 0;
  s.c_a = x->c32;
  s.c_b = x->c32b;
  s.state = 1;
  b->active.push_back(id);
  b->tables_dirty = b->graph_dirty = true;
  *slot = id;
  return F3D_OK;
}

int f3d_batch_step(f3d_batch* b, int* n_running) {
  if (!b) return ctx_error(F3D_ERR_ARG, "NULL batch");
  // host side of every running scenario's time loop up to its step
  bool synced = false;
  for (size_t q = 0; q < b->active.size();) {
    const int id = b->active[q];
    Scen& s = b->slot[id];
    f3d_ctx* x = s.x;
    if (x->source_time <= x->time || x->meteo_time <= x->time) {  // an update is due
      if (!synced) {  // the coefficients and sources are read by the step in flight
        BK(cudaStreamSynchronize(b->stream));
        synced = true;
      }
      int rc = ctx_run_prepare(x, s.met, s.src, s.end);
      if (!rc && cudaStreamSynchronize(x->stream) != cudaSuccess)
        rc = ctx_error(F3D_ERR_CUDA, "meteo/source update failed");
      if (rc) {
        s.status = rc;
        s.error = "scenario failed in its source or meteo update";
        finish_slot(b, id, 3);
        continue;
      }
      b->tables_dirty = true;  // dt, the wet rate or the sources changed
    }
    ctx_advance(x);
    ++q;
  }
  if (b->active.empty()) {
    if (n_running) *n_running = 0;
    return F3D_OK;
  }
  if (b->tables_dirty) {
    if (int rc = table_rebuild(b)) return rc;
  }
  if (b->graph_dirty) {
    if (int rc = graph_rebuild(b)) return rc;
  }
  if (b->exec) {
    BK(cudaGraphLaunch(b->exec, b->stream));
    count_launch(b->graph_kernels);
  } else {
    if (int rc = enqueue_step(b, 0)) return rc;
  }
  ++b->batch_steps;
  // the step's host bookkeeping: buffers swap, logs, finished scenarios
  synced = false;
  std::vector<int> done;
  for (int id : b->active) {
    Scen& s = b->slot[id];
    f3d_ctx* x = s.x;
    b->cell_class_steps += (double)x->d.cells() * x->g.nc;
    ++s.bstep;
    ++s.steps;
    std::swap(x->c32, x->c32b);
    if (x->iiter == 1 || std::fmod(x->time, 600.0) <= x->dt) {  // endstep.f90:51
      if (s.log && s.nlog < s.log_cap) {
        if (!synced) {
          BK(cudaStreamSynchronize(b->stream));
          synced = true;
        }
        if (int rc = ctx_log(x, s.log, s.log_cap, &s.nlog)) return rc;
      }
    }
    if (x->time >= s.end || (s.max_steps > 0 && s.steps >= s.max_steps)) done.push_back(id);
  }
  for (int id : done) finish_slot(b, id, 2);
  if (n_running) *n_running = (int)b->active.size();
  return F3D_OK;
}

int f3d_batch_poll(f3d_batch* b, int slot, int* state, int* steps, int* nlog) {
  if (!b || slot < 0 || slot >= b->cap) return ctx_error(F3D_ERR_ARG, "invalid batch slot");
  const Scen& s = b->slot[slot];
  if (state) *state = s.state;
  if (steps) *steps = s.steps;
  if (nlog) *nlog = s.nlog;
  if (s.state == 3) return ctx_error(s.status ? s.status : F3D_ERR_STATE, s.error.c_str());
  return F3D_OK;
}

int f3d_batch_release(f3d_batch* b, int slot) {
  if (!b || slot < 0 || slot >= b->cap) return ctx_error(F3D_ERR_ARG, "invalid batch slot");
  Scen& s = b->slot[slot];
  if (s.state == 1) finish_slot(b, slot, 2);
  BK(cudaStreamSynchronize(b->stream));
  s = Scen{};
  return F3D_OK;
}

int f3d_batch_sync(f3d_batch* b) {
  if (!b) return ctx_error(F3D_ERR_ARG, "NULL batch");
  BK(cudaStreamSynchronize(b->stream));
  return F3D_OK;
}

int f3d_batch_set_option(f3d_batch* b, int key, int value) {
  if (!b) return ctx_error(F3D_ERR_ARG, "NULL batch");
  if (key == F3D_OPT_TILE) {
    if (value < 0 || value > 3) return ctx_error(F3D_ERR_ARG, "tile shape outside 0..3");
    b->shape = value;
  } else if (key == F3D_OPT_GRAPH) {
    b->use_graph = value ? 1 : 0;
  } else {
    return ctx_error(F3D_ERR_ARG, "unknown batch option");
  }
  b->tables_dirty = b->graph_dirty = true;
  return F3D_OK;
}

int f3d_batch_get_option(const f3d_batch* b, int key, int* value) {
  if (!b || !value) return ctx_error(F3D_ERR_ARG, "NULL argument");
  if (key == F3D_OPT_TILE) *value = b->shape;
  else if (key == F3D_OPT_GRAPH) *value = b->use_graph;
  else return ctx_error(F3D_ERR_ARG, "unknown batch option");
  return F3D_OK;
}

// Times the persistent step kernel of the running scenarios for every tile
// shape (deposit writes off, so the state does not change: the kernel reads
// one buffer and writes the other, which the next real step overwrites) and
// keeps the fastest.
int f3d_batch_autotune(f3d_batch* b, int reps, int* best, float* ms) {
  if (!b) return ctx_error(F3D_ERR_ARG, "NULL batch");
  if (b->active.empty()) return ctx_error(F3D_ERR_STATE, "no running scenario to tune on");
  for (int q : b->active)
    if (!b->slot[q].x->have_met) return ctx_error(F3D_ERR_STATE, "autotune before the first batch step");
  if (reps < 1) reps = 3;
  cudaEvent_t e0, e1;
  BK(cudaEventCreate(&e0));
  BK(cudaEventCreate(&e1));
  float bestms = 1e30f;
  int bestshape = b->shape;
  for (int shape = 0; shape < 4; ++shape) {
    b->shape = shape;
    if (int rc = table_rebuild(b)) return rc;

    b->grid = fused_batch_grid(shape, std::max(b->max_nz, 3));
    if (b->grid < 1) {
      if (ms) ms[shape] = -1.0f;
      continue;
    }
    enqueue_step(b, 1);  // warm-up
    BK(cudaEventRecord(e0, b->stream));
    for (int r = 0; r < reps; ++r) enqueue_step(b, 1);
    BK(cudaEventRecord(e1, b->stream));
    BK(cudaEventSynchronize(e1));
    float t = 0.0f;
    BK(cudaEventElapsedTime(&t, e0, e1));
    t /= (float)reps;
    if (ms) ms[shape] = t;
    if (t < bestms) {
      bestms = t;
      bestshape = shape;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  b->shape = bestshape;
  b->tables_dirty = b->graph_dirty = true;
  if (best) *best = bestshape;
  return F3D_OK;
}

int f3d_batch_stats(const f3d_batch* b, long long* batch_steps, double* cell_class_steps, int* n_running) {
  if (!b) return ctx_error(F3D_ERR_ARG, "NULL batch");
  if (batch_steps) *batch_steps = b->batch_steps;
  if (cell_class_steps) *cell_class_steps = b->cell_class_steps;
  if (n_running) *n_running = (int)b->active.size();
  return F3D_OK;
}

int f3d_batch_stream(const f3d_batch* b, void** stream) {
  if (!b || !stream) return ctx_error(F3D_ERR_ARG, "NULL argument");
  *stream = (void*)b->stream;
  return F3D_OK;
}

}  // extern "C"
