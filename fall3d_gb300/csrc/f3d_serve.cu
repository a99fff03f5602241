// f3d_serve.cu -- the serving form: continuous batching of forecast requests.
//
// Requests (one scenario each) are submitted as they arrive and queue in
// arrival order.  Between batch steps the server admits queued requests
// while the device-memory footprint of the resident scenarios stays under
// the cap and a batch slot is free: it creates the request's precision-form
// context (state and met fields resident in HBM for the whole run) and joins
// it to the running batch, whose next step then advances it together with
// every other running request.  A request that finishes leaves the batch,
// its outputs (LOAD, COL_MASS, C_GRND of printres_nc.f90 and the mass-budget
// log) are copied to host memory, and its context is destroyed, which frees
// its footprint for the next admission.  Each request's results are those of
// running it alone (f3d_run on the same scenario): the batch never mixes the
// arithmetic of two scenarios.
#include <algorithm>
#include <chrono>
#include <cstring>
#include <deque>
#include <string>
#include <vector>

#include "f3d_ctx_impl.h"

using namespace f3d;

namespace {

double now_s() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

struct Request {
  f3d_grid grid{};
  const f3d_met_series* met = nullptr;
  const f3d_src_series* src = nullptr;
  double beg = 0.0, end = 0.0;
  int state = 0;  // 0 queued, 1 running, 2 done, 3 failed, 4 forgotten
  long long footprint = 0;
  f3d_ctx* ctx = nullptr;
  int slot = -1;
  double t_submit = 0.0, t_admit = 0.0, t_done = 0.0;
  std::vector<f3d_log_record> log;
  int nlog = 0;
  std::vector<double> load, col_mass, c_grnd;
  double cell_classes = 0.0;
  long long steps = 0;
  int status = 0;
  std::string error;
};

}  // namespace

struct f3d_server {
  f3d_batch* batch = nullptr;
  long long cap = 0, used = 0;
  int max_running = 0, running = 0;
  std::deque<int> queue;
  std::vector<Request> req;
  double cell_class_steps = 0.0;
  long long batch_steps = 0;
};

namespace {

int complete(f3d_server* v, int id) {
  Request& r = v->req[id];
  int st = 0, steps = 0, nlog = 0;
  const int prc = f3d_batch_poll(v->batch, r.slot, &st, &steps, &nlog);
  r.steps = steps;
  r.nlog = nlog;
  if (st == 2 && prc == F3D_OK) {
    const size_t pl = (size_t)r.grid.nx * r.grid.ny;
    r.load.resize(pl);
    r.col_mass.resize(pl);
    r.c_grnd.resize(pl);
    const int rc = f3d_outputs(r.ctx, r.load.data(), r.col_mass.data(), r.c_grnd.data());
    r.state = rc ? 3 : 2;
    if (rc) {
      r.status = rc;
      r.error = "output reduction failed";
    }
  } else {
    r.state = 3;
    r.status = prc ? prc : F3D_ERR_STATE;
    r.error = "request failed in its time loop";
  }
  r.t_done = now_s();
  f3d_batch_release(v->batch, r.slot);
  f3d_ctx_destroy(r.ctx);
  r.ctx = nullptr;
  r.slot = -1;
  v->used -= r.footprint;
  --v->running;
  return F3D_OK;
}

// Admits queued requests in arrival order while they fit.
int admit(f3d_server* v) {
  while (!v->queue.empty() && v->running < v->max_running) {
    const int id = v->queue.front();
    Request& r = v->req[id];
    if (v->used + r.footprint > v->cap) {
      if (v->running > 0) break;  // wait for memory to free up
      r.state = 3;                // larger than the whole cap: can never run
      r.status = F3D_ERR_OOM;
      r.error = "request footprint exceeds the admission cap";
      r.t_done = now_s();
      v->queue.pop_front();
      continue;
    }
    v->queue.pop_front();
    f3d_ctx* x = nullptr;
    int rc = f3d_ctx_create(&r.grid, &x);
    int slot = -1;
    if (!rc)
      rc = f3d_batch_add(v->batch, x, r.met, r.src, r.beg, r.end, 0, r.log.data(), (int)r.log.size(), &slot);
    if (rc) {
      if (x) f3d_ctx_destroy(x);
      r.state = 3;
      r.status = rc;
      r.error = "admission failed";
      r.t_done = now_s();
      continue;
    }
    r.ctx = x;
    r.slot = slot;
    r.state = 1;
    r.t_admit = now_s();
    v->used += r.footprint;
    ++v->running;
  }
  return F3D_OK;
}

}  // namespace

extern "C" {

int f3d_server_create(long long hbm_cap_bytes, int max_running, f3d_server** out) {
  if (!out) return ctx_error(F3D_ERR_ARG, "NULL argument");
  *out = nullptr;
  if (hbm_cap_bytes <= 0 || max_running < 1 || max_running > F3D_BATCH_MAX)
    return ctx_error(F3D_ERR_ARG, "invalid cap or max_running (1..F3D_BATCH_MAX)");
  f3d_server* v = new f3d_server();
  v->cap = hbm_cap_bytes;
  v->max_running = max_running;
  if (int rc = f3d_batch_create(max_running, &v->batch)) {
    delete v;
    return rc;
  }
  *out = v;
  return F3D_OK;
}

int f3d_server_destroy(f3d_server* v) {
  if (!v) return F3D_OK;
  for (Request& r : v->req) {
    if (r.ctx) {
      f3d_batch_release(v->batch, r.slot);
      f3d_ctx_destroy(r.ctx);
    }
  }
  f3d_batch_destroy(v->batch);
  delete v;
  return F3D_OK;
}

int f3d_server_submit(f3d_server* v, const f3d_grid* grid, const f3d_met_series* met,
                      const f3d_src_series* src, double beg_time, double end_time, int log_cap,
                      int* request_id) {
  if (!v || !grid || !met || !src || !request_id) return ctx_error(F3D_ERR_ARG, "NULL argument");
  Request r;
  r.grid = *grid;
  r.grid.precision = F3D_PREC_FP32;
  r.met = met;
  r.src = src;
  r.beg = beg_time;
  r.end = end_time;
  r.log.resize(log_cap > 0 ? log_cap : 1);
  if (int rc = f3d_ctx_footprint(&r.grid, &r.footprint)) return rc;
  r.cell_classes = (double)grid->nx * grid->ny * grid->nz * grid->nc;
  r.t_submit = now_s();
  v->req.push_back(std::move(r));
  const int id = (int)v->req.size() - 1;
  v->queue.push_back(id);
  *request_id = id;
  return F3D_OK;
}

// Admits what fits, runs up to max_steps batch steps (stopping early when a
// request completes, so that its memory is reused at once), and collects
// completed requests.
int f3d_server_progress(f3d_server* v, int max_steps, int* n_running, int* n_queued) {
  if (!v) return ctx_error(F3D_ERR_ARG, "NULL server");
  if (int rc = admit(v)) return rc;
  for (int k = 0; k < (max_steps > 0 ? max_steps : 1) && v->running > 0; ++k) {
    int n = 0;
    if (int rc = f3d_batch_step(v->batch, &n)) return rc;
    ++v->batch_steps;
    bool any_done = false;
    for (size_t id = 0; id < v->req.size(); ++id) {
      Request& r = v->req[id];
      if (r.state != 1) continue;
      int st = 0;
      f3d_batch_poll(v->batch, r.slot, &st, nullptr, nullptr);
      if (st == 1) {
        v->cell_class_steps += r.cell_classes;
        continue;
      }
      v->cell_class_steps += r.cell_classes;  // its last step
      complete(v, (int)id);
      any_done = true;
    }
    if (any_done) {
      admit(v);
      break;
    }
  }
  if (n_running) *n_running = v->running;
  if (n_queued) *n_queued = (int)v->queue.size();
  return F3D_OK;
}

// state: 0 queued, 1 running, 2 done, 3 failed; times in seconds of a
// monotonic clock (submit, admit, done).
int f3d_server_poll(f3d_server* v, int id, int* state, double* t_submit, double* t_admit,
                    double* t_done, long long* steps) {
  if (!v || id < 0 || id >= (int)v->req.size()) return ctx_error(F3D_ERR_ARG, "invalid request id");
  const Request& r = v->req[id];
  if (state) *state = r.state;
  if (t_submit) *t_submit = r.t_submit;
  if (t_admit) *t_admit = r.t_admit;
  if (t_done) *t_done = r.t_done;
  if (steps) *steps = r.steps;
  if (r.state == 3) return ctx_error(r.status ? r.status : F3D_ERR_STATE, r.error.c_str());
  return F3D_OK;
}

// Outputs of a completed request (nx*ny each; NULL to skip) and its log.
int f3d_server_result(f3d_server* v, int id, double* load, double* col_mass, double* c_grnd,
                      f3d_log_record* log, int log_cap, int* nlog) {
  if (!v || id < 0 || id >= (int)v->req.size()) return ctx_error(F3D_ERR_ARG, "invalid request id");
  const Request& r = v->req[id];
  if (r.state != 2) return ctx_error(F3D_ERR_STATE, "request has no result (not done, failed or forgotten)");
  const size_t pl = r.load.size();
  if (load) memcpy(load, r.load.data(), pl * sizeof(double));
  if (col_mass) memcpy(col_mass, r.col_mass.data(), pl * sizeof(double));
  if (c_grnd) memcpy(c_grnd, r.c_grnd.data(), pl * sizeof(double));
  const int n = std::min(r.nlog, log_cap);
  if (log && n > 0) memcpy(log, r.log.data(), sizeof(f3d_log_record) * (size_t)n);
  if (nlog) *nlog = r.nlog;
  return F3D_OK;
}

// Drops a completed request's host copies.
int f3d_server_forget(f3d_server* v, int id) {
  if (!v || id < 0 || id >= (int)v->req.size()) return ctx_error(F3D_ERR_ARG, "invalid request id");
  Request& r = v->req[id];
  if (r.state == 0 || r.state == 1) return ctx_error(F3D_ERR_STATE, "request still queued or running");
  r.load = std::vector<double>();
  r.col_mass = std::vector<double>();
  r.c_grnd = std::vector<double>();
  r.log = std::vector<f3d_log_record>();
  r.state = 4;
  return F3D_OK;
}

int f3d_server_stats(const f3d_server* v, long long* used_bytes, double* cell_class_steps,
                     long long* batch_steps, int* n_running, int* n_queued) {
  if (!v) return ctx_error(F3D_ERR_ARG, "NULL server");
  if (used_bytes) *used_bytes = v->used;
  if (cell_class_steps) *cell_class_steps = v->cell_class_steps;
  if (batch_steps) *batch_steps = v->batch_steps;
  if (n_running) *n_running = v->running;
  if (n_queued) *n_queued = (int)v->queue.size();
  return F3D_OK;
}

int f3d_server_batch(f3d_server* v, f3d_batch** batch) {
  if (!v || !batch) return ctx_error(F3D_ERR_ARG, "NULL argument");
  *batch = v->batch;
  return F3D_OK;
}

}  // extern "C"
