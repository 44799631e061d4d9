// serve.cpp -- continuous batching of independent VL+CT solves.
//
// Each request is a periodic box of n^3 cells advanced `cycles` VL+CT cycles
// in FP32 with its own Riemann solver / reconstruction.  Requests queue on
// submit; the scheduler admits them (first fit, in arrival order) whenever
// the device-memory budget and the active-slot limit allow, uploads their
// state once, and enqueues all their cycles on a private stream, so the work
// of every active request overlaps on the device.  Completion is detected by
// polling an event; the final state is copied to a host buffer, the request's
// device memory is released and waiting requests are admitted into the freed
// room.  Each request's dt comes from its own CFL reduction in a private
// device slot, so a result does not depend on what else is running.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <deque>
#include <string>
#include <vector>

#include "../../include/mhdvlct_gb300.h"

namespace {

double now_s() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

enum { Q_QUEUED = 0, Q_RUNNING = 1, Q_DONE = 2, Q_FAILED = 3 };

struct Req {
  int ticket = 0;
  int n = 0, cycles = 0, mhd = 1;
  MhdVlctParams params;
  double box = 1.0;
  std::vector<float> init[12];
  int state = Q_QUEUED;
  mhdvlct_handle* h = nullptr;
  mhdvlct_batch* b = nullptr;
  cudaStream_t st = nullptr;
  cudaEvent_t done = nullptr;
  size_t bytes = 0;
  double t_submit = 0, t_admit = 0, t_done = 0, sim_time = 0;
  std::vector<float> result[8];
  std::string err;
};

// Device bytes a request will hold (the batch pool of one n^3 block, see
// mhdvlct_batch_create) plus a small allowance for descriptors.
size_t request_bytes(int n, int g, int mhd, int de) {
  const size_t m = (size_t)n + 2 * g;
  const size_t M = m * m * m, F = (m + 1) * m * m;
  const size_t cells = 5 + (mhd ? 3 : 0) + (de ? 1 : 0);
  return 4 * (2 * cells * M + (mhd ? 9 * F : 0) + M) + (1 << 20);
}

}  // namespace

struct mhdserve {
  MhdVlctParams base;
  size_t budget = 0;
  int max_active = 0;
  size_t in_use = 0;
  std::vector<Req*> reqs;
  std::deque<int> queue;
  std::vector<int> active;
  std::string err;
};

namespace {

int sfail(mhdserve* s, int code, const std::string& m) {
  s->err = m;
  return code;
}

void release(mhdserve* s, Req* r) {
  if (r->b) mhdvlct_batch_destroy(r->b);
  if (r->h) mhdvlct_destroy(r->h);
  if (r->done) cudaEventDestroy(r->done);
  if (r->st) cudaStreamDestroy(r->st);
  r->b = nullptr;
  r->h = nullptr;
  r->done = nullptr;
  r->st = nullptr;
  s->in_use -= std::min(s->in_use, r->bytes);
  for (auto& v : r->init) std::vector<float>().swap(v);
}

void fail_req(mhdserve* s, Req* r, const std::string& m) {
  r->err = m;
  r->state = Q_FAILED;
  r->t_done = now_s();
  release(s, r);
}

// Admit one request: allocate, upload, refresh ghosts, enqueue every cycle.
bool start(mhdserve* s, Req* r) {
  int rc = mhdvlct_create(&r->params, &r->h);
  if (rc != MHD_OK) {
    fail_req(s, r, std::string("create: ") + (r->h ? mhdvlct_last_error_string(r->h) : ""));
    return false;
  }
  const int dims[3] = {r->n, r->n, r->n};
  const double w = r->box / r->n;
  const double widths[3] = {w, w, w};
  s->in_use += r->bytes;
  rc = mhdvlct_batch_create(r->h, dims, widths, 1, 3, MHD_DTYPE_F32, &r->b);
  if (rc != MHD_OK) {
    fail_req(s, r, std::string("batch: ") + mhdvlct_last_error_string(r->h));
    return false;
  }
  if (cudaStreamCreateWithFlags(&r->st, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&r->done, cudaEventDisableTiming) != cudaSuccess) {
    fail_req(s, r, "stream/event creation");
    return false;
  }
  MhdBlockView v;
  mhdvlct_batch_block_view(r->b, 0, &v);
  void* dst[12] = {v.density, v.velocity[0], v.velocity[1], v.velocity[2],
                   v.total_energy, v.bfield[0], v.bfield[1], v.bfield[2],
                   v.bfieldi[0], v.bfieldi[1], v.bfieldi[2], nullptr};
  const int nf = r->mhd ? 11 : 5;
  for (int k = 0; k < nf; k++) {
    if (r->init[k].empty()) continue;
    if (cudaMemcpyAsync(dst[k], r->init[k].data(), r->init[k].size() * sizeof(float),
                        cudaMemcpyHostToDevice, r->st) != cudaSuccess) {
      fail_req(s, r, "upload");
      return false;
    }
  }
  // the host copy must stay alive until the copies have run
  cudaStreamSynchronize(r->st);
  for (auto& x : r->init) std::vector<float>().swap(x);
  if (mhdvlct_batch_refresh(r->b, r->st) != MHD_OK ||
      mhdvlct_batch_run(r->b, r->cycles, 1, nullptr, r->st) != MHD_OK ||
      cudaEventRecord(r->done, r->st) != cudaSuccess) {
    fail_req(s, r, std::string("launch: ") + mhdvlct_last_error_string(r->h));
    return false;
  }
  r->state = Q_RUNNING;
  r->t_admit = now_s();
  return true;
}

void finish(mhdserve* s, Req* r) {
  MhdBlockView v;
  mhdvlct_batch_block_view(r->b, 0, &v);
  double t = 0;
  mhdvlct_batch_run(r->b, 0, 1, &t, r->st);
  r->sim_time = t;
  const int g = 3, n = r->n, m = n + 2 * g;
  void* src[8] = {v.density, v.velocity[0], v.velocity[1], v.velocity[2],
                  v.total_energy, v.bfield[0], v.bfield[1], v.bfield[2]};
  const int nf = r->mhd ? 8 : 5;
  std::vector<float> full((size_t)m * m * m);
  bool finite = true;
  for (int k = 0; k < nf; k++) {
    if (cudaMemcpy(full.data(), src[k], full.size() * sizeof(float),
                   cudaMemcpyDeviceToHost) != cudaSuccess) {
      fail_req(s, r, "download");
      return;
    }
    r->result[k].resize((size_t)n * n * n);
    for (int z = 0; z < n; z++)
      for (int y = 0; y < n; y++)
        for (int x = 0; x < n; x++) {
          const float val = full[((size_t)(z + g) * m + (y + g)) * m + (x + g)];
          finite = finite && std::isfinite(val);
          r->result[k][((size_t)z * n + y) * n + x] = val;
        }
  }
  r->t_done = now_s();
  if (!finite) {
    fail_req(s, r, "non-finite state");
    return;
  }
  r->state = Q_DONE;
  release(s, r);
}

}  // namespace

extern "C" int mhdserve_create(const MhdVlctParams* base, size_t budget,
                               int max_active, mhdserve** out) {
  if (!base || !out || budget == 0 || max_active <= 0) return MHD_ERR_INVALID;
  mhdserve* s = new mhdserve();
  s->base = *base;
  s->budget = budget;
  s->max_active = max_active;
  *out = s;
  return MHD_OK;
}

extern "C" int mhdserve_destroy(mhdserve* s) {
  if (!s) return MHD_ERR_INVALID;
  for (Req* r : s->reqs) {
    if (r->st) cudaStreamSynchronize(r->st);
    release(s, r);
    delete r;
  }
  delete s;
  return MHD_OK;
}

extern "C" int mhdserve_submit(mhdserve* s, const MhdServeRequest* q, int* ticket) {
  if (!s || !q || !ticket) return MHD_ERR_INVALID;
  if (q->n < 4 || q->n > 1024 || q->cycles < 0 || !(q->box_size > 0))
    return sfail(s, MHD_ERR_INVALID, "malformed request");
  Req* r = new Req();
  r->n = q->n;
  r->cycles = q->cycles;
  r->mhd = q->mhd ? 1 : 0;
  r->box = q->box_size;
  r->params = s->base;
  std::snprintf(r->params.mhd_choice, sizeof(r->params.mhd_choice), "%s",
                r->mhd ? "constrained_transport" : "no_bfield");
  std::snprintf(r->params.riemann_solver, sizeof(r->params.riemann_solver), "%.15s",
                q->riemann_solver);
  std::snprintf(r->params.reconstruct_method, sizeof(r->params.reconstruct_method),
                "%.15s", q->reconstruct_method);
  // validate the options now (a handle is cheap: no device memory)
  mhdvlct_handle* probe = nullptr;
  int rc = mhdvlct_create(&r->params, &probe);
  if (rc != MHD_OK) {
    std::string m = probe ? mhdvlct_last_error_string(probe) : "bad parameters";
    if (probe) mhdvlct_destroy(probe);
    delete r;
    return sfail(s, MHD_ERR_INVALID, m);
  }
  mhdvlct_destroy(probe);
  r->bytes = request_bytes(r->n, 3, r->mhd, r->params.dual_energy);
  if (r->bytes > s->budget) {
    delete r;
    return sfail(s, MHD_ERR_NOMEM, "request can never fit in the memory budget");
  }
  const size_t m = (size_t)r->n + 6;
  const size_t M = m * m * m, F = (m + 1) * m * m;
  const int nf = r->mhd ? 11 : 5;
  for (int k = 0; k < nf; k++) {
    if (!q->init[k]) {
      delete r;
      return sfail(s, MHD_ERR_INVALID, "missing initial field");
    }
    const size_t cnt = k < 8 ? M : F;
    r->init[k].assign(q->init[k], q->init[k] + cnt);
  }
  r->ticket = (int)s->reqs.size();
  r->t_submit = now_s();
  s->reqs.push_back(r);
  s->queue.push_back(r->ticket);
  *ticket = r->ticket;
  return MHD_OK;
}

extern "C" int mhdserve_pump(mhdserve* s, int max_iterations) {
  if (!s) return MHD_ERR_INVALID;
  for (int it = 0; it < max_iterations; it++) {
    // retire finished requests
    for (size_t i = 0; i < s->active.size();) {
      Req* r = s->reqs[s->active[i]];
      const cudaError_t q = cudaEventQuery(r->done);
      if (q == cudaErrorNotReady) {
        i++;
        continue;
      }
      if (q == cudaSuccess) finish(s, r);
      else fail_req(s, r, cudaGetErrorString(q));
      s->active.erase(s->active.begin() + i);
    }
    // admit queued requests that fit (first fit in arrival order)
    for (auto itq = s->queue.begin(); itq != s->queue.end();) {
      Req* r = s->reqs[*itq];
      if ((int)s->active.size() >= s->max_active) break;
      if (s->in_use + r->bytes > s->budget) {
        ++itq;
        continue;
      }
      const int t = *itq;
      itq = s->queue.erase(itq);
      if (start(s, r)) s->active.push_back(t);
    }
    if (s->active.empty() && s->queue.empty()) break;
  }
  return MHD_OK;
}

extern "C" int mhdserve_poll(mhdserve* s, int ticket, int* state) {
  if (!s || !state || ticket < 0 || ticket >= (int)s->reqs.size()) return MHD_ERR_INVALID;
  *state = s->reqs[ticket]->state;
  return MHD_OK;
}

extern "C" int mhdserve_result(mhdserve* s, int ticket, float* const* out,
                               double* sim_time_out) {
  if (!s || ticket < 0 || ticket >= (int)s->reqs.size()) return MHD_ERR_INVALID;
  Req* r = s->reqs[ticket];
  if (r->state == Q_FAILED) return sfail(s, MHD_ERR_NONFINITE, r->err);
  if (r->state != Q_DONE) return MHD_ERR_BUSY;
  if (out) {
    const int nf = r->mhd ? 8 : 5;
    for (int k = 0; k < nf; k++)
      if (out[k]) std::memcpy(out[k], r->result[k].data(), r->result[k].size() * sizeof(float));
  }
  if (sim_time_out) *sim_time_out = r->sim_time;
  return MHD_OK;
}

extern "C" int mhdserve_timing(mhdserve* s, int ticket, double* t_submit,
                               double* t_admit, double* t_done) {
  if (!s || ticket < 0 || ticket >= (int)s->reqs.size()) return MHD_ERR_INVALID;
  const Req* r = s->reqs[ticket];
  if (t_submit) *t_submit = r->t_submit;
  if (t_admit) *t_admit = r->t_admit;
  if (t_done) *t_done = r->t_done;
  return MHD_OK;
}

extern "C" const char* mhdserve_last_error_string(const mhdserve* s) {
  return s ? s->err.c_str() : "null server";
}
