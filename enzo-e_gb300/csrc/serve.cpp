// serve.cpp -- continuous batching of independent VL+CT solves.
//
// Each request is a periodic box of n^3 cells advanced `cycles` VL+CT cycles
// in FP32 with its own Riemann solver / reconstruction.  Requests queue on
// submit; the scheduler admits them (first fit, in arrival order) whenever
// the device-memory budget and the active-slot limit allow.  Admission
// enqueues the whole request on a private stream: the upload of its initial
// state from a pinned staging buffer, the ghost refresh, every cycle, and the
// download of its final state back into the same staging buffer, so the work
// of every active request overlaps on the device and the host never waits
// for it.  The request's device memory comes from the server's stream-ordered
// memory pool and is freed in stream order too, so neither admission nor
// retirement waits for other requests' work (a cudaMalloc / cudaFree or a
// device synchronisation would).  Completion is detected by polling an
// event; the host then copies the active cells out of the staging buffer.
// Each request's dt comes from its own CFL reduction in a private device
// slot, so a result does not depend on what else is running.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <deque>
#include <string>
#include <vector>

#include "capi_internal.h"

namespace {

double now_s() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

enum { Q_QUEUED = 0, Q_RUNNING = 1, Q_DONE = 2, Q_FAILED = 3 };

// A pinned host staging buffer, reused by later requests once free.
struct Pinned {
  char* p = nullptr;
  size_t bytes = 0;
  bool busy = false;
};

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
  int pin = -1;  // staging buffer (index into the server's list)
  void* d_out = nullptr;  // the packed final state and its non-finite count
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

// Staging layout of a request: the uploaded fields back to back (cells of
// m^3, faces of (m+1) m^2, 256-byte aligned), reused for the downloaded cell
// fields, and the simulated time in the last 8 bytes.
size_t stage_offset(int k, size_t M, size_t F) {
  size_t o = 0;
  for (int j = 0; j < k; j++) o += ((j < 8 ? M : F) * sizeof(float) + 255) & ~(size_t)255;
  return o;
}
size_t stage_bytes(int nf, size_t M, size_t F) { return stage_offset(nf, M, F) + 256; }

// The active cells of the final cell fields packed densely (field after
// field, x fastest) and the number of non-finite values among them, so that
// completion is one contiguous copy and no host pass over the state.
struct PackSrc {
  const float* f[8];
};
__global__ void pack_active_kernel(PackSrc src, int nf, int n, int g, float* out,
                                   unsigned* bad) {
  const size_t m = (size_t)n + 2 * g, nn = (size_t)n * n, cells = nn * n;
  unsigned local = 0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < cells * nf;
       i += (size_t)gridDim.x * blockDim.x) {
    const int k = (int)(i / cells);
    const size_t c = i - (size_t)k * cells;
    const size_t z = c / nn, y = (c / n) % n, x = c % n;
    const float v = src.f[k][((z + g) * m + (y + g)) * m + (x + g)];
    out[i] = v;
    local += isfinite(v) ? 0u : 1u;
  }
  if (local) atomicAdd(bad, local);
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
  std::vector<Pinned> pinned;
  cudaMemPool_t pool = nullptr;  // device memory of every request
  std::string err;
};

namespace {

int sfail(mhdserve* s, int code, const std::string& m) {
  s->err = m;
  return code;
}

void release(mhdserve* s, Req* r) {
  // the batch frees its memory on the request's stream, after its work
  if (r->d_out) cudaFreeAsync(r->d_out, r->st);
  r->d_out = nullptr;
  if (r->b) mhdvlct_batch_destroy(r->b);
  if (r->h) mhdvlct_destroy(r->h);
  if (r->done) cudaEventDestroy(r->done);
  if (r->st) cudaStreamDestroy(r->st);  // returns at once; the frees still run
  r->b = nullptr;
  r->h = nullptr;
  r->done = nullptr;
  r->st = nullptr;
  if (r->pin >= 0) s->pinned[r->pin].busy = false;
  r->pin = -1;
  s->in_use -= std::min(s->in_use, r->bytes);
  for (auto& v : r->init) std::vector<float>().swap(v);
}

void fail_req(mhdserve* s, Req* r, const std::string& m) {
  r->err = m;
  r->state = Q_FAILED;
  r->t_done = now_s();
  // a request that fails after its work was queued must not hand its staging
  // buffer on before that work is over
  if (r->st) cudaStreamSynchronize(r->st);
  release(s, r);
}

// A free staging buffer of at least `bytes` (the smallest that fits), or a
// new one; -1 if pinned memory cannot be had.
int take_pinned(mhdserve* s, size_t bytes) {
  int best = -1;
  for (int i = 0; i < (int)s->pinned.size(); i++) {
    const Pinned& p = s->pinned[i];
    if (!p.busy && p.bytes >= bytes && (best < 0 || p.bytes < s->pinned[best].bytes)) best = i;
  }
  if (best < 0) {
    Pinned p;
    if (cudaHostAlloc((void**)&p.p, bytes, cudaHostAllocDefault) != cudaSuccess) return -1;
    p.bytes = bytes;
    s->pinned.push_back(p);
    best = (int)s->pinned.size() - 1;
  }
  s->pinned[best].busy = true;
  return best;
}

// Admit one request: allocate, then enqueue upload, refresh, every cycle and
// the download of the final state on the request's stream.
bool start(mhdserve* s, Req* r) {
  int rc = mhdvlct_create(&r->params, &r->h);
  if (rc != MHD_OK) {
    fail_req(s, r, std::string("create: ") + (r->h ? mhdvlct_last_error_string(r->h) : ""));
    return false;
  }
  s->in_use += r->bytes;
  if (cudaStreamCreateWithFlags(&r->st, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&r->done, cudaEventDisableTiming) != cudaSuccess) {
    fail_req(s, r, "stream/event creation");
    return false;
  }
  const int dims[3] = {r->n, r->n, r->n};
  const double w = r->box / r->n;
  const double widths[3] = {w, w, w};
  rc = mhdint::batch_create(r->h, dims, widths, 1, 3, MHD_DTYPE_F32, 0, 0, r->st, s->pool,
                            &r->b);
  if (rc != MHD_OK) {
    fail_req(s, r, std::string("batch: ") + mhdvlct_last_error_string(r->h));
    return false;
  }
  const int g = 3;
  const size_t m = (size_t)r->n + 2 * g;
  const size_t M = m * m * m, F = (m + 1) * m * m;
  const int nf = r->mhd ? 11 : 5;
  r->pin = take_pinned(s, stage_bytes(nf, M, F));
  if (r->pin < 0) {
    fail_req(s, r, "pinned staging buffer");
    return false;
  }
  char* stage = s->pinned[r->pin].p;
  MhdBlockView v;
  mhdvlct_batch_block_view(r->b, 0, &v);
  void* dst[11] = {v.density, v.velocity[0], v.velocity[1], v.velocity[2],
                   v.total_energy, v.bfield[0], v.bfield[1], v.bfield[2],
                   v.bfieldi[0], v.bfieldi[1], v.bfieldi[2]};
  for (int k = 0; k < nf; k++) {
    char* h = stage + stage_offset(k, M, F);
    std::memcpy(h, r->init[k].data(), r->init[k].size() * sizeof(float));
    if (cudaMemcpyAsync(dst[k], h, r->init[k].size() * sizeof(float),
                        cudaMemcpyHostToDevice, r->st) != cudaSuccess) {
      fail_req(s, r, "upload");
      return false;
    }
  }
  for (auto& x : r->init) std::vector<float>().swap(x);
  if (mhdvlct_batch_refresh(r->b, r->st) != MHD_OK ||
      mhdvlct_batch_run(r->b, r->cycles, 1, nullptr, r->st) != MHD_OK) {
    fail_req(s, r, std::string("launch: ") + mhdvlct_last_error_string(r->h));
    return false;
  }
  // the final cell fields (the same arrays whatever the face-buffer parity)
  // packed on the device with their non-finite count, then one copy of that
  // and one of the simulated time into the staging buffer
  const int nd = r->mhd ? 8 : 5;
  const size_t active = (size_t)r->n * r->n * r->n;
  const size_t out_bytes = nd * active * sizeof(float);
  PackSrc ps{};
  const void* src[8] = {v.density, v.velocity[0], v.velocity[1], v.velocity[2],
                        v.total_energy, v.bfield[0], v.bfield[1], v.bfield[2]};
  for (int k = 0; k < nd; k++) ps.f[k] = (const float*)src[k];
  bool ok = cudaMallocFromPoolAsync(&r->d_out, out_bytes + 256, s->pool, r->st) == cudaSuccess;
  unsigned* d_bad = ok ? (unsigned*)((char*)r->d_out + out_bytes) : nullptr;
  if (ok) ok = cudaMemsetAsync(d_bad, 0, sizeof(unsigned), r->st) == cudaSuccess;
  if (ok) {
    const int grid = (int)std::min<size_t>((nd * active + 255) / 256, 4096);
    pack_active_kernel<<<grid, 256, 0, r->st>>>(ps, nd, r->n, g, (float*)r->d_out, d_bad);
    ok = cudaGetLastError() == cudaSuccess;
  }
  if (ok)
    ok = cudaMemcpyAsync(stage, r->d_out, out_bytes + sizeof(unsigned), cudaMemcpyDeviceToHost,
                         r->st) == cudaSuccess &&
         cudaMemcpyAsync(stage + stage_offset(nf, M, F), mhdint::batch_time_device(r->b),
                         sizeof(double), cudaMemcpyDeviceToHost, r->st) == cudaSuccess &&
         cudaEventRecord(r->done, r->st) == cudaSuccess;
  if (!ok) {
    fail_req(s, r, "download");
    return false;
  }
  r->state = Q_RUNNING;
  r->t_admit = now_s();
  return true;
}

// A request whose event has completed: its packed final state, the count of
// non-finite values in it and its simulated time are in the staging buffer.
void finish(mhdserve* s, Req* r) {
  const int g = 3, n = r->n;
  const size_t m = (size_t)n + 2 * g;
  const size_t M = m * m * m, F = (m + 1) * m * m;
  const int nf = r->mhd ? 11 : 5, nd = r->mhd ? 8 : 5;
  const size_t active = (size_t)n * n * n;
  const char* stage = s->pinned[r->pin].p;
  std::memcpy(&r->sim_time, stage + stage_offset(nf, M, F), sizeof(double));
  unsigned bad = 0;
  std::memcpy(&bad, stage + nd * active * sizeof(float), sizeof(unsigned));
  r->t_done = now_s();
  if (bad) {
    fail_req(s, r, "non-finite state");
    return;
  }
  for (int k = 0; k < nd; k++) {
    const float* f = (const float*)stage + k * active;
    r->result[k].assign(f, f + active);
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
  // the requests' device memory: a pool of the current device that keeps
  // what the finished requests freed (up to the budget) for the next ones
  int dev = 0;
  cudaMemPoolProps props = {};
  props.allocType = cudaMemAllocationTypePinned;
  props.location.type = cudaMemLocationTypeDevice;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      (props.location.id = dev, cudaMemPoolCreate(&s->pool, &props)) != cudaSuccess) {
    delete s;
    return MHD_ERR_CUDA;
  }
  uint64_t keep = budget;
  cudaMemPoolSetAttribute(s->pool, cudaMemPoolAttrReleaseThreshold, &keep);
  // reserve the budget now: one allocation of it, freed back into the pool,
  // so that admissions never wait for the pool to map new memory
  void* p = nullptr;
  if (cudaMallocFromPoolAsync(&p, budget, s->pool, 0) == cudaSuccess) {
    cudaFreeAsync(p, 0);
    cudaStreamSynchronize(0);
  } else {
    cudaGetLastError();  // a budget beyond free memory: the pool grows on demand
  }
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
  // every request's stream-ordered frees must have run before the pool goes
  cudaDeviceSynchronize();
  if (s->pool) cudaMemPoolDestroy(s->pool);
  for (Pinned& p : s->pinned) cudaFreeHost(p.p);
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
