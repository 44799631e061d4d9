// batch.cu -- many blocks advanced together (the batched form).
//
// All blocks live in one library-owned device pool in Cello's per-field
// layout.  A cycle is: timestep (reference semantics: whole ghosted block,
// before the refresh), the global or per-block dt, the same-level ghost
// refresh, and the two VL stages, each ONE persistent launch over the tiles of
// every block (tiles sorted largest-first and pulled from a device work
// queue).  The face-centred B is double buffered: the last stage reads the
// start-of-step faces and writes the other buffer, so no stage updates a
// field in place that another CTA may still read.  The whole cycle is
// captured once as a CUDA graph per face-buffer parity and replayed.  The
// pool holds every block's cell fields, then face buffer A of every block,
// then buffer B, so the current state is at most two contiguous segments.
// Tiles, z-chunks and CTA sizes come from the autotuner per block-size class
// and stage (or a default that z-chunks a batch too small to fill the GPU).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "capi_internal.h"
#include "vlct_aux.cuh"
#include "vlct_stage.cuh"

using namespace vlct;
using namespace mhdint;

namespace {

__global__ void add_scalar_kernel(double* acc, const double* v) { *acc += *v; }

// Work decomposition of one block-size class, per stage (0: half dt, NN;
// 1: full dt, the configured reconstruction).
struct TileChoice {
  int tile_x[2] = {0, 0};  // x tile extent (0 = default)
  int tile_y[2] = {0, 0};  // y tile extent (0 = default)
  int zchunk[2] = {0, 0};  // z-chunk length (0 = whole block)
};

}  // namespace

struct mhdvlct_batch {
  mhdvlct_handle* h = nullptr;
  int dtype = MHD_DTYPE_F32;
  int nblocks = 0;
  int g = 3;
  int npass = 0;    // passive scalars of every block (0..4)
  int gravity = 0;  // 1: every block carries acceleration_x/y/z
  std::vector<int> dims;       // 3 per block (active)
  std::vector<double> widths;  // 3 per block
  void* pool = nullptr;
  size_t pool_bytes = 0;
  size_t state_elems = 0;  // leading part of the pool holding the state
  size_t cells_elems = 0;  // cell fields of every block: [0, cells_elems)
  size_t fa_end = 0;       // face buffer A of every block: [cells_elems, fa_end),
                           // buffer B: [fa_end, state_elems)
  // element offsets (in units of the real type) of every array of block i
  struct Off {
    size_t ext[NCELL], tmp[NCELL], fa[3], fb[3], tf[3], pres;
    size_t pas[4], ptmp[4], acc[3];  // passive scalars (state, half step),
                                     // acceleration; (size_t)-1 when absent
    size_t dfl[3];                   // with passive scalars: the stages'
                                     // density fluxes (scratch)
    int m[3];
  };
  std::vector<Off> off;
  int parity = 0;  // 0: current faces in fa, 1: in fb
  // device descriptors: [parity][stage] StageBlocks, [parity] AuxBlocks
  void* d_sblocks[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
  void* d_aux[2] = {nullptr, nullptr};
  StageTile* d_tiles[2] = {nullptr, nullptr};
  int ntiles[2] = {0, 0};
  int tile_tx[2] = {0, 0}, tile_ty[2] = {0, 0};
  int tile_full[2] = {0, 0};  // 1: every tile of the stage is tile_tx x tile_ty
  int block_m = 0;            // every block's extent along all axes, if equal; else 0
  int* d_queue = nullptr;     // 2 counters
  int* d_nbr = nullptr;
  // mesh refresh from a face list (replaces the 27-neighbour same-level
  // refresh when set): pointer tables of both face-buffer parities, the
  // regions and their CTA chunks
  char* d_rf = nullptr;
  size_t rf_ptr[2] = {0, 0}, rf_items = 0, rf_chunks = 0;
  int rf_nchunks = -1;  // -1: no face list
  // flux correction inside the cycle (hydro): every block's stored boundary
  // fluxes, their per-block FluxOut records, and the correction's plan
  void* d_flux = nullptr;
  void* d_fluxout = nullptr;
  char* d_fcplan = nullptr;
  FluxCorrectPlan fcplan;
  bool fc_on = false;
  // host-state runs (mhdvlct_batch_run_host): the full-dt stage's tiles by
  // group of consecutive blocks, the groups' block ranges, their queue
  // counters, and the copy streams and events
  std::vector<StageTile> h_tiles1;  // host copy of the full-dt stage's tiles
  int hg_n = 0;
  std::vector<int> hg_first;        // first block of each group (+ end)
  StageTile* d_gtiles = nullptr;
  std::vector<int> hg_tile0, hg_ntile;
  int* d_gqueue = nullptr;
  cudaStream_t s_d2h = nullptr, s_h2d = nullptr;
  std::vector<cudaEvent_t> ev;      // 3 per group: stage done, out, in
  double* d_dt = nullptr;     // per block
  double* d_dtmin = nullptr;
  double* d_time = nullptr;
  void* d_smax = nullptr;
  double* d_diag = nullptr;   // diagnostics: partial rows then the 8 totals
  int diag_rows = 0;
  int grid = 0;               // persistent grid size (0 = fill the GPU)
  int threads[2] = {256, 256};  // CTA size of each stage's launches
  std::map<std::vector<int>, TileChoice> tune;  // per block-size class
  cudaGraphExec_t graph[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
  // stream-ordered batch (a serving request's): every device allocation and
  // free is ordered on `ost` (cudaMallocAsync / cudaFreeAsync), and set-up
  // copies run on it, so creating and destroying the batch never waits for
  // work on other streams
  bool ordered = false;
  cudaStream_t ost = nullptr;
  cudaMemPool_t mpool = nullptr;  // the pool of an ordered batch (null: default)
  std::string err;

  template <class R> R* ptr(size_t o) const { return (R*)pool + o; }
};

namespace {

int bfail(mhdvlct_batch* b, int code, const std::string& m) {
  b->err = m;
  if (b->h) b->h->err = m;
  return code;
}

// Device memory of a batch: stream-ordered on the batch's stream for an
// ordered batch, plain cudaMalloc / cudaFree otherwise.
cudaError_t bmalloc(mhdvlct_batch* b, void** p, size_t n) {
  if (!b->ordered) return cudaMalloc(p, n);
  return b->mpool ? cudaMallocFromPoolAsync(p, n, b->mpool, b->ost)
                  : cudaMallocAsync(p, n, b->ost);
}
void bfree(mhdvlct_batch* b, void* p) {
  if (!p) return;
  if (b->ordered) cudaFreeAsync(p, b->ost);
  else cudaFree(p);
}
// The stream of a batch's own set-up work (its ordered stream, else the
// caller's).
cudaStream_t setup_stream(const mhdvlct_batch* b, cudaStream_t st) {
  return b->ordered ? b->ost : st;
}

void drop_graphs(mhdvlct_batch* b) {
  for (int p = 0; p < 2; p++)
    for (int d = 0; d < 2; d++)
      if (b->graph[p][d]) {
        cudaGraphExecDestroy(b->graph[p][d]);
        b->graph[p][d] = nullptr;
      }
}

TileChoice choice_for(const mhdvlct_batch* b, int i) {
  std::vector<int> key(b->dims.begin() + 3 * i, b->dims.begin() + 3 * i + 3);
  auto it = b->tune.find(key);
  TileChoice c;
  const bool tuned = it != b->tune.end();
  if (tuned) c = it->second;
  const StagePlan sp = stage_plan(b->h);
  for (int s = 0; s < 2; s++)
    if (c.tile_x[s] <= 0 || c.tile_y[s] <= 0) {
      default_tile_xy(b->dtype, b->h->solver, sp.recon[s], b->h->de, c.tile_x[s],
                      c.tile_y[s]);
    }
  if (!tuned) {
    // untuned default: when the batch has too few column tiles to fill the
    // GPU (a few large blocks, e.g. one serving request), cut the columns
    // into z-chunks so that a stage has about two waves of tiles
    // SM count of the current device (thread-safe one-time initialisation)
    static const int nsm = [] {
      int dev = 0, n = 0;
      cudaGetDevice(&dev);
      if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
          n <= 0)
        n = 1;
      return n;
    }();
    const int target = 4 * nsm;
    auto columns_of = [&](int tx, int ty) {
      long columns = 0;
      for (int k = 0; k < b->nblocks; k++) {
        const int mx = b->dims[3 * k] + 2 * b->g, my = b->dims[3 * k + 1] + 2 * b->g;
        columns += (long)((mx + tx - 1) / tx) * ((my + ty - 1) / ty);
      }
      return columns;
    };
    for (int s = 0; s < 2; s++) {
      long columns = columns_of(c.tile_x[s], c.tile_y[s]);
      if (columns < target && c.tile_x[s] != c.tile_y[s]) {
        // a batch too small to fill the GPU with the large rectangular
        // tiles: the smaller square tile (several CTAs per SM) instead
        const int t = default_tile(b->dtype, b->h->solver, sp.recon[s], b->h->de);
        c.tile_x[s] = c.tile_y[s] = t;
        columns = columns_of(t, t);
      }
      const int mz = b->dims[3 * i + 2] + 2 * b->g;
      if (columns < target && mz > 24) {
        const long chunks = (target + columns - 1) / columns;
        c.zchunk[s] = std::max(8, (int)((mz + chunks - 1) / chunks));
      }
    }
  }
  return c;
}

// (Re)build the descriptor arrays and tile lists on the device.
template <class R>
int build_descriptors(mhdvlct_batch* b, cudaStream_t st) {
  const StagePlan sp = stage_plan(b->h);
  if (sp.nstages != 2)
    return bfail(b, MHD_ERR_INVALID, "the batched form runs the two-stage vl scheme");
  std::vector<StageBlock<R>> sb[2][2];
  std::vector<AuxBlock<R>> aux[2];
  std::vector<StageTile> tiles[2];
  int tx[2] = {1, 1}, ty[2] = {1, 1};
  std::vector<std::pair<double, StageTile>> order[2];
  for (int i = 0; i < b->nblocks; i++) {
    const auto& O = b->off[i];
    FieldSet<R> ext, tmp;
    for (int k = 0; k < NCELL; k++) {
      ext.c[k] = (O.ext[k] == (size_t)-1) ? nullptr : b->ptr<R>(O.ext[k]);
      tmp.c[k] = (O.tmp[k] == (size_t)-1) ? nullptr : b->ptr<R>(O.tmp[k]);
    }
    for (int d = 0; d < 3; d++) tmp.f[d] = b->h->mhd ? b->ptr<R>(O.tf[d]) : nullptr;
    for (int p = 0; p < 2; p++) {
      FieldSet<R> cur_faces = ext, next_faces = ext;
      for (int d = 0; d < 3; d++) {
        R* fa = b->h->mhd ? b->ptr<R>(O.fa[d]) : nullptr;
        R* fb = b->h->mhd ? b->ptr<R>(O.fb[d]) : nullptr;
        cur_faces.f[d] = p == 0 ? fa : fb;
        next_faces.f[d] = p == 0 ? fb : fa;
      }
      for (int s = 0; s < 2; s++) {
        StageBlock<R> B;
        for (int a = 0; a < 3; a++) {
          B.m[a] = O.m[a];
          B.cw[a] = b->widths[3 * i + a];
        }
        B.dt = b->d_dt + i;
        B.base = cur_faces;
        for (int d = 0; d < 3; d++) B.accel[d] = b->gravity ? b->ptr<R>(O.acc[d]) : nullptr;
        for (int k = 0; k < b->npass; k++) {
          // half dt: state -> half step; full dt: half step -> state
          R* ep = b->ptr<R>(O.pas[k]);
          R* tp = b->ptr<R>(O.ptmp[k]);
          B.pass_base[k] = ep;
          B.pass_cur[k] = s == 0 ? ep : tp;
          B.pass_out[k] = s == 0 ? tp : ep;
        }
        for (int d = 0; d < 3; d++) B.dflux[d] = b->npass > 0 ? b->ptr<R>(O.dfl[d]) : nullptr;
        if (s == 0) {
          B.cur = cur_faces;
          B.out = tmp;
        } else {
          B.cur = tmp;
          B.out = next_faces;  // cells in place, faces into the other buffer
          if (b->fc_on) B.fc = (const char*)b->d_fluxout + (size_t)i * sizeof(FluxOut<R>);
        }
        sb[p][s].push_back(B);
      }
      AuxBlock<R> A;
      for (int a = 0; a < 3; a++) {
        A.m[a] = O.m[a];
        A.cw[a] = b->widths[3 * i + a];
      }
      A.f = cur_faces;
      A.pressure = b->ptr<R>(O.pres);
      for (int k = 0; k < b->npass; k++) A.pass[k] = b->ptr<R>(O.pas[k]);
      for (int d = 0; d < 3; d++) A.accel[d] = b->gravity ? b->ptr<R>(O.acc[d]) : nullptr;
      aux[p].push_back(A);
    }
    const TileChoice c = choice_for(b, i);
    for (int s = 0; s < 2; s++) {
      std::vector<StageTile> t;
      make_tiles(i, O.m, sp.S[s], s == 1, c.tile_x[s], c.tile_y[s], c.zchunk[s], t);
      for (auto& x : t) {
        tx[s] = std::max(tx[s], x.xb - x.xa);
        ty[s] = std::max(ty[s], x.yb - x.ya);
        const double cost = (double)(x.xb - x.xa + 2) * (x.yb - x.ya + 2) *
                            (x.zb - x.za + 2);
        order[s].push_back({cost, x});
      }
    }
  }
  // the launch shape: every tile at the largest extent; one cubic extent
  // shared by every block
  int block_m = b->off[0].m[0];
  for (int i = 0; i < b->nblocks; i++)
    for (int a = 0; a < 3; a++)
      if (b->off[i].m[a] != block_m) block_m = 0;
  b->block_m = block_m;
  for (int s = 0; s < 2; s++) {
    b->tile_full[s] = 1;
    for (auto& o : order[s])
      if (o.second.xb - o.second.xa != tx[s] || o.second.yb - o.second.ya != ty[s])
        b->tile_full[s] = 0;
  }
  for (int s = 0; s < 2; s++) {
    std::stable_sort(order[s].begin(), order[s].end(),
                     [](const std::pair<double, StageTile>& a,
                        const std::pair<double, StageTile>& c) { return a.first > c.first; });
    for (auto& o : order[s]) tiles[s].push_back(o.second);
    b->ntiles[s] = (int)tiles[s].size();
    if (s == 1) b->h_tiles1 = tiles[s];
    b->tile_tx[s] = tx[s];
    b->tile_ty[s] = ty[s];
  }
  st = setup_stream(b, st);
  auto upload = [&](void** dst, const void* src, size_t bytes) -> int {
    if (*dst) bfree(b, *dst);
    *dst = nullptr;
    if (bmalloc(b, dst, std::max<size_t>(bytes, 16)) != cudaSuccess)
      return bfail(b, MHD_ERR_NOMEM, "descriptor allocation");
    if (cudaMemcpyAsync(*dst, src, bytes, cudaMemcpyHostToDevice, st) != cudaSuccess)
      return bfail(b, MHD_ERR_CUDA, "descriptor upload");
    return MHD_OK;
  };
  int rc;
  for (int p = 0; p < 2; p++) {
    for (int s = 0; s < 2; s++)
      if ((rc = upload(&b->d_sblocks[p][s], sb[p][s].data(),
                       sb[p][s].size() * sizeof(StageBlock<R>))))
        return rc;
    if ((rc = upload(&b->d_aux[p], aux[p].data(), aux[p].size() * sizeof(AuxBlock<R>))))
      return rc;
  }
  for (int s = 0; s < 2; s++)
    if ((rc = upload((void**)&b->d_tiles[s], tiles[s].data(),
                     tiles[s].size() * sizeof(StageTile))))
      return rc;
  cudaStreamSynchronize(st);
  drop_graphs(b);
  b->hg_n = 0;  // the host-run groups are rebuilt from the new tiles
  return MHD_OK;
}

int build_descriptors_any(mhdvlct_batch* b, cudaStream_t st) {
  return b->dtype == MHD_DTYPE_F64 ? build_descriptors<double>(b, st)
                                   : build_descriptors<float>(b, st);
}

// The per-launch scalars of stage s (0: half dt, 1: full dt) of the batch,
// taking tiles from the work counter `queue`.  Every launch of a stage (the
// whole-batch launch and the per-group launches of a host-state run) gets
// its StageInfo here, so none of them can miss an optional term.
StageInfo batch_stage_info(const mhdvlct_batch* b, int s, int* queue) {
  const StagePlan sp = stage_plan(b->h);
  StageInfo info;
  info.s = sp.s[s];
  info.S = sp.S[s];
  info.final_stage = s == 1;
  info.dt_factor = sp.dt_factor[s];
  info.tx = b->tile_tx[s];
  info.ty = b->tile_ty[s];
  info.queue = queue;
  info.threads = b->threads[s];
  info.block_fc = (s == 1 && b->fc_on) ? 1 : 0;
  info.fc_g = b->g;
  // the gravity source enters the full-dt stage only
  // (EnzoMHDIntegratorStageCommands.cpp:279)
  info.gravity = s == 1 ? b->gravity : 0;
  info.npass = b->npass;
  info.full_tiles = b->tile_full[s];
  info.block_m = b->block_m;
  return info;
}

template <class R>
cudaError_t launch_one_stage(mhdvlct_batch* b, int s, cudaStream_t st) {
  const StagePlan sp = stage_plan(b->h);
  const StageInfo info = batch_stage_info(b, s, b->d_queue + s);
  return launch_stage<R>(b->h->solver, sp.recon[s], b->h->de != 0,
                         (const StageBlock<R>*)b->d_sblocks[b->parity][s],
                         b->d_tiles[s], b->ntiles[s], info, b->h->phys, b->grid, st);
}

template <class R>
cudaError_t launch_stages(mhdvlct_batch* b, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(b->d_queue, 0, 2 * sizeof(int), st);
  if (e != cudaSuccess) return e;
  for (int s = 0; s < 2; s++)
    if ((e = launch_one_stage<R>(b, s, st)) != cudaSuccess) return e;
  if (b->fc_on) return launch_flux_correct(b->fcplan, b->d_fcplan, st);
  return cudaSuccess;
}

// 256-thread CTAs that fill the GPU about four times over (SM count of the
// current device, thread-safe one-time initialisation)
size_t fill_ctas() {
  static const size_t n = [] {
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        nsm <= 0)
      nsm = 1;
    return (size_t)nsm * 8 * 4;
  }();
  return n;
}

template <class R>
cudaError_t launch_timestep_b(mhdvlct_batch* b, int global_min, cudaStream_t st) {
  // chunks per block so that the grid covers the GPU a few times over, also
  // when there are few blocks (a single large serving request)
  size_t cells = 0;
  for (auto& o : b->off) cells += (size_t)o.m[0] * o.m[1] * o.m[2];
  const size_t per = std::max<size_t>(1, cells / b->nblocks);
  const int cpb = (int)std::max<size_t>(
      1, std::min<size_t>(per / 8192, std::max<size_t>(64, fill_ctas() / b->nblocks)));
  return launch_timestep<R>(b->h->mhd != 0, b->h->de != 0,
                            (const AuxBlock<R>*)b->d_aux[b->parity], b->nblocks, cpb,
                            b->h->phys, b->d_smax, b->h->params.courant, global_min,
                            b->d_dt, b->d_dtmin, st);
}

template <class R>
cudaError_t launch_refresh_b(mhdvlct_batch* b, cudaStream_t st) {
  if (b->rf_nchunks >= 0)
    return launch_refresh_faces(b->dtype, b->d_rf + b->rf_items, b->d_rf + b->rf_chunks,
                                b->rf_nchunks, (void* const*)(b->d_rf + b->rf_ptr[b->parity]),
                                st);
  size_t cells = 0;
  for (auto& o : b->off) cells += (size_t)o.m[0] * o.m[1] * o.m[2];
  const size_t per = std::max<size_t>(1, cells / b->nblocks);
  const int cpb = (int)std::max<size_t>(
      1, std::min<size_t>(per / 4096, std::max<size_t>(32, fill_ctas() / b->nblocks)));
  int max_m = 0;
  for (auto& o : b->off) max_m = std::max(max_m, std::max(o.m[0], std::max(o.m[1], o.m[2])));
  return launch_refresh<R>((const AuxBlock<R>*)b->d_aux[b->parity], b->d_nbr,
                           b->nblocks, b->g, cpb, max_m, st);
}

template <class R>
cudaError_t record_cycle(mhdvlct_batch* b, int dt_mode, cudaStream_t st) {
  cudaError_t e = launch_timestep_b<R>(b, dt_mode == 0, st);
  if (e != cudaSuccess) return e;
  add_scalar_kernel<<<1, 1, 0, st>>>(b->d_time, b->d_dtmin);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if ((e = launch_refresh_b<R>(b, st)) != cudaSuccess) return e;
  return launch_stages<R>(b, st);
}

}  // namespace

// ------------------------------------------------------------------- C ABI
extern "C" int mhdvlct_batch_create(mhdvlct_handle* h, const int* dims,
                                    const double* widths, int nblocks, int ghost,
                                    int dtype, mhdvlct_batch** out) {
  return mhdvlct_batch_create_ex(h, dims, widths, nblocks, ghost, dtype, 0, 0, out);
}

extern "C" int mhdvlct_batch_create_ex(mhdvlct_handle* h, const int* dims,
                                       const double* widths, int nblocks, int ghost,
                                       int dtype, int npassive, int gravity,
                                       mhdvlct_batch** out) {
  return mhdint::batch_create(h, dims, widths, nblocks, ghost, dtype, npassive, gravity,
                              nullptr, nullptr, out);
}

int mhdint::batch_create(mhdvlct_handle* h, const int* dims, const double* widths,
                         int nblocks, int ghost, int dtype, int npassive, int gravity,
                         cudaStream_t ordered_stream, cudaMemPool_t pool,
                         mhdvlct_batch** out) {
  if (!h || !dims || !widths || !out || nblocks <= 0) return MHD_ERR_INVALID;
  *out = nullptr;
  if (npassive < 0 || npassive > 4 || (gravity != 0 && gravity != 1))
    return fail(h, MHD_ERR_INVALID, "npassive must be 0..4 and gravity 0 or 1");
  if (dtype != MHD_DTYPE_F64 && dtype != MHD_DTYPE_F32)
    return fail(h, MHD_ERR_INVALID, "unknown dtype");
  if (h->euler) return fail(h, MHD_ERR_INVALID, "the batched form runs the vl scheme");
  if (ghost < mhdvlct_required_ghost_depth(h))
    return fail(h, MHD_ERR_GHOST, "ghost depth must be at least 3");
  mhdvlct_batch* b = new mhdvlct_batch();
  b->h = h;
  b->ordered = ordered_stream != nullptr;
  b->ost = ordered_stream;
  b->mpool = pool;
  b->dtype = dtype;
  b->nblocks = nblocks;
  b->g = ghost;
  b->npass = npassive;
  b->gravity = gravity;
  b->dims.assign(dims, dims + 3 * nblocks);
  b->widths.assign(widths, widths + 3 * nblocks);
  const size_t esz = dtype == MHD_DTYPE_F64 ? 8 : 4;
  size_t o = 0;
  auto take = [&](size_t n) {
    const size_t r = o;
    o += (n + 63) & ~(size_t)63;  // 256-byte aligned for FP32, 512 for FP64
    return r;
  };
  b->off.resize(nblocks);
  // state region (cell fields and both face buffers of every block) first,
  // so that a bulk host transfer is one copy; scratch after it
  for (int pass = 0; pass < 2; pass++) {
    for (int i = 0; i < nblocks; i++) {
      auto& O = b->off[i];
      for (int a = 0; a < 3; a++) {
        if (dims[3 * i + a] < 1 || !(widths[3 * i + a] > 0)) {
          delete b;
          return fail(h, MHD_ERR_INVALID, "bad block extents or widths");
        }
        O.m[a] = dims[3 * i + a] + 2 * ghost;
      }
      const size_t M = (size_t)O.m[0] * O.m[1] * O.m[2];
      const size_t F[3] = {(size_t)(O.m[0] + 1) * O.m[1] * O.m[2],
                           (size_t)O.m[0] * (O.m[1] + 1) * O.m[2],
                           (size_t)O.m[0] * O.m[1] * (O.m[2] + 1)};
      for (int k = 0; k < NCELL; k++) {
        const bool used = (k != F_EINT || h->de) && (k < F_BX || h->mhd);
        if (pass == 0) O.ext[k] = used ? take(M) : (size_t)-1;
        else O.tmp[k] = used ? take(M) : (size_t)-1;
      }
      // passive scalars and the acceleration follow the block's cell fields
      // in the state region (a block's state stays one contiguous range)
      for (int k = 0; k < 4; k++) {
        if (pass == 0) O.pas[k] = k < npassive ? take(M) : (size_t)-1;
        else O.ptmp[k] = k < npassive ? take(M) : (size_t)-1;
      }
      for (int d = 0; d < 3; d++)
        if (pass == 0) O.acc[d] = gravity ? take(M) : (size_t)-1;
      for (int d = 0; d < 3; d++)
        if (pass == 1) O.dfl[d] = npassive > 0 ? take(M) : (size_t)-1;
      for (int d = 0; d < 3; d++)
        if (pass == 1) O.tf[d] = h->mhd ? take(F[d]) : (size_t)-1;
      if (pass == 1) O.pres = take(M);
    }
    if (pass == 0) {
      // the face-B buffers after all cell fields, buffer A of every block
      // then buffer B of every block: the current state (cells + the current
      // buffer) is then at most two contiguous segments
      b->cells_elems = o;
      for (int buf = 0; buf < 2; buf++) {
        for (int i = 0; i < nblocks; i++) {
          auto& O = b->off[i];
          const size_t F[3] = {(size_t)(O.m[0] + 1) * O.m[1] * O.m[2],
                               (size_t)O.m[0] * (O.m[1] + 1) * O.m[2],
                               (size_t)O.m[0] * O.m[1] * (O.m[2] + 1)};
          for (int d = 0; d < 3; d++) {
            const size_t at = h->mhd ? take(F[d]) : (size_t)-1;
            (buf == 0 ? O.fa[d] : O.fb[d]) = at;
          }
        }
        if (buf == 0) b->fa_end = o;
      }
      b->state_elems = o;
    }
  }
  b->pool_bytes = o * esz;
  cudaError_t e = bmalloc(b, &b->pool, b->pool_bytes);
  if (e != cudaSuccess) {
    b->pool = nullptr;
    delete b;
    return fail(h, MHD_ERR_NOMEM, std::string("batch pool: ") + cudaGetErrorString(e));
  }
  bool ok = bmalloc(b, (void**)&b->d_queue, 2 * sizeof(int)) == cudaSuccess &&
            bmalloc(b, (void**)&b->d_nbr, 27 * sizeof(int) * (size_t)nblocks) == cudaSuccess &&
            bmalloc(b, (void**)&b->d_dt, sizeof(double) * (size_t)nblocks) == cudaSuccess &&
            bmalloc(b, (void**)&b->d_dtmin, sizeof(double)) == cudaSuccess &&
            bmalloc(b, (void**)&b->d_time, sizeof(double)) == cudaSuccess &&
            bmalloc(b, &b->d_smax, 3 * sizeof(unsigned long long) * (size_t)nblocks) ==
                cudaSuccess;
  if (!ok) {
    mhdvlct_batch_destroy(b);
    return fail(h, MHD_ERR_NOMEM, "batch descriptors");
  }
  std::vector<int> nbr(27 * (size_t)nblocks);
  for (int i = 0; i < nblocks; i++)
    for (int k = 0; k < 27; k++) nbr[27 * (size_t)i + k] = i;
  if (b->ordered) {
    // everything on the batch's own stream; build_descriptors below waits
    // for that stream (and only it) before the host vector goes away
    cudaMemsetAsync(b->pool, 0, b->pool_bytes, b->ost);
    cudaMemsetAsync(b->d_time, 0, sizeof(double), b->ost);
    cudaMemcpyAsync(b->d_nbr, nbr.data(), nbr.size() * sizeof(int), cudaMemcpyHostToDevice,
                    b->ost);
  } else {
    cudaMemset(b->pool, 0, b->pool_bytes);
    cudaMemset(b->d_time, 0, sizeof(double));
    cudaMemcpy(b->d_nbr, nbr.data(), nbr.size() * sizeof(int), cudaMemcpyHostToDevice);
  }
  b->grid = 0;
  if (int rc = build_descriptors_any(b, 0)) {
    mhdvlct_batch_destroy(b);
    return rc;
  }
  *out = b;
  return MHD_OK;
}

extern "C" int mhdvlct_batch_destroy(mhdvlct_batch* b) {
  if (!b) return MHD_ERR_INVALID;
  // an ordered batch frees on its own stream after the work queued there;
  // any other batch waits for the device (its memory may be in use on any
  // stream the caller ran it on)
  if (!b->ordered) cudaDeviceSynchronize();
  drop_graphs(b);
  for (int p = 0; p < 2; p++) {
    for (int s = 0; s < 2; s++) bfree(b, b->d_sblocks[p][s]);
    bfree(b, b->d_aux[p]);
  }
  for (int s = 0; s < 2; s++) bfree(b, b->d_tiles[s]);
  bfree(b, b->d_queue);
  bfree(b, b->d_nbr);
  bfree(b, b->d_rf);
  bfree(b, b->d_flux);
  bfree(b, b->d_fluxout);
  bfree(b, b->d_fcplan);
  bfree(b, b->d_gtiles);
  bfree(b, b->d_gqueue);
  for (cudaEvent_t x : b->ev) cudaEventDestroy(x);
  if (b->s_d2h) cudaStreamDestroy(b->s_d2h);
  if (b->s_h2d) cudaStreamDestroy(b->s_h2d);
  bfree(b, b->d_dt);
  bfree(b, b->d_dtmin);
  bfree(b, b->d_time);
  bfree(b, b->d_smax);
  bfree(b, b->d_diag);
  bfree(b, b->pool);
  delete b;
  return MHD_OK;
}

namespace {
void fill_view(const mhdvlct_batch* b, int i, int parity, MhdBlockView* v);
}

extern "C" int mhdvlct_batch_block_view(mhdvlct_batch* b, int i, MhdBlockView* v) {
  if (!b || !v || i < 0 || i >= b->nblocks) return MHD_ERR_INVALID;
  fill_view(b, i, b->parity, v);
  return MHD_OK;
}

namespace {
template <class R>
int set_flux_correction_t(mhdvlct_batch* b, unsigned quantities, const MhdRefreshFace* faces,
                          int nfaces, unsigned conservative) {
  const int nx = b->dims[0], ny = b->dims[1], nz = b->dims[2];
  const size_t face_elems[3] = {(size_t)ny * nz, (size_t)nx * nz, (size_t)nx * ny};
  int nq = 0;
  for (int q = 0; q < MHD_FC_NQ; q++) nq += (quantities >> q) & 1u;
  const size_t per_block = 2 * (face_elems[0] + face_elems[1] + face_elems[2]) * nq;
  if (bmalloc(b, &b->d_flux, per_block * b->nblocks * sizeof(R)) != cudaSuccess) {
    b->d_flux = nullptr;
    return bfail(b, MHD_ERR_NOMEM, "flux buffers");
  }
  std::vector<FluxOut<R>> outs(b->nblocks);
  std::vector<MhdFluxCorrection> fcs(b->nblocks);
  std::vector<MhdBlockView> views(b->nblocks);
  R* p = (R*)b->d_flux;
  for (int i = 0; i < b->nblocks; i++) {
    std::memset(&outs[i], 0, sizeof(outs[i]));
    std::memset(&fcs[i], 0, sizeof(fcs[i]));
    outs[i].g = b->g;
    for (int a = 0; a < 3; a++)
      for (int sd = 0; sd < 2; sd++)
        for (int q = 0; q < MHD_FC_NQ; q++)
          if ((quantities >> q) & 1u) {
            outs[i].f[a][sd][q] = p;
            fcs[i].flux[a][sd][q] = p;
            p += face_elems[a];
          }
    fill_view(b, i, 0, &views[i]);  // cell fields: the same for both parities
  }
  int rc = plan_flux_correct(b->h, views.data(), b->nblocks, fcs.data(), faces, nfaces,
                             conservative, b->fcplan);
  if (rc != MHD_OK) return bfail(b, rc, b->h->err);
  if (bmalloc(b, &b->d_fluxout, outs.size() * sizeof(FluxOut<R>)) != cudaSuccess ||
      bmalloc(b, (void**)&b->d_fcplan, std::max<size_t>(b->fcplan.blob.size(), 16)) !=
          cudaSuccess)
    return bfail(b, MHD_ERR_NOMEM, "flux-correction tables");
  cudaError_t e = cudaMemcpy(b->d_fluxout, outs.data(), outs.size() * sizeof(FluxOut<R>),
                             cudaMemcpyHostToDevice);
  if (e == cudaSuccess && !b->fcplan.blob.empty())
    e = cudaMemcpy(b->d_fcplan, b->fcplan.blob.data(), b->fcplan.blob.size(),
                   cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return bfail(b, MHD_ERR_CUDA, cudaGetErrorString(e));
  b->fc_on = true;
  return MHD_OK;
}
}  // namespace

extern "C" int mhdvlct_batch_set_flux_correction(mhdvlct_batch* b, unsigned quantities,
                                                 const MhdRefreshFace* faces, int nfaces,
                                                 unsigned conservative) {
  if (!b || quantities >= (1u << MHD_FC_NQ) || nfaces < 0 || (nfaces > 0 && !faces))
    return MHD_ERR_INVALID;
  cudaDeviceSynchronize();
  b->fc_on = false;
  bfree(b, b->d_flux);
  bfree(b, b->d_fluxout);
  bfree(b, b->d_fcplan);
  b->d_flux = b->d_fluxout = nullptr;
  b->d_fcplan = nullptr;
  b->fcplan = FluxCorrectPlan();
  if (quantities != 0) {
    if (b->h->mhd)
      return bfail(b, MHD_ERR_INVALID,
                   "Flux corrections are currently only supported in hydro-mode");
    if (((quantities >> MHD_Q_INTERNAL_ENERGY) & 1u) && !b->h->de)
      return bfail(b, MHD_ERR_INVALID, "internal_energy fluxes need dual energy");
    if (quantities >> (MHD_Q_PASSIVE_0 + b->npass))
      return bfail(b, MHD_ERR_INVALID, "a passive-scalar flux names a scalar the batch lacks");
    for (int i = 1; i < b->nblocks; i++)
      for (int a = 0; a < 3; a++)
        if (b->dims[3 * i + a] != b->dims[a])
          return bfail(b, MHD_ERR_INVALID, "flux correction needs blocks of equal extents");
    const int rc = b->dtype == MHD_DTYPE_F64
                       ? set_flux_correction_t<double>(b, quantities, faces, nfaces, conservative)
                       : set_flux_correction_t<float>(b, quantities, faces, nfaces, conservative);
    if (rc != MHD_OK) return rc;
  }
  return build_descriptors_any(b, 0);  // the final stage's flux outputs; drops the graphs
}

extern "C" int mhdvlct_batch_set_refresh_faces(mhdvlct_batch* b, const MhdRefreshFace* faces,
                                               int nfaces, unsigned conservative) {
  if (!b || nfaces < 0 || (nfaces > 0 && !faces)) return MHD_ERR_INVALID;
  drop_graphs(b);
  bfree(b, b->d_rf);
  b->d_rf = nullptr;
  b->rf_nchunks = -1;
  if (nfaces == 0) return MHD_OK;  // back to the 27-neighbour refresh
  std::vector<MhdBlockView> views(b->nblocks);
  RefreshPlan plan[2];
  for (int p = 0; p < 2; p++) {
    for (int i = 0; i < b->nblocks; i++) fill_view(b, i, p, &views[i]);
    const int rc = plan_refresh(b->h, views.data(), b->nblocks, faces, nfaces, conservative,
                                plan[p]);
    if (rc != MHD_OK) return bfail(b, rc, b->h->err);
  }
  auto up = [](size_t x) { return (x + 255) / 256 * 256; };
  const size_t bp = plan[0].ptrs.size() * sizeof(void*);
  b->rf_ptr[0] = 0;
  b->rf_ptr[1] = up(bp);
  b->rf_items = b->rf_ptr[1] + up(bp);
  b->rf_chunks = b->rf_items + up(plan[0].items.size());
  const size_t total = b->rf_chunks + plan[0].chunks.size() + 1;
  std::vector<char> host(total, 0);
  memcpy(host.data() + b->rf_ptr[0], plan[0].ptrs.data(), bp);
  memcpy(host.data() + b->rf_ptr[1], plan[1].ptrs.data(), bp);
  memcpy(host.data() + b->rf_items, plan[0].items.data(), plan[0].items.size());
  memcpy(host.data() + b->rf_chunks, plan[0].chunks.data(), plan[0].chunks.size());
  if (bmalloc(b, (void**)&b->d_rf, total) != cudaSuccess) {
    b->d_rf = nullptr;
    return bfail(b, MHD_ERR_NOMEM, "refresh tables");
  }
  cudaError_t e = cudaMemcpy(b->d_rf, host.data(), total, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return bfail(b, MHD_ERR_CUDA, cudaGetErrorString(e));
  b->rf_nchunks = plan[0].nchunks;
  return MHD_OK;
}

namespace {
void fill_view(const mhdvlct_batch* b, int i, int parity, MhdBlockView* v) {
  std::memset(v, 0, sizeof(*v));
  const auto& O = b->off[i];
  const size_t esz = b->dtype == MHD_DTYPE_F64 ? 8 : 4;
  char* base = (char*)b->pool;
  auto p = [&](size_t o) -> void* { return o == (size_t)-1 ? nullptr : base + o * esz; };
  v->dtype = b->dtype;
  for (int a = 0; a < 3; a++) {
    v->n[a] = b->dims[3 * i + a];
    v->ghost[a] = b->g;
    v->cell_width[a] = b->widths[3 * i + a];
  }
  v->density = p(O.ext[F_RHO]);
  v->velocity[0] = p(O.ext[F_VX]);
  v->velocity[1] = p(O.ext[F_VY]);
  v->velocity[2] = p(O.ext[F_VZ]);
  v->total_energy = p(O.ext[F_ETOT]);
  v->internal_energy = p(O.ext[F_EINT]);
  for (int d = 0; d < 3; d++) {
    v->bfield[d] = p(O.ext[F_BX + d]);
    v->bfieldi[d] = p(parity == 0 ? O.fa[d] : O.fb[d]);
  }
  v->pressure = p(O.pres);
  for (int d = 0; d < 3; d++) v->acceleration[d] = p(O.acc[d]);
  for (int k = 0; k < b->npass; k++) v->passive[k] = p(O.pas[k]);
  v->npassive = b->npass;
}
}  // namespace

extern "C" int mhdvlct_batch_set_neighbors(mhdvlct_batch* b, const int* nbr) {
  if (!b || !nbr) return MHD_ERR_INVALID;
  for (int i = 0; i < b->nblocks; i++)
    for (int k = 0; k < 27; k++) {
      const int j = nbr[27 * (size_t)i + k];
      if (j < 0 || j >= b->nblocks) return bfail(b, MHD_ERR_INVALID, "neighbour index out of range");
      for (int a = 0; a < 3; a++)
        if (b->dims[3 * j + a] != b->dims[3 * i + a])
          return bfail(b, MHD_ERR_INVALID, "neighbours must have equal extents");
    }
  cudaError_t e = cudaMemcpy(b->d_nbr, nbr, 27 * sizeof(int) * (size_t)b->nblocks,
                             cudaMemcpyHostToDevice);
  return e == cudaSuccess ? MHD_OK : bfail(b, MHD_ERR_CUDA, cudaGetErrorString(e));
}

extern "C" int mhdvlct_batch_refresh(mhdvlct_batch* b, void* stream) {
  if (!b) return MHD_ERR_INVALID;
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e = b->dtype == MHD_DTYPE_F64 ? launch_refresh_b<double>(b, st)
                                            : launch_refresh_b<float>(b, st);
  return e == cudaSuccess ? MHD_OK : bfail(b, MHD_ERR_CUDA, cudaGetErrorString(e));
}

extern "C" int mhdvlct_batch_step(mhdvlct_batch* b, const double* dt_per_block,
                                  void* stream) {
  if (!b || !dt_per_block) return MHD_ERR_INVALID;
  for (int i = 0; i < b->nblocks; i++)
    if (!(dt_per_block[i] > 0) || !std::isfinite(dt_per_block[i]))
      return bfail(b, MHD_ERR_INVALID, "dt must be positive and finite");
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e = cudaMemcpyAsync(b->d_dt, dt_per_block, sizeof(double) * b->nblocks,
                                  cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = b->dtype == MHD_DTYPE_F64 ? launch_stages<double>(b, st) : launch_stages<float>(b, st);
  if (e != cudaSuccess) return bfail(b, MHD_ERR_CUDA, cudaGetErrorString(e));
  b->parity ^= 1;
  return MHD_OK;
}

extern "C" int mhdvlct_batch_timestep(mhdvlct_batch* b, double* dt_out, void* stream) {
  if (!b || !dt_out) return MHD_ERR_INVALID;
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e = b->dtype == MHD_DTYPE_F64 ? launch_timestep_b<double>(b, 0 + 0, st)
                                            : launch_timestep_b<float>(b, 0, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(dt_out, b->d_dt, sizeof(double) * b->nblocks,
                        cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  return e == cudaSuccess ? MHD_OK : bfail(b, MHD_ERR_CUDA, cudaGetErrorString(e));
}

extern "C" int mhdvlct_batch_run(mhdvlct_batch* b, int ncycles, int dt_mode,
                                 double* elapsed_out, void* stream) {
  if (!b || ncycles < 0 || (dt_mode != 0 && dt_mode != 1)) return MHD_ERR_INVALID;
  cudaStream_t st = (cudaStream_t)stream;
  // the simulated-time accumulator restarts with every call that advances;
  // a call with ncycles == 0 just reads it
  cudaError_t e = ncycles > 0 ? cudaMemsetAsync(b->d_time, 0, sizeof(double), st)
                              : cudaSuccess;
  for (int c = 0; c < ncycles && e == cudaSuccess; c++) {
    cudaGraphExec_t& ge = b->graph[b->parity][dt_mode];
    if (!ge) {
      // capture this parity's cycle once on a private stream
      cudaStream_t cs;
      if ((e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking)) != cudaSuccess) break;
      cudaGraph_t gph = nullptr;
      e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
      if (e == cudaSuccess) {
        cudaError_t e2 = b->dtype == MHD_DTYPE_F64 ? record_cycle<double>(b, dt_mode, cs)
                                                   : record_cycle<float>(b, dt_mode, cs);
        e = cudaStreamEndCapture(cs, &gph);
        if (e2 != cudaSuccess) e = e2;
      }
      if (e == cudaSuccess) e = cudaGraphInstantiate(&ge, gph, 0);
      if (gph) cudaGraphDestroy(gph);
      cudaStreamDestroy(cs);
      if (e != cudaSuccess) {
        ge = nullptr;
        break;
      }
    }
    e = cudaGraphLaunch(ge, st);
    b->parity ^= 1;
  }
  if (e == cudaSuccess && elapsed_out) {
    e = cudaMemcpyAsync(elapsed_out, b->d_time, sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  }
  return e == cudaSuccess ? MHD_OK : bfail(b, MHD_ERR_CUDA, cudaGetErrorString(e));
}

extern "C" int mhdvlct_batch_set_tile(mhdvlct_batch* b, int tile_x, int tile_y) {
  if (!b || tile_x < 0 || tile_y < 0) return MHD_ERR_INVALID;
  const int tmax = b->dtype == MHD_DTYPE_F64 ? TileLimits<double>::TMAX
                                             : TileLimits<float>::TMAX;
  if (tile_x > tmax || tile_y > tmax) return bfail(b, MHD_ERR_INVALID, "tile too large");
  b->tune.clear();
  for (int i = 0; i < b->nblocks; i++) {
    std::vector<int> key(b->dims.begin() + 3 * i, b->dims.begin() + 3 * i + 3);
    TileChoice c;
    for (int s = 0; s < 2; s++) {
      c.tile_x[s] = tile_x;
      c.tile_y[s] = tile_y;
    }
    b->tune[key] = c;
  }
  return build_descriptors_any(b, 0);
}

extern "C" int mhdvlct_batch_set_stage_tile(mhdvlct_batch* b, int stage, int tile_x,
                                            int tile_y, int zchunk, int threads) {
  if (!b || stage < 0 || stage > 1 || tile_x < 0 || tile_y < 0 || zchunk < 0)
    return MHD_ERR_INVALID;
  const int tmax = b->dtype == MHD_DTYPE_F64 ? TileLimits<double>::TMAX
                                             : TileLimits<float>::TMAX;
  if (tile_x > tmax || tile_y > tmax) return bfail(b, MHD_ERR_INVALID, "tile too large");
  const StagePlan sp = stage_plan(b->h);
  const int tmax_threads = b->dtype == MHD_DTYPE_F64
                               ? stage_max_threads<double>(sp.recon[stage])
                               : stage_max_threads<float>(sp.recon[stage]);
  if (threads != 0 && threads != 256 && !(threads == 512 && tmax_threads >= 512))
    return bfail(b, MHD_ERR_INVALID, "threads must be 256 (or 512 where the stage allows it)");
  for (int i = 0; i < b->nblocks; i++) {
    std::vector<int> key(b->dims.begin() + 3 * i, b->dims.begin() + 3 * i + 3);
    TileChoice c = choice_for(b, i);
    c.tile_x[stage] = tile_x;
    c.tile_y[stage] = tile_y;
    c.zchunk[stage] = zchunk;
    b->tune[key] = c;
  }
  b->threads[stage] = threads ? threads : 256;
  return build_descriptors_any(b, 0);
}

namespace {

// Groups of consecutive blocks of about equal zone counts, and the full-dt
// stage's tiles of each group (in the batch's largest-first order).
int setup_host_groups(mhdvlct_batch* b, int ngroups) {
  if (b->hg_n == ngroups) return MHD_OK;
  long total = 0;
  std::vector<long> zones(b->nblocks);
  for (int i = 0; i < b->nblocks; i++) {
    zones[i] = (long)b->dims[3 * i] * b->dims[3 * i + 1] * b->dims[3 * i + 2];
    total += zones[i];
  }
  b->hg_first.assign(1, 0);
  long acc = 0;
  for (int i = 0; i < b->nblocks; i++) {
    acc += zones[i];
    const int k = (int)b->hg_first.size();  // the group being filled
    if (k < ngroups && acc * ngroups >= total * k && i + 1 < b->nblocks)
      b->hg_first.push_back(i + 1);
  }
  b->hg_first.push_back(b->nblocks);
  const int ng = (int)b->hg_first.size() - 1;
  std::vector<int> group_of(b->nblocks);
  for (int g = 0; g < ng; g++)
    for (int i = b->hg_first[g]; i < b->hg_first[g + 1]; i++) group_of[i] = g;
  std::vector<StageTile> sorted;
  b->hg_tile0.assign(ng, 0);
  b->hg_ntile.assign(ng, 0);
  for (int g = 0; g < ng; g++) {
    b->hg_tile0[g] = (int)sorted.size();
    for (const StageTile& t : b->h_tiles1)
      if (group_of[t.block] == g) sorted.push_back(t);
    b->hg_ntile[g] = (int)sorted.size() - b->hg_tile0[g];
  }
  bfree(b, b->d_gtiles);
  bfree(b, b->d_gqueue);
  b->d_gtiles = nullptr;
  b->d_gqueue = nullptr;
  if (bmalloc(b, (void**)&b->d_gtiles, std::max<size_t>(1, sorted.size()) * sizeof(StageTile)) !=
          cudaSuccess ||
      bmalloc(b, (void**)&b->d_gqueue, ng * sizeof(int)) != cudaSuccess)
    return bfail(b, MHD_ERR_NOMEM, "host-run tables");
  cudaError_t e = cudaMemcpy(b->d_gtiles, sorted.data(), sorted.size() * sizeof(StageTile),
                             cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return bfail(b, MHD_ERR_CUDA, cudaGetErrorString(e));
  if (!b->s_d2h && cudaStreamCreateWithFlags(&b->s_d2h, cudaStreamNonBlocking) != cudaSuccess)
    return bfail(b, MHD_ERR_CUDA, "copy stream");
  if (!b->s_h2d && cudaStreamCreateWithFlags(&b->s_h2d, cudaStreamNonBlocking) != cudaSuccess)
    return bfail(b, MHD_ERR_CUDA, "copy stream");
  while ((int)b->ev.size() < 3 * ng) {
    cudaEvent_t x;
    if (cudaEventCreateWithFlags(&x, cudaEventDisableTiming) != cudaSuccess)
      return bfail(b, MHD_ERR_CUDA, "events");
    b->ev.push_back(x);
  }
  b->hg_n = ng;
  return MHD_OK;
}

// The state bytes of group g: its cells and its current face B, as offsets
// in the pool and in the host buffer (cells of all blocks, then the current
// faces of all blocks).
struct GroupSpan {
  size_t dev[2], host[2], bytes[2];
  int n;
};
GroupSpan group_span(const mhdvlct_batch* b, int g, int parity, size_t esz) {
  GroupSpan sp{};
  const int i0 = b->hg_first[g], i1 = b->hg_first[g + 1];
  // cells: from the first field of block i0 to the first field of block i1
  auto first_cell = [&](int i) -> size_t {
    if (i >= b->nblocks) return b->cells_elems;
    size_t lo = (size_t)-1;
    for (int k = 0; k < NCELL; k++)
      if (b->off[i].ext[k] != (size_t)-1) lo = std::min(lo, b->off[i].ext[k]);
    return lo;
  };
  const size_t c0 = first_cell(i0), c1 = first_cell(i1);
  sp.dev[0] = c0 * esz;
  sp.host[0] = c0 * esz;
  sp.bytes[0] = (c1 - c0) * esz;
  sp.n = 1;
  if (b->h->mhd) {
    const size_t base = parity == 0 ? b->cells_elems : b->fa_end;
    const size_t end = parity == 0 ? b->fa_end : b->state_elems;
    auto first_face = [&](int i) -> size_t {
      if (i >= b->nblocks) return end;
      return parity == 0 ? b->off[i].fa[0] : b->off[i].fb[0];
    };
    const size_t f0 = first_face(i0), f1 = first_face(i1);
    sp.dev[1] = f0 * esz;
    sp.host[1] = (b->cells_elems + (f0 - base)) * esz;
    sp.bytes[1] = (f1 - f0) * esz;
    sp.n = 2;
  }
  return sp;
}

template <class R>
int run_host_t(mhdvlct_batch* b, char* host, int ncycles, cudaStream_t st) {
  const size_t esz = sizeof(R);
  char* dev = (char*)b->pool;
  const int ng = b->hg_n;
  cudaError_t e = cudaSuccess;
  auto copy = [&](const GroupSpan& sp, bool in, cudaStream_t cs) {
    for (int k = 0; k < sp.n && e == cudaSuccess; k++)
      e = in ? cudaMemcpyAsync(dev + sp.dev[k], host + sp.host[k], sp.bytes[k],
                               cudaMemcpyHostToDevice, cs)
             : cudaMemcpyAsync(host + sp.host[k], dev + sp.dev[k], sp.bytes[k],
                               cudaMemcpyDeviceToHost, cs);
  };
  cudaEvent_t* ev = b->ev.data();  // [0, ng): stage done; [ng, 2ng): out; [2ng, 3ng): in
  e = cudaMemsetAsync(b->d_time, 0, sizeof(double), st);
  // the first cycle's input, on the compute stream
  for (int g = 0; g < ng && e == cudaSuccess; g++) copy(group_span(b, g, b->parity, esz), true, st);
  for (int c = 0; c < ncycles && e == cudaSuccess; c++) {
    if (c > 0)  // the input of this cycle: every group's copy back in
      for (int g = 0; g < ng && e == cudaSuccess; g++)
        e = cudaStreamWaitEvent(st, ev[2 * ng + g], 0);
    if (e == cudaSuccess) e = launch_timestep_b<R>(b, 1, st);
    if (e == cudaSuccess) {
      add_scalar_kernel<<<1, 1, 0, st>>>(b->d_time, b->d_dtmin);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = launch_refresh_b<R>(b, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->d_queue, 0, 2 * sizeof(int), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->d_gqueue, 0, ng * sizeof(int), st);
    if (e == cudaSuccess) e = launch_one_stage<R>(b, 0, st);
    const StagePlan sp = stage_plan(b->h);
    for (int g = 0; g < ng && e == cudaSuccess; g++) {
      const StageInfo info = batch_stage_info(b, 1, b->d_gqueue + g);
      e = launch_stage<R>(b->h->solver, sp.recon[1], b->h->de != 0,
                          (const StageBlock<R>*)b->d_sblocks[b->parity][1],
                          b->d_gtiles + b->hg_tile0[g], b->hg_ntile[g], info, b->h->phys,
                          b->grid, st);
      if (e == cudaSuccess && !b->fc_on) e = cudaEventRecord(ev[g], st);
    }
    if (e == cudaSuccess && b->fc_on) {
      // the correction needs every block's fluxes: the groups leave after it
      e = launch_flux_correct(b->fcplan, b->d_fcplan, st);
      for (int g = 0; g < ng && e == cudaSuccess; g++) e = cudaEventRecord(ev[g], st);
    }
    b->parity ^= 1;  // the new face B is in the other buffer
    const bool more = c + 1 < ncycles;
    for (int g = 0; g < ng && e == cudaSuccess; g++) {
      const GroupSpan sp_g = group_span(b, g, b->parity, esz);
      e = cudaStreamWaitEvent(b->s_d2h, ev[g], 0);
      if (e == cudaSuccess) copy(sp_g, false, b->s_d2h);
      if (e == cudaSuccess) e = cudaEventRecord(ev[ng + g], b->s_d2h);
      if (more && e == cudaSuccess) {
        // the next cycle's input: this group's state, back from the host
        e = cudaStreamWaitEvent(b->s_h2d, ev[ng + g], 0);
        if (e == cudaSuccess) copy(sp_g, true, b->s_h2d);
        if (e == cudaSuccess) e = cudaEventRecord(ev[2 * ng + g], b->s_h2d);
      }
    }
  }
  // the call's stream completes once the last state is on the host
  for (int g = 0; g < ng && e == cudaSuccess; g++) e = cudaStreamWaitEvent(st, ev[ng + g], 0);
  if (e != cudaSuccess) return bfail(b, MHD_ERR_CUDA, cudaGetErrorString(e));
  return MHD_OK;
}

}  // namespace

extern "C" int mhdvlct_batch_run_host(mhdvlct_batch* b, void* host, size_t bytes, int ncycles,
                                      int ngroups, double* elapsed_out, void* stream) {
  if (!b || !host || ncycles < 0 || ngroups < 1) return MHD_ERR_INVALID;
  const size_t esz = b->dtype == MHD_DTYPE_F64 ? 8 : 4;
  const size_t need = (b->h->mhd ? b->fa_end : b->cells_elems) * esz;
  if (bytes < need) return bfail(b, MHD_ERR_INVALID, "host buffer smaller than the state");
  if (int rc = setup_host_groups(b, std::min(ngroups, b->nblocks))) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  const int rc = b->dtype == MHD_DTYPE_F64 ? run_host_t<double>(b, (char*)host, ncycles, st)
                                           : run_host_t<float>(b, (char*)host, ncycles, st);
  if (rc != MHD_OK) return rc;
  if (elapsed_out) {
    cudaError_t e = cudaMemcpyAsync(elapsed_out, b->d_time, sizeof(double),
                                    cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return bfail(b, MHD_ERR_CUDA, cudaGetErrorString(e));
  }
  return MHD_OK;
}

extern "C" int mhdvlct_batch_state_segments(mhdvlct_batch* b, void** dev_ptrs,
                                            size_t* bytes, int max_segments,
                                            int* nsegments) {
  if (!b || !dev_ptrs || !bytes || !nsegments || max_segments < 2) return MHD_ERR_INVALID;
  const size_t esz = b->dtype == MHD_DTYPE_F64 ? 8 : 4;
  char* base = (char*)b->pool;
  dev_ptrs[0] = base;
  if (!b->h->mhd || b->parity == 0) {
    // cells followed by the current face buffer A: one segment
    bytes[0] = (b->h->mhd ? b->fa_end : b->cells_elems) * esz;
    *nsegments = 1;
  } else {
    bytes[0] = b->cells_elems * esz;
    dev_ptrs[1] = base + b->fa_end * esz;
    bytes[1] = (b->state_elems - b->fa_end) * esz;
    *nsegments = 2;
  }
  return MHD_OK;
}

const double* mhdint::batch_time_device(const mhdvlct_batch* b) { return b->d_time; }

extern "C" int mhdvlct_batch_state_region(mhdvlct_batch* b, void** dev_ptr,
                                          size_t* bytes) {
  if (!b || !dev_ptr || !bytes) return MHD_ERR_INVALID;
  *dev_ptr = b->pool;
  *bytes = b->state_elems * (b->dtype == MHD_DTYPE_F64 ? 8 : 4);
  return MHD_OK;
}

namespace {
template <class R>
int profile_t(mhdvlct_batch* b, int reps, int dt_mode, float* ms, cudaStream_t st) {
  cudaEvent_t ev[5];
  for (auto& e : ev) cudaEventCreate(&e);
  double acc[5] = {0, 0, 0, 0, 0};
  cudaError_t e = cudaSuccess;
  for (int r = 0; r < reps && e == cudaSuccess; r++) {
    cudaEventRecord(ev[0], st);
    e = launch_timestep_b<R>(b, dt_mode == 0, st);
    cudaEventRecord(ev[1], st);
    if (e == cudaSuccess) e = launch_refresh_b<R>(b, st);
    cudaEventRecord(ev[2], st);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->d_queue, 0, 2 * sizeof(int), st);
    if (e == cudaSuccess) e = launch_one_stage<R>(b, 0, st);
    cudaEventRecord(ev[3], st);
    if (e == cudaSuccess) e = launch_one_stage<R>(b, 1, st);
    if (e == cudaSuccess && b->fc_on) e = launch_flux_correct(b->fcplan, b->d_fcplan, st);
    cudaEventRecord(ev[4], st);
    if (e == cudaSuccess) e = cudaEventSynchronize(ev[4]);
    b->parity ^= 1;
    float t;
    for (int k = 0; k < 4; k++) {
      cudaEventElapsedTime(&t, ev[k], ev[k + 1]);
      acc[k] += t;
    }
    cudaEventElapsedTime(&t, ev[0], ev[4]);
    acc[4] += t;
  }
  for (auto& x : ev) cudaEventDestroy(x);
  if (e != cudaSuccess) return bfail(b, MHD_ERR_CUDA, cudaGetErrorString(e));
  for (int k = 0; k < 5; k++) ms[k] = (float)(acc[k] / std::max(1, reps));
  return MHD_OK;
}

template <class R>
int autotune_t(mhdvlct_batch* b, int reps, std::string& json, cudaStream_t st) {
  // save the state so the trial steps leave no trace
  const size_t bytes = b->state_elems * sizeof(R);
  void* save = nullptr;
  if (bmalloc(b, &save, bytes) != cudaSuccess)
    return bfail(b, MHD_ERR_NOMEM, "autotune state copy");
  const int parity0 = b->parity;
  cudaMemcpyAsync(save, b->pool, bytes, cudaMemcpyDeviceToDevice, st);
  // a dt for the trial steps (per-block CFL of the current state)
  cudaError_t e = launch_timestep_b<R>(b, 0, st);
  if (e != cudaSuccess) {
    bfree(b, save);
    return bfail(b, MHD_ERR_CUDA, cudaGetErrorString(e));
  }
  const int tmax = TileLimits<R>::TMAX;
  std::vector<std::vector<int>> classes;
  for (int i = 0; i < b->nblocks; i++) {
    std::vector<int> key(b->dims.begin() + 3 * i, b->dims.begin() + 3 * i + 3);
    if (std::find(classes.begin(), classes.end(), key) == classes.end())
      classes.push_back(key);
  }
  // largest classes first: they dominate the cost
  std::sort(classes.begin(), classes.end(), [](const std::vector<int>& a,
                                               const std::vector<int>& c) {
    return (long)a[0] * a[1] * a[2] > (long)c[0] * c[1] * c[2];
  });
  const size_t smem_cap = 227 * 1024;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  json = "{";
  bool first_cls = true;
  const StagePlan sp = stage_plan(b->h);
  for (const auto& cls : classes) {
    const int m_lat = std::max(cls[0], cls[1]) + 2 * b->g;
    std::vector<std::pair<int, int>> shapes;
    for (int ty : {6, 8, 10, 12, 14, 16}) {
      for (int tx : {ty, (3 * ty) / 2, 2 * ty, 3 * ty, m_lat - 2, m_lat - 4})
        if (tx >= ty && tx <= std::min(tmax, m_lat) && ty <= m_lat)
          shapes.push_back({tx, ty});
    }
    std::sort(shapes.begin(), shapes.end());
    shapes.erase(std::unique(shapes.begin(), shapes.end()), shapes.end());
    int rep_block = 0;
    for (int i = 0; i < b->nblocks; i++)
      if (b->dims[3 * i] == cls[0] && b->dims[3 * i + 1] == cls[1] &&
          b->dims[3 * i + 2] == cls[2]) {
        rep_block = i;
        break;
      }
    TileChoice bestc = choice_for(b, rep_block);
    float best_stage[2] = {0.f, 0.f};
    size_t ncand = 0;
    // the stages are tuned one after the other (each candidate is timed on
    // the whole two-stage step, the other stage at its current choice)
    for (int s = 0; s < 2; s++) {
      // one launch serves every class, so its shared memory is sized by the
      // largest tile extents over all classes: a candidate is kept only if
      // that combined shape fits
      int other_tx = 1, other_ty = 1;
      for (int i = 0; i < b->nblocks; i++) {
        if (b->dims[3 * i] == cls[0] && b->dims[3 * i + 1] == cls[1] &&
            b->dims[3 * i + 2] == cls[2])
          continue;
        const TileChoice oc = choice_for(b, i);
        other_tx = std::max(other_tx, oc.tile_x[s]);
        other_ty = std::max(other_ty, oc.tile_y[s]);
      }
      std::vector<TileChoice> cands;
      for (auto& sh : shapes) {
        if (stage_smem<R>(b->h->solver, sp.recon[s], b->h->de != 0,
                          std::max(sh.first, other_tx), std::max(sh.second, other_ty)) >
            smem_cap)
          continue;
        for (int zc : {0, 16}) {
          if (zc && zc >= cls[2]) continue;
          TileChoice c = bestc;
          c.tile_x[s] = sh.first;
          c.tile_y[s] = sh.second;
          c.zchunk[s] = zc;
          cands.push_back(c);
        }
      }
      float best = 1e30f;
      int best_threads = b->threads[s];
      for (int threads : {256, 512}) {
        if (threads > stage_max_threads<R>(sp.recon[s])) continue;
        b->threads[s] = threads;
        for (const auto& c : cands) {
          ncand++;
          b->tune[cls] = c;
          if (int rc = build_descriptors<R>(b, st)) {
            bfree(b, save);
            return rc;
          }
          // one untimed step, then reps timed steps
          e = launch_stages<R>(b, st);
          cudaEventRecord(e0, st);
          for (int r = 0; r < reps && e == cudaSuccess; r++) e = launch_stages<R>(b, st);
          cudaEventRecord(e1, st);
          cudaEventSynchronize(e1);
          cudaMemcpyAsync(b->pool, save, bytes, cudaMemcpyDeviceToDevice, st);
          if (e == cudaErrorInvalidValue || e == cudaErrorInvalidConfiguration) {
            // a launch shape this GPU refuses (nothing ran): skip the candidate
            e = cudaSuccess;
            continue;
          }
          if (e != cudaSuccess) break;
          float t;
          cudaEventElapsedTime(&t, e0, e1);
          if (t < best) {
            best = t;
            bestc = c;
            best_threads = threads;
          }
        }
        if (e != cudaSuccess) break;
      }
      b->threads[s] = best_threads;
      b->tune[cls] = bestc;
      best_stage[s] = best / std::max(1, reps);
      if (e != cudaSuccess) break;
    }
    char buf[512];
    std::snprintf(buf, sizeof(buf),
                  "%s\"%dx%dx%d\": {\"stage1\": {\"tile_x\": %d, \"tile_y\": %d, "
                  "\"zchunk\": %d, \"threads\": %d}, \"stage2\": {\"tile_x\": %d, "
                  "\"tile_y\": %d, \"zchunk\": %d, \"threads\": %d}, "
                  "\"ms_per_step\": %.4f, \"candidates\": %zu}",
                  first_cls ? "" : ", ", cls[0], cls[1], cls[2], bestc.tile_x[0],
                  bestc.tile_y[0], bestc.zchunk[0], b->threads[0], bestc.tile_x[1],
                  bestc.tile_y[1], bestc.zchunk[1], b->threads[1], best_stage[1], ncand);
    json += buf;
    first_cls = false;
    if (e != cudaSuccess) break;
  }
  json += "}";
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  b->parity = parity0;
  cudaMemcpyAsync(b->pool, save, bytes, cudaMemcpyDeviceToDevice, st);
  cudaStreamSynchronize(st);
  bfree(b, save);
  if (e != cudaSuccess) return bfail(b, MHD_ERR_CUDA, cudaGetErrorString(e));
  return build_descriptors<R>(b, st);
}
}  // namespace

extern "C" int mhdvlct_batch_profile(mhdvlct_batch* b, int reps, int dt_mode,
                                     float* ms_out, void* stream) {
  if (!b || !ms_out || reps < 1) return MHD_ERR_INVALID;
  cudaStream_t st = (cudaStream_t)stream;
  return b->dtype == MHD_DTYPE_F64 ? profile_t<double>(b, reps, dt_mode, ms_out, st)
                                   : profile_t<float>(b, reps, dt_mode, ms_out, st);
}

extern "C" int mhdvlct_batch_diagnostics(mhdvlct_batch* b, double* out, void* stream) {
  if (!b || !out) return MHD_ERR_INVALID;
  cudaStream_t st = (cudaStream_t)stream;
  size_t cells = 0;
  for (auto& o : b->off) cells += (size_t)o.m[0] * o.m[1] * o.m[2];
  const size_t per = std::max<size_t>(1, cells / b->nblocks);
  const int cpb = (int)std::max<size_t>(1, std::min<size_t>(per / 4096, 64));
  const int rows = b->nblocks * cpb;
  if (!b->d_diag || b->diag_rows < rows) {
    cudaStreamSynchronize(st);
    bfree(b, b->d_diag);
    b->d_diag = nullptr;
    if (bmalloc(b, (void**)&b->d_diag, ((size_t)rows + 1) * NDIAG * sizeof(double)) !=
        cudaSuccess) {
      b->d_diag = nullptr;
      return bfail(b, MHD_ERR_NOMEM, "diagnostics scratch");
    }
    b->diag_rows = rows;
  }
  double* tot = b->d_diag + (size_t)b->diag_rows * NDIAG;
  cudaError_t e =
      b->dtype == MHD_DTYPE_F64
          ? launch_diag<double>((const AuxBlock<double>*)b->d_aux[b->parity], b->nblocks,
                                b->g, cpb, b->h->mhd != 0, b->h->de != 0, b->d_diag, tot, st)
          : launch_diag<float>((const AuxBlock<float>*)b->d_aux[b->parity], b->nblocks,
                               b->g, cpb, b->h->mhd != 0, b->h->de != 0, b->d_diag, tot, st);
  if (e != cudaSuccess) return bfail(b, MHD_ERR_CUDA, std::string("diagnostics: ") + cudaGetErrorString(e));
  e = cudaMemcpyAsync(out, tot, NDIAG * sizeof(double), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return bfail(b, MHD_ERR_CUDA, std::string("diagnostics: ") + cudaGetErrorString(e));
  return MHD_OK;
}

extern "C" int mhdvlct_batch_autotune(mhdvlct_batch* b, int reps, char* json_out,
                                      size_t json_len, void* stream) {
  if (!b || reps < 1) return MHD_ERR_INVALID;
  cudaStream_t st = (cudaStream_t)stream;
  std::string json;
  int rc = b->dtype == MHD_DTYPE_F64 ? autotune_t<double>(b, reps, json, st)
                                     : autotune_t<float>(b, reps, json, st);
  if (json_out && json_len) std::snprintf(json_out, json_len, "%s", json.c_str());
  return rc;
}
