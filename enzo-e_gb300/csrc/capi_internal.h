// capi_internal.h -- host-side internals shared by the C ABI translation units.
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/mhdvlct_gb300.h"
#include "vlct_launch.h"
#include "vlct_types.h"

struct mhdvlct_handle {
  MhdVlctParams params;
  int solver = 2;        // vlct::Solver
  int recon = 1;         // reconstruction of the last stage
  int mhd = 1;
  int de = 0;
  int euler = 0;
  vlct::PhysParams phys;
  std::string err;
  // plain-path scratch, reused while the block geometry and dtype repeat
  int cache_dtype = -1;
  int cache_m[3] = {0, 0, 0};
  int cache_np = 0;            // passive-scalar scratch fields in the cache
  void* scratch = nullptr;     // one device allocation
  size_t scratch_bytes = 0;
  int tile = 0;                // tile extent used by the plain path
  int zchunk = 0;              // z-chunk length used by the plain path
  // mesh-refresh tables (pointer table, regions, chunks), reused across calls
  void* rf_dev = nullptr;
  size_t rf_bytes = 0;
  cudaEvent_t rf_done = nullptr;  // recorded after the last refresh launch
  std::vector<char> rf_host;
};

namespace mhdint {

// Set the handle's error text and return the code.
int fail(mhdvlct_handle* h, int code, const std::string& msg);

// Stage geometry of the VL scheme: stale depth at entry and after the
// immediate staling of the reconstruction (EnzoReconstructorNN.hpp:31-35,
// EnzoReconstructorPLM.hpp:153-157).
struct StagePlan {
  int nstages;
  int recon[2];
  int s[2];
  int S[2];
  double dt_factor[2];
};
StagePlan stage_plan(const mhdvlct_handle* h);

// Split the output window of a stage into tiles.  m: ghosted extents of the
// block, S: stale depth after reconstruction, final: last stage.
void make_tiles(int block, const int m[3], int S, bool final, int tile_x,
                int tile_y, int zchunk, std::vector<vlct::StageTile>& out);

// Device field pointers of a block view.
template <class R>
vlct::FieldSet<R> fieldset_of(const MhdBlockView* b);

// Default tile extent for a precision (fits the shared-memory budget).
int default_tile(int dtype, int solver, int recon, int de);
// Default tile shape of the batched form (tx x ty columns).
void default_tile_xy(int dtype, int solver, int recon, int de, int& tx, int& ty);

// The batched form (batch.cu).  batch_create is mhdvlct_batch_create_ex with,
// when ordered_stream is not null, every device allocation, free and set-up
// copy of the batch ordered on that stream (cudaMallocFromPoolAsync from
// `pool`, or cudaMallocAsync when pool is null; cudaFreeAsync), so that
// creating or destroying it never waits for other streams' work.
int batch_create(mhdvlct_handle* h, const int* dims, const double* widths, int nblocks,
                 int ghost, int dtype, int npassive, int gravity,
                 cudaStream_t ordered_stream, cudaMemPool_t pool, mhdvlct_batch** out);
// Device address of the batch's simulated-time accumulator: the sum of dt
// over the cycles of the last mhdvlct_batch_run call.
const double* batch_time_device(const mhdvlct_batch* b);

// Mesh ghost refresh (refresh.cu): a validated plan of refresh faces over a
// set of block views -- the per-block field pointer table and the device
// records of the regions and their CTA chunks.
struct RefreshPlan {
  std::vector<void*> ptrs;  // MHD_NFIELD_SLOTS pointers per block
  std::vector<char> items;  // region records
  std::vector<char> chunks; // CTA chunk records
  int nchunks = 0;
  int dtype = MHD_DTYPE_F64;
};
int plan_refresh(mhdvlct_handle* h, const MhdBlockView* blocks, int nblocks,
                 const MhdRefreshFace* faces, int nfaces, unsigned conservative,
                 RefreshPlan& plan);
cudaError_t launch_refresh_faces(int dtype, const void* d_items, const void* d_chunks,
                                 int nchunks, void* const* d_ptrs, cudaStream_t st);

// Flux correction (fluxcorrect.cu): a validated plan -- the corrected faces,
// their CTA chunks and the blocks' field and flux pointers in one blob to
// upload once -- and its launch.
struct FluxCorrectPlan {
  std::vector<char> blob;
  size_t o_chunks = 0, o_blocks = 0;
  int nchunks = 0;
  int dtype = MHD_DTYPE_F64;
  int params[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};  // kernel parameters
};
int plan_flux_correct(mhdvlct_handle* h, const MhdBlockView* blocks, int nblocks,
                      const MhdFluxCorrection* fluxes, const MhdRefreshFace* faces,
                      int nfaces, unsigned conservative, FluxCorrectPlan& plan);
cudaError_t launch_flux_correct(const FluxCorrectPlan& plan, const void* d_blob,
                                cudaStream_t st);

}  // namespace mhdint
