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

}  // namespace mhdint
