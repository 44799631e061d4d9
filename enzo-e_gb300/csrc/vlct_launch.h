// vlct_launch.h -- typed launch entry points of the kernels (one set per
// precision; FP64 lives in kern_f64.cu compiled with --fmad=false, FP32 in
// kern_f32.cu).
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>

#include "vlct_types.h"

namespace vlct {

template <class R> struct AuxBlock;

// Largest tile extent compiled for each precision.
template <class R> struct TileLimits;
template <> struct TileLimits<double> { static constexpr int TMAX = 16; };
template <> struct TileLimits<float> { static constexpr int TMAX = 40; };

template <class R>
cudaError_t launch_stage(int solver, int recon, bool de,
                         const StageBlock<R>* d_blocks, const StageTile* d_tiles,
                         int ntiles, const StageInfo& info,
                         const PhysParams& phys, int grid, cudaStream_t st);

template <class R>
size_t stage_smem(int solver, int recon, bool de, int tx, int ty);

template <class R>
cudaError_t launch_timestep(bool mhd, bool de, const AuxBlock<R>* d_blocks,
                            int nblocks, int chunks_per_block,
                            const PhysParams& phys, void* d_smax,
                            double courant, int global_min, double* d_dt,
                            double* d_dt_min, cudaStream_t st);

// max_m: the largest ghosted extent of any block (selects the multiply-high
// shell decode when it is exact for every block)
template <class R>
cudaError_t launch_refresh(const AuxBlock<R>* d_blocks, const int* d_nbr,
                           int nblocks, int g, int chunks_per_block, int max_m,
                           cudaStream_t st);

template <class R>
cudaError_t launch_copy_faces(int m0, int m1, int m2, int S1, const R* fx,
                              const R* fy, const R* fz, R* ox, R* oy, R* oz,
                              cudaStream_t st);

// FP64 conserved totals / div B of every block's active zones into out[8];
// partial: nb * cpb * 8 doubles of scratch.
template <class R>
cudaError_t launch_diag(const AuxBlock<R>* d_blocks, int nblocks, int g, int cpb,
                        bool mhd, bool de, double* partial, double* out,
                        cudaStream_t st);

// face B from an edge vector potential (double), then the centred B
template <class R>
cudaError_t launch_bfield_from_potential(int m0, int m1, int m2, const double* ax,
                                         const double* ay, const double* az, double dx,
                                         double dy, double dz, R* bfx, R* bfy, R* bfz,
                                         R* bx, R* by, R* bz, cudaStream_t st);

cudaError_t launch_set_scalar(double* p, double v, cudaStream_t st);

}  // namespace vlct
