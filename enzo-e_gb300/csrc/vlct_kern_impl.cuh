// vlct_kern_impl.cuh -- explicit instantiation and runtime dispatch of the
// kernel templates for one precision R.  Included once per precision TU.
#pragma once
#include <algorithm>
#include <type_traits>

#include "vlct_aux.cuh"
#include "vlct_launch.h"
#include "vlct_passive.cuh"
#include "vlct_stage.cuh"

namespace vlct {

namespace {
typedef void (*StageKernelFn)(const StageBlock<VLCT_REAL>*, const StageTile*, int, StageInfo,
                              PhysParams);

// Stage kernels compiled for one launch shape (FixedShape: tile, block
// extent, stale depths as constants), for the FP32 launches of the
// production workloads, where the constants save about 12% of a stage:
//   - 32^3 blocks with 3 ghost zones (extent 38), MHD (HLLD), the two-stage
//     scheme with NN then PLM: the half-dt stage's 36 x 36 columns in tiles
//     of 18 x 9, the full-dt stage's 34 x 34 in tiles of at most 17 x 12
//     (both the default tiles and the autotuner's choice for this block),
//     plain and with the gravity source / passive scalars;
//   - 32^3 blocks with 4 ghost zones (extent 40), hydro (HLLC), the default
//     tiles: 38 x 38 columns in tiles of at most 19 x 10, and 36 x 36 in
//     tiles of 18 x 12, with and without flux storing.
// Returns null unless the launch has exactly one of these shapes.
template <int SOLVER, int RECON, bool DE, int EXTRA>
StageKernelFn fixed_shape(const StageInfo& in) {
  if constexpr (std::is_same<VLCT_REAL, float>::value && !DE) {
    // the launch's (tile, every-tile-full, block extent, s, S, final) against
    // one compiled shape
    auto is = [&](int lx, int ly, bool full, int bm, int s, int S, bool fin) {
      return in.tx == lx && in.ty == ly && (!full || in.full_tiles) && in.block_m == bm &&
             in.s == s && in.S == S && (in.final_stage != 0) == fin;
    };
    if constexpr (SOLVER == SOLVER_HLLD && RECON == RECON_NN && EXTRA != EXTRA_FC) {
      if (is(18, 9, true, 38, 0, 0, false))
        return stage_kernel<float, SOLVER, RECON, DE, EXTRA,
                            FixedShape<18, 9, true, 38, 0, 0, false>>;
    }
    if constexpr (SOLVER == SOLVER_HLLD && RECON == RECON_PLM && EXTRA != EXTRA_FC) {
      if (is(17, 12, false, 38, 1, 2, true))
        return stage_kernel<float, SOLVER, RECON, DE, EXTRA,
                            FixedShape<17, 12, false, 38, 1, 2, true>>;
    }
    if constexpr (SOLVER == SOLVER_HLLC && RECON == RECON_NN && EXTRA == EXTRA_NONE) {
      if (is(19, 10, false, 40, 0, 0, false))
        return stage_kernel<float, SOLVER, RECON, DE, EXTRA,
                            FixedShape<19, 10, false, 40, 0, 0, false>>;
    }
    if constexpr (SOLVER == SOLVER_HLLC && RECON == RECON_PLM && EXTRA != EXTRA_ALL) {
      if (is(18, 12, true, 40, 1, 2, true))
        return stage_kernel<float, SOLVER, RECON, DE, EXTRA,
                            FixedShape<18, 12, true, 40, 1, 2, true>>;
    }
  }
  (void)in;
  return nullptr;
}

template <int SOLVER, int RECON, bool DE, int EXTRA>
StageKernelFn stage_fn(const StageInfo& info) {
  const StageKernelFn f = fixed_shape<SOLVER, RECON, DE, EXTRA>(info);
  return f ? f : stage_kernel<VLCT_REAL, SOLVER, RECON, DE, EXTRA>;
}

template <class R, int SOLVER, int RECON, bool DE>
cudaError_t stage_one(const StageBlock<R>* b, const StageTile* t, int nt,
                      const StageInfo& info, const PhysParams& phys, int grid,
                      cudaStream_t st) {
  const bool all = info.gravity != 0 || info.npass > 0;
  const bool fc = info.fc != nullptr || info.block_fc != 0;
  const size_t smem = stage_smem_bytes<R, SOLVER, RECON, DE>(info.tx, info.ty);
  // the flux-storing-only variant exists for the hydro solver (flux
  // correction is hydro only); the others take the full variant
  StageKernelFn k = all ? stage_fn<SOLVER, RECON, DE, EXTRA_ALL>(info)
                        : stage_fn<SOLVER, RECON, DE, EXTRA_NONE>(info);
  if (fc && !all) {
    if constexpr (SOLVER == SOLVER_HLLC)
      k = stage_fn<SOLVER, RECON, DE, EXTRA_FC>(info);
    else
      k = stage_fn<SOLVER, RECON, DE, EXTRA_ALL>(info);
  }
  cudaError_t e = cudaFuncSetAttribute(
      k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  if (nt <= 0) return cudaSuccess;
  const int threads =
      (info.threads == 512 && StageBounds<R, RECON>::threads >= 512) ? 512 : 256;
  if (grid <= 0) {
    // persistent grid: as many CTAs as fit on the GPU at once
    int dev = 0, nsm = 1, per_sm = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, threads, smem);
    grid = std::max(1, per_sm) * nsm;
  }
  if (grid > nt) grid = nt;
  k<<<grid, threads, smem, st>>>(b, t, nt, info, phys);
  e = cudaGetLastError();
  // the passive scalars, on the same tiles, with the density fluxes the
  // stage kernel wrote
  if (e == cudaSuccess && info.npass > 0) {
    passive_kernel<R, RECON><<<nt, 256, 0, st>>>(b, t, info, phys);
    e = cudaGetLastError();
  }
  return e;
}

template <class R, int SOLVER, bool DE>
cudaError_t stage_recon(int recon, const StageBlock<R>* b, const StageTile* t,
                        int nt, const StageInfo& info, const PhysParams& phys,
                        int grid, cudaStream_t st) {
  switch (recon) {
    case RECON_NN: return stage_one<R, SOLVER, RECON_NN, DE>(b, t, nt, info, phys, grid, st);
    case RECON_PLM: return stage_one<R, SOLVER, RECON_PLM, DE>(b, t, nt, info, phys, grid, st);
    case RECON_PLM_ATHENA:
      return stage_one<R, SOLVER, RECON_PLM_ATHENA, DE>(b, t, nt, info, phys, grid, st);
  }
  return cudaErrorInvalidValue;
}

template <class R, int SOLVER>
cudaError_t stage_de(int recon, bool de, const StageBlock<R>* b,
                     const StageTile* t, int nt, const StageInfo& info,
                     const PhysParams& phys, int grid, cudaStream_t st) {
  return de ? stage_recon<R, SOLVER, true>(recon, b, t, nt, info, phys, grid, st)
            : stage_recon<R, SOLVER, false>(recon, b, t, nt, info, phys, grid, st);
}

template <class R, int SOLVER, bool DE>
size_t smem_recon(int recon, int tx, int ty) {
  switch (recon) {
    case RECON_NN: return stage_smem_bytes<R, SOLVER, RECON_NN, DE>(tx, ty);
    case RECON_PLM: return stage_smem_bytes<R, SOLVER, RECON_PLM, DE>(tx, ty);
    default: return stage_smem_bytes<R, SOLVER, RECON_PLM_ATHENA, DE>(tx, ty);
  }
}
}  // namespace

template <>
cudaError_t launch_stage<VLCT_REAL>(int solver, int recon, bool de,
                                    const StageBlock<VLCT_REAL>* b,
                                    const StageTile* t, int nt,
                                    const StageInfo& info,
                                    const PhysParams& phys, int grid,
                                    cudaStream_t st) {
  switch (solver) {
    case SOLVER_HLLE: return stage_de<VLCT_REAL, SOLVER_HLLE>(recon, de, b, t, nt, info, phys, grid, st);
    case SOLVER_HLLC: return stage_de<VLCT_REAL, SOLVER_HLLC>(recon, de, b, t, nt, info, phys, grid, st);
    case SOLVER_HLLD: return stage_de<VLCT_REAL, SOLVER_HLLD>(recon, de, b, t, nt, info, phys, grid, st);
  }
  return cudaErrorInvalidValue;
}

template <>
size_t stage_smem<VLCT_REAL>(int solver, int recon, bool de, int tx, int ty) {
  // the solver changes only NF (hydro vs MHD)
  if (solver == SOLVER_HLLC) {
    return de ? smem_recon<VLCT_REAL, SOLVER_HLLC, true>(recon, tx, ty)
              : smem_recon<VLCT_REAL, SOLVER_HLLC, false>(recon, tx, ty);
  }
  return de ? smem_recon<VLCT_REAL, SOLVER_HLLD, true>(recon, tx, ty)
            : smem_recon<VLCT_REAL, SOLVER_HLLD, false>(recon, tx, ty);
}

template <>
cudaError_t launch_timestep<VLCT_REAL>(bool mhd, bool de,
                                       const AuxBlock<VLCT_REAL>* b, int nb,
                                       int cpb, const PhysParams& phys,
                                       void* d_smax, double courant,
                                       int global_min, double* d_dt,
                                       double* d_dt_min, cudaStream_t st) {
  typedef typename SpeedBits<VLCT_REAL>::T T;
  T* smax = (T*)d_smax;
  cudaError_t e = cudaMemsetAsync(smax, 0, sizeof(T) * 3 * (size_t)nb, st);
  if (e != cudaSuccess) return e;
  const int grid = nb * cpb;
  if (mhd) {
    if (de) timestep_kernel<VLCT_REAL, true, true><<<grid, 256, 0, st>>>(b, nb, cpb, phys, smax);
    else timestep_kernel<VLCT_REAL, true, false><<<grid, 256, 0, st>>>(b, nb, cpb, phys, smax);
  } else {
    if (de) timestep_kernel<VLCT_REAL, false, true><<<grid, 256, 0, st>>>(b, nb, cpb, phys, smax);
    else timestep_kernel<VLCT_REAL, false, false><<<grid, 256, 0, st>>>(b, nb, cpb, phys, smax);
  }
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  timestep_finish_kernel<VLCT_REAL><<<1, 256, 0, st>>>(b, nb, smax, courant, global_min,
                                                       d_dt, d_dt_min);
  return cudaGetLastError();
}

template <>
cudaError_t launch_refresh<VLCT_REAL>(const AuxBlock<VLCT_REAL>* b, const int* nbr,
                                      int nb, int g, int cpb, int max_m, cudaStream_t st) {
  // the decode of refresh_shell_kernel is exact while (shell elements of a
  // field) x (largest divisor) < 2^32; bound the shell by the whole field
  const unsigned long long mm = (unsigned long long)max_m + 1;
  if (mm * mm * mm * mm < (1ull << 32))
    refresh_shell_kernel<VLCT_REAL><<<nb * cpb, 256, 0, st>>>(b, nbr, nb, g, cpb);
  else
    refresh_kernel<VLCT_REAL><<<nb * cpb, 256, 0, st>>>(b, nbr, nb, g, NCELL + 11, cpb);
  return cudaGetLastError();
}

template <>
cudaError_t launch_copy_faces<VLCT_REAL>(int m0, int m1, int m2, int S1,
                                         const VLCT_REAL* fx, const VLCT_REAL* fy,
                                         const VLCT_REAL* fz, VLCT_REAL* ox,
                                         VLCT_REAL* oy, VLCT_REAL* oz,
                                         cudaStream_t st) {
  copy_faces_kernel<VLCT_REAL><<<256, 256, 0, st>>>(m0, m1, m2, S1, S1, fx, fy, fz,
                                                    ox, oy, oz);
  return cudaGetLastError();
}

template <>
cudaError_t launch_diag<VLCT_REAL>(const AuxBlock<VLCT_REAL>* b, int nb, int g, int cpb,
                                   bool mhd, bool de, double* partial, double* out,
                                   cudaStream_t st) {
  diag_kernel<VLCT_REAL><<<nb * cpb, 256, 0, st>>>(b, nb, g, cpb, mhd ? 1 : 0, de ? 1 : 0,
                                                   partial);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  diag_finish_kernel<<<1, 256, 0, st>>>(partial, nb * cpb, out);
  return cudaGetLastError();
}

template <>
cudaError_t launch_bfield_from_potential<VLCT_REAL>(
    int m0, int m1, int m2, const double* ax, const double* ay, const double* az,
    double dx, double dy, double dz, VLCT_REAL* bfx, VLCT_REAL* bfy, VLCT_REAL* bfz,
    VLCT_REAL* bx, VLCT_REAL* by, VLCT_REAL* bz, cudaStream_t st) {
  bfield_from_potential_kernel<VLCT_REAL><<<1024, 256, 0, st>>>(m0, m1, m2, ax, ay, az, dx, dy,
                                                               dz, bfx, bfy, bfz);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  center_bfield_kernel<VLCT_REAL><<<1024, 256, 0, st>>>(m0, m1, m2, bfx, bfy, bfz, bx, by, bz);
  return cudaGetLastError();
}

}  // namespace vlct
