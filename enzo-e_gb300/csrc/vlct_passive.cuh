// vlct_passive.cuh -- the passive scalars of one VL+CT stage.
//
// Launched after the stage kernel on the same tiles.  The stage kernel has
// written the density flux of every face of its update region
// (StageBlock::dflux); this kernel advects each scalar with it, per updated
// cell:
//   - the scalar in specific form, conserved value / density of the stage's
//     input state (EnzoPhysicsFluidProps.cpp:120-133);
//   - at both faces of the cell along each axis, the specific scalar
//     reconstructed like the primitives but without floors (nearest
//     neighbour, or PLM with the stage's limiter) and upwinded with the sign
//     of the density flux, times that flux (EnzoRiemannUtils.hpp:224-314);
//   - conserved = start-of-step value + dU, dU the flux divergence x, y, z
//     (EnzoIntegrationQuanUpdate.cpp:105-147, :242-270);
//   - on the final stage, dt/dx times the flux through the block's active
//     boundary faces when the flux-correction outputs ask for the scalar
//     (EnzoMethodMHDVlct.cpp:250-330).
// The cells, faces and operation order are those of the stage kernel's own
// update, so FP64 results are the reference's bit for bit.  The scalars'
// arithmetic is a small part of a zone's work; kept out of the fused kernel
// it costs that kernel neither shared memory nor registers.  Each face's
// flux is formed by both cells that share it (the same value twice), and
// the stencil values come straight from global memory through L1.
#pragma once
#include "vlct_stage.cuh"

namespace vlct {

template <class R, int RECON>
__global__ void __launch_bounds__(256)
    passive_kernel(const StageBlock<R>* __restrict__ blocks, const StageTile* __restrict__ tiles,
                   StageInfo info, PhysParams phys) {
  // the tile's block descriptor in shared memory (its pointers would be
  // reloaded from global memory after every store otherwise)
  __shared__ __align__(16) unsigned long long s_blk_raw[(sizeof(StageBlock<R>) + 7) / 8];
  __shared__ R s_dtdx[3];
  const StageTile tl = tiles[blockIdx.x];
  {
    const unsigned long long* src =
        reinterpret_cast<const unsigned long long*>(blocks + tl.block);
    for (int w = threadIdx.x; w < (int)((sizeof(StageBlock<R>) + 7) / 8); w += blockDim.x)
      s_blk_raw[w] = src[w];
  }
  const StageBlock<R>& B = *reinterpret_cast<const StageBlock<R>*>(s_blk_raw);
  const StageBlock<R>& Bg = blocks[tl.block];
  if (threadIdx.x == 0) {
    // dt / dx per axis exactly as the stage kernel forms them
    const double dt = *Bg.dt * info.dt_factor;
    for (int d = 0; d < 3; d++) s_dtdx[d] = R(dt / Bg.cw[d]);
  }
  __syncthreads();
  const int m0 = Bg.m[0], m1 = Bg.m[1], m2 = Bg.m[2];
  const int S = info.S;
  // the stage kernel's update region [S + 1, m - S - 1) within the tile
  const int x0 = max(tl.xa, S + 1), x1 = min(tl.xb, m0 - S - 1);
  const int y0 = max(tl.ya, S + 1), y1 = min(tl.yb, m1 - S - 1);
  const int z0 = max(tl.za, S + 1), z1 = min(tl.zb, m2 - S - 1);
  if (x0 >= x1 || y0 >= y1 || z0 >= z1) return;
  const int nx = x1 - x0, ny = y1 - y0;
  const int ncell = nx * ny * (z1 - z0);
  const R dtdx0 = s_dtdx[0], dtdx1 = s_dtdx[1], dtdx2 = s_dtdx[2];
  const R theta = R(phys.theta_limiter);
  const int np = info.npass;
  const size_t sy = (size_t)m0, sz = (size_t)m0 * m1;
  const FluxOut<R>* fo =
      info.final_stage
          ? static_cast<const FluxOut<R>*>(B.fc != nullptr ? B.fc : info.fc)
          : nullptr;
  const int gg = info.fc_g;
  const R* __restrict__ rho = B.cur.c[F_RHO];
  const R* __restrict__ Dx = B.dflux[0];
  const R* __restrict__ Dy = B.dflux[1];
  const R* __restrict__ Dz = B.dflux[2];

  // flux through the face between stencil cells b0 and b1 (a, c: their
  // outer neighbours), df the face's density flux
  auto face_flux = [&](R a, R b0, R b1, R c, R df) -> R {
    R lv, rv;
    if (RECON == RECON_NN) {
      lv = b0;
      rv = b1;
    } else {
      R dl, dr;
      if (RECON == RECON_PLM) {
        dl = limiter_enzo_rk(a, b0, b1, theta);
        dr = limiter_enzo_rk(b0, b1, c, theta);
      } else {
        dl = limiter_athena(a, b0, b1);
        dr = limiter_athena(b0, b1, c);
      }
      lv = b0 + dl * R(0.5);
      rv = b1 - dr * R(0.5);
    }
    const R upwind = ((df > R(0)) ? R(1) : R(0)) * lv + ((df <= R(0)) ? R(1) : R(0)) * rv;
    return upwind * df;
  };

  for (int i = threadIdx.x; i < ncell; i += blockDim.x) {
    const int q = i / nx, x = x0 + (i - q * nx);
    const int t = z0 + q / ny, y = y0 + (q - (q / ny) * ny);
    const size_t c = (size_t)t * sz + (size_t)y * sy + x;
    // density fluxes of the six faces
    const R fdx0 = Dx[c], fdx1 = Dx[c + 1];
    const R fdy0 = Dy[c], fdy1 = Dy[c + sy];
    const R fdz0 = Dz[c], fdz1 = Dz[c + sz];
    // stencil densities: offsets -2 .. 2 along each axis (-1 .. 1 for NN)
    constexpr int RR = (RECON == RECON_NN) ? 1 : 2;
    R rx[2 * RR + 1], ry[2 * RR + 1], rz[2 * RR + 1];
#pragma unroll
    for (int k = -RR; k <= RR; k++) {
      rx[k + RR] = rho[c + k];
      ry[k + RR] = rho[c + (long long)k * (long long)sy];
      rz[k + RR] = rho[c + (long long)k * (long long)sz];
    }
    for (int k = 0; k < np; k++) {
      const R* __restrict__ P = B.pass_cur[k];
      R wx[2 * RR + 1], wy[2 * RR + 1], wz[2 * RR + 1];
#pragma unroll
      for (int j = -RR; j <= RR; j++) {
        wx[j + RR] = P[c + j] / rx[j + RR];
        if (j == 0) {
          wy[RR] = wz[RR] = wx[RR];
        } else {
          wy[j + RR] = P[c + (long long)j * (long long)sy] / ry[j + RR];
          wz[j + RR] = P[c + (long long)j * (long long)sz] / rz[j + RR];
        }
      }
      R fx0, fx1, fy0, fy1, fz0, fz1;
      if (RECON == RECON_NN) {
        fx0 = face_flux(R(0), wx[0], wx[1], R(0), fdx0);
        fx1 = face_flux(R(0), wx[1], wx[2], R(0), fdx1);
        fy0 = face_flux(R(0), wy[0], wy[1], R(0), fdy0);
        fy1 = face_flux(R(0), wy[1], wy[2], R(0), fdy1);
        fz0 = face_flux(R(0), wz[0], wz[1], R(0), fdz0);
        fz1 = face_flux(R(0), wz[1], wz[2], R(0), fdz1);
      } else {
        fx0 = face_flux(wx[0], wx[1], wx[2], wx[3], fdx0);
        fx1 = face_flux(wx[1], wx[2], wx[3], wx[4], fdx1);
        fy0 = face_flux(wy[0], wy[1], wy[2], wy[3], fdy0);
        fy1 = face_flux(wy[1], wy[2], wy[3], wy[4], fdy1);
        fz0 = face_flux(wz[0], wz[1], wz[2], wz[3], fdz0);
        fz1 = face_flux(wz[1], wz[2], wz[3], wz[4], fdz1);
      }
      R a = R(0.0);
      a -= dtdx0 * (fx1 - fx0);
      a -= dtdx1 * (fy1 - fy0);
      a -= dtdx2 * (fz1 - fz0);
      B.pass_out[k][c] = B.pass_base[k][c] + a;
      if (fo) {
        // the block's active boundary faces: each belongs to one cell here
        const int q6 = 6 + k;
        const bool in_y = inr(y, gg, m1 - gg), in_z = inr(t, gg, m2 - gg);
        const bool in_x = inr(x, gg, m0 - gg);
        if (in_y && in_z) {
          const size_t at = (size_t)(t - gg) * (m1 - 2 * gg) + (y - gg);
          if (x == gg && fo->f[0][0][q6]) fo->f[0][0][q6][at] = dtdx0 * fx0;
          if (x == m0 - gg - 1 && fo->f[0][1][q6]) fo->f[0][1][q6][at] = dtdx0 * fx1;
        }
        if (in_x && in_z) {
          const size_t at = (size_t)(t - gg) * (m0 - 2 * gg) + (x - gg);
          if (y == gg && fo->f[1][0][q6]) fo->f[1][0][q6][at] = dtdx1 * fy0;
          if (y == m1 - gg - 1 && fo->f[1][1][q6]) fo->f[1][1][q6][at] = dtdx1 * fy1;
        }
        if (in_x && in_y) {
          const size_t at = (size_t)(y - gg) * (m0 - 2 * gg) + (x - gg);
          if (t == gg && fo->f[2][0][q6]) fo->f[2][0][q6][at] = dtdx2 * fz0;
          if (t == m2 - gg - 1 && fo->f[2][1][q6]) fo->f[2][1][q6][at] = dtdx2 * fz1;
        }
      }
    }
  }
}

}  // namespace vlct
