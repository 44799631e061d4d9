// vlct_stage.cuh -- one fused VL+CT stage (half or full step) for a set of
// blocks, as a z-marching CUDA kernel.
//
// A CTA owns a column tile [xa, xb) x [ya, yb) of one block and marches up
// the block's z range (or one z-chunk of it).  Everything between the global
// state read and the stage's outputs stays in shared memory: the primitives
// and cell-centred E of a ring of z-planes, the x/y face fluxes of two
// planes, the z-face fluxes of two faces, the edge EMFs and the new face B.
// Per z-plane t the CTA runs three phases separated by __syncthreads():
//
//   B  Riemann solves: z-faces at t+1/2, x- and y-faces of plane t+1 (when
//      the boundary fluxes are stored, a short pass after B copies the
//      tile's block-boundary faces out of shared memory)
//   C  upwinded edge EMFs: E_x, E_y at t+1/2 and E_z of plane t
//   D  per column of the tile: its constrained-transport face updates (Bz
//      at t+1, Bx / By at both faces of cell t), then the cell update of
//      plane t -- centred B, flux divergence + dual-energy source, density
//      floor, energy floor / dual-energy sync, store -- and the primitives
//      + cell-centred E of plane t+1+L (L = 1 for NN, 2 for PLM) loaded into
//      the ring for the next plane (in the PLM stages, and in NN stages
//      compiled for a fixed launch shape, the raw fields are copied
//      asynchronously right after B and converted here).
//
// The index windows of every quantity are those of the reference's array
// passes (EnzoMHDIntegratorStageCommands::compute_update_stage,
// src/Enzo/hydro-mhd/EnzoMHDIntegratorStageCommands.cpp:102-261, with the
// stale-depth bookkeeping of EnzoMethodMHDVlct::compute, :459-496), so the
// values written are the reference's values wherever the reference defines
// them.  The FP64 instantiation is compiled with --fmad=false and matches the
// reference bit for bit; in the FP32 instantiation the pressure recovery
// (total minus kinetic minus magnetic energy) and the energy floor / sync run
// in float-float (vlct_energy.cuh).  Further instantiations (EXTRA) also
// store the boundary fluxes for flux correction (EXTRA_FC) or, in addition,
// add the gravity source and write the density flux of every updated face
// for the passive scalars' advection (EXTRA_ALL; the scalars themselves are
// advected by passive_kernel, vlct_passive.cuh); the default one compiles
// all of these out.
#pragma once
#include <type_traits>

#include "vlct_energy.cuh"
#include "vlct_physics.cuh"
#include "vlct_types.h"

namespace vlct {

// global primitive slot order: rho, Bx, By, Bz, vx, vy, vz, p
enum { Q_RHO = 0, Q_BX = 1, Q_VX = 4, Q_P = 7, NQ = 8 };
// shared flux slots: rho, mom x/y/z, etot, B_(d+1), B_(d+2), eint, vbar
enum { S_RHO = 0, S_MX = 1, S_E = 4, S_BJ = 5, S_BK = 6, S_EINT = 7, S_VBAR = 8 };

__device__ __forceinline__ bool inr(int a, int lo, int hi) {
  return a >= lo && a < hi;
}

// Asynchronous global -> shared copy of one element (cp.async, cached in
// L1), and the calls that close a group of them and wait for the calling
// thread's own copies.
template <class R>
__device__ __forceinline__ void cp_async_elem(R* smem, const R* gmem) {
  static_assert(sizeof(R) == 4 || sizeof(R) == 8, "element size");
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  if (sizeof(R) == 4)
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(sa), "l"(gmem) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;\n" ::: "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_group 0;\n" ::: "memory");
}

// Upwind weight of CT from the sign of the density flux
// (EnzoBfieldMethodCT.cpp:198-213).
template <class R> __device__ __forceinline__ R upw(R fd) {
  return (fd > R(0)) ? R(1.0) : ((fd < R(0)) ? R(0.0) : R(0.5));
}

// compute_edge_<true> (EnzoBfieldMethodCT.cpp:384-457)
template <class R>
__device__ __forceinline__ R edge_emf(R Ej, R Ej_kp1, R Ek, R Ek_jp1, R Wj,
                                      R Wj_kp1, R Wk, R Wk_jp1, R Ec, R Ec_jp1,
                                      R Ec_kp1, R Ec_jkp1) {
  R dEdj_r = Wk_jp1 * (Ec_jp1 + Ej) + (R(1) - Wk_jp1) * (Ec_jkp1 + Ej_kp1);
  R dEdj_l = Wk * (-Ej - Ec) + (R(1) - Wk) * (-Ej_kp1 - Ec_kp1);
  R dEdk_r = Wj_kp1 * (Ec_kp1 - Ek) + (R(1) - Wj_kp1) * (Ec_jkp1 - Ek_jp1);
  R dEdk_l = Wj * (Ek - Ec) + (R(1) - Wj) * (Ek_jp1 - Ec_jp1);
  R Ej_sum = Ej + Ej_kp1;
  Ej_sum *= R(-1);
  R Ek_sum = Ek + Ek_jp1;
  return R(0.25) * (Ej_sum + Ek_sum + (dEdj_l - dEdj_r) + (dEdk_l - dEdk_r));
}

template <class R, int SOLVER, int RECON, bool DE> struct StageCfg {
  static constexpr bool MHD = SOLVER != SOLVER_HLLC;
  static constexpr int LOOK = (RECON == RECON_NN) ? 1 : 2;
  // ring of primitive planes: the planes a step reads plus the plane loaded
  // ahead for the next step
  static constexpr int NRING = (RECON == RECON_NN) ? 3 : 4;
  static constexpr int RP = (RECON == RECON_NN) ? 0 : 1;
  static constexpr int NF = DE ? 9 : (MHD ? 7 : 5);
};

// Shared-memory carve-up for a launch whose tiles are at most tx x ty.
struct SmemLayout {
  int PP, QP;   // primitive tile pitch / rows
  int HP, HQ;   // halo grid pitch / rows (tile + 1 cell each side)
  int G;        // HP * HQ
  int o_prim, o_xf, o_yf, o_zf, o_ec, o_ex, o_ey, o_ez, o_bz;
  int total;    // in elements of R
  __host__ __device__ void init(int tx, int ty, int rp, int nring, int nf) {
    PP = tx + 2 + 2 * rp;
    QP = ty + 2 + 2 * rp;
    HP = tx + 2;
    HQ = ty + 2;
    G = HP * HQ;
    int o = 0;
    o_prim = o; o += nring * NQ * PP * QP;
    o_xf = o; o += 2 * nf * G;
    o_yf = o; o += 2 * nf * G;
    o_zf = o; o += 2 * nf * G;
    o_ec = o; o += nring * 3 * G;
    o_ex = o; o += 2 * G;
    o_ey = o; o += 2 * G;
    o_ez = o; o += G;
    o_bz = o; o += 2 * G;
    total = o;
  }
};

template <class R, int SOLVER, int RECON, bool DE>
size_t stage_smem_bytes(int tx, int ty) {
  using C = StageCfg<R, SOLVER, RECON, DE>;
  SmemLayout L;
  L.init(tx, ty, C::RP, C::NRING, C::NF);
  return (size_t)L.total * sizeof(R);
}

// Launch bounds per precision and reconstruction.  FP32 PLM: 256 or 512
// threads (the tuner's choice), registers capped at 128 so that a 512-thread
// CTA fits an SM.  FP32 NN (the half-dt stage, smaller ring and no slopes):
// 256 threads, registers capped at 85 so that three CTAs share an SM.
// FP64: 256 threads with up to 255 registers (the FP64 solver does not fit
// in 128 without spilling).
template <class R, int RECON> struct StageBounds {
  static constexpr int threads = 256, min_blocks = 1;
};
template <> struct StageBounds<float, RECON_NN> {
  static constexpr int threads = 256, min_blocks = 3;
};
template <> struct StageBounds<float, RECON_PLM> {
  static constexpr int threads = 512, min_blocks = 1;
};
template <> struct StageBounds<float, RECON_PLM_ATHENA> {
  static constexpr int threads = 512, min_blocks = 1;
};
// largest CTA a stage of this precision and reconstruction takes
template <class R>
inline int stage_max_threads(int recon) {
  return recon == RECON_NN          ? StageBounds<R, RECON_NN>::threads
         : recon == RECON_PLM       ? StageBounds<R, RECON_PLM>::threads
                                    : StageBounds<R, RECON_PLM_ATHENA>::threads;
}

enum { EXTRA_NONE = 0, EXTRA_FC = 1, EXTRA_ALL = 2 };

// Launch shapes of the stage kernel.  RuntimeShape takes every value from
// the launch.  FixedShape<LX, LY, FULL, BM, s, S, FINAL> is a launch whose
// largest tile is LX x LY (every tile exactly that when FULL), whose blocks
// all have extent BM (ghosts included) along each axis, and whose stage has
// stale depths s (start) and S (after reconstruction) and is the final
// stage when FINAL.  A fixed-shape kernel runs only launches of exactly
// that shape; its arithmetic is the run-time kernel's.
struct RuntimeShape {
  static constexpr int LX = 0, LY = 0, BM = 0, s = -1, S = -1;
  static constexpr bool FULL = false, FINAL = false;
};
template <int LX_, int LY_, bool FULL_, int BM_, int s_, int S_, bool FINAL_>
struct FixedShape {
  static_assert(LX_ > 0 && LY_ > 0 && BM_ > 0 && s_ >= 0 && S_ >= s_, "fixed shape");
  static constexpr int LX = LX_, LY = LY_, BM = BM_, s = s_, S = S_;
  static constexpr bool FULL = FULL_, FINAL = FINAL_;
};

// EXTRA: EXTRA_NONE compiles the optional work out (its run-time checks alone
// cost ~4% of a stage); EXTRA_FC can store the boundary fluxes; EXTRA_ALL
// can also add the gravity source and write the density fluxes that
// passive_kernel advects the passive scalars with.
// SH: the launch's shape -- RuntimeShape (everything read from the launch's
// StageInfo and the block descriptors) or a FixedShape, whose values are
// compile-time constants so that the index arithmetic of shared- and
// global-memory accesses folds.
template <class R, int SOLVER, int RECON, bool DE, int EXTRA, class SH = RuntimeShape>
__global__ void __launch_bounds__(StageBounds<R, RECON>::threads,
                                  StageBounds<R, RECON>::min_blocks)
stage_kernel(const StageBlock<R>* __restrict__ blocks,
             const StageTile* __restrict__ tiles, int ntiles, StageInfo info,
             PhysParams phys) {
  using C = StageCfg<R, SOLVER, RECON, DE>;
  constexpr bool MHD = C::MHD;
  constexpr int LOOK = C::LOOK, NRING = C::NRING, RP = C::RP, NF = C::NF;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  R* sm = reinterpret_cast<R*>(smem_raw);
  SmemLayout Ls;
  Ls.init(SH::LX > 0 ? SH::LX : info.tx, SH::LY > 0 ? SH::LY : info.ty, RP, NRING, NF);
  // passive scalars (EXTRA_ALL only) are advected by passive_kernel after
  // this kernel, with the density flux of every face written here
  const int PP = Ls.PP, QP = Ls.QP, HP = Ls.HP, G = Ls.G;
  const int PQ = PP * QP;
  R* s_prim = sm + Ls.o_prim;
  R* s_xf = sm + Ls.o_xf;
  R* s_yf = sm + Ls.o_yf;
  R* s_zf = sm + Ls.o_zf;
  R* s_ec = sm + Ls.o_ec;
  R* s_ex = sm + Ls.o_ex;
  R* s_ey = sm + Ls.o_ey;
  R* s_ez = sm + Ls.o_ez;
  R* s_bz = sm + Ls.o_bz;
  const int tid = threadIdx.x, nthr = blockDim.x;
  const int s = SH::S >= 0 ? SH::s : info.s, S = SH::S >= 0 ? SH::S : info.S;
  const bool final_stage = SH::S >= 0 ? SH::FINAL : info.final_stage != 0;
  // the physical constants in R.  In the FP32 NN stage (registers capped for
  // three CTAs per SM, so the compiler reloads constants from the
  // parameters) they are the values rounded on the host, which need no FP64
  // conversion on the device; the same values as the conversions here.
  constexpr bool F32 = std::is_same<R, float>::value && RECON == RECON_NN;
  const R g = F32 ? R(phys.gamma_f) : R(phys.gamma);
  const R theta = F32 ? R(phys.theta_limiter_f) : R(phys.theta_limiter);
  const R dfloor = F32 ? R(phys.density_floor_f) : R(phys.density_floor);
  const R pfloor = F32 ? R(phys.pressure_floor_f) : R(phys.pressure_floor);
  EnergyConsts<R> econ;
  if constexpr (F32)
    econ.init_rounded(phys, DE);
  else
    econ.init(phys.gamma, phys.pressure_floor, DE ? phys.eta : 0.0);
  const FastDiv divPP(Ls.PP), divHP(Ls.HP);

  __shared__ int s_next;
  // the current tile's block descriptor, copied into shared memory once per
  // tile: read from global memory, its field pointers would be reloaded after
  // every global store (the compiler cannot rule out aliasing)
  __shared__ __align__(16) unsigned long long s_blk_raw[(sizeof(StageBlock<R>) + 7) / 8];
  // the block's flux-correction outputs on a flux-storing final stage, also
  // copied once per tile: read from global memory, every boundary-face store
  // would first wait for its pointer
  constexpr int kFoWords = EXTRA != EXTRA_NONE ? (int)((sizeof(FluxOut<R>) + 7) / 8) : 1;
  __shared__ __align__(16) unsigned long long s_fo_raw[kFoWords];
  __shared__ R s_dtdx[3];
  __shared__ R s_dt;
  int it = blockIdx.x;
  if (info.queue) {
    if (tid == 0) s_next = atomicAdd(info.queue, 1);
    __syncthreads();
    it = s_next;
  }
  while (it < ntiles) {
    const StageTile tl = tiles[it];
    {
      const unsigned long long* src =
          reinterpret_cast<const unsigned long long*>(blocks + tl.block);
      for (int w = tid; w < (int)((sizeof(StageBlock<R>) + 7) / 8); w += nthr)
        s_blk_raw[w] = src[w];
      if (EXTRA != EXTRA_NONE && final_stage && (info.fc != nullptr || info.block_fc)) {
        const void* fsrc = blocks[tl.block].fc != nullptr ? blocks[tl.block].fc : info.fc;
        const unsigned long long* fw = reinterpret_cast<const unsigned long long*>(fsrc);
        for (int w = tid; w < kFoWords; w += nthr) s_fo_raw[w] = fw[w];
      }
    }
    const StageBlock<R>& B = *reinterpret_cast<const StageBlock<R>*>(s_blk_raw);
    const StageBlock<R>& Bg = blocks[tl.block];
    const int m0 = SH::BM > 0 ? SH::BM : Bg.m[0];
    const int m1 = SH::BM > 0 ? SH::BM : Bg.m[1];
    const int m2 = SH::BM > 0 ? SH::BM : Bg.m[2];
    const int xa = tl.xa, xb = tl.xb, ya = tl.ya, yb = tl.yb;
    const int tx = SH::FULL ? SH::LX : xb - xa, ty = SH::FULL ? SH::LY : yb - ya;
    // dt / dx per axis, once per tile (FP64 divisions: one thread)
    if (tid == 0) {
      const double dt = *Bg.dt * info.dt_factor;
      s_dtdx[0] = R(dt / Bg.cw[0]);
      s_dtdx[1] = R(dt / Bg.cw[1]);
      s_dtdx[2] = R(dt / Bg.cw[2]);
      s_dt = R(dt);
    }
    __syncthreads();  // also publishes the descriptor copy
    const R dtdx[3] = {s_dtdx[0], s_dtdx[1], s_dtdx[2]};
    // output window of centred B (and the z-march range)
    const int olo = final_stage ? S : S + 1;
    const int ohi_x = final_stage ? m0 - S : m0 - S - 1;
    const int ohi_y = final_stage ? m1 - S : m1 - S - 1;
    const int za = tl.za, zb = tl.zb;  // output planes of this chunk
    const int t0 = za - 1;
    // prim-tile origin and halo-grid origin
    const int px0 = xa - 1 - RP, py0 = ya - 1 - RP;
    const int hx0 = xa - 1, hy0 = ya - 1;
    const size_t cstr_y = (size_t)m0, cstr_z = (size_t)m0 * m1;

    // offset of cell (x, y) of ring slot `slot` in s_prim (add q * PQ)
    auto poff = [&](int slot, int x, int y) -> int {
      return slot * NQ * PQ + (y - py0) * PP + (x - px0);
    };

    // ---- primitives (and the cell-centred E) of plane p into its ring slot,
    // in two steps.  With ASYNC_LOADS (the PLM stages) issue_plane starts
    // asynchronous copies of the raw cell fields into the slot (the energy
    // field into the pressure plane) and finish_plane, after the copies have
    // landed, turns them into primitives in place.  Every thread finishes
    // exactly the cells it issued, so the two need no barrier between them;
    // in the z-march the copies of plane t+1+L go out right after phase B of
    // plane t (the slot they overwrite, plane t-1's, is no longer read) and
    // land while phases C and D run.  The NN stage with the run-time shape,
    // already close to its issue limit, loads in finish_plane directly: the
    // extra shared-memory pass costs it more than the latency it would hide.
    // With a fixed shape it issues fewer instructions, and the asynchronous
    // copies pay there too.
    constexpr bool ASYNC_LOADS = RECON != RECON_NN || SH::BM > 0;
    auto issue_plane = [&](int p) {
      if (!ASYNC_LOADS || !inr(p, s, m2 - s)) return;
      const int slot = p % NRING;
      const int fe = DE ? F_EINT : F_ETOT;
      for (int idx = tid; idx < PQ; idx += nthr) {
        const int qy = divPP.div(idx);
        const int x = px0 + (idx - qy * PP), y = py0 + qy;
        if (!inr(x, s, m0 - s) || !inr(y, s, m1 - s)) continue;
        const size_t c = (size_t)p * cstr_z + (size_t)y * cstr_y + x;
        R* w = s_prim + poff(slot, x, y);
        cp_async_elem(w + Q_RHO * PQ, B.cur.c[F_RHO] + c);
        cp_async_elem(w + (Q_VX + 0) * PQ, B.cur.c[F_VX] + c);
        cp_async_elem(w + (Q_VX + 1) * PQ, B.cur.c[F_VY] + c);
        cp_async_elem(w + (Q_VX + 2) * PQ, B.cur.c[F_VZ] + c);
        if (MHD) {
          cp_async_elem(w + (Q_BX + 0) * PQ, B.cur.c[F_BX] + c);
          cp_async_elem(w + (Q_BX + 1) * PQ, B.cur.c[F_BY] + c);
          cp_async_elem(w + (Q_BX + 2) * PQ, B.cur.c[F_BZ] + c);
        }
        cp_async_elem(w + Q_P * PQ, B.cur.c[fe] + c);
      }
      cp_async_commit();
    };
    auto finish_plane = [&](int p) {
      if (!inr(p, s, m2 - s)) return;
      if (ASYNC_LOADS) cp_async_wait_all();
      const int slot = p % NRING;
      const int fe = DE ? F_EINT : F_ETOT;
      for (int idx = tid; idx < PQ; idx += nthr) {
        const int qy = divPP.div(idx);
        const int x = px0 + (idx - qy * PP), y = py0 + qy;
        if (!inr(x, s, m0 - s) || !inr(y, s, m1 - s)) continue;
        R* w = s_prim + poff(slot, x, y);
        const size_t c = (size_t)p * cstr_z + (size_t)y * cstr_y + x;
        // the fields: from the slot (copied there) or from global memory
        auto field = [&](int q, int f) -> R { return ASYNC_LOADS ? w[q * PQ] : B.cur.c[f][c]; };
        const R rho = field(Q_RHO, F_RHO);
        const R vx = field(Q_VX + 0, F_VX), vy = field(Q_VX + 1, F_VY), vz = field(Q_VX + 2, F_VZ);
        R bx = R(0), by = R(0), bz = R(0);
        if (MHD) {
          bx = field(Q_BX + 0, F_BX);
          by = field(Q_BX + 1, F_BY);
          bz = field(Q_BX + 2, F_BZ);
        }
        // EnzoComputePressure::compute_pressure (EnzoComputePressure.cpp:127-190)
        const R e_in = field(Q_P, fe);
        if (!ASYNC_LOADS) {
          w[Q_RHO * PQ] = rho;
          w[(Q_VX + 0) * PQ] = vx;
          w[(Q_VX + 1) * PQ] = vy;
          w[(Q_VX + 2) * PQ] = vz;
          if (MHD) {
            w[(Q_BX + 0) * PQ] = bx;
            w[(Q_BX + 1) * PQ] = by;
            w[(Q_BX + 2) * PQ] = bz;
          }
        }
        R p_out;
        if (DE) {
          p_out = econ.gm1 * rho * e_in;
        } else {
          p_out = pressure_from_etot<R, MHD>(econ, rho, e_in, vx, vy, vz, bx, by, bz);
        }
        w[Q_P * PQ] = p_out;
        // cell-centred E = -v x B (EnzoBfieldMethodCT.cpp:267-292), on the
        // halo grid and inside [S, m - S)
        const int hi = x - hx0, hj = y - hy0;
        if (MHD && hi >= 0 && hi < HP && hj >= 0 && hj < Ls.HQ &&
            inr(x, S, m0 - S) && inr(y, S, m1 - S) && inr(p, S, m2 - S)) {
          R* e = s_ec + slot * 3 * G + hj * HP + hi;
          e[0] = (-vy * bz + vz * by);
          e[G] = (-vz * bx + vx * bz);
          e[2 * G] = (-vx * by + vy * bx);
        }
      }
    };

    // ---- Riemann solves: z-faces at t+1/2 (if zfaces) and the x- and
    // y-faces of plane pl.  One code path for all three directions.
    auto phase_b = [&](int t, bool zfaces, int pl) {
      const int HQv = Ls.HQ;
      const FastDiv divX(tx + 1);
      const int nz = zfaces ? HP * HQv : 0;
      const int nx = (tx + 1) * HQv;
      const int ny = HP * (ty + 1);
      const bool plane_ok = inr(pl, S, m2 - S);
      for (int idx = tid; idx < nz + nx + ny; idx += nthr) {
        int d, i, j;
        if (idx < nz) {
          d = 2; j = divHP.div(idx); i = idx - j * HP;
        } else if (idx < nz + nx) {
          const int q = idx - nz;
          d = 0; j = divX.div(q); i = q - j * (tx + 1);
        } else {
          const int q = idx - nz - nx;
          d = 1; j = divHP.div(q); i = q - j * HP;
        }
        const int x = hx0 + i, y = hy0 + j;
        // face index f along d: the face between cells f and f+1
        int off[4];  // s_prim offsets of the cells f-1 .. f+2 along d
        const R* bface;
        R* dst;
        const int r = j * HP + i;
        if (d == 2) {
          const int fz = t;
          if (!inr(fz, S, m2 - 1 - S) || !inr(x, S, m0 - S) || !inr(y, S, m1 - S))
            continue;
#pragma unroll
          for (int k = 0; k < 4; k++) off[k] = poff((fz - 1 + k + NRING) % NRING, x, y);
          bface = B.cur.f[2] + ((size_t)(fz + 1) * cstr_z + (size_t)y * cstr_y + x);
          dst = s_zf + (size_t)(fz & 1) * NF * G + r;
        } else {
          if (!plane_ok) continue;
          const int slot = pl % NRING;
          if (d == 0) {
            if (!inr(x, S, m0 - 1 - S) || !inr(y, S, m1 - S)) continue;
#pragma unroll
            for (int k = 0; k < 4; k++) off[k] = poff(slot, x - 1 + k, y);
            bface = B.cur.f[0] + ((size_t)pl * ((size_t)m1 * (m0 + 1)) +
                                  (size_t)y * (m0 + 1) + (x + 1));
            dst = s_xf + (size_t)(pl & 1) * NF * G + r;
          } else {
            if (!inr(y, S, m1 - 1 - S) || !inr(x, S, m0 - S)) continue;
#pragma unroll
            for (int k = 0; k < 4; k++) off[k] = poff(slot, x, y - 1 + k);
            bface = B.cur.f[1] + ((size_t)pl * ((size_t)(m1 + 1) * m0) +
                                  (size_t)(y + 1) * m0 + x);
            dst = s_yf + (size_t)(pl & 1) * NF * G + r;
          }
        }
        // reconstruction (EnzoReconstructorNN.cpp:14-49,
        // EnzoReconstructorPLM.hpp:167-345), in the face frame
        R wl[8], wr[8];
        const int d1 = (d + 1) % 3, d2 = (d + 2) % 3;
#pragma unroll
        for (int k = 0; k < 8; k++) {
          if (!MHD && (k == L_BI || k == L_BJ || k == L_BK)) {
            wl[k] = wr[k] = R(0);
            continue;
          }
          const int q = (k == L_RHO) ? Q_RHO
                      : (k == L_BI) ? Q_BX + d : (k == L_BJ) ? Q_BX + d1
                      : (k == L_BK) ? Q_BX + d2 : (k == L_VI) ? Q_VX + d
                      : (k == L_VJ) ? Q_VX + d1 : (k == L_VK) ? Q_VX + d2 : Q_P;
          const R* w = s_prim + q * PQ;
          if (RECON == RECON_NN) {
            wl[k] = w[off[1]];
            wr[k] = w[off[2]];
          } else {
            const R a = w[off[0]], b0 = w[off[1]], b1 = w[off[2]], c = w[off[3]];
            R dl, dr;
            if (RECON == RECON_PLM) {
              dl = limiter_enzo_rk(a, b0, b1, theta);
              dr = limiter_enzo_rk(b0, b1, c, theta);
            } else {
              dl = limiter_athena(a, b0, b1);
              dr = limiter_athena(b0, b1, c);
            }
            R lv = b0 + dl * R(0.5), rv = b1 - dr * R(0.5);
            if (k == L_RHO) {
              lv = smax(lv, dfloor);
              rv = smax(rv, dfloor);
            } else if (k == L_E) {
              lv = smax(lv, pfloor);
              rv = smax(rv, pfloor);
            }
            wl[k] = lv;
            wr[k] = rv;
          }
        }
        if (MHD) {  // correct_reconstructed_bfield (EnzoBfieldMethodCT.cpp:122-166)
          const R bf = *bface;
          wl[L_BI] = bf;
          wr[L_BI] = bf;
        }
        FaceFlux<R> F;
        riemann<SOLVER, R>(g, wl, wr, F);
        dst[S_RHO * G] = F.f[L_RHO];
        dst[(S_MX + d) * G] = F.f[L_VI];
        dst[(S_MX + d1) * G] = F.f[L_VJ];
        dst[(S_MX + d2) * G] = F.f[L_VK];
        dst[S_E * G] = F.f[L_E];
        if (MHD) {
          dst[S_BJ * G] = F.f[L_BJ];
          dst[S_BK * G] = F.f[L_BK];
        }
        if (DE) {
          dst[S_EINT * G] = F.eflux;
          dst[S_VBAR * G] = F.vbar;
        }
      }
    };

    // ---- store_fluxes_for_corrections (EnzoMethodMHDVlct.cpp:250-330): on
    // the final stage, dt/dx times the fluxes through the block's active
    // boundary faces, read back from the face fluxes phase B left in shared
    // memory (valid until phase B overwrites that plane parity two steps
    // later).  Every face is written by exactly one tile: the tile (and
    // z-chunk) that owns the cells on its high side.
    // (the outputs are looked up inside the pass: nothing extra stays live
    // across the z-march)
    const bool store_fc =
        EXTRA != EXTRA_NONE && final_stage && (info.fc != nullptr || info.block_fc);
    auto store_fluxes = [&](int t, bool zfaces, int pl) {
      const FluxOut<R>* fo = reinterpret_cast<const FluxOut<R>*>(s_fo_raw);
      const int gg = info.fc_g;
      // f: the face's fluxes (the passive scalars' are stored by
      // passive_kernel)
      auto put = [&](int d, int side, size_t at, const R* f) {
        const R sc = dtdx[d];
#pragma unroll
        for (int q = 0; q < 6; q++) {
          R* p = fo->f[d][side][q];
          if (!p) continue;
          const R v = q == 0 ? f[S_RHO * G]
                    : q <= 3 ? f[(S_MX + q - 1) * G]
                    : q == 4 ? f[S_E * G] : (DE ? f[S_EINT * G] : R(0));
          p[at] = sc * v;
        }
      };
      const int xlo = xa > gg ? xa : gg, xhi = xb < m0 - gg ? xb : m0 - gg;
      const int ylo = ya > gg ? ya : gg, yhi = yb < m1 - gg ? yb : m1 - gg;
      if (pl >= za && pl < zb && inr(pl, gg, m2 - gg)) {
        const R* xf = s_xf + (size_t)(pl & 1) * NF * G;
        const R* yf = s_yf + (size_t)(pl & 1) * NF * G;
        for (int side = 0; side < 2; side++) {
          const int x = side == 0 ? gg - 1 : m0 - gg - 1;  // x faces
          if (x >= xa - 1 && x < xb - 1)
            for (int y = ylo + tid; y < yhi; y += nthr) {
              const int r = (y - hy0) * HP + (x - hx0);
              put(0, side, (size_t)(pl - gg) * (m1 - 2 * gg) + (y - gg), xf + r);
            }
          const int y = side == 0 ? gg - 1 : m1 - gg - 1;  // y faces
          if (y >= ya - 1 && y < yb - 1)
            for (int x2 = xlo + tid; x2 < xhi; x2 += nthr) {
              const int r = (y - hy0) * HP + (x2 - hx0);
              put(1, side, (size_t)(pl - gg) * (m0 - 2 * gg) + (x2 - gg), yf + r);
            }
        }
      }
      const int side = t == gg - 1 ? 0 : (t == m2 - gg - 1 ? 1 : -1);  // z faces at t+1/2
      if (zfaces && side >= 0 && t >= za - 1 && t < zb - 1) {
        const R* zf = s_zf + (size_t)(t & 1) * NF * G;
        const int w = xhi - xlo;
        for (int k = tid; k < w * (yhi - ylo); k += nthr) {
          const int y = ylo + k / w, x = xlo + k % w;
          const int r = (y - hy0) * HP + (x - hx0);
          put(2, side, (size_t)(y - gg) * (m0 - 2 * gg) + (x - gg), zf + r);
        }
      }
    };

    // ---------------------------------------------------------- prologue --
    for (int p = t0 - (LOOK - 1); p <= t0 + LOOK; p++) issue_plane(p);
    for (int p = t0 - (LOOK - 1); p <= t0 + LOOK; p++) finish_plane(p);
    __syncthreads();
    phase_b(t0 - 1, false, t0);
    __syncthreads();
    if (store_fc) store_fluxes(t0 - 1, false, t0);

    for (int t = t0; t < zb; t++) {
      // ---- B: z-faces at t+1/2, x/y faces of plane t+1
      phase_b(t, true, t + 1);
      __syncthreads();
      // plane t+1+L's fields start towards the ring slot phase B just
      // released (plane t-1's)
      if (t + 1 < zb) issue_plane(t + 1 + LOOK);
      if (store_fc) store_fluxes(t, true, t + 1);
      // ---- C: edge EMFs (EnzoBfieldMethodCT.cpp:480-590)
      if (MHD) {
        const R* xf0 = s_xf + (size_t)(t & 1) * NF * G;
        const R* xf1 = s_xf + (size_t)((t + 1) & 1) * NF * G;
        const R* yf0 = s_yf + (size_t)(t & 1) * NF * G;
        const R* yf1 = s_yf + (size_t)((t + 1) & 1) * NF * G;
        const R* zf = s_zf + (size_t)(t & 1) * NF * G;
        const R* ec0 = s_ec + (size_t)(t % NRING) * 3 * G;
        const R* ec1 = s_ec + (size_t)((t + 1) % NRING) * 3 * G;
        for (int idx = tid; idx < 3 * G; idx += nthr) {
          const int kind = idx < G ? 0 : (idx < 2 * G ? 1 : 2), r = idx - kind * G;
          const int j = divHP.div(r), i = r - j * HP;
          const int x = hx0 + i, y = hy0 + j;
          if (kind == 0) {  // E_x at (x, y+1/2, t+1/2)
            if (i < 1 || i > tx || j > ty) continue;
            if (!inr(x, S + 1, m0 - S - 1) || !inr(y, S, m1 - S - 1) ||
                !inr(t, S, m2 - S - 1))
              continue;
            s_ex[(t & 1) * G + r] = edge_emf<R>(
                yf0[S_BJ * G + r], yf1[S_BJ * G + r], zf[S_BK * G + r],
                zf[S_BK * G + r + HP], upw(yf0[r]), upw(yf1[r]), upw(zf[r]),
                upw(zf[r + HP]), ec0[r], ec0[r + HP], ec1[r], ec1[r + HP]);
          } else if (kind == 1) {  // E_y at (x+1/2, y, t+1/2)
            if (i > tx || j < 1 || j > ty) continue;
            if (!inr(x, S, m0 - S - 1) || !inr(y, S + 1, m1 - S - 1) ||
                !inr(t, S, m2 - S - 1))
              continue;
            s_ey[(t & 1) * G + r] = edge_emf<R>(
                zf[S_BJ * G + r], zf[S_BJ * G + r + 1], xf0[S_BK * G + r],
                xf1[S_BK * G + r], upw(zf[r]), upw(zf[r + 1]), upw(xf0[r]),
                upw(xf1[r]), ec0[G + r], ec1[G + r], ec0[G + r + 1],
                ec1[G + r + 1]);
          } else {  // E_z at (x+1/2, y+1/2, t)
            if (i > tx || j > ty) continue;
            if (!inr(x, S, m0 - S - 1) || !inr(y, S, m1 - S - 1) ||
                !inr(t, S + 1, m2 - S - 1))
              continue;
            s_ez[r] = edge_emf<R>(
                xf0[S_BJ * G + r], xf0[S_BJ * G + r + HP], yf0[S_BK * G + r],
                yf0[S_BK * G + r + 1], upw(xf0[r]), upw(xf0[r + HP]),
                upw(yf0[r]), upw(yf0[r + 1]), ec0[2 * G + r],
                ec0[2 * G + r + 1], ec0[2 * G + r + HP], ec0[2 * G + r + HP + 1]);
          }
        }
        __syncthreads();
      }
      // ---- D: per column (x, y) of the tile, the constrained-transport
      // face updates it needs (EnzoBfieldMethodCT.cpp:617-687) -- Bz at the
      // face t+1 above it and, when plane t is output, Bx at faces x, x+1 and
      // By at faces y, y+1 of plane t -- then the update of cell (x, y, t).
      // A face between two cells of the tile is computed by both (the same
      // expression) and written by the one that owns it: the cell on its high
      // side, or the cell below the block's outermost written face.  A face
      // not updated in this stage keeps its start-of-step value.  Bz at t+1
      // stays in shared memory for the same column's next plane, so the
      // mapping of columns to threads is the same for every plane.  The
      // primitives of plane t+1+LOOK are finished into the ring in the same
      // phase.
      {
        const bool do_plane = t >= za;
        // the lowest face of a chunk is written by the chunk below it
        const bool own_bz = t >= za || za == olo;
        const bool in_t = inr(t, S + 1, m2 - S - 1);
        // Bx at face kx of row y, plane t; rx: the halo index of face kx
        auto face_x = [&](int kx, int y, int rx, bool own) -> R {
          const size_t fi = (size_t)t * ((size_t)m1 * (m0 + 1)) + (size_t)y * (m0 + 1) + kx;
          if (!(inr(kx, S + 1, m0 - S) && inr(y, S + 1, m1 - S - 1) && in_t))
            return B.base.f[0][fi];
          // E_z at (kx-1/2, y -+ 1/2), E_y at (kx-1/2, t -+ 1/2)
          const int re = rx - 1;  // edge ex = kx - 1
          const R Ek_term = dtdx[1] * (s_ez[re] - s_ez[re - HP]);
          const R Ej_term = dtdx[2] * (s_ey[(t & 1) * G + re] - s_ey[((t - 1) & 1) * G + re]);
          const R v = B.base.f[0][fi] - Ek_term + Ej_term;
          if (own) B.out.f[0][fi] = v;
          return v;
        };
        // By at face ky of column x, plane t; ry: the halo index of face ky
        auto face_y = [&](int ky, int x, int ry, bool own) -> R {
          const size_t fi = (size_t)t * ((size_t)(m1 + 1) * m0) + (size_t)ky * m0 + x;
          if (!(inr(ky, S + 1, m1 - S) && inr(x, S + 1, m0 - S - 1) && in_t))
            return B.base.f[1][fi];
          // E_x at (x, ky-1/2, t -+ 1/2), E_z at (x -+ 1/2, ky-1/2)
          const int re = ry - HP;  // edge ey = ky - 1
          const R Ek_term = dtdx[2] * (s_ex[(t & 1) * G + re] - s_ex[((t - 1) & 1) * G + re]);
          const R Ej_term = dtdx[0] * (s_ez[re] - s_ez[re - 1]);
          const R v = B.base.f[1][fi] - Ek_term + Ej_term;
          if (own) B.out.f[1][fi] = v;
          return v;
        };
        const R* xf0 = s_xf + (size_t)(t & 1) * NF * G;
        const R* yf0 = s_yf + (size_t)(t & 1) * NF * G;
        const R* zfm = s_zf + (size_t)((t - 1) & 1) * NF * G;
        const R* zfp = s_zf + (size_t)(t & 1) * NF * G;
        const int slot = t % NRING;
        const FastDiv divT(tx);
        for (int idx = tid; idx < tx * ty; idx += nthr) {
          const int qy = divT.div(idx);
          const int x = xa + (idx - qy * tx), y = ya + qy;
          const int r = (y - hy0) * HP + (x - hx0);
          R bcx = R(0), bcy = R(0), bcz = R(0);
          if (MHD) {
            // Bz at face kz = t+1 of column (x, y)
            const int kz = t + 1;
            R bz_hi = R(0);
            if (kz <= m2) {
              const size_t fi = (size_t)kz * cstr_z + (size_t)y * cstr_y + x;
              const bool upd = inr(kz, S + 1, m2 - S) && inr(x, S + 1, m0 - S - 1) &&
                               inr(y, S + 1, m1 - S - 1);
              if (upd) {
                const R Ek_term = dtdx[0] * (s_ey[(t & 1) * G + r] - s_ey[(t & 1) * G + r - 1]);
                const R Ej_term = dtdx[1] * (s_ex[(t & 1) * G + r] - s_ex[(t & 1) * G + r - HP]);
                bz_hi = B.base.f[2][fi] - Ek_term + Ej_term;
                if (own_bz) B.out.f[2][fi] = bz_hi;
              } else {
                bz_hi = B.base.f[2][fi];
              }
            }
            const R bz_lo = s_bz[(t & 1) * G + r];  // face t, from the previous plane
            s_bz[((t + 1) & 1) * G + r] = bz_hi;
            if (do_plane) {
              // compute_center_bfield (EnzoBfieldMethodCT.cpp:702-728)
              const R bx_lo = face_x(x, y, r, true);
              const R bx_hi = face_x(x + 1, y, r + 1, x + 1 == xb && xb == ohi_x);
              const R by_lo = face_y(y, x, r, true);
              const R by_hi = face_y(y + 1, x, r + HP, y + 1 == yb && yb == ohi_y);
              bcx = R(0.5) * (bx_lo + bx_hi);
              bcy = R(0.5) * (by_lo + by_hi);
              bcz = R(0.5) * (bz_lo + bz_hi);
            }
          }
          if (!do_plane) continue;
          const size_t c = (size_t)t * cstr_z + (size_t)y * cstr_y + x;
          if (MHD) {
            B.out.c[F_BX][c] = bcx;
            B.out.c[F_BY][c] = bcy;
            B.out.c[F_BZ][c] = bcz;
          }
          if (!inr(x, S + 1, m0 - S - 1) || !inr(y, S + 1, m1 - S - 1) ||
              !inr(t, S + 1, m2 - S - 1))
            continue;
          // flux divergence, x then y then z
          // (EnzoIntegrationQuanUpdate.cpp:105-147, EnzoSourceInternalEnergy.cpp:16-92)
          R du[6];
#pragma unroll
          for (int k = 0; k < 5; k++) {
            R a = R(0.0);
            a -= dtdx[0] * (xf0[k * G + r] - xf0[k * G + r - 1]);
            a -= dtdx[1] * (yf0[k * G + r] - yf0[k * G + r - HP]);
            a -= dtdx[2] * (zfp[k * G + r] - zfm[k * G + r]);
            du[k] = a;
          }
          if (DE) {
            const R p = smax(s_prim[poff(slot, x, y) + Q_P * PQ], pfloor);
            R a = R(0.0);
            a -= dtdx[0] * (xf0[S_EINT * G + r] - xf0[S_EINT * G + r - 1]);
            a -= dtdx[0] * p * (xf0[S_VBAR * G + r] - xf0[S_VBAR * G + r - 1]);
            a -= dtdx[1] * (yf0[S_EINT * G + r] - yf0[S_EINT * G + r - HP]);
            a -= dtdx[1] * p * (yf0[S_VBAR * G + r] - yf0[S_VBAR * G + r - HP]);
            a -= dtdx[2] * (zfp[S_EINT * G + r] - zfm[S_EINT * G + r]);
            a -= dtdx[2] * p * (zfp[S_VBAR * G + r] - zfm[S_VBAR * G + r]);
            du[5] = a;
          }
          // gravity source on the full-dt stage (EnzoSourceGravity.cpp:17-69,
          // EnzoMHDIntegratorStageCommands.cpp:267-297): start-of-step
          // density and velocity
          if (EXTRA == EXTRA_ALL && info.gravity) {
            const R dt = s_dt;
            const R rho0 = B.base.c[F_RHO][c];
            const R ax = B.accel[0][c], ay = B.accel[1][c], az = B.accel[2][c];
            du[1] += dt * rho0 * ax;
            du[2] += dt * rho0 * ay;
            du[3] += dt * rho0 * az;
            du[4] += dt * rho0 * ((B.base.c[F_VX][c] * ax) + (B.base.c[F_VY][c] * ay) +
                                  (B.base.c[F_VZ][c] * az));
          }
          // update_quantities (EnzoIntegrationQuanUpdate.cpp:183-231)
          const R old_rho = B.base.c[F_RHO][c];
          R new_rho = old_rho + du[0];
          new_rho = smax(new_rho, dfloor);
          const R inv_new_rho = R(1.) / new_rho;
          R vx = (B.base.c[F_VX][c] * old_rho + du[1]) * inv_new_rho;
          R vy = (B.base.c[F_VY][c] * old_rho + du[2]) * inv_new_rho;
          R vz = (B.base.c[F_VZ][c] * old_rho + du[3]) * inv_new_rho;
          R etot = (B.base.c[F_ETOT][c] * old_rho + du[4]) * inv_new_rho;
          R eint = R(0);
          if (DE) eint = (B.base.c[F_EINT][c] * old_rho + du[5]) * inv_new_rho;
          // apply_floor_to_energy_and_sync (EnzoPhysicsFluidProps.cpp:162-290)
          energy_floor_sync<MHD, DE>(econ, new_rho, vx, vy, vz, bcx, bcy, bcz, etot,
                                     eint);
          B.out.c[F_RHO][c] = new_rho;
          B.out.c[F_VX][c] = vx;
          B.out.c[F_VY][c] = vy;
          B.out.c[F_VZ][c] = vz;
          B.out.c[F_ETOT][c] = etot;
          if (DE) B.out.c[F_EINT][c] = eint;
          // the passive scalars' advection (passive_kernel) needs the
          // density flux of both faces of every updated cell along each
          // axis: the low faces here, the high faces at the region's edges
          if (EXTRA == EXTRA_ALL && info.npass > 0) {
            R* const* D = B.dflux;
            D[0][c] = xf0[S_RHO * G + r - 1];
            D[1][c] = yf0[S_RHO * G + r - HP];
            D[2][c] = zfm[S_RHO * G + r];
            if (x + 1 == m0 - S - 1) D[0][c + 1] = xf0[S_RHO * G + r];
            if (y + 1 == m1 - S - 1) D[1][c + cstr_y] = yf0[S_RHO * G + r];
            if (t + 1 == m2 - S - 1) D[2][c + cstr_z] = zfp[S_RHO * G + r];
          }
        }
      }
      if (t + 1 < zb) finish_plane(t + 1 + LOOK);
      __syncthreads();
    }
    // next tile: dynamic queue (persistent grid) or static grid stride
    if (info.queue) {
      if (tid == 0) s_next = atomicAdd(info.queue, 1);
      __syncthreads();
      it = s_next;
      __syncthreads();
    } else {
      it += gridDim.x;
    }
  }
}

}  // namespace vlct
