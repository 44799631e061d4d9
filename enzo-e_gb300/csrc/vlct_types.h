// vlct_types.h -- host/device descriptors shared by the kernels and the C ABI.
#pragma once
#include <stdint.h>

namespace vlct {

// Cell-centred integration quantities of one block, in Cello's layout
// (src/Cello/data_FieldData.cpp:585-619): (z, y, x), x fastest, ghosted
// extent m = n + 2g per axis.  Face field d has extent m_d + 1 along d.
enum CellField {
  F_RHO = 0, F_VX, F_VY, F_VZ, F_ETOT, F_EINT, F_BX, F_BY, F_BZ, NCELL
};

template <class R> struct FieldSet {
  R* c[NCELL];  // cell fields (F_EINT / F_B* may be null)
  R* f[3];      // face-centred B (null in hydro mode)
};

// One block as seen by a stage kernel.
template <class R> struct StageBlock {
  int m[3];              // ghosted extents along x, y, z
  double cw[3];          // cell widths
  const double* dt;      // device pointer to this block's full step dt
  FieldSet<R> cur;       // state the fluxes are computed from
  FieldSet<R> base;      // start-of-step state (U^n, face B^n)
  FieldSet<R> out;       // where the stage writes (out.f = new face B)
  const R* accel[3] = {nullptr, nullptr, nullptr};  // gravity source fields
  // passive scalars (conserved form): current-stage input, start of step,
  // output; the first StageInfo::npass entries are used
  const R* pass_cur[4] = {nullptr, nullptr, nullptr, nullptr};
  const R* pass_base[4] = {nullptr, nullptr, nullptr, nullptr};
  R* pass_out[4] = {nullptr, nullptr, nullptr, nullptr};
  // with passive scalars: per axis d, the density flux through the low
  // d-face of every cell the stage updates (and through the high face of the
  // last cell), written by the stage kernel for passive_kernel; cell-shaped
  // arrays of the ghosted block
  R* dflux[3] = {nullptr, nullptr, nullptr};
  // FluxOut<R> (device) of this block on the final stage when a batch stores
  // the boundary fluxes for flux correction; null otherwise
  const void* fc = nullptr;
};

// One unit of work: a column tile [xa, xb) x [ya, yb) of one block, whose
// output planes are [za, zb) (a z-chunk; za/zb span the whole output range
// when the block is not chunked).
struct StageTile {
  int block;
  int xa, xb, ya, yb, za, zb;
};

struct PhysParams {
  double gamma;
  double density_floor;
  double pressure_floor;
  double theta_limiter;
  double eta;
  // derived on the host (set_derived), so that no kernel thread spends FP64
  // divisions on them: gamma - 1, 1 / (gamma - 1), gamma (gamma - 1)
  double gm1 = 0.0, inv_gm1 = 0.0, ggm1 = 0.0;
  // the FP32 kernels' constants, each rounded once here from the double
  // above: read from the kernel parameters, they need no FP64 conversion on
  // the device (GB300's FP64 pipe is narrow)
  float gamma_f = 0.f, density_floor_f = 0.f, pressure_floor_f = 0.f;
  float theta_limiter_f = 0.f, eta_f = 0.f;
  float gm1_f = 0.f, inv_gm1_f = 0.f, ggm1_f = 0.f;
  void set_derived() {
    gm1 = gamma - 1.0;
    inv_gm1 = 1. / (gamma - 1.);
    ggm1 = gamma * (gamma - 1.);
    gamma_f = (float)gamma;
    density_floor_f = (float)density_floor;
    pressure_floor_f = (float)pressure_floor;
    theta_limiter_f = (float)theta_limiter;
    eta_f = (float)eta;
    gm1_f = (float)gm1;
    inv_gm1_f = (float)inv_gm1;
    ggm1_f = (float)ggm1;
  }
};

// Per-stage scalars.
struct StageInfo {
  int s;            // stale depth at stage start
  int S;            // stale depth after reconstruction (s + immediate rate)
  int final_stage;  // 1 on the last stage (writes layer S of centred B)
  double dt_factor; // 0.5 for the half step, 1 for the full step
  int tx, ty;       // maximum tile extent of the launch (sizes shared memory)
  int* queue;       // work counter (zeroed before the launch) for a persistent
                    // grid pulling tiles dynamically; null = static grid stride
  int threads;      // CTA size (256 or 512); 0 = 256
  int gravity = 0;           // 1: add the gravity source (the blocks' accel)
  int npass = 0;             // passive scalars advected (0..4)
  const void* fc = nullptr;  // FluxOut<R> (device) on the final stage when the
                             // boundary fluxes are stored; null otherwise
  int block_fc = 0;          // 1: the blocks carry their own FluxOut (StageBlock::fc)
  int fc_g = 0;              // ghost depth of the blocks whose fluxes are stored
  // shape of the launch, for the stage kernels compiled with it as constants
  // (zero: not known, the run-time shape is used)
  int full_tiles = 0;        // 1: every tile of the launch is tx x ty
  int block_m = 0;           // every block's extent (ghosts included) along all
                             // three axes, when they are all equal
};

// Boundary fluxes for flux correction (EnzoMethodMHDVlct.cpp:250-330):
// f[dim][side][q] receives dt/dx_dim times the flux of quantity q (0 density,
// 1-3 velocity x/y/z, 4 total energy, 5 internal energy, 6-9 passive
// scalars 0-3 in conserved form) through the low
// (side 0, face g-1) or high (side 1, face m-g-1) active face of axis dim,
// as an array of the active face, last index fastest: axis 0 (nz, ny),
// axis 1 (nz, nx), axis 2 (ny, nx).  Null pointers are skipped.
constexpr int kFluxQuantities = 10;  // MHD_FC_NQ of the C interface
template <class R> struct FluxOut {
  R* f[3][2][kFluxQuantities];  // [axis][side][MHD_Q_*]
  int g;
};

#ifdef __CUDACC__
// Division by a runtime divisor d > 0 by a multiply-high with ceil(2^32 / d):
// exact for every numerator n with n * d < 2^32 (m d = 2^32 + e, 0 < e <= d,
// so n m / 2^32 = n / d + n e / (d 2^32) and n e < 2^32).
struct FastDiv {
  unsigned d, m;
  // ceil(2^32 / d) == floor((2^32 - 1) / d) + 1 for every d > 1
  __device__ __forceinline__ explicit FastDiv(unsigned dd)
      : d(dd), m(dd > 1 ? 0xFFFFFFFFu / dd + 1u : 0u) {}
  __device__ __forceinline__ int div(int n) const {
    return d > 1 ? (int)__umulhi((unsigned)n, m) : n;
  }
};
#endif

}  // namespace vlct
