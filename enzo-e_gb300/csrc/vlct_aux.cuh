// vlct_aux.cuh -- the kernels around the fused stages: the CFL timestep
// reduction, the same-level ghost refresh gather, the FP64 conserved-total /
// div B diagnostics and small copy helpers.
#pragma once
#include <type_traits>

#include "vlct_energy.cuh"
#include "vlct_physics.cuh"
#include "vlct_types.h"

namespace vlct {

// A block as seen by the timestep and refresh kernels.
template <class R> struct AuxBlock {
  int m[3];
  double cw[3];
  FieldSet<R> f;     // fields (cell + face)
  R* pressure;       // optional [w] pressure field
  R* pass[4] = {nullptr, nullptr, nullptr, nullptr};  // passive scalars
  R* accel[3] = {nullptr, nullptr, nullptr};          // acceleration_x/y/z
};

// ---------------------------------------------------------------------------
// Timestep (EnzoMethodMHDVlct::timestep, EnzoMethodMHDVlct.cpp:551-588, and
// EnzoMHDIntegratorStageCommands::timestep, .cpp:299-366).  Per cell:
//   dual energy on: energy floor + sync (mutates etot/eint over the whole block)
//   p from the integration quantities (written to the pressure field if given)
//   s_d = |v_d| + c_fast  (c_fast = sqrt(B^2/rho + gamma p/rho))
// and the kernel reduces max_cells s_d per block and axis.  Because a
// correctly rounded division is monotone,
//   min_cells min_d dx_d / s_d  ==  min_d dx_d / max_cells s_d
// exactly, so the finishing kernel reproduces the reference's dt bit for bit.
// Speeds are non-negative, so their IEEE bit patterns order like unsigned
// integers and atomicMax on the bits is an exact max.
// ---------------------------------------------------------------------------
template <class R> struct SpeedBits;
template <> struct SpeedBits<double> {
  typedef unsigned long long T;
  static __device__ T bits(double v) { return (T)__double_as_longlong(v); }
  static __device__ double val(T b) { return __longlong_as_double((long long)b); }
};
template <> struct SpeedBits<float> {
  typedef unsigned int T;
  static __device__ T bits(float v) { return (T)__float_as_uint(v); }
  static __device__ float val(T b) { return __uint_as_float(b); }
};

template <class R, bool MHD, bool DE>
__global__ void __launch_bounds__(256)
timestep_kernel(const AuxBlock<R>* __restrict__ blocks, int nblocks,
                int chunks_per_block, PhysParams phys,
                typename SpeedBits<R>::T* __restrict__ smax_out) {
  typedef typename SpeedBits<R>::T T;
  __shared__ T red[3][8];
  const int b = blockIdx.x / chunks_per_block;
  const int chunk = blockIdx.x - b * chunks_per_block;
  if (b >= nblocks) return;
  const AuxBlock<R>& B = blocks[b];
  const size_t ncell = (size_t)B.m[0] * B.m[1] * B.m[2];
  const R g = R(phys.gamma);
  EnergyConsts<R> econ;
  econ.init(phys, DE);
  R s[3] = {R(0), R(0), R(0)};
  // the block's field pointers in registers: the descriptor lives in global
  // memory, and the stores below would otherwise force a reload per cell
  // (distinct arrays: restrict lets the loads of later cells move ahead of
  // the stores of earlier ones)
  const R* __restrict__ const f_rho = B.f.c[F_RHO];
  const R* __restrict__ const f_vx = B.f.c[F_VX];
  const R* __restrict__ const f_vy = B.f.c[F_VY];
  const R* __restrict__ const f_vz = B.f.c[F_VZ];
  const R* __restrict__ const f_bx = B.f.c[F_BX];
  const R* __restrict__ const f_by = B.f.c[F_BY];
  const R* __restrict__ const f_bz = B.f.c[F_BZ];
  R* __restrict__ const f_etot = B.f.c[F_ETOT];
  R* __restrict__ const f_eint = B.f.c[F_EINT];
  R* __restrict__ const f_p = B.pressure;
  // U cells per thread per pass, every load of the pass issued before the
  // arithmetic (the pass's stores would otherwise hold later loads back)
  constexpr int U = 4;
  const size_t stride = (size_t)chunks_per_block * blockDim.x;
  for (size_t c0 = (size_t)chunk * blockDim.x + threadIdx.x; c0 < ncell; c0 += U * stride) {
    R rho[U], vx[U], vy[U], vz[U], bx[U], by[U], bz[U], et[U], ei[U];
#pragma unroll
    for (int u = 0; u < U; u++) {
      const size_t c = c0 + u * stride;
      const bool ok = c < ncell;
      const size_t cc = ok ? c : c0;  // a valid index; the result is unused
      rho[u] = f_rho[cc];
      vx[u] = f_vx[cc];
      vy[u] = f_vy[cc];
      vz[u] = f_vz[cc];
      bx[u] = by[u] = bz[u] = R(0);
      if (MHD) {
        bx[u] = f_bx[cc];
        by[u] = f_by[cc];
        bz[u] = f_bz[cc];
      }
      et[u] = f_etot[cc];
      ei[u] = DE ? f_eint[cc] : R(0);
    }
#pragma unroll
    for (int u = 0; u < U; u++) {
      const size_t c = c0 + u * stride;
      if (c >= ncell) break;
      R p;
      if (DE) {
        // apply_floor_to_energy_and_sync over the whole block (stale depth 0)
        R etot = et[u], eint = ei[u];
        energy_floor_sync<MHD, true>(econ, rho[u], vx[u], vy[u], vz[u], bx[u], by[u], bz[u],
                                     etot, eint);
        f_eint[c] = eint;
        f_etot[c] = etot;
        p = econ.gm1 * rho[u] * eint;
      } else {
        p = pressure_from_etot<R, MHD>(econ, rho[u], et[u], vx[u], vy[u], vz[u], bx[u], by[u],
                                       bz[u]);
      }
      if (f_p) f_p[c] = p;
      R cf;
      if (MHD) {  // fast_magnetosonic_speed<0> (EnzoEOSIdeal.hpp:124-126)
        const R B2 = sqmag(bx[u], by[u], bz[u]);
        const R c2 = cs2(g, rho[u], p);
        const R va2 = B2 / rho[u];
        cf = sqrt(va2 + c2);
      } else {
        cf = sqrt(cs2(g, rho[u], p));
      }
      s[0] = fmax(s[0], fabs(vx[u]) + cf);
      s[1] = fmax(s[1], fabs(vy[u]) + cf);
      s[2] = fmax(s[2], fabs(vz[u]) + cf);
    }
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int d = 0; d < 3; d++) {
    T v = SpeedBits<R>::bits(s[d]);
    for (int o = 16; o > 0; o >>= 1) {
      T w = __shfl_xor_sync(0xffffffffu, v, o);
      v = (w > v) ? w : v;
    }
    if (lane == 0) red[d][warp] = v;
  }
  __syncthreads();
  if (threadIdx.x < 3) {
    const int d = threadIdx.x;
    T v = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) v = (red[d][w] > v) ? red[d][w] : v;
    atomicMax(&smax_out[3 * b + d], v);
  }
}

// dt_block = courant * min_d dx_d / max s_d; optionally the global minimum
// (the Cello CkReduction::min_double, src/Cello/control_stopping.cpp:66-135)
// is written to every block's slot.
template <class R>
__global__ void timestep_finish_kernel(const AuxBlock<R>* __restrict__ blocks,
                                       int nblocks,
                                       const typename SpeedBits<R>::T* smax_in,
                                       double courant, int global_min,
                                       double* dt_out, double* dt_min_out) {
  __shared__ double red[32];
  double local = 1.7976931348623157e308;
  for (int b = threadIdx.x; b < nblocks; b += blockDim.x) {
    const AuxBlock<R>& B = blocks[b];
    const double sx = (double)SpeedBits<R>::val(smax_in[3 * b + 0]);
    const double sy = (double)SpeedBits<R>::val(smax_in[3 * b + 1]);
    const double sz = (double)SpeedBits<R>::val(smax_in[3 * b + 2]);
    const double dt = min3(B.cw[0] / sx, B.cw[1] / sy, B.cw[2] / sz) * courant;
    dt_out[b] = dt;
    local = smin(local, dt);
  }
  for (int o = 16; o > 0; o >>= 1) local = fmin(local, __shfl_xor_sync(0xffffffffu, local, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = local;
  __syncthreads();
  if (threadIdx.x == 0) {
    double v = red[0];
    for (int w = 1; w < (int)(blockDim.x >> 5); w++) v = fmin(v, red[w]);
    if (dt_min_out) *dt_min_out = v;
    red[0] = v;
  }
  __syncthreads();
  if (global_min) {
    const double v = red[0];
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x) dt_out[b] = v;
  }
}

// ---------------------------------------------------------------------------
// Same-level ghost refresh (src/Cello/control_refresh.cpp:243-360,
// data_FieldFace.cpp:439-520, mesh_Box.cpp:150-206).  For every ghost element
// the source along each axis is: cell-centred axis, index c < g -> c + n from
// the low neighbour, c >= g + n -> c - n from the high neighbour; face-centred
// axis, k < g -> k + n, k > g + n -> k - n, and the block's own boundary faces
// (k = g, g + n) are never overwritten.  nbr[27 * b + (sz+1)*9 + (sy+1)*3 +
// (sx+1)] is the block that supplies offset (sx, sy, sz) of block b.
// The kernel enumerates only the ghost shell of each field.
// ---------------------------------------------------------------------------
template <class R>
__global__ void __launch_bounds__(256)
refresh_kernel(const AuxBlock<R>* __restrict__ blocks, const int* __restrict__ nbr,
               int nblocks, int g, int nfield_slots, int chunks_per_block) {
  const int b = blockIdx.x / chunks_per_block;
  const int chunk = blockIdx.x - b * chunks_per_block;
  if (b >= nblocks) return;
  const AuxBlock<R>& B = blocks[b];
  const int n[3] = {B.m[0] - 2 * g, B.m[1] - 2 * g, B.m[2] - 2 * g};
  for (int fs = 0; fs < nfield_slots; fs++) {
    // slots 0..8 cell fields, 9..11 face fields, 12 the pressure field,
    // 13..16 passive scalars, 17..19 the acceleration (Cello refreshes every field,
    // EnzoMethodMHDVlct.cpp:146-151)
    auto slot_ptr = [&](const AuxBlock<R>& X) -> R* {
      if (fs < NCELL) return X.f.c[fs];
      if (fs < NCELL + 3) return X.f.f[fs - NCELL];
      if (fs == NCELL + 3) return X.pressure;
      if (fs < NCELL + 8) return X.pass[fs - NCELL - 4];
      return X.accel[fs - NCELL - 8];
    };
    R* dst = slot_ptr(B);
    if (!dst) continue;
    const int face = (fs >= NCELL && fs < NCELL + 3) ? fs - NCELL : -1;
    int e[3], lo[3], hi[3];
    for (int a = 0; a < 3; a++) {
      e[a] = B.m[a] + (a == face);
      lo[a] = g;
      hi[a] = (a == face) ? g + n[a] + 1 : g + n[a];
    }
    // ghost shell = z-slabs, then y-slabs of the interior z range, then the
    // x-ends of the interior rows (32-bit index arithmetic: a block field has
    // far fewer than 2^31 elements)
    const int wz = e[2] - (hi[2] - lo[2]), wy = e[1] - (hi[1] - lo[1]),
              wx = e[0] - (hi[0] - lo[0]);
    const int iz = hi[2] - lo[2], iy = hi[1] - lo[1];
    const int cz = wz * e[1] * e[0];
    const int cy = iz * wy * e[0];
    const int cx = iz * iy * wx;
    const int total = cz + cy + cx;
    for (int q = chunk * blockDim.x + threadIdx.x; q < total;
         q += chunks_per_block * blockDim.x) {
      int x, y, z;
      if (q < cz) {
        int r = q;
        x = r % e[0]; r /= e[0];
        y = r % e[1]; r /= e[1];
        z = (r < lo[2]) ? r : r + iz;
      } else if (q < cz + cy) {
        int r = q - cz;
        x = r % e[0]; r /= e[0];
        const int yy = r % wy; r /= wy;
        y = (yy < lo[1]) ? yy : yy + iy;
        z = lo[2] + r;
      } else {
        int r = q - cz - cy;
        const int xx = r % wx; r /= wx;
        x = (xx < lo[0]) ? xx : xx + (hi[0] - lo[0]);
        y = lo[1] + r % iy; r /= iy;
        z = lo[2] + r;
      }
      int idx[3] = {x, y, z}, src[3], side[3];
      for (int a = 0; a < 3; a++) {
        const int i = idx[a];
        if (a == face) {
          if (i < g) { side[a] = -1; src[a] = i + n[a]; }
          else if (i > g + n[a]) { side[a] = 1; src[a] = i - n[a]; }
          else { side[a] = 0; src[a] = i; }
        } else {
          if (i < g) { side[a] = -1; src[a] = i + n[a]; }
          else if (i >= g + n[a]) { side[a] = 1; src[a] = i - n[a]; }
          else { side[a] = 0; src[a] = i; }
        }
      }
      const int sb = nbr[27 * b + (side[2] + 1) * 9 + (side[1] + 1) * 3 + (side[0] + 1)];
      const AuxBlock<R>& SB = blocks[sb];
      const R* sp = slot_ptr(SB);
      dst[((size_t)z * e[1] + y) * e[0] + x] = sp[((size_t)src[2] * e[1] + src[1]) * e[0] + src[0]];
    }
  }
}

// The same refresh, cell-major: a thread decodes one ghost-shell position
// once and copies every cell-centred field of the block there (the fields'
// source arrays for all 27 neighbour offsets staged in shared memory once
// per CTA), then the face-centred fields follow over their own shells.  The
// copies are the same as refresh_kernel's element for element (every source
// is an active cell of its block, so the order of the copies is free).  The
// shell decode divides by a multiply-high with ceil(2^32 / d), exact while
// every numerator times divisor stays below 2^32, which the host checks
// (blocks up to ~250 cells per side with 3 ghost layers); larger blocks use
// refresh_kernel.
template <class R>
__global__ void __launch_bounds__(256)
refresh_shell_kernel(const AuxBlock<R>* __restrict__ blocks, const int* __restrict__ nbr,
                     int nblocks, int g, int chunks_per_block) {
  // cell-centred slots: the 9 cell fields, the pressure field, 4 passive
  // scalars, 3 acceleration components
  constexpr int NC = NCELL + 8;
  __shared__ R* s_src[NC][27];
  __shared__ R* s_dst[NC];
  __shared__ R* s_fsrc[3][27];
  __shared__ R* s_fdst[3];
  __shared__ int s_slot[NC];
  __shared__ int s_nc;
  const int b = blockIdx.x / chunks_per_block;
  const int chunk = blockIdx.x - b * chunks_per_block;
  if (b >= nblocks) return;
  const AuxBlock<R>& B = blocks[b];
  auto cell_slot = [](const AuxBlock<R>& X, int fs) -> R* {
    if (fs < NCELL) return X.f.c[fs];
    if (fs == NCELL) return X.pressure;
    if (fs < NCELL + 5) return X.pass[fs - NCELL - 1];
    return X.accel[fs - NCELL - 5];
  };
  if (threadIdx.x == 0) {
    int k = 0;
    for (int fs = 0; fs < NC; fs++)
      if (cell_slot(B, fs)) s_slot[k++] = fs;
    s_nc = k;
  }
  __syncthreads();
  const int nc = s_nc;
  for (int i = threadIdx.x; i < nc * 27; i += blockDim.x) {
    const int j = i / 27, k = i - 27 * j;
    s_src[j][k] = cell_slot(blocks[nbr[27 * b + k]], s_slot[j]);
  }
  for (int j = threadIdx.x; j < nc; j += blockDim.x) s_dst[j] = cell_slot(B, s_slot[j]);
  for (int i = threadIdx.x; i < 81; i += blockDim.x) {
    const int d = i / 27, k = i - 27 * d;
    s_fsrc[d][k] = B.f.f[d] ? blocks[nbr[27 * b + k]].f.f[d] : nullptr;
    if (k == 0) s_fdst[d] = B.f.f[d];
  }
  __syncthreads();
  const int n[3] = {B.m[0] - 2 * g, B.m[1] - 2 * g, B.m[2] - 2 * g};
  auto magic = [](unsigned d) -> unsigned { return d > 1 ? 0xFFFFFFFFu / d + 1u : 0u; };
  auto mdiv = [](int v, unsigned d, unsigned m) -> int {
    return d > 1 ? (int)__umulhi((unsigned)v, m) : v;
  };
  // Pass 1: the cell shell -- z-slabs, then y-slabs, then the x-ends.  Each
  // ghost cell copies every cell field and, with face-centred B, the face
  // values on its low side along each axis (bfieldi_a at the cell's index),
  // so one position decode serves up to 12 fields.  Face index g + n along
  // its own axis is the block's own boundary face: along that axis it sits
  // "inside" (neighbour offset 0), and it is skipped when it is inside along
  // every axis.  Pass 2 covers the face layers above the last cell
  // (bfieldi_a at index m along a).
  const int M[3] = {B.m[0], B.m[1], B.m[2]};
  const int HI[3] = {g + n[0], g + n[1], g + n[2]};
  const int wz = M[2] - n[2], wy = M[1] - n[1], wx = M[0] - n[0];
  const int iz = n[2], iy = n[1];
  const unsigned m0 = magic(M[0]), m1 = magic(M[1]), mwy = magic(wy), mwx = magic(wx),
                 miy = magic(iy);
  const int cz = wz * M[1] * M[0];
  const int cy = iz * wy * M[0];
  const int cx = iz * iy * wx;
  const int total = cz + cy + cx;
  const int stride = chunks_per_block * blockDim.x;
  const bool faces = s_fdst[0] != nullptr;  // MHD: all three, or none
  auto side_of = [&](int a, int i) { return (i < g) ? -1 : ((i >= HI[a]) ? 1 : 0); };
  auto slot_of = [](const int* sd) { return (sd[2] + 1) * 9 + (sd[1] + 1) * 3 + (sd[0] + 1); };
  // index of (x, y, z) in the face array of axis a
  auto face_index = [&](int a, const int* i) -> size_t {
    const int e0 = M[0] + (a == 0), e1 = M[1] + (a == 1);
    return ((size_t)i[2] * e1 + i[1]) * e0 + i[0];
  };
  auto copy_shell = [&](auto count, auto with_faces) {
    constexpr int N = decltype(count)::value;
    constexpr bool F = decltype(with_faces)::value;
    for (int q = chunk * blockDim.x + threadIdx.x; q < total; q += stride) {
      int idx[3];
      if (q < cz) {
        const int r1 = mdiv(q, M[0], m0);
        idx[0] = q - r1 * M[0];
        const int r2 = mdiv(r1, M[1], m1);
        idx[1] = r1 - r2 * M[1];
        idx[2] = (r2 < g) ? r2 : r2 + iz;
      } else if (q < cz + cy) {
        const int r0 = q - cz;
        const int r1 = mdiv(r0, M[0], m0);
        idx[0] = r0 - r1 * M[0];
        const int r2 = mdiv(r1, wy, mwy);
        const int yy = r1 - r2 * wy;
        idx[1] = (yy < g) ? yy : yy + iy;
        idx[2] = g + r2;
      } else {
        const int r0 = q - cz - cy;
        const int r1 = mdiv(r0, wx, mwx);
        const int xx = r0 - r1 * wx;
        idx[0] = (xx < g) ? xx : xx + n[0];
        const int r2 = mdiv(r1, iy, miy);
        idx[1] = g + (r1 - r2 * iy);
        idx[2] = g + r2;
      }
      int side[3], src[3];
#pragma unroll
      for (int a = 0; a < 3; a++) {
        side[a] = side_of(a, idx[a]);
        src[a] = idx[a] - side[a] * n[a];
      }
      const int k = slot_of(side);
      const size_t di = ((size_t)idx[2] * M[1] + idx[1]) * M[0] + idx[0];
      const size_t si = ((size_t)src[2] * M[1] + src[1]) * M[0] + src[0];
      // all loads of the cell before any store (through the pointer tables
      // the compiler cannot rule out aliasing, and would otherwise wait out
      // one memory round trip per field)
      R v[N];
#pragma unroll
      for (int j = 0; j < N; j++) v[j] = s_src[j][k][si];
      R fv[3];
      size_t fdi[3];
      bool fon[3] = {false, false, false};
      if (F) {
#pragma unroll
        for (int a = 0; a < 3; a++) {
          int fs[3] = {side[0], side[1], side[2]};
          if (idx[a] == HI[a]) fs[a] = 0;  // the face at g + n along a
          if (fs[0] == 0 && fs[1] == 0 && fs[2] == 0) continue;
          const int fsrc[3] = {idx[0] - fs[0] * n[0], idx[1] - fs[1] * n[1],
                               idx[2] - fs[2] * n[2]};
          fon[a] = true;
          fdi[a] = face_index(a, idx);
          fv[a] = s_fsrc[a][slot_of(fs)][face_index(a, fsrc)];
        }
      }
#pragma unroll
      for (int j = 0; j < N; j++) s_dst[j][di] = v[j];
      if (F) {
#pragma unroll
        for (int a = 0; a < 3; a++)
          if (fon[a]) s_fdst[a][fdi[a]] = fv[a];
      }
    }
  };
  auto dispatch = [&](auto with_faces) {
    switch (nc) {
      case 1: copy_shell(std::integral_constant<int, 1>{}, with_faces); break;
      case 2: copy_shell(std::integral_constant<int, 2>{}, with_faces); break;
      case 3: copy_shell(std::integral_constant<int, 3>{}, with_faces); break;
      case 4: copy_shell(std::integral_constant<int, 4>{}, with_faces); break;
      case 5: copy_shell(std::integral_constant<int, 5>{}, with_faces); break;
      case 6: copy_shell(std::integral_constant<int, 6>{}, with_faces); break;
      case 7: copy_shell(std::integral_constant<int, 7>{}, with_faces); break;
      case 8: copy_shell(std::integral_constant<int, 8>{}, with_faces); break;
      case 9: copy_shell(std::integral_constant<int, 9>{}, with_faces); break;
      case 10: copy_shell(std::integral_constant<int, 10>{}, with_faces); break;
      case 11: copy_shell(std::integral_constant<int, 11>{}, with_faces); break;
      case 12: copy_shell(std::integral_constant<int, 12>{}, with_faces); break;
      case 13: copy_shell(std::integral_constant<int, 13>{}, with_faces); break;
      case 14: copy_shell(std::integral_constant<int, 14>{}, with_faces); break;
      case 15: copy_shell(std::integral_constant<int, 15>{}, with_faces); break;
      case 16: copy_shell(std::integral_constant<int, 16>{}, with_faces); break;
      default: copy_shell(std::integral_constant<int, NC>{}, with_faces); break;
    }
  };
  if (faces)
    dispatch(std::integral_constant<bool, true>{});
  else
    dispatch(std::integral_constant<bool, false>{});
  if (!faces) return;
  // Pass 2: bfieldi_a at index m along a (above the last cell), every
  // position across; neighbour offset +1 along a
  for (int a = 0; a < 3; a++) {
    const int b0 = a == 0 ? 1 : 0, b1 = a == 2 ? 1 : 2;  // the other axes, inner first
    const int layer = M[b0] * M[b1];
    const unsigned mb = magic(M[b0]);
    constexpr int U = 4;
    for (int q0 = chunk * blockDim.x + threadIdx.x; q0 < layer; q0 += U * stride) {
      size_t fdi[U];
      R fv[U];
#pragma unroll
      for (int u = 0; u < U; u++) {
        const int q = q0 + u * stride;
        if (q >= layer) continue;
        const int r = mdiv(q, M[b0], mb);
        int idx[3];
        idx[a] = M[a];
        idx[b0] = q - r * M[b0];
        idx[b1] = r;
        int fs[3];
        fs[a] = 1;
        fs[b0] = side_of(b0, idx[b0]);
        fs[b1] = side_of(b1, idx[b1]);
        const int fsrc[3] = {idx[0] - fs[0] * n[0], idx[1] - fs[1] * n[1],
                             idx[2] - fs[2] * n[2]};
        fdi[u] = face_index(a, idx);
        fv[u] = s_fsrc[a][slot_of(fs)][face_index(a, fsrc)];
      }
#pragma unroll
      for (int u = 0; u < U; u++)
        if (q0 + u * stride < layer) s_fdst[a][fdi[u]] = fv[u];
    }
  }
}

// Face-centred B from an edge-centred vector potential and the centred B
// (EnzoInitialBCenter::initialize_bfield_interface / bfieldi_helper_,
// src/Enzo/initial/EnzoInitialBCenter.cpp:41-127, then
// initialize_bfield_center, :27-38): in double, cast to the block's type,
//   Bx(k, j, i-1/2) = (Az(k, j+1/2) - Az(k, j-1/2)) / dy - (Ay(k+1/2, j) - Ay(k-1/2, j)) / dz
// and the cyclic permutations.  A_x has extents (m0, m1+1, m2+1) along
// (x, y, z), A_y (m0+1, m1, m2+1), A_z (m0+1, m1+1, m2), x fastest.
template <class R>
__global__ void bfield_from_potential_kernel(int m0, int m1, int m2, const double* ax,
                                             const double* ay, const double* az, double dx,
                                             double dy, double dz, R* bfx, R* bfy, R* bfz) {
  const size_t fx = (size_t)(m0 + 1) * m1 * m2, fy = (size_t)m0 * (m1 + 1) * m2,
               fz = (size_t)m0 * m1 * (m2 + 1);
  for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < fx + fy + fz;
       q += (size_t)gridDim.x * blockDim.x) {
    if (q < fx) {  // bfieldi_x (m2, m1, m0+1): Aj = Ay, Ak = Az, dj = dy, dk = dz
      const size_t r = q;
      const int i = (int)(r % (m0 + 1)), j = (int)((r / (m0 + 1)) % m1),
                k = (int)(r / ((size_t)(m0 + 1) * m1));
      const double akr = az[((size_t)k * (m1 + 1) + (j + 1)) * (m0 + 1) + i];
      const double akl = az[((size_t)k * (m1 + 1) + j) * (m0 + 1) + i];
      const double ajr = ay[((size_t)(k + 1) * m1 + j) * (m0 + 1) + i];
      const double ajl = ay[((size_t)k * m1 + j) * (m0 + 1) + i];
      bfx[r] = (R)(((akr - akl) / dy - (ajr - ajl) / dz));
    } else if (q < fx + fy) {  // bfieldi_y (m2, m1+1, m0): Aj = Az, Ak = Ax, dj = dz, dk = dx
      const size_t r = q - fx;
      const int i = (int)(r % m0), j = (int)((r / m0) % (m1 + 1)),
                k = (int)(r / ((size_t)m0 * (m1 + 1)));
      const double akr = ax[((size_t)(k + 1) * (m1 + 1) + j) * m0 + i];
      const double akl = ax[((size_t)k * (m1 + 1) + j) * m0 + i];
      const double ajr = az[((size_t)k * (m1 + 1) + j) * (m0 + 1) + (i + 1)];
      const double ajl = az[((size_t)k * (m1 + 1) + j) * (m0 + 1) + i];
      bfy[r] = (R)(((akr - akl) / dz - (ajr - ajl) / dx));
    } else {  // bfieldi_z (m2+1, m1, m0): Aj = Ax, Ak = Ay, dj = dx, dk = dy
      const size_t r = q - fx - fy;
      const int i = (int)(r % m0), j = (int)((r / m0) % m1), k = (int)(r / ((size_t)m0 * m1));
      const double akr = ay[((size_t)k * m1 + j) * (m0 + 1) + (i + 1)];
      const double akl = ay[((size_t)k * m1 + j) * (m0 + 1) + i];
      const double ajr = ax[((size_t)k * (m1 + 1) + (j + 1)) * m0 + i];
      const double ajl = ax[((size_t)k * (m1 + 1) + j) * m0 + i];
      bfz[r] = (R)(((akr - akl) / dx - (ajr - ajl) / dy));
    }
  }
}

// compute_center_bfield over the whole block (EnzoBfieldMethodCT.cpp:702-728)
template <class R>
__global__ void center_bfield_kernel(int m0, int m1, int m2, const R* bfx, const R* bfy,
                                     const R* bfz, R* bx, R* by, R* bz) {
  const size_t M = (size_t)m0 * m1 * m2;
  for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < M;
       c += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(c % m0), j = (int)((c / m0) % m1), k = (int)(c / ((size_t)m0 * m1));
    const size_t ix = ((size_t)k * m1 + j) * (m0 + 1) + i;
    const size_t iy = ((size_t)k * (m1 + 1) + j) * m0 + i;
    bx[c] = R(0.5) * (bfx[ix] + bfx[ix + 1]);
    by[c] = R(0.5) * (bfy[iy] + bfy[iy + m0]);
    bz[c] = R(0.5) * (bfz[c] + bfz[c + (size_t)m0 * m1]);
  }
}

// Copy the face-B box updated by the final stage (faces k in [lo, hi_d) along
// d, transverse [lo, hi)) from the stage's face buffer into the caller's field.
template <class R>
__global__ void copy_faces_kernel(int m0, int m1, int m2, int lo_t, int S1,
                                  const R* __restrict__ fx, const R* __restrict__ fy,
                                  const R* __restrict__ fz, R* __restrict__ ox,
                                  R* __restrict__ oy, R* __restrict__ oz) {
  const int m[3] = {m0, m1, m2};
  const R* src[3] = {fx, fy, fz};
  R* dst[3] = {ox, oy, oz};
  for (int d = 0; d < 3; d++) {
    int e[3] = {m0 + (d == 0), m1 + (d == 1), m2 + (d == 2)};
    int lo[3], cnt[3];
    for (int a = 0; a < 3; a++) {
      lo[a] = (a == d) ? S1 : lo_t;
      const int hi = (a == d) ? m[a] - S1 + 1 : m[a] - lo_t;
      cnt[a] = hi - lo[a];
    }
    const long long total = (long long)cnt[0] * cnt[1] * cnt[2];
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < total;
         q += (long long)gridDim.x * blockDim.x) {
      long long r = q;
      const int x = lo[0] + (int)(r % cnt[0]); r /= cnt[0];
      const int y = lo[1] + (int)(r % cnt[1]); r /= cnt[1];
      const int z = lo[2] + (int)r;
      const size_t i = ((size_t)z * e[1] + y) * e[0] + x;
      dst[d][i] = src[d][i];
    }
  }
}

static __global__ void set_scalar_kernel(double* p, double v) { *p = v; }

}  // namespace vlct

namespace vlct {

// ---------------------------------------------------------------------------
// Conserved totals and constraint diagnostics over the active zones of every
// block, accumulated in FP64 whatever the storage precision:
//   [0] mass  sum rho dV            [1..3] momentum  sum rho v_d dV
//   [4] energy sum rho e_tot dV     [5] sum rho e_int dV (dual energy)
//   [6] max |div B| (face B, per cell, 1/length units)
//   [7] max |B_cell|
// Each CTA reduces its share in a fixed order and writes one partial row; the
// finishing kernel adds the rows in a fixed order, so the totals are
// bit-reproducible run to run.
// ---------------------------------------------------------------------------
constexpr int NDIAG = 8;

__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
// max that keeps a NaN (a NaN in a diagnostic must not be hidden)
__device__ __forceinline__ double nan_max(double a, double b) {
  return (b > a || b != b) ? b : a;
}
__device__ __forceinline__ double warp_max(double v) {
  for (int o = 16; o > 0; o >>= 1) v = nan_max(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

template <class R>
__global__ void __launch_bounds__(256)
diag_kernel(const AuxBlock<R>* __restrict__ blocks, int nblocks, int g, int cpb,
            int mhd, int de, double* __restrict__ partial) {
  __shared__ double red[NDIAG][8];
  const int b = blockIdx.x / cpb;
  const int chunk = blockIdx.x - b * cpb;
  if (b >= nblocks) return;
  const AuxBlock<R>& B = blocks[b];
  const int m0 = B.m[0], m1 = B.m[1];
  const int n0 = B.m[0] - 2 * g, n1 = B.m[1] - 2 * g, n2 = B.m[2] - 2 * g;
  const size_t nact = (size_t)n0 * n1 * n2;
  double acc[NDIAG] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (size_t idx = (size_t)chunk * blockDim.x + threadIdx.x; idx < nact;
       idx += (size_t)cpb * blockDim.x) {
    const size_t row = idx / n0;
    const int x = (int)(idx - row * n0) + g;
    const int y = (int)(row % n1) + g;
    const int z = (int)(row / n1) + g;
    const size_t c = ((size_t)z * m1 + y) * m0 + x;
    const double rho = (double)B.f.c[F_RHO][c];
    acc[0] += rho;
    acc[1] += rho * (double)B.f.c[F_VX][c];
    acc[2] += rho * (double)B.f.c[F_VY][c];
    acc[3] += rho * (double)B.f.c[F_VZ][c];
    acc[4] += rho * (double)B.f.c[F_ETOT][c];
    if (de) acc[5] += rho * (double)B.f.c[F_EINT][c];
    if (mhd) {
      const R* fx = B.f.f[0];
      const R* fy = B.f.f[1];
      const R* fz = B.f.f[2];
      const size_t ix = ((size_t)z * m1 + y) * (m0 + 1) + x;
      const size_t iy = ((size_t)z * (m1 + 1) + y) * m0 + x;
      const size_t iz = c;
      const size_t sz = (size_t)m0 * m1;
      const double div = ((double)fx[ix + 1] - (double)fx[ix]) / B.cw[0] +
                         ((double)fy[iy + m0] - (double)fy[iy]) / B.cw[1] +
                         ((double)fz[iz + sz] - (double)fz[iz]) / B.cw[2];
      acc[6] = nan_max(acc[6], fabs(div));
      const double bx = B.f.c[F_BX][c], by = B.f.c[F_BY][c], bz = B.f.c[F_BZ][c];
      acc[7] = nan_max(acc[7], sqrt(bx * bx + by * by + bz * bz));
    }
  }
  const double dV = B.cw[0] * B.cw[1] * B.cw[2];
  for (int k = 0; k < 6; k++) acc[k] *= dV;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NDIAG; k++) {
    const double v = k < 6 ? warp_sum(acc[k]) : warp_max(acc[k]);
    if (lane == 0) red[k][warp] = v;
  }
  __syncthreads();
  if (threadIdx.x < NDIAG) {
    const int k = threadIdx.x;
    double v = red[k][0];
    for (int w = 1; w < (int)(blockDim.x >> 5); w++)
      v = k < 6 ? v + red[k][w] : nan_max(v, red[k][w]);
    partial[(size_t)blockIdx.x * NDIAG + k] = v;
  }
}

static __global__ void __launch_bounds__(256)
diag_finish_kernel(const double* __restrict__ partial, int nrows, double* __restrict__ out) {
  __shared__ double red[NDIAG][8];
  double acc[NDIAG] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (int r = threadIdx.x; r < nrows; r += blockDim.x)
#pragma unroll
    for (int k = 0; k < NDIAG; k++) {
      const double v = partial[(size_t)r * NDIAG + k];
      acc[k] = k < 6 ? acc[k] + v : nan_max(acc[k], v);
    }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NDIAG; k++) {
    const double v = k < 6 ? warp_sum(acc[k]) : warp_max(acc[k]);
    if (lane == 0) red[k][warp] = v;
  }
  __syncthreads();
  if (threadIdx.x < NDIAG) {
    const int k = threadIdx.x;
    double v = red[k][0];
    for (int w = 1; w < (int)(blockDim.x >> 5); w++)
      v = k < 6 ? v + red[k][w] : nan_max(v, red[k][w]);
    out[k] = v;
  }
}

}  // namespace vlct
