// vlct_energy.cuh -- the internal-energy recovery and the energy floor /
// dual-energy sync, in the precision each form needs.
//
// The recovery e_int = e_tot - |v|^2/2 - |B|^2/(2 rho) cancels when the flow
// is kinetically or magnetically dominated.  FP64 path: the reference's
// expressions in double, operation for operation.  FP32 path: the products
// and differences are carried in float-float (an unevaluated sum hi + lo of
// two floats, ~48-bit significand) with error-free transformations (Knuth's
// TwoSum, the FMA-based TwoProduct), so the recovery is as accurate as an
// FP64 evaluation of the same float inputs while running on the FP32 pipes
// (GB300's FP64 rate is 1/64 of its FP32 rate).  The result is rounded to
// float once.
// Reference: src/Enzo/fluid-props/EnzoComputePressure.cpp:127-190,
// EnzoPhysicsFluidProps.cpp:162-290.
#pragma once
#include <cuda_runtime.h>

#include "vlct_physics.cuh"
#include "vlct_types.h"

namespace vlct {

struct ff {
  float hi, lo;
};
__device__ __forceinline__ ff two_prod(float a, float b) {
  const float p = __fmul_rn(a, b);
  return {p, __fmaf_rn(a, b, -p)};
}
__device__ __forceinline__ ff two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}
__device__ __forceinline__ ff fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ ff ff_add(ff x, ff y) {
  const ff s = two_sum(x.hi, y.hi);
  return fast_two_sum(s.hi, __fadd_rn(__fadd_rn(s.lo, x.lo), y.lo));
}
__device__ __forceinline__ ff ff_neg(ff x) { return {-x.hi, -x.lo}; }
__device__ __forceinline__ ff ff_scale(ff x, float s) {  // s a power of two
  return {x.hi * s, x.lo * s};
}
__device__ __forceinline__ ff ff_mul(ff x, float b) {
  const ff p = two_prod(x.hi, b);
  return fast_two_sum(p.hi, __fmaf_rn(x.lo, b, p.lo));
}
__device__ __forceinline__ ff ff_div(ff x, float b) {
  const float q = __fdiv_rn(x.hi, b);
  const float r = __fadd_rn(__fmaf_rn(-q, b, x.hi), x.lo);
  return fast_two_sum(q, __fdiv_rn(r, b));
}
__device__ __forceinline__ ff ff_sqsum(float a, float b, float c) {
  return ff_add(ff_add(two_prod(a, a), two_prod(b, b)), two_prod(c, c));
}
__device__ __forceinline__ float ff_round(ff x) { return __fadd_rn(x.hi, x.lo); }

// Constants of the EOS / floors, evaluated once per kernel in the working
// precision (in FP64 they are the reference's expressions bit for bit).
template <class R> struct EnergyConsts {
  R gm1;          // gamma - 1
  R inv_gm1;      // 1 / (gamma - 1)
  float ggm1;     // gamma (gamma - 1), a float in the reference (:234)
  R pfloor;       // pressure floor
  R eta;          // dual-energy eta (0 when dual energy is off)
  R half_factor;  // 0.5 when eta != 0, else 0
  __host__ __device__ void init(double gamma, double pressure_floor, double eta_) {
    gm1 = R(gamma - 1.0);
    inv_gm1 = R(1. / (gamma - 1.));
    ggm1 = (float)(gamma * (gamma - 1.));
    pfloor = R(pressure_floor);
    eta = R(eta_);
    half_factor = (eta_ != 0.) ? R(0.5) : R(0.);
  }
  // FP32 only: the constants rounded on the host (PhysParams::set_derived),
  // the same values as init(gamma, pressure_floor, eta) gives
  __host__ __device__ void init_rounded(const PhysParams& ph, bool de) {
    gm1 = ph.gm1_f;
    inv_gm1 = ph.inv_gm1_f;
    ggm1 = ph.ggm1_f;
    pfloor = ph.pressure_floor_f;
    eta = de ? ph.eta_f : 0.f;
    half_factor = (de && ph.eta != 0.) ? 0.5f : 0.f;
  }
  // the same values from the host-derived constants of the physics
  // parameters, without the FP64 division: for kernels whose threads are
  // short-lived (the timestep), where it would be a noticeable share
  __host__ __device__ void init(const PhysParams& ph, bool de) {
    gm1 = R(ph.gm1);
    inv_gm1 = R(ph.inv_gm1);
    ggm1 = (float)ph.ggm1;
    pfloor = R(ph.pressure_floor);
    const double eta_ = de ? ph.eta : 0.0;
    eta = R(eta_);
    half_factor = (eta_ != 0.) ? R(0.5) : R(0.);
  }
};

// p = (gamma - 1) (rho (e_tot - |v|^2/2) - |B|^2/2)
template <class R, bool MHD>
__device__ __forceinline__ R pressure_from_etot(const EnergyConsts<R>& ec, R rho, R etot,
                                                R vx, R vy, R vz, R bx, R by, R bz);

template <>
__device__ __forceinline__ double pressure_from_etot<double, true>(
    const EnergyConsts<double>& ec, double rho, double etot, double vx, double vy,
    double vz, double bx, double by, double bz) {
  const double gm1 = ec.gm1;
  const double ke = 0.5 * (vx * vx + vy * vy + vz * vz);
  const double me = 0.5 * (bx * bx + by * by + bz * bz);
  return gm1 * (rho * (etot - ke) - me);
}
template <>
__device__ __forceinline__ double pressure_from_etot<double, false>(
    const EnergyConsts<double>& ec, double rho, double etot, double vx, double vy,
    double vz, double, double, double) {
  const double gm1 = ec.gm1;
  const double ke = 0.5 * (vx * vx + vy * vy + vz * vz);
  return gm1 * (rho * (etot - ke) - 0.);
}
template <bool MHD>
__device__ __forceinline__ float pressure_ff(float gm1, float rho, float etot,
                                             float vx, float vy, float vz, float bx,
                                             float by, float bz) {
  const ff ke = ff_scale(ff_sqsum(vx, vy, vz), 0.5f);
  ff d = ff_mul(ff_add({etot, 0.f}, ff_neg(ke)), rho);
  if (MHD) d = ff_add(d, ff_neg(ff_scale(ff_sqsum(bx, by, bz), 0.5f)));
  return gm1 * ff_round(d);
}
template <>
__device__ __forceinline__ float pressure_from_etot<float, true>(
    const EnergyConsts<float>& ec, float rho, float etot, float vx, float vy,
    float vz, float bx, float by, float bz) {
  return pressure_ff<true>(ec.gm1, rho, etot, vx, vy, vz, bx, by, bz);
}
template <>
__device__ __forceinline__ float pressure_from_etot<float, false>(
    const EnergyConsts<float>& ec, float rho, float etot, float vx, float vy,
    float vz, float bx, float by, float bz) {
  return pressure_ff<false>(ec.gm1, rho, etot, vx, vy, vz, bx, by, bz);
}

// apply_floor_to_energy_and_sync for one cell (EnzoPhysicsFluidProps.cpp:
// 245-287).  etot / eint are updated in place.
template <bool MHD, bool DE>
__device__ __forceinline__ void energy_floor_sync(const EnergyConsts<double>& ec,
                                                  double rho, double vx, double vy,
                                                  double vz, double bx, double by,
                                                  double bz, double& etot,
                                                  double& eint) {
  const double eta = DE ? ec.eta : 0.0;
  const double half_factor = DE ? ec.half_factor : 0.0;
  const double inv_rho = 1. / rho;
  const double eint_floor = ec.pfloor * ec.inv_gm1 * inv_rho;
  const double v2 = (vx * vx + vy * vy + vz * vz);
  double nte = 0.5 * v2;
  double b2 = 0;
  if (MHD) {
    b2 = (bx * bx + by * by + bz * bz);
    nte += (0.5 * b2 * inv_rho);
  }
  if (DE) {
    const double eint_1 = etot - nte;
    double cur = eint;
    const double cs2_1 = fmax(0., (double)ec.ggm1 * eint_1);
    if ((cs2_1 > fmax(eta * v2, eta * b2 * inv_rho)) && (eint_1 > half_factor * cur))
      cur = eint_1;
    cur = smax(cur, eint_floor);
    eint = cur;
    etot = cur + nte;
  } else {
    const double etot_floor = eint_floor + nte;
    etot = smax(etot, etot_floor);
  }
}

template <bool MHD, bool DE>
__device__ __forceinline__ void energy_floor_sync(const EnergyConsts<float>& ec,
                                                  float rho, float vx, float vy,
                                                  float vz, float bx, float by,
                                                  float bz, float& etot, float& eint) {
  const float eta = DE ? ec.eta : 0.f;
  const float half_factor = DE ? ec.half_factor : 0.f;
  const float inv_rho = 1.f / rho;
  const float eint_floor = ec.pfloor * ec.inv_gm1 * inv_rho;
  // non-thermal energy |v|^2/2 + |B|^2/(2 rho) in float-float
  const ff v2 = ff_sqsum(vx, vy, vz);
  ff nte = ff_scale(v2, 0.5f);
  ff b2 = {0.f, 0.f};
  if (MHD) {
    b2 = ff_sqsum(bx, by, bz);
    nte = ff_add(nte, ff_div(ff_scale(b2, 0.5f), rho));
  }
  if (DE) {
    const float eint_1 = ff_round(ff_add({etot, 0.f}, ff_neg(nte)));
    float cur = eint;
    const float cs2_1 = fmaxf(0.f, ec.ggm1 * eint_1);
    if ((cs2_1 > fmaxf(eta * ff_round(v2), eta * ff_round(b2) * inv_rho)) &&
        (eint_1 > half_factor * cur))
      cur = eint_1;
    cur = smax(cur, eint_floor);
    eint = cur;
    etot = ff_round(ff_add({cur, 0.f}, nte));
  } else {
    const float etot_floor = ff_round(ff_add({eint_floor, 0.f}, nte));
    etot = smax(etot, etot_floor);
  }
}

}  // namespace vlct
